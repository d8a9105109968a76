// Load-balanced SpMM for CSR matrices with skewed row lengths.
//
// Merge-path partitioning: the walk over a CSR matrix is the merge of two
// sorted lists -- the row ends (ptr) and the stored-entry positions -- of
// total length nrows + nnz.  Cutting that path into equal items gives every
// warp the same amount of work whether it lands on one long row or on many
// empty ones.  A small plan kernel finds each item's start (row, entry) by
// binary search along its diagonal.
//
// One warp walks one item at a time over a column slab [c0, c0 + 4L) of C
// (fp32; 2L for fp64): the warp splits into P = 32/L sub-groups of L lanes,
// every sub-group takes a different stored entry of the current row, and
// each lane gathers its 16-byte piece of that entry's row of B.  Control
// flow is uniform across the warp.  At a row end the P partial sums are
// combined with xor-shuffles and L lanes store the row's slab of C.  Row ends
// are read 32 at a time into a register window, so walking empty rows costs
// no dependent loads.  Rows that end inside the item are stored directly
// (their first portion may belong to earlier items); the partial sum of the
// row still open at the item's end goes to a carry slot, and a fix-up kernel
// adds every run of carries of one row to that row in item order -- results
// are deterministic run to run.
//
// Stored entries are read 32*E at a time with coalesced evict-first loads and
// broadcast by shuffles; up to BATCH gathers of B are in flight per lane.  The
// grid is persistent: occupancy-many blocks per SM, items handed out by warp.
#include "spmm_common.cuh"
#include "spmm_noalloc_plan.h"

namespace fgb {

constexpr int MP_BATCH = 8;
constexpr int MP_THREADS = 256;
constexpr int MP_MIN_BLOCKS = 3;  // <= 85 registers per thread: 24 warps per SM

template <class PtrT>
__global__ void merge_plan_k(int64_t nrows, int64_t nnz, const PtrT* __restrict__ ptr, int base,
                             int64_t path, int64_t n_items, int64_t* __restrict__ plan_row,
                             int64_t* __restrict__ plan_k) {
  const int64_t total = nrows + nnz;
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w <= n_items;
       w += (int64_t)gridDim.x * blockDim.x) {
    const int64_t d = min(w * path, total);
    int64_t lo = d > nnz ? d - nnz : 0;
    int64_t hi = d < nrows ? d : nrows;
    // largest i in [lo, hi] whose first i rows end within the first d - i entries
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (ld_ptr(ptr, mid) - base <= d - mid) lo = mid; else hi = mid - 1;
    }
    plan_row[w] = lo;
    plan_k[w] = d - lo;
  }
}

// Sums the P sub-group partials (lanes congruent mod L) into every lane.
template <class T, int V, int L>
__device__ __forceinline__ void reduce_subgroups(VecT<T, V>& acc) {
#pragma unroll
  for (int m = L; m < 32; m <<= 1)
#pragma unroll
    for (int q = 0; q < V; ++q) acc.v[q] += __shfl_xor_sync(0xffffffffu, acc.v[q], m);
}

template <class T, class VT, class PtrT, int L, int V>
__global__ void __launch_bounds__(MP_THREADS, MP_MIN_BLOCKS) spmm_merge_k(
    int64_t nrows, const PtrT* __restrict__ ptr, const int* __restrict__ idx,
    const VT* __restrict__ val, const T* __restrict__ B, int64_t ldb, T* __restrict__ C,
    int64_t ldc, int64_t c0, int64_t nk, int base, int accumulate, int64_t n_items,
    const int64_t* __restrict__ plan_row, const int64_t* __restrict__ plan_k,
    int64_t* __restrict__ carry_row, T* __restrict__ carry, const int32_t* __restrict__ row_map) {
  constexpr int P = 32 / L;                          // entries in flight per warp step
  constexpr int E = (MP_BATCH + L - 1) / L;          // so every sub-group gets >= BATCH
  constexpr int CH = 32 * E;                         // entries per chunk
  constexpr int PER_SUB = CH / P;                    // entries per sub-group per chunk
  const int lane = threadIdx.x & 31;
  const int sub = lane / L, sl = lane % L;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t col = c0 + (int64_t)sl * V;
  const bool active_col = col < nk;
  const T* Bc = B + col;
  const uint64_t pol_stream = policy_evict_first();
  const uint64_t pol_keep = policy_evict_last();

  for (int64_t w = warp; w < n_items; w += nwarps) {
    int64_t r = plan_row[w], k = plan_k[w];
    const int64_t r1 = plan_row[w + 1], k1 = plan_k[w + 1];
    // row-end window: lane l holds the end of row rw + l
    int64_t rw = r;
    int64_t re = rw + lane < nrows ? ld_ptr(ptr, rw + 1 + lane) - base : INT64_MAX;
    VecT<T, V> acc;
#pragma unroll
    for (int q = 0; q < V; ++q) acc.v[q] = T(0);
    bool touched = false;
    while (true) {
      if (r - rw >= 32) {
        rw = r;
        re = rw + lane < nrows ? ld_ptr(ptr, rw + 1 + lane) - base : INT64_MAX;
      }
      const int64_t e = r < r1 ? __shfl_sync(0xffffffffu, re, (int)(r - rw)) : k1;
      touched |= k < e;
      for (int64_t kb = k; kb < e; kb += CH) {
        int jj[E];
        T aa[E];
#pragma unroll
        for (int q = 0; q < E; ++q) {
          const int64_t p = kb + lane + 32 * q;
          jj[q] = 0;
          aa[q] = T(0);
          if (p < e) {
            jj[q] = ld_stream_i32(idx + p, pol_stream) - base;
            aa[q] = load_val<T, VT>(val, p, pol_stream);
          }
        }
        const int cnt = (e - kb) < (int64_t)CH ? (int)(e - kb) : CH;
#pragma unroll
        for (int t0 = 0; t0 < PER_SUB; t0 += MP_BATCH) {
          if (t0 * P >= cnt) break;
          VecT<T, V> b[MP_BATCH];
          // issue the batch's gathers first, then consume them
#pragma unroll
          for (int t = 0; t < MP_BATCH; ++t) {
            const int tt = t0 + t;                 // step inside the chunk
            const int q = (tt * P) / 32;           // compile-time register slot
            const int src = (tt * P) % 32 + sub;   // lane that loaded the entry
            const int j = __shfl_sync(0xffffffffu, jj[q < E ? q : 0], src);
            if (tt < PER_SUB && tt * P + sub < cnt && active_col)
              b[t] = gather<T, V>(Bc + (int64_t)j * ldb, pol_keep);
          }
#pragma unroll
          for (int t = 0; t < MP_BATCH; ++t) {
            const int tt = t0 + t;
            const int q = (tt * P) / 32;
            const int src = (tt * P) % 32 + sub;
            const T a = __shfl_sync(0xffffffffu, aa[q < E ? q : 0], src);
            if (tt < PER_SUB && tt * P + sub < cnt && active_col)
              acc_step<T, V>(acc, a, b[t], FM_DEFAULT);
          }
        }
      }
      k = e;
      if (r >= r1) break;
      if (touched) reduce_subgroups<T, V, L>(acc);
      if (sub == 0 && active_col) {
        T* dst = C + (row_map ? (int64_t)__ldg(row_map + r) : r) * ldc + col;
        if (accumulate) {
          const VecT<T, V> old = load_out<T, V>(dst);
#pragma unroll
          for (int q = 0; q < V; ++q) acc.v[q] += old.v[q];
        }
        store_out<T, V>(dst, acc, pol_stream);
      }
#pragma unroll
      for (int q = 0; q < V; ++q) acc.v[q] = T(0);
      touched = false;
      ++r;
    }
    // the row left open at the item's end (if any) carries its partial sum
    if (touched) reduce_subgroups<T, V, L>(acc);
    if (lane == 0 && c0 == 0)
      carry_row[w] = r1 < nrows ? (row_map ? (int64_t)__ldg(row_map + r1) : r1) : -1;
    if (sub == 0 && active_col) {
      T* cdst = carry + w * nk + col;
#pragma unroll
      for (int q = 0; q < V; ++q) cdst[q] = acc.v[q];
    }
  }
}

// Adds each run of carries of one row to that row, in item order.
template <class T>
__global__ void spmm_fixup_k(int64_t n_items, int64_t nk, const int64_t* __restrict__ carry_row,
                             const T* __restrict__ carry, T* __restrict__ C, int64_t ldc) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n_items * nk;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w = t / nk, c = t - w * nk;
    const int64_t r = carry_row[w];
    if (r < 0 || (w > 0 && carry_row[w - 1] == r)) continue;
    T sum = carry[w * nk + c];
    for (int64_t w2 = w + 1; w2 < n_items && carry_row[w2] == r; ++w2) sum += carry[w2 * nk + c];
    C[r * ldc + c] += sum;
  }
}

static inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

size_t spmm_merge_scratch_bytes(int64_t nrows, int64_t nnz, int64_t nk, size_t esz, int64_t path) {
  return merge_scratch_bytes(nrows, nnz, nk, esz, path);  // the layout launch_merge carves below
}

template <class T, class VT, class PtrT, int L>
static int launch_merge(fgb_ctx* ctx, const fgb_sparse* A, const T* B, int64_t ldb, int64_t nk,
                        T* C, int64_t ldc, int accumulate, int64_t path, char* scratch,
                        cudaStream_t s, bool plan_ready, const int32_t* row_map, int variant) {
  constexpr int V = sizeof(T) == 4 ? 4 : 2;
  const int64_t nrows = A->nrows, nnz = A->nnz;
  const int64_t n_items = (nrows + nnz + path - 1) / path;
  int64_t* plan_row = (int64_t*)scratch;
  int64_t* plan_k = (int64_t*)(scratch + align256(sizeof(int64_t) * (n_items + 1)));
  int64_t* carry_row = (int64_t*)((char*)plan_k + align256(sizeof(int64_t) * (n_items + 1)));
  T* carry = (T*)((char*)carry_row + align256(sizeof(int64_t) * n_items));
  const PtrT* ptr = (const PtrT*)A->ptr;
  int rc = FGB_OK;
  if (!plan_ready) {
    merge_plan_k<PtrT><<<grid_for(n_items + 1, 256, ctx->num_sms, 4), 256, 0, s>>>(
        nrows, nnz, ptr, A->index_base, path, n_items, plan_row, plan_k);
    rc = check_launch("merge_plan_k");
    if (rc) return rc;
  }
  static thread_local int occ_cache[2][6] = {};
  int& occ = occ_cache[sizeof(T) == 8][L == 1 ? 0 : L == 2 ? 1 : L == 4 ? 2 : L == 8 ? 3 : L == 16 ? 4 : 5];
  if (occ == 0) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, spmm_merge_k<T, VT, PtrT, L, V>, MP_THREADS, 0);
    if (occ <= 0) occ = 1;
  }
  const int64_t warps_needed = n_items;
  int64_t grid = (int64_t)ctx->num_sms * occ;
  const int64_t grid_need = (warps_needed * 32 + MP_THREADS - 1) / MP_THREADS;
  if (grid > grid_need) grid = grid_need;
  if (grid < 1) grid = 1;
  if (variant == 1 && sizeof(T) == 4) {  // B rows staged through shared memory by TMA
    rc = spmm_tma_items(ctx, A, B, ldb, nk, C, ldc, accumulate, n_items, plan_row, plan_k,
                        carry_row, carry, row_map, ctx->d_err, s);
    if (rc) return rc;
  } else
  for (int64_t c0 = 0; c0 < nk; c0 += (int64_t)L * V) {
    spmm_merge_k<T, VT, PtrT, L, V><<<(int)grid, MP_THREADS, 0, s>>>(
        nrows, ptr, (const int*)A->idx, (const VT*)A->val, B, ldb, C, ldc, c0, nk, A->index_base,
        accumulate, n_items, plan_row, plan_k, carry_row, carry, row_map);
    rc = check_launch("spmm_merge_k");
    if (rc) return rc;
  }
  spmm_fixup_k<T><<<grid_for(n_items * nk, 256, ctx->num_sms, 8), 256, 0, s>>>(
      n_items, nk, carry_row, carry, C, ldc);
  return check_launch("spmm_fixup_k");
}

template <class T, class VT, class PtrT>
static int merge_lanes(fgb_ctx* ctx, const fgb_sparse* A, const T* B, int64_t ldb, int64_t nk,
                       T* C, int64_t ldc, int accumulate, int lanes, int64_t path, char* scratch,
                       cudaStream_t s, bool plan_ready, const int32_t* row_map, int variant) {
  switch (lanes) {
    case 2: return launch_merge<T, VT, PtrT, 2>(ctx, A, B, ldb, nk, C, ldc, accumulate, path, scratch, s, plan_ready, row_map, variant);
    case 4: return launch_merge<T, VT, PtrT, 4>(ctx, A, B, ldb, nk, C, ldc, accumulate, path, scratch, s, plan_ready, row_map, variant);
    case 8: return launch_merge<T, VT, PtrT, 8>(ctx, A, B, ldb, nk, C, ldc, accumulate, path, scratch, s, plan_ready, row_map, variant);
    case 16: return launch_merge<T, VT, PtrT, 16>(ctx, A, B, ldb, nk, C, ldc, accumulate, path, scratch, s, plan_ready, row_map, variant);
    default: return launch_merge<T, VT, PtrT, 32>(ctx, A, B, ldb, nk, C, ldc, accumulate, path, scratch, s, plan_ready, row_map, variant);
  }
}

// Entry used by fgb_spmm for aligned CSR operands (nk, ldb, ldc multiples of
// the vector width).  scratch == NULL allocates it on the stream.
int spmm_merge(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk, void* C,
               int64_t ldc, int dtype, int accumulate, int lanes, int64_t path, void* scratch,
               size_t scratch_bytes, cudaStream_t s, bool plan_ready, const int32_t* row_map,
               int variant) {
  const size_t esz = dtype == FGB_F64 ? 8 : 4;
  const size_t need = spmm_merge_scratch_bytes(A->nrows, A->nnz, nk, esz, path);
  char* buf = (char*)scratch;
  if (buf && scratch_bytes < need)
    return set_error(FGB_EINVAL, "spmm: scratch of %zu bytes is below the %zu needed", scratch_bytes, need);
  if (!buf) FGB_CUDA_TRY(cudaMallocAsync((void**)&buf, need, s));
  int rc;
  const bool i32 = A->ptr_t == FGB_I32;
  if (dtype == FGB_F64)
    rc = i32 ? merge_lanes<double, double, int32_t>(ctx, A, (const double*)B, ldb, nk, (double*)C, ldc, accumulate, lanes, path, buf, s, plan_ready && scratch, row_map, variant)
             : merge_lanes<double, double, int64_t>(ctx, A, (const double*)B, ldb, nk, (double*)C, ldc, accumulate, lanes, path, buf, s, plan_ready && scratch, row_map, variant);
  else if (A->val_t == FGB_BF16)
    rc = i32 ? merge_lanes<float, __nv_bfloat16, int32_t>(ctx, A, (const float*)B, ldb, nk, (float*)C, ldc, accumulate, lanes, path, buf, s, plan_ready && scratch, row_map, variant)
             : merge_lanes<float, __nv_bfloat16, int64_t>(ctx, A, (const float*)B, ldb, nk, (float*)C, ldc, accumulate, lanes, path, buf, s, plan_ready && scratch, row_map, variant);
  else
    rc = i32 ? merge_lanes<float, float, int32_t>(ctx, A, (const float*)B, ldb, nk, (float*)C, ldc, accumulate, lanes, path, buf, s, plan_ready && scratch, row_map, variant)
             : merge_lanes<float, float, int64_t>(ctx, A, (const float*)B, ldb, nk, (float*)C, ldc, accumulate, lanes, path, buf, s, plan_ready && scratch, row_map, variant);
  if (!scratch) cudaFreeAsync(buf, s);
  return rc;
}

}  // namespace fgb
