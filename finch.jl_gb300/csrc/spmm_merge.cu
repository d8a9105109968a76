// Load-balanced SpMM for CSR matrices with skewed row lengths.
//
// Merge-path partitioning: the walk over a CSR matrix is the merge of two
// sorted lists -- the row ends (ptr) and the stored-entry positions -- of
// total length nrows + nnz.  Cutting that path into equal items gives every
// group of lanes the same amount of work whether it lands on one long row or
// on many empty ones.  A small plan kernel finds each item's start (row,
// entry) by binary search along its diagonal.
//
// Each item is walked by a group of G lanes holding a V-wide piece of a
// column slab [c0, c0 + G*V) of C.  Rows that end inside the item are
// stored directly (their first portion may belong to earlier items); the
// partial sum of the row still open at the item's end goes to a carry slot.
// A fix-up kernel then adds every run of carries of the same row to that row
// in item order, so results are deterministic run to run.
//
// Stored entries are read in chunks of G*E with coalesced evict-first loads,
// broadcast by shuffles, and up to BATCH gathers of B are kept in flight per
// lane.  One launch per slab keeps the gathered slab of B L2-resident.
#include "spmm_common.cuh"

namespace fgb {

constexpr int MP_BATCH = 8;

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

template <class T, class VT, class PtrT, int G, int V>
__global__ void __launch_bounds__(256) spmm_merge_k(
    int64_t nrows, const PtrT* __restrict__ ptr, const int* __restrict__ idx,
    const VT* __restrict__ val, const T* __restrict__ B, int64_t ldb, T* __restrict__ C,
    int64_t ldc, int64_t c0, int64_t nk, int base, int accumulate, int64_t n_items,
    const int64_t* __restrict__ plan_row, const int64_t* __restrict__ plan_k,
    int64_t* __restrict__ carry_row, T* __restrict__ carry) {
  constexpr int E = G >= MP_BATCH ? 1 : MP_BATCH / G;  // entries per lane per chunk
  constexpr int CH = G * E;
  const int lane = threadIdx.x & (G - 1);
  const unsigned gmask = group_mask<G>();
  const int64_t group = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t col = c0 + (int64_t)lane * V;
  const bool active_col = col < nk;
  const uint64_t pol_stream = policy_evict_first();
  const uint64_t pol_keep = policy_evict_last();

  for (int64_t w = group; w < n_items; w += ngroups) {
    int64_t r = plan_row[w], k = plan_k[w];
    const int64_t r1 = plan_row[w + 1], k1 = plan_k[w + 1];
    VecT<T, V> acc;
#pragma unroll
    for (int q = 0; q < V; ++q) acc.v[q] = T(0);
    while (true) {
      const int64_t e = r < r1 ? ld_ptr(ptr, r + 1) - base : k1;
      for (int64_t kb = k; kb < e; kb += CH) {
        int jj[E];
        T aa[E];
#pragma unroll
        for (int q = 0; q < E; ++q) {
          const int64_t p = kb + lane + q * G;
          jj[q] = 0;
          aa[q] = T(0);
          if (p < e) {
            jj[q] = ld_stream_i32(idx + p, pol_stream) - base;
            aa[q] = load_val<T, VT>(val, p, pol_stream);
          }
        }
        const int cnt = (e - kb) < (int64_t)CH ? (int)(e - kb) : CH;
#pragma unroll
        for (int t0 = 0; t0 < CH; t0 += MP_BATCH) {
          if (t0 >= cnt) break;
          VecT<T, V> b[MP_BATCH];
          T a[MP_BATCH];
#pragma unroll
          for (int t = 0; t < MP_BATCH; ++t) {
            const int tt = t0 + t < CH ? t0 + t : 0;
            const int j = __shfl_sync(gmask, jj[tt / G], tt % G, G);
            a[t] = __shfl_sync(gmask, aa[tt / G], tt % G, G);
            if (t0 + t < cnt && active_col) b[t] = gather<T, V>(B + (int64_t)j * ldb + col, pol_keep);
          }
#pragma unroll
          for (int t = 0; t < MP_BATCH; ++t)
            if (t0 + t < cnt && active_col) acc_step<T, V>(acc, a[t], b[t], FM_DEFAULT);
        }
      }
      k = e;
      if (r >= r1) break;
      if (active_col) {
        T* dst = C + r * ldc + col;
        if (accumulate) {
          const VecT<T, V> old = load_out<T, V>(dst);
#pragma unroll
          for (int q = 0; q < V; ++q) acc.v[q] += old.v[q];
        }
        store_out<T, V>(dst, acc, pol_stream);
      }
#pragma unroll
      for (int q = 0; q < V; ++q) acc.v[q] = T(0);
      ++r;
    }
    // the row left open at the item's end (if any) carries its partial sum
    if (lane == 0 && c0 == 0) carry_row[w] = r1 < nrows ? r1 : -1;
    if (active_col) {
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
  const int64_t n_items = (nrows + nnz + path - 1) / path;
  return align256(sizeof(int64_t) * (n_items + 1)) * 2 + align256(sizeof(int64_t) * n_items) +
         align256(esz * n_items * nk);
}

template <class T, class VT, class PtrT, int G>
static int launch_merge(fgb_ctx* ctx, const fgb_sparse* A, const T* B, int64_t ldb, int64_t nk,
                        T* C, int64_t ldc, int accumulate, int64_t path, char* scratch,
                        cudaStream_t s) {
  constexpr int V = sizeof(T) == 4 ? 4 : 2;
  const int64_t nrows = A->nrows, nnz = A->nnz;
  const int64_t n_items = (nrows + nnz + path - 1) / path;
  int64_t* plan_row = (int64_t*)scratch;
  int64_t* plan_k = (int64_t*)(scratch + align256(sizeof(int64_t) * (n_items + 1)));
  int64_t* carry_row = (int64_t*)((char*)plan_k + align256(sizeof(int64_t) * (n_items + 1)));
  T* carry = (T*)((char*)carry_row + align256(sizeof(int64_t) * n_items));
  const PtrT* ptr = (const PtrT*)A->ptr;
  merge_plan_k<PtrT><<<grid_for(n_items + 1, 256, ctx->num_sms, 4), 256, 0, s>>>(
      nrows, nnz, ptr, A->index_base, path, n_items, plan_row, plan_k);
  int rc = check_launch("merge_plan_k");
  if (rc) return rc;
  const int threads = 256;
  const int grid = grid_for(n_items * G, threads, ctx->num_sms, 16);
  for (int64_t c0 = 0; c0 < nk; c0 += (int64_t)G * V) {
    spmm_merge_k<T, VT, PtrT, G, V><<<grid, threads, 0, s>>>(
        nrows, ptr, (const int*)A->idx, (const VT*)A->val, B, ldb, C, ldc, c0, nk, A->index_base,
        accumulate, n_items, plan_row, plan_k, carry_row, carry);
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
                       cudaStream_t s) {
  switch (lanes) {
    case 2: return launch_merge<T, VT, PtrT, 2>(ctx, A, B, ldb, nk, C, ldc, accumulate, path, scratch, s);
    case 4: return launch_merge<T, VT, PtrT, 4>(ctx, A, B, ldb, nk, C, ldc, accumulate, path, scratch, s);
    case 8: return launch_merge<T, VT, PtrT, 8>(ctx, A, B, ldb, nk, C, ldc, accumulate, path, scratch, s);
    case 16: return launch_merge<T, VT, PtrT, 16>(ctx, A, B, ldb, nk, C, ldc, accumulate, path, scratch, s);
    default: return launch_merge<T, VT, PtrT, 32>(ctx, A, B, ldb, nk, C, ldc, accumulate, path, scratch, s);
  }
}

// Entry used by fgb_spmm for aligned CSR operands (nk, ldb, ldc multiples of
// the vector width).  scratch == NULL allocates it on the stream.
int spmm_merge(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk, void* C,
               int64_t ldc, int dtype, int accumulate, int lanes, int64_t path, void* scratch,
               size_t scratch_bytes, cudaStream_t s) {
  const size_t esz = dtype == FGB_F64 ? 8 : 4;
  const size_t need = spmm_merge_scratch_bytes(A->nrows, A->nnz, nk, esz, path);
  char* buf = (char*)scratch;
  if (buf && scratch_bytes < need)
    return set_error(FGB_EINVAL, "spmm: scratch of %zu bytes is below the %zu needed", scratch_bytes, need);
  if (!buf) FGB_CUDA_TRY(cudaMallocAsync((void**)&buf, need, s));
  int rc;
  const bool i32 = A->ptr_t == FGB_I32;
  if (dtype == FGB_F64)
    rc = i32 ? merge_lanes<double, double, int32_t>(ctx, A, (const double*)B, ldb, nk, (double*)C, ldc, accumulate, lanes, path, buf, s)
             : merge_lanes<double, double, int64_t>(ctx, A, (const double*)B, ldb, nk, (double*)C, ldc, accumulate, lanes, path, buf, s);
  else if (A->val_t == FGB_BF16)
    rc = i32 ? merge_lanes<float, __nv_bfloat16, int32_t>(ctx, A, (const float*)B, ldb, nk, (float*)C, ldc, accumulate, lanes, path, buf, s)
             : merge_lanes<float, __nv_bfloat16, int64_t>(ctx, A, (const float*)B, ldb, nk, (float*)C, ldc, accumulate, lanes, path, buf, s);
  else
    rc = i32 ? merge_lanes<float, float, int32_t>(ctx, A, (const float*)B, ldb, nk, (float*)C, ldc, accumulate, lanes, path, buf, s)
             : merge_lanes<float, float, int64_t>(ctx, A, (const float*)B, ldb, nk, (float*)C, ldc, accumulate, lanes, path, buf, s);
  if (!scratch) cudaFreeAsync(buf, s);
  return rc;
}

}  // namespace fgb
