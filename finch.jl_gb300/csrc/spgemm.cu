// SpGEMM C = A * B (plus-times, F64/F32), Gustavson's row-wise algorithm.
//
// Finch's Gustavson (docs/examples/spgemm.jl:56-72; test/suites/
// kernel_tests.jl:89-129) walks, for each output fiber, the stored entries k
// of the other operand in order and accumulates w[i] += A[i,k] * B[k,j] in
// a SparseByteMap workspace, then copies the touched coordinates out in
// order.  Here one CSR kernel does the row form C[r,:] = sum_k L[r,k] R[k,:];
// Finch's column form (CSC operands) is the same kernel on the transposed
// problem C^T = B^T A^T, whose CSR buffers are A's and B's CSC buffers.
//
// Per output row: an upper bound ub = sum of |R[k,:]| over the row's k picks
// a tier -- 8 lanes (ub <= 64) or a warp (ub <= 256) with a hash table in
// shared memory, or a block with a hash table in global scratch.  The symbolic pass inserts the
// column keys and counts them (C's ptr); the numeric pass walks the row's k
// in storage order, one k at a time (a barrier between them), with the
// lanes spread over R[k,:] -- every column occurs once per k, so each output
// accumulates its products in k order without atomics, exactly Gustavson's
// order: bit-identical to the serial nest for the same fused/unfused
// choice.  Touched keys are stored even if their sum is zero (like the
// workspace).  A warp writes each pair at its rank among the row's keys, so
// small rows come out ordered; a segmented sort orders the large rows.
#include <cub/cub.cuh>

#include "fgb_internal.cuh"
#include "semiring.cuh"

namespace fgb {

constexpr int SG_WARP_SLOTS = 512;  // hash slots per warp (ub <= SG_WARP_UB)
constexpr int SG_WARP_UB = 256;
constexpr int SG_SMALL_UB = 64;      // rows up to this bound take 8 lanes (128 slots)
constexpr int SG_WARPS = 4;          // warps per block of the warp tier
constexpr int SG_BLOCK = 256;        // threads of the block tier
constexpr int32_t SG_EMPTY = -1;
// table slots per lane in the warp tiers: 8 lanes with at most 2 * 64 slots,
// a warp with at most SG_WARP_SLOTS
constexpr int SG_SLOTS_PER_LANE = 16;
static_assert(SG_WARP_SLOTS / 32 <= SG_SLOTS_PER_LANE && 2 * SG_SMALL_UB / 8 <= SG_SLOTS_PER_LANE,
              "a lane's share of a warp-tier table");

__device__ __forceinline__ uint32_t sg_hash(int32_t c) { return (uint32_t)c * 2654435761u; }

template <class PtrT>
__global__ void sg_bound_k(int64_t m, const PtrT* __restrict__ lp, const int* __restrict__ li, int lbase,
                           const PtrT* __restrict__ rp, int64_t* __restrict__ ub) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
       r += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = 0;
    for (int64_t q = ld_ptr(lp, r) - lbase; q < ld_ptr(lp, r + 1) - lbase; ++q) {
      const int64_t k = __ldg(li + q) - lbase;
      s += ld_ptr(rp, k + 1) - ld_ptr(rp, k);
    }
    ub[r] = s;
  }
}

// Global-hash sizes of the block-tier rows (0 for warp-tier rows).
__global__ void sg_gsize_k(int64_t m, const int64_t* __restrict__ ub, int64_t* __restrict__ gsize) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
       r += (int64_t)gridDim.x * blockDim.x) {
    int64_t h = 0;
    if (ub[r] > SG_WARP_UB) {
      h = 1;
      while (h < 2 * ub[r]) h <<= 1;
    }
    gsize[r] = h;
  }
}

// Inserts key c into a table of `cap` slots (power of two); returns its slot
// and whether this call created it.  I: the slot index type (32-bit for the
// shared-memory tables).
template <class I>
__device__ __forceinline__ I sg_insert(int32_t* keys, I cap, int32_t c, bool* created) {
  I s = (I)(sg_hash(c) & (uint32_t)(cap - 1));
  while (true) {
    const int32_t k = ((volatile int32_t*)keys)[s];
    if (k == c) {
      *created = false;
      return s;
    }
    if (k == SG_EMPTY) {
      const int32_t old = atomicCAS(keys + s, SG_EMPTY, c);
      if (old == SG_EMPTY) {
        *created = true;
        return s;
      }
      if (old == c) {
        *created = false;
        return s;
      }
    }
    s = (s + 1) & (cap - 1);
  }
}

template <class T>
__device__ __forceinline__ T sg_acc(T w, T a, T b, int fm) {
  return Semi<SR_PT, T>::step(w, a, b, fm);
}

// One row with `nthreads` cooperating threads (a warp or a block) over a
// table of `cap` slots.  SYMB: count keys into *cnt.  Else: accumulate and
// write the row's (column, value) pairs, unsorted, from out_pos.  Positions
// in A and B are counted in their ptr type, table slots in I (32-bit for the
// shared-memory tables): the narrower loop arithmetic issues fewer
// instructions.
template <class T, class PtrT, bool SYMB, class I>
__device__ void sg_row(int64_t r, int tid, int nthreads, const PtrT* __restrict__ lp,
                       const int* __restrict__ li, const T* __restrict__ lv, int lbase,
                       const PtrT* __restrict__ rp, const int* __restrict__ ri,
                       const T* __restrict__ rv, int rbase, int32_t* keys, T* vals, I cap,
                       int fm, int* cnt, int out_base, int32_t* __restrict__ out_idx,
                       T* __restrict__ out_val, int64_t out_pos, unsigned smask) {
  // smask: the lanes of a (sub-)warp group; 0 for a whole block
  const bool warp = smask != 0;
  auto sync = [&]() {
    if (warp) __syncwarp(smask); else __syncthreads();
  };
  for (I s = tid; s < cap; s += nthreads) keys[s] = SG_EMPTY;
  if (tid == 0) *cnt = 0;
  sync();
  const PtrT q0 = __ldg(lp + r) - lbase, q1 = __ldg(lp + r + 1) - lbase;
  int made = 0;  // SYMB in a warp tier: keys this lane created
  for (PtrT q = q0; q < q1; ++q) {  // k in storage order
    const int k = __ldg(li + q) - lbase;
    const T a = SYMB ? T(0) : lv[q];
    const PtrT p0 = __ldg(rp + k) - rbase, p1 = __ldg(rp + k + 1) - rbase;
    for (PtrT p = p0 + tid; p < p1; p += nthreads) {
      const int32_t c = __ldg(ri + p) - rbase;
      bool created;
      const I s = sg_insert<I>(keys, cap, c, &created);
      if (SYMB) {
        if (warp) made += created ? 1 : 0;
        else if (created) atomicAdd(cnt, 1);
      } else {
        const T b = rv[p];
        vals[s] = sg_acc(created ? T(0) : vals[s], a, b, fm);
      }
    }
    sync();  // the next k sees this one's sums
  }
  if (SYMB && warp) {  // the group's count: a shuffle sum, not an atomic per key
    for (int m = nthreads >> 1; m >= 1; m >>= 1) made += __shfl_xor_sync(smask, made, m, nthreads);
    if (tid == 0) *cnt = made;
  }
  if (!SYMB && warp) {
    // Small table: the row's keys are first listed compactly -- (key, slot)
    // pairs written over the key table, which holds at least twice as many
    // slots as the row has keys -- and each key's rank among the n listed
    // keys is its sorted position.  Ranking against the whole table instead
    // ran a cap-long loop per occupied slot on every lane of the warp.
    int32_t myk[SG_SLOTS_PER_LANE];
    int cnt_mine = 0;
#pragma unroll
    for (int u = 0; u < SG_SLOTS_PER_LANE; ++u) {
      const I s = tid + u * nthreads;
      myk[u] = s < cap ? keys[s] : SG_EMPTY;
      cnt_mine += myk[u] != SG_EMPTY ? 1 : 0;
    }
    int incl = cnt_mine;  // inclusive scan over the group's lanes
    for (int m = 1; m < nthreads; m <<= 1) {
      const int t = __shfl_up_sync(smask, incl, m, nthreads);
      if (tid >= m) incl += t;
    }
    const int n = __shfl_sync(smask, incl, nthreads - 1, nthreads);
    int pos = incl - cnt_mine;
    sync();  // every lane has read its keys before the list overwrites them
    int2* list = reinterpret_cast<int2*>(keys);
#pragma unroll
    for (int u = 0; u < SG_SLOTS_PER_LANE; ++u)
      if (myk[u] != SG_EMPTY) list[pos++] = make_int2(myk[u], (int)(tid + u * nthreads));
    sync();
    for (int p = tid; p < n; p += nthreads) {
      const int2 e = list[p];
      int o = 0;
      for (int q = 0; q < n; ++q) o += list[q].x < e.x ? 1 : 0;
      out_idx[out_pos + o] = e.x + out_base;
      out_val[out_pos + o] = vals[e.y];
    }
  } else if (!SYMB) {  // large rows: unsorted here, ordered by a segmented sort afterwards
    for (I s = tid; s < cap; s += nthreads) {
      const int32_t c = keys[s];
      if (c != SG_EMPTY) {
        const int o = atomicAdd(cnt, 1);
        out_idx[out_pos + o] = c + out_base;
        out_val[out_pos + o] = vals[s];
      }
    }
  }
  sync();
}

// Rows whose bound lies in (LO, HI] with G lanes per row (32 / G rows per
// warp), each group with a table of 16 * G slots in shared memory.
template <class T, class PtrT, bool SYMB, int G>
__global__ void __launch_bounds__(SG_WARPS * 32) sg_warp_k(
    int64_t m, const int64_t* __restrict__ ub, int64_t lo, int64_t hi, const PtrT* __restrict__ lp,
    const int* __restrict__ li, const T* __restrict__ lv, int lbase, const PtrT* __restrict__ rp,
    const int* __restrict__ ri, const T* __restrict__ rv, int rbase, int fm,
    int64_t* __restrict__ cnt_out, const int64_t* __restrict__ cptr, int out_base,
    int32_t* __restrict__ out_idx, T* __restrict__ out_val) {
  constexpr int NG = SG_WARPS * 32 / G;      // groups per block
  constexpr int SLOTS = SG_WARP_SLOTS * G / 32;
  __shared__ __align__(8) int32_t s_keys[NG][SLOTS];  // 8-byte aligned: the key list is int2 pairs
  __shared__ T s_vals[SYMB ? 1 : NG][SYMB ? 1 : SLOTS];
  __shared__ int s_cnt[NG];
  __shared__ int64_t s_rows[SG_WARPS * 32];  // this tile's rows of the tier
  __shared__ int s_n;
  const int grp = threadIdx.x / G, gl = threadIdx.x % G;
  const unsigned gmask = group_mask<G>();
  // tiles of one row per thread: one coalesced look at the bounds, then the
  // groups take the tile's rows of this tier
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < m; base += (int64_t)gridDim.x * blockDim.x) {
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    const int64_t rr = base + threadIdx.x;
    if (rr < m) {
      const int64_t u = ub[rr];
      if (u > lo && u <= hi) s_rows[atomicAdd(&s_n, 1)] = rr;
    }
    __syncthreads();
    const int n = s_n;
    for (int t = grp; t < n; t += NG) {
      const int64_t r = s_rows[t];
      const int64_t u = ub[r];
      int cap = 16;  // a table sized to the row: at least twice its bound
      while (cap < 2 * u) cap <<= 1;
      sg_row<T, PtrT, SYMB, int>(r, gl, G, lp, li, lv, lbase, rp, ri, rv, rbase, s_keys[grp],
                            SYMB ? nullptr : &s_vals[SYMB ? 0 : grp][0], cap, fm, &s_cnt[grp],
                            out_base, out_idx, out_val, SYMB ? 0 : cptr[r] - out_base, gmask);
      if (SYMB && gl == 0) cnt_out[r] = s_cnt[grp];
    }
    __syncthreads();  // s_rows is refilled for the next tile
  }
}

template <class T, class PtrT, bool SYMB>
__global__ void __launch_bounds__(SG_BLOCK) sg_block_k(
    int64_t m, const int64_t* __restrict__ ub, const int64_t* __restrict__ goff,
    int32_t* __restrict__ gkeys, T* __restrict__ gvals, const PtrT* __restrict__ lp,
    const int* __restrict__ li, const T* __restrict__ lv, int lbase, const PtrT* __restrict__ rp,
    const int* __restrict__ ri, const T* __restrict__ rv, int rbase, int fm,
    int64_t* __restrict__ cnt_out, const int64_t* __restrict__ cptr, int out_base,
    int32_t* __restrict__ out_idx, T* __restrict__ out_val) {
  __shared__ int s_cnt;
  __shared__ int64_t s_rows[SG_BLOCK];
  __shared__ int s_n;
  for (int64_t base = blockIdx.x * (int64_t)SG_BLOCK; base < m; base += (int64_t)gridDim.x * SG_BLOCK) {
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    const int64_t rr = base + threadIdx.x;
    if (rr < m && ub[rr] > SG_WARP_UB) s_rows[atomicAdd(&s_n, 1)] = rr;
    __syncthreads();
    const int n = s_n;
    for (int t = 0; t < n; ++t) {  // block-uniform
      const int64_t r = s_rows[t];
      const int64_t off = goff[r], cap = goff[r + 1] - off;
      sg_row<T, PtrT, SYMB, int64_t>(r, threadIdx.x, SG_BLOCK, lp, li, lv, lbase, rp, ri, rv, rbase,
                            gkeys + off, SYMB ? nullptr : gvals + off, cap, fm, &s_cnt, out_base,
                            out_idx, out_val, SYMB ? 0 : cptr[r] - out_base, 0u);
      if (SYMB && threadIdx.x == 0) cnt_out[r] = s_cnt;
    }
    __syncthreads();
  }
}

// Segment bounds for the final sort: the block-tier rows only (warp-tier
// rows are written in order already and become empty segments).
__global__ void sg_segs_k(int64_t m, const int64_t* __restrict__ ub, const int64_t* __restrict__ cptr,
                          int base, int64_t* __restrict__ sb, int64_t* __restrict__ se) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
       r += (int64_t)gridDim.x * blockDim.x) {
    const bool big = ub[r] > SG_WARP_UB;
    sb[r] = cptr[r] - base;
    se[r] = big ? cptr[r + 1] - base : cptr[r] - base;
  }
}

__global__ void sg_rebase_k(int64_t n, const int64_t* __restrict__ in, int base, int64_t* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = in[i] - base;
}

static inline size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

struct SgProblem {
  const fgb_sparse* L;  // row operand (CSR view)
  const fgb_sparse* R;
  int64_t m, n;         // rows of the CSR result, columns
};

// ub, block-tier hash offsets and the scratch for the hash tables.
struct SgScratch {
  char* mem = nullptr;
  int64_t* ub = nullptr;
  int64_t* gsize = nullptr;
  int64_t* goff = nullptr;
  int64_t* cnt = nullptr;
  int32_t* gkeys = nullptr;
  void* gvals = nullptr;
  void* cub_tmp = nullptr;
  size_t cub_bytes = 0;
};

template <class PtrT>
static int sg_prepare(fgb_ctx* ctx, const SgProblem& P, size_t esz, SgScratch* S, cudaStream_t s) {
  const int64_t m = P.m;
  size_t cub_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, cub_bytes, (int64_t*)nullptr, (int64_t*)nullptr, (int)(m + 1), s);
  const size_t head = a256(8 * (m + 1)) * 4 + a256(cub_bytes);
  char* mem = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&mem, head, s);
  if (e != cudaSuccess) return set_error(FGB_ENOMEM, "fgb_spgemm: scratch: %s", cudaGetErrorString(e));
  S->mem = mem;
  S->ub = (int64_t*)mem;
  S->gsize = (int64_t*)(mem + a256(8 * (m + 1)));
  S->goff = (int64_t*)(mem + 2 * a256(8 * (m + 1)));
  S->cnt = (int64_t*)(mem + 3 * a256(8 * (m + 1)));
  S->cub_tmp = mem + 4 * a256(8 * (m + 1));
  S->cub_bytes = cub_bytes;
  const int grid = grid_for(m, 256, ctx->num_sms);
  cudaMemsetAsync(S->ub + m, 0, 8, s);
  sg_bound_k<PtrT><<<grid, 256, 0, s>>>(m, (const PtrT*)P.L->ptr, (const int*)P.L->idx, P.L->index_base,
                                        (const PtrT*)P.R->ptr, S->ub);
  sg_gsize_k<<<grid, 256, 0, s>>>(m + 1, S->ub, S->gsize);
  size_t cb = cub_bytes;
  e = cub::DeviceScan::ExclusiveSum(S->cub_tmp, cb, S->gsize, S->goff, (int)(m + 1), s);
  int64_t total = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, S->goff + m, 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(FGB_ECUDA, "fgb_spgemm: bounds: %s", cudaGetErrorString(e));
  if (total > 0) {
    char* g = nullptr;
    e = cudaMallocAsync((void**)&g, a256(4 * total) + a256(esz * total), s);
    if (e != cudaSuccess) return set_error(FGB_ENOMEM, "fgb_spgemm: %lld hash slots: %s", (long long)total, cudaGetErrorString(e));
    S->gkeys = (int32_t*)g;
    S->gvals = g + a256(4 * total);
  }
  return FGB_OK;
}

static void sg_release(SgScratch* S, cudaStream_t s) {
  if (S->gkeys) cudaFreeAsync(S->gkeys, s);
  if (S->mem) cudaFreeAsync(S->mem, s);
  *S = SgScratch{};
}

template <class T, class PtrT, bool SYMB>
static void sg_launch(fgb_ctx* ctx, const SgProblem& P, const SgScratch& S, int fm, const int64_t* cptr,
                      int out_base, int32_t* out_idx, T* out_val, cudaStream_t s) {
  const fgb_sparse *L = P.L, *R = P.R;
  // small rows: 8 lanes each (bound <= 64); medium: a warp each (<= 256)
  const int g8 = grid_for(P.m, SG_WARPS * 32, ctx->num_sms, 16);
  sg_warp_k<T, PtrT, SYMB, 8><<<g8, SG_WARPS * 32, 0, s>>>(
      P.m, S.ub, -1, SG_SMALL_UB, (const PtrT*)L->ptr, (const int*)L->idx, (const T*)L->val,
      L->index_base, (const PtrT*)R->ptr, (const int*)R->idx, (const T*)R->val, R->index_base, fm,
      S.cnt, cptr, out_base, out_idx, out_val);
  const int g32 = grid_for(P.m, SG_WARPS * 32, ctx->num_sms, 16);
  sg_warp_k<T, PtrT, SYMB, 32><<<g32, SG_WARPS * 32, 0, s>>>(
      P.m, S.ub, SG_SMALL_UB, SG_WARP_UB, (const PtrT*)L->ptr, (const int*)L->idx, (const T*)L->val,
      L->index_base, (const PtrT*)R->ptr, (const int*)R->idx, (const T*)R->val, R->index_base, fm,
      S.cnt, cptr, out_base, out_idx, out_val);
  sg_block_k<T, PtrT, SYMB><<<ctx->num_sms * 4, SG_BLOCK, 0, s>>>(
      P.m, S.ub, S.goff, S.gkeys, (T*)S.gvals, (const PtrT*)L->ptr, (const int*)L->idx,
      (const T*)L->val, L->index_base, (const PtrT*)R->ptr, (const int*)R->idx, (const T*)R->val,
      R->index_base, fm, S.cnt, cptr, out_base, out_idx, out_val);
}

static int sg_problem(const fgb_sparse* A, const fgb_sparse* B, SgProblem* P, const char* who) {
  if (A->orient != B->orient) return set_error(FGB_EUNSUPPORTED, "%s: A and B must share an orientation", who);
  if (A->ncols != B->nrows) return set_error(FGB_EINVAL, "%s: inner dimensions differ", who);
  if (A->ptr_t != B->ptr_t) return set_error(FGB_EUNSUPPORTED, "%s: A and B must share a ptr type", who);
  if (A->idx_t != FGB_I32 || B->idx_t != FGB_I32) return set_error(FGB_EUNSUPPORTED, "%s: int32 indices only", who);
  if (A->orient == FGB_CSR) {
    *P = SgProblem{A, B, A->nrows, B->ncols};
  } else {  // CSC: C^T = B^T A^T in CSR terms
    *P = SgProblem{B, A, B->ncols, A->nrows};
  }
  if (P->n > INT32_MAX) return set_error(FGB_EUNSUPPORTED, "%s: more than 2^31 columns", who);
  return FGB_OK;
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_spgemm_symbolic(fgb_ctx* ctx, const fgb_sparse* A, const fgb_sparse* B, int64_t* c_ptr,
                                   int64_t* nnz_c, void* stream) {
  if (!ctx || !A || !B || !c_ptr || !nnz_c) return set_error(FGB_EINVAL, "fgb_spgemm_symbolic: null argument");
  *nnz_c = 0;
  int rc = check_sparse(A, "fgb_spgemm_symbolic: A", false);
  if (!rc) rc = check_sparse(B, "fgb_spgemm_symbolic: B", false);
  SgProblem P;
  if (!rc) rc = sg_problem(A, B, &P, "fgb_spgemm_symbolic");
  if (rc) return rc;
  cudaStream_t s = pick_stream(ctx, stream);
  SgScratch S;
  rc = A->ptr_t == FGB_I32 ? sg_prepare<int32_t>(ctx, P, 1, &S, s) : sg_prepare<int64_t>(ctx, P, 1, &S, s);
  if (rc) {
    sg_release(&S, s);
    return rc;
  }
  cudaMemsetAsync(S.cnt + P.m, 0, 8, s);
  if (A->ptr_t == FGB_I32)
    sg_launch<float, int32_t, true>(ctx, P, S, 0, nullptr, 0, nullptr, nullptr, s);
  else
    sg_launch<float, int64_t, true>(ctx, P, S, 0, nullptr, 0, nullptr, nullptr, s);
  size_t cb = S.cub_bytes;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(S.cub_tmp, cb, S.cnt, c_ptr, (int)(P.m + 1), s);
  // C's ptr in A's index base
  if (e == cudaSuccess && A->index_base != 0) {
    sg_rebase_k<<<grid_for(P.m + 1, 256, ctx->num_sms), 256, 0, s>>>(P.m + 1, c_ptr, -A->index_base, c_ptr);
    e = cudaGetLastError();
  }
  int64_t total = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, c_ptr + P.m, 8, cudaMemcpyDeviceToHost, s);
  sg_release(&S, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(FGB_ECUDA, "fgb_spgemm_symbolic: %s", cudaGetErrorString(e));
  *nnz_c = total - A->index_base;
  return FGB_OK;
}

extern "C" int fgb_spgemm_numeric(fgb_ctx* ctx, const fgb_sparse* A, const fgb_sparse* B, int dtype,
                                  unsigned flags, fgb_sparse* C, void* stream) {
  if (!ctx || !A || !B || !C) return set_error(FGB_EINVAL, "fgb_spgemm_numeric: null argument");
  int rc = check_sparse(A, "fgb_spgemm_numeric: A", true);
  if (!rc) rc = check_sparse(B, "fgb_spgemm_numeric: B", true);
  SgProblem P;
  if (!rc) rc = sg_problem(A, B, &P, "fgb_spgemm_numeric");
  if (rc) return rc;
  if (A->val_t != dtype || B->val_t != dtype || (dtype != FGB_F64 && dtype != FGB_F32))
    return set_error(FGB_EUNSUPPORTED, "fgb_spgemm_numeric: F64 or F32 values of the given dtype");
  if (C->orient != A->orient || C->ptr_t != FGB_I64 || C->idx_t != FGB_I32 || C->val_t != dtype ||
      C->index_base != A->index_base || C->nrows != A->nrows || C->ncols != B->ncols)
    return set_error(FGB_EINVAL, "fgb_spgemm_numeric: C must be A's orientation and base, int64 ptr "
                                 "(from fgb_spgemm_symbolic), int32 idx, dtype values, shape A.nrows x B.ncols");
  if (C->nnz > 0 && (!C->idx || !C->val)) return set_error(FGB_EINVAL, "fgb_spgemm_numeric: null C buffers");
  const int fm = (flags & FGB_NO_FMA) ? FM_NOFMA : FM_FMA;
  cudaStream_t s = pick_stream(ctx, stream);
  SgScratch S;
  const size_t esz = dtype == FGB_F64 ? 8 : 4;
  rc = A->ptr_t == FGB_I32 ? sg_prepare<int32_t>(ctx, P, esz, &S, s) : sg_prepare<int64_t>(ctx, P, esz, &S, s);
  if (rc) {
    sg_release(&S, s);
    return rc;
  }
  const int64_t* cptr = (const int64_t*)C->ptr;
  int32_t* cidx = (int32_t*)C->idx;
  const int ob = C->index_base;
#define SG_NUM(T, PT) sg_launch<T, PT, false>(ctx, P, S, fm, cptr, ob, cidx, (T*)C->val, s)
  if (dtype == FGB_F64) {
    if (A->ptr_t == FGB_I32) SG_NUM(double, int32_t); else SG_NUM(double, int64_t);
  } else {
    if (A->ptr_t == FGB_I32) SG_NUM(float, int32_t); else SG_NUM(float, int64_t);
  }
#undef SG_NUM
  cudaError_t e = cudaGetLastError();
  // order the large rows' columns (keys compared with the base added: same order)
  int64_t n_big = 0;
  if (e == cudaSuccess && C->nnz > 0) e = cudaMemcpyAsync(&n_big, S.goff + P.m, 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && C->nnz > 0 && n_big > 0) {
    int64_t* seg = nullptr;  // begin offsets, then end offsets (0-based)
    int32_t* k2 = nullptr;
    void* v2 = nullptr;
    void* tmp = nullptr;
    size_t tb = 0;
    const int nseg = (int)P.m;
    const int nnz = (int)C->nnz;
    e = cudaMallocAsync((void**)&seg, 16 * (P.m + 1), s);
    int64_t* seg_end = seg + (P.m + 1);
    if (e == cudaSuccess) {
      sg_segs_k<<<grid_for(P.m, 256, ctx->num_sms), 256, 0, s>>>(P.m, S.ub, cptr, ob, seg, seg_end);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&k2, 4 * (size_t)nnz, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&v2, esz * (size_t)nnz, s);
    // the sort writes only items inside segments: the small rows keep these copies
    if (e == cudaSuccess) e = cudaMemcpyAsync(k2, cidx, 4 * (size_t)nnz, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(v2, C->val, esz * (size_t)nnz, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) {
      if (dtype == FGB_F64)
        cub::DeviceSegmentedSort::SortPairs(nullptr, tb, cidx, k2, (const double*)C->val, (double*)v2, nnz, nseg, seg, seg_end, s);
      else
        cub::DeviceSegmentedSort::SortPairs(nullptr, tb, cidx, k2, (const float*)C->val, (float*)v2, nnz, nseg, seg, seg_end, s);
      e = cudaMallocAsync(&tmp, tb ? tb : 1, s);
    }
    if (e == cudaSuccess) {
      if (dtype == FGB_F64)
        e = cub::DeviceSegmentedSort::SortPairs(tmp, tb, cidx, k2, (const double*)C->val, (double*)v2, nnz, nseg, seg, seg_end, s);
      else
        e = cub::DeviceSegmentedSort::SortPairs(tmp, tb, cidx, k2, (const float*)C->val, (float*)v2, nnz, nseg, seg, seg_end, s);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(cidx, k2, 4 * (size_t)nnz, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(const_cast<void*>(C->val), v2, esz * (size_t)nnz, cudaMemcpyDeviceToDevice, s);
    if (tmp) cudaFreeAsync(tmp, s);
    if (v2) cudaFreeAsync(v2, s);
    if (k2) cudaFreeAsync(k2, s);
    if (seg) cudaFreeAsync(seg, s);
  }
  sg_release(&S, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(FGB_ECUDA, "fgb_spgemm_numeric: %s", cudaGetErrorString(e));
  return FGB_OK;
}
