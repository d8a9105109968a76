// SpMM: C[i,k] += A[i,j] * B[j,k] over a SparseList matrix A and a
// row-major dense B (k fastest).
//
// CSR (pull).  A group of G lanes owns one row i and a column slab
// [c0, c0 + G*V) of C; each lane holds V consecutive k in registers.  The
// group walks the row's stored entries in order, G at a time: every lane
// loads one (j, a) pair with a coalesced streaming load, then the pairs are
// broadcast by shuffles and each lane gathers its V-wide piece of B[j, :]
// (one 16-byte load for fp32) and updates its accumulators.  Every C[i,k] is
// therefore one running sum over j ascending -- Finch's serial order -- and
// the results equal Finch's CPU nest for the same contraction choice.
//
// When B does not fit in L2 the columns are processed as slabs (one launch
// per slab, slab width G*V): the rows of a slab of B are gathered from L2
// while A's idx/val stream through with evict-first hints.
//
// CSC (push).  A group owns column j of A (row j of B) and adds a*B[j, :]
// into C[i, :] with atomics.
#include "fgb_internal.cuh"
#include "semiring.cuh"
#include "spmm_common.cuh"

namespace fgb {

// One launch = one column slab [c0, c0 + G*V) (clipped to nk) of every row.
template <class T, class VT, class PtrT, int G, int V>
__global__ void __launch_bounds__(256) spmm_csr_pull(
    int64_t nrows, const PtrT* __restrict__ ptr, const int* __restrict__ idx,
    const VT* __restrict__ val, const T* __restrict__ B, int64_t ldb, T* __restrict__ C,
    int64_t ldc, int64_t c0, int64_t nk, int base, int accumulate, int fm) {
  constexpr int BATCH = 8;
  const int lane = threadIdx.x & (G - 1);
  const unsigned gmask =
      G == 32 ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
  const int64_t group = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
  const int64_t col = c0 + (int64_t)lane * V;
  const bool active_col = col < nk;  // V divides nk - c0 in the vector path
  const uint64_t pol_stream = policy_evict_first();
  const uint64_t pol_keep = policy_evict_last();
  for (int64_t row = group; row < nrows; row += ngroups) {
    const int64_t p0 = ld_ptr(ptr, row) - base;
    const int64_t p1 = ld_ptr(ptr, row + 1) - base;
    VecT<T, V> acc;
    if (accumulate && active_col)
      acc = load_out<T, V>(C + row * ldc + col);
    else
#pragma unroll
      for (int q = 0; q < V; ++q) acc.v[q] = T(0);
    for (int64_t pb = p0; pb < p1; pb += G) {
      const int64_t pe = pb + lane;
      int my_j = 0;
      T my_a = T(0);
      if (pe < p1) {
        my_j = ld_stream_i32(idx + pe, pol_stream) - base;
        my_a = load_val<T, VT>(val, pe, pol_stream);
      }
      const int cnt = (p1 - pb) < (int64_t)G ? (int)(p1 - pb) : G;
#pragma unroll
      for (int t0 = 0; t0 < G; t0 += BATCH) {
        if (t0 >= cnt) break;
        VecT<T, V> b[BATCH];
        T a[BATCH];
#pragma unroll
        for (int t = 0; t < BATCH; ++t) {
          const int src = t0 + t < G ? t0 + t : 0;
          const int j = __shfl_sync(gmask, my_j, src, G);
          a[t] = __shfl_sync(gmask, my_a, src, G);
          if (t0 + t < cnt && active_col)
            b[t] = gather<T, V>(B + (int64_t)j * ldb + col, pol_keep);
        }
#pragma unroll
        for (int t = 0; t < BATCH; ++t)
          if (t0 + t < cnt && active_col) acc_step<T, V>(acc, a[t], b[t], fm);
      }
    }
    if (active_col) store_out<T, V>(C + row * ldc + col, acc, pol_stream);
  }
}

template <class T, class VT, class PtrT>
__global__ void __launch_bounds__(256) spmm_csc_push(int64_t ncols_a, const PtrT* __restrict__ ptr,
                                                     const int* __restrict__ idx,
                                                     const VT* __restrict__ val,
                                                     const T* __restrict__ B, int64_t ldb,
                                                     T* __restrict__ C, int64_t ldc, int64_t nk,
                                                     int base) {
  // one warp per column j of A; lanes stride over k
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t j = w; j < ncols_a; j += nw) {
    const int64_t p0 = ld_ptr(ptr, j) - base, p1 = ld_ptr(ptr, j + 1) - base;
    for (int64_t p = p0; p < p1; ++p) {
      const int i = __ldg(idx + p) - base;
      const T a = to_acc<T>(__ldg(val + p));
      for (int64_t k = lane; k < nk; k += 32) atomicAdd(C + (int64_t)i * ldc + k, a * __ldg(B + j * ldb + k));
    }
  }
}

template <class T>
__global__ void zero_rows(T* C, int64_t m, int64_t nk, int64_t ldc) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m * nk;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / nk, k = e - i * nk;
    C[i * ldc + k] = T(0);
  }
}

template <class T, class VT, class PtrT, int G, int V>
static int launch_pull(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk,
                       void* C, int64_t ldc, int accumulate, int fm, cudaStream_t s) {
  const int64_t m = A->nrows;
  const int64_t slab = (int64_t)G * V;
  const int threads = 256;
  const int grid = grid_for(m * G, threads, ctx->num_sms, 8);
  for (int64_t c0 = 0; c0 < nk; c0 += slab) {
    spmm_csr_pull<T, VT, PtrT, G, V><<<grid, threads, 0, s>>>(
        m, (const PtrT*)A->ptr, (const int*)A->idx, (const VT*)A->val, (const T*)B, ldb, (T*)C,
        ldc, c0, nk, A->index_base, accumulate, fm);
    int rc = check_launch("spmm_csr_pull");
    if (rc) return rc;
  }
  return FGB_OK;
}

// Slab width in lanes: the whole of nk when it fits one warp, else the
// widest group that keeps the gathered slab of B near L2 capacity.
template <class T, class VT, class PtrT>
static int dispatch_pull(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk,
                         void* C, int64_t ldc, int accumulate, int fm, int lanes, cudaStream_t s) {
  constexpr int VN = sizeof(T) == 4 ? 4 : 2;
  const bool vec_ok = (nk % VN == 0) && (ldb % VN == 0) && (ldc % VN == 0) &&
                      ((uintptr_t)B % (VN * sizeof(T)) == 0) && ((uintptr_t)C % (VN * sizeof(T)) == 0);
  if (vec_ok) {
    switch (lanes) {
      case 4: return launch_pull<T, VT, PtrT, 4, VN>(ctx, A, B, ldb, nk, C, ldc, accumulate, fm, s);
      case 8: return launch_pull<T, VT, PtrT, 8, VN>(ctx, A, B, ldb, nk, C, ldc, accumulate, fm, s);
      case 16: return launch_pull<T, VT, PtrT, 16, VN>(ctx, A, B, ldb, nk, C, ldc, accumulate, fm, s);
      default: return launch_pull<T, VT, PtrT, 32, VN>(ctx, A, B, ldb, nk, C, ldc, accumulate, fm, s);
    }
  }
  switch (lanes) {
    case 4: return launch_pull<T, VT, PtrT, 4, 1>(ctx, A, B, ldb, nk, C, ldc, accumulate, fm, s);
    case 8: return launch_pull<T, VT, PtrT, 8, 1>(ctx, A, B, ldb, nk, C, ldc, accumulate, fm, s);
    case 16: return launch_pull<T, VT, PtrT, 16, 1>(ctx, A, B, ldb, nk, C, ldc, accumulate, fm, s);
    default: return launch_pull<T, VT, PtrT, 32, 1>(ctx, A, B, ldb, nk, C, ldc, accumulate, fm, s);
  }
}

static int default_lanes(int64_t nk, int vn, int64_t b_bytes) {
  // lanes needed to cover nk in one slab
  int64_t need = (nk + vn - 1) / vn;
  int lanes = need <= 4 ? 4 : need <= 8 ? 8 : need <= 16 ? 16 : 32;
  (void)b_bytes;
  return lanes;
}

// Default merge-path tuning: lanes enough for all of nk (up to 32, i.e.
// whole 512-byte rows of fp32 B per gather), items of 256 path steps.
// Narrower column slabs do not shrink B's L2 footprint on row-major B --
// a 64-byte slice still occupies a whole 128-byte line -- and they re-read
// A once per slab: on the 1M x 1M Zipf matrix with k = 128, 4 lanes (16
// columns) take 6.0 ms and 32 lanes 2.1 ms.
static void default_merge_tuning(const fgb_sparse* A, int64_t nk, size_t esz, int* lanes,
                                 int64_t* path) {
  (void)A;
  const int vn = esz == 4 ? 4 : 2;
  const int64_t need = (nk + vn - 1) / vn;
  int l = 4;
  while (l < need && l < 32) l *= 2;
  if (*lanes <= 0) *lanes = l;
  if (*path <= 0) *path = 256;
}

template <class T, class VT>
static int run_typed(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk,
                     void* C, int64_t ldc, unsigned flags, int lanes, int64_t path,
                     cudaStream_t s, int variant) {
  const int accumulate = (flags & FGB_ACCUMULATE) ? 1 : 0;
  int fm = FM_DEFAULT;
  if (flags & FGB_NO_FMA) fm = FM_NOFMA;
  if (flags & FGB_FMA) fm = FM_FMA;
  if (A->orient == FGB_CSR) {
    if (A->nrows == 0 || nk == 0) return FGB_OK;
    constexpr int VN = sizeof(T) == 4 ? 4 : 2;
    const bool vec_ok = (nk % VN == 0) && (ldb % VN == 0) && (ldc % VN == 0) &&
                        ((uintptr_t)B % (VN * sizeof(T)) == 0) &&
                        ((uintptr_t)C % (VN * sizeof(T)) == 0);
    if (!(flags & FGB_FINCH_ORDER) && vec_ok) {
      default_merge_tuning(A, nk, sizeof(T), &lanes, &path);
      return spmm_merge(ctx, A, B, ldb, nk, C, ldc, sizeof(T) == 8 ? FGB_F64 : FGB_F32,
                        accumulate, lanes, path, nullptr, 0, s, false, nullptr, variant);
    }
    if (lanes <= 0) lanes = default_lanes(nk, sizeof(T) == 4 ? 4 : 2, A->ncols * nk * (int64_t)sizeof(T));
    if (A->ptr_t == FGB_I32)
      return dispatch_pull<T, VT, int32_t>(ctx, A, B, ldb, nk, C, ldc, accumulate, fm, lanes, s);
    return dispatch_pull<T, VT, int64_t>(ctx, A, B, ldb, nk, C, ldc, accumulate, fm, lanes, s);
  }
  if (flags & FGB_FINCH_ORDER)
    return set_error(FGB_EUNSUPPORTED, "fgb_spmm: FGB_FINCH_ORDER needs a CSR matrix");
  if (A->nrows == 0 || nk == 0) return FGB_OK;
  const int threads = 256;
  if (!accumulate) {
    zero_rows<T><<<grid_for(A->nrows * nk, threads, ctx->num_sms, 4), threads, 0, s>>>((T*)C, A->nrows, nk, ldc);
    int rc = check_launch("zero_rows");
    if (rc) return rc;
  }
  const int grid = grid_for(A->ncols * 32, threads, ctx->num_sms, 8);
  if (A->ptr_t == FGB_I32)
    spmm_csc_push<T, VT, int32_t><<<grid, threads, 0, s>>>(A->ncols, (const int32_t*)A->ptr, (const int*)A->idx,
                                                          (const VT*)A->val, (const T*)B, ldb, (T*)C, ldc, nk, A->index_base);
  else
    spmm_csc_push<T, VT, int64_t><<<grid, threads, 0, s>>>(A->ncols, (const int64_t*)A->ptr, (const int*)A->idx,
                                                          (const VT*)A->val, (const T*)B, ldb, (T*)C, ldc, nk, A->index_base);
  return check_launch("spmm_csc_push");
}

int spmm_impl(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk, void* C,
              int64_t ldc, int dtype, unsigned flags, int lanes, int64_t path, void* stream,
              int variant, int bands) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_spmm: null ctx");
  int rc = check_sparse(A, "fgb_spmm: A", true);
  if (rc) return rc;
  if (nk < 0 || ldb < nk || ldc < nk) return set_error(FGB_EINVAL, "fgb_spmm: bad nk/ldb/ldc");
  if ((A->ncols > 0 && nk > 0 && !B) || (A->nrows > 0 && nk > 0 && !C))
    return set_error(FGB_EINVAL, "fgb_spmm: null B or C");
  cudaStream_t s = pick_stream(ctx, stream);
  // No schedule given: a B far larger than L2 with many stored entries takes
  // the virtual-row slab schedule with cp.async gathers (32-column slabs,
  // 256-entry virtual rows, two column bands; on the 1M x 1M Zipf matrix with
  // k = 128, 1.38 ms per call with its schedule built, against 1.40 ms with
  // 128-entry rows, 1.48 ms without bands and 2.1 ms for the best merge path).
  if (variant == 0 && lanes <= 0 && path <= 0 && A->orient == FGB_CSR && dtype == FGB_F32 &&
      A->val_t == FGB_F32 && A->idx_t == FGB_I32 && !(flags & FGB_FINCH_ORDER) && nk >= 32 && nk % 4 == 0 &&
      ldb % 4 == 0 && ldc % 4 == 0 && ldb <= INT32_MAX && (uintptr_t)B % 16 == 0 && (uintptr_t)C % 16 == 0 &&
      A->nrows <= INT32_MAX && A->nnz >= (1 << 20) && A->nnz <= INT32_MAX &&
      (double)A->ncols * (double)nk * 4.0 > 64.0 * 1024 * 1024 && !stream_capturing(s)) {
    variant = 3;
    lanes = 8;
    path = 256;
    bands = 2;
  }
  if (variant == 2 || variant == 3) {  // virtual-row column slabs: schedule built for this call
    if (A->orient != FGB_CSR || dtype != FGB_F32 || (flags & FGB_FINCH_ORDER))
      return set_error(FGB_EUNSUPPORTED, "fgb_spmm: variants 2 and 3 need CSR, F32 and no FGB_FINCH_ORDER");
    if (A->nrows == 0 || nk == 0) return FGB_OK;
    // the schedule and partial sums come from the stream-ordered pool and go
    // back to it behind the launches (no device-wide synchronisation)
    VrowSchedule v;
    rc = vrow_build(ctx, A, path > 0 ? (int)std::min<int64_t>(path, 4096) : 64, &v, s, true,
                    bands > 1 ? bands : 1);
    if (rc) return rc;
    void* part = nullptr;
    const int slab = 4 * (lanes > 0 ? lanes : 4);
    const size_t pb = spmm_vrow_scratch_bytes(v, nk);
    if (pb && cudaMallocAsync(&part, pb, s) != cudaSuccess) {
      vrow_free(&v, s);
      return set_error(FGB_ENOMEM, "fgb_spmm: partial sums (%zu bytes)", pb);
    }
    rc = spmm_vrow(ctx, v, A, B, ldb, nk, C, ldc, (flags & FGB_ACCUMULATE) ? 1 : 0, slab, part, s,
                   variant == 3);
    if (part) cudaFreeAsync(part, s);
    vrow_free(&v, s);
    return rc;
  }
  if (dtype == FGB_F32) {
    if (A->val_t == FGB_F32) return run_typed<float, float>(ctx, A, B, ldb, nk, C, ldc, flags, lanes, path, s, variant);
    if (A->val_t == FGB_BF16)
      return run_typed<float, __nv_bfloat16>(ctx, A, B, ldb, nk, C, ldc, flags, lanes, path, s, variant);
  } else if (dtype == FGB_F64) {
    if (A->val_t == FGB_F64) return run_typed<double, double>(ctx, A, B, ldb, nk, C, ldc, flags, lanes, path, s, variant);
  }
  return set_error(FGB_EUNSUPPORTED, "fgb_spmm: no kernel for val %d / dtype %d", A->val_t, dtype);
}

}  // namespace fgb

extern "C" int fgb_spmm(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk,
                        void* C, int64_t ldc, int dtype, unsigned flags, void* stream) {
  return fgb::spmm_impl(ctx, A, B, ldb, nk, C, ldc, dtype, flags, 0, 0, stream);
}

extern "C" int fgb_spmm_ex(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb,
                           int64_t nk, void* C, int64_t ldc, int dtype, unsigned flags,
                           const fgb_spmm_tuning* tune, void* stream) {
  int lanes = tune ? tune->lanes : 0;
  int64_t path = tune ? tune->path : 0;
  const int variant = tune ? tune->variant : 0;
  const int bands = tune ? tune->bands : 0;
  if (variant < 0 || variant > 3) return fgb::set_error(FGB_EINVAL, "fgb_spmm_ex: variant must be 0, 1, 2 or 3");
  if (bands < 0 || bands > 8) return fgb::set_error(FGB_EINVAL, "fgb_spmm_ex: bands must be in [0, 8]");
  if (bands > 1 && variant < 2)
    return fgb::set_error(FGB_EINVAL, "fgb_spmm_ex: column bands need variant 2 or 3");
  if (variant >= 2 && lanes != 0 && lanes != 2 && lanes != 4 && lanes != 8)
    return fgb::set_error(FGB_EINVAL, "fgb_spmm_ex: variants 2 and 3 take lanes 2, 4 or 8");
  if (lanes != 0 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32)
    return fgb::set_error(FGB_EINVAL, "fgb_spmm_ex: lanes must be 0, 2, 4, 8, 16 or 32");
  if (path < 0) return fgb::set_error(FGB_EINVAL, "fgb_spmm_ex: negative path");
  return fgb::spmm_impl(ctx, A, B, ldb, nk, C, ldc, dtype, flags, lanes, path, stream, variant, bands);
}
