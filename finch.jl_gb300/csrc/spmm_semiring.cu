// Semiring SpMM: C[i,k] <<add>>= mul(A[i,j], B[j,k]) for the exact
// semirings (min-plus, max-plus, or-and), i.e. many semiring SpMVs over the
// columns of a dense B at once.  Replaces
// `@einsum init=-Inf R[i,j] <<max>>= P[i,k] + Q[k,j]` (the max-plus product
// of test/suites/interface_tests.jl:72-82) and its min-plus / or-and forms.
//
// CSR pull: one warp per row, lanes over the columns of B; each output is
// one fold over the row's entries in storage order.  min, max and | are
// exact and order-free, so any schedule gives Finch's result bit for bit.
#include "spmm_common.cuh"

namespace fgb {

template <int SR, class T, class VT, class PtrT>
__global__ void spmm_sr_pull_k(int64_t nrows, const PtrT* __restrict__ ptr, const int* __restrict__ idx,
                               const VT* __restrict__ val, int base, const T* __restrict__ B, int64_t ldb,
                               T* __restrict__ C, int64_t ldc, int64_t nk, int accumulate) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < nrows; i += nwarps) {
    const int64_t b = ld_ptr(ptr, i) - base, e = ld_ptr(ptr, i + 1) - base;
    for (int64_t k = lane; k < nk; k += 32) {
      T acc = accumulate ? C[i * ldc + k] : Semi<SR, T>::identity();
      for (int64_t p = b; p < e; ++p) {
        const int64_t j = (int64_t)idx[p] - base;
        const T a = val ? (T)val[p] : Semi<SR, T>::one();
        acc = Semi<SR, T>::step(acc, a, B[j * ldb + k], FM_DEFAULT);
      }
      C[i * ldc + k] = acc;
    }
  }
}

template <int SR, class T, class VT>
static int launch_sr(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk, void* C,
                     int64_t ldc, int accumulate, cudaStream_t s) {
  const int grid = grid_for(A->nrows * 32, 256, ctx->num_sms);
  if (A->ptr_t == FGB_I32)
    spmm_sr_pull_k<SR, T, VT, int32_t><<<grid, 256, 0, s>>>(A->nrows, (const int32_t*)A->ptr, (const int*)A->idx,
                                                            (const VT*)A->val, A->index_base, (const T*)B, ldb,
                                                            (T*)C, ldc, nk, accumulate);
  else
    spmm_sr_pull_k<SR, T, VT, int64_t><<<grid, 256, 0, s>>>(A->nrows, (const int64_t*)A->ptr, (const int*)A->idx,
                                                            (const VT*)A->val, A->index_base, (const T*)B, ldb,
                                                            (T*)C, ldc, nk, accumulate);
  return check_launch("spmm_sr_pull_k");
}

template <int SR>
static int dispatch_sr(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk, void* C,
                       int64_t ldc, int dtype, int accumulate, cudaStream_t s) {
  if (A->val_t != dtype)
    return set_error(FGB_EUNSUPPORTED, "fgb_spmm_semiring: values of dtype %d with operands of dtype %d",
                     A->val_t, dtype);
  switch (dtype) {
    case FGB_F64: return launch_sr<SR, double, double>(ctx, A, B, ldb, nk, C, ldc, accumulate, s);
    case FGB_F32: return launch_sr<SR, float, float>(ctx, A, B, ldb, nk, C, ldc, accumulate, s);
    case FGB_I32: return launch_sr<SR, int32_t, int32_t>(ctx, A, B, ldb, nk, C, ldc, accumulate, s);
    case FGB_I64: return launch_sr<SR, int64_t, int64_t>(ctx, A, B, ldb, nk, C, ldc, accumulate, s);
    default: return set_error(FGB_EUNSUPPORTED, "fgb_spmm_semiring: dtype %d", dtype);
  }
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_spmm_semiring(fgb_ctx* ctx, int semiring, const fgb_sparse* A, const void* B, int64_t ldb,
                                 int64_t nk, void* C, int64_t ldc, int dtype, unsigned flags, void* stream) {
  FGB_REQUIRE(ctx && A, "fgb_spmm_semiring: null argument");
  int rc = check_sparse(A, "fgb_spmm_semiring: A", true);
  if (rc) return rc;
  FGB_REQUIRE(nk >= 0 && ldb >= nk && ldc >= nk, "fgb_spmm_semiring: bad nk/ldb/ldc");
  if (semiring == FGB_PLUS_TIMES) return spmm_impl(ctx, A, B, ldb, nk, C, ldc, dtype, flags, 0, 0, stream);
  FGB_REQUIRE(A->orient == FGB_CSR, "fgb_spmm_semiring: A must be CSR");
  if (A->nrows == 0 || nk == 0) return FGB_OK;
  FGB_REQUIRE(C && (B || A->ncols == 0), "fgb_spmm_semiring: null B or C");
  cudaStream_t s = pick_stream(ctx, stream);
  const int acc = (flags & FGB_ACCUMULATE) ? 1 : 0;
  switch (semiring) {
    case FGB_MIN_PLUS: return dispatch_sr<SR_MINP>(ctx, A, B, ldb, nk, C, ldc, dtype, acc, s);
    case FGB_MAX_PLUS: return dispatch_sr<SR_MAXP>(ctx, A, B, ldb, nk, C, ldc, dtype, acc, s);
    case FGB_OR_AND:
      FGB_REQUIRE(dtype == FGB_BOOL && (A->val_t == FGB_BOOL || A->val_t == FGB_NONE),
                  "fgb_spmm_semiring: or-and needs Bool (or Pattern) A and Bool B/C");
      return launch_sr<SR_OA, uint8_t, uint8_t>(ctx, A, B, ldb, nk, C, ldc, acc, s);
    default: return set_error(FGB_EINVAL, "fgb_spmm_semiring: unknown semiring %d", semiring);
  }
}
