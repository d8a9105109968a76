// SpGEMM with a dense output: C = A * B (plus-times) for two sparse
// operands whose product is dense-ish, written into a dense row-major C --
// the format Galley picks for an output whose estimated density passes one
// half (src/Galley/PhysicalOptimizer/format-selector.jl:27-65).
//
// Gustavson's nest as docs/examples/spgemm.jl:56-72 writes it: one warp per
// output fiber walks that fiber's entries of the left operand in order (k
// ascending) and, for each, spreads the lanes over the right operand's
// fiber k; every output element therefore sums its products in the order of
// k, fused unless FGB_NO_FMA -- the sums of fgb_spgemm_numeric, so the
// stored values equal the sparse product's bit for bit.  Lanes of one k
// touch distinct outputs; __syncwarp orders successive k.
#include "fgb_internal.cuh"
#include "semiring.cuh"

namespace fgb {

// CSR: fiber i of A (row), B's rows k; C[i, j].  CSC: fiber j of B
// (column), A's columns k; C[i, j].  `outer` is the operand whose fibers the
// warps take, `inner` the one gathered per k (each with its own ptr type and
// index base).
template <class T, class PO, class PI>
__global__ void spgemm_dense_k(int64_t nf, const PO* __restrict__ op_, const int* __restrict__ oi,
                               const T* __restrict__ ov, int obase, const PI* __restrict__ ip,
                               const int* __restrict__ ii, const T* __restrict__ iv, int ibase, int csc,
                               T* __restrict__ C, int64_t ldc, int64_t nout, int fm) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t f = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; f < nf; f += nwarps) {
    // zero the fiber of C: row f (CSR) or column f (CSC)
    for (int64_t t = lane; t < nout; t += 32) C[csc ? t * ldc + f : f * ldc + t] = T(0);
    __syncwarp();
    for (int64_t p = ld_ptr(op_, f) - obase; p < ld_ptr(op_, f + 1) - obase; ++p) {
      const int64_t k = (int64_t)oi[p] - obase;
      const T a = ov[p];
      for (int64_t q = ld_ptr(ip, k) - ibase + lane; q < ld_ptr(ip, k + 1) - ibase; q += 32) {
        const int64_t t = (int64_t)ii[q] - ibase;
        T* c = C + (csc ? t * ldc + f : f * ldc + t);
        *c = fm == FM_NOFMA ? Semi<SR_PT, T>::add(*c, Semi<SR_PT, T>::mul(iv[q], a)) : fused(a, iv[q], *c);
      }
      __syncwarp();
    }
  }
}

template <class T, class PO, class PI>
static int spgemm_dense_t(fgb_ctx* ctx, const fgb_sparse* O, const fgb_sparse* I, int64_t nf, int64_t nout,
                          bool csc, int fm, T* C, int64_t ldc, cudaStream_t s) {
  spgemm_dense_k<T, PO, PI><<<grid_for(nf * 32, 256, ctx->num_sms), 256, 0, s>>>(
      nf, (const PO*)O->ptr, (const int*)O->idx, (const T*)O->val, O->index_base, (const PI*)I->ptr,
      (const int*)I->idx, (const T*)I->val, I->index_base, csc ? 1 : 0, C, ldc, nout, fm);
  return check_launch("spgemm_dense_k");
}

template <class T>
static int spgemm_dense_d(fgb_ctx* ctx, const fgb_sparse* A, const fgb_sparse* B, int fm, T* C, int64_t ldc,
                          cudaStream_t s) {
  const bool csc = A->orient == FGB_CSC;
  const fgb_sparse* O = csc ? B : A;  // the operand whose fibers are the output's
  const fgb_sparse* I = csc ? A : B;
  const int64_t nf = csc ? B->ncols : A->nrows;
  const int64_t nout = csc ? A->nrows : B->ncols;
  const bool o32 = O->ptr_t == FGB_I32, i32 = I->ptr_t == FGB_I32;
  if (o32 && i32) return spgemm_dense_t<T, int32_t, int32_t>(ctx, O, I, nf, nout, csc, fm, C, ldc, s);
  if (o32) return spgemm_dense_t<T, int32_t, int64_t>(ctx, O, I, nf, nout, csc, fm, C, ldc, s);
  if (i32) return spgemm_dense_t<T, int64_t, int32_t>(ctx, O, I, nf, nout, csc, fm, C, ldc, s);
  return spgemm_dense_t<T, int64_t, int64_t>(ctx, O, I, nf, nout, csc, fm, C, ldc, s);
}

}  // namespace fgb

extern "C" int fgb_spgemm_dense(fgb_ctx* ctx, const fgb_sparse* A, const fgb_sparse* B, int dtype, unsigned flags,
                                void* C, int64_t ldc, void* stream) {
  using namespace fgb;
  FGB_REQUIRE(ctx && A && B, "fgb_spgemm_dense: null argument");
  int rc = check_sparse(A, "fgb_spgemm_dense: A", true);
  if (!rc) rc = check_sparse(B, "fgb_spgemm_dense: B", true);
  if (rc) return rc;
  FGB_REQUIRE(A->orient == B->orient, "fgb_spgemm_dense: A and B must share an orientation");
  FGB_REQUIRE(A->ncols == B->nrows, "fgb_spgemm_dense: inner dimensions %lld and %lld differ",
              (long long)A->ncols, (long long)B->nrows);
  FGB_REQUIRE(ldc >= B->ncols, "fgb_spgemm_dense: leading dimension below the column count");
  if (A->val_t != dtype || B->val_t != dtype || (dtype != FGB_F64 && dtype != FGB_F32))
    return set_error(FGB_EUNSUPPORTED, "fgb_spgemm_dense: F64 or F32 values of the given dtype");
  if (A->nrows == 0 || B->ncols == 0) return FGB_OK;
  FGB_REQUIRE(C, "fgb_spgemm_dense: null C");
  const int fm = (flags & FGB_NO_FMA) ? FM_NOFMA : FM_FMA;
  cudaStream_t s = pick_stream(ctx, stream);
  if (dtype == FGB_F64) return spgemm_dense_d<double>(ctx, A, B, fm, (double*)C, ldc, s);
  return spgemm_dense_d<float>(ctx, A, B, fm, (float*)C, ldc, s);
}
