// Conjugate gradients for SPD CSR systems with a low-precision SpMV and FP64
// everything else, the Finch-expressed solver
//
//   q = A p          @einsum q[i] += A[i,j] * p[j]
//   alpha = rr / p.q @einsum s[] += p[i] * q[i]
//   x += alpha p;  r -= alpha q;  rr' = r.r;  p = r + (rr'/rr) p
//
// run on the GPU.  The iteration SpMV reads FP32 or BF16 values (or FP64),
// converts p to FP32 per product and accumulates in FP32 (or, when asked,
// widens the values to FP64 and accumulates in FP64); x, r, p, q, the dot
// products and the updates are FP64.  A matrix whose columns lie within
// 32,767 of the diagonal is read through 16-bit column offsets j - i.  Accuracy is won back by reliable
// updates: every `replace_every` iterations, and whenever the recursive
// residual reaches the tolerance, the true residual r = b - A x is recomputed
// with the FP64 matrix and replaces the recursive one (residual replacement
// keeping the search direction), and the solve stops only when that true
// residual is below rtol * ||b||.
//
// One iteration is three kernels -- SpMV fused with the p.q partials; the r
// update (every block folds the p.q partials itself) fused with the r.r
// partials; the x and p updates fused with the folds -- so no scalar ever
// leaves the device, and p is read once by the updates.  Every partial is folded in a fixed order: the solve is
// deterministic.  A chunk of iterations is captured once in a CUDA graph and
// replayed; the host reads the residual history once per chunk.
#include <chrono>
#include <vector>

#include "fgb_internal.cuh"
#include "semiring.cuh"

namespace fgb {

constexpr int CG_THREADS = 256;
constexpr int CG_ILP = 4;  // elements per thread in flight in the streaming updates
// The updates run one block of 1024 threads per SM, each thread with CG_ILP
// elements in flight (up to 64 registers): few partials, one load per thread
// in each block's fold of the previous kernel's partials.
constexpr int CG_UPD_THREADS = 1024;

template <class T>
__device__ __forceinline__ T cg_block_sum(T v, T* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : T(0);
  if (w == 0) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
  }
  return v;  // valid in thread 0
}

// Every block folds the same partials in the same order.
__device__ __forceinline__ double fold_parts(const double* __restrict__ part, int nparts, double* sh) {
  double s = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += part[i];
  s = cg_block_sum(s, sh);
  __syncthreads();
  if (threadIdx.x == 0) sh[32] = s;
  __syncthreads();
  return sh[32];
}

template <class VT>
__device__ __forceinline__ float cg_val(const VT* v, int64_t k) {
  return to_acc<float>(v[k]);
}

// Column j of stored entry k of row i: from the int32 index, or (IX =
// int16_t) from the 16-bit offset j - i of a banded matrix's compact copy.
template <class IX>
__device__ __forceinline__ int64_t cg_col(const IX* __restrict__ ix, int64_t k, int64_t i, int base) {
  if constexpr (sizeof(IX) == 2) return i + (int64_t)__ldg(ix + k);
  else return (int64_t)__ldg(ix + k) - base;
}

// q = A p (one row per thread, j ascending) and the block partial of p.q.
// ACC = float: values converted to FP32 and p rounded to FP32 per product;
// ACC = double: values (FP64, FP32 or BF16) widened to FP64 and the products
// summed in FP64 -- with the FP64 values, the FP64 SpMV.
template <class VT, class ACC, class PtrT, class IX>
__global__ void __launch_bounds__(CG_THREADS) cg_spmv_dot(
    int64_t n, const PtrT* __restrict__ ptr, const IX* __restrict__ idx, const VT* __restrict__ val,
    int base, const double* __restrict__ p, double* __restrict__ q, double* __restrict__ part) {
  __shared__ double sh[33];
  double dot = 0.0;
  auto term = [&](int64_t k, int64_t row, ACC acc) -> ACC {
    const int64_t j = cg_col(idx, k, row, base);
    if constexpr (sizeof(ACC) == 4)
      return __fmaf_rn(cg_val(val, k), (float)__ldg(p + j), acc);
    else if constexpr (sizeof(VT) == 8)
      return __fma_rn((double)__ldg((const double*)val + k), __ldg(p + j), acc);
    else
      return __fma_rn((double)cg_val(val, k), __ldg(p + j), acc);
  };
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // two rows (i, i + stride) per thread in flight; rows and their products
  // in the plain loop's order, so q and the partial are bit-identical
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += 2 * stride) {
    const int64_t i2 = i + stride;
    const bool two = i2 < n;
    const int64_t a0 = ld_ptr(ptr, i) - base, a1 = ld_ptr(ptr, i + 1) - base;
    const int64_t b0 = two ? ld_ptr(ptr, i2) - base : 0, b1 = two ? ld_ptr(ptr, i2 + 1) - base : 0;
    ACC acc_a = ACC(0), acc_b = ACC(0);
    const int64_t la = a1 - a0, lb = b1 - b0;
    for (int64_t t = 0; t < (la > lb ? la : lb); ++t) {
      if (t < la) acc_a = term(a0 + t, i, acc_a);
      if (t < lb) acc_b = term(b0 + t, i2, acc_b);
    }
    const double qa = (double)acc_a;
    q[i] = qa;
    dot = __fma_rn(__ldg(p + i), qa, dot);
    if (two) {
      const double qb = (double)acc_b;
      q[i2] = qb;
      dot = __fma_rn(__ldg(p + i2), qb, dot);
    }
  }
  dot = cg_block_sum(dot, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = dot;
}

// The compact index of a banded matrix: off[k] = j - i for the stored
// entries of row i, and *bad set when some |j - i| does not fit 16 bits.
template <class PtrT>
__global__ void cg_offsets(int64_t n, const PtrT* __restrict__ ptr, const int* __restrict__ idx, int base,
                           int16_t* __restrict__ off, int* __restrict__ bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    for (int64_t k = ld_ptr(ptr, i) - base; k < ld_ptr(ptr, i + 1) - base; ++k) {
      const int64_t d = (int64_t)idx[k] - base - i;
      if (d < -32768 || d > 32767) {
        *bad = 1;
        off[k] = 0;
      } else {
        off[k] = (int16_t)d;
      }
    }
  }
}

// alpha = rr[slot] / (p.q);  r -= alpha q;  partials of r.r.  (x += alpha p
// waits for the p update, which reads p anyway: one pass over p less.)
__global__ void __launch_bounds__(CG_UPD_THREADS, 1) cg_update_r(
    int64_t n, double* __restrict__ r, const double* __restrict__ q, const double* __restrict__ part_pq,
    int nparts, const double* __restrict__ rr, int slot, double* __restrict__ part_rr) {
  __shared__ double sh[33];
  const double pq = fold_parts(part_pq, nparts, sh);
  // a vanished curvature (p.q == 0) only happens once r is exactly zero
  const double alpha = pq != 0.0 ? rr[slot] / pq : 0.0;
  double acc = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // CG_ILP elements per thread in flight: all loads first, then the updates
  // in the same element order as the plain loop (bit-identical partials)
  for (; i + (CG_ILP - 1) * stride < n; i += CG_ILP * stride) {
    double qv[CG_ILP], rv[CG_ILP];
#pragma unroll
    for (int u = 0; u < CG_ILP; ++u) {
      qv[u] = q[i + u * stride];
      rv[u] = r[i + u * stride];
    }
#pragma unroll
    for (int u = 0; u < CG_ILP; ++u) {
      const double ri = __fma_rn(-alpha, qv[u], rv[u]);
      r[i + u * stride] = ri;
      acc = __fma_rn(ri, ri, acc);
    }
  }
  for (; i < n; i += stride) {
    const double ri = __fma_rn(-alpha, q[i], r[i]);
    r[i] = ri;
    acc = __fma_rn(ri, ri, acc);
  }
  acc = cg_block_sum(acc, sh);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = acc;
}

// alpha as cg_update_r formed it (the same fold of the p.q partials);
// x += alpha p; rr' = fold(r.r partials); p = r + (rr' / rr[slot_in]) p;
// rr[slot_out] = rr'.  x's update is the one of the plain loop, bit for bit.
__global__ void __launch_bounds__(CG_UPD_THREADS, 1) cg_update_xp(
    int64_t n, double* __restrict__ x, const double* __restrict__ r, double* __restrict__ p,
    const double* __restrict__ part_pq, int nparts_pq, const double* __restrict__ part_rr, int nparts,
    double* __restrict__ rr, int slot_in, int slot_out, double* __restrict__ hist, int64_t it) {
  __shared__ double sh[33];
  const double pq = fold_parts(part_pq, nparts_pq, sh);
  const double alpha = pq != 0.0 ? rr[slot_in] / pq : 0.0;
  const double rr_new = fold_parts(part_rr, nparts, sh);
  const double beta = rr[slot_in] != 0.0 ? rr_new / rr[slot_in] : 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; i + (CG_ILP - 1) * stride < n; i += CG_ILP * stride) {
    double pv[CG_ILP], rv[CG_ILP], xv[CG_ILP];
#pragma unroll
    for (int u = 0; u < CG_ILP; ++u) {
      pv[u] = p[i + u * stride];
      rv[u] = r[i + u * stride];
      xv[u] = x[i + u * stride];
    }
#pragma unroll
    for (int u = 0; u < CG_ILP; ++u) {
      x[i + u * stride] = __fma_rn(alpha, pv[u], xv[u]);
      p[i + u * stride] = __fma_rn(beta, pv[u], rv[u]);
    }
  }
  for (; i < n; i += stride) {
    const double pi = p[i];
    x[i] = __fma_rn(alpha, pi, x[i]);
    p[i] = __fma_rn(beta, pi, r[i]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {  // slot_out != slot_in: no block reads it here
    rr[slot_out] = rr_new;
    hist[it] = rr_new;
  }
}

// r = b - A x (FP64) and partials of r.r (and of b.b when bb != NULL).
template <class PtrT>
__global__ void __launch_bounds__(CG_THREADS) cg_residual(
    int64_t n, const PtrT* __restrict__ ptr, const int* __restrict__ idx,
    const double* __restrict__ val, int base, const double* __restrict__ x,
    const double* __restrict__ b, double* __restrict__ r, double* __restrict__ part_rr,
    double* __restrict__ part_bb) {
  __shared__ double sh[33];
  double acc_r = 0.0, acc_b = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k0 = ld_ptr(ptr, i) - base, k1 = ld_ptr(ptr, i + 1) - base;
    double ax = 0.0;
    for (int64_t k = k0; k < k1; ++k) ax = __fma_rn(__ldg(val + k), __ldg(x + __ldg(idx + k) - base), ax);
    const double bi = b[i];
    const double ri = bi - ax;
    r[i] = ri;
    acc_r = __fma_rn(ri, ri, acc_r);
    acc_b = __fma_rn(bi, bi, acc_b);
  }
  acc_r = cg_block_sum(acc_r, sh);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = acc_r;
  if (part_bb) {
    __syncthreads();
    acc_b = cg_block_sum(acc_b, sh);
    if (threadIdx.x == 0) part_bb[blockIdx.x] = acc_b;
  }
}

// out[slot] = fold(part); optionally p = r (restart of the direction).
__global__ void __launch_bounds__(CG_THREADS) cg_fold_set(const double* __restrict__ part, int nparts,
                                                          double* __restrict__ out, int slot) {
  __shared__ double sh[33];
  const double s = fold_parts(part, nparts, sh);
  if (threadIdx.x == 0) out[slot] = s;
}

__global__ void cg_copy(int64_t n, const double* __restrict__ src, double* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

struct CgBuffers {
  double *r = nullptr, *p = nullptr, *q = nullptr, *part_a = nullptr, *part_b = nullptr,
         *part_c = nullptr, *rr = nullptr, *bb = nullptr, *hist = nullptr;
};

// The SpMV's own grid: at most `grid` blocks and no more than fit the SMs at
// once (its two rows per thread take more registers than the updates).
template <class VT, class ACC, class PtrT, class IX>
static int dot_grid_t(int grid, int sms) {
  static const int occ = [] {  // once per process (one device model); thread-safe
    int o = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, cg_spmv_dot<VT, ACC, PtrT, IX>, CG_THREADS, 0);
    return o > 0 ? o : 1;
  }();
  return std::max(1, std::min(grid, occ * sms));
}

// The iteration SpMV: value type (precision), accumulation (FP64 for the
// FP64 matrix or when asked) and index form (16-bit offsets when compact).
template <class VT, class ACC, class PtrT, class IX>
static int spmv_dot_t(const fgb_sparse* A, const IX* ix, int grid, int sms, const double* p, double* q,
                      double* part, cudaStream_t s, bool launch) {
  const int g = dot_grid_t<VT, ACC, PtrT, IX>(grid, sms);
  if (launch)
    cg_spmv_dot<VT, ACC, PtrT, IX><<<g, CG_THREADS, 0, s>>>(A->nrows, (const PtrT*)A->ptr, ix, (const VT*)A->val,
                                                           A->index_base, p, q, part);
  return g;
}

template <class PtrT, class IX>
static int spmv_dot_ix(const fgb_sparse* A, const IX* ix, int precision, bool acc64, int grid, int sms,
                       const double* p, double* q, double* part, cudaStream_t s, bool launch) {
  if (precision == FGB_F64)
    return spmv_dot_t<double, double, PtrT, IX>(A, ix, grid, sms, p, q, part, s, launch);
  if (precision == FGB_BF16)
    return acc64 ? spmv_dot_t<__nv_bfloat16, double, PtrT, IX>(A, ix, grid, sms, p, q, part, s, launch)
                 : spmv_dot_t<__nv_bfloat16, float, PtrT, IX>(A, ix, grid, sms, p, q, part, s, launch);
  return acc64 ? spmv_dot_t<float, double, PtrT, IX>(A, ix, grid, sms, p, q, part, s, launch)
               : spmv_dot_t<float, float, PtrT, IX>(A, ix, grid, sms, p, q, part, s, launch);
}

// Launches (launch = true) or sizes (false) the iteration SpMV; returns its grid.
static int spmv_dot(const fgb_sparse* A, const int16_t* off, int precision, bool acc64, int grid, int sms,
                    const double* p, double* q, double* part, cudaStream_t s, bool launch) {
  const bool i32 = A->ptr_t == FGB_I32;
  if (off)
    return i32 ? spmv_dot_ix<int32_t, int16_t>(A, off, precision, acc64, grid, sms, p, q, part, s, launch)
               : spmv_dot_ix<int64_t, int16_t>(A, off, precision, acc64, grid, sms, p, q, part, s, launch);
  const int* idx = (const int*)A->idx;
  return i32 ? spmv_dot_ix<int32_t, int>(A, idx, precision, acc64, grid, sms, p, q, part, s, launch)
             : spmv_dot_ix<int64_t, int>(A, idx, precision, acc64, grid, sms, p, q, part, s, launch);
}

template <class PtrT>
static void launch_residual(const fgb_sparse* A64, int grid, const double* x, const double* b,
                            double* r, double* part_rr, double* part_bb, cudaStream_t s) {
  cg_residual<PtrT><<<grid, CG_THREADS, 0, s>>>(A64->nrows, (const PtrT*)A64->ptr, (const int*)A64->idx,
                                                (const double*)A64->val, A64->index_base, x, b, r,
                                                part_rr, part_bb);
}

static int check_cg_matrix(const fgb_sparse* A, const char* who, int want_val) {
  int rc = check_sparse(A, who, true);
  if (rc) return rc;
  if (A->orient != FGB_CSR) return set_error(FGB_EUNSUPPORTED, "%s: CG needs a CSR matrix", who);
  if (A->nrows != A->ncols) return set_error(FGB_EINVAL, "%s: CG needs a square matrix", who);
  if (A->val_t != want_val) return set_error(FGB_EINVAL, "%s: value dtype %d, expected %d", who, A->val_t, want_val);
  return FGB_OK;
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_cg_solve(fgb_ctx* ctx, const fgb_sparse* A64, const fgb_sparse* Alow,
                            const double* b, double* x, const fgb_cg_options* opt,
                            fgb_cg_result* res, void* stream) {
  if (!ctx || !opt || !res || !b || !x) return set_error(FGB_EINVAL, "fgb_cg_solve: null argument");
  int rc = check_cg_matrix(A64, "fgb_cg_solve: A64", FGB_F64);
  if (rc) return rc;
  const int precision = opt->precision;
  if (precision != FGB_F64 && precision != FGB_F32 && precision != FGB_BF16)
    return set_error(FGB_EINVAL, "fgb_cg_solve: precision must be F64, F32 or BF16");
  const fgb_sparse* Ait = A64;
  if (precision != FGB_F64) {
    if (!Alow) return set_error(FGB_EINVAL, "fgb_cg_solve: low-precision matrix missing");
    rc = check_cg_matrix(Alow, "fgb_cg_solve: Alow", precision);
    if (rc) return rc;
    if (Alow->nrows != A64->nrows || Alow->nnz != A64->nnz)
      return set_error(FGB_EINVAL, "fgb_cg_solve: Alow and A64 differ in shape or pattern size");
    Ait = Alow;
  }
  if (opt->rtol <= 0.0 || opt->max_iter <= 0 || opt->chunk <= 0 || (opt->chunk & 1))
    return set_error(FGB_EINVAL, "fgb_cg_solve: need rtol > 0, max_iter > 0 and an even chunk > 0");
  const int64_t n = A64->nrows;
  const int chunk = opt->chunk;
  const int64_t replace_every = opt->replace_every > 0 ? opt->replace_every : 0;
  *res = fgb_cg_result{};
  if (n == 0) {
    res->converged = 1;
    return FGB_OK;
  }
  cudaStream_t user = pick_stream(ctx, stream);
  cudaStream_t s = nullptr;
  FGB_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaEvent_t ev = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  CgBuffers bufs;
  int16_t* off = nullptr;  // the compact index (16-bit column offsets), when it fits
  const bool acc64 = precision == FGB_F64 || opt->accumulate_fp64 != 0;
  int64_t hist_cap = 0;
  const int grid = grid_for(n, CG_THREADS, ctx->num_sms, 8);  // full occupancy: streaming kernels
  const bool i32 = A64->ptr_t == FGB_I32;  // ptr width of the FP64 matrix
  auto t0 = std::chrono::steady_clock::now();
  auto fail = [&](int code, const char* what, cudaError_t e) {
    rc = set_error(code, "fgb_cg_solve: %s: %s", what, cudaGetErrorString(e));
  };
  do {
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ev, user);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev, 0);
    const size_t vec = sizeof(double) * n;
    hist_cap = opt->max_iter + chunk;
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&bufs.r, vec * 3 + sizeof(double) * (3 * grid + 4 + hist_cap), s);
    if (e != cudaSuccess) { fail(FGB_ENOMEM, "setup", e); break; }
    bufs.p = bufs.r + n;
    bufs.q = bufs.p + n;
    bufs.part_a = bufs.q + n;
    bufs.part_b = bufs.part_a + grid;
    bufs.part_c = bufs.part_b + grid;
    bufs.rr = bufs.part_c + grid;  // [0], [1]: r.r slots; [2]: b.b
    bufs.hist = bufs.rr + 4;
    // r = b - A x0, rr[0] = r.r, bb = b.b, p = r
    if (i32) launch_residual<int32_t>(A64, grid, x, b, bufs.r, bufs.part_a, bufs.part_b, s);
    else launch_residual<int64_t>(A64, grid, x, b, bufs.r, bufs.part_a, bufs.part_b, s);
    cg_fold_set<<<1, CG_THREADS, 0, s>>>(bufs.part_a, grid, bufs.rr, 0);
    cg_fold_set<<<1, CG_THREADS, 0, s>>>(bufs.part_b, grid, bufs.rr, 2);
    cg_copy<<<grid, CG_THREADS, 0, s>>>(n, bufs.r, bufs.p);
    if ((e = cudaGetLastError()) != cudaSuccess) { fail(FGB_ECUDA, "setup kernels", e); break; }
    double rr_bb[3];
    if ((e = cudaMemcpyAsync(rr_bb, bufs.rr, sizeof(rr_bb), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) { fail(FGB_ECUDA, "setup sync", e); break; }
    const double bnorm = sqrt(rr_bb[2]);
    const double target = opt->rtol * (bnorm > 0 ? bnorm : 1.0);
    if (sqrt(rr_bb[0]) <= target) {
      res->converged = 1;
      res->true_rel_residual = bnorm > 0 ? sqrt(rr_bb[0]) / bnorm : 0.0;
      break;
    }
    // The compact index: 16-bit column offsets j - i when the matrix is
    // banded that tightly (built once; the int32 index otherwise).
    if (n > 0 && Ait->nnz > 0) {
      int bad = 0;
      if ((e = cudaMallocAsync((void**)&off, sizeof(int16_t) * Ait->nnz + 256, s)) != cudaSuccess) { fail(FGB_ENOMEM, "offsets", e); break; }
      int* dbad = (int*)((char*)off + ((sizeof(int16_t) * Ait->nnz + 15) & ~size_t(15)));
      cudaMemsetAsync(dbad, 0, sizeof(int), s);
      if (Ait->ptr_t == FGB_I32)
        cg_offsets<int32_t><<<grid, CG_THREADS, 0, s>>>(n, (const int32_t*)Ait->ptr, (const int*)Ait->idx, Ait->index_base, off, dbad);
      else
        cg_offsets<int64_t><<<grid, CG_THREADS, 0, s>>>(n, (const int64_t*)Ait->ptr, (const int*)Ait->idx, Ait->index_base, off, dbad);
      if ((e = cudaMemcpyAsync(&bad, dbad, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
          (e = cudaStreamSynchronize(s)) != cudaSuccess) { fail(FGB_ECUDA, "offsets", e); break; }
      if (bad) {
        cudaFreeAsync(off, s);
        off = nullptr;
      }
    }
    res->compact_index = off ? 1 : 0;
    // one chunk of iterations, captured once (slots alternate; chunk is even)
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) { fail(FGB_ECUDA, "capture", e); break; }
    const int grid_upd = grid_for(n, CG_UPD_THREADS, ctx->num_sms, 1);  // <= grid partial slots
    const int grid_dot = spmv_dot(Ait, off, precision, acc64, grid, ctx->num_sms, nullptr, nullptr, nullptr, s, false);
    for (int t = 0; t < chunk; ++t) {
      const int si = t & 1, so = si ^ 1;
      spmv_dot(Ait, off, precision, acc64, grid, ctx->num_sms, bufs.p, bufs.q, bufs.part_a, s, true);
      cg_update_r<<<grid_upd, CG_UPD_THREADS, 0, s>>>(n, bufs.r, bufs.q, bufs.part_a, grid_dot, bufs.rr, si,
                                                     bufs.part_b);
      cg_update_xp<<<grid_upd, CG_UPD_THREADS, 0, s>>>(n, x, bufs.r, bufs.p, bufs.part_a, grid_dot, bufs.part_b,
                                                      grid_upd, bufs.rr, si, so, bufs.hist, t);
    }
    e = cudaStreamEndCapture(s, &graph);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) { fail(FGB_ECUDA, "graph", e); break; }
    std::vector<double> hist(chunk);
    int64_t it = 0, since_replace = 0;
    while (it < opt->max_iter) {
      if ((e = cudaGraphLaunch(exec, s)) != cudaSuccess) { fail(FGB_ECUDA, "graph launch", e); break; }
      if ((e = cudaMemcpyAsync(hist.data(), bufs.hist, sizeof(double) * chunk, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
          (e = cudaStreamSynchronize(s)) != cudaSuccess) { fail(FGB_ECUDA, "chunk sync", e); break; }
      it += chunk;
      since_replace += chunk;
      const bool small = sqrt(hist[chunk - 1]) <= target;
      const bool broken = !(hist[chunk - 1] == hist[chunk - 1]);  // NaN: breakdown
      if (broken) { rc = set_error(FGB_EINVAL, "fgb_cg_solve: breakdown (NaN residual) after %lld iterations", (long long)it); break; }
      if (small || (replace_every && since_replace >= replace_every)) {
        // reliable update: r = b - A x in FP64 and rr[0] = r.r (slot 0 starts
        // the next chunk); the search direction is kept.  If p has vanished
        // (the recursive residual reached zero), p.q = 0 gives alpha = 0 and
        // the next update rebuilds p from the replaced residual.
        if (i32) launch_residual<int32_t>(A64, grid, x, b, bufs.r, bufs.part_a, nullptr, s);
        else launch_residual<int64_t>(A64, grid, x, b, bufs.r, bufs.part_a, nullptr, s);
        cg_fold_set<<<1, CG_THREADS, 0, s>>>(bufs.part_a, grid, bufs.rr, 0);
        double rr_true = 0;
        if ((e = cudaMemcpyAsync(&rr_true, bufs.rr, sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess) { fail(FGB_ECUDA, "replacement sync", e); break; }
        res->replacements++;
        since_replace = 0;
        // When the recursive residual has drifted far below the true one, the
        // kept direction no longer matches r: restart it from the replaced r.
        if (hist[chunk - 1] < 1e-6 * rr_true) {
          cg_copy<<<grid, CG_THREADS, 0, s>>>(n, bufs.r, bufs.p);
          if ((e = cudaGetLastError()) != cudaSuccess) { fail(FGB_ECUDA, "restart", e); break; }
        }
        res->true_rel_residual = sqrt(rr_true) / (bnorm > 0 ? bnorm : 1.0);
        if (sqrt(rr_true) <= target) {
          res->converged = 1;
          break;
        }
      }
    }
    res->iterations = it;
  } while (0);
  if (rc == FGB_OK && !res->converged && res->iterations >= opt->max_iter) {
    // report the true residual reached
    if (i32) launch_residual<int32_t>(A64, grid, x, b, bufs.r, bufs.part_a, nullptr, s);
    else launch_residual<int64_t>(A64, grid, x, b, bufs.r, bufs.part_a, nullptr, s);
    cg_fold_set<<<1, CG_THREADS, 0, s>>>(bufs.part_a, grid, bufs.rr, 0);
    double rr_true = 0, bb = 0;
    cudaMemcpyAsync(&rr_true, bufs.rr, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&bb, bufs.rr + 2, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    res->true_rel_residual = sqrt(rr_true) / (bb > 0 ? sqrt(bb) : 1.0);
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (bufs.r) cudaFreeAsync(bufs.r, s);
  if (off) cudaFreeAsync(off, s);
  // the caller's stream waits for the solve
  if (ev) {
    cudaEventRecord(ev, s);
    cudaStreamWaitEvent(user, ev, 0);
  }
  cudaStreamSynchronize(s);
  if (ev) cudaEventDestroy(ev);
  cudaStreamDestroy(s);
  res->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}
