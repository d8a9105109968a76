// reduce(min | max, A; dims) of a SparseList matrix whatever its fill:
// maximum(A; dims) and minimum(A; dims) (src/interface/eager.jl:153-158).
//
// Finch folds every coordinate, the fill where nothing is stored.  min and
// max are idempotent, so a run of fills folds like one fill: each fiber
// folds its stored entries in coordinate order and the fill once before an
// entry that follows a gap, and once after the last entry when the fiber
// ends short of its extent.  That is the sequence of Finch's loop with its
// fill runs folded once, so the results are Finch's bit for bit, including
// the first-operand rule of @fastmath min/max for NaN and signed zeros
// (src/execute.jl:116-120).  Folding per-fiber results in fiber order gives
// the fold of the whole sequence, as "keep the first unless strictly
// smaller (larger)" is associative.
#include <limits>
#include <type_traits>

#include "fgb_internal.cuh"
#include "semiring.cuh"

namespace fgb {

// The identities of max and min, Finch's initial values: -Inf / +Inf, or
// typemin / typemax for integers.
template <class T>
static T host_lo() {
  if constexpr (std::is_floating_point_v<T>) return -std::numeric_limits<T>::infinity();
  else return std::numeric_limits<T>::min();
}
template <class T>
static T host_hi() {
  if constexpr (std::is_floating_point_v<T>) return std::numeric_limits<T>::infinity();
  else return std::numeric_limits<T>::max();
}

template <class T, bool MAX>
__device__ __forceinline__ T fold_mm(T acc, T v) {
  return MAX ? jmax(acc, v) : jmin(acc, v);
}

template <class T, bool MAX, class P>
__global__ void minmax_fiber_k(int64_t nf, const P* __restrict__ ptr, const int* __restrict__ idx,
                               const T* __restrict__ val, int base, int64_t extent, T fill, T init,
                               T* __restrict__ out) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    const int64_t lo = ld_ptr(ptr, f) - base, hi = ld_ptr(ptr, f + 1) - base;
    T acc = init;
    int64_t next = 0;  // the first coordinate not yet folded
    for (int64_t p = lo; p < hi; ++p) {
      const int64_t c = (int64_t)__ldg(idx + p) - base;
      if (c > next) acc = fold_mm<T, MAX>(acc, fill);
      acc = fold_mm<T, MAX>(acc, val[p]);
      next = c + 1;
    }
    if (next < extent) acc = fold_mm<T, MAX>(acc, fill);
    out[f] = acc;
  }
}

// out[0] = the fold of n partial results in order: each thread folds a
// contiguous run, then one thread folds the runs in thread order.
template <class T, bool MAX>
__global__ void minmax_fold_k(const T* __restrict__ part, int64_t n, T init, T* __restrict__ out) {
  __shared__ T runs[1024];
  const int64_t per = (n + blockDim.x - 1) / blockDim.x;
  const int64_t a = (int64_t)threadIdx.x * per;
  const int64_t b = a + per < n ? a + per : n;
  T acc = init;
  for (int64_t k = a; k < b; ++k) acc = fold_mm<T, MAX>(acc, part[k]);
  runs[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    T r = init;
    for (int t = 0; t < (int)blockDim.x; ++t) r = fold_mm<T, MAX>(r, runs[t]);
    out[0] = r;
  }
}

template <class T, bool MAX>
static int reduce_mm_typed(fgb_ctx* ctx, int dims, const fgb_sparse* A, const void* fill, const void* init,
                           void* y, cudaStream_t s) {
  const T f = *(const T*)fill;
  const T i0 = init ? *(const T*)init : (MAX ? host_lo<T>() : host_hi<T>());
  const int64_t nf = n_fibers(A);
  const int64_t extent = A->orient == FGB_CSC ? A->nrows : A->ncols;
  T* target = (T*)y;
  if (dims == 0) {
    if (nf == 0) {
      FGB_CUDA_TRY(cudaMemcpyAsync(y, &i0, sizeof(T), cudaMemcpyHostToDevice, s));
      FGB_CUDA_TRY(cudaStreamSynchronize(s));
      return FGB_OK;
    }
    FGB_CUDA_TRY(cudaMallocAsync((void**)&target, sizeof(T) * nf, s));
  }
  const int grid = grid_for(nf, 256, ctx->num_sms, 8);
  if (nf > 0) {
    if (A->ptr_t == FGB_I32)
      minmax_fiber_k<T, MAX, int32_t><<<grid, 256, 0, s>>>(nf, (const int32_t*)A->ptr, (const int*)A->idx,
                                                           (const T*)A->val, A->index_base, extent, f, i0, target);
    else
      minmax_fiber_k<T, MAX, int64_t><<<grid, 256, 0, s>>>(nf, (const int64_t*)A->ptr, (const int*)A->idx,
                                                           (const T*)A->val, A->index_base, extent, f, i0, target);
  }
  int rc = check_launch("fgb_reduce_minmax");
  if (rc == FGB_OK && dims == 0) {
    minmax_fold_k<T, MAX><<<1, 1024, 0, s>>>(target, nf, i0, (T*)y);
    rc = check_launch("fgb_reduce_minmax fold");
  }
  if (target != (T*)y) cudaFreeAsync(target, s);
  return rc;
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_reduce_minmax(fgb_ctx* ctx, int op, int dims, const fgb_sparse* A, const void* fill,
                                 const void* init, void* y, void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_reduce_minmax: null ctx");
  int rc = check_sparse(A, "fgb_reduce_minmax: A", true);
  if (rc) return rc;
  if (op != FGB_MAP_MIN && op != FGB_MAP_MAX)
    return set_error(FGB_EINVAL, "fgb_reduce_minmax: op must be FGB_MAP_MIN or FGB_MAP_MAX");
  if (dims < 0 || dims > 2) return set_error(FGB_EINVAL, "fgb_reduce_minmax: dims must be 0, 1 or 2");
  if (dims == 1 && A->orient != FGB_CSC)
    return set_error(FGB_EINVAL, "fgb_reduce_minmax: dims 1 (over rows) needs the CSC storage");
  if (dims == 2 && A->orient != FGB_CSR)
    return set_error(FGB_EINVAL, "fgb_reduce_minmax: dims 2 (over columns) needs the CSR storage");
  if (!fill || !y) return set_error(FGB_EINVAL, "fgb_reduce_minmax: null fill or y");
  cudaStream_t s = pick_stream(ctx, stream);
  const bool mx = op == FGB_MAP_MAX;
  switch (A->val_t) {
    case FGB_F64: return mx ? reduce_mm_typed<double, true>(ctx, dims, A, fill, init, y, s)
                            : reduce_mm_typed<double, false>(ctx, dims, A, fill, init, y, s);
    case FGB_F32: return mx ? reduce_mm_typed<float, true>(ctx, dims, A, fill, init, y, s)
                            : reduce_mm_typed<float, false>(ctx, dims, A, fill, init, y, s);
    case FGB_I64: return mx ? reduce_mm_typed<int64_t, true>(ctx, dims, A, fill, init, y, s)
                            : reduce_mm_typed<int64_t, false>(ctx, dims, A, fill, init, y, s);
    case FGB_I32: return mx ? reduce_mm_typed<int32_t, true>(ctx, dims, A, fill, init, y, s)
                            : reduce_mm_typed<int32_t, false>(ctx, dims, A, fill, init, y, s);
    default: return set_error(FGB_EUNSUPPORTED, "fgb_reduce_minmax: values must be F64, F32, I64 or I32");
  }
}
