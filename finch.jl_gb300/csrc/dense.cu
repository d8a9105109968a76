// Dense-vector operations of Finch programs over Dense(Element) levels:
// the dot products, updates and pointwise maps that surround the sparse
// kernels in iterative solvers and graph relaxations (CG's
// `@einsum s[] += p[i]*q[i]`, `x[i] = x[i] + alpha[]*p[i]`, Bellman-Ford's
// `x = min.(x, y)`).  Scalars (Finch's 0-d Scalar, src/tensors/scalars.jl)
// live in device memory, so a chain of these calls never waits on the host.
//
// The dot product is deterministic: every block writes one partial in a
// fixed tree order, and one block folds the partials in index order.
#include "fgb_internal.cuh"
#include "semiring.cuh"

namespace fgb {

constexpr int DOT_THREADS = 512;
constexpr int DOT_MAX_BLOCKS = 1024;

template <class T>
__device__ __forceinline__ T block_sum(T v, T* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < (int)(blockDim.x >> 5) ? sh[lane] : T(0);
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
  }
  return v;
}

template <class T>
__global__ void __launch_bounds__(DOT_THREADS) dot_partials(int64_t n, const T* __restrict__ x,
                                                            const T* __restrict__ y,
                                                            T* __restrict__ part) {
  __shared__ T sh[32];
  T acc = T(0);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    acc = fused(x[i], y[i], acc);
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

template <class T>
__global__ void __launch_bounds__(DOT_THREADS) dot_fold(const T* __restrict__ part, int nparts,
                                                        T* __restrict__ out) {
  __shared__ T sh[32];
  T acc = T(0);
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += part[i];
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) out[0] = acc;
}

// out = alpha*x + beta with alpha/beta device scalars (NULL: 1 and 0), or
// out = beta with x NULL; fused (one rounding), like the Finch-order SpMV
// and axpby around it.
template <class T>
__global__ void affine_k(int64_t n, const T* __restrict__ alpha, const T* __restrict__ x,
                         const T* __restrict__ beta, T* __restrict__ out) {
  const T a = alpha ? alpha[0] : T(1);
  const T b = beta ? beta[0] : T(0);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = x ? fused(a, x[i], b) : b;
}

// out = alpha*x + beta*y with alpha/beta device scalars (NULL means 1),
// optional negation of each term (sign bits: 1 = -alpha, 2 = -beta).
template <class T>
__global__ void axpby_k(int64_t n, const T* __restrict__ alpha, const T* __restrict__ x,
                        const T* __restrict__ beta, const T* __restrict__ y, T* __restrict__ out,
                        int signs) {
  T a = alpha ? alpha[0] : T(1);
  T b = beta ? beta[0] : T(1);
  if (signs & 1) a = -a;
  if (signs & 2) b = -b;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T yv = y ? y[i] : T(0);
    out[i] = fused(a, x[i], wmul(b, yv));
  }
}

template <class T>
__global__ void map2_k(int op, int64_t n, const T* __restrict__ x, const T* __restrict__ y,
                       T* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T a = x[i], b = y[i];
    T r;
    switch (op) {
      case FGB_MAP_ADD: r = wadd(a, b); break;
      case FGB_MAP_SUB: r = wadd(a, T(0) - b); break;
      case FGB_MAP_MUL: r = wmul(a, b); break;
      case FGB_MAP_MIN: r = jmin(a, b); break;
      case FGB_MAP_MAX: r = jmax(a, b); break;
      default: r = a; break;
    }
    out[i] = r;
  }
}

// scalar ops on 0-d device values: out = op(a, b)
template <class T>
__global__ void scalar_k(int op, const T* a, const T* b, T* out) {
  const T x = a[0], y = b ? b[0] : T(0);
  T r;
  switch (op) {
    case FGB_MAP_ADD: r = x + y; break;
    case FGB_MAP_SUB: r = x - y; break;
    case FGB_MAP_MUL: r = x * y; break;
    case FGB_MAP_DIV: r = x / y; break;
    case FGB_MAP_MIN: r = jmin(x, y); break;
    case FGB_MAP_MAX: r = jmax(x, y); break;
    default: r = x; break;
  }
  out[0] = r;
}

template <class T>
__global__ void convert_k(int64_t n, const T* __restrict__ x, float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)x[i];
}

template <class T>
static int dot_typed(fgb_ctx* ctx, int64_t n, const T* x, const T* y, T* out, T* scratch,
                     int scratch_cap, cudaStream_t s) {
  const int blocks = grid_for(n, DOT_THREADS, ctx->num_sms, 4) < scratch_cap
                         ? grid_for(n, DOT_THREADS, ctx->num_sms, 4)
                         : scratch_cap;
  dot_partials<T><<<blocks, DOT_THREADS, 0, s>>>(n, x, y, scratch);
  dot_fold<T><<<1, DOT_THREADS, 0, s>>>(scratch, blocks, out);
  return check_launch("fgb_dense_dot");
}

int dense_dot_impl(fgb_ctx* ctx, int dtype, int64_t n, const void* x, const void* y, void* out,
                   void* scratch, int scratch_cap, cudaStream_t s) {
  if (dtype == FGB_F64)
    return dot_typed<double>(ctx, n, (const double*)x, (const double*)y, (double*)out,
                             (double*)scratch, scratch_cap, s);
  return dot_typed<float>(ctx, n, (const float*)x, (const float*)y, (float*)out, (float*)scratch,
                          scratch_cap, s);
}

}  // namespace fgb

using namespace fgb;

extern "C" {

int fgb_dense_dot(fgb_ctx* ctx, int dtype, int64_t n, const void* x, const void* y, void* out,
                  void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_dense_dot: null ctx");
  if (dtype != FGB_F64 && dtype != FGB_F32) return set_error(FGB_EUNSUPPORTED, "fgb_dense_dot: dtype %d", dtype);
  if (n < 0 || (n > 0 && (!x || !y)) || !out) return set_error(FGB_EINVAL, "fgb_dense_dot: bad argument");
  cudaStream_t s = pick_stream(ctx, stream);
  void* part = nullptr;
  FGB_CUDA_TRY(cudaMallocAsync(&part, DOT_MAX_BLOCKS * 8, s));
  int rc = dense_dot_impl(ctx, dtype, n, x, y, out, part, DOT_MAX_BLOCKS, s);
  cudaFreeAsync(part, s);
  return rc;
}

int fgb_dense_axpby(fgb_ctx* ctx, int dtype, int64_t n, const void* alpha, const void* x,
                    const void* beta, const void* y, void* out, int signs, void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_dense_axpby: null ctx");
  if (n < 0 || (n > 0 && (!x || !out))) return set_error(FGB_EINVAL, "fgb_dense_axpby: bad argument");
  if (n == 0) return FGB_OK;
  cudaStream_t s = pick_stream(ctx, stream);
  const int grid = grid_for(n, 256, ctx->num_sms, 8);
  if (dtype == FGB_F64)
    axpby_k<double><<<grid, 256, 0, s>>>(n, (const double*)alpha, (const double*)x,
                                         (const double*)beta, (const double*)y, (double*)out, signs);
  else if (dtype == FGB_F32)
    axpby_k<float><<<grid, 256, 0, s>>>(n, (const float*)alpha, (const float*)x,
                                        (const float*)beta, (const float*)y, (float*)out, signs);
  else
    return set_error(FGB_EUNSUPPORTED, "fgb_dense_axpby: dtype %d", dtype);
  return check_launch("fgb_dense_axpby");
}

int fgb_dense_affine(fgb_ctx* ctx, int dtype, int64_t n, const void* alpha, const void* x,
                     const void* beta, void* out, void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_dense_affine: null ctx");
  if (n < 0 || (n > 0 && !out)) return set_error(FGB_EINVAL, "fgb_dense_affine: bad argument");
  if (n == 0) return FGB_OK;
  cudaStream_t s = pick_stream(ctx, stream);
  const int grid = grid_for(n, 256, ctx->num_sms, 8);
  if (dtype == FGB_F64)
    affine_k<double><<<grid, 256, 0, s>>>(n, (const double*)alpha, (const double*)x, (const double*)beta,
                                          (double*)out);
  else if (dtype == FGB_F32)
    affine_k<float><<<grid, 256, 0, s>>>(n, (const float*)alpha, (const float*)x, (const float*)beta,
                                         (float*)out);
  else
    return set_error(FGB_EUNSUPPORTED, "fgb_dense_affine: dtype %d", dtype);
  return check_launch("fgb_dense_affine");
}

int fgb_dense_map(fgb_ctx* ctx, int op, int dtype, int64_t n, const void* x, const void* y,
                  void* out, void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_dense_map: null ctx");
  if (op < FGB_MAP_ADD || op > FGB_MAP_MAX || op == FGB_MAP_DIV)
    return set_error(FGB_EINVAL, "fgb_dense_map: bad op %d", op);
  if (n < 0 || (n > 0 && (!x || !y || !out))) return set_error(FGB_EINVAL, "fgb_dense_map: bad argument");
  if (n == 0) return FGB_OK;
  cudaStream_t s = pick_stream(ctx, stream);
  const int grid = grid_for(n, 256, ctx->num_sms, 8);
  switch (dtype) {
    case FGB_F64: map2_k<double><<<grid, 256, 0, s>>>(op, n, (const double*)x, (const double*)y, (double*)out); break;
    case FGB_F32: map2_k<float><<<grid, 256, 0, s>>>(op, n, (const float*)x, (const float*)y, (float*)out); break;
    case FGB_I32: map2_k<int32_t><<<grid, 256, 0, s>>>(op, n, (const int32_t*)x, (const int32_t*)y, (int32_t*)out); break;
    case FGB_I64: map2_k<int64_t><<<grid, 256, 0, s>>>(op, n, (const int64_t*)x, (const int64_t*)y, (int64_t*)out); break;
    default: return set_error(FGB_EUNSUPPORTED, "fgb_dense_map: dtype %d", dtype);
  }
  return check_launch("fgb_dense_map");
}

int fgb_scalar_op(fgb_ctx* ctx, int op, int dtype, const void* a, const void* b, void* out,
                  void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_scalar_op: null ctx");
  if (!a || !out || (op != FGB_MAP_ADD && op != FGB_MAP_SUB && op != FGB_MAP_MUL &&
                     op != FGB_MAP_DIV && op != FGB_MAP_MIN && op != FGB_MAP_MAX))
    return set_error(FGB_EINVAL, "fgb_scalar_op: bad argument");
  if (!b) return set_error(FGB_EINVAL, "fgb_scalar_op: null b");
  cudaStream_t s = pick_stream(ctx, stream);
  if (dtype == FGB_F64)
    scalar_k<double><<<1, 1, 0, s>>>(op, (const double*)a, (const double*)b, (double*)out);
  else if (dtype == FGB_F32)
    scalar_k<float><<<1, 1, 0, s>>>(op, (const float*)a, (const float*)b, (float*)out);
  else
    return set_error(FGB_EUNSUPPORTED, "fgb_scalar_op: dtype %d", dtype);
  return check_launch("fgb_scalar_op");
}

}  // extern "C"
