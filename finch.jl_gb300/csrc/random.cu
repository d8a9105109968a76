// Seeded random CSR matrices generated on the device, with the distribution
// of Finch's fsprand(m, n, p) (src/interface/fsparse.jl:173-290): every
// (i, j) is stored independently with probability p, so row lengths are
// Binomial(n, p) and coordinates are uniform without replacement.  Rows are
// drawn by geometric gaps between stored columns from a counter-based hash,
// so pass 1 (counts) and pass 2 (fill) draw the same columns and the result
// depends only on (seed, m, n, p).
#include <cub/cub.cuh>

#include "fgb_internal.cuh"

namespace fgb {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Uniform in (0, 1) from a 64-bit hash (53 random bits, never 0).
__device__ __forceinline__ double unit(uint64_t h) {
  return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

// Calls emit(k, col) for the stored columns of row `row`, ascending.
template <class F>
__device__ __forceinline__ int64_t walk_row(uint64_t seed, int64_t row, int64_t n, double p, F&& emit) {
  if (p <= 0.0) return 0;
  const double lq = p >= 1.0 ? 0.0 : log1p(-p);
  const uint64_t base = mix64(seed ^ mix64((uint64_t)row));
  int64_t col = -1, k = 0;
  while (true) {
    int64_t gap = 0;
    if (p < 1.0) {
      const double u = unit(mix64(base + 2 * (uint64_t)k));
      const double g = floor(log(u) / lq);
      gap = g > (double)n ? n : (int64_t)g;
    }
    col += gap + 1;
    if (col >= n) break;
    emit(k, col);
    ++k;
  }
  return k;
}

__global__ void random_count_k(uint64_t seed, int64_t m, int64_t n, double p, int32_t* __restrict__ counts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
    counts[i] = (int32_t)walk_row(seed, i, n, p, [](int64_t, int64_t) {});
}

template <class T>
__global__ void random_fill_k(uint64_t seed, int64_t m, int64_t n, double p,
                              const int32_t* __restrict__ ptr, int32_t* __restrict__ idx,
                              T* __restrict__ val) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q0 = ptr[i];
    const uint64_t vseed = mix64(seed ^ 0x5DEECE66Dull) ^ mix64((uint64_t)i * 0x2545F4914F6CDD1Dull);
    walk_row(seed, i, n, p, [&](int64_t k, int64_t col) {
      idx[q0 + k] = (int32_t)col;
      const double u1 = unit(mix64(vseed + 2 * (uint64_t)k)), u2 = unit(mix64(vseed + 2 * (uint64_t)k + 1));
      if (sizeof(T) == 4)  // N(0, 1) by Box-Muller
        val[q0 + k] = (T)(sqrt(-2.0 * log(u1)) * cospi(2.0 * u2));
      else  // U[0, 1)
        val[q0 + k] = (T)(u1 - 0.5 / 9007199254740992.0);
    });
  }
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_random_csr(fgb_ctx* ctx, uint64_t seed, int64_t m, int64_t n, double p,
                              int val_t, int32_t* ptr, int32_t* idx, void* val, int64_t* nnz,
                              void* stream) {
  if (!ctx || !ptr || !nnz) return set_error(FGB_EINVAL, "fgb_random_csr: null argument");
  if (m < 0 || n < 0 || n > INT32_MAX || !(p >= 0.0 && p <= 1.0))
    return set_error(FGB_EINVAL, "fgb_random_csr: bad shape or probability");
  if (val_t != FGB_F32 && val_t != FGB_F64)
    return set_error(FGB_EUNSUPPORTED, "fgb_random_csr: values must be F32 or F64");
  if ((double)m * (double)n * p > 1.5e9)  // int32 ptr: keep the expected total far below 2^31
    return set_error(FGB_EUNSUPPORTED, "fgb_random_csr: expected stored entries exceed the int32 ptr");
  cudaStream_t s = pick_stream(ctx, stream);
  const int grid = grid_for(m, 128, ctx->num_sms, 8);
  if (!idx) {  // pass 1: counts -> ptr, nnz
    int32_t* counts = nullptr;
    size_t tmp_bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, counts, ptr, m + 1, s);
    FGB_CUDA_TRY(cudaMallocAsync((void**)&counts, sizeof(int32_t) * (m + 1) + tmp_bytes, s));
    void* tmp = counts + (m + 1);
    FGB_CUDA_TRY(cudaMemsetAsync(counts + m, 0, sizeof(int32_t), s));
    if (m > 0) random_count_k<<<grid, 128, 0, s>>>(seed, m, n, p, counts);
    int rc = check_launch("random_count_k");
    if (rc == FGB_OK) {
      cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, counts, ptr, m + 1, s);
      rc = check_launch("random_csr scan");
    }
    cudaFreeAsync(counts, s);
    if (rc) return rc;
    int32_t total = 0;
    FGB_CUDA_TRY(cudaMemcpyAsync(&total, ptr + m, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    FGB_CUDA_TRY(cudaStreamSynchronize(s));
    *nnz = total;
    return FGB_OK;
  }
  if (m > 0) {
    if (val_t == FGB_F32)
      random_fill_k<float><<<grid, 128, 0, s>>>(seed, m, n, p, ptr, idx, (float*)val);
    else
      random_fill_k<double><<<grid, 128, 0, s>>>(seed, m, n, p, ptr, idx, (double*)val);
  }
  return check_launch("random_fill_k");
}
