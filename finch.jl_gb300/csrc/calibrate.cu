// Random-gather ceiling (fgb_gather_ceiling): the throughput at which random
// gathers of one width are served from a working set of one size.  The
// kernels that gather dense rows (SpMM, SDDMM, pull SpMV) are bound by this,
// not by streaming HBM bandwidth: a working set that fits L2 is served at the
// L2's request rate, a larger one partly from DRAM.
#include "../../include/finchgb_calibrate.h"
#include "fgb_internal.cuh"

namespace fgb {

constexpr int CAL_THREADS = 256;
constexpr int CAL_INFLIGHT = 8;

__device__ __forceinline__ uint32_t cal_hash(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

// A uniform place in [0, n) for a 32-bit hash: the high word of hash * n
// (one multiply) for n < 2^32, so the index arithmetic stays a few
// instructions per gather.  A 64-bit `%` costs dozens of instructions per
// gather and made the probe issue-bound below the memory system's rate.
__device__ __forceinline__ uint64_t cal_place(uint32_t h, uint64_t n) {
  return n <= 0xffffffffull ? (uint64_t)__umulhi(h, (uint32_t)n) : (uint64_t)h % n;
}

// G lanes (16 bytes each) per gather; every lane keeps CAL_INFLIGHT loads in
// flight.  `lines` = working set / gather width, so every address is inside
// the buffer: line < lines and part < G.
template <int G>
__global__ void __launch_bounds__(CAL_THREADS) gather_ceiling_k(const float* __restrict__ buf, uint64_t lines,
                                                              int iters, float* __restrict__ sink) {
  const int part = (threadIdx.x & 31) % G;
  const uint32_t gid = (blockIdx.x * (uint32_t)blockDim.x + threadIdx.x) / G;
  const uint64_t pol = policy_evict_last();
  float acc = 0.f;
#pragma unroll 1
  for (int it = 0; it < iters; it += CAL_INFLIGHT) {
    float4 v[CAL_INFLIGHT];
#pragma unroll
    for (int u = 0; u < CAL_INFLIGHT; ++u) {
      const uint64_t line = cal_place(cal_hash(gid * 0x9E3779B9u + (uint32_t)(it + u)), lines);
      v[u] = ld_gather_f32x4(buf + (line * G + part) * 4, pol);
    }
#pragma unroll
    for (int u = 0; u < CAL_INFLIGHT; ++u) acc += (v[u].x + v[u].y) + (v[u].z + v[u].w);
  }
  if (acc == 1.2345f) sink[0] = acc;  // keeps the loads; the buffer is zero, so never taken
}

// 4- or 8-byte gathers, one per lane (the x gathers of a pull SpMV): each
// costs one 32-byte sector request, so this measures the request rate.
template <class T>
__global__ void __launch_bounds__(CAL_THREADS) gather_ceiling_word_k(const T* __restrict__ buf, uint64_t n,
                                                                   int iters, T* __restrict__ sink) {
  const uint32_t gid = blockIdx.x * (uint32_t)blockDim.x + threadIdx.x;
  T acc = 0;
#pragma unroll 1
  for (int it = 0; it < iters; it += CAL_INFLIGHT) {
    T v[CAL_INFLIGHT];
#pragma unroll
    for (int u = 0; u < CAL_INFLIGHT; ++u)
      v[u] = __ldg(buf + cal_place(cal_hash(gid * 0x9E3779B9u + (uint32_t)(it + u)), n));
#pragma unroll
    for (int u = 0; u < CAL_INFLIGHT; ++u) acc += v[u];
  }
  if (acc == T(12345)) sink[0] = acc;  // keeps the loads; the buffer is zero, so never taken
}

template <class T>
static int run_word_ceiling(fgb_ctx* ctx, int64_t ws, int64_t gathers, double* gbs, cudaStream_t s) {
  int occ = 0;
  FGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gather_ceiling_word_k<T>, CAL_THREADS, 0));
  const int grid = ctx->num_sms * (occ > 0 ? occ : 1);
  const int64_t per_launch = (int64_t)grid * CAL_THREADS;
  int64_t it = (gathers + per_launch - 1) / per_launch;
  it = (it + CAL_INFLIGHT - 1) / CAL_INFLIGHT * CAL_INFLIGHT;
  if (it > (1 << 24)) return set_error(FGB_EINVAL, "fgb_gather_ceiling: too many gathers");
  const uint64_t n = (uint64_t)ws / sizeof(T);
  T* buf = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = FGB_OK;
  cudaError_t e = cudaMallocAsync((void**)&buf, (n + 1) * sizeof(T), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(buf, 0, (n + 1) * sizeof(T), s);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float ms = 0.f;
  constexpr int reps = 5;
  if (e == cudaSuccess) {
    for (int w = 0; w < 2; ++w) gather_ceiling_word_k<T><<<grid, CAL_THREADS, 0, s>>>(buf, n, (int)it, buf + n);
    e = cudaEventRecord(e0, s);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) {
      gather_ceiling_word_k<T><<<grid, CAL_THREADS, 0, s>>>(buf, n, (int)it, buf + n);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e != cudaSuccess) rc = set_error(FGB_ECUDA, "fgb_gather_ceiling: %s", cudaGetErrorString(e));
  if (buf) cudaFreeAsync(buf, s);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc == FGB_OK) {
    const double bytes = (double)per_launch * it * sizeof(T) * reps;
    *gbs = ms > 0.f ? bytes / (ms * 1e-3) / 1e9 : 0.0;
    FGB_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return rc;
}

template <int G>
static int run_ceiling(fgb_ctx* ctx, int64_t ws, int64_t gathers, double* gbs, cudaStream_t s) {
  int occ = 0;
  FGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gather_ceiling_k<G>, CAL_THREADS, 0));
  const int grid = ctx->num_sms * (occ > 0 ? occ : 1);
  const int64_t per_launch_gathers = (int64_t)grid * CAL_THREADS / G;
  int64_t it = (gathers + per_launch_gathers - 1) / per_launch_gathers;
  it = (it + CAL_INFLIGHT - 1) / CAL_INFLIGHT * CAL_INFLIGHT;
  if (it > (1 << 24)) return set_error(FGB_EINVAL, "fgb_gather_ceiling: too many gathers");
  const uint64_t lines = (uint64_t)ws / (16 * G);
  float* buf = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = FGB_OK;
  cudaError_t e = cudaMallocAsync((void**)&buf, (size_t)lines * 16 * G + sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(buf, 0, (size_t)lines * 16 * G + sizeof(float), s);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float ms = 0.f;
  constexpr int reps = 5;
  if (e == cudaSuccess) {
    float* sink = buf + lines * 4 * G;
    for (int w = 0; w < 2; ++w) gather_ceiling_k<G><<<grid, CAL_THREADS, 0, s>>>(buf, lines, (int)it, sink);
    e = cudaEventRecord(e0, s);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) {
      gather_ceiling_k<G><<<grid, CAL_THREADS, 0, s>>>(buf, lines, (int)it, sink);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e != cudaSuccess) rc = set_error(FGB_ECUDA, "fgb_gather_ceiling: %s", cudaGetErrorString(e));
  if (buf) cudaFreeAsync(buf, s);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc == FGB_OK) {
    const double bytes = (double)per_launch_gathers * it * 16 * G * reps;
    *gbs = ms > 0.f ? bytes / (ms * 1e-3) / 1e9 : 0.0;
    FGB_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return rc;
}

}  // namespace fgb

extern "C" int fgb_gather_ceiling(fgb_ctx* ctx, int64_t working_set_bytes, int32_t gather_bytes,
                                  int64_t gathers, double* gbs, void* stream) {
  using namespace fgb;
  FGB_REQUIRE(ctx && gbs, "fgb_gather_ceiling: null argument");
  FGB_REQUIRE(gathers > 0, "fgb_gather_ceiling: gathers must be positive");
  FGB_REQUIRE(gather_bytes >= 4 && gather_bytes <= 512 && (gather_bytes & (gather_bytes - 1)) == 0,
              "fgb_gather_ceiling: gather width must be 4, 8, 16, 32, 64, 128, 256 or 512 bytes");
  FGB_REQUIRE(working_set_bytes / gather_bytes >= 64, "fgb_gather_ceiling: working set below 64 gathers");
  cudaStream_t s = pick_stream(ctx, stream);
  switch (gather_bytes) {
    case 4: return run_word_ceiling<float>(ctx, working_set_bytes, gathers, gbs, s);
    case 8: return run_word_ceiling<double>(ctx, working_set_bytes, gathers, gbs, s);
    case 16: return run_ceiling<1>(ctx, working_set_bytes, gathers, gbs, s);
    case 32: return run_ceiling<2>(ctx, working_set_bytes, gathers, gbs, s);
    case 64: return run_ceiling<4>(ctx, working_set_bytes, gathers, gbs, s);
    case 128: return run_ceiling<8>(ctx, working_set_bytes, gathers, gbs, s);
    case 256: return run_ceiling<16>(ctx, working_set_bytes, gathers, gbs, s);
    default: return run_ceiling<32>(ctx, working_set_bytes, gathers, gbs, s);
  }
}
