// Internal helpers shared by the CUDA translation units of libfinchgb.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "../../include/finchgb.h"

struct fgb_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int* d_err = nullptr;  // device flag: a kernel's bounded wait ran out (read by fgb_ctx_device_error)
  std::mutex mu;  // guards lazily created per-context state
};

namespace fgb {

// Records a message as the calling thread's last error and returns `code`.
int set_error(int code, const char* fmt, ...);
void clear_error();

// NULL is CUDA's legacy default stream (the convention of every CUDA
// library), so calls order with other work issued on it; the context's own
// stream is used only when a caller passes it explicitly.
inline cudaStream_t pick_stream(fgb_ctx*, void* s) {
  return s ? static_cast<cudaStream_t>(s) : cudaStreamLegacy;
}

// True while `s` is being captured into a CUDA graph: paths that synchronise
// (a schedule built for one call reads its sizes back) are then not taken.
inline bool stream_capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone;
}

// Returns FGB_ECUDA with a message if the last launch failed.
int check_launch(const char* what);

#define FGB_CUDA_TRY(expr)                                                              \
  do {                                                                                  \
    cudaError_t e_ = (expr);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return ::fgb::set_error(FGB_ECUDA, "%s: %s (%s:%d)", #expr, cudaGetErrorString(e_), \
                              __FILE__, __LINE__);                                      \
  } while (0)

#define FGB_REQUIRE(cond, ...)                                  \
  do {                                                          \
    if (!(cond)) return ::fgb::set_error(FGB_EINVAL, __VA_ARGS__); \
  } while (0)

// Validates a sparse descriptor's fields (not its contents).
int check_sparse(const fgb_sparse* A, const char* name, bool need_i32_idx);

inline int64_t n_fibers(const fgb_sparse* A) {
  return A->orient == FGB_CSR ? A->nrows : A->ncols;
}
inline int64_t fiber_extent(const fgb_sparse* A) {
  return A->orient == FGB_CSR ? A->ncols : A->nrows;
}

inline int grid_for(int64_t work_items, int threads, int num_sms, int blocks_per_sm = 8) {
  int64_t b = (work_items + threads - 1) / threads;
  int64_t cap = (int64_t)num_sms * blocks_per_sm;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

// ---------------------------------------------------------------- device side

// Cache policies for loads/stores (PTX createpolicy).  Streams that are read
// once (idx, val, output) are marked evict_first so the gathered dense
// operand keeps its L2 lines; gathers are marked evict_last.
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ int ld_stream_i32(const int* p, uint64_t pol) {
  int v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.b32 %0, [%1], %2;"
               : "=r"(v)
               : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ float ld_stream_f32(const float* p, uint64_t pol) {
  float v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;"
               : "=f"(v)
               : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ float4 ld_gather_f32x4(const float* p, uint64_t pol) {
  float4 v;
  asm volatile("ld.global.nc.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ void st_stream_f32x4(float* p, float4 v, uint64_t pol) {
  asm volatile("st.global.L1::no_allocate.L2::cache_hint.v4.f32 [%0], {%1,%2,%3,%4}, %5;" ::"l"(p),
               "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void st_stream_f32(float* p, float v, uint64_t pol) {
  asm volatile("st.global.L1::no_allocate.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v),
               "l"(pol)
               : "memory");
}

template <class PtrT>
__device__ __forceinline__ int64_t ld_ptr(const PtrT* p, int64_t i) {
  return (int64_t)__ldg(p + i);
}

// Value loads with conversion to the accumulation type.
template <class T>
struct ValLoad;
template <>
struct ValLoad<double> {
  __device__ static double get(const void* v, int64_t i) { return __ldg((const double*)v + i); }
};
template <>
struct ValLoad<float> {
  __device__ static float get(const void* v, int64_t i) { return __ldg((const float*)v + i); }
};

}  // namespace fgb
