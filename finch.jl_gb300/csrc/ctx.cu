// Context, error reporting, memory and index narrowing.
#include <cstring>

#include "fgb_internal.cuh"

namespace fgb {

static thread_local char tls_error[1024] = {0};

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(tls_error, sizeof(tls_error), fmt, ap);
  va_end(ap);
  return code;
}

void clear_error() { tls_error[0] = 0; }

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(FGB_ECUDA, "%s: launch failed: %s", what, cudaGetErrorString(e));
  return FGB_OK;
}

int check_sparse(const fgb_sparse* A, const char* name, bool need_i32_idx) {
  if (!A) return set_error(FGB_EINVAL, "%s: null descriptor", name);
  if (A->nrows < 0 || A->ncols < 0 || A->nnz < 0)
    return set_error(FGB_EINVAL, "%s: negative size (%lld x %lld, nnz %lld)", name,
                     (long long)A->nrows, (long long)A->ncols, (long long)A->nnz);
  if (A->orient != FGB_CSR && A->orient != FGB_CSC)
    return set_error(FGB_EINVAL, "%s: orient must be FGB_CSR or FGB_CSC", name);
  if (A->index_base != 0 && A->index_base != 1)
    return set_error(FGB_EINVAL, "%s: index_base must be 0 or 1", name);
  if (A->ptr_t != FGB_I32 && A->ptr_t != FGB_I64)
    return set_error(FGB_EINVAL, "%s: ptr_t must be FGB_I32 or FGB_I64", name);
  if (need_i32_idx && A->idx_t != FGB_I32)
    return set_error(FGB_EUNSUPPORTED, "%s: kernels read 32-bit idx; narrow with fgb_narrow_index",
                     name);
  if (fiber_extent(A) > INT32_MAX)
    return set_error(FGB_EUNSUPPORTED, "%s: fiber extent %lld exceeds int32", name,
                     (long long)fiber_extent(A));
  if (A->ptr_t == FGB_I32 && A->nnz > INT32_MAX)
    return set_error(FGB_EINVAL, "%s: nnz %lld does not fit an int32 ptr", name, (long long)A->nnz);
  if (!A->ptr) return set_error(FGB_EINVAL, "%s: null ptr buffer", name);
  if (A->nnz > 0 && !A->idx) return set_error(FGB_EINVAL, "%s: null idx buffer", name);
  if (A->nnz > 0 && A->val_t != FGB_NONE && !A->val)
    return set_error(FGB_EINVAL, "%s: null val buffer", name);
  return FGB_OK;
}

__global__ void narrow_kernel(const int64_t* __restrict__ src, int32_t* __restrict__ dst, int64_t n,
                              int64_t delta, int* __restrict__ bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t v = src[i] - delta;
    if (v < INT32_MIN || v > INT32_MAX) atomicExch(bad, 1);
    dst[i] = (int32_t)v;
  }
}

}  // namespace fgb

using namespace fgb;

extern "C" {

int fgb_version(void) { return FGB_VERSION_MAJOR * 1000 + FGB_VERSION_MINOR; }

const char* fgb_last_error(void) { return tls_error; }

int fgb_ctx_create(int device, fgb_ctx** out) {
  if (!out) return set_error(FGB_EINVAL, "fgb_ctx_create: null out");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess) return set_error(FGB_ECUDA, "fgb_ctx_create: no CUDA device: %s", cudaGetErrorString(e));
  if (device < 0 || device >= count)
    return set_error(FGB_EINVAL, "fgb_ctx_create: device %d out of range [0,%d)", device, count);
  FGB_CUDA_TRY(cudaSetDevice(device));
  fgb_ctx* c = new fgb_ctx();
  c->device = device;
  e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(c->d_err, 0, sizeof(int));
  // The library's scratch comes from this process's default stream-ordered
  // pool of the device.  With the default release threshold (0) the pool
  // unmaps freed blocks at every synchronisation and the next call maps them
  // again; keeping up to FGB_POOL_KEEP_BYTES mapped makes repeated calls
  // (COO assembly, SpGEMM, schedules built per call) reuse their scratch.
  cudaMemPool_t pool = nullptr;
  if (e == cudaSuccess) e = cudaDeviceGetDefaultMemPool(&pool, device);
  if (e == cudaSuccess) {
    uint64_t keep = FGB_POOL_KEEP_BYTES, cur = 0;
    e = cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &cur);
    if (e == cudaSuccess && cur < keep) e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (e != cudaSuccess) {
    delete c;
    return set_error(FGB_ECUDA, "fgb_ctx_create: %s", cudaGetErrorString(e));
  }
  *out = c;
  return FGB_OK;
}

int fgb_ctx_destroy(fgb_ctx* ctx) {
  if (!ctx) return FGB_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) {
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
  }
  if (ctx->d_err) cudaFree(ctx->d_err);
  delete ctx;
  return FGB_OK;
}

void* fgb_ctx_stream(fgb_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int fgb_ctx_device_error(fgb_ctx* ctx, int* flag) {
  if (!ctx || !flag) return set_error(FGB_EINVAL, "fgb_ctx_device_error: null argument");
  FGB_CUDA_TRY(cudaDeviceSynchronize());
  FGB_CUDA_TRY(cudaMemcpy(flag, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  FGB_CUDA_TRY(cudaMemset(ctx->d_err, 0, sizeof(int)));
  return FGB_OK;
}

int fgb_ctx_num_sms(fgb_ctx* ctx) { return ctx ? ctx->num_sms : 0; }

int fgb_malloc(fgb_ctx* ctx, size_t bytes, void** out) {
  if (!ctx || !out) return set_error(FGB_EINVAL, "fgb_malloc: null argument");
  *out = nullptr;
  if (bytes == 0) return FGB_OK;
  cudaError_t e = cudaMalloc(out, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return set_error(e == cudaErrorMemoryAllocation ? FGB_ENOMEM : FGB_ECUDA,
                     "fgb_malloc(%zu): %s", bytes, cudaGetErrorString(e));
  }
  return FGB_OK;
}

int fgb_free(fgb_ctx* ctx, void* p) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_free: null ctx");
  if (p) FGB_CUDA_TRY(cudaFree(p));
  return FGB_OK;
}

int fgb_host_alloc(fgb_ctx* ctx, size_t bytes, void** out) {
  if (!ctx || !out) return set_error(FGB_EINVAL, "fgb_host_alloc: null argument");
  *out = nullptr;
  if (bytes == 0) return FGB_OK;
  cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocPortable);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return set_error(FGB_ENOMEM, "fgb_host_alloc(%zu): %s", bytes, cudaGetErrorString(e));
  }
  return FGB_OK;
}

int fgb_host_free(fgb_ctx* ctx, void* p) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_host_free: null ctx");
  if (p) FGB_CUDA_TRY(cudaFreeHost(p));
  return FGB_OK;
}

int fgb_upload(fgb_ctx* ctx, void* dst, const void* src, size_t bytes, void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_upload: null ctx");
  if (bytes == 0) return FGB_OK;
  if (!dst || !src) return set_error(FGB_EINVAL, "fgb_upload: null pointer");
  FGB_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, pick_stream(ctx, stream)));
  return FGB_OK;
}

int fgb_download(fgb_ctx* ctx, void* dst, const void* src, size_t bytes, void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_download: null ctx");
  if (bytes == 0) return FGB_OK;
  if (!dst || !src) return set_error(FGB_EINVAL, "fgb_download: null pointer");
  FGB_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, pick_stream(ctx, stream)));
  return FGB_OK;
}

int fgb_stream_sync(fgb_ctx* ctx, void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_stream_sync: null ctx");
  FGB_CUDA_TRY(cudaStreamSynchronize(pick_stream(ctx, stream)));
  return FGB_OK;
}

int fgb_narrow_index(fgb_ctx* ctx, const int64_t* src, int32_t* dst, int64_t n, int64_t delta,
                     void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_narrow_index: null ctx");
  if (n < 0) return set_error(FGB_EINVAL, "fgb_narrow_index: negative length");
  if (n == 0) return FGB_OK;
  if (!src || !dst) return set_error(FGB_EINVAL, "fgb_narrow_index: null pointer");
  cudaStream_t s = pick_stream(ctx, stream);
  int* bad = nullptr;
  FGB_CUDA_TRY(cudaMallocAsync((void**)&bad, sizeof(int), s));
  FGB_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), s));
  narrow_kernel<<<grid_for(n, 256, ctx->num_sms), 256, 0, s>>>(src, dst, n, delta, bad);
  int rc = check_launch("narrow_kernel");
  int h_bad = 0;
  if (rc == FGB_OK) FGB_CUDA_TRY(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  cudaFreeAsync(bad, s);
  FGB_CUDA_TRY(cudaStreamSynchronize(s));
  if (rc != FGB_OK) return rc;
  if (h_bad) return set_error(FGB_EINVAL, "fgb_narrow_index: value outside int32 range");
  return FGB_OK;
}

}  // extern "C"
