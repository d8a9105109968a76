// COO triplets -> SparseList (CSC or CSR) assembled on the device.
//
// The contract is fsparse's (src/interface/fsparse.jl:60-100): the stored
// entries come out sorted by (fiber, coordinate) -- column then row for
// Finch's Dense(SparseList) -- and duplicate coordinates are folded left to
// right, in input order, with `combine` (+ by default, | for Bool).  Steps:
//   1. 64-bit keys fiber * inner + coordinate (coordinates checked in range);
//   2. a stable radix sort of the keys carrying each entry's input position;
//   3. run heads (key changes) and their exclusive sum = output positions;
//   4. one thread per run folds its values in sorted (= input) order;
//   5. each fiber's start is a binary search of the unique keys.
// Sorting stably and folding sequentially make float sums bit-identical to
// Julia's foldl over the same duplicates.
#include <cub/cub.cuh>

#include <cmath>
#include <type_traits>

#include "fgb_internal.cuh"

namespace fgb {

template <class IT>
__global__ void coo_keys_k(int64_t n, const IT* __restrict__ I, const IT* __restrict__ J, int base,
                           int64_t nrows, int64_t ncols, int csc, uint64_t* __restrict__ keys,
                           int32_t* __restrict__ perm, int* __restrict__ bad) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)I[k] - base, j = (int64_t)J[k] - base;
    uint64_t key = 0;
    if (i < 0 || i >= nrows || j < 0 || j >= ncols) {
      atomicOr(bad, 1);
    } else {
      key = csc ? (uint64_t)j * (uint64_t)nrows + (uint64_t)i : (uint64_t)i * (uint64_t)ncols + (uint64_t)j;
    }
    keys[k] = key;
    perm[k] = (int32_t)k;
  }
}

__global__ void coo_heads_k(int64_t n, const uint64_t* __restrict__ keys, int32_t* __restrict__ head) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    head[k] = (k == 0 || keys[k] != keys[k - 1]) ? 1 : 0;
}

// Julia semantics of the combine functions (non-fastmath: fsparse folds with
// plain Base functions).
template <int OP, class T>
struct Combine;
template <class T>
struct Combine<FGB_COMBINE_ADD, T> {
  __device__ static T f(T a, T b) { return (T)((std::make_unsigned_t<T>)a + (std::make_unsigned_t<T>)b); }
};
template <>
struct Combine<FGB_COMBINE_ADD, double> {
  __device__ static double f(double a, double b) { return __dadd_rn(a, b); }
};
template <>
struct Combine<FGB_COMBINE_ADD, float> {
  __device__ static float f(float a, float b) { return __fadd_rn(a, b); }
};
template <class T>
struct Combine<FGB_COMBINE_OR, T> {
  __device__ static T f(T a, T b) { return (T)(a | b); }
};
template <class T>
struct Combine<FGB_COMBINE_LAST, T> {
  __device__ static T f(T, T b) { return b; }
};
template <class T>
__device__ __forceinline__ bool fnan(T) { return false; }
__device__ __forceinline__ bool fnan(double v) { return v != v; }
__device__ __forceinline__ bool fnan(float v) { return v != v; }
template <class T>
__device__ __forceinline__ bool fneg(T v) {
  if constexpr (std::is_signed<T>::value) return v < 0;
  else return false;
}
__device__ __forceinline__ bool fneg(double v) { return signbit(v); }
__device__ __forceinline__ bool fneg(float v) { return signbit(v); }
// min(x, y): a NaN operand wins; otherwise the smaller, with -0.0 below +0.0
template <class T>
struct Combine<FGB_COMBINE_MIN, T> {
  __device__ static T f(T a, T b) {
    if (fnan(a)) return a;
    if (fnan(b)) return b;
    return (b < a || (b == a && fneg(b) && !fneg(a))) ? b : a;
  }
};
template <class T>
struct Combine<FGB_COMBINE_MAX, T> {
  __device__ static T f(T a, T b) {
    if (fnan(a)) return a;
    if (fnan(b)) return b;
    return (b > a || (b == a && !fneg(b) && fneg(a))) ? b : a;
  }
};

template <class VT, int OP, bool PATTERN>
__global__ void coo_fold_k(int64_t n, const uint64_t* __restrict__ keys, const int32_t* __restrict__ perm,
                           const int32_t* __restrict__ head, const int32_t* __restrict__ pos,
                           const VT* __restrict__ val, uint64_t inner, int out_base,
                           int32_t* __restrict__ out_idx, VT* __restrict__ out_val,
                           uint64_t* __restrict__ ukeys) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    if (!head[k]) continue;
    const uint64_t key = keys[k];
    const int64_t o = pos[k];
    if (!PATTERN) {
      VT v = val[perm[k]];
      for (int64_t r = k + 1; r < n && !head[r]; ++r) v = Combine<OP, VT>::f(v, val[perm[r]]);
      out_val[o] = v;
    }
    out_idx[o] = (int32_t)(key % inner) + out_base;
    ukeys[o] = key;
  }
}

template <class PtrT>
__global__ void coo_ptr_k(int64_t nfib, const uint64_t* __restrict__ ukeys, int64_t nnz, uint64_t inner,
                          int out_base, PtrT* __restrict__ ptr) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f <= nfib;
       f += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t target = (uint64_t)f * inner;  // first key of fiber f
    int64_t lo = 0, hi = nnz;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (ukeys[mid] < target) lo = mid + 1; else hi = mid;
    }
    ptr[f] = (PtrT)(lo + out_base);
  }
}

static inline size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

template <class VT, bool PATTERN>
static void launch_fold(int combine, int grid, cudaStream_t s, int64_t n, const uint64_t* keys,
                        const int32_t* perm, const int32_t* head, const int32_t* pos, const void* val,
                        uint64_t inner, int out_base, int32_t* out_idx, void* out_val, uint64_t* ukeys) {
#define FGB_FOLD(OP)                                                                              \
  coo_fold_k<VT, OP, PATTERN><<<grid, 256, 0, s>>>(n, keys, perm, head, pos, (const VT*)val, inner, \
                                                   out_base, out_idx, (VT*)out_val, ukeys)
  switch (combine) {
    case FGB_COMBINE_ADD: FGB_FOLD(FGB_COMBINE_ADD); break;
    case FGB_COMBINE_MIN: FGB_FOLD(FGB_COMBINE_MIN); break;
    case FGB_COMBINE_MAX: FGB_FOLD(FGB_COMBINE_MAX); break;
    default: FGB_FOLD(FGB_COMBINE_LAST); break;
  }
#undef FGB_FOLD
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_coo_assemble(fgb_ctx* ctx, int64_t nrows, int64_t ncols, int64_t n_in, int idx_t,
                                const void* I, const void* J, int in_base, int val_t,
                                const void* val, int combine, fgb_sparse* out, int64_t* nnz_out,
                                void* stream) {
  if (!ctx || !out || !nnz_out) return set_error(FGB_EINVAL, "fgb_coo_assemble: null argument");
  *nnz_out = 0;
  if (nrows < 0 || ncols < 0 || n_in < 0) return set_error(FGB_EINVAL, "fgb_coo_assemble: negative size");
  if (n_in > INT32_MAX) return set_error(FGB_EUNSUPPORTED, "fgb_coo_assemble: more than 2^31 - 1 triplets");
  if (idx_t != FGB_I32 && idx_t != FGB_I64) return set_error(FGB_EINVAL, "fgb_coo_assemble: idx_t must be I32 or I64");
  if (out->orient != FGB_CSR && out->orient != FGB_CSC) return set_error(FGB_EINVAL, "fgb_coo_assemble: bad orient");
  if (out->ptr_t != FGB_I32 && out->ptr_t != FGB_I64) return set_error(FGB_EINVAL, "fgb_coo_assemble: ptr_t must be I32 or I64");
  if (out->idx_t != FGB_I32) return set_error(FGB_EUNSUPPORTED, "fgb_coo_assemble: output idx_t must be I32");
  if (out->val_t != val_t) return set_error(FGB_EINVAL, "fgb_coo_assemble: output and input value types differ");
  const bool pattern = val_t == FGB_NONE;
  if (combine < FGB_COMBINE_ADD || combine > FGB_COMBINE_LAST)
    return set_error(FGB_EINVAL, "fgb_coo_assemble: unknown combine %d", combine);
  if (val_t == FGB_BOOL && combine == FGB_COMBINE_ADD) combine = FGB_COMBINE_OR;  // Bool folds with |
  if (combine == FGB_COMBINE_OR && val_t != FGB_BOOL && !pattern)
    return set_error(FGB_EUNSUPPORTED, "fgb_coo_assemble: | combines Bool values only");
  if (val_t == FGB_BF16) return set_error(FGB_EUNSUPPORTED, "fgb_coo_assemble: bf16 values");
  const bool csc = out->orient == FGB_CSC;
  const int64_t nfib = csc ? ncols : nrows, inner = csc ? nrows : ncols;
  if (out->nrows != nrows || out->ncols != ncols) return set_error(FGB_EINVAL, "fgb_coo_assemble: output shape differs");
  if (nfib > 0 && !out->ptr) return set_error(FGB_EINVAL, "fgb_coo_assemble: null output ptr");
  if (inner > INT32_MAX) return set_error(FGB_EUNSUPPORTED, "fgb_coo_assemble: coordinates above 2^31");
  if (nrows > 0 && ncols > 0 && (double)nrows * (double)ncols > 1.8e19)
    return set_error(FGB_EUNSUPPORTED, "fgb_coo_assemble: shape too large for 64-bit keys");
  if (n_in > 0 && (!I || !J || (!pattern && !val) || !out->idx || (!pattern && !out->val)))
    return set_error(FGB_EINVAL, "fgb_coo_assemble: null buffer");
  cudaStream_t s = pick_stream(ctx, stream);
  const int ob = out->index_base;
  const int grid_n = grid_for(n_in, 256, ctx->num_sms);
  const int grid_f = grid_for(nfib + 1, 256, ctx->num_sms);
  if (n_in == 0) {
    if (nfib >= 0 && out->ptr) {
      if (out->ptr_t == FGB_I32)
        coo_ptr_k<int32_t><<<grid_f, 256, 0, s>>>(nfib, nullptr, 0, (uint64_t)(inner > 0 ? inner : 1), ob, (int32_t*)out->ptr);
      else
        coo_ptr_k<int64_t><<<grid_f, 256, 0, s>>>(nfib, nullptr, 0, (uint64_t)(inner > 0 ? inner : 1), ob, (int64_t*)out->ptr);
      FGB_CUDA_TRY(cudaGetLastError());
      FGB_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return FGB_OK;
  }
  // keys, keys_sorted, ukeys (8 B); perm, perm_sorted, head, pos (4 B); flag; CUB temp
  const size_t n = (size_t)n_in;
  int end_bit = 1;
  const uint64_t max_key = (uint64_t)nfib * (uint64_t)inner;
  while (end_bit < 64 && (uint64_t(1) << end_bit) < max_key) ++end_bit;
  size_t sort_bytes = 0, scan_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, (uint64_t*)nullptr, (uint64_t*)nullptr,
                                  (int32_t*)nullptr, (int32_t*)nullptr, (int)n, 0, end_bit, s);
  cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (int32_t*)nullptr, (int32_t*)nullptr, (int)n, s);
  const size_t cub_bytes = std::max(sort_bytes, scan_bytes);
  const size_t total = a256(8 * n) * 3 + a256(4 * n) * 4 + 256 + a256(cub_bytes);
  char* mem = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&mem, total, s);
  if (e != cudaSuccess) return set_error(FGB_ENOMEM, "fgb_coo_assemble: scratch (%zu bytes): %s", total, cudaGetErrorString(e));
  uint64_t* keys = (uint64_t*)mem;
  uint64_t* keys2 = (uint64_t*)(mem + a256(8 * n));
  uint64_t* ukeys = (uint64_t*)(mem + 2 * a256(8 * n));
  char* p4 = mem + 3 * a256(8 * n);
  int32_t* perm = (int32_t*)p4;
  int32_t* perm2 = (int32_t*)(p4 + a256(4 * n));
  int32_t* head = (int32_t*)(p4 + 2 * a256(4 * n));
  int32_t* pos = (int32_t*)(p4 + 3 * a256(4 * n));
  int* bad = (int*)(p4 + 4 * a256(4 * n));
  void* cub_tmp = p4 + 4 * a256(4 * n) + 256;
  size_t cb = cub_bytes;
  int rc = FGB_OK;
  e = cudaMemsetAsync(bad, 0, sizeof(int), s);
  if (e == cudaSuccess) {
    if (idx_t == FGB_I32)
      coo_keys_k<int32_t><<<grid_n, 256, 0, s>>>(n_in, (const int32_t*)I, (const int32_t*)J, in_base, nrows,
                                                 ncols, csc ? 1 : 0, keys, perm, bad);
    else
      coo_keys_k<int64_t><<<grid_n, 256, 0, s>>>(n_in, (const int64_t*)I, (const int64_t*)J, in_base, nrows,
                                                 ncols, csc ? 1 : 0, keys, perm, bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cub::DeviceRadixSort::SortPairs(cub_tmp, cb, keys, keys2, perm, perm2, (int)n, 0, end_bit, s);
  if (e == cudaSuccess) {
    coo_heads_k<<<grid_n, 256, 0, s>>>(n_in, keys2, head);
    e = cudaGetLastError();
  }
  cb = cub_bytes;
  if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(cub_tmp, cb, head, pos, (int)n, s);
  if (e == cudaSuccess) {
    const void* v = val;
    void* ov = const_cast<void*>(out->val);
    switch (pattern ? FGB_NONE : val_t) {
      case FGB_NONE:
        coo_fold_k<uint8_t, FGB_COMBINE_LAST, true><<<grid_n, 256, 0, s>>>(
            n_in, keys2, perm2, head, pos, nullptr, (uint64_t)inner, ob, (int32_t*)out->idx, nullptr, ukeys);
        break;
      case FGB_F64: launch_fold<double, false>(combine, grid_n, s, n_in, keys2, perm2, head, pos, v, inner, ob, (int32_t*)out->idx, ov, ukeys); break;
      case FGB_F32: launch_fold<float, false>(combine, grid_n, s, n_in, keys2, perm2, head, pos, v, inner, ob, (int32_t*)out->idx, ov, ukeys); break;
      case FGB_I32: launch_fold<int32_t, false>(combine, grid_n, s, n_in, keys2, perm2, head, pos, v, inner, ob, (int32_t*)out->idx, ov, ukeys); break;
      case FGB_I64: launch_fold<int64_t, false>(combine, grid_n, s, n_in, keys2, perm2, head, pos, v, inner, ob, (int32_t*)out->idx, ov, ukeys); break;
      case FGB_BOOL:
        if (combine == FGB_COMBINE_OR)
          coo_fold_k<uint8_t, FGB_COMBINE_OR, false><<<grid_n, 256, 0, s>>>(
              n_in, keys2, perm2, head, pos, (const uint8_t*)v, (uint64_t)inner, ob, (int32_t*)out->idx,
              (uint8_t*)ov, ukeys);
        else
          launch_fold<uint8_t, false>(combine, grid_n, s, n_in, keys2, perm2, head, pos, v, inner, ob, (int32_t*)out->idx, ov, ukeys);
        break;
      default: rc = set_error(FGB_EUNSUPPORTED, "fgb_coo_assemble: value type %d", val_t);
    }
    e = cudaGetLastError();
  }
  int32_t tail[2] = {0, 0};
  int bad_h = 0;
  if (e == cudaSuccess && rc == FGB_OK) {
    e = cudaMemcpyAsync(&tail[0], pos + n - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&tail[1], head + n - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad_h, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  const int64_t nnz = (int64_t)tail[0] + tail[1];
  if (e == cudaSuccess && rc == FGB_OK && !bad_h) {
    if (out->ptr_t == FGB_I32 && nnz + ob > INT32_MAX) {
      rc = set_error(FGB_EUNSUPPORTED, "fgb_coo_assemble: %lld entries need 64-bit ptr", (long long)nnz);
    } else {
      if (out->ptr_t == FGB_I32)
        coo_ptr_k<int32_t><<<grid_f, 256, 0, s>>>(nfib, ukeys, nnz, (uint64_t)inner, ob, (int32_t*)out->ptr);
      else
        coo_ptr_k<int64_t><<<grid_f, 256, 0, s>>>(nfib, ukeys, nnz, (uint64_t)inner, ob, (int64_t*)out->ptr);
      e = cudaGetLastError();
    }
  }
  cudaFreeAsync(mem, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(FGB_ECUDA, "fgb_coo_assemble: %s", cudaGetErrorString(e));
  if (rc) return rc;
  if (bad_h) return set_error(FGB_EINVAL, "fgb_coo_assemble: a coordinate lies outside %lld x %lld",
                              (long long)nrows, (long long)ncols);
  *nnz_out = nnz;
  out->nnz = nnz;
  return FGB_OK;
}
