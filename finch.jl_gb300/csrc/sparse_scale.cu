// Stored entries of a sparse matrix combined with a dense vector over one
// of its indices and filtered by another: the masked broadcast that builds
// PageRank's transition matrix (docs/examples/pagerank.jl:17-25)
//
//     for j=_, i=_; if keep[k] != 0; out[i, j] = A[i, j] / by[l]; end; end
//
// Kept entries stay in A's order.  Each entry gets a keep flag; an
// exclusive scan of the flags is its position in the result, and a fiber's
// new ptr is the scan at the fiber's first entry, the prefix sum SparseList
// assembly uses (src/tensors/levels/sparse_list_levels.jl:310-327).
#include <cub/cub.cuh>

#include "fgb_internal.cuh"

namespace fgb {

// A value of type t at element i, widened to T.  t is FGB_NONE for a
// Pattern (every stored entry is true = 1).
template <class T>
__device__ __forceinline__ T load_as(const void* p, int t, int64_t i) {
  switch (t) {
    case FGB_F64: return (T)((const double*)p)[i];
    case FGB_F32: return (T)((const float*)p)[i];
    case FGB_I64: return (T)((const long long*)p)[i];
    case FGB_I32: return (T)((const int*)p)[i];
    case FGB_BOOL: return ((const unsigned char*)p)[i] ? T(1) : T(0);
    default: return T(1);
  }
}

// x != 0 for an element of type t (NaN != 0 is true, as in Julia).
__device__ __forceinline__ bool nonzero_at(const void* p, int t, int64_t i) {
  switch (t) {
    case FGB_F64: return ((const double*)p)[i] != 0.0;
    case FGB_F32: return ((const float*)p)[i] != 0.0f;
    case FGB_I64: return ((const long long*)p)[i] != 0;
    case FGB_I32: return ((const int*)p)[i] != 0;
    default: return ((const unsigned char*)p)[i] != 0;
  }
}

// Whether 0 op by[l] differs from 0 (0/0, 0/NaN; 0*Inf, 0*NaN): the fill
// of A turned into something else where A stores nothing.
__device__ __forceinline__ bool changes_fill(const void* p, int t, int64_t l, int op) {
  if (t != FGB_F64 && t != FGB_F32) return op == FGB_MAP_DIV && !nonzero_at(p, t, l);
  const double b = t == FGB_F64 ? ((const double*)p)[l] : (double)((const float*)p)[l];
  if (op == FGB_MAP_DIV) return b == 0.0 || isnan(b);
  return isinf(b) || isnan(b);
}

__global__ void count_fill_changed(int64_t n, const void* by, int by_t, int op,
                                   unsigned long long* count) {
  unsigned long long mine = 0;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x)
    mine += changes_fill(by, by_t, l, op) ? 1ull : 0ull;
  for (int m = 16; m >= 1; m >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, m);
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(count, mine);
}

// Fiber of entry p: the largest f with ptr[f] - base <= p.
template <class PtrT>
__device__ __forceinline__ int64_t fiber_of(const PtrT* __restrict__ ptr, int64_t nf, int base, int64_t p) {
  int64_t lo = 0, hi = nf;
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (ld_ptr(ptr, mid) - base <= p) lo = mid;
    else hi = mid;
  }
  return lo;
}

struct ScaleArgs {
  int64_t nnz, nf;
  int base, csc, op, by_axis, by_t, keep_axis, keep_t, val_t, out_t;
  const int* idx;
  const void *val, *by, *keep;
};

// flag[p] = 1 when entry p is kept (flag[nnz] = 0 closes the scan).
template <class PtrT>
__global__ void scale_flags(ScaleArgs a, const PtrT* __restrict__ ptr, int64_t* __restrict__ flag) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p <= a.nnz;
       p += (int64_t)gridDim.x * blockDim.x) {
    if (p == a.nnz) {
      flag[p] = 0;
      continue;
    }
    if (!a.keep) {
      flag[p] = 1;
      continue;
    }
    const int64_t f = fiber_of(ptr, a.nf, a.base, p);
    const int64_t c = (int64_t)__ldg(a.idx + p) - a.base;
    const int64_t i = a.csc ? c : f, j = a.csc ? f : c;
    flag[p] = nonzero_at(a.keep, a.keep_t, a.keep_axis == FGB_AXIS_ROW ? i : j) ? 1 : 0;
  }
}

template <class T>
__device__ __forceinline__ T combine(T v, T b, int op) {
  return op == FGB_MAP_DIV ? v / b : v * b;
}

template <class PtrT>
__global__ void scale_write(ScaleArgs a, const PtrT* __restrict__ ptr, const int64_t* __restrict__ flag,
                            const int64_t* __restrict__ pos, int32_t* __restrict__ out_idx,
                            void* __restrict__ out_val, bool in_f32) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.nnz;
       p += (int64_t)gridDim.x * blockDim.x) {
    if (!flag[p]) continue;
    const int64_t f = fiber_of(ptr, a.nf, a.base, p);
    const int c = __ldg(a.idx + p) - a.base;
    const int64_t i = a.csc ? c : f, j = a.csc ? f : c;
    const int64_t l = a.by_axis == FGB_AXIS_ROW ? i : j;
    const int64_t q = pos[p];
    out_idx[q] = c;
    if (in_f32) {  // Julia's promotion: F32 with F32 or an integer stays F32
      const float r = combine(load_as<float>(a.val, a.val_t, p), load_as<float>(a.by, a.by_t, l), a.op);
      if (a.out_t == FGB_F32) ((float*)out_val)[q] = r;
      else ((double*)out_val)[q] = (double)r;
    } else {
      const double r = combine(load_as<double>(a.val, a.val_t, p), load_as<double>(a.by, a.by_t, l), a.op);
      if (a.out_t == FGB_F32) ((float*)out_val)[q] = (float)r;
      else ((double*)out_val)[q] = r;
    }
  }
}

// out_ptr[f] = pos[ptr[f] - base] for f <= nf: pos[nnz] is the kept count.
template <class PtrT>
__global__ void scale_ptr(int64_t nf, const PtrT* __restrict__ ptr, int base, const int64_t* __restrict__ pos,
                          int64_t* __restrict__ out_ptr) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f <= nf; f += (int64_t)gridDim.x * blockDim.x)
    out_ptr[f] = pos[ld_ptr(ptr, f) - base];
}

static bool value_type_ok(int t) {
  return t == FGB_F64 || t == FGB_F32 || t == FGB_I64 || t == FGB_I32 || t == FGB_BOOL;
}

template <class PtrT>
static int sparse_scale_typed(fgb_ctx* ctx, const fgb_sparse* A, const ScaleArgs& a, int64_t* out_ptr,
                              int32_t* out_idx, void* out_val, int64_t* out_nnz, bool in_f32,
                              cudaStream_t s) {
  const PtrT* ptr = (const PtrT*)A->ptr;
  int64_t *flag = nullptr, *pos = nullptr;
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, flag, pos, a.nnz + 1, s);
  int rc = FGB_OK;
  cudaError_t e = cudaMallocAsync((void**)&flag, sizeof(int64_t) * (a.nnz + 1) * 2, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&tmp, tmp_bytes, s);
  if (e != cudaSuccess) {
    rc = set_error(FGB_ENOMEM, "fgb_sparse_scale: scratch allocation failed: %s", cudaGetErrorString(e));
  } else {
    pos = flag + (a.nnz + 1);
    const int grid = grid_for(a.nnz + 1, 256, ctx->num_sms, 8);
    scale_flags<PtrT><<<grid, 256, 0, s>>>(a, ptr, flag);
    cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, flag, pos, a.nnz + 1, s);
    scale_write<PtrT><<<grid, 256, 0, s>>>(a, ptr, flag, pos, out_idx, out_val, in_f32);
    scale_ptr<PtrT><<<grid_for(a.nf + 1, 256, ctx->num_sms, 8), 256, 0, s>>>(a.nf, ptr, a.base, pos, out_ptr);
    rc = check_launch("fgb_sparse_scale");
    if (rc == FGB_OK) {
      e = cudaMemcpyAsync(out_nnz, pos + a.nnz, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) rc = set_error(FGB_ECUDA, "fgb_sparse_scale: %s", cudaGetErrorString(e));
    }
  }
  if (flag) cudaFreeAsync(flag, s);
  if (tmp) cudaFreeAsync(tmp, s);
  cudaError_t se = cudaStreamSynchronize(s);
  if (rc == FGB_OK && se != cudaSuccess) rc = set_error(FGB_ECUDA, "fgb_sparse_scale: %s", cudaGetErrorString(se));
  return rc;
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_sparse_scale(fgb_ctx* ctx, const fgb_sparse* A, int op, int by_axis, int by_t, const void* by,
                                int keep_axis, int keep_t, const void* keep, int out_t, int64_t* out_ptr,
                                int32_t* out_idx, void* out_val, int64_t* out_nnz, int64_t* n_fill_changed,
                                void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_sparse_scale: null ctx");
  int rc = check_sparse(A, "fgb_sparse_scale: A", true);
  if (rc) return rc;
  if (op != FGB_MAP_DIV && op != FGB_MAP_MUL)
    return set_error(FGB_EINVAL, "fgb_sparse_scale: op must be FGB_MAP_MUL or FGB_MAP_DIV");
  if ((by_axis != FGB_AXIS_ROW && by_axis != FGB_AXIS_COL) || (keep && keep_axis != FGB_AXIS_ROW &&
                                                               keep_axis != FGB_AXIS_COL))
    return set_error(FGB_EINVAL, "fgb_sparse_scale: axes must be FGB_AXIS_ROW or FGB_AXIS_COL");
  if (!by || !value_type_ok(by_t) || (keep && !value_type_ok(keep_t)))
    return set_error(FGB_EINVAL, "fgb_sparse_scale: by (and keep) must be F64, F32, I64, I32 or BOOL vectors");
  if (!value_type_ok(A->val_t) && A->val_t != FGB_NONE)
    return set_error(FGB_EUNSUPPORTED, "fgb_sparse_scale: A's values must be F64, F32, I64, I32, BOOL or none");
  if (out_t != FGB_F64 && out_t != FGB_F32)
    return set_error(FGB_EINVAL, "fgb_sparse_scale: out_t must be FGB_F64 or FGB_F32");
  if (!out_ptr || !out_nnz || (A->nnz > 0 && (!out_idx || !out_val)))
    return set_error(FGB_EINVAL, "fgb_sparse_scale: null output buffer");
  cudaStream_t s = pick_stream(ctx, stream);
  const int64_t by_len = by_axis == FGB_AXIS_ROW ? A->nrows : A->ncols;
  if (n_fill_changed) {
    *n_fill_changed = 0;
    if (by_len > 0) {
      unsigned long long* cnt = nullptr;
      FGB_CUDA_TRY(cudaMallocAsync((void**)&cnt, sizeof(unsigned long long), s));
      cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s);
      if (e == cudaSuccess) {
        count_fill_changed<<<grid_for(by_len, 256, ctx->num_sms, 4), 256, 0, s>>>(by_len, by, by_t, op, cnt);
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaMemcpyAsync(n_fill_changed, cnt, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
      cudaFreeAsync(cnt, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return set_error(FGB_ECUDA, "fgb_sparse_scale: %s", cudaGetErrorString(e));
    }
  }
  ScaleArgs a{};
  a.nnz = A->nnz;
  a.nf = n_fibers(A);
  a.base = A->index_base;
  a.csc = A->orient == FGB_CSC;
  a.op = op;
  a.by_axis = by_axis;
  a.by_t = by_t;
  a.keep_axis = keep_axis;
  a.keep_t = keep_t;
  a.val_t = A->val_t;
  a.out_t = out_t;
  a.idx = (const int*)A->idx;
  a.val = A->val;
  a.by = by;
  a.keep = keep;
  const bool f32_in = (A->val_t == FGB_F32 || by_t == FGB_F32) && A->val_t != FGB_F64 && by_t != FGB_F64;
  if (A->ptr_t == FGB_I32)
    return sparse_scale_typed<int32_t>(ctx, A, a, out_ptr, out_idx, out_val, out_nnz, f32_in, s);
  return sparse_scale_typed<int64_t>(ctx, A, a, out_ptr, out_idx, out_val, out_nnz, f32_in, s);
}
