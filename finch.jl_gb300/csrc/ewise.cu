// Elementwise ops of two SparseList matrices and the fused
// elementwise-multiply + reduction.
//
// C = A .* B / A .+ B: one thread per fiber runs Finch's two-finger merge of
// the two sorted coordinate lists (test/reference64/typical/
// typical_merge_twofinger.txt: advance the smaller coordinate, emit on a
// match).  Pass 1 counts each output fiber and an exclusive scan turns the
// counts into out_ptr; pass 2 re-runs the merge and writes idx/val.
//
// sum(A .* B; dims): every fiber is reduced by a group of lanes (dense B) or
// one merging thread (sparse B).  Reductions along the compressed coordinate
// scatter into y with atomics; the all-dims reduction writes one partial per
// fiber and folds them in a fixed order, so it is deterministic.
#include <cub/cub.cuh>

#include "fgb_internal.cuh"
#include "semiring.cuh"

namespace fgb {

template <class PtrT>
struct Fiber {
  const PtrT* ptr;
  const int* idx;
  int base;
  __device__ int64_t lo(int64_t f) const { return ld_ptr(ptr, f) - base; }
  __device__ int64_t hi(int64_t f) const { return ld_ptr(ptr, f + 1) - base; }
  __device__ int at(int64_t p) const { return __ldg(idx + p) - base; }
};

template <class PA, class PB>
__global__ void ewise_count_k(int64_t nf, Fiber<PA> a, Fiber<PB> b, int op, int64_t* __restrict__ cnt) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
       f += (int64_t)gridDim.x * blockDim.x) {
    int64_t pa = a.lo(f), ea = a.hi(f), pb = b.lo(f), eb = b.hi(f);
    int64_t n = 0;
    if (op == FGB_EW_MUL) {
      while (pa < ea && pb < eb) {
        const int ia = a.at(pa), ib = b.at(pb);
        n += (ia == ib);
        pa += (ia <= ib);
        pb += (ib <= ia);
      }
    } else {
      while (pa < ea && pb < eb) {
        const int ia = a.at(pa), ib = b.at(pb);
        ++n;
        pa += (ia <= ib);
        pb += (ib <= ia);
      }
      n += (ea - pa) + (eb - pb);
    }
    cnt[f] = n;
  }
}

template <class T, class PA, class PB>
__global__ void ewise_fill_k(int64_t nf, Fiber<PA> a, const T* __restrict__ va, Fiber<PB> b,
                             const T* __restrict__ vb, int op, const int64_t* __restrict__ optr,
                             int32_t* __restrict__ oidx, T* __restrict__ oval) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
       f += (int64_t)gridDim.x * blockDim.x) {
    int64_t pa = a.lo(f), ea = a.hi(f), pb = b.lo(f), eb = b.hi(f);
    int64_t q = optr[f];
    if (op == FGB_EW_MUL) {
      while (pa < ea && pb < eb) {
        const int ia = a.at(pa), ib = b.at(pb);
        if (ia == ib) {
          oidx[q] = ia;
          oval[q] = wmul(va[pa], vb[pb]);
          ++q;
        }
        pa += (ia <= ib);
        pb += (ib <= ia);
      }
    } else {
      while (pa < ea || pb < eb) {
        const int ia = pa < ea ? a.at(pa) : INT32_MAX;
        const int ib = pb < eb ? b.at(pb) : INT32_MAX;
        if (ia == ib) {
          oidx[q] = ia;
          oval[q] = wadd(va[pa], vb[pb]);
          ++pa;
          ++pb;
        } else if (ia < ib) {
          oidx[q] = ia;
          oval[q] = va[pa];
          ++pa;
        } else {
          oidx[q] = ib;
          oval[q] = vb[pb];
          ++pb;
        }
        ++q;
      }
    }
  }
}

// ---- fused elementwise multiply + reduce

// Per-fiber sums, sparse B (merge), one thread per fiber, j ascending.
template <class T, class PA, class PB>
__global__ void reduce_fiber_sparse(int64_t nf, Fiber<PA> a, const T* __restrict__ va, Fiber<PB> b,
                                    const T* __restrict__ vb, T* __restrict__ y) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
       f += (int64_t)gridDim.x * blockDim.x) {
    int64_t pa = a.lo(f), ea = a.hi(f), pb = b.lo(f), eb = b.hi(f);
    T acc = T(0);
    while (pa < ea && pb < eb) {
      const int ia = a.at(pa), ib = b.at(pb);
      if (ia == ib) acc = fused(va[pa], vb[pb], acc);
      pa += (ia <= ib);
      pb += (ib <= ia);
    }
    y[f] = acc;
  }
}

// Per-fiber sums, dense B, G lanes per fiber.
template <int G, class T, class PA>
__global__ void reduce_fiber_dense(int64_t nf, Fiber<PA> a, const T* __restrict__ va,
                                   const T* __restrict__ D, int64_t ld, int csr, T* __restrict__ y) {
  const int lane = threadIdx.x & (G - 1);
  const int64_t group = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
  for (int64_t f = group; f < nf; f += ngroups) {
    T acc = T(0);
    for (int64_t p = a.lo(f) + lane; p < a.hi(f); p += G) {
      const int64_t c = a.at(p);
      const T d = !D ? T(1) : csr ? __ldg(D + f * ld + c) : __ldg(D + c * ld + f);
      acc = fused(va[p], d, acc);
    }
#pragma unroll
    for (int m = G / 2; m >= 1; m >>= 1) acc += __shfl_xor_sync(group_mask<G>(), acc, m, G);
    if (lane == 0) y[f] = acc;
  }
}

// Scatter sums along the compressed coordinate: y[c] += A[f,c] * B[f,c].
template <class T, class PA, class PB>
__global__ void reduce_scatter_sparse(int64_t nf, Fiber<PA> a, const T* __restrict__ va, Fiber<PB> b,
                                      const T* __restrict__ vb, T* __restrict__ y) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
       f += (int64_t)gridDim.x * blockDim.x) {
    int64_t pa = a.lo(f), ea = a.hi(f), pb = b.lo(f), eb = b.hi(f);
    while (pa < ea && pb < eb) {
      const int ia = a.at(pa), ib = b.at(pb);
      if (ia == ib) atomicAdd(y + ia, wmul(va[pa], vb[pb]));
      pa += (ia <= ib);
      pb += (ib <= ia);
    }
  }
}

template <class T, class PA>
__global__ void reduce_scatter_dense(int64_t nf, Fiber<PA> a, const T* __restrict__ va,
                                     const T* __restrict__ D, int64_t ld, int csr, T* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t f = w; f < nf; f += nw)
    for (int64_t p = a.lo(f) + lane; p < a.hi(f); p += 32) {
      const int64_t c = a.at(p);
      const T d = !D ? T(1) : csr ? __ldg(D + f * ld + c) : __ldg(D + c * ld + f);
      atomicAdd(y + c, wmul(va[p], d));
    }
}

// Deterministic fold of n partials into out[0] with one block.
template <class T>
__global__ void fold_partials(const T* __restrict__ part, int64_t n, T* __restrict__ out) {
  __shared__ T sh[1024];
  T acc = T(0);
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sh[0];
}

template <class T>
__global__ void zero_vec(T* y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = T(0);
}

// Counts for reduce(+, A; dims) of a Pattern (every stored entry is true)
// or Bool matrix: Julia sums Bools into Int64.  v NULL for a Pattern.
template <class P>
__global__ void count_fiber_k(int64_t nf, Fiber<P> a, const unsigned char* __restrict__ v,
                              long long* __restrict__ out) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf;
       f += (int64_t)gridDim.x * blockDim.x) {
    const int64_t lo = a.lo(f), hi = a.hi(f);
    long long c = 0;
    if (!v) c = hi - lo;
    else
      for (int64_t p = lo; p < hi; ++p) c += v[p] ? 1 : 0;
    out[f] = c;
  }
}

template <class P>
__global__ void count_scatter_k(int64_t nnz, Fiber<P> a, const unsigned char* __restrict__ v,
                                unsigned long long* __restrict__ out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz;
       p += (int64_t)gridDim.x * blockDim.x)
    if (!v || v[p]) atomicAdd(out + a.at(p), 1ull);
}

template <class P>
static Fiber<P> fiber_of(const fgb_sparse* A) {
  return Fiber<P>{(const P*)A->ptr, (const int*)A->idx, A->index_base};
}

// Calls fn(Fiber<PA>, Fiber<PB>) with both ptr widths resolved.
template <class F>
static int with_fibers(const fgb_sparse* A, const fgb_sparse* B, F&& fn) {
  if (A->ptr_t == FGB_I32) {
    if (!B || B->ptr_t == FGB_I32) return fn(fiber_of<int32_t>(A), B ? fiber_of<int32_t>(B) : Fiber<int32_t>{});
    return fn(fiber_of<int32_t>(A), fiber_of<int64_t>(B));
  }
  if (!B || B->ptr_t == FGB_I32) return fn(fiber_of<int64_t>(A), B ? fiber_of<int32_t>(B) : Fiber<int32_t>{});
  return fn(fiber_of<int64_t>(A), fiber_of<int64_t>(B));
}

static int check_pair(const fgb_sparse* A, const fgb_sparse* B, const char* who) {
  int rc = check_sparse(A, who, true);
  if (rc) return rc;
  rc = check_sparse(B, who, true);
  if (rc) return rc;
  if (A->nrows != B->nrows || A->ncols != B->ncols)
    return set_error(FGB_EINVAL, "%s: shape mismatch (%lld x %lld vs %lld x %lld)", who,
                     (long long)A->nrows, (long long)A->ncols, (long long)B->nrows,
                     (long long)B->ncols);
  if (A->orient != B->orient) return set_error(FGB_EINVAL, "%s: operands differ in orientation", who);
  if (A->val_t != B->val_t) return set_error(FGB_EUNSUPPORTED, "%s: operands differ in dtype", who);
  return FGB_OK;
}

}  // namespace fgb

using namespace fgb;

extern "C" {

int fgb_ewise_count(fgb_ctx* ctx, int op, const fgb_sparse* A, const fgb_sparse* B,
                    int64_t* out_ptr, int64_t* out_nnz, void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_ewise_count: null ctx");
  if (op != FGB_EW_MUL && op != FGB_EW_ADD) return set_error(FGB_EINVAL, "fgb_ewise_count: bad op");
  int rc = check_pair(A, B, "fgb_ewise_count");
  if (rc) return rc;
  if (!out_ptr || !out_nnz) return set_error(FGB_EINVAL, "fgb_ewise_count: null output");
  cudaStream_t s = pick_stream(ctx, stream);
  const int64_t nf = n_fibers(A);
  FGB_CUDA_TRY(cudaMemsetAsync(out_ptr, 0, sizeof(int64_t), s));
  if (nf > 0) {
    size_t tmp_bytes = 0;
    int64_t* counts = nullptr;
    cub::DeviceScan::InclusiveSum(nullptr, tmp_bytes, counts, out_ptr + 1, nf, s);
    void* tmp = nullptr;
    FGB_CUDA_TRY(cudaMallocAsync((void**)&counts, sizeof(int64_t) * nf + tmp_bytes, s));
    tmp = counts + nf;
    rc = with_fibers(A, B, [&](auto fa, auto fb) {
      ewise_count_k<<<grid_for(nf, 256, ctx->num_sms, 8), 256, 0, s>>>(nf, fa, fb, op, counts);
      return check_launch("ewise_count_k");
    });
    if (rc == FGB_OK) {
      cub::DeviceScan::InclusiveSum(tmp, tmp_bytes, counts, out_ptr + 1, nf, s);
      rc = check_launch("DeviceScan");
    }
    cudaFreeAsync(counts, s);
    if (rc) return rc;
  }
  FGB_CUDA_TRY(cudaMemcpyAsync(out_nnz, out_ptr + nf, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  FGB_CUDA_TRY(cudaStreamSynchronize(s));
  return FGB_OK;
}

int fgb_ewise_fill(fgb_ctx* ctx, int op, const fgb_sparse* A, const fgb_sparse* B,
                   const int64_t* out_ptr, int32_t* out_idx, void* out_val, void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_ewise_fill: null ctx");
  if (op != FGB_EW_MUL && op != FGB_EW_ADD) return set_error(FGB_EINVAL, "fgb_ewise_fill: bad op");
  int rc = check_pair(A, B, "fgb_ewise_fill");
  if (rc) return rc;
  const int64_t nf = n_fibers(A);
  if (nf == 0) return FGB_OK;
  if (!out_ptr) return set_error(FGB_EINVAL, "fgb_ewise_fill: null out_ptr");
  cudaStream_t s = pick_stream(ctx, stream);
  const int grid = grid_for(nf, 256, ctx->num_sms, 8);
  return with_fibers(A, B, [&](auto fa, auto fb) {
    switch (A->val_t) {
      case FGB_F64:
        ewise_fill_k<<<grid, 256, 0, s>>>(nf, fa, (const double*)A->val, fb, (const double*)B->val, op,
                                          out_ptr, out_idx, (double*)out_val);
        break;
      case FGB_F32:
        ewise_fill_k<<<grid, 256, 0, s>>>(nf, fa, (const float*)A->val, fb, (const float*)B->val, op,
                                          out_ptr, out_idx, (float*)out_val);
        break;
      case FGB_I32:
        ewise_fill_k<<<grid, 256, 0, s>>>(nf, fa, (const int32_t*)A->val, fb, (const int32_t*)B->val, op,
                                          out_ptr, out_idx, (int32_t*)out_val);
        break;
      case FGB_I64:
        ewise_fill_k<<<grid, 256, 0, s>>>(nf, fa, (const int64_t*)A->val, fb, (const int64_t*)B->val, op,
                                          out_ptr, out_idx, (int64_t*)out_val);
        break;
      default: return set_error(FGB_EUNSUPPORTED, "fgb_ewise_fill: dtype %d", A->val_t);
    }
    return check_launch("ewise_fill_k");
  });
}

int fgb_ewise_reduce(fgb_ctx* ctx, int dims, const fgb_sparse* A, const fgb_sparse* B,
                     const void* B_dense, int64_t ldb, void* y, int dtype, unsigned flags,
                     void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_ewise_reduce: null ctx");
  if (dims < 0 || dims > 2) return set_error(FGB_EINVAL, "fgb_ewise_reduce: dims must be 0, 1 or 2");
  int rc = B ? check_pair(A, B, "fgb_ewise_reduce") : check_sparse(A, "fgb_ewise_reduce: A", true);
  if (rc) return rc;
  if (!B && B_dense && ldb < A->ncols) return set_error(FGB_EINVAL, "fgb_ewise_reduce: ldb < ncols");
  if (!B && !B_dense && (A->val_t == FGB_NONE || A->val_t == FGB_BOOL) && dtype == FGB_I64) {
    // reduce(+, A; dims) of a Pattern or Bool matrix: Int64 counts
    if (!y) return set_error(FGB_EINVAL, "fgb_ewise_reduce: null y");
    cudaStream_t s = pick_stream(ctx, stream);
    const int64_t nf = n_fibers(A);
    const bool per_fiber = dims == 0 || (A->orient == FGB_CSR ? dims == 2 : dims == 1);
    const int64_t out_len = dims == 0 ? 1 : (dims == 2 ? A->nrows : A->ncols);
    const unsigned char* v = A->val_t == FGB_BOOL ? (const unsigned char*)A->val : nullptr;
    if (!per_fiber || nf == 0)
      FGB_CUDA_TRY(cudaMemsetAsync(y, 0, sizeof(long long) * out_len, s));
    if (!per_fiber)
      return with_fibers(A, nullptr, [&](auto fa, auto) {
        count_scatter_k<<<grid_for(A->nnz, 256, ctx->num_sms, 8), 256, 0, s>>>(A->nnz, fa, v,
                                                                                 (unsigned long long*)y);
        return check_launch("count_scatter");
      });
    if (nf == 0) return FGB_OK;
    long long* target = (long long*)y;
    if (dims == 0) FGB_CUDA_TRY(cudaMallocAsync((void**)&target, sizeof(long long) * nf, s));
    rc = with_fibers(A, nullptr, [&](auto fa, auto) {
      count_fiber_k<<<grid_for(nf, 256, ctx->num_sms, 8), 256, 0, s>>>(nf, fa, v, target);
      return check_launch("count_fiber");
    });
    if (rc == FGB_OK && dims == 0) {
      fold_partials<long long><<<1, 1024, 0, s>>>(target, nf, (long long*)y);
      rc = check_launch("fold_partials");
    }
    if (target != (long long*)y) cudaFreeAsync(target, s);
    return rc;
  }
  if (A->val_t != dtype) return set_error(FGB_EUNSUPPORTED, "fgb_ewise_reduce: A dtype != dtype");
  if (dtype != FGB_F32 && dtype != FGB_F64)
    return set_error(FGB_EUNSUPPORTED, "fgb_ewise_reduce: dtype %d", dtype);
  if (!y) return set_error(FGB_EINVAL, "fgb_ewise_reduce: null y");
  cudaStream_t s = pick_stream(ctx, stream);
  const int64_t nf = n_fibers(A);
  const bool csr = A->orient == FGB_CSR;
  // per-fiber reduction when the reduced dimension is the uncompressed one
  const bool per_fiber = dims == 0 || (csr ? dims == 2 : dims == 1);
  const int64_t out_len = dims == 0 ? 1 : (dims == 2 ? A->nrows : A->ncols);
  const size_t esz = dtype == FGB_F64 ? 8 : 4;
  void* target = y;
  if (dims == 0 && nf > 0) FGB_CUDA_TRY(cudaMallocAsync(&target, nf * esz, s));
  const int grid = grid_for(nf * 8, 256, ctx->num_sms, 8);
  auto body = [&](auto tag) -> int {
    using T = decltype(tag);
    const T* va = (const T*)A->val;
    if (!per_fiber) {
      zero_vec<T><<<grid_for(out_len, 256, ctx->num_sms, 4), 256, 0, s>>>((T*)y, out_len);
      return with_fibers(A, B, [&](auto fa, auto fb) {
        if (B)
          reduce_scatter_sparse<<<grid_for(nf, 256, ctx->num_sms, 8), 256, 0, s>>>(nf, fa, va, fb, (const T*)B->val, (T*)y);
        else
          reduce_scatter_dense<<<grid_for(nf * 32, 256, ctx->num_sms, 8), 256, 0, s>>>(nf, fa, va, (const T*)B_dense, ldb, csr ? 1 : 0, (T*)y);
        return check_launch("reduce_scatter");
      });
    }
    if (nf == 0) {
      zero_vec<T><<<1, 32, 0, s>>>((T*)y, out_len);
      return check_launch("zero_vec");
    }
    int r = with_fibers(A, B, [&](auto fa, auto fb) {
      if (B)
        reduce_fiber_sparse<<<grid_for(nf, 256, ctx->num_sms, 8), 256, 0, s>>>(nf, fa, va, fb, (const T*)B->val, (T*)target);
      else
        reduce_fiber_dense<8><<<grid, 256, 0, s>>>(nf, fa, va, (const T*)B_dense, ldb, csr ? 1 : 0, (T*)target);
      return check_launch("reduce_fiber");
    });
    if (r) return r;
    if (dims == 0) {
      fold_partials<T><<<1, 1024, 0, s>>>((const T*)target, nf, (T*)y);
      return check_launch("fold_partials");
    }
    return FGB_OK;
  };
  rc = dtype == FGB_F64 ? body(double(0)) : body(float(0));
  if (target != y) cudaFreeAsync(target, s);
  (void)flags;
  return rc;
}

}  // extern "C"
