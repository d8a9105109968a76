// Level-format conversion on the device: stable CSC <-> CSR transpose.
//
// The entries of A arrive ordered by (fiber f, coordinate c).  A stable
// radix sort of the coordinates, carrying each entry's position, orders them
// by (c, f): exactly the order of the transposed SparseList, with every new
// fiber's coordinates ascending (Finch's SparseList invariant,
// src/tensors/levels/sparse_list_levels.jl:37-53).  The new ptr comes from a
// histogram of c and an exclusive scan, like SparseList's freeze_level!
// prefix sum (sparse_list_levels.jl:310-327).
#include <cub/cub.cuh>

#include "fgb_internal.cuh"

namespace fgb {

template <class PtrT>
__global__ void expand_keys(int64_t nnz, const int* __restrict__ idx, int base,
                            uint32_t* __restrict__ keys, int64_t* __restrict__ pos,
                            unsigned long long* __restrict__ hist) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int c = __ldg(idx + p) - base;
    keys[p] = c;
    pos[p] = p;
    atomicAdd(hist + c, 1ull);
  }
}

template <class PtrT>
__global__ void gather_transposed(int64_t nnz, int64_t nf, const PtrT* __restrict__ ptr, int base,
                                  const int64_t* __restrict__ perm, const char* __restrict__ val,
                                  int esz, int32_t* __restrict__ out_idx,
                                  char* __restrict__ out_val) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = perm[q];
    // fiber of entry p: largest f with ptr[f] - base <= p
    int64_t lo = 0, hi = nf;
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (ld_ptr(ptr, mid) - base <= p) lo = mid; else hi = mid;
    }
    out_idx[q] = (int32_t)lo;
    if (val) {
      switch (esz) {
        case 8: ((int64_t*)out_val)[q] = ((const int64_t*)val)[p]; break;
        case 4: ((int32_t*)out_val)[q] = ((const int32_t*)val)[p]; break;
        case 2: ((int16_t*)out_val)[q] = ((const int16_t*)val)[p]; break;
        default: out_val[q] = val[p]; break;
      }
    }
  }
}

__global__ void hist_to_ptr_first(int64_t* out_ptr) { out_ptr[0] = 0; }

int dtype_size(int t) {
  switch (t) {
    case FGB_F64: case FGB_I64: return 8;
    case FGB_F32: case FGB_I32: return 4;
    case FGB_BF16: return 2;
    case FGB_BOOL: return 1;
    default: return 0;
  }
}

template <class PtrT>
static int transpose_typed(fgb_ctx* ctx, const fgb_sparse* A, int64_t* out_ptr, int32_t* out_idx,
                           void* out_val, cudaStream_t s) {
  const int64_t nnz = A->nnz;
  const int64_t nf = n_fibers(A);
  const int64_t ne = fiber_extent(A);
  const int base = A->index_base;
  // hist[c] counts coordinate c; out_ptr[1..ne] is its inclusive scan.
  FGB_CUDA_TRY(cudaMemsetAsync(out_ptr, 0, sizeof(int64_t), s));
  if (nnz == 0) {
    if (ne > 0) FGB_CUDA_TRY(cudaMemsetAsync(out_ptr + 1, 0, sizeof(int64_t) * ne, s));
    FGB_CUDA_TRY(cudaStreamSynchronize(s));
    return FGB_OK;
  }
  uint32_t *k_in = nullptr, *k_out = nullptr;
  int64_t *v_in = nullptr, *v_out = nullptr, *hist = nullptr;
  void* tmp = nullptr;
  size_t tmp_sort = 0, tmp_scan = 0;
  int end_bit = 1;
  while (end_bit < 31 && (int64_t(1) << end_bit) < ne) ++end_bit;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_sort, k_in, k_out, v_in, v_out, nnz, 0, end_bit, s);
  cub::DeviceScan::InclusiveSum(nullptr, tmp_scan, hist, out_ptr + 1, ne, s);
  const size_t tmp_bytes = tmp_sort > tmp_scan ? tmp_sort : tmp_scan;
  int rc = FGB_OK;
  cudaError_t e = cudaMallocAsync((void**)&k_in, sizeof(uint32_t) * nnz * 2, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&v_in, sizeof(int64_t) * nnz * 2, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&hist, sizeof(int64_t) * ne, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&tmp, tmp_bytes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(hist, 0, sizeof(int64_t) * ne, s);
  if (e != cudaSuccess) {
    rc = set_error(FGB_ENOMEM, "fgb_transpose: scratch allocation failed: %s", cudaGetErrorString(e));
  } else {
    k_out = k_in + nnz;
    v_out = v_in + nnz;
    const int grid = grid_for(nnz, 256, ctx->num_sms, 8);
    expand_keys<PtrT><<<grid, 256, 0, s>>>(nnz, (const int*)A->idx, base, k_in, v_in,
                                           (unsigned long long*)hist);
    cub::DeviceRadixSort::SortPairs(tmp, tmp_sort, k_in, k_out, v_in, v_out, nnz, 0, end_bit, s);
    cub::DeviceScan::InclusiveSum(tmp, tmp_scan, hist, out_ptr + 1, ne, s);
    const int esz = A->val_t == FGB_NONE ? 0 : dtype_size(A->val_t);
    gather_transposed<PtrT><<<grid, 256, 0, s>>>(nnz, nf, (const PtrT*)A->ptr, base, v_out,
                                                 esz ? (const char*)A->val : nullptr, esz, out_idx,
                                                 (char*)out_val);
    rc = check_launch("fgb_transpose");
  }
  if (k_in) cudaFreeAsync(k_in, s);
  if (hist) cudaFreeAsync(hist, s);
  if (v_in) cudaFreeAsync(v_in, s);
  if (tmp) cudaFreeAsync(tmp, s);
  cudaError_t se = cudaStreamSynchronize(s);
  if (rc == FGB_OK && se != cudaSuccess)
    rc = set_error(FGB_ECUDA, "fgb_transpose: %s", cudaGetErrorString(se));
  return rc;
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_transpose(fgb_ctx* ctx, const fgb_sparse* A, int64_t* out_ptr, int32_t* out_idx,
                             void* out_val, void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_transpose: null ctx");
  int rc = check_sparse(A, "fgb_transpose: A", true);
  if (rc) return rc;
  if (!out_ptr || (A->nnz > 0 && !out_idx) || (A->nnz > 0 && A->val_t != FGB_NONE && !out_val))
    return set_error(FGB_EINVAL, "fgb_transpose: null output buffer");
  if (n_fibers(A) > INT32_MAX)
    return set_error(FGB_EUNSUPPORTED, "fgb_transpose: %lld fibers exceed int32 coordinates",
                     (long long)n_fibers(A));
  cudaStream_t s = pick_stream(ctx, stream);
  if (A->ptr_t == FGB_I32) return transpose_typed<int32_t>(ctx, A, out_ptr, out_idx, out_val, s);
  return transpose_typed<int64_t>(ctx, A, out_ptr, out_idx, out_val, s);
}

namespace fgb {

// out = fill everywhere (esz-byte elements, row-major m x n with leading
// dimension ld), then the stored entries of A over it.
__global__ void fill_bytes_k(int64_t m, int64_t n, int64_t ld, int esz, const unsigned char* __restrict__ fillv,
                             unsigned char* __restrict__ out) {
  unsigned char f[8];
  for (int b = 0; b < esz; ++b) f[b] = fillv[b];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m * n; e += (int64_t)gridDim.x * blockDim.x) {
    unsigned char* dst = out + ((e / n) * ld + e % n) * esz;
    for (int b = 0; b < esz; ++b) dst[b] = f[b];
  }
}

template <class PtrT>
__global__ void scatter_dense_k(int64_t nf, const PtrT* __restrict__ ptr, const int* __restrict__ idx, int base,
                                const unsigned char* __restrict__ val, int esz, int csc, int64_t ld,
                                unsigned char* __restrict__ out) {
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    for (int64_t p = ld_ptr(ptr, f) - base; p < ld_ptr(ptr, f + 1) - base; ++p) {
      const int64_t c = (int64_t)idx[p] - base;
      const int64_t i = csc ? c : f, j = csc ? f : c;
      unsigned char* dst = out + (i * ld + j) * esz;
      if (val)
        for (int b = 0; b < esz; ++b) dst[b] = val[p * esz + b];
      else
        dst[0] = 1;  // a Pattern entry is true
    }
  }
}

}  // namespace fgb

extern "C" int fgb_sparse_to_dense(fgb_ctx* ctx, const fgb_sparse* A, const void* fill, void* out, int64_t ld,
                                   void* stream) {
  using namespace fgb;
  FGB_REQUIRE(ctx && A && fill, "fgb_sparse_to_dense: null argument");
  int rc = check_sparse(A, "fgb_sparse_to_dense: A", true);
  if (rc) return rc;
  FGB_REQUIRE(ld >= A->ncols, "fgb_sparse_to_dense: leading dimension below the column count");
  if (A->nrows == 0 || A->ncols == 0) return FGB_OK;
  FGB_REQUIRE(out, "fgb_sparse_to_dense: null output");
  const int esz = A->val_t == FGB_NONE ? 1 : dtype_size(A->val_t);
  cudaStream_t s = pick_stream(ctx, stream);
  unsigned char* fdev = nullptr;
  FGB_CUDA_TRY(cudaMallocAsync((void**)&fdev, 8, s));
  cudaError_t e = cudaMemcpyAsync(fdev, fill, esz, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    fill_bytes_k<<<grid_for(A->nrows * A->ncols, 256, ctx->num_sms), 256, 0, s>>>(A->nrows, A->ncols, ld, esz, fdev,
                                                                                  (unsigned char*)out);
    const int64_t nf = A->orient == FGB_CSC ? A->ncols : A->nrows;
    const int grid = grid_for(nf, 256, ctx->num_sms);
    if (A->ptr_t == FGB_I32)
      scatter_dense_k<int32_t><<<grid, 256, 0, s>>>(nf, (const int32_t*)A->ptr, (const int*)A->idx, A->index_base,
                                                    (const unsigned char*)A->val, esz, A->orient == FGB_CSC, ld,
                                                    (unsigned char*)out);
    else
      scatter_dense_k<int64_t><<<grid, 256, 0, s>>>(nf, (const int64_t*)A->ptr, (const int*)A->idx, A->index_base,
                                                    (const unsigned char*)A->val, esz, A->orient == FGB_CSC, ld,
                                                    (unsigned char*)out);
    e = cudaGetLastError();
  }
  cudaFreeAsync(fdev, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the fill value's host memory may go after return
  if (e != cudaSuccess) return set_error(FGB_ECUDA, "fgb_sparse_to_dense: %s", cudaGetErrorString(e));
  return FGB_OK;
}
