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
