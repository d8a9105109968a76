// Column-panel layout of a CSR matrix for SpMM with an L2-resident dense
// operand.
//
// In C = A B every stored entry A[i,j] gathers row j of B.  When B is larger
// than L2 those gathers mostly miss.  Splitting A's columns into P panels of
// consecutive columns makes each panel touch only rows [p*w, (p+1)*w) of B --
// a slice P times smaller that stays in L2 while the panel runs.  The price
// is that C rows with entries in several panels are read and written once per
// panel: panel 0 is a full CSR over all rows and writes every row of C
// (zeros included); panels 1.. list only their non-empty rows (a row map:
// Finch's SparseList over rows, i.e. DCSR) and accumulate into C.
//
// The layout is built on the device once: a stable radix sort of the entries
// by panel keeps row-major order inside every panel; row ends and row maps
// come from scans.  Each panel runs through the merge-path SpMM, so long
// rows stay balanced and results are deterministic.
#include <cub/cub.cuh>

#include <vector>

#include "spmm_common.cuh"

namespace fgb {
int dtype_size(int t);

template <class PtrT>
__global__ void rows_of_entries_k(int64_t m, const PtrT* __restrict__ ptr, int base,
                                  int32_t* __restrict__ row_of) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
       r += (int64_t)gridDim.x * blockDim.x)
    for (int64_t q = ld_ptr(ptr, r) - base; q < ld_ptr(ptr, r + 1) - base; ++q) row_of[q] = (int32_t)r;
}

__global__ void panel_keys_k(int64_t nnz, const int* __restrict__ idx, int base, int64_t width,
                             uint32_t* __restrict__ key, int32_t* __restrict__ pos) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz;
       q += (int64_t)gridDim.x * blockDim.x) {
    key[q] = (uint32_t)((__ldg(idx + q) - base) / width);
    pos[q] = (int32_t)q;
  }
}

__global__ void panel_gather_k(int64_t nnz, const int32_t* __restrict__ perm, const int* __restrict__ idx,
                               int base, const char* __restrict__ val, int esz,
                               const int32_t* __restrict__ row_of, int32_t* __restrict__ out_idx,
                               char* __restrict__ out_val, int32_t* __restrict__ out_row) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = perm[q];
    out_idx[q] = __ldg(idx + e) - base;
    out_row[q] = row_of[e];
    switch (esz) {
      case 8: ((int64_t*)out_val)[q] = ((const int64_t*)val)[e]; break;
      case 4: ((int32_t*)out_val)[q] = ((const int32_t*)val)[e]; break;
      default: ((int16_t*)out_val)[q] = ((const int16_t*)val)[e]; break;
    }
  }
}

// Panel 0: ptr over all m rows; its entries are rows-sorted, so
// ptr[r] = first position with row >= r.
__global__ void panel0_ptr_k(int64_t m, int64_t e1, const int32_t* __restrict__ row_s,
                             int32_t* __restrict__ ptr0) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r <= m;
       r += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = e1;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (row_s[mid] < r) lo = mid + 1; else hi = mid;
    }
    ptr0[r] = (int32_t)lo;
  }
}

// Row starts of panels 1..: flag[q] = 1 where (panel, row) changes.
__global__ void panel_flags_k(int64_t lo, int64_t nnz, const uint32_t* __restrict__ key,
                              const int32_t* __restrict__ row_s, int32_t* __restrict__ flag) {
  for (int64_t q = lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz;
       q += (int64_t)gridDim.x * blockDim.x)
    flag[q - lo] = (q == lo || key[q] != key[q - 1] || row_s[q] != row_s[q - 1]) ? 1 : 0;
}

__global__ void panel_rows_k(int64_t lo, int64_t nnz, const uint32_t* __restrict__ key,
                             const int32_t* __restrict__ row_s, const int32_t* __restrict__ flag,
                             const int32_t* __restrict__ cpos, const int64_t* __restrict__ e0,
                             const int64_t* __restrict__ c0, const int64_t* __restrict__ ptr_off,
                             int32_t* __restrict__ ptr_all, int32_t* __restrict__ rows_all) {
  for (int64_t q = lo + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz;
       q += (int64_t)gridDim.x * blockDim.x) {
    if (!flag[q - lo]) continue;
    const uint32_t p = key[q];
    const int64_t local = cpos[q - lo] - c0[p];
    ptr_all[ptr_off[p] + local] = (int32_t)(q - e0[p]);
    rows_all[c0[p] + local] = row_s[q];
  }
}

}  // namespace fgb

using namespace fgb;

struct fgb_panels {
  fgb_ctx* ctx = nullptr;
  int64_t m = 0, n = 0, nnz = 0, width = 0;
  int npanels = 0;
  int val_t = FGB_F32;
  int32_t* idx = nullptr;
  void* val = nullptr;
  int32_t* ptr_all = nullptr;
  int32_t* rows_all = nullptr;
  std::vector<int64_t> e0, rows, ptr_off, rows_off;  // per panel
  std::vector<fgb_sparse> desc;
  // merge-path scratch per panel, kept so item boundaries are computed once
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  std::vector<size_t> scratch_off;
  int64_t scratch_nk = -1, scratch_path = -1;
};

extern "C" {

int fgb_panels_create(fgb_ctx* ctx, const fgb_sparse* A, int32_t npanels, fgb_panels** out) {
  if (!ctx || !out) return set_error(FGB_EINVAL, "fgb_panels_create: null argument");
  *out = nullptr;
  int rc = check_sparse(A, "fgb_panels_create: A", true);
  if (rc) return rc;
  if (A->orient != FGB_CSR) return set_error(FGB_EUNSUPPORTED, "fgb_panels_create: needs CSR");
  if (A->val_t != FGB_F32 && A->val_t != FGB_F64 && A->val_t != FGB_BF16)
    return set_error(FGB_EUNSUPPORTED, "fgb_panels_create: values must be F32, F64 or BF16");
  if (npanels < 1 || npanels > 1024) return set_error(FGB_EINVAL, "fgb_panels_create: 1..1024 panels");
  if (A->nnz >= INT32_MAX || A->nrows >= INT32_MAX)
    return set_error(FGB_EUNSUPPORTED, "fgb_panels_create: int32 positions");
  cudaStream_t s = ctx->stream;
  const int64_t m = A->nrows, n = A->ncols, nnz = A->nnz;
  const int P = npanels;
  const int64_t width = n > 0 ? (n + P - 1) / P : 1;
  const int esz = dtype_size(A->val_t);
  fgb_panels* pn = new fgb_panels();
  pn->ctx = ctx;
  pn->m = m, pn->n = n, pn->nnz = nnz, pn->width = width, pn->npanels = P, pn->val_t = A->val_t;
  // temporaries
  int32_t *row_of = nullptr, *pos_in = nullptr, *pos_out = nullptr, *row_s = nullptr, *flag = nullptr,
          *cpos = nullptr;
  uint32_t *key_in = nullptr, *key_out = nullptr;
  int64_t *d_e0 = nullptr, *d_c0 = nullptr, *d_ptr_off = nullptr;
  void* tmp = nullptr;
  auto cleanup = [&]() {
    for (void* p : {(void*)row_of, (void*)pos_in, (void*)pos_out, (void*)row_s, (void*)flag,
                    (void*)cpos, (void*)key_in, (void*)key_out, (void*)d_e0, (void*)d_c0,
                    (void*)d_ptr_off, tmp})
      if (p) cudaFree(p);
  };
  auto fail = [&](int code, const char* what, cudaError_t e) {
    cleanup();
    fgb_panels_destroy(pn);
    return set_error(code, "fgb_panels_create: %s: %s", what, cudaGetErrorString(e));
  };
  const size_t nz = (size_t)(nnz > 0 ? nnz : 1);
  cudaError_t e = cudaSuccess;
  for (auto pr : {std::make_pair((void**)&row_of, nz * 4), std::make_pair((void**)&pos_in, nz * 4),
                  std::make_pair((void**)&pos_out, nz * 4), std::make_pair((void**)&row_s, nz * 4),
                  std::make_pair((void**)&flag, nz * 4), std::make_pair((void**)&cpos, nz * 4),
                  std::make_pair((void**)&key_in, nz * 4), std::make_pair((void**)&key_out, nz * 4),
                  std::make_pair((void**)&pn->idx, nz * 4), std::make_pair((void**)&pn->val, nz * esz)})
    if (e == cudaSuccess) e = cudaMalloc(pr.first, pr.second);
  if (e != cudaSuccess) return fail(FGB_ENOMEM, "allocation", e);
  const int grid = grid_for(nnz > m ? nnz : m, 256, ctx->num_sms, 8);
  if (A->ptr_t == FGB_I32)
    rows_of_entries_k<int32_t><<<grid_for(m, 256, ctx->num_sms, 8), 256, 0, s>>>(m, (const int32_t*)A->ptr, A->index_base, row_of);
  else
    rows_of_entries_k<int64_t><<<grid_for(m, 256, ctx->num_sms, 8), 256, 0, s>>>(m, (const int64_t*)A->ptr, A->index_base, row_of);
  panel_keys_k<<<grid, 256, 0, s>>>(nnz, (const int*)A->idx, A->index_base, width, key_in, pos_in);
  int end_bit = 1;
  while ((1 << end_bit) < P) ++end_bit;
  size_t tmp_sort = 0, tmp_scan = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_sort, key_in, key_out, pos_in, pos_out, nnz, 0, end_bit, s);
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_scan, flag, cpos, nnz, s);
  if ((e = cudaMalloc(&tmp, std::max(tmp_sort, tmp_scan) + 16)) != cudaSuccess) return fail(FGB_ENOMEM, "scratch", e);
  cub::DeviceRadixSort::SortPairs(tmp, tmp_sort, key_in, key_out, pos_in, pos_out, nnz, 0, end_bit, s);
  panel_gather_k<<<grid, 256, 0, s>>>(nnz, pos_out, (const int*)A->idx, A->index_base, (const char*)A->val,
                                     esz, row_of, pn->idx, (char*)pn->val, row_s);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(FGB_ECUDA, "sort", e);
  // panel boundaries e0[p] (host): lower bound of each panel key in the sorted keys
  std::vector<uint32_t> keys_h(nnz);
  if (nnz && (e = cudaMemcpyAsync(keys_h.data(), key_out, nnz * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return fail(FGB_ECUDA, "keys", e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(FGB_ECUDA, "sync", e);
  pn->e0.assign(P + 1, nnz);
  {
    int64_t q = 0;
    for (int p = 0; p <= P; ++p) {
      while (q < nnz && (int64_t)keys_h[q] < p) ++q;
      pn->e0[p] = q;
    }
    pn->e0[P] = nnz;
  }
  // panel 0: full CSR over all rows; panels 1..: compact rows
  const int64_t lo = pn->e0[1];
  const int64_t rest = nnz - lo;
  pn->rows.assign(P, 0);
  pn->rows[0] = m;
  std::vector<int64_t> c0(P + 1, 0);
  int64_t total_rows = 0;
  if (rest > 0) {
    panel_flags_k<<<grid_for(rest, 256, ctx->num_sms, 8), 256, 0, s>>>(lo, nnz, key_out, row_s, flag);
    cub::DeviceScan::ExclusiveSum(tmp, tmp_scan, flag, cpos, rest, s);
    std::vector<int32_t> fl(rest), cp(rest);
    if ((e = cudaMemcpyAsync(cp.data(), cpos, rest * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(fl.data(), flag, rest * 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
      return fail(FGB_ECUDA, "row starts", e);
    total_rows = cp[rest - 1] + fl[rest - 1];
    for (int p = 1; p <= P; ++p) c0[p] = pn->e0[p] < nnz ? cp[pn->e0[p] - lo] : total_rows;
    c0[1] = 0;
    for (int p = 1; p < P; ++p) pn->rows[p] = c0[p + 1] - c0[p];
  }
  // ptr arrays: panel 0 has m+1 entries at offset 0; panel p>=1 has rows+1
  pn->ptr_off.assign(P, 0);
  pn->rows_off.assign(P, 0);
  int64_t ptr_total = m + 1;
  for (int p = 1; p < P; ++p) {
    pn->ptr_off[p] = ptr_total;
    ptr_total += pn->rows[p] + 1;
    pn->rows_off[p] = c0[p];
  }
  if ((e = cudaMalloc((void**)&pn->ptr_all, sizeof(int32_t) * ptr_total)) != cudaSuccess ||
      (e = cudaMalloc((void**)&pn->rows_all, sizeof(int32_t) * (total_rows > 0 ? total_rows : 1))) != cudaSuccess)
    return fail(FGB_ENOMEM, "panel ptr", e);
  panel0_ptr_k<<<grid_for(m + 1, 256, ctx->num_sms, 8), 256, 0, s>>>(m, pn->e0[1], row_s, pn->ptr_all);
  if (rest > 0) {
    std::vector<int64_t> ptr_off_h(P), e0_h(P), c0_h(P);
    for (int p = 0; p < P; ++p) ptr_off_h[p] = pn->ptr_off[p], e0_h[p] = pn->e0[p], c0_h[p] = c0[p];
    if ((e = cudaMalloc((void**)&d_e0, 8 * P)) != cudaSuccess || (e = cudaMalloc((void**)&d_c0, 8 * P)) != cudaSuccess ||
        (e = cudaMalloc((void**)&d_ptr_off, 8 * P)) != cudaSuccess)
      return fail(FGB_ENOMEM, "panel tables", e);
    cudaMemcpyAsync(d_e0, e0_h.data(), 8 * P, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_c0, c0_h.data(), 8 * P, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_ptr_off, ptr_off_h.data(), 8 * P, cudaMemcpyHostToDevice, s);
    panel_rows_k<<<grid_for(rest, 256, ctx->num_sms, 8), 256, 0, s>>>(lo, nnz, key_out, row_s, flag, cpos, d_e0,
                                                                     d_c0, d_ptr_off, pn->ptr_all, pn->rows_all);
    // the end of every compact panel's ptr
    for (int p = 1; p < P; ++p) {
      const int32_t end = (int32_t)(pn->e0[p + 1] - pn->e0[p]);
      cudaMemcpyAsync(pn->ptr_all + pn->ptr_off[p] + pn->rows[p], &end, 4, cudaMemcpyHostToDevice, s);
      if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(FGB_ECUDA, "panel ends", e);
    }
  }
  if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(FGB_ECUDA, "build", e);
  cleanup();
  pn->desc.resize(P);
  for (int p = 0; p < P; ++p) {
    fgb_sparse& d = pn->desc[p];
    d.nrows = pn->rows[p];
    d.ncols = n;
    d.nnz = pn->e0[p + 1] - pn->e0[p];
    d.orient = FGB_CSR;
    d.index_base = 0;
    d.ptr_t = FGB_I32;
    d.idx_t = FGB_I32;
    d.val_t = A->val_t;
    d.reserved = 0;
    d.ptr = pn->ptr_all + pn->ptr_off[p];
    d.idx = pn->idx + pn->e0[p];
    d.val = (const char*)pn->val + pn->e0[p] * esz;
  }
  *out = pn;
  return FGB_OK;
}

int fgb_panels_spmm(fgb_ctx* ctx, fgb_panels* pn, const void* B, int64_t ldb, int64_t nk, void* C,
                    int64_t ldc, int dtype, unsigned flags, const fgb_spmm_tuning* tune, void* stream) {
  if (!ctx || !pn) return set_error(FGB_EINVAL, "fgb_panels_spmm: null argument");
  if (nk < 0 || ldb < nk || ldc < nk || (pn->n > 0 && nk > 0 && !B) || (pn->m > 0 && nk > 0 && !C))
    return set_error(FGB_EINVAL, "fgb_panels_spmm: bad B/C");
  const bool ok_type = (dtype == FGB_F32 && (pn->val_t == FGB_F32 || pn->val_t == FGB_BF16)) ||
                       (dtype == FGB_F64 && pn->val_t == FGB_F64);
  if (!ok_type) return set_error(FGB_EUNSUPPORTED, "fgb_panels_spmm: dtype %d with values %d", dtype, pn->val_t);
  const size_t esz = dtype == FGB_F64 ? 8 : 4;
  const int vn = esz == 4 ? 4 : 2;
  if (nk % vn || ldb % vn || ldc % vn || (uintptr_t)B % (vn * esz) || (uintptr_t)C % (vn * esz))
    return set_error(FGB_EUNSUPPORTED, "fgb_panels_spmm: nk, ldb, ldc and pointers must be vector-aligned");
  if (pn->m == 0 || nk == 0) return FGB_OK;
  int lanes = tune && tune->lanes ? tune->lanes : 32;
  while (lanes > 4 && (int64_t)(lanes / 2) * vn >= nk) lanes /= 2;
  const int64_t path = tune && tune->path ? tune->path : 512;
  const int variant = tune ? tune->variant : 0;
  cudaStream_t s = pick_stream(ctx, stream);
  bool ready = pn->scratch && pn->scratch_nk == nk && pn->scratch_path == path;
  if (!ready) {
    if (pn->scratch) {
      cudaStreamSynchronize(s);
      cudaFree(pn->scratch);
      pn->scratch = nullptr;
    }
    pn->scratch_off.assign(pn->npanels, 0);
    size_t total = 0;
    for (int p = 0; p < pn->npanels; ++p) {
      pn->scratch_off[p] = total;
      total += (spmm_merge_scratch_bytes(pn->desc[p].nrows, pn->desc[p].nnz, nk, esz, path) + 255) & ~size_t(255);
    }
    FGB_CUDA_TRY(cudaMalloc(&pn->scratch, total));
    pn->scratch_bytes = total;
    pn->scratch_nk = nk;
    pn->scratch_path = path;
  }
  for (int p = 0; p < pn->npanels; ++p) {
    const fgb_sparse& d = pn->desc[p];
    if (p > 0 && d.nrows == 0) continue;
    const int accumulate = (p > 0 || (flags & FGB_ACCUMULATE)) ? 1 : 0;
    const size_t bytes = (p + 1 < pn->npanels ? pn->scratch_off[p + 1] : pn->scratch_bytes) - pn->scratch_off[p];
    const int rc = spmm_merge(ctx, &d, B, ldb, nk, C, ldc, dtype, accumulate, lanes, path,
                              (char*)pn->scratch + pn->scratch_off[p], bytes, s, ready,
                              p == 0 ? nullptr : pn->rows_all + pn->rows_off[p], variant);
    if (rc) return rc;
  }
  return FGB_OK;
}

int fgb_panels_destroy(fgb_panels* pn) {
  if (!pn) return FGB_OK;
  if (pn->ctx) cudaStreamSynchronize(pn->ctx->stream);
  for (void* p : {(void*)pn->idx, pn->val, (void*)pn->ptr_all, (void*)pn->rows_all, pn->scratch})
    if (p) cudaFree(p);
  delete pn;
  return FGB_OK;
}

}  // extern "C"
