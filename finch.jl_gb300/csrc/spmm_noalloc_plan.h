// Host-side sizing of the merge-path SpMM schedule's scratch, and the item
// length fgb_spmm_noalloc picks so that scratch fits its fixed array.
//
// Plain C++ (no CUDA), so the decision can be checked on a machine without a
// GPU: fgb_spmm_noalloc makes it before touching any device memory.
#pragma once

#include <cstddef>
#include <cstdint>

namespace fgb {

inline size_t plan_align256(size_t x) { return (x + 255) & ~size_t(255); }

// Scratch of the merge-path schedule for `path`-step items over nrows + nnz
// steps (spmm_merge.cu's layout): the item boundaries in rows and entries
// (n_items + 1 each), the carry row of every item and its carry values
// (n_items x nk of esz bytes).  Saturates at SIZE_MAX instead of wrapping.
inline size_t merge_scratch_bytes(int64_t nrows, int64_t nnz, int64_t nk, size_t esz, int64_t path) {
  if (nrows < 0 || nnz < 0 || nk < 0 || path <= 0) return SIZE_MAX;
  const double steps = (double)nrows + (double)nnz;
  const double items_d = (steps + (double)path - 1.0) / (double)path;
  const double approx = items_d * (24.0 + (double)esz * (double)nk) + 1024.0;
  if (approx > 9.0e18) return SIZE_MAX;  // far beyond any device: no exact figure needed
  const int64_t n_items = (nrows + nnz + path - 1) / path;
  return plan_align256(sizeof(int64_t) * (size_t)(n_items + 1)) * 2 + plan_align256(sizeof(int64_t) * (size_t)n_items) +
         plan_align256(esz * (size_t)n_items * (size_t)nk);
}

// The item length of fgb_spmm_noalloc: the shortest of 256, 512, ... 2^24
// steps whose scratch fits `limit` bytes.  Returns false (and the need at
// 2^24) when none fits.
inline bool noalloc_pick_path(int64_t nrows, int64_t nnz, int64_t nk, size_t esz, size_t limit, int64_t* path,
                              size_t* need) {
  int64_t p = 256;
  while (p < (int64_t(1) << 24) && merge_scratch_bytes(nrows, nnz, nk, esz, p) > limit) p *= 2;
  *path = p;
  *need = merge_scratch_bytes(nrows, nnz, nk, esz, p);
  return *need <= limit;
}

}  // namespace fgb
