/* libfinchgb measurement helpers.
 *
 * These entry points have no counterpart in Finch.jl: they measure the
 * device ceilings that bound the sparse kernels, so a kernel's throughput can
 * be read against the hardware limit that actually applies to it.  Every
 * sparse kernel that gathers rows of a dense operand (SpMM, SDDMM, the pull
 * SpMV) is bound by how fast random gathers of that width are served from a
 * working set of that size, not by streaming HBM bandwidth.
 */
#ifndef FINCHGB_CALIBRATE_H
#define FINCHGB_CALIBRATE_H

#include "finchgb.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Random-gather ceiling: times `gathers` loads of `gather_bytes` contiguous
 * bytes each (4, 8, 16, 32, 64, 128, 256 or 512; aligned to their size) at
 * uniformly random places of a device buffer of `working_set_bytes`, issued
 * the way the gather kernels issue them (16 bytes per lane, 8 loads in flight
 * per lane, L2 evict_last; 4- and 8-byte gathers one per lane, as the x
 * gathers of a pull SpMV).  `*gbs` receives gathered bytes / device time in
 * GB/s (CUDA events on `stream`, after warm-up).  Synchronous; allocates and
 * frees its buffer on `stream`.  EINVAL for a width outside the list, a
 * working set smaller than 64 gathers or `gathers` <= 0. */
FGB_API int fgb_gather_ceiling(fgb_ctx* ctx, int64_t working_set_bytes, int32_t gather_bytes,
                               int64_t gathers, double* gbs, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FINCHGB_CALIBRATE_H */
