// fgb_spmm_noalloc: the SpMM entry point for callers that cannot allocate
// device memory.
//
// fgb_spmm obtains the scratch of its load-balanced CSR schedule (merge-path
// item boundaries and the per-item carry rows) from cudaMallocAsync on every
// call.  Some hosts cannot allow that: a Julia process whose device memory
// is owned by CUDA.jl's pool, a serving loop whose latency budget forbids an
// allocator call (it can synchronise the device), or a plugin that runs while
// an allocation of its caller is in progress.  This variant takes its scratch
// from one file-scope device array of FGB_NOALLOC_SCRATCH_BYTES instead and
// calls no allocating routine at all; the caller still passes A, B and C.
//
// The array exists once per device that loads the library and lives until
// the process exits.  Its device address is looked up with
// cudaGetSymbolAddress the first time the entry point runs on a device (with
// that device current) and cached; that first call should therefore happen
// before any stream capture.  Every call reuses the same array, so two calls
// that overlap on the GPU (different streams, or different host threads)
// race on it: serialise them.  The kernels write every scratch word they
// later read, so nothing has to be cleared between calls.
#include <mutex>

#include "spmm_common.cuh"
#include "spmm_noalloc_plan.h"

namespace fgb {

static __device__ __align__(256) unsigned char g_spmm_noalloc_scratch[FGB_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device`, which is current (looked
// up once per device).
static int noalloc_scratch(int device, void** out) {
  if (device < 0 || device >= kMaxDevices)
    return set_error(FGB_EINVAL, "fgb_spmm_noalloc: device %d out of range", device);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_spmm_noalloc_scratch);
    if (e != cudaSuccess)
      return set_error(FGB_ECUDA, "fgb_spmm_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_noalloc_ptr[device] = p;
  }
  *out = g_noalloc_ptr[device];
  return FGB_OK;
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_spmm_noalloc(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb,
                                int64_t nk, void* C, int64_t ldc, int dtype, unsigned flags,
                                void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_spmm_noalloc: null ctx");
  int rc = check_sparse(A, "fgb_spmm_noalloc: A", true);
  if (rc) return rc;
  if (nk < 0 || ldb < nk || ldc < nk) return set_error(FGB_EINVAL, "fgb_spmm_noalloc: bad nk/ldb/ldc");
  if ((A->ncols > 0 && nk > 0 && !B) || (A->nrows > 0 && nk > 0 && !C))
    return set_error(FGB_EINVAL, "fgb_spmm_noalloc: null B or C");
  const size_t esz = dtype == FGB_F64 ? 8 : 4;
  const int vn = esz == 4 ? 4 : 2;
  const bool merge = A->orient == FGB_CSR && !(flags & FGB_FINCH_ORDER) && A->nrows > 0 && nk > 0 &&
                     nk % vn == 0 && ldb % vn == 0 && ldc % vn == 0 &&
                     (uintptr_t)B % (vn * esz) == 0 && (uintptr_t)C % (vn * esz) == 0 &&
                     ((dtype == FGB_F32 && (A->val_t == FGB_F32 || A->val_t == FGB_BF16)) ||
                      (dtype == FGB_F64 && A->val_t == FGB_F64));
  if (!merge)  // the schedules that use no scratch: per-row pull, CSC push
    return spmm_impl(ctx, A, B, ldb, nk, C, ldc, dtype, flags, 0, 0, stream);
  // The merge-path schedule: lengthen the items until the scratch fits.
  int64_t path = 256;
  size_t need = 0;
  if (!noalloc_pick_path(A->nrows, A->nnz, nk, esz, FGB_NOALLOC_SCRATCH_BYTES, &path, &need))
    return set_error(FGB_EINVAL,
                     "fgb_spmm_noalloc: %lld rows, %lld stored entries and %lld columns need %zu "
                     "bytes of scratch, above the fixed %zu",
                     (long long)A->nrows, (long long)A->nnz, (long long)nk, need,
                     (size_t)FGB_NOALLOC_SCRATCH_BYTES);
  // The kernels run on the current device, so the scratch address must be
  // that device's: the context's device must be current.
  int cur = -1;
  FGB_CUDA_TRY(cudaGetDevice(&cur));
  if (cur != ctx->device)
    return set_error(FGB_EINVAL, "fgb_spmm_noalloc: device %d is current, the context is on device %d", cur,
                     ctx->device);
  void* scratch = nullptr;
  rc = noalloc_scratch(ctx->device, &scratch);
  if (rc) return rc;
  int lanes = 4;
  while (lanes < 32 && (int64_t)lanes * vn < nk) lanes *= 2;
  return spmm_merge(ctx, A, B, ldb, nk, C, ldc, dtype, (flags & FGB_ACCUMULATE) ? 1 : 0, lanes,
                    path, scratch, FGB_NOALLOC_SCRATCH_BYTES, pick_stream(ctx, stream));
}
