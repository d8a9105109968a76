// SDDMM over the virtual-row schedule of the slab SpMM (FP32, CSR, k <= 128,
// k a multiple of 4).
//
// out[e] = A.val[e] * <X[i,:], Y[j,:]>.  A sub-group of L lanes (4 columns
// of k per lane) takes one virtual row -- at most T stored entries of one
// row -- so the row's slice of X is loaded once into registers and every
// entry only gathers its row of Y.  NB entries are in flight per sub-group;
// each dot product is reduced over the L lanes with xor-shuffles (a fixed
// tree: deterministic).  Virtual rows are sorted by length class, so the
// sub-groups of a warp run similar trip counts.  Optionally k is cut into
// column slabs of one 128-byte line of Y, one launch each (fewer L2 lines per
// launch); the dot then accumulates in `out` across launches and the last
// launch multiplies by A's value.  A schedule with column bands runs each
// band's virtual rows in launches of their own, so a launch gathers from
// 1/nbands of Y; entries do not combine, so bands change no result.
#include "spmm_common.cuh"

namespace fgb {

constexpr int SV_THREADS = 256;

template <int L, int NB>
__global__ void __launch_bounds__(SV_THREADS, 4) sddmm_vrow_k(
    int64_t nv, const int4* __restrict__ vr, const int* __restrict__ idx, const float* __restrict__ val,
    const float* __restrict__ X, int64_t ldx, const float* __restrict__ Y, int64_t ldy, int64_t k,
    float* __restrict__ out, int base, int mode) {
  const int lane = threadIdx.x & 31, sl = lane % L;
  const unsigned gmask = group_mask<L>();
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / L;
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / L;
  const int64_t col = (int64_t)sl * 4;
  const bool active = col < k;
  const uint64_t pol_stream = policy_evict_first();
  const uint64_t pol_keep = policy_evict_last();
  for (int64_t v = gid; v < nv; v += ngroups) {
    const int4 rec = __ldg(vr + v);  // row, first entry, length, (slot: unused here)
    float4 xr = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) xr = __ldg(reinterpret_cast<const float4*>(X + (int64_t)rec.x * ldx + col));
    for (int t = 0; t < rec.z; t += NB) {
      float d[NB];
#pragma unroll
      for (int u = 0; u < NB; ++u) {
        d[u] = 0.f;
        if (t + u < rec.z && active) {
          const int j = __ldg(idx + rec.y + t + u) - base;
          const float4 y = ld_gather_f32x4(Y + (int64_t)j * ldy + col, pol_keep);
          d[u] = __fmaf_rn(xr.x, y.x, __fmaf_rn(xr.y, y.y, __fmaf_rn(xr.z, y.z, xr.w * y.w)));
        }
      }
#pragma unroll
      for (int m = L / 2; m >= 1; m >>= 1)
#pragma unroll
        for (int u = 0; u < NB; ++u) d[u] += __shfl_xor_sync(gmask, d[u], m, L);
      if (sl < NB && t + sl < rec.z) {  // lane u of the sub-group stores entry t + u
        float mine = d[0];
#pragma unroll
        for (int u = 1; u < NB; ++u)
          if (sl == u) mine = d[u];
        const int64_t e = (int64_t)rec.y + t + sl;
        // mode 0: all of k; 1: first slab; 2: middle slab; 3: last slab
        const float dsum = mode >= 2 ? out[e] + mine : mine;
        out[e] = (mode == 0 || mode == 3) ? __fmul_rn(ld_stream_f32(val + e, pol_stream), dsum) : dsum;
      }
    }
  }
}

// The same launch with each lane's NB gathers of Y staged in its own
// shared-memory slots by cp.async (NB <= L: lane u of the sub-group stores
// entry t + u).  No registers wait on memory, so more warps fit per SM and
// twice the gathers are in flight per lane; the dot products and their
// reduction are the register kernel's, so results are identical.
__device__ __forceinline__ void sv_cp_async16(void* smem, const void* gmem, uint64_t pol) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(sa), "l"(gmem), "l"(pol)
               : "memory");
}

// ALL: every lane's 4 columns lie inside k, so no lane is masked; a full
// batch (NB entries left) then issues and reduces without per-entry predicates.
template <int L, int NB, int MINB, bool ALL>
__global__ void __launch_bounds__(SV_THREADS, MINB) sddmm_vrow_async_k(
    int64_t nv, const int4* __restrict__ vr, const int* __restrict__ idx, const float* __restrict__ val,
    const float* __restrict__ X, int64_t ldx, const float* __restrict__ Y, int ldy, int64_t k,
    float* __restrict__ out, int base, int mode) {
  static_assert(NB <= L, "lane u of the sub-group stores entry u of a batch");
  extern __shared__ float4 sv_stage[];  // [NB][SV_THREADS]
  const int lane = threadIdx.x & 31, sl = lane % L;
  const unsigned gmask = group_mask<L>();
  const int gid = (int)((blockIdx.x * blockDim.x + threadIdx.x) / L);  // nv < 2^31 (vrow_build)
  const int ngroups = (int)((gridDim.x * blockDim.x) / L);
  const int64_t col = (int64_t)sl * 4;
  const bool active = ALL || col < k;
  const float* Yc = Y + col;
  float4* slot = sv_stage + threadIdx.x;
  const uint64_t pol_stream = policy_evict_first();
  const uint64_t pol_keep = policy_evict_last();
  for (int v = gid; v < nv; v += ngroups) {
    const int4 rec = __ldg(vr + v);  // row, first entry, length, (slot: unused here)
    float4 xr = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) xr = __ldg(reinterpret_cast<const float4*>(X + (int64_t)rec.x * ldx + col));
    for (int t = 0; t < rec.z; t += NB) {
      // lane u of the sub-group loads entry t + u's column; the sub-group shares it
      int jm = 0;
      if (sl < NB && t + sl < rec.z) jm = __ldg(idx + rec.y + t + sl) - base;
      float d[NB];
      if (ALL && t + NB <= rec.z) {  // full batch, no masked lane
#pragma unroll
        for (int u = 0; u < NB; ++u)
          sv_cp_async16(slot + u * SV_THREADS, Yc + (int64_t)__shfl_sync(gmask, jm, u, L) * ldy, pol_keep);
        asm volatile("cp.async.wait_all;" ::: "memory");
#pragma unroll
        for (int u = 0; u < NB; ++u) {
          const float4 y = slot[u * SV_THREADS];
          d[u] = __fmaf_rn(xr.x, y.x, __fmaf_rn(xr.y, y.y, __fmaf_rn(xr.z, y.z, xr.w * y.w)));
        }
      } else {
#pragma unroll
        for (int u = 0; u < NB; ++u) {
          const int j = __shfl_sync(gmask, jm, u, L);
          if (t + u < rec.z && active) sv_cp_async16(slot + u * SV_THREADS, Yc + (int64_t)j * ldy, pol_keep);
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
#pragma unroll
        for (int u = 0; u < NB; ++u) {
          d[u] = 0.f;
          if (t + u < rec.z && active) {
            const float4 y = slot[u * SV_THREADS];
            d[u] = __fmaf_rn(xr.x, y.x, __fmaf_rn(xr.y, y.y, __fmaf_rn(xr.z, y.z, xr.w * y.w)));
          }
        }
      }
#pragma unroll
      for (int m = L / 2; m >= 1; m >>= 1)
#pragma unroll
        for (int u = 0; u < NB; ++u) d[u] += __shfl_xor_sync(gmask, d[u], m, L);
      if (sl < NB && t + sl < rec.z) {
        float mine = d[0];
#pragma unroll
        for (int u = 1; u < NB; ++u)
          if (sl == u) mine = d[u];
        const int64_t e = (int64_t)rec.y + t + sl;
        const float dsum = mode >= 2 ? out[e] + mine : mine;
        out[e] = (mode == 0 || mode == 3) ? __fmul_rn(ld_stream_f32(val + e, pol_stream), dsum) : dsum;
      }
    }
  }
}

template <int L, bool ALL>
static int launch_sddmm_vrow_async_t(fgb_ctx* ctx, const VrowSchedule& v, const fgb_sparse* A, const float* X,
                                     int64_t ldx, const float* Y, int64_t ldy, int64_t k, float* out,
                                     int mode, cudaStream_t s) {
  constexpr int NB = L >= 8 ? 8 : L;
  constexpr size_t smem = sizeof(float4) * NB * SV_THREADS;
  static const int occ = [] {  // once per process (one device model); thread-safe
    cudaFuncSetAttribute(sddmm_vrow_async_k<L, NB, 6, ALL>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    int o = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, sddmm_vrow_async_k<L, NB, 6, ALL>, SV_THREADS, smem);
    return o > 0 ? o : 1;
  }();
  for (int b = 0; b < v.nbands; ++b) {  // column bands: one launch each (1/nbands of Y per launch)
    const int64_t nvb = v.nbands > 1 ? v.band_off[b + 1] - v.band_off[b] : v.nv;
    if (nvb == 0) continue;
    const int64_t need = (nvb * L + SV_THREADS - 1) / SV_THREADS;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)occ * ctx->num_sms));
    sddmm_vrow_async_k<L, NB, 6, ALL><<<grid, SV_THREADS, smem, s>>>(
        nvb, v.vr + (v.nbands > 1 ? v.band_off[b] : 0), (const int*)A->idx, (const float*)A->val, X, ldx, Y,
        (int)ldy, k, out, A->index_base, mode);
  }
  FGB_CUDA_TRY(cudaGetLastError());
  return FGB_OK;
}

// The unmasked build when the launch's k fills every lane (k == 4L).
template <int L>
static int launch_sddmm_vrow_async(fgb_ctx* ctx, const VrowSchedule& v, const fgb_sparse* A, const float* X,
                                   int64_t ldx, const float* Y, int64_t ldy, int64_t k, float* out,
                                   int mode, cudaStream_t s) {
  if (k == 4 * L) return launch_sddmm_vrow_async_t<L, true>(ctx, v, A, X, ldx, Y, ldy, k, out, mode, s);
  return launch_sddmm_vrow_async_t<L, false>(ctx, v, A, X, ldx, Y, ldy, k, out, mode, s);
}

template <int L>
static int launch_sddmm_vrow(fgb_ctx* ctx, const VrowSchedule& v, const fgb_sparse* A, const float* X,
                             int64_t ldx, const float* Y, int64_t ldy, int64_t k, float* out,
                             int mode, cudaStream_t s) {
  constexpr int NB = L >= 4 ? 4 : L;
  static const int occ = [] {  // once per process (one device model); thread-safe
    int o = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, sddmm_vrow_k<L, NB>, SV_THREADS, 0);
    return o > 0 ? o : 1;
  }();
  for (int b = 0; b < v.nbands; ++b) {
    const int64_t nvb = v.nbands > 1 ? v.band_off[b + 1] - v.band_off[b] : v.nv;
    if (nvb == 0) continue;
    const int64_t need = (nvb * L + SV_THREADS - 1) / SV_THREADS;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)occ * ctx->num_sms));
    sddmm_vrow_k<L, NB><<<grid, SV_THREADS, 0, s>>>(nvb, v.vr + (v.nbands > 1 ? v.band_off[b] : 0),
                                                    (const int*)A->idx, (const float*)A->val, X, ldx, Y, ldy,
                                                    k, out, A->index_base, mode);
  }
  FGB_CUDA_TRY(cudaGetLastError());
  return FGB_OK;
}

int sddmm_vrow(fgb_ctx* ctx, const VrowSchedule& v, const fgb_sparse* A, const void* X, int64_t ldx,
               const void* Y, int64_t ldy, int64_t k, void* out, cudaStream_t s, int64_t slab,
               bool async_gather) {
  if (A->orient != FGB_CSR || A->val_t != FGB_F32 || A->idx_t != FGB_I32)
    return set_error(FGB_EUNSUPPORTED, "sddmm vrow: CSR with F32 values and int32 indices only");
  if (k <= 0 || k > 128 || k % 4 || ldx % 4 || ldy % 4 || (uintptr_t)X % 16 || (uintptr_t)Y % 16)
    return set_error(FGB_EUNSUPPORTED, "sddmm vrow: needs k in (0, 128], a multiple of 4, and 16-byte rows");
  const float* x = (const float*)X;
  const float* y = (const float*)Y;
  float* o = (float*)out;
  if (slab <= 0 || slab >= k || slab % 4) slab = k;
  for (int64_t c0 = 0; c0 < k; c0 += slab) {
    const int64_t kw = k - c0 < slab ? k - c0 : slab;
    const int mode = slab >= k ? 0 : c0 == 0 ? 1 : c0 + slab >= k ? 3 : 2;
    const int64_t need = (slab + 3) / 4;
    int rc;
    if (async_gather) {
      if (ldy > INT32_MAX)
        return set_error(FGB_EUNSUPPORTED, "sddmm vrow: cp.async gathers need a leading dimension below 2^31");
      if (need <= 4) rc = launch_sddmm_vrow_async<4>(ctx, v, A, x + c0, ldx, y + c0, ldy, kw, o, mode, s);
      else if (need <= 8) rc = launch_sddmm_vrow_async<8>(ctx, v, A, x + c0, ldx, y + c0, ldy, kw, o, mode, s);
      else if (need <= 16) rc = launch_sddmm_vrow_async<16>(ctx, v, A, x + c0, ldx, y + c0, ldy, kw, o, mode, s);
      else rc = launch_sddmm_vrow_async<32>(ctx, v, A, x + c0, ldx, y + c0, ldy, kw, o, mode, s);
      if (rc) return rc;
      continue;
    }
    if (need <= 4) rc = launch_sddmm_vrow<4>(ctx, v, A, x + c0, ldx, y + c0, ldy, kw, o, mode, s);
    else if (need <= 8) rc = launch_sddmm_vrow<8>(ctx, v, A, x + c0, ldx, y + c0, ldy, kw, o, mode, s);
    else if (need <= 16) rc = launch_sddmm_vrow<16>(ctx, v, A, x + c0, ldx, y + c0, ldy, kw, o, mode, s);
    else rc = launch_sddmm_vrow<32>(ctx, v, A, x + c0, ldx, y + c0, ldy, kw, o, mode, s);
    if (rc) return rc;
  }
  return FGB_OK;
}

}  // namespace fgb
