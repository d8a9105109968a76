// Merge-path SpMM with the B-row gathers staged through shared memory by TMA.
//
// The register-gather kernel (spmm_merge.cu) can keep only a few 16-byte
// gathers per lane in flight, so on a 1M x 1M power-law matrix it waits on
// memory most of the time.  Here every warp owns a ring of S stages in
// shared memory; a stage holds R rows of a W-column slab of B.  The warp's
// lane 0 fills a stage with `cp.async.bulk.tensor.2d ... tile::gather4` --
// one instruction fetches four B rows named by four column indices of A --
// and the stage's mbarrier counts the bytes in.  While up to S*R rows are in
// flight the warp consumes the oldest stage: each lane reads its four
// columns of a row with one 16-byte shared load and accumulates.  Items,
// rows, carries and the fix-up are those of the merge-path schedule, so the
// result is the same up to float summation order and deterministic.
//
// Every wait on an mbarrier is bounded; a wait that runs out sets an error
// flag, drains the warp's outstanding copies (again bounded) and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "spmm_common.cuh"

namespace fgb {

constexpr int TMA_WARPS = 8;
constexpr int TMA_THREADS = 32 * TMA_WARPS;
constexpr uint32_t TMA_WAIT_LIMIT = 1u << 26;  // polls before a wait gives up

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void tma_gather4(uint32_t dst, const CUtensorMap* map, int x, int r0,
                                            int r1, int r2, int r3, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cta.global.tile::gather4.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
      "l"(map), "r"(x), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(bar)
      : "memory");
}

// Bounded wait on one stage; false if it ran out.
__device__ __forceinline__ bool wait_stage(uint32_t bar, uint32_t parity) {
  for (uint32_t i = 0; i < TMA_WAIT_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

template <class VT, class PtrT, int W, int R, int S>
__global__ void __launch_bounds__(TMA_THREADS, 1) spmm_tma_k(
    const __grid_constant__ CUtensorMap bmap, int64_t nrows, const PtrT* __restrict__ ptr,
    const int* __restrict__ idx, const VT* __restrict__ val, float* __restrict__ C, int64_t ldc,
    int c0, int64_t nk, int base, int accumulate, int64_t n_items,
    const int64_t* __restrict__ plan_row, const int64_t* __restrict__ plan_k,
    int64_t* __restrict__ carry_row, float* __restrict__ carry, const int32_t* __restrict__ row_map,
    int* __restrict__ err) {
  static_assert(R % 4 == 0 && R <= 32, "R rows per stage, multiple of 4, at most 32");
  static_assert(W % 4 == 0 && W <= 128, "W columns, at most 128 (one float4 per lane)");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float* ring = reinterpret_cast<float*>(smem_raw) + (size_t)wib * S * R * W;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + (size_t)TMA_WARPS * S * R * W * sizeof(float)) + wib * S;
  if (lane == 0) {
    for (int s = 0; s < S; ++s) mbar_init(smem_addr(bars + s), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t col = (int64_t)c0 + (int64_t)lane * 4;
  const bool active = lane * 4 < W && col < nk;
  const uint64_t pol_stream = policy_evict_first();
  uint64_t issued = 0, consumed = 0;  // stages, monotonic over the warp's items
  bool failed = false;

  for (int64_t w = warp; w < n_items && !failed; w += nwarps) {
    int64_t r = plan_row[w];
    const int64_t k0 = plan_k[w];
    const int64_t r1 = plan_row[w + 1], k1 = plan_k[w + 1];
    const int64_t nst = (k1 - k0 + R - 1) / R;  // stages of this item
    int64_t next_fetch = 0;                    // next stage of this item to issue

    auto issue = [&](int64_t st) {
      const int64_t e0 = k0 + st * R;
      const int cnt = (k1 - e0) < (int64_t)R ? (int)(k1 - e0) : R;
      int j = 0;
      if (lane < cnt) j = ld_stream_i32(idx + e0 + lane, pol_stream) - base;
      const int jlast = __shfl_sync(0xffffffffu, j, cnt - 1);
      if (lane >= cnt) j = jlast;  // pad the last gather4 with a repeated row
      const uint32_t slot = (uint32_t)(issued % S);
      const uint32_t bar = smem_addr(bars + slot);
      const int ngather = (cnt + 3) / 4;
      if (lane == 0) mbar_expect_tx(bar, (uint32_t)(ngather * 4 * W * sizeof(float)));
#pragma unroll
      for (int g = 0; g < R / 4; ++g) {
        const int q0 = __shfl_sync(0xffffffffu, j, 4 * g), q1 = __shfl_sync(0xffffffffu, j, 4 * g + 1);
        const int q2 = __shfl_sync(0xffffffffu, j, 4 * g + 2), q3 = __shfl_sync(0xffffffffu, j, 4 * g + 3);
        if (lane == 0 && g < ngather)
          tma_gather4(smem_addr(ring + ((size_t)slot * R + 4 * g) * W), &bmap, c0, q0, q1, q2, q3, bar);
      }
      ++issued;
    };

    for (; next_fetch < nst && next_fetch < S; ++next_fetch) issue(next_fetch);

    // row-end window: lane l holds the end of row rw + l
    int64_t rw = r;
    int64_t re = rw + lane < nrows ? ld_ptr(ptr, rw + 1 + lane) - base : INT64_MAX;
    auto row_end = [&](int64_t row) -> int64_t {
      if (row >= r1) return k1;
      if (row - rw >= 32) {
        rw = row;
        re = rw + lane < nrows ? ld_ptr(ptr, rw + 1 + lane) - base : INT64_MAX;
      }
      return __shfl_sync(0xffffffffu, re, (int)(row - rw));
    };
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    auto store_row = [&](int64_t row) {
      if (active) {
        float* dst = C + (row_map ? (int64_t)__ldg(row_map + row) : row) * ldc + col;
        if (accumulate) {
          const float4 old = *reinterpret_cast<const float4*>(dst);
          acc.x += old.x, acc.y += old.y, acc.z += old.z, acc.w += old.w;
        }
        st_stream_f32x4(dst, acc, pol_stream);
      }
      acc = make_float4(0.f, 0.f, 0.f, 0.f);
    };
    int64_t e_end = row_end(r);

    for (int64_t st = 0; st < nst; ++st) {
      const int64_t e0 = k0 + st * R;
      const int cnt = (k1 - e0) < (int64_t)R ? (int)(k1 - e0) : R;
      const uint32_t slot = (uint32_t)(consumed % S);
      const uint32_t parity = (uint32_t)((consumed / S) & 1);
      float a_l = 0.f;
      if (lane < cnt) a_l = load_val<float, VT>(val, e0 + lane, pol_stream);
      if (!__all_sync(0xffffffffu, wait_stage(smem_addr(bars + slot), parity))) {
        failed = true;
        break;
      }
      ++consumed;
      const float* rows = ring + (size_t)slot * R * W;
      for (int t = 0; t < cnt; ++t) {
        const int64_t e = e0 + t;
        while (e >= e_end) {  // rows that end before entry e (empty ones included)
          store_row(r);
          ++r;
          e_end = row_end(r);
        }
        const float a = __shfl_sync(0xffffffffu, a_l, t);
        if (active) {
          const float4 b = *reinterpret_cast<const float4*>(rows + (size_t)t * W + lane * 4);
          acc.x = __fmaf_rn(a, b.x, acc.x);
          acc.y = __fmaf_rn(a, b.y, acc.y);
          acc.z = __fmaf_rn(a, b.z, acc.z);
          acc.w = __fmaf_rn(a, b.w, acc.w);
        }
      }
      __syncwarp();
      if (next_fetch < nst) {
        if (lane == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        issue(next_fetch);
        ++next_fetch;
      }
    }
    if (failed) break;
    while (r < r1) {  // rows that end at the item's last entry, or are empty
      store_row(r);
      ++r;
    }
    // the row left open at the item's end carries its partial sum
    if (lane == 0 && c0 == 0)
      carry_row[w] = r1 < nrows ? (row_map ? (int64_t)__ldg(row_map + r1) : r1) : -1;
    if (active) *reinterpret_cast<float4*>(carry + w * nk + col) = acc;
  }
  if (failed) {
    if (lane == 0) atomicExch(err, 1);
    // drain the copies still in flight into this warp's ring (bounded)
    while (consumed < issued) {
      const uint32_t slot = (uint32_t)(consumed % S);
      if (!__all_sync(0xffffffffu, wait_stage(smem_addr(bars + slot), (uint32_t)((consumed / S) & 1))))
        break;
      ++consumed;
    }
  }
}

// ---------------------------------------------------------------- host side

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {  // looked up once; thread-safe
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000)p;
    return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
  }();
  return fn;
}

constexpr int TMA_R = 8, TMA_S = 4;

template <int W>
static size_t tma_smem_bytes() {
  return (size_t)TMA_WARPS * TMA_S * TMA_R * W * sizeof(float) + (size_t)TMA_WARPS * TMA_S * 8;
}

template <class VT, class PtrT, int W>
static int launch_tma_w(fgb_ctx* ctx, const fgb_sparse* A, const float* B, int64_t ldb, int64_t nk,
                        float* C, int64_t ldc, int accumulate, int64_t n_items,
                        const int64_t* plan_row, const int64_t* plan_k, int64_t* carry_row,
                        float* carry, const int32_t* row_map, int* err, cudaStream_t s) {
  auto fn = encode_fn();
  if (!fn) return set_error(FGB_EUNSUPPORTED, "spmm: cuTensorMapEncodeTiled unavailable");
  CUtensorMap map;
  const cuuint64_t dims[2] = {(cuuint64_t)nk, (cuuint64_t)A->ncols};
  const cuuint64_t strides[1] = {(cuuint64_t)ldb * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)W, 1};
  const cuuint32_t estr[2] = {1, 1};
  CUresult cr = fn(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)B, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return set_error(FGB_EINVAL, "spmm: tensor map of B rejected (%d)", (int)cr);
  auto kern = spmm_tma_k<VT, PtrT, W, TMA_R, TMA_S>;
  const size_t smem = tma_smem_bytes<W>();
  static thread_local int configured[2][2][4] = {};
  int& cfg = configured[sizeof(VT) == 2][sizeof(PtrT) == 8][W == 32 ? 0 : W == 64 ? 1 : W == 128 ? 2 : 3];
  if (!cfg) {
    FGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    cfg = 1;
  }
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, TMA_THREADS, smem);
  if (occ < 1) occ = 1;
  int64_t grid = (int64_t)ctx->num_sms * occ;
  const int64_t need = (n_items * 32 + TMA_THREADS - 1) / TMA_THREADS;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  for (int64_t c0 = 0; c0 < nk; c0 += W) {
    kern<<<(int)grid, TMA_THREADS, smem, s>>>(map, A->nrows, (const PtrT*)A->ptr, (const int*)A->idx,
                                              (const VT*)A->val, C, ldc, (int)c0, nk, A->index_base,
                                              accumulate, n_items, plan_row, plan_k, carry_row,
                                              carry, row_map, err);
    int rc = check_launch("spmm_tma_k");
    if (rc) return rc;
  }
  return FGB_OK;
}

// Stage-ring SpMM over merge-path items already planned in plan_row/plan_k.
// fp32 only; nk a multiple of 4; B 16-byte aligned with ldb*4 a multiple of
// 16 (the TMA rules).
int spmm_tma_items(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk,
                   void* C, int64_t ldc, int accumulate, int64_t n_items, const int64_t* plan_row,
                   const int64_t* plan_k, int64_t* carry_row, void* carry, const int32_t* row_map,
                   int* err, cudaStream_t s) {
  const bool bf = A->val_t == FGB_BF16;
  const bool p64 = A->ptr_t == FGB_I64;
#define FGB_TMA(VT, PT, WW)                                                                       \
  return launch_tma_w<VT, PT, WW>(ctx, A, (const float*)B, ldb, nk, (float*)C, ldc, accumulate,   \
                                  n_items, plan_row, plan_k, carry_row, (float*)carry, row_map,   \
                                  err, s)
  if (nk <= 32) {
    if (bf) { if (p64) FGB_TMA(__nv_bfloat16, int64_t, 32); FGB_TMA(__nv_bfloat16, int32_t, 32); }
    if (p64) FGB_TMA(float, int64_t, 32);
    FGB_TMA(float, int32_t, 32);
  }
  if (nk <= 64) {
    if (bf) { if (p64) FGB_TMA(__nv_bfloat16, int64_t, 64); FGB_TMA(__nv_bfloat16, int32_t, 64); }
    if (p64) FGB_TMA(float, int64_t, 64);
    FGB_TMA(float, int32_t, 64);
  }
  if (bf) { if (p64) FGB_TMA(__nv_bfloat16, int64_t, 128); FGB_TMA(__nv_bfloat16, int32_t, 128); }
  if (p64) FGB_TMA(float, int64_t, 128);
  FGB_TMA(float, int32_t, 128);
#undef FGB_TMA
}

}  // namespace fgb
