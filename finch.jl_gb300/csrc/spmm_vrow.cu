// Column-slab SpMM over length-sorted virtual rows (FP32, CSR).
//
// For a B much larger than L2 whose rows are gathered at random (columns of
// A spread over all of B), walking C's full width per stored entry re-reads
// most B rows from HBM once per entry.  This schedule cuts C's columns into
// slabs of SW = 16 or 32 and runs one launch per slab: while a launch runs,
// only B's slab (ncols * SW * 4 bytes) is gathered, and it stays in L2;
// A is re-read once per slab instead (its index and value streams are small
// next to the B rows).
//
// Inside a launch, rows are cut into virtual rows of at most T stored
// entries and handed to sub-groups of L = SW/4 lanes (each lane owns 4
// columns), 32/L virtual rows per warp at once.  A sub-group sums its
// virtual row's entries in storage order with up to BATCH gathers of B in
// flight per lane, with no cross-lane reduction.  Virtual rows are sorted by
// length class (longest first), so the sub-groups of a warp run similar trip
// counts.  The first virtual row of each row writes C; the others of a long
// row write partial sums that a fix-up kernel adds to C in order.  Results
// are deterministic.
//
// The schedule (virtual rows and their order) depends only on the matrix:
// plans build it once.
#include <cub/cub.cuh>

#include "spmm_common.cuh"

namespace fgb {

constexpr int VR_BATCH = 8;
constexpr int VR_THREADS = 256;

template <class PtrT>
__global__ void vrow_count_k(int64_t nrows, const PtrT* __restrict__ ptr, int T,
                             int64_t* __restrict__ nv, int64_t* __restrict__ nl) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t len = ld_ptr(ptr, r + 1) - ld_ptr(ptr, r);
    const int64_t nch = len <= T ? 1 : (len + T - 1) / T;
    nv[r] = nch;
    nl[r] = nch - 1;
  }
}

__device__ __forceinline__ uint8_t vrow_class(int64_t len) {
  // longest first: class 0 holds the longest lengths
  const int b = len <= 0 ? 0 : 64 - __clzll((unsigned long long)len);  // 1 + floor(log2 len)
  return (uint8_t)(15 - b);
}

template <class PtrT>
__global__ void vrow_fill_k(int64_t nrows, const PtrT* __restrict__ ptr, int T,
                            const int64_t* __restrict__ voff, const int64_t* __restrict__ loff,
                            uint8_t* __restrict__ key, int32_t* __restrict__ ord,
                            int32_t* __restrict__ u_row, int32_t* __restrict__ u_off,
                            int32_t* __restrict__ u_slot, int64_t* __restrict__ part_row) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t len = ld_ptr(ptr, r + 1) - ld_ptr(ptr, r);
    const int64_t v0 = voff[r], l0 = loff[r];
    const int64_t nch = voff[r + 1] - v0;
    for (int64_t c = 0; c < nch; ++c) {
      const int64_t v = v0 + c;
      const int64_t clen = len - c * T < T ? len - c * T : T;
      key[v] = vrow_class(clen);
      ord[v] = (int32_t)v;
      u_row[v] = (int32_t)r;
      u_off[v] = (int32_t)(c * T);
      u_slot[v] = c == 0 ? -1 : (int32_t)(l0 + c - 1);
      if (c > 0) part_row[l0 + c - 1] = r;
    }
  }
}

__global__ void vrow_gather_k(int64_t nv, const int32_t* __restrict__ ord,
                              const int32_t* __restrict__ u_row, const int32_t* __restrict__ u_off,
                              const int32_t* __restrict__ u_slot, int32_t* __restrict__ row,
                              int32_t* __restrict__ off, int32_t* __restrict__ slot) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = ord[i];
    row[i] = u_row[v];
    off[i] = u_off[v];
    slot[i] = u_slot[v];
  }
}

// One launch: C[:, c0 : c0 + 4L] (or the partial sums) for every virtual row.
template <class PtrT, int L>
__global__ void __launch_bounds__(VR_THREADS, 4) spmm_vrow_k(
    int64_t nv, const int32_t* __restrict__ vr_row, const int32_t* __restrict__ vr_off,
    const int32_t* __restrict__ vr_slot, const PtrT* __restrict__ ptr, const int* __restrict__ idx,
    const float* __restrict__ val, const float* __restrict__ B, int64_t ldb, float* __restrict__ C,
    int64_t ldc, int64_t c0, int64_t nk, int base, int accumulate, int T, float* __restrict__ partial) {
  constexpr int PER = VR_BATCH / L > 0 ? VR_BATCH / L : 1;  // entries each lane loads per batch
  constexpr int NB = PER * L;                                // entries per batch
  const int lane = threadIdx.x & 31, sl = lane % L;
  const unsigned gmask = group_mask<L>();
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / L;
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / L;
  const int64_t col = c0 + (int64_t)sl * 4;
  const bool active = col < nk;
  const float* Bc = B + col;
  const uint64_t pol_stream = policy_evict_first();
  const uint64_t pol_keep = policy_evict_last();
  for (int64_t v = gid; v < nv; v += ngroups) {
    const int64_t r = __ldg(vr_row + v);
    const int64_t rs = ld_ptr(ptr, r) - base + __ldg(vr_off + v);
    const int64_t rend = ld_ptr(ptr, r + 1) - base;
    const int len = (int)(rend - rs < (int64_t)T ? rend - rs : (int64_t)T);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int t = 0; t < len; t += NB) {
      int j[PER];
      float a[PER];
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int p = t + sl + L * q;
        j[q] = 0;
        a[q] = 0.f;
        if (p < len) {
          j[q] = ld_stream_i32(idx + rs + p, pol_stream) - base;
          a[q] = ld_stream_f32(val + rs + p, pol_stream);
        }
      }
      float4 b[NB];
#pragma unroll
      for (int u = 0; u < NB; ++u) {
        const int jj = __shfl_sync(gmask, j[u / L], u % L, L);
        b[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (t + u < len && active) b[u] = ld_gather_f32x4(Bc + (int64_t)jj * ldb, pol_keep);
      }
#pragma unroll
      for (int u = 0; u < NB; ++u) {
        const float aa = __shfl_sync(gmask, a[u / L], u % L, L);
        if (t + u < len) {
          acc.x = __fmaf_rn(aa, b[u].x, acc.x);
          acc.y = __fmaf_rn(aa, b[u].y, acc.y);
          acc.z = __fmaf_rn(aa, b[u].z, acc.z);
          acc.w = __fmaf_rn(aa, b[u].w, acc.w);
        }
      }
    }
    if (!active) continue;
    const int32_t slot = __ldg(vr_slot + v);
    if (slot < 0) {
      float* dst = C + r * ldc + col;
      if (accumulate) {
        const float4 o = *reinterpret_cast<const float4*>(dst);
        acc.x += o.x;
        acc.y += o.y;
        acc.z += o.z;
        acc.w += o.w;
      }
      st_stream_f32x4(dst, acc, pol_stream);
    } else {
      *reinterpret_cast<float4*>(partial + (int64_t)slot * nk + col) = acc;
    }
  }
}

// Adds each row's partial sums (slots in chunk order) to that row of C.
__global__ void vrow_fixup_k(int64_t nl, int64_t nk, const int64_t* __restrict__ part_row,
                             const float* __restrict__ partial, float* __restrict__ C, int64_t ldc) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nl * nk;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w = t / nk, c = t - w * nk;
    const int64_t r = part_row[w];
    if (w > 0 && part_row[w - 1] == r) continue;
    float sum = partial[w * nk + c];
    for (int64_t w2 = w + 1; w2 < nl && part_row[w2] == r; ++w2) sum += partial[w2 * nk + c];
    C[r * ldc + c] += sum;
  }
}

static inline size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

template <class PtrT>
static int vrow_build_t(fgb_ctx* ctx, const fgb_sparse* A, int T, VrowSchedule* out, cudaStream_t s) {
  const int64_t nrows = A->nrows;
  const PtrT* ptr = (const PtrT*)A->ptr;
  const int grid = grid_for(nrows, 256, ctx->num_sms);
  int64_t *cnt_v = nullptr, *cnt_l = nullptr, *voff = nullptr, *loff = nullptr;
  void* cub_tmp = nullptr;
  size_t cub_bytes = 0, b2 = 0;
  cudaError_t e = cudaSuccess;
  auto fail = [&](const char* what) {
    cudaFree(cnt_v);
    cudaFree(cnt_l);
    cudaFree(voff);
    cudaFree(loff);
    cudaFree(cub_tmp);
    return set_error(e == cudaErrorMemoryAllocation ? FGB_ENOMEM : FGB_ECUDA, "vrow schedule: %s: %s",
                     what, cudaGetErrorString(e));
  };
  if ((e = cudaMalloc(&cnt_v, sizeof(int64_t) * (nrows + 1))) != cudaSuccess) return fail("alloc");
  if ((e = cudaMalloc(&cnt_l, sizeof(int64_t) * (nrows + 1))) != cudaSuccess) return fail("alloc");
  if ((e = cudaMalloc(&voff, sizeof(int64_t) * (nrows + 1))) != cudaSuccess) return fail("alloc");
  if ((e = cudaMalloc(&loff, sizeof(int64_t) * (nrows + 1))) != cudaSuccess) return fail("alloc");
  cudaMemsetAsync(cnt_v + nrows, 0, sizeof(int64_t), s);
  cudaMemsetAsync(cnt_l + nrows, 0, sizeof(int64_t), s);
  vrow_count_k<PtrT><<<grid, 256, 0, s>>>(nrows, ptr, T, cnt_v, cnt_l);
  cub::DeviceScan::ExclusiveSum(nullptr, cub_bytes, cnt_v, voff, nrows + 1, s);
  if ((e = cudaMalloc(&cub_tmp, cub_bytes)) != cudaSuccess) return fail("alloc");
  if ((e = cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, cnt_v, voff, nrows + 1, s)) != cudaSuccess)
    return fail("scan");
  if ((e = cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, cnt_l, loff, nrows + 1, s)) != cudaSuccess)
    return fail("scan");
  int64_t tot[2] = {0, 0};
  cudaMemcpyAsync(&tot[0], voff + nrows, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(&tot[1], loff + nrows, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail("count");
  const int64_t nv = tot[0], nl = tot[1];
  if (nv > INT32_MAX || nl > INT32_MAX) {
    e = cudaSuccess;
    cudaFree(cnt_v);
    cudaFree(cnt_l);
    cudaFree(voff);
    cudaFree(loff);
    cudaFree(cub_tmp);
    return set_error(FGB_EUNSUPPORTED, "vrow schedule: too many virtual rows");
  }
  // persistent: row, off, slot (sorted), part_row; temporary: keys, order, unsorted copies
  const size_t keep = a256(4 * nv) * 3 + a256(8 * (nl > 0 ? nl : 1));
  char* mem = nullptr;
  if ((e = cudaMalloc(&mem, keep)) != cudaSuccess) return fail("alloc");
  out->row = (int32_t*)mem;
  out->off = (int32_t*)(mem + a256(4 * nv));
  out->slot = (int32_t*)(mem + 2 * a256(4 * nv));
  out->part_row = (int64_t*)(mem + 3 * a256(4 * nv));
  out->mem = mem;
  out->nv = nv;
  out->nl = nl;
  out->T = T;
  char* tmp = nullptr;
  const size_t tmp_bytes = a256(nv) * 2 + a256(4 * nv) * 5;
  if ((e = cudaMalloc(&tmp, tmp_bytes)) != cudaSuccess) {
    cudaFree(mem);
    out->mem = nullptr;
    return fail("alloc");
  }
  uint8_t* key = (uint8_t*)tmp;
  uint8_t* key2 = (uint8_t*)(tmp + a256(nv));
  int32_t* ord = (int32_t*)(tmp + 2 * a256(nv));
  int32_t* ord2 = ord + a256(4 * nv) / 4;
  int32_t* u_row = ord2 + a256(4 * nv) / 4;
  int32_t* u_off = u_row + a256(4 * nv) / 4;
  int32_t* u_slot = u_off + a256(4 * nv) / 4;
  vrow_fill_k<PtrT><<<grid, 256, 0, s>>>(nrows, ptr, T, voff, loff, key, ord, u_row, u_off, u_slot,
                                         out->part_row);
  b2 = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, b2, key, key2, ord, ord2, (int)nv, 0, 4, s);
  if (b2 > cub_bytes) {
    cudaFree(cub_tmp);
    cub_tmp = nullptr;
    if ((e = cudaMalloc(&cub_tmp, b2)) != cudaSuccess) {
      cudaFree(tmp);
      cudaFree(mem);
      out->mem = nullptr;
      return fail("alloc");
    }
    cub_bytes = b2;
  }
  e = cub::DeviceRadixSort::SortPairs(cub_tmp, cub_bytes, key, key2, ord, ord2, (int)nv, 0, 4, s);
  if (e == cudaSuccess) {
    vrow_gather_k<<<grid_for(nv, 256, ctx->num_sms), 256, 0, s>>>(nv, ord2, u_row, u_off, u_slot,
                                                                  out->row, out->off, out->slot);
    e = cudaStreamSynchronize(s);
  }
  cudaFree(tmp);
  if (e != cudaSuccess) {
    cudaFree(mem);
    out->mem = nullptr;
    return fail("sort");
  }
  cudaFree(cnt_v);
  cudaFree(cnt_l);
  cudaFree(voff);
  cudaFree(loff);
  cudaFree(cub_tmp);
  return FGB_OK;
}

int vrow_build(fgb_ctx* ctx, const fgb_sparse* A, int T, VrowSchedule* out, cudaStream_t s) {
  *out = VrowSchedule{};
  if (A->orient != FGB_CSR) return set_error(FGB_EUNSUPPORTED, "vrow schedule: CSR only");
  if (T < 8 || T > 4096) return set_error(FGB_EINVAL, "vrow schedule: chunk %d outside [8, 4096]", T);
  if (A->nrows > INT32_MAX) return set_error(FGB_EUNSUPPORTED, "vrow schedule: too many rows");
  return A->ptr_t == FGB_I32 ? vrow_build_t<int32_t>(ctx, A, T, out, s)
                             : vrow_build_t<int64_t>(ctx, A, T, out, s);
}

void vrow_free(VrowSchedule* v) {
  if (v && v->mem) cudaFree(v->mem);
  if (v) *v = VrowSchedule{};
}

template <class PtrT, int L>
static int launch_vrow(fgb_ctx* ctx, const VrowSchedule& v, const fgb_sparse* A, const float* B,
                       int64_t ldb, int64_t nk, float* C, int64_t ldc, int accumulate, float* partial,
                       cudaStream_t s) {
  static int occ = -1;  // per process: one device model
  if (occ < 0) {
    int o = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, spmm_vrow_k<PtrT, L>, VR_THREADS, 0);
    occ = o > 0 ? o : 1;
  }
  const int64_t need = (v.nv * L + VR_THREADS - 1) / VR_THREADS;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)occ * ctx->num_sms));
  for (int64_t c0 = 0; c0 < nk; c0 += 4 * L) {
    spmm_vrow_k<PtrT, L><<<grid, VR_THREADS, 0, s>>>(
        v.nv, v.row, v.off, v.slot, (const PtrT*)A->ptr, (const int*)A->idx, (const float*)A->val, B,
        ldb, C, ldc, c0, nk, A->index_base, accumulate, v.T, partial);
  }
  if (v.nl > 0)
    vrow_fixup_k<<<grid_for(v.nl * nk, 256, ctx->num_sms), 256, 0, s>>>(v.nl, nk, v.part_row, partial,
                                                                        C, ldc);
  FGB_CUDA_TRY(cudaGetLastError());
  return FGB_OK;
}

size_t spmm_vrow_scratch_bytes(const VrowSchedule& v, int64_t nk) {
  return sizeof(float) * (size_t)(v.nl > 0 ? v.nl : 0) * (size_t)nk;
}

int spmm_vrow(fgb_ctx* ctx, const VrowSchedule& v, const fgb_sparse* A, const void* B, int64_t ldb,
              int64_t nk, void* C, int64_t ldc, int accumulate, int slab, void* partial,
              cudaStream_t s) {
  if (A->val_t != FGB_F32 || A->idx_t != FGB_I32)
    return set_error(FGB_EUNSUPPORTED, "spmm vrow: F32 values and int32 indices only");
  if (nk % 4 || ldb % 4 || ldc % 4 || (uintptr_t)B % 16 || (uintptr_t)C % 16)
    return set_error(FGB_EUNSUPPORTED, "spmm vrow: needs 16-byte aligned rows of B and C");
  if (v.nl > 0 && !partial) return set_error(FGB_EINVAL, "spmm vrow: no partial-sum scratch");
  const bool p32 = A->ptr_t == FGB_I32;
  const float* b = (const float*)B;
  float* c = (float*)C;
  float* part = (float*)partial;
  if (slab == 16)
    return p32 ? launch_vrow<int32_t, 4>(ctx, v, A, b, ldb, nk, c, ldc, accumulate, part, s)
               : launch_vrow<int64_t, 4>(ctx, v, A, b, ldb, nk, c, ldc, accumulate, part, s);
  if (slab == 32)
    return p32 ? launch_vrow<int32_t, 8>(ctx, v, A, b, ldb, nk, c, ldc, accumulate, part, s)
               : launch_vrow<int64_t, 8>(ctx, v, A, b, ldb, nk, c, ldc, accumulate, part, s);
  return set_error(FGB_EINVAL, "spmm vrow: slab %d not in {16, 32}", slab);
}

}  // namespace fgb
