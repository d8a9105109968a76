// SDDMM: out[e] = A.val[e] * sum_k X[i,k] * Y[j,k] for every stored entry
// e = (i, j) of a CSR matrix A (for CSC the roles of X and Y swap: the
// compressed coordinate indexes X).
//
// Work is split by stored entries, not by rows, so the power-law row
// lengths of real graphs do not unbalance the grid: warp w owns entries
// [w*CH, (w+1)*CH), finds its first row by a binary search of ptr and walks
// rows forward from there.  Inside the warp, groups of L lanes each own one
// entry at a time; a lane holds V consecutive k of X[i,:] and Y[j,:] (one
// 16-byte load each for fp32), the group reduces the L partial dot products
// with xor-shuffles, and one lane writes out[e].  Y rows are gathered with
// an evict-last L2 hint; A's idx/val and the output stream with evict-first.
//
// Column slabs: when Y is far larger than L2, k is cut into slabs of one
// 128-byte line per row of Y, one launch per slab, so that a launch gathers
// from ncols lines instead of ncols * k * esz / 128.  The first slab writes
// the partial dot into out, middle slabs add to it, and the last one adds
// its part and multiplies by A.val[e].
//
// FGB_FINCH_ORDER selects one thread per entry and a sequential dot over k
// ascending, then the product with A.val[e].
#include "fgb_internal.cuh"
#include "semiring.cuh"
#include "spmm_common.cuh"

namespace fgb {

template <class PtrT>
__device__ __forceinline__ int64_t row_of(const PtrT* ptr, int64_t nrows, int64_t e, int base) {
  // largest r with ptr[r] - base <= e  (ptr is non-decreasing)
  int64_t lo = 0, hi = nrows;  // answer in [lo, hi)
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (ld_ptr(ptr, mid) - base <= e) lo = mid; else hi = mid;
  }
  return lo;
}

template <class T, int V>
struct SVec {
  T v[V];
};

template <class T, int V>
__device__ __forceinline__ SVec<T, V> ldv(const T* p, uint64_t pol, bool use_pol) {
  SVec<T, V> r;
#pragma unroll
  for (int q = 0; q < V; ++q) r.v[q] = __ldg(p + q);
  return r;
}
template <>
__device__ __forceinline__ SVec<float, 4> ldv<float, 4>(const float* p, uint64_t pol, bool use_pol) {
  float4 f;
  if (use_pol)
    f = ld_gather_f32x4(p, pol);
  else
    f = __ldg(reinterpret_cast<const float4*>(p));
  return SVec<float, 4>{{f.x, f.y, f.z, f.w}};
}

template <class T, class PtrT, int L, int V, int U>
__global__ void __launch_bounds__(256) sddmm_csr(int64_t nrows, int64_t nnz,
                                                 const PtrT* __restrict__ ptr,
                                                 const int* __restrict__ idx,
                                                 const T* __restrict__ val,
                                                 const T* __restrict__ X, int64_t ldx,
                                                 const T* __restrict__ Y, int64_t ldy, int64_t k,
                                                 T* __restrict__ out, int base, int64_t chunk,
                                                 int mode) {
  constexpr int GPW = 32 / L;  // groups per warp
  const int lane = threadIdx.x & 31;
  const int gl = lane & (L - 1);  // lane inside group
  const int g = lane / L;         // group inside warp
  const unsigned gmask = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << (g * L));
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t pol_stream = policy_evict_first();
  const uint64_t pol_keep = policy_evict_last();
  for (int64_t c = warp * chunk; c < nnz; c += nwarps * chunk) {
    const int64_t cend = min(c + chunk, nnz);
    int64_t row = row_of(ptr, nrows, c, base);
    int64_t row_end = ld_ptr(ptr, row + 1) - base;
    for (int64_t e0 = c + g; e0 < cend; e0 += (int64_t)GPW * U) {
      int64_t e[U];
      int64_t r[U];
      bool ok[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        e[u] = e0 + (int64_t)u * GPW;
        ok[u] = e[u] < cend;
        if (ok[u]) {
          while (e[u] >= row_end) {
            ++row;
            row_end = ld_ptr(ptr, row + 1) - base;
          }
        }
        r[u] = row;
      }
      T dot[U];
#pragma unroll
      for (int u = 0; u < U; ++u) dot[u] = T(0);
      int jj[U];
#pragma unroll
      for (int u = 0; u < U; ++u) jj[u] = ok[u] ? ld_stream_i32(idx + e[u], pol_stream) - base : 0;
      for (int64_t k0 = (int64_t)gl * V; k0 < k; k0 += (int64_t)L * V) {
        SVec<T, V> xv[U], yv[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (ok[u]) {
            xv[u] = ldv<T, V>(X + r[u] * ldx + k0, pol_keep, false);
            yv[u] = ldv<T, V>(Y + (int64_t)jj[u] * ldy + k0, pol_keep, true);
          }
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (ok[u])
#pragma unroll
            for (int q = 0; q < V; ++q) dot[u] = fused(xv[u].v[q], yv[u].v[q], dot[u]);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
#pragma unroll
        for (int m = L / 2; m >= 1; m >>= 1) dot[u] += __shfl_xor_sync(gmask, dot[u], m, L);
        if (ok[u] && gl == 0) {
          // mode 0: the whole k; 1: first slab; 2: middle slab; 3: last slab
          const T d = mode >= 2 ? out[e[u]] + dot[u] : dot[u];
          out[e[u]] = (mode == 0 || mode == 3) ? wmul(__ldg(val + e[u]), d) : d;
        }
      }
    }
  }
}

// One thread per entry, sequential dot over k ascending.
template <class T, class PtrT>
__global__ void sddmm_csr_serial(int64_t nrows, int64_t nnz, const PtrT* __restrict__ ptr,
                                 const int* __restrict__ idx, const T* __restrict__ val,
                                 const T* __restrict__ X, int64_t ldx, const T* __restrict__ Y,
                                 int64_t ldy, int64_t k, T* __restrict__ out, int base, int fm) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = row_of(ptr, nrows, e, base);
    const int64_t j = __ldg(idx + e) - base;
    T acc = T(0);
    for (int64_t q = 0; q < k; ++q)
      acc = Semi<SR_PT, T>::step(acc, X[i * ldx + q], Y[j * ldy + q], fm);
    out[e] = wmul(val[e], acc);
  }
}

template <class T, class PtrT>
static int run(fgb_ctx* ctx, const fgb_sparse* A, const T* X, int64_t ldx, const T* Y,
               int64_t ldy, int64_t k, T* out, unsigned flags, int lanes, int64_t chunk,
               int64_t slab, cudaStream_t s) {
  const int64_t nf = n_fibers(A);
  const int64_t nnz = A->nnz;
  if (nnz == 0) return FGB_OK;
  const PtrT* ptr = (const PtrT*)A->ptr;
  const int* idx = (const int*)A->idx;
  const T* val = (const T*)A->val;
  const int base = A->index_base;
  const int threads = 256;
  if (flags & FGB_FINCH_ORDER) {
    const int fm = (flags & FGB_NO_FMA) ? FM_NOFMA : FM_FMA;
    sddmm_csr_serial<T, PtrT><<<grid_for(nnz, threads, ctx->num_sms, 8), threads, 0, s>>>(
        nf, nnz, ptr, idx, val, X, ldx, Y, ldy, k, out, base, fm);
    return check_launch("sddmm_csr_serial");
  }
  if (chunk <= 0) chunk = 128;
  const int64_t nchunks = (nnz + chunk - 1) / chunk;
  const int grid = grid_for(nchunks * 32, threads, ctx->num_sms, 8);
  constexpr int VN = sizeof(T) == 4 ? 4 : 1;
  const bool vec_ok = VN > 1 && k % VN == 0 && ldx % VN == 0 && ldy % VN == 0 &&
                      (uintptr_t)X % 16 == 0 && (uintptr_t)Y % 16 == 0;
  if (slab <= 0 || slab >= k || (vec_ok && slab % VN)) slab = k;  // one pass
  if (lanes <= 0) {  // at most 8 lanes per entry: more entries in flight per warp
    const int64_t need = vec_ok ? (slab + VN - 1) / VN : slab;
    lanes = need <= 4 ? 4 : 8;
  }
  for (int64_t c0 = 0; c0 < k; c0 += slab) {
    const int64_t kw = k - c0 < slab ? k - c0 : slab;
    const int mode = slab >= k ? 0 : c0 == 0 ? 1 : c0 + slab >= k ? 3 : 2;
    const T* Xs = X + c0;
    const T* Ys = Y + c0;
#define FGB_SDDMM(LL, VV, UU)                                                                   \
  sddmm_csr<T, PtrT, LL, VV, UU><<<grid, threads, 0, s>>>(nf, nnz, ptr, idx, val, Xs, ldx, Ys, \
                                                          ldy, kw, out, base, chunk, mode)
    if (vec_ok) {
      switch (lanes) {
        case 4: FGB_SDDMM(4, VN, 2); break;
        case 8: FGB_SDDMM(8, VN, 2); break;
        case 16: FGB_SDDMM(16, VN, 4); break;
        default: FGB_SDDMM(32, VN, 4); break;
      }
    } else {
      switch (lanes) {
        case 4: FGB_SDDMM(4, 1, 2); break;
        case 8: FGB_SDDMM(8, 1, 2); break;
        case 16: FGB_SDDMM(16, 1, 4); break;
        default: FGB_SDDMM(32, 1, 4); break;
      }
    }
#undef FGB_SDDMM
    const int rc = check_launch("sddmm_csr");
    if (rc) return rc;
  }
  return FGB_OK;
}

int sddmm_impl(fgb_ctx* ctx, const fgb_sparse* A, const void* X, int64_t ldx, const void* Y,
               int64_t ldy, int64_t k, void* out, int dtype, unsigned flags, int lanes,
               int64_t chunk, void* stream, int64_t slab) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_sddmm: null ctx");
  int rc = check_sparse(A, "fgb_sddmm: A", true);
  if (rc) return rc;
  if (k < 0 || ldx < k || ldy < k) return set_error(FGB_EINVAL, "fgb_sddmm: bad k/ldx/ldy");
  if (A->val_t != dtype)
    return set_error(FGB_EUNSUPPORTED, "fgb_sddmm: A values must have the output dtype");
  if (A->nnz > 0 && (!X || !Y || !out)) return set_error(FGB_EINVAL, "fgb_sddmm: null operand");
  // For CSC the compressed coordinate is j, so X and Y trade places.
  const void* Xc = A->orient == FGB_CSR ? X : Y;
  const void* Yc = A->orient == FGB_CSR ? Y : X;
  const int64_t ldxc = A->orient == FGB_CSR ? ldx : ldy;
  const int64_t ldyc = A->orient == FGB_CSR ? ldy : ldx;
  cudaStream_t s = pick_stream(ctx, stream);
  if (slab < 0) {  // default: slabs of one 128-byte line when Y is far larger than L2
    const int64_t esz = dtype == FGB_F64 ? 8 : 4;
    const int64_t ny = A->orient == FGB_CSR ? A->ncols : A->nrows;
    slab = ((double)ny * (double)k * (double)esz > 256.0 * 1024 * 1024) ? 128 / esz : 0;
  }
  if (dtype == FGB_F32) {
    if (A->ptr_t == FGB_I32)
      return run<float, int32_t>(ctx, A, (const float*)Xc, ldxc, (const float*)Yc, ldyc, k,
                                 (float*)out, flags, lanes, chunk, slab, s);
    return run<float, int64_t>(ctx, A, (const float*)Xc, ldxc, (const float*)Yc, ldyc, k,
                               (float*)out, flags, lanes, chunk, slab, s);
  }
  if (dtype == FGB_F64) {
    if (A->ptr_t == FGB_I32)
      return run<double, int32_t>(ctx, A, (const double*)Xc, ldxc, (const double*)Yc, ldyc, k,
                                  (double*)out, flags, lanes, chunk, slab, s);
    return run<double, int64_t>(ctx, A, (const double*)Xc, ldxc, (const double*)Yc, ldyc, k,
                                (double*)out, flags, lanes, chunk, slab, s);
  }
  return set_error(FGB_EUNSUPPORTED, "fgb_sddmm: dtype %d", dtype);
}

}  // namespace fgb

namespace fgb {
// No schedule given: a Y far larger than L2 with many stored entries takes the
// virtual rows with cp.async gathers in 32-column slabs, built for the call
// (the plan autotuner's choice for the 1M x 1M Zipf matrix with k = 64).
static bool sddmm_default_vrow(const fgb_sparse* A, const void* X, int64_t ldx, const void* Y, int64_t ldy,
                               int64_t k, int dtype, unsigned flags) {
  return A && A->orient == FGB_CSR && A->val_t == FGB_F32 && A->idx_t == FGB_I32 && dtype == FGB_F32 &&
         !(flags & FGB_FINCH_ORDER) && k > 0 && k <= 128 && k % 4 == 0 && ldx % 4 == 0 && ldy % 4 == 0 &&
         ldy <= INT32_MAX && (uintptr_t)X % 16 == 0 && (uintptr_t)Y % 16 == 0 && A->nrows <= INT32_MAX &&
         A->nnz >= (1 << 20) && A->nnz <= INT32_MAX && (double)A->ncols * (double)k * 4.0 > 64.0 * 1024 * 1024;
}
}  // namespace fgb

extern "C" int fgb_sddmm(fgb_ctx* ctx, const fgb_sparse* A, const void* X, int64_t ldx,
                         const void* Y, int64_t ldy, int64_t k, void* out_val, int dtype,
                         unsigned flags, void* stream) {
  if (fgb::sddmm_default_vrow(A, X, ldx, Y, ldy, k, dtype, flags) &&
      !fgb::stream_capturing(fgb::pick_stream(ctx, stream))) {
    const fgb_sddmm_tuning t{0, 2, 256, k > 32 ? 32 : 0};
    return fgb_sddmm_ex(ctx, A, X, ldx, Y, ldy, k, out_val, dtype, flags, &t, stream);
  }
  return fgb::sddmm_impl(ctx, A, X, ldx, Y, ldy, k, out_val, dtype, flags, 0, 0, stream, -1);
}

extern "C" int fgb_sddmm_ex(fgb_ctx* ctx, const fgb_sparse* A, const void* X, int64_t ldx,
                            const void* Y, int64_t ldy, int64_t k, void* out_val, int dtype,
                            unsigned flags, const fgb_sddmm_tuning* tune, void* stream) {
  if (!tune || (tune->lanes == 0 && tune->variant == 0 && tune->chunk == 0 && tune->slab == -1 &&
                tune->bands <= 1))
    return fgb_sddmm(ctx, A, X, ldx, Y, ldy, k, out_val, dtype, flags, stream);  // no schedule given
  const int lanes = tune->lanes;
  if (lanes != 0 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32)
    return fgb::set_error(FGB_EINVAL, "fgb_sddmm_ex: lanes must be 0, 4, 8, 16 or 32");
  if (tune && (tune->chunk < 0 || tune->slab < -1))
    return fgb::set_error(FGB_EINVAL, "fgb_sddmm_ex: negative chunk or slab");
  if (tune->bands < 0 || tune->bands > 8) return fgb::set_error(FGB_EINVAL, "fgb_sddmm_ex: bands must be in [0, 8]");
  if (tune->bands > 1 && tune->variant != 1 && tune->variant != 2)
    return fgb::set_error(FGB_EINVAL, "fgb_sddmm_ex: column bands need variant 1 or 2");
  if (tune && (tune->variant == 1 || tune->variant == 2)) {  // virtual rows: schedule built for this call
    if (!ctx) return fgb::set_error(FGB_EINVAL, "fgb_sddmm_ex: null ctx");
    int rc = fgb::check_sparse(A, "fgb_sddmm_ex: A", true);
    if (rc) return rc;
    if (dtype != FGB_F32 || A->val_t != FGB_F32 || (flags & FGB_FINCH_ORDER))
      return fgb::set_error(FGB_EUNSUPPORTED, "fgb_sddmm_ex: variants 1 and 2 need F32 and no FGB_FINCH_ORDER");
    if (A->nnz == 0) return FGB_OK;
    cudaStream_t s = fgb::pick_stream(ctx, stream);
    fgb::VrowSchedule v;
    rc = fgb::vrow_build(ctx, A, tune->chunk > 0 ? (int)std::min<int64_t>(tune->chunk, 4096) : 128, &v, s,
                         true, tune->bands > 1 ? tune->bands : 1);
    if (rc) return rc;
    rc = fgb::sddmm_vrow(ctx, v, A, X, ldx, Y, ldy, k, out_val, s, tune->slab > 0 ? tune->slab : 0,
                         tune->variant == 2);
    fgb::vrow_free(&v, s);  // stream-ordered, behind the launches
    return rc;
  }
  if (tune && tune->variant != 0) return fgb::set_error(FGB_EINVAL, "fgb_sddmm_ex: variant must be 0, 1 or 2");
  return fgb::sddmm_impl(ctx, A, X, ldx, Y, ldy, k, out_val, dtype, flags, lanes,
                         tune ? tune->chunk : 0, stream, tune ? tune->slab : -1);
}
