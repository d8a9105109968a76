// Column-slab SpMM over length-sorted virtual rows (FP32, CSR).
//
// For a B much larger than L2 whose rows are gathered at random (columns of
// A spread over all of B), walking C's full width per stored entry re-reads
// most B rows from HBM once per entry.  This schedule cuts C's columns into
// slabs of SW = 8, 16 or 32 and runs one launch per slab: while a launch
// runs, only B's slab is gathered, so more of it stays in L2; A is re-read
// once per slab instead (its index and value streams are small next to the
// B rows).
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

constexpr int VR_THREADS = 256;
constexpr int VR_SEG = 16;  // partial-sum slots per fix-up segment

// Column bands.  With P > 1 bands the columns of A are cut into P ranges of
// W consecutive columns, and a row's entries in band b (a contiguous run of
// its ascending columns) are scheduled in band b's launches only: a launch
// then gathers from 1/P of B's slab, which stays in L2.  A light row (no
// band holds more than T of its entries) keeps one running sum in C: its
// first non-empty band writes C and each later band continues from it,
// launch after launch, so its sum runs over its entries in storage order and
// equals the unbanded schedule's bit for bit.  A heavy row is
// cut at band boundaries and every T entries; its first chunk writes C and
// the others write partial-sum slots that the fix-up adds in order.  P = 1 is
// the unbanded schedule.
constexpr int VR_MAX_BANDS = 8;

struct RowBands {
  int64_t pos[VR_MAX_BANDS + 1];  // storage offsets (from the row's first entry) of the band starts
};

// Band starts of one row: pos[b] = number of the row's entries with column
// < b * W (columns ascending; for unsorted columns the runs still cover the
// row exactly once, only the locality is lost).
__device__ __forceinline__ void row_bands(const int* __restrict__ idx, int64_t b0, int64_t len, int base,
                                          int P, int64_t W, RowBands& rb) {
  rb.pos[0] = 0;
  rb.pos[P] = len;
  for (int b = 1; b < P; ++b) {
    const int64_t c = (int64_t)b * W;  // first column of band b
    int64_t lo = rb.pos[b - 1], hi = len;
    while (lo < hi) {  // first entry with column >= c
      const int64_t mid = (lo + hi) >> 1;
      if ((int64_t)idx[b0 + mid] - base < c) lo = mid + 1;
      else hi = mid;
    }
    rb.pos[b] = lo;
  }
}

// Virtual rows of one row, in storage order: per band, ceil(len_b / T)
// chunks for a heavy row, one chunk per non-empty band for a light row (an
// empty row keeps one empty virtual row in band 0, which writes its zeros).
__device__ __forceinline__ bool row_is_light(const RowBands& rb, int P, int T) {
  for (int b = 0; b < P; ++b)
    if (rb.pos[b + 1] - rb.pos[b] > T) return false;
  return true;
}

// Per row: virtual rows, partial-sum slots, fix-up segments (a row's slots in
// runs of at most VR_SEG), whether it is a long row (more than one segment:
// its segment sums are combined by a second pass) and its segment sums; per
// band (atomically, into band_cnt): the virtual rows of that band.
template <class PtrT>
__global__ void vrow_count_k(int64_t nrows, const PtrT* __restrict__ ptr, const int* __restrict__ idx,
                             int base, int T, int P, int64_t W, int64_t* __restrict__ nv,
                             int64_t* __restrict__ nl, int64_t* __restrict__ nseg,
                             int64_t* __restrict__ nlong, int64_t* __restrict__ nss,
                             unsigned long long* __restrict__ band_cnt) {
  unsigned long long mine[VR_MAX_BANDS] = {};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b0 = ld_ptr(ptr, r) - base;
    const int64_t len = ld_ptr(ptr, r + 1) - base - b0;
    RowBands rb;
    if (P > 1) row_bands(idx, b0, len, base, P, W, rb);
    else {
      rb.pos[0] = 0;
      rb.pos[1] = len;
    }
    int64_t nch = 0, slots = 0;
    if (row_is_light(rb, P, T)) {
      for (int b = 0; b < P; ++b)
        if (rb.pos[b + 1] > rb.pos[b]) {
          ++nch;
          ++mine[b];
        }
      if (nch == 0) {
        nch = 1;
        ++mine[0];
      }
    } else {
      for (int b = 0; b < P; ++b) {
        const int64_t lb = rb.pos[b + 1] - rb.pos[b];
        const int64_t c = (lb + T - 1) / T;
        nch += c;
        mine[b] += (unsigned long long)c;
      }
      slots = nch - 1;
    }
    const int64_t segs = (slots + VR_SEG - 1) / VR_SEG;
    nv[r] = nch;
    nl[r] = slots;
    nseg[r] = segs;
    nlong[r] = segs > 1 ? 1 : 0;
    nss[r] = segs > 1 ? segs : 0;
  }
  for (int b = 0; b < P; ++b)
    if (mine[b]) atomicAdd(band_cnt + b, mine[b]);
}

__device__ __forceinline__ uint8_t vrow_class(int64_t len) {
  // longest first: class 0 holds the longest lengths
  const int b = len <= 0 ? 0 : 64 - __clzll((unsigned long long)len);  // 1 + floor(log2 len)
  return (uint8_t)(15 - b);
}

// The virtual rows of every row (unsorted, with their band and length-class
// keys) and its fix-up records.  soff/goff/ssoff: exclusive scans of the
// segments, the long rows and the segment sums (vrow_count_k).  Record w:
// -1 writes C, -2 adds to C (a light row's later band), >= 0 a partial slot.
template <class PtrT>
__global__ void vrow_fill_k(int64_t nrows, const PtrT* __restrict__ ptr, const int* __restrict__ idx,
                            int base, int T, int P, int64_t W, const int64_t* __restrict__ voff,
                            const int64_t* __restrict__ loff, const int64_t* __restrict__ soff,
                            const int64_t* __restrict__ goff, const int64_t* __restrict__ ssoff,
                            uint8_t* __restrict__ key, int32_t* __restrict__ ord,
                            int4* __restrict__ unsorted, int4* __restrict__ seg, int4* __restrict__ lrow) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b0 = ld_ptr(ptr, r) - base;
    const int64_t len = ld_ptr(ptr, r + 1) - base - b0;
    RowBands rb;
    if (P > 1) row_bands(idx, b0, len, base, P, W, rb);
    else {
      rb.pos[0] = 0;
      rb.pos[1] = len;
    }
    const int64_t v0 = voff[r], l0 = loff[r];
    int64_t c = 0;  // virtual rows written so far
    auto emit = [&](int b, int64_t first, int64_t clen, int w) {
      const int64_t v = v0 + c;
      // band, then the records that continue C (w = -2) after all others,
      // then length class: a launch reaches the records that need the
      // previous launch's C last (programmatic dependent launch)
      key[v] = (uint8_t)((b << 5) | (w == -2 ? 16 : 0) | vrow_class(clen));
      ord[v] = (int32_t)v;
      unsorted[v] = make_int4((int)r, (int)(b0 + first), (int)clen, w);
      ++c;
    };
    if (row_is_light(rb, P, T)) {
      for (int b = 0; b < P; ++b) {
        const int64_t lb = rb.pos[b + 1] - rb.pos[b];
        if (lb > 0) emit(b, rb.pos[b], lb, c == 0 ? -1 : -2);
      }
      if (c == 0) emit(0, 0, 0, -1);
    } else {
      for (int b = 0; b < P; ++b)
        for (int64_t f = rb.pos[b]; f < rb.pos[b + 1]; f += T) {
          const int64_t clen = rb.pos[b + 1] - f < T ? rb.pos[b + 1] - f : T;
          emit(b, f, clen, c == 0 ? -1 : (int)(l0 + c - 1));
        }
    }
    const int64_t slots = loff[r + 1] - l0, s0 = soff[r], segs = soff[r + 1] - s0;
    if (segs == 1) {
      seg[s0] = make_int4((int)r, (int)l0, (int)slots, -1);
    } else if (segs > 1) {
      const int64_t ss0 = ssoff[r];
      for (int64_t g = 0; g < segs; ++g) {
        const int64_t first = g * VR_SEG;
        const int64_t n = slots - first < VR_SEG ? slots - first : VR_SEG;
        seg[s0 + g] = make_int4((int)r, (int)(l0 + first), (int)n, (int)(ss0 + g));
      }
      lrow[goff[r]] = make_int4((int)r, (int)ss0, (int)segs, 0);
    }
  }
}

__global__ void vrow_gather_k(int64_t nv, const int32_t* __restrict__ ord,
                              const int4* __restrict__ unsorted, int4* __restrict__ vr) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv;
       i += (int64_t)gridDim.x * blockDim.x)
    vr[i] = unsorted[ord[i]];
}

// Programmatic dependent launch: the launches of one SpMM after its first
// may start while the previous one drains (its blocks take the SMs the
// previous launch frees).  A launch signals at once that its successor may
// start, waits for its predecessor before its first record that reads C
// (w = -2, sorted last) and before it exits, so a launch that completes
// implies that every earlier one did.  In a launch made without the
// attribute both instructions return at once.
__device__ __forceinline__ void pdl_allow_next() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait_prev() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// The start of a virtual row: a light row's later column band (w = -2)
// continues the running sum its earlier bands left in C, so the row is one
// sequential sum over its entries in storage order, as without bands.
__device__ __forceinline__ float4 vrow_init(const int4& rec, const float* __restrict__ C, int64_t ldc,
                                            int64_t col, bool active) {
  if (rec.w == -2 && active) return *reinterpret_cast<const float4*>(C + (int64_t)rec.x * ldc + col);
  return make_float4(0.f, 0.f, 0.f, 0.f);
}

// The end of a virtual row: w = -1 writes C (adds to it under `accumulate`),
// w = -2 writes the continued running sum back to C, w >= 0 writes
// partial-sum slot w.
__device__ __forceinline__ void vrow_store(const int4& rec, float4 acc, float* __restrict__ C, int64_t ldc,
                                           int64_t col, int64_t nk, int accumulate, float* __restrict__ partial,
                                           uint64_t pol_stream) {
  if (rec.w < 0) {
    float* dst = C + (int64_t)rec.x * ldc + col;
    if (accumulate && rec.w == -1) {
      const float4 o = *reinterpret_cast<const float4*>(dst);
      acc.x += o.x;
      acc.y += o.y;
      acc.z += o.z;
      acc.w += o.w;
    }
    st_stream_f32x4(dst, acc, pol_stream);
  } else {
    *reinterpret_cast<float4*>(partial + (int64_t)rec.w * nk + col) = acc;
  }
}

// One launch: C[:, c0 : c0 + 4L] (or the partial sums) for every virtual row.
// NB gathers of B are in flight per lane; fewer blocks per SM leave room for
// more (the 128-byte gathers of 32-column slabs want the extra depth).
template <int L, int NB, int MINB>
__global__ void __launch_bounds__(VR_THREADS, MINB) spmm_vrow_k(
    int64_t nv, const int4* __restrict__ vr, const int* __restrict__ idx,
    const float* __restrict__ val, const float* __restrict__ B, int64_t ldb, float* __restrict__ C,
    int64_t ldc, int64_t c0, int64_t nk, int base, int accumulate, float* __restrict__ partial) {
  constexpr int PER = NB / L;  // entries each lane loads per batch
  static_assert(PER * L == NB, "batch must be a multiple of the sub-group");
  const int lane = threadIdx.x & 31, sl = lane % L;
  const unsigned gmask = group_mask<L>();
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / L;
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / L;
  const int64_t col = c0 + (int64_t)sl * 4;
  const bool active = col < nk;
  const float* Bc = B + col;
  const uint64_t pol_stream = policy_evict_first();
  const uint64_t pol_keep = policy_evict_last();
  pdl_allow_next();
  bool waited = false;
  for (int64_t v = gid; v < nv; v += ngroups) {
    const int4 rec = __ldg(vr + v);  // row, first entry, length, partial slot
    if (rec.w == -2 && !waited) {
      pdl_wait_prev();
      waited = true;
    }
    const int len = rec.z;
    const int* ix = idx + rec.y;
    const float* vx = val + rec.y;
    float4 acc = vrow_init(rec, C, ldc, col, active);
    for (int t = 0; t < len; t += NB) {
      int j[PER];
      float a[PER];
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int p = t + sl + L * q;
        j[q] = 0;
        a[q] = 0.f;
        if (p < len) {
          j[q] = ld_stream_i32(ix + p, pol_stream) - base;
          a[q] = ld_stream_f32(vx + p, pol_stream);
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
    vrow_store(rec, acc, C, ldc, col, nk, accumulate, partial, pol_stream);
  }
  if (!waited) pdl_wait_prev();  // completion of this launch implies its predecessor's
}

// The same launch with the gathers staged in shared memory by cp.async
// instead of held in registers: a lane's NB float4 gathers land in its own
// slots, so no registers wait on memory, more warps fit per SM and more
// gathers are in flight per SM for the same NB.  Accumulation order is the
// register kernel's, so results are identical.
__device__ __forceinline__ void cp_async16_keep(void* smem, const void* gmem, uint64_t pol) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(sa), "l"(gmem), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// ALL: every lane's 4 columns lie inside nk (nk a multiple of 4L), so no
// lane is masked.  A full batch (NB entries left) runs without per-entry
// predicates; ldb fits 32 bits, so a gather address is one 32x32->64
// multiply-add.
template <int L, int NB, int MINB, bool ALL>
__global__ void __launch_bounds__(VR_THREADS, MINB) spmm_vrow_async_k(
    int64_t nv, const int4* __restrict__ vr, const int* __restrict__ idx,
    const float* __restrict__ val, const float* __restrict__ B, int ldb, float* __restrict__ C,
    int64_t ldc, int64_t c0, int64_t nk, int base, int accumulate, float* __restrict__ partial) {
  constexpr int PER = NB / L;
  static_assert(PER * L == NB, "batch must be a multiple of the sub-group");
  extern __shared__ float4 vr_stage[];  // [NB][VR_THREADS]: slot u of thread t at u * VR_THREADS + t
  const int lane = threadIdx.x & 31, sl = lane % L;
  const unsigned gmask = group_mask<L>();
  const int gid = (int)((blockIdx.x * blockDim.x + threadIdx.x) / L);  // nv < 2^31 (vrow_build)
  const int ngroups = (int)((gridDim.x * blockDim.x) / L);
  const int64_t col = c0 + (int64_t)sl * 4;
  const bool active = ALL || col < nk;
  const float* Bc = B + col;
  float4* slot = vr_stage + threadIdx.x;
  const uint64_t pol_stream = policy_evict_first();
  const uint64_t pol_keep = policy_evict_last();
  pdl_allow_next();
  bool waited = false;
  for (int v = gid; v < nv; v += ngroups) {
    const int4 rec = __ldg(vr + v);
    if (rec.w == -2 && !waited) {
      pdl_wait_prev();
      waited = true;
    }
    const int len = rec.z;
    const int* ix = idx + rec.y;
    const float* vx = val + rec.y;
    float4 acc = vrow_init(rec, C, ldc, col, active);
    for (int t = 0; t < len; t += NB) {
      int j[PER];
      float a[PER];
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int p = t + sl + L * q;
        j[q] = 0;
        a[q] = 0.f;
        if (p < len) {
          j[q] = ld_stream_i32(ix + p, pol_stream) - base;
          a[q] = ld_stream_f32(vx + p, pol_stream);
        }
      }
      if (t + NB <= len && active) {  // full batch
#pragma unroll
        for (int u = 0; u < NB; ++u) {
          const int jj = __shfl_sync(gmask, j[u / L], u % L, L);
          cp_async16_keep(slot + u * VR_THREADS, Bc + (int64_t)jj * ldb, pol_keep);
        }
        cp_async_wait_all();
#pragma unroll
        for (int u = 0; u < NB; ++u) {
          const float aa = __shfl_sync(gmask, a[u / L], u % L, L);
          const float4 b = slot[u * VR_THREADS];
          acc.x = __fmaf_rn(aa, b.x, acc.x);
          acc.y = __fmaf_rn(aa, b.y, acc.y);
          acc.z = __fmaf_rn(aa, b.z, acc.z);
          acc.w = __fmaf_rn(aa, b.w, acc.w);
        }
        continue;
      }
#pragma unroll
      for (int u = 0; u < NB; ++u) {
        const int jj = __shfl_sync(gmask, j[u / L], u % L, L);
        if (t + u < len && active) cp_async16_keep(slot + u * VR_THREADS, Bc + (int64_t)jj * ldb, pol_keep);
      }
      cp_async_wait_all();
#pragma unroll
      for (int u = 0; u < NB; ++u) {
        const float aa = __shfl_sync(gmask, a[u / L], u % L, L);
        if (t + u < len && active) {
          const float4 b = slot[u * VR_THREADS];
          acc.x = __fmaf_rn(aa, b.x, acc.x);
          acc.y = __fmaf_rn(aa, b.y, acc.y);
          acc.z = __fmaf_rn(aa, b.z, acc.z);
          acc.w = __fmaf_rn(aa, b.w, acc.w);
        }
      }
    }
    if (!active) continue;
    vrow_store(rec, acc, C, ldc, col, nk, accumulate, partial, pol_stream);
  }
  if (!waited) pdl_wait_prev();  // completion of this launch implies its predecessor's
}

// Sums `n` partial-sum slots starting at `p` (rows of nk floats) in slot
// order, 4 columns per lane starting at column c.
__device__ __forceinline__ float4 vrow_sum_slots(const float* __restrict__ p, int64_t n, int64_t nk) {
  float4 sum = *reinterpret_cast<const float4*>(p);
  for (int64_t k0 = 1; k0 < n; k0 += 8) {
    float4 x[8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (k0 + u < n) x[u] = *reinterpret_cast<const float4*>(p + (k0 + u) * nk);
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (k0 + u < n) {
        sum.x += x[u].x;
        sum.y += x[u].y;
        sum.z += x[u].z;
        sum.w += x[u].w;
      }
  }
  return sum;
}

__device__ __forceinline__ void vrow_add_row(float* __restrict__ dst, float4 sum) {
  float4 o = *reinterpret_cast<float4*>(dst);
  o.x += sum.x;
  o.y += sum.y;
  o.z += sum.z;
  o.w += sum.w;
  *reinterpret_cast<float4*>(dst) = o;
}

// Fix-up, pass 1: one warp per segment (at most VR_SEG partial-sum slots of
// one row, 4 columns per lane), its slots summed in order.  A row with one
// segment adds the sum to C; a long row's segments leave their sums in
// `segsum` for pass 2.  A long row's slots are thus summed by many warps at
// once instead of one warp walking all of them.
__global__ void vrow_fixup_seg_k(int64_t nseg, int64_t nk, const int4* __restrict__ seg,
                                 const float* __restrict__ partial, float* __restrict__ segsum,
                                 float* __restrict__ C, int64_t ldc) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < nseg; w += nwarps) {
    const int4 rec = seg[w];  // row, first slot, slots, segment-sum slot (-1: C)
    for (int64_t c = (int64_t)lane * 4; c < nk; c += 128) {
      const float4 sum = vrow_sum_slots(partial + (int64_t)rec.y * nk + c, rec.z, nk);
      if (rec.w < 0) vrow_add_row(C + (int64_t)rec.x * ldc + c, sum);
      else *reinterpret_cast<float4*>(segsum + (int64_t)rec.w * nk + c) = sum;
    }
  }
}

// Fix-up, pass 2: one warp per long row, its segment sums added in order to C.
__global__ void vrow_fixup_rows_k(int64_t nlong, int64_t nk, const int4* __restrict__ lrow,
                                  const float* __restrict__ segsum, float* __restrict__ C, int64_t ldc) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < nlong; w += nwarps) {
    const int4 rec = lrow[w];  // row, first segment sum, segments
    for (int64_t c = (int64_t)lane * 4; c < nk; c += 128)
      vrow_add_row(C + (int64_t)rec.x * ldc + c, vrow_sum_slots(segsum + (int64_t)rec.y * nk + c, rec.z, nk));
  }
}

static inline size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

template <class PtrT>
static int vrow_build_t(fgb_ctx* ctx, const fgb_sparse* A, int T, int P, VrowSchedule* out, cudaStream_t s,
                        bool pooled) {
  const int64_t nrows = A->nrows;
  const PtrT* ptr = (const PtrT*)A->ptr;
  const int grid = grid_for(nrows, 256, ctx->num_sms);
  // Temporaries come from the stream-ordered pool (kept mapped across calls);
  // the schedule itself too when `pooled` (a schedule built for one call).
  int64_t *cnt_v = nullptr, *cnt_l = nullptr, *voff = nullptr, *loff = nullptr;
  int64_t *cnt_s = nullptr, *cnt_g = nullptr, *cnt_ss = nullptr, *soff = nullptr, *goff = nullptr,
          *ssoff = nullptr;
  void* cub_tmp = nullptr;
  char* tmp = nullptr;
  char* mem = nullptr;
  unsigned long long* band_cnt = nullptr;
  size_t cub_bytes = 0, b2 = 0;
  cudaError_t e = cudaSuccess;
  auto release = [&](bool keep_schedule) {
    for (void* q : {(void*)cnt_v, (void*)cnt_l, (void*)voff, (void*)loff, (void*)cnt_s, (void*)cnt_g,
                    (void*)cnt_ss, (void*)soff, (void*)goff, (void*)ssoff, cub_tmp, (void*)tmp,
                    (void*)band_cnt})
      if (q) cudaFreeAsync(q, s);
    if (!keep_schedule && mem) {
      if (pooled) cudaFreeAsync(mem, s);
      else cudaFree(mem);
      *out = VrowSchedule{};
    }
  };
  auto fail = [&](const char* what) {
    release(false);
    return set_error(e == cudaErrorMemoryAllocation ? FGB_ENOMEM : FGB_ECUDA, "vrow schedule: %s: %s",
                     what, cudaGetErrorString(e));
  };
  const size_t rows_bytes = sizeof(int64_t) * (nrows + 1);
  if ((e = cudaMallocAsync((void**)&cnt_v, rows_bytes, s)) != cudaSuccess) return fail("alloc");
  if ((e = cudaMallocAsync((void**)&cnt_l, rows_bytes, s)) != cudaSuccess) return fail("alloc");
  if ((e = cudaMallocAsync((void**)&voff, rows_bytes, s)) != cudaSuccess) return fail("alloc");
  if ((e = cudaMallocAsync((void**)&loff, rows_bytes, s)) != cudaSuccess) return fail("alloc");
  for (int64_t** q : {&cnt_s, &cnt_g, &cnt_ss, &soff, &goff, &ssoff})
    if ((e = cudaMallocAsync((void**)q, rows_bytes, s)) != cudaSuccess) return fail("alloc");
  if ((e = cudaMallocAsync((void**)&band_cnt, sizeof(unsigned long long) * VR_MAX_BANDS, s)) != cudaSuccess)
    return fail("alloc");
  cudaMemsetAsync(band_cnt, 0, sizeof(unsigned long long) * VR_MAX_BANDS, s);
  for (int64_t* q : {cnt_v, cnt_l, cnt_s, cnt_g, cnt_ss}) cudaMemsetAsync(q + nrows, 0, sizeof(int64_t), s);
  const int64_t W = (A->ncols + P - 1) / P;  // columns per band
  const int* idx = (const int*)A->idx;
  vrow_count_k<PtrT><<<grid, 256, 0, s>>>(nrows, ptr, idx, A->index_base, T, P, W, cnt_v, cnt_l, cnt_s, cnt_g,
                                          cnt_ss, band_cnt);
  cub::DeviceScan::ExclusiveSum(nullptr, cub_bytes, cnt_v, voff, nrows + 1, s);
  if ((e = cudaMallocAsync(&cub_tmp, cub_bytes, s)) != cudaSuccess) return fail("alloc");
  if ((e = cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, cnt_v, voff, nrows + 1, s)) != cudaSuccess)
    return fail("scan");
  const int64_t* cnts[5] = {cnt_v, cnt_l, cnt_s, cnt_g, cnt_ss};
  int64_t* offs[5] = {voff, loff, soff, goff, ssoff};
  for (int q = 1; q < 5; ++q)
    if ((e = cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, cnts[q], offs[q], nrows + 1, s)) != cudaSuccess)
      return fail("scan");
  int64_t tot[5] = {0, 0, 0, 0, 0};
  unsigned long long bcnt[VR_MAX_BANDS] = {};
  for (int q = 0; q < 5; ++q)
    cudaMemcpyAsync(&tot[q], offs[q] + nrows, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(bcnt, band_cnt, sizeof(bcnt), cudaMemcpyDeviceToHost, s);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail("count");
  const int64_t nv = tot[0], nl = tot[1], nseg = tot[2], nlong = tot[3], nss = tot[4];
  if (nv > INT32_MAX || nl > INT32_MAX) {
    release(false);
    return set_error(FGB_EUNSUPPORTED, "vrow schedule: too many virtual rows");
  }
  // the schedule: sorted records and fix-up records; temporaries: keys, order, unsorted records
  const size_t keep = a256(16 * nv) + a256(16 * (nseg > 0 ? nseg : 1)) + a256(16 * (nlong > 0 ? nlong : 1));
  e = pooled ? cudaMallocAsync((void**)&mem, keep, s) : cudaMalloc((void**)&mem, keep);
  if (e != cudaSuccess) return fail("alloc");
  out->vr = (int4*)mem;
  out->seg = (int4*)(mem + a256(16 * nv));
  out->lrow = (int4*)(mem + a256(16 * nv) + a256(16 * (nseg > 0 ? nseg : 1)));
  out->nseg = nseg;
  out->nlong = nlong;
  out->nss = nss;
  out->mem = mem;
  out->pooled = pooled;
  out->nv = nv;
  out->nl = nl;
  out->T = T;
  out->nbands = P;
  out->band_off[0] = 0;
  for (int b = 0; b < P; ++b) out->band_off[b + 1] = out->band_off[b] + (int64_t)bcnt[b];
  const size_t tmp_bytes = a256(nv) * 2 + a256(4 * nv) * 2 + a256(16 * nv);
  if ((e = cudaMallocAsync((void**)&tmp, tmp_bytes, s)) != cudaSuccess) return fail("alloc");
  uint8_t* key = (uint8_t*)tmp;
  uint8_t* key2 = (uint8_t*)(tmp + a256(nv));
  int32_t* ord = (int32_t*)(tmp + 2 * a256(nv));
  int32_t* ord2 = (int32_t*)(tmp + 2 * a256(nv) + a256(4 * nv));
  int4* unsorted = (int4*)(tmp + 2 * a256(nv) + 2 * a256(4 * nv));
  vrow_fill_k<PtrT><<<grid, 256, 0, s>>>(nrows, ptr, idx, A->index_base, T, P, W, voff, loff, soff, goff, ssoff,
                                         key, ord, unsorted, out->seg, out->lrow);
  const int end_bit = P > 1 ? 8 : 4;  // key: band << 5 | continues-C << 4 | length class
  b2 = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, b2, key, key2, ord, ord2, (int)nv, 0, end_bit, s);
  if (b2 > cub_bytes) {
    cudaFreeAsync(cub_tmp, s);
    cub_tmp = nullptr;
    if ((e = cudaMallocAsync(&cub_tmp, b2, s)) != cudaSuccess) return fail("alloc");
    cub_bytes = b2;
  }
  e = cub::DeviceRadixSort::SortPairs(cub_tmp, cub_bytes, key, key2, ord, ord2, (int)nv, 0, end_bit, s);
  if (e == cudaSuccess) {
    vrow_gather_k<<<grid_for(nv, 256, ctx->num_sms), 256, 0, s>>>(nv, ord2, unsorted, out->vr);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return fail("sort");
  release(true);  // stream-ordered: the schedule is ready for the next launch on s
  return FGB_OK;
}

int vrow_build(fgb_ctx* ctx, const fgb_sparse* A, int T, VrowSchedule* out, cudaStream_t s, bool pooled,
               int bands) {
  *out = VrowSchedule{};
  if (A->orient != FGB_CSR) return set_error(FGB_EUNSUPPORTED, "vrow schedule: CSR only");
  if (T < 8 || T > 4096) return set_error(FGB_EINVAL, "vrow schedule: chunk %d outside [8, 4096]", T);
  if (bands < 1 || bands > VR_MAX_BANDS)
    return set_error(FGB_EINVAL, "vrow schedule: %d column bands outside [1, %d]", bands, VR_MAX_BANDS);
  if (bands > 1 && A->idx_t != FGB_I32)
    return set_error(FGB_EUNSUPPORTED, "vrow schedule: column bands need int32 indices");
  if (A->nrows > INT32_MAX || A->nnz > INT32_MAX)
    return set_error(FGB_EUNSUPPORTED, "vrow schedule: needs fewer than 2^31 rows and entries");
  return A->ptr_t == FGB_I32 ? vrow_build_t<int32_t>(ctx, A, T, bands, out, s, pooled)
                             : vrow_build_t<int64_t>(ctx, A, T, bands, out, s, pooled);
}

void vrow_free(VrowSchedule* v, cudaStream_t s) {
  if (v && v->mem) {
    if (v->pooled) cudaFreeAsync(v->mem, s);
    else cudaFree(v->mem);
  }
  if (v) *v = VrowSchedule{};
}

template <int L, int NB, int MINB, bool ASYNC, bool ALL = false>
static int launch_vrow(fgb_ctx* ctx, const VrowSchedule& v, const fgb_sparse* A, const float* B,
                       int64_t ldb, int64_t nk, float* C, int64_t ldc, int accumulate, float* partial,
                       cudaStream_t s) {
  if constexpr (ASYNC) {
    if (!ALL && nk % (4 * L) == 0)  // no masked lanes: the unmasked build
      return launch_vrow<L, NB, MINB, true, true>(ctx, v, A, B, ldb, nk, C, ldc, accumulate, partial, s);
  }
  auto kern = [] {
    if constexpr (ASYNC) return spmm_vrow_async_k<L, NB, MINB, ALL>;
    else return spmm_vrow_k<L, NB, MINB>;
  }();
  using LdT = std::conditional_t<ASYNC, int, int64_t>;
  const size_t smem = ASYNC ? sizeof(float4) * NB * VR_THREADS : 0;
  static const int occ = [&] {  // once per process (one device model); thread-safe
    if (ASYNC) {
      cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    int o = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, VR_THREADS, smem);
    return o > 0 ? o : 1;
  }();
  // slab after slab; inside a slab, band after band (a light row's later
  // bands continue what its earlier bands wrote).  Every launch after the
  // first may start while its predecessor drains (programmatic dependent
  // launch); the first waits for whatever the stream ran before.
  cudaLaunchAttribute pdl[1];
  pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  pdl[0].val.programmaticStreamSerializationAllowed = 1;
  bool first = true;
  for (int64_t c0 = 0; c0 < nk; c0 += 4 * L)
    for (int b = 0; b < v.nbands; ++b) {
      const int64_t nvb = v.nbands > 1 ? v.band_off[b + 1] - v.band_off[b] : v.nv;
      if (nvb == 0) continue;
      const int64_t need = (nvb * L + VR_THREADS - 1) / VR_THREADS;
      const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)occ * ctx->num_sms));
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(grid);
      cfg.blockDim = dim3(VR_THREADS);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = s;
      cfg.attrs = first ? nullptr : pdl;
      cfg.numAttrs = first ? 0 : 1;
      FGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, (int64_t)nvb, (const int4*)(v.vr + (v.nbands > 1 ? v.band_off[b] : 0)),
                                      (const int*)A->idx, (const float*)A->val, B, (LdT)ldb, C, (int64_t)ldc,
                                      (int64_t)c0, (int64_t)nk, (int)A->index_base, accumulate, partial));
      first = false;
    }
  if (v.nseg > 0) {  // segment sums live after the nl partial-sum slots
    float* segsum = partial + (int64_t)v.nl * nk;
    vrow_fixup_seg_k<<<grid_for(v.nseg * 32, 256, ctx->num_sms), 256, 0, s>>>(v.nseg, nk, v.seg, partial,
                                                                            segsum, C, ldc);
    if (v.nlong > 0)
      vrow_fixup_rows_k<<<grid_for(v.nlong * 32, 256, ctx->num_sms), 256, 0, s>>>(v.nlong, nk, v.lrow, segsum,
                                                                                 C, ldc);
  }
  FGB_CUDA_TRY(cudaGetLastError());
  return FGB_OK;
}

size_t spmm_vrow_scratch_bytes(const VrowSchedule& v, int64_t nk) {
  return sizeof(float) * (size_t)(v.nl + v.nss) * (size_t)nk;  // partial sums, then segment sums
}

int spmm_vrow(fgb_ctx* ctx, const VrowSchedule& v, const fgb_sparse* A, const void* B, int64_t ldb,
              int64_t nk, void* C, int64_t ldc, int accumulate, int slab, void* partial,
              cudaStream_t s, bool async_gather) {
  if (A->val_t != FGB_F32 || A->idx_t != FGB_I32)
    return set_error(FGB_EUNSUPPORTED, "spmm vrow: F32 values and int32 indices only");
  if (nk % 4 || ldb % 4 || ldc % 4 || (uintptr_t)B % 16 || (uintptr_t)C % 16)
    return set_error(FGB_EUNSUPPORTED, "spmm vrow: needs 16-byte aligned rows of B and C");
  if (v.nl > 0 && !partial) return set_error(FGB_EINVAL, "spmm vrow: no partial-sum scratch");
  const float* b = (const float*)B;
  float* c = (float*)C;
  float* part = (float*)partial;
  if (async_gather && ldb > INT32_MAX)
    return set_error(FGB_EUNSUPPORTED, "spmm vrow: cp.async gathers need a leading dimension below 2^31");
  if (async_gather) {  // 32 KB of gather slots per block: 6 blocks (48 warps) per SM
    if (slab == 8) return launch_vrow<2, 8, 6, true>(ctx, v, A, b, ldb, nk, c, ldc, accumulate, part, s);
    if (slab == 16) return launch_vrow<4, 8, 6, true>(ctx, v, A, b, ldb, nk, c, ldc, accumulate, part, s);
    if (slab == 32) return launch_vrow<8, 8, 6, true>(ctx, v, A, b, ldb, nk, c, ldc, accumulate, part, s);
  } else {
    if (slab == 8) return launch_vrow<2, 8, 4, false>(ctx, v, A, b, ldb, nk, c, ldc, accumulate, part, s);
    if (slab == 16) return launch_vrow<4, 8, 4, false>(ctx, v, A, b, ldb, nk, c, ldc, accumulate, part, s);
    if (slab == 32) return launch_vrow<8, 8, 4, false>(ctx, v, A, b, ldb, nk, c, ldc, accumulate, part, s);
  }
  return set_error(FGB_EINVAL, "spmm vrow: slab %d not in {8, 16, 32}", slab);
}

}  // namespace fgb
