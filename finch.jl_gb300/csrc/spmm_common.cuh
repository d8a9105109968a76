// Vector helpers shared by the SpMM kernels: V consecutive k of a row of B
// or C per lane, gathered with an L2 cache policy.
#pragma once

#include "fgb_internal.cuh"
#include "semiring.cuh"

namespace fgb {

// fgb_spmm's dispatcher (spmm.cu); lanes/path 0 = defaults.
int spmm_impl(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk, void* C,
              int64_t ldc, int dtype, unsigned flags, int lanes, int64_t path, void* stream,
              int variant = 0, int bands = 1);

// Merge-path SpMM (spmm_merge.cu).
size_t spmm_merge_scratch_bytes(int64_t nrows, int64_t nnz, int64_t nk, size_t esz, int64_t path);
// plan_ready: the item boundaries in `scratch` are already those of (A, path)
// (computed by an earlier call on the same scratch), so only the slab kernels
// and the fix-up run.  row_map (optional): row r of A is row row_map[r] of C
// (A lists only some rows of the product, e.g. one column panel's rows).
int spmm_merge(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk, void* C,
               int64_t ldc, int dtype, int accumulate, int lanes, int64_t path, void* scratch,
               size_t scratch_bytes, cudaStream_t s, bool plan_ready = false,
               const int32_t* row_map = nullptr, int variant = 0);

// Virtual-row column-slab SpMM (spmm_vrow.cu): rows cut into virtual rows of
// at most T entries, sorted by length class; built once per matrix.
struct VrowSchedule {
  int64_t nv = 0, nl = 0;  // virtual rows; partial-sum slots (chunks after a row's first)
  int T = 0;
  int4* vr = nullptr;      // per virtual row (sorted): row, first entry, length, partial
                           // slot (-1: writes C, -2: adds to C)
  // fix-up of the partial sums: segments of at most 16 slots of one row
  // {row, first slot, slots, segment-sum slot (-1: add to C directly)}, and the
  // long rows {row, first segment-sum slot, segments, 0} whose segment sums a
  // second pass adds to C in order
  int64_t nseg = 0, nlong = 0, nss = 0;
  int4* seg = nullptr;
  int4* lrow = nullptr;
  void* mem = nullptr;
  bool pooled = false;  // mem from the stream-ordered pool (a schedule for one call)
  // column bands: band b's virtual rows are vr[band_off[b] .. band_off[b+1])
  // and run in launches of their own, band after band (1 = no bands)
  int nbands = 1;
  int64_t band_off[9] = {};
};
// pooled: allocate the schedule from the stream-ordered pool, to be freed by
// vrow_free on a stream (a schedule built for one call); else cudaMalloc
// (a plan's).  Stream-ordered: the schedule is ready for launches on s.
// bands (1..8): cut A's columns into that many bands of consecutive columns,
// each band's entries in launches of their own (SpMM only).
int vrow_build(fgb_ctx* ctx, const fgb_sparse* A, int T, VrowSchedule* out, cudaStream_t s,
               bool pooled = false, int bands = 1);
void vrow_free(VrowSchedule* v, cudaStream_t s = nullptr);
// partial: the long rows' partial sums (spmm_vrow_scratch_bytes).
size_t spmm_vrow_scratch_bytes(const VrowSchedule& v, int64_t nk);
// slab: 8, 16 or 32 columns per launch.  async_gather: gathers staged in
// shared memory by cp.async (more warps per SM) instead of in registers.
int spmm_vrow(fgb_ctx* ctx, const VrowSchedule& v, const fgb_sparse* A, const void* B, int64_t ldb,
              int64_t nk, void* C, int64_t ldc, int accumulate, int slab, void* partial,
              cudaStream_t s, bool async_gather = false);

// SDDMM over the same virtual rows (sddmm_vrow.cu): F32 CSR, k <= 128, k % 4 == 0.
// slab: columns of k per launch (0 = all of k), a multiple of 4.
// async_gather: gathers of Y staged in shared memory by cp.async.
int sddmm_vrow(fgb_ctx* ctx, const VrowSchedule& v, const fgb_sparse* A, const void* X, int64_t ldx,
               const void* Y, int64_t ldy, int64_t k, void* out, cudaStream_t s, int64_t slab = 0,
               bool async_gather = false);

// Stage-ring (TMA gather4) kernels over planned merge-path items (spmm_tma.cu).
int spmm_tma_items(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk,
                   void* C, int64_t ldc, int accumulate, int64_t n_items, const int64_t* plan_row,
                   const int64_t* plan_k, int64_t* carry_row, void* carry, const int32_t* row_map,
                   int* err, cudaStream_t s);

template <class T, int V>
struct VecT {
  T v[V];
};

template <class T, int V>
__device__ __forceinline__ VecT<T, V> gather(const T* p, uint64_t pol);

template <>
__device__ __forceinline__ VecT<float, 4> gather<float, 4>(const float* p, uint64_t pol) {
  float4 f = ld_gather_f32x4(p, pol);
  return VecT<float, 4>{{f.x, f.y, f.z, f.w}};
}
template <>
__device__ __forceinline__ VecT<double, 2> gather<double, 2>(const double* p, uint64_t pol) {
  double2 d;
  asm volatile("ld.global.nc.L2::cache_hint.v2.f64 {%0,%1}, [%2], %3;"
               : "=d"(d.x), "=d"(d.y)
               : "l"(p), "l"(pol));
  return VecT<double, 2>{{d.x, d.y}};
}
template <>
__device__ __forceinline__ VecT<float, 1> gather<float, 1>(const float* p, uint64_t) {
  return VecT<float, 1>{{__ldg(p)}};
}
template <>
__device__ __forceinline__ VecT<double, 1> gather<double, 1>(const double* p, uint64_t) {
  return VecT<double, 1>{{__ldg(p)}};
}

template <class T, int V>
__device__ __forceinline__ void store_out(T* p, const VecT<T, V>& a, uint64_t pol) {
#pragma unroll
  for (int q = 0; q < V; ++q) p[q] = a.v[q];
}
template <>
__device__ __forceinline__ void store_out<float, 4>(float* p, const VecT<float, 4>& a,
                                                     uint64_t pol) {
  st_stream_f32x4(p, make_float4(a.v[0], a.v[1], a.v[2], a.v[3]), pol);
}

template <class T, int V>
__device__ __forceinline__ VecT<T, V> load_out(const T* p) {
  VecT<T, V> r;
#pragma unroll
  for (int q = 0; q < V; ++q) r.v[q] = p[q];
  return r;
}

// Value of stored entry p as the accumulation type.
template <class T, class VT>
__device__ __forceinline__ T load_val(const VT* val, int64_t p, uint64_t pol) {
  return to_acc<T>(__ldg(val + p));
}
template <>
__device__ __forceinline__ float load_val<float, float>(const float* val, int64_t p, uint64_t pol) {
  return ld_stream_f32(val + p, pol);
}

template <class T, int V>
__device__ __forceinline__ void acc_step(VecT<T, V>& acc, T a, const VecT<T, V>& b, int fm) {
#pragma unroll
  for (int q = 0; q < V; ++q) acc.v[q] = Semi<SR_PT, T>::step(acc.v[q], a, b.v[q], fm);
}

}  // namespace fgb
