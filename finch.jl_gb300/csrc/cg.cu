// Conjugate gradients for SPD CSR systems, the Finch-expressed solver
//
//   q = A p          @einsum q[i] += A[i,j] * p[j]
//   alpha = rr / p.q @einsum s[] += p[i] * q[i]
//   x += alpha p;  r -= alpha q;  rr' = r.r;  p = r + (rr'/rr) p
//
// run on the GPU in one of five arithmetic modes:
//   FP64          values, sums, vectors and updates in FP64;
//   FP32 sums     FP32 or BF16 values times an FP32 copy of p, summed in
//                 FP32; x, r, p, q, dots and updates FP64;
//   FP64 sums     FP32 or BF16 values widened to FP64 and summed in FP64;
//   SpMV pairs    FP32 or BF16 values times p split into a pair of FP32
//                 numbers by integer operations, each row summed as a pair;
//                 x, r, p, q, dots and updates FP64;
//   pair sums     FP32 or BF16 values, and everything per row or per stored
//                 entry -- the SpMV sums, x, r, p, q, the dot products and
//                 updates -- in pairs of FP32 numbers (an unevaluated sum
//                 hi + lo with about 48 significant bits: Dekker's exact
//                 product through an FMA and Knuth's TwoSum, in the
//                 double-single arithmetic of Bailey's DSFUN and the QD
//                 library of Hida, Li and Bailey).  GB300 runs FP32 far
//                 faster than FP64, whose narrow pipe bounds the FP64 modes
//                 (an FP64 convert costs about as much as an FP64 FMA), so
//                 this mode executes no FP64 instruction per row or entry.
// A matrix whose columns lie within 32,767 of the diagonal is read through
// 16-bit column offsets j - i.  Accuracy is won back by reliable updates:
// every `replace_every` iterations, and whenever the recursive residual
// reaches the tolerance, the true residual r = b - A x is recomputed with
// the FP64 matrix in FP64 and replaces the recursive one (residual
// replacement keeping the search direction while the two residuals agree
// within a factor of two, restarting it from the new residual otherwise),
// and the solve stops only when that true residual is below rtol * ||b||.
//
// One iteration is three kernels -- SpMV fused with the p.q partials; the r
// update (every block folds the p.q partials itself) fused with the r.r
// partials; the x and p updates fused with the folds -- so no scalar ever
// leaves the device, and p is read once by the updates.  They are chained by
// programmatic dependent launch.  Partials are FP64
// and folded by one warp per block in a fixed order: the solve is
// deterministic.  A chunk of iterations is captured once in a CUDA graph and
// replayed; the host reads the residual history once per chunk.
#include <chrono>
#include <vector>

#include "fgb_internal.cuh"
#include "semiring.cuh"

namespace fgb {

constexpr int CG_THREADS = 256;
constexpr int CG_ILP = 4;  // elements per thread in flight in the streaming updates
// The updates run one block of 1024 threads per SM, each thread with CG_ILP
// elements in flight (up to 64 registers): few partials, one load per thread
// in each block's fold of the previous kernel's partials.
constexpr int CG_UPD_THREADS = 1024;
// Rows in flight per thread in the pair SpMVs (32-bit index build): 4
// measured slower than 2 (BF16 pair CG 0.694 against 0.637 s).
constexpr int CG_PAIR_ROWS = 2;

// The iteration kernels are chained by programmatic dependent launch: each
// lets the next one launch as soon as it starts, and waits for the previous
// one to complete (its writes visible) before touching any data.  Launched
// without the attribute, the wait returns at once.
__device__ __forceinline__ void cg_pdl_enter() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <class T>
__device__ __forceinline__ T cg_block_sum(T v, T* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : T(0);
  if (w == 0) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
  }
  return v;  // valid in thread 0
}

// The partials folded by one warp: lane l sums l, l + 32, ..., then a fixed
// shuffle tree, so every block folds them in the same order and the other
// warps spend no FP64 instruction on it.  Call from warp 0; every lane of
// it gets the sum.
__device__ __forceinline__ double warp_fold(const double* __restrict__ part, int nparts) {
  double s = 0.0;
  for (int i = threadIdx.x & 31; i < nparts; i += 32) s += part[i];
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
  return s;
}

// ---- pairs of FP32 numbers (hi + lo, |lo| <= ulp(hi) / 2)
// The intrinsics keep every operation a separately rounded IEEE operation.
__device__ __forceinline__ float2 two_sum(float a, float b) {  // Knuth: s + e == a + b exactly
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ float2 quick_two_sum(float a, float b) {  // Dekker, |a| >= |b|
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {  // the accurate pair sum
  float2 s = two_sum(a.x, b.x);
  const float2 t = two_sum(a.y, b.y);
  s = quick_two_sum(s.x, __fadd_rn(s.y, t.x));
  return quick_two_sum(s.x, __fadd_rn(s.y, t.y));
}
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {  // exact hi product by FMA
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, e));
  return quick_two_sum(p, e);
}
__device__ __forceinline__ float2 ff_from_double(double d) {
  const float hi = __double2float_rn(d);
  return make_float2(hi, __double2float_rn(d - (double)hi));
}
__device__ __forceinline__ double ff_to_double(float2 v) { return (double)v.x + (double)v.y; }

__device__ __forceinline__ float2 ff_block_sum(float2 v, float2* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1)
    v = ff_add(v, make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m)));
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : make_float2(0.f, 0.f);
  if (w == 0) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1)
      v = ff_add(v, make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m)));
  }
  return v;  // valid in thread 0
}

template <class VT>
__device__ __forceinline__ float cg_val(const VT* v, int64_t k) {
  return to_acc<float>(v[k]);
}

// Column j of stored entry k of row i: from the int32 index, or (IX =
// int16_t) from the 16-bit offset j - i of a banded matrix's compact copy.
template <class IX>
__device__ __forceinline__ int64_t cg_col(const IX* __restrict__ ix, int64_t k, int64_t i, int base) {
  if constexpr (sizeof(IX) == 2) return i + (int64_t)__ldg(ix + k);
  else return (int64_t)__ldg(ix + k) - base;
}

// q = A p (one row per thread, j ascending) and the block partial of p.q.
// ACC = float: values converted to FP32 times p32, the FP32 copy of p that
// the p update writes, summed in FP32; ACC = double: values (FP64, FP32 or
// BF16) widened to FP64 and the products summed in FP64 -- with the FP64
// values, the FP64 SpMV.
template <class VT, class ACC, class PtrT, class IX>
__global__ void __launch_bounds__(CG_THREADS) cg_spmv_dot(
    int64_t n, const PtrT* __restrict__ ptr, const IX* __restrict__ idx, const VT* __restrict__ val,
    int base, const double* __restrict__ p, const float* __restrict__ p32, double* __restrict__ q,
    double* __restrict__ part) {
  cg_pdl_enter();
  __shared__ double sh[33];
  double dot = 0.0;
  auto term = [&](int64_t k, int64_t row, ACC acc) -> ACC {
    const int64_t j = cg_col(idx, k, row, base);
    if constexpr (sizeof(ACC) == 4)
      return __fmaf_rn(cg_val(val, k), __ldg(p32 + j), acc);
    else if constexpr (sizeof(VT) == 8)
      return __fma_rn((double)__ldg((const double*)val + k), __ldg(p + j), acc);
    else
      return __fma_rn((double)cg_val(val, k), __ldg(p + j), acc);
  };
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // two rows (i, i + stride) per thread in flight; rows and their products
  // in the plain loop's order, so q and the partial are bit-identical
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += 2 * stride) {
    const int64_t i2 = i + stride;
    const bool two = i2 < n;
    const int64_t a0 = ld_ptr(ptr, i) - base, a1 = ld_ptr(ptr, i + 1) - base;
    const int64_t b0 = two ? ld_ptr(ptr, i2) - base : 0, b1 = two ? ld_ptr(ptr, i2 + 1) - base : 0;
    ACC acc_a = ACC(0), acc_b = ACC(0);
    const int64_t la = a1 - a0, lb = b1 - b0;
    for (int64_t t = 0; t < (la > lb ? la : lb); ++t) {
      if (t < la) acc_a = term(a0 + t, i, acc_a);
      if (t < lb) acc_b = term(b0 + t, i2, acc_b);
    }
    const double qa = (double)acc_a;
    q[i] = qa;
    dot = __fma_rn(__ldg(p + i), qa, dot);
    if (two) {
      const double qb = (double)acc_b;
      q[i2] = qb;
      dot = __fma_rn(__ldg(p + i2), qb, dot);
    }
  }
  dot = cg_block_sum(dot, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = dot;
}

// One product a * p[j] added to a row's running pair sum (h, l): TwoSum on
// the high parts, the product's exact error (an FMA) and p's low part
// folded into l in FP32, so each entry costs 11 FP32 operations; (h, l) is
// normalised once per row.  l's own rounding keeps the sum within about
// 2^-48 of the sum of |terms| (Dekker's pair addition without the
// per-term renormalisation).
__device__ __forceinline__ void ff_row_term(float& h, float& l, float a, float2 pj) {
  const float ph = __fmul_rn(a, pj.x);
  const float pe = __fmaf_rn(a, pj.y, __fmaf_rn(a, pj.x, -ph));
  const float2 s = two_sum(h, ph);
  h = s.x;
  l = __fadd_rn(l, __fadd_rn(s.y, pe));
}

// The pair-sum SpMV: q = A p and the block partial of p.q, all in pairs;
// the partial leaves the block as one FP64 number.  IT: the row, entry and
// column arithmetic (int32 when rows and entries stay below 2^31, which
// halves the integer instructions per entry).
template <class VT, class PtrT, class IX, class IT, int R>
__global__ void __launch_bounds__(CG_THREADS) cgp_spmv_dot(
    int64_t n64, const PtrT* __restrict__ ptr, const IX* __restrict__ idx, const VT* __restrict__ val,
    int base, const float2* __restrict__ p, float2* __restrict__ q, double* __restrict__ part) {
  cg_pdl_enter();
  __shared__ float2 sh[32];
  float2 dot = make_float2(0.f, 0.f);
  const IT n = (IT)n64;
  const IT stride = (IT)gridDim.x * (IT)blockDim.x;
  auto col = [&](IT k, IT row) -> IT {
    if constexpr (sizeof(IX) == 2) return row + (IT)__ldg(idx + k);
    else return (IT)__ldg(idx + k) - (IT)base;
  };
  // R rows (i, i + stride, ...) per thread in flight; the rows, and each
  // row's products, in the plain loop's order, so q and the partial do not
  // depend on R
  for (IT i = (IT)blockIdx.x * (IT)blockDim.x + (IT)threadIdx.x; i < n; i += R * stride) {
    IT s0[R], len[R];
    IT lmax = 0;
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const IT row = i + (IT)u * stride;
      s0[u] = 0;
      len[u] = 0;
      if (row < n) {
        s0[u] = (IT)(ld_ptr(ptr, row) - base);
        len[u] = (IT)(ld_ptr(ptr, row + 1) - base) - s0[u];
      }
      lmax = len[u] > lmax ? len[u] : lmax;
    }
    float h[R], l[R];
#pragma unroll
    for (int u = 0; u < R; ++u) h[u] = l[u] = 0.f;
    for (IT t = 0; t < lmax; ++t) {
#pragma unroll
      for (int u = 0; u < R; ++u)
        if (t < len[u])
          ff_row_term(h[u], l[u], cg_val(val, s0[u] + t), __ldg(p + col(s0[u] + t, i + (IT)u * stride)));
    }
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const IT row = i + (IT)u * stride;
      if (row < n) {
        const float2 acc = two_sum(h[u], l[u]);  // l may exceed h after cancellation
        q[row] = acc;
        dot = ff_add(dot, ff_mul(__ldg(p + row), acc));
      }
    }
  }
  dot = ff_block_sum(dot, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = ff_to_double(dot);
}

// p (FP64) as a pair of FP32 numbers with integer operations only, so the
// SpMV below executes no FP64 instruction per entry: hi = p's top 24
// significand bits (a truncation), lo = the remaining 29 bits rounded to
// FP32, scaled by p's exponent.  |hi + lo - p| <= 2^-48 |p| for
// 2^-102 <= |p| < 2^128; below that lo, then hi, flush to zero (and
// beyond it hi is an infinity).
__device__ __forceinline__ float2 split_f64(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned int hw = (unsigned int)(b >> 32), lw = (unsigned int)b;
  const int e = (int)((hw >> 20) & 0x7FFu) - 1023;
  const unsigned int sign = hw & 0x80000000u;
  if (e < -126) return make_float2(0.f, 0.f);
  if (e > 127) return make_float2(__uint_as_float(sign | 0x7F800000u), 0.f);
  const float hi = __uint_as_float(sign | ((unsigned int)(e + 127) << 23) | ((hw & 0xFFFFFu) << 3) | (lw >> 29));
  float lo = __uint2float_rn(lw & 0x1FFFFFFFu);  // 29 bits, rounded to 24
  if (e >= -74) {
    lo = __fmul_rn(lo, __uint_as_float((unsigned int)(e + 75) << 23));  // 2^(e - 52)
  } else {  // 2^(e - 52) below FP32's normal range: two exact steps
    lo = __fmul_rn(__fmul_rn(lo, __uint_as_float((unsigned int)(e + 139) << 23)), 5.421010862427522e-20f);  // 2^-64
  }
  return make_float2(hi, sign ? -lo : lo);
}

// The SpMV of the pair-sum SpMV mode: FP64 p split into pairs as it is
// gathered, each row summed as a pair (ff_row_term), q and the p.q partial
// in FP64 -- the vectors, dots and updates stay FP64.
template <class VT, class PtrT, class IX, class IT, int R>
__global__ void __launch_bounds__(CG_THREADS) cgs_spmv_dot(
    int64_t n64, const PtrT* __restrict__ ptr, const IX* __restrict__ idx, const VT* __restrict__ val,
    int base, const double* __restrict__ p, double* __restrict__ q, double* __restrict__ part) {
  cg_pdl_enter();
  __shared__ double sh[33];
  double dot = 0.0;
  const IT n = (IT)n64;
  const IT stride = (IT)gridDim.x * (IT)blockDim.x;
  auto col = [&](IT k, IT row) -> IT {
    if constexpr (sizeof(IX) == 2) return row + (IT)__ldg(idx + k);
    else return (IT)__ldg(idx + k) - (IT)base;
  };
  for (IT i = (IT)blockIdx.x * (IT)blockDim.x + (IT)threadIdx.x; i < n; i += R * stride) {
    IT s0[R], len[R];
    IT lmax = 0;
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const IT row = i + (IT)u * stride;
      s0[u] = 0;
      len[u] = 0;
      if (row < n) {
        s0[u] = (IT)(ld_ptr(ptr, row) - base);
        len[u] = (IT)(ld_ptr(ptr, row + 1) - base) - s0[u];
      }
      lmax = len[u] > lmax ? len[u] : lmax;
    }
    float h[R], l[R];
#pragma unroll
    for (int u = 0; u < R; ++u) h[u] = l[u] = 0.f;
    for (IT t = 0; t < lmax; ++t) {
#pragma unroll
      for (int u = 0; u < R; ++u)
        if (t < len[u])
          ff_row_term(h[u], l[u], cg_val(val, s0[u] + t), split_f64(__ldg(p + col(s0[u] + t, i + (IT)u * stride))));
    }
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const IT row = i + (IT)u * stride;
      if (row < n) {
        const double qv = ff_to_double(two_sum(h[u], l[u]));
        q[row] = qv;
        dot = __fma_rn(__ldg(p + row), qv, dot);
      }
    }
  }
  dot = cg_block_sum(dot, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = dot;
}

// The compact index of a banded matrix: off[k] = j - i for the stored
// entries of row i, and *bad set when some |j - i| does not fit 16 bits.
template <class PtrT>
__global__ void cg_offsets(int64_t n, const PtrT* __restrict__ ptr, const int* __restrict__ idx, int base,
                           int16_t* __restrict__ off, int* __restrict__ bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    for (int64_t k = ld_ptr(ptr, i) - base; k < ld_ptr(ptr, i + 1) - base; ++k) {
      const int64_t d = (int64_t)idx[k] - base - i;
      if (d < -32768 || d > 32767) {
        *bad = 1;
        off[k] = 0;
      } else {
        off[k] = (int16_t)d;
      }
    }
  }
}

// alpha = rr[slot] / (p.q), formed once per block by thread 0 (a vanished
// curvature, p.q == 0, only happens once r is exactly zero).
__device__ __forceinline__ double cg_alpha(const double* __restrict__ part_pq, int nparts,
                                           const double* __restrict__ rr, int slot) {
  const double pq = warp_fold(part_pq, nparts);
  return pq != 0.0 ? rr[slot] / pq : 0.0;
}

// alpha;  r -= alpha q;  partials of r.r.  (x += alpha p waits for the p
// update, which reads p anyway: one pass over p less.)
__global__ void __launch_bounds__(CG_UPD_THREADS, 1) cg_update_r(
    int64_t n, double* __restrict__ r, const double* __restrict__ q, const double* __restrict__ part_pq,
    int nparts, const double* __restrict__ rr, int slot, double* __restrict__ part_rr) {
  cg_pdl_enter();
  __shared__ double sh[33];
  __shared__ double s_alpha;
  if (threadIdx.x < 32) {
    const double a = cg_alpha(part_pq, nparts, rr, slot);
    if (threadIdx.x == 0) s_alpha = a;
  }
  __syncthreads();
  const double alpha = s_alpha;
  double acc = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // CG_ILP elements per thread in flight: all loads first, then the updates
  // in the same element order as the plain loop (bit-identical partials)
  for (; i + (CG_ILP - 1) * stride < n; i += CG_ILP * stride) {
    double qv[CG_ILP], rv[CG_ILP];
#pragma unroll
    for (int u = 0; u < CG_ILP; ++u) {
      qv[u] = q[i + u * stride];
      rv[u] = r[i + u * stride];
    }
#pragma unroll
    for (int u = 0; u < CG_ILP; ++u) {
      const double ri = __fma_rn(-alpha, qv[u], rv[u]);
      r[i + u * stride] = ri;
      acc = __fma_rn(ri, ri, acc);
    }
  }
  for (; i < n; i += stride) {
    const double ri = __fma_rn(-alpha, q[i], r[i]);
    r[i] = ri;
    acc = __fma_rn(ri, ri, acc);
  }
  acc = cg_block_sum(acc, sh);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = acc;
}

// alpha as cg_update_r formed it (the same fold of the p.q partials);
// x += alpha p; rr' = fold(r.r partials); p = r + (rr' / rr[slot_in]) p;
// rr[slot_out] = rr'; p32 (when given) = p rounded to FP32, the FP32-sum
// SpMV's operand.  x's update is the one of the plain loop, bit for bit.
__global__ void __launch_bounds__(CG_UPD_THREADS, 1) cg_update_xp(
    int64_t n, double* __restrict__ x, const double* __restrict__ r, double* __restrict__ p,
    float* __restrict__ p32, const double* __restrict__ part_pq, int nparts_pq,
    const double* __restrict__ part_rr, int nparts, double* __restrict__ rr, int slot_in, int slot_out,
    double* __restrict__ hist, int64_t it) {
  cg_pdl_enter();
  __shared__ double s_ab[2];
  if (threadIdx.x < 32) {
    const double a = cg_alpha(part_pq, nparts_pq, rr, slot_in);
    const double rr_new = warp_fold(part_rr, nparts);
    if (threadIdx.x == 0) {
      s_ab[0] = a;
      s_ab[1] = rr[slot_in] != 0.0 ? rr_new / rr[slot_in] : 0.0;
      if (blockIdx.x == 0) {  // slot_out != slot_in: no block reads it here
        rr[slot_out] = rr_new;
        hist[it] = rr_new;
      }
    }
  }
  __syncthreads();
  const double alpha = s_ab[0], beta = s_ab[1];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; i + (CG_ILP - 1) * stride < n; i += CG_ILP * stride) {
    double pv[CG_ILP], rv[CG_ILP], xv[CG_ILP];
#pragma unroll
    for (int u = 0; u < CG_ILP; ++u) {
      pv[u] = p[i + u * stride];
      rv[u] = r[i + u * stride];
      xv[u] = x[i + u * stride];
    }
#pragma unroll
    for (int u = 0; u < CG_ILP; ++u) {
      x[i + u * stride] = __fma_rn(alpha, pv[u], xv[u]);
      const double pn = __fma_rn(beta, pv[u], rv[u]);
      p[i + u * stride] = pn;
      if (p32) p32[i + u * stride] = __double2float_rn(pn);
    }
  }
  for (; i < n; i += stride) {
    const double pi = p[i];
    x[i] = __fma_rn(alpha, pi, x[i]);
    const double pn = __fma_rn(beta, pi, r[i]);
    p[i] = pn;
    if (p32) p32[i] = __double2float_rn(pn);
  }
}

// The pair-sum r update: r -= alpha q in pairs, partials of r.r.
__global__ void __launch_bounds__(CG_UPD_THREADS, 1) cgp_update_r(
    int64_t n, float2* __restrict__ r, const float2* __restrict__ q, const double* __restrict__ part_pq,
    int nparts, const double* __restrict__ rr, int slot, double* __restrict__ part_rr) {
  cg_pdl_enter();
  __shared__ float2 sh[32];
  __shared__ float2 s_na;
  if (threadIdx.x < 32) {
    const double a = cg_alpha(part_pq, nparts, rr, slot);
    if (threadIdx.x == 0) s_na = ff_from_double(-a);
  }
  __syncthreads();
  const float2 na = s_na;
  float2 acc = make_float2(0.f, 0.f);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; i + (CG_ILP - 1) * stride < n; i += CG_ILP * stride) {
    float2 qv[CG_ILP], rv[CG_ILP];
#pragma unroll
    for (int u = 0; u < CG_ILP; ++u) {
      qv[u] = q[i + u * stride];
      rv[u] = r[i + u * stride];
    }
#pragma unroll
    for (int u = 0; u < CG_ILP; ++u) {
      const float2 ri = ff_add(rv[u], ff_mul(na, qv[u]));
      r[i + u * stride] = ri;
      acc = ff_add(acc, ff_mul(ri, ri));
    }
  }
  for (; i < n; i += stride) {
    const float2 ri = ff_add(r[i], ff_mul(na, q[i]));
    r[i] = ri;
    acc = ff_add(acc, ff_mul(ri, ri));
  }
  acc = ff_block_sum(acc, sh);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = ff_to_double(acc);
}

// The pair-sum x and p updates (alpha, beta formed in FP64 as above).
__global__ void __launch_bounds__(CG_UPD_THREADS, 1) cgp_update_xp(
    int64_t n, float2* __restrict__ x, const float2* __restrict__ r, float2* __restrict__ p,
    const double* __restrict__ part_pq, int nparts_pq, const double* __restrict__ part_rr, int nparts,
    double* __restrict__ rr, int slot_in, int slot_out, double* __restrict__ hist, int64_t it) {
  cg_pdl_enter();
  __shared__ float2 s_ab[2];
  if (threadIdx.x < 32) {
    const double a = cg_alpha(part_pq, nparts_pq, rr, slot_in);
    const double rr_new = warp_fold(part_rr, nparts);
    if (threadIdx.x == 0) {
      s_ab[0] = ff_from_double(a);
      s_ab[1] = ff_from_double(rr[slot_in] != 0.0 ? rr_new / rr[slot_in] : 0.0);
      if (blockIdx.x == 0) {
        rr[slot_out] = rr_new;
        hist[it] = rr_new;
      }
    }
  }
  __syncthreads();
  const float2 alpha = s_ab[0], beta = s_ab[1];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; i + (CG_ILP - 1) * stride < n; i += CG_ILP * stride) {
    float2 pv[CG_ILP], rv[CG_ILP], xv[CG_ILP];
#pragma unroll
    for (int u = 0; u < CG_ILP; ++u) {
      pv[u] = p[i + u * stride];
      rv[u] = r[i + u * stride];
      xv[u] = x[i + u * stride];
    }
#pragma unroll
    for (int u = 0; u < CG_ILP; ++u) {
      x[i + u * stride] = ff_add(xv[u], ff_mul(alpha, pv[u]));
      p[i + u * stride] = ff_add(rv[u], ff_mul(beta, pv[u]));
    }
  }
  for (; i < n; i += stride) {
    const float2 pi = p[i];
    x[i] = ff_add(x[i], ff_mul(alpha, pi));
    p[i] = ff_add(r[i], ff_mul(beta, pi));
  }
}

// r = b - A x (FP64) and partials of r.r (and of b.b when bb != NULL).
template <class PtrT>
__global__ void __launch_bounds__(CG_THREADS) cg_residual(
    int64_t n, const PtrT* __restrict__ ptr, const int* __restrict__ idx,
    const double* __restrict__ val, int base, const double* __restrict__ x,
    const double* __restrict__ b, double* __restrict__ r, double* __restrict__ part_rr,
    double* __restrict__ part_bb) {
  __shared__ double sh[33];
  double acc_r = 0.0, acc_b = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k0 = ld_ptr(ptr, i) - base, k1 = ld_ptr(ptr, i + 1) - base;
    double ax = 0.0;
    for (int64_t k = k0; k < k1; ++k) ax = __fma_rn(__ldg(val + k), __ldg(x + __ldg(idx + k) - base), ax);
    const double bi = b[i];
    const double ri = bi - ax;
    r[i] = ri;
    acc_r = __fma_rn(ri, ri, acc_r);
    acc_b = __fma_rn(bi, bi, acc_b);
  }
  acc_r = cg_block_sum(acc_r, sh);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = acc_r;
  if (part_bb) {
    __syncthreads();
    acc_b = cg_block_sum(acc_b, sh);
    if (threadIdx.x == 0) part_bb[blockIdx.x] = acc_b;
  }
}

// out[slot] = fold(part).
__global__ void cg_fold_set(const double* __restrict__ part, int nparts, double* __restrict__ out, int slot) {
  const double s = warp_fold(part, nparts);  // launched with one warp
  if (threadIdx.x == 0) out[slot] = s;
}

// p = r (a restart of the search direction), with p's FP32 copy when given.
__global__ void cg_copy(int64_t n, const double* __restrict__ src, double* __restrict__ dst,
                        float* __restrict__ dst32) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    dst[i] = src[i];
    if (dst32) dst32[i] = __double2float_rn(src[i]);
  }
}

// FP64 vector <-> pairs (the pair mode's entry to and exit from FP64).
__global__ void cgp_from_f64(int64_t n, const double* __restrict__ src, float2* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = ff_from_double(src[i]);
}
__global__ void cgp_to_f64(int64_t n, const float2* __restrict__ src, double* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = ff_to_double(src[i]);
}
__global__ void cgp_copy(int64_t n, const float2* __restrict__ src, float2* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

// A launch of an iteration kernel, chained to the previous one (pdl) or not.
template <class... KArgs, class... Args>
static void cg_launch(void (*kern)(KArgs...), int grid, int block, cudaStream_t s, bool pdl, Args... args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.stream = s;
  cfg.attrs = pdl ? at : nullptr;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kern, (KArgs)args...);  // errors surface at the capture's end
}

struct CgBuffers {
  double *r = nullptr, *p = nullptr, *q = nullptr, *part_a = nullptr, *part_b = nullptr,
         *part_c = nullptr, *rr = nullptr, *bb = nullptr, *hist = nullptr;
  float* p32 = nullptr;                      // FP32-sum mode: p rounded to FP32
  float2 *r2 = nullptr, *p2 = nullptr, *q2 = nullptr, *x2 = nullptr;  // pair mode
};

enum CgMode { CG_F32_SUMS = 0, CG_F64_SUMS = 1, CG_PAIR_SUMS = 2, CG_SPMV_PAIR = 3 };

// The SpMV's own grid: at most `grid` blocks and no more than fit the SMs at
// once (its two rows per thread take more registers than the updates).
template <class K>
static int occupancy_grid(K kernel, int grid, int sms) {
  int o = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kernel, CG_THREADS, 0);
  return std::max(1, std::min(grid, (o > 0 ? o : 1) * sms));
}

// The iteration SpMV of one mode, value type and index form.
template <class VT, class PtrT, class IX>
static int spmv_dot_t(const fgb_sparse* A, const IX* ix, int mode, int grid, int sms, const CgBuffers& b,
                      cudaStream_t s, bool launch, bool pdl) {
  const int64_t n = A->nrows;
  const PtrT* ptr = (const PtrT*)A->ptr;
  const VT* val = (const VT*)A->val;
  const int base = A->index_base;
  if constexpr (sizeof(VT) == 8) {  // the FP64 matrix: FP64 sums
    static const int g0 = occupancy_grid(cg_spmv_dot<VT, double, PtrT, IX>, 1 << 30, 1);
    const int g = std::max(1, std::min(grid, g0 * sms));
    if (launch)
      cg_launch(cg_spmv_dot<VT, double, PtrT, IX>, g, CG_THREADS, s, pdl, n, ptr, ix, val, base, (const double*)b.p,
                (const float*)nullptr, b.q, b.part_a);
    return g;
  } else {
    if (mode == CG_PAIR_SUMS) {
      // 32-bit index arithmetic while rows (two per thread, a grid-stride
      // apart) and entries stay below 2^31
      const bool i32 = n + (int64_t)CG_PAIR_ROWS * grid * CG_THREADS < INT32_MAX && A->nnz < INT32_MAX;
      if (i32) {
        static const int g0 = occupancy_grid(cgp_spmv_dot<VT, PtrT, IX, int32_t, CG_PAIR_ROWS>, 1 << 30, 1);
        const int g = std::max(1, std::min(grid, g0 * sms));
        if (launch)
          cg_launch(cgp_spmv_dot<VT, PtrT, IX, int32_t, CG_PAIR_ROWS>, g, CG_THREADS, s, pdl, n, ptr, ix, val, base,
                    (const float2*)b.p2, b.q2, b.part_a);
        return g;
      }
      static const int g0 = occupancy_grid(cgp_spmv_dot<VT, PtrT, IX, int64_t, 2>, 1 << 30, 1);
      const int g = std::max(1, std::min(grid, g0 * sms));
      if (launch)
        cg_launch(cgp_spmv_dot<VT, PtrT, IX, int64_t, 2>, g, CG_THREADS, s, pdl, n, ptr, ix, val, base,
                  (const float2*)b.p2, b.q2, b.part_a);
      return g;
    }
    if (mode == CG_SPMV_PAIR) {
      const bool i32 = n + (int64_t)CG_PAIR_ROWS * grid * CG_THREADS < INT32_MAX && A->nnz < INT32_MAX;
      if (i32) {
        static const int g0 = occupancy_grid(cgs_spmv_dot<VT, PtrT, IX, int32_t, CG_PAIR_ROWS>, 1 << 30, 1);
        const int g = std::max(1, std::min(grid, g0 * sms));
        if (launch)
          cg_launch(cgs_spmv_dot<VT, PtrT, IX, int32_t, CG_PAIR_ROWS>, g, CG_THREADS, s, pdl, n, ptr, ix, val, base,
                    (const double*)b.p, b.q, b.part_a);
        return g;
      }
      static const int g0 = occupancy_grid(cgs_spmv_dot<VT, PtrT, IX, int64_t, 2>, 1 << 30, 1);
      const int g = std::max(1, std::min(grid, g0 * sms));
      if (launch)
        cg_launch(cgs_spmv_dot<VT, PtrT, IX, int64_t, 2>, g, CG_THREADS, s, pdl, n, ptr, ix, val, base,
                  (const double*)b.p, b.q, b.part_a);
      return g;
    }
    if (mode == CG_F64_SUMS) {
      static const int g0 = occupancy_grid(cg_spmv_dot<VT, double, PtrT, IX>, 1 << 30, 1);
      const int g = std::max(1, std::min(grid, g0 * sms));
      if (launch)
        cg_launch(cg_spmv_dot<VT, double, PtrT, IX>, g, CG_THREADS, s, pdl, n, ptr, ix, val, base, (const double*)b.p,
                  (const float*)nullptr, b.q, b.part_a);
      return g;
    }
    static const int g0 = occupancy_grid(cg_spmv_dot<VT, float, PtrT, IX>, 1 << 30, 1);
    const int g = std::max(1, std::min(grid, g0 * sms));
    if (launch)
      cg_launch(cg_spmv_dot<VT, float, PtrT, IX>, g, CG_THREADS, s, pdl, n, ptr, ix, val, base, (const double*)b.p,
                (const float*)b.p32, b.q, b.part_a);
    return g;
  }
}

template <class PtrT, class IX>
static int spmv_dot_ix(const fgb_sparse* A, const IX* ix, int precision, int mode, int grid, int sms,
                       const CgBuffers& b, cudaStream_t s, bool launch, bool pdl) {
  if (precision == FGB_F64) return spmv_dot_t<double, PtrT, IX>(A, ix, mode, grid, sms, b, s, launch, pdl);
  if (precision == FGB_BF16) return spmv_dot_t<__nv_bfloat16, PtrT, IX>(A, ix, mode, grid, sms, b, s, launch, pdl);
  return spmv_dot_t<float, PtrT, IX>(A, ix, mode, grid, sms, b, s, launch, pdl);
}

// Launches (launch = true) or sizes (false) the iteration SpMV; returns its grid.
static int spmv_dot(const fgb_sparse* A, const int16_t* off, int precision, int mode, int grid, int sms,
                    const CgBuffers& b, cudaStream_t s, bool launch, bool pdl = false) {
  const bool i32 = A->ptr_t == FGB_I32;
  if (off)
    return i32 ? spmv_dot_ix<int32_t, int16_t>(A, off, precision, mode, grid, sms, b, s, launch, pdl)
               : spmv_dot_ix<int64_t, int16_t>(A, off, precision, mode, grid, sms, b, s, launch, pdl);
  const int* idx = (const int*)A->idx;
  return i32 ? spmv_dot_ix<int32_t, int>(A, idx, precision, mode, grid, sms, b, s, launch, pdl)
             : spmv_dot_ix<int64_t, int>(A, idx, precision, mode, grid, sms, b, s, launch, pdl);
}

template <class PtrT>
static void launch_residual(const fgb_sparse* A64, int grid, const double* x, const double* b,
                            double* r, double* part_rr, double* part_bb, cudaStream_t s) {
  cg_residual<PtrT><<<grid, CG_THREADS, 0, s>>>(A64->nrows, (const PtrT*)A64->ptr, (const int*)A64->idx,
                                                (const double*)A64->val, A64->index_base, x, b, r,
                                                part_rr, part_bb);
}

static int check_cg_matrix(const fgb_sparse* A, const char* who, int want_val) {
  int rc = check_sparse(A, who, true);
  if (rc) return rc;
  if (A->orient != FGB_CSR) return set_error(FGB_EUNSUPPORTED, "%s: CG needs a CSR matrix", who);
  if (A->nrows != A->ncols) return set_error(FGB_EINVAL, "%s: CG needs a square matrix", who);
  if (A->val_t != want_val) return set_error(FGB_EINVAL, "%s: value dtype %d, expected %d", who, A->val_t, want_val);
  return FGB_OK;
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_cg_solve(fgb_ctx* ctx, const fgb_sparse* A64, const fgb_sparse* Alow,
                            const double* b, double* x, const fgb_cg_options* opt,
                            fgb_cg_result* res, void* stream) {
  if (!ctx || !opt || !res || !b || !x) return set_error(FGB_EINVAL, "fgb_cg_solve: null argument");
  int rc = check_cg_matrix(A64, "fgb_cg_solve: A64", FGB_F64);
  if (rc) return rc;
  const int precision = opt->precision;
  if (precision != FGB_F64 && precision != FGB_F32 && precision != FGB_BF16)
    return set_error(FGB_EINVAL, "fgb_cg_solve: precision must be F64, F32 or BF16");
  if (opt->accumulate < FGB_CG_SUM_F32 || opt->accumulate > FGB_CG_SUM_SPMV_PAIR)
    return set_error(FGB_EINVAL, "fgb_cg_solve: accumulate must be FGB_CG_SUM_F32, _F64, _PAIR or _SPMV_PAIR");
  if (precision == FGB_F64 && (opt->accumulate == FGB_CG_SUM_PAIR || opt->accumulate == FGB_CG_SUM_SPMV_PAIR))
    return set_error(FGB_EINVAL, "fgb_cg_solve: pair sums take FP32 or BF16 values");
  const fgb_sparse* Ait = A64;
  if (precision != FGB_F64) {
    if (!Alow) return set_error(FGB_EINVAL, "fgb_cg_solve: low-precision matrix missing");
    rc = check_cg_matrix(Alow, "fgb_cg_solve: Alow", precision);
    if (rc) return rc;
    if (Alow->nrows != A64->nrows || Alow->nnz != A64->nnz)
      return set_error(FGB_EINVAL, "fgb_cg_solve: Alow and A64 differ in shape or pattern size");
    Ait = Alow;
  }
  if (opt->rtol <= 0.0 || opt->max_iter <= 0 || opt->chunk <= 0 || (opt->chunk & 1))
    return set_error(FGB_EINVAL, "fgb_cg_solve: need rtol > 0, max_iter > 0 and an even chunk > 0");
  const int64_t n = A64->nrows;
  const int chunk = opt->chunk;
  const int64_t replace_every = opt->replace_every > 0 ? opt->replace_every : 0;
  *res = fgb_cg_result{};
  if (n == 0) {
    res->converged = 1;
    return FGB_OK;
  }
  cudaStream_t user = pick_stream(ctx, stream);
  cudaStream_t s = nullptr;
  FGB_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaEvent_t ev = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  CgBuffers bufs;
  int16_t* off = nullptr;  // the compact index (16-bit column offsets), when it fits
  const int mode = precision == FGB_F64 ? CG_F64_SUMS : opt->accumulate;
  const bool pair = mode == CG_PAIR_SUMS;
  bool pair_live = false;  // x2 holds the iterate (x is refreshed from it)
  int64_t hist_cap = 0;
  const int grid = grid_for(n, CG_THREADS, ctx->num_sms, 8);  // full occupancy: streaming kernels
  const bool i32 = A64->ptr_t == FGB_I32;  // ptr width of the FP64 matrix
  auto t0 = std::chrono::steady_clock::now();
  auto fail = [&](int code, const char* what, cudaError_t e) {
    rc = set_error(code, "fgb_cg_solve: %s: %s", what, cudaGetErrorString(e));
  };
  do {
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ev, user);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev, 0);
    const size_t vec = sizeof(double) * n;
    hist_cap = opt->max_iter + chunk;
    // FP64 r, p, q (pair mode: r only, for the replacements), the pair
    // vectors or p's FP32 copy, then partials, scalars and the history
    const size_t f64_bytes = vec * (pair ? 1 : 3);
    const size_t extra = pair ? sizeof(float2) * n * 4 : (mode == CG_F32_SUMS ? sizeof(float) * n : 0);
    const size_t extra_off = (f64_bytes + 255) & ~size_t(255);
    const size_t tail_off = (extra_off + extra + 255) & ~size_t(255);
    char* base_ptr = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&base_ptr, tail_off + sizeof(double) * (3 * grid + 4 + hist_cap), s);
    if (e != cudaSuccess) { fail(FGB_ENOMEM, "setup", e); break; }
    bufs.r = (double*)base_ptr;
    if (!pair) {
      bufs.p = bufs.r + n;
      bufs.q = bufs.p + n;
    }
    if (pair) {
      bufs.r2 = (float2*)(base_ptr + extra_off);
      bufs.p2 = bufs.r2 + n;
      bufs.q2 = bufs.p2 + n;
      bufs.x2 = bufs.q2 + n;
    } else if (mode == CG_F32_SUMS) {
      bufs.p32 = (float*)(base_ptr + extra_off);
    }
    bufs.part_a = (double*)(base_ptr + tail_off);
    bufs.part_b = bufs.part_a + grid;
    bufs.part_c = bufs.part_b + grid;
    bufs.rr = bufs.part_c + grid;  // [0], [1]: r.r slots; [2]: b.b
    bufs.hist = bufs.rr + 4;
    // r = b - A x0, rr[0] = r.r, bb = b.b, p = r
    if (i32) launch_residual<int32_t>(A64, grid, x, b, bufs.r, bufs.part_a, bufs.part_b, s);
    else launch_residual<int64_t>(A64, grid, x, b, bufs.r, bufs.part_a, bufs.part_b, s);
    cg_fold_set<<<1, 32, 0, s>>>(bufs.part_a, grid, bufs.rr, 0);
    cg_fold_set<<<1, 32, 0, s>>>(bufs.part_b, grid, bufs.rr, 2);
    if (pair) {
      cgp_from_f64<<<grid, CG_THREADS, 0, s>>>(n, bufs.r, bufs.r2);
      cgp_from_f64<<<grid, CG_THREADS, 0, s>>>(n, x, bufs.x2);
      cgp_copy<<<grid, CG_THREADS, 0, s>>>(n, bufs.r2, bufs.p2);
    } else {
      cg_copy<<<grid, CG_THREADS, 0, s>>>(n, bufs.r, bufs.p, bufs.p32);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) { fail(FGB_ECUDA, "setup kernels", e); break; }
    double rr_bb[3];
    if ((e = cudaMemcpyAsync(rr_bb, bufs.rr, sizeof(rr_bb), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) { fail(FGB_ECUDA, "setup sync", e); break; }
    const double bnorm = sqrt(rr_bb[2]);
    const double target = opt->rtol * (bnorm > 0 ? bnorm : 1.0);
    if (sqrt(rr_bb[0]) <= target) {
      res->converged = 1;
      res->true_rel_residual = bnorm > 0 ? sqrt(rr_bb[0]) / bnorm : 0.0;
      break;
    }
    pair_live = pair;
    // The compact index: 16-bit column offsets j - i when the matrix is
    // banded that tightly (built once; the int32 index otherwise).
    if (n > 0 && Ait->nnz > 0) {
      int bad = 0;
      if ((e = cudaMallocAsync((void**)&off, sizeof(int16_t) * Ait->nnz + 256, s)) != cudaSuccess) { fail(FGB_ENOMEM, "offsets", e); break; }
      int* dbad = (int*)((char*)off + ((sizeof(int16_t) * Ait->nnz + 15) & ~size_t(15)));
      cudaMemsetAsync(dbad, 0, sizeof(int), s);
      if (Ait->ptr_t == FGB_I32)
        cg_offsets<int32_t><<<grid, CG_THREADS, 0, s>>>(n, (const int32_t*)Ait->ptr, (const int*)Ait->idx, Ait->index_base, off, dbad);
      else
        cg_offsets<int64_t><<<grid, CG_THREADS, 0, s>>>(n, (const int64_t*)Ait->ptr, (const int*)Ait->idx, Ait->index_base, off, dbad);
      if ((e = cudaMemcpyAsync(&bad, dbad, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
          (e = cudaStreamSynchronize(s)) != cudaSuccess) { fail(FGB_ECUDA, "offsets", e); break; }
      if (bad) {
        cudaFreeAsync(off, s);
        off = nullptr;
      }
    }
    res->compact_index = off ? 1 : 0;
    // one chunk of iterations, captured once (slots alternate; chunk is even)
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) { fail(FGB_ECUDA, "capture", e); break; }
    const int grid_upd = grid_for(n, CG_UPD_THREADS, ctx->num_sms, 1);  // <= grid partial slots
    const int grid_dot = spmv_dot(Ait, off, precision, mode, grid, ctx->num_sms, bufs, s, false);
    for (int t = 0; t < chunk; ++t) {
      const int si = t & 1, so = si ^ 1;
      // every launch after the chunk's first is chained to its predecessor
      spmv_dot(Ait, off, precision, mode, grid, ctx->num_sms, bufs, s, true, t > 0);
      if (pair) {
        cg_launch(cgp_update_r, grid_upd, CG_UPD_THREADS, s, true, n, bufs.r2, (const float2*)bufs.q2,
                  (const double*)bufs.part_a, grid_dot, (const double*)bufs.rr, si, bufs.part_b);
        cg_launch(cgp_update_xp, grid_upd, CG_UPD_THREADS, s, true, n, bufs.x2, (const float2*)bufs.r2, bufs.p2,
                  (const double*)bufs.part_a, grid_dot, (const double*)bufs.part_b, grid_upd, bufs.rr, si, so,
                  bufs.hist, (int64_t)t);
      } else {
        cg_launch(cg_update_r, grid_upd, CG_UPD_THREADS, s, true, n, bufs.r, (const double*)bufs.q,
                  (const double*)bufs.part_a, grid_dot, (const double*)bufs.rr, si, bufs.part_b);
        cg_launch(cg_update_xp, grid_upd, CG_UPD_THREADS, s, true, n, x, (const double*)bufs.r, bufs.p, bufs.p32,
                  (const double*)bufs.part_a, grid_dot, (const double*)bufs.part_b, grid_upd, bufs.rr, si, so,
                  bufs.hist, (int64_t)t);
      }
    }
    e = cudaStreamEndCapture(s, &graph);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) { fail(FGB_ECUDA, "graph", e); break; }
    std::vector<double> hist(chunk);
    int64_t it = 0, since_replace = 0;
    while (it < opt->max_iter) {
      if ((e = cudaGraphLaunch(exec, s)) != cudaSuccess) { fail(FGB_ECUDA, "graph launch", e); break; }
      if ((e = cudaMemcpyAsync(hist.data(), bufs.hist, sizeof(double) * chunk, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
          (e = cudaStreamSynchronize(s)) != cudaSuccess) { fail(FGB_ECUDA, "chunk sync", e); break; }
      it += chunk;
      since_replace += chunk;
      const bool small = sqrt(hist[chunk - 1]) <= target;
      const bool broken = !(hist[chunk - 1] == hist[chunk - 1]);  // NaN: breakdown
      if (broken) { rc = set_error(FGB_EINVAL, "fgb_cg_solve: breakdown (NaN residual) after %lld iterations", (long long)it); break; }
      if (small || (replace_every && since_replace >= replace_every)) {
        // reliable update: r = b - A x in FP64 and rr[0] = r.r (slot 0 starts
        // the next chunk); the search direction is kept.  If p has vanished
        // (the recursive residual reached zero), p.q = 0 gives alpha = 0 and
        // the next update rebuilds p from the replaced residual.
        if (pair) cgp_to_f64<<<grid, CG_THREADS, 0, s>>>(n, bufs.x2, x);
        if (i32) launch_residual<int32_t>(A64, grid, x, b, bufs.r, bufs.part_a, nullptr, s);
        else launch_residual<int64_t>(A64, grid, x, b, bufs.r, bufs.part_a, nullptr, s);
        cg_fold_set<<<1, 32, 0, s>>>(bufs.part_a, grid, bufs.rr, 0);
        if (pair) cgp_from_f64<<<grid, CG_THREADS, 0, s>>>(n, bufs.r, bufs.r2);
        double rr_true = 0;
        if ((e = cudaMemcpyAsync(&rr_true, bufs.rr, sizeof(double), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess) { fail(FGB_ECUDA, "replacement sync", e); break; }
        res->replacements++;
        since_replace = 0;
        // When the recursive residual has drifted below half the true one
        // (an iteration operator rounded to FP32 or BF16 leaves such a gap),
        // the kept direction no longer matches r: the next step would take
        // alpha = r.r / p.Ap, far above r.p / p.Ap, and the iteration would
        // diverge.  Restart the direction from the replaced r.
        if (hist[chunk - 1] < 0.25 * rr_true) {
          if (pair) cgp_copy<<<grid, CG_THREADS, 0, s>>>(n, bufs.r2, bufs.p2);
          else cg_copy<<<grid, CG_THREADS, 0, s>>>(n, bufs.r, bufs.p, bufs.p32);
          if ((e = cudaGetLastError()) != cudaSuccess) { fail(FGB_ECUDA, "restart", e); break; }
        }
        res->true_rel_residual = sqrt(rr_true) / (bnorm > 0 ? bnorm : 1.0);
        if (sqrt(rr_true) <= target) {
          res->converged = 1;
          break;
        }
      }
    }
    res->iterations = it;
  } while (0);
  if (pair_live && rc == FGB_OK) cgp_to_f64<<<grid, CG_THREADS, 0, s>>>(n, bufs.x2, x);  // the solution
  if (rc == FGB_OK && !res->converged && res->iterations >= opt->max_iter) {
    // report the true residual reached
    if (i32) launch_residual<int32_t>(A64, grid, x, b, bufs.r, bufs.part_a, nullptr, s);
    else launch_residual<int64_t>(A64, grid, x, b, bufs.r, bufs.part_a, nullptr, s);
    cg_fold_set<<<1, 32, 0, s>>>(bufs.part_a, grid, bufs.rr, 0);
    double rr_true = 0, bb = 0;
    cudaMemcpyAsync(&rr_true, bufs.rr, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&bb, bufs.rr + 2, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    res->true_rel_residual = sqrt(rr_true) / (bb > 0 ? sqrt(bb) : 1.0);
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (bufs.r) cudaFreeAsync(bufs.r, s);
  if (off) cudaFreeAsync(off, s);
  // the caller's stream waits for the solve
  if (ev) {
    cudaEventRecord(ev, s);
    cudaStreamWaitEvent(user, ev, 0);
  }
  cudaStreamSynchronize(s);
  if (ev) cudaEventDestroy(ev);
  cudaStreamDestroy(s);
  res->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}
