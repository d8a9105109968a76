// Semiring SpMV over SparseList fibers.
//
// CSR (pull): a group of G lanes owns one row i and folds
//   acc = (+)_{j ascending} A[i,j] (*) x[j]
// lane-strided over the row's stored entries, then combines the G partials
// with xor-shuffles.  G = 1 is Finch's serial order: one running value per
// output, updated j ascending, exactly the update
//   y[i] = x[j] * A[i,j] + y[i]
// of Finch's CSC nest (test/reference64/typical/typical_spmv_csc.txt:61-79),
// so FGB_FINCH_ORDER results equal Finch's bit for bit.
//
// CSC (push): a group of G lanes owns one column j, reads x[j] once and
// applies y[i] <<(+)>>= A[i,j] (*) x[j] for every stored i with an atomic
// update.  For exact semirings (integer +, min, max, |) the atomics commute,
// so results are exact; float sums are exact up to summation order.
//
// OR-AND works on Bool (0 or 1) bytes, where `true` absorbs under | and
// `false` annihilates under &: the push skips the columns whose x[j] is
// false and the pull stops a lane's scan at its first true product.  The
// result is the full nest's, bit for bit; a sparse frontier touches only its
// own columns' entries.
#include "fgb_internal.cuh"
#include "semiring.cuh"

namespace fgb {

template <int SR, class VT, class A, class PtrT, int G, bool PATTERN>
__global__ void __launch_bounds__(256) spmv_csr_pull(int64_t nrows, const PtrT* __restrict__ ptr,
                                                     const int* __restrict__ idx,
                                                     const VT* __restrict__ val,
                                                     const A* __restrict__ x, A* __restrict__ y,
                                                     int base, int accumulate, int fm) {
  using S = Semi<SR, A>;
  const int lane = threadIdx.x & (G - 1);
  const int64_t group = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
  for (int64_t row = group; row < nrows; row += ngroups) {
    const int64_t p0 = ld_ptr(ptr, row) - base;
    const int64_t p1 = ld_ptr(ptr, row + 1) - base;
    A acc = (G == 1 && accumulate) ? y[row] : S::identity();
#pragma unroll 4
    for (int64_t p = p0 + lane; p < p1; p += G) {
      const int j = __ldg(idx + p) - base;
      const A a = PATTERN ? S::one() : to_acc<A>(val[p]);
      acc = S::step(acc, a, __ldg(x + j), fm);
      if (SR == SR_OA && acc) break;  // Bool: true absorbs every later product
    }
    if (G > 1) {
#pragma unroll
      for (int m = G / 2; m >= 1; m >>= 1) acc = S::add(acc, shfl_xor(group_mask<G>(), acc, m, G));
      if (lane == 0) y[row] = accumulate ? S::add(y[row], acc) : acc;
    } else {
      y[row] = acc;
    }
  }
}

// CSR pull with lanes per row chosen row by row: a warp owns 32 consecutive
// rows; a row of at most SPMV_LONG entries is folded by its own lane (j
// ascending, one running value, as G = 1), and the warp's longer rows are
// then folded one after another by all 32 lanes (lane-strided, xor-shuffle
// combine, as G = 32).  Uniform short rows run at one lane per row, the long
// rows of a skewed matrix still spread over a warp, and the host needs no
// row-length statistics.  Not for OR-AND (its pull stops at the first true
// product).
constexpr int SPMV_LONG = 32;

template <int SR, class VT, class A, class PtrT, bool PATTERN>
__global__ void __launch_bounds__(256) spmv_csr_adaptive(int64_t nrows, const PtrT* __restrict__ ptr,
                                                         const int* __restrict__ idx,
                                                         const VT* __restrict__ val,
                                                         const A* __restrict__ x, A* __restrict__ y,
                                                         int base, int accumulate, int fm) {
  using S = Semi<SR, A>;
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r0 = warp * 32; r0 < nrows; r0 += nwarps * 32) {  // warp-uniform
    const int64_t row = r0 + lane;
    int64_t p0 = 0, p1 = 0;
    if (row < nrows) {
      p0 = ld_ptr(ptr, row) - base;
      p1 = ld_ptr(ptr, row + 1) - base;
    }
    const bool is_long = p1 - p0 > SPMV_LONG;
    if (row < nrows && !is_long) {
      A acc = accumulate ? y[row] : S::identity();
#pragma unroll 4
      for (int64_t p = p0; p < p1; ++p) {
        const int j = __ldg(idx + p) - base;
        const A a = PATTERN ? S::one() : to_acc<A>(val[p]);
        acc = S::step(acc, a, __ldg(x + j), fm);
      }
      y[row] = acc;
    }
    unsigned longs = __ballot_sync(FULL, is_long);
    while (longs) {
      const int l = __ffs(longs) - 1;
      longs &= longs - 1;
      const int64_t q0 = __shfl_sync(FULL, p0, l), q1 = __shfl_sync(FULL, p1, l);
      A acc = S::identity();
#pragma unroll 4
      for (int64_t p = q0 + lane; p < q1; p += 32) {
        const int j = __ldg(idx + p) - base;
        const A a = PATTERN ? S::one() : to_acc<A>(val[p]);
        acc = S::step(acc, a, __ldg(x + j), fm);
      }
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) acc = S::add(acc, shfl_xor(FULL, acc, m, 32));
      if (lane == 0) y[r0 + l] = accumulate ? S::add(y[r0 + l], acc) : acc;
    }
  }
}

template <int SR, class VT, class A, class PtrT, int G, bool PATTERN>
__global__ void __launch_bounds__(256) spmv_csc_push(int64_t ncols, const PtrT* __restrict__ ptr,
                                                     const int* __restrict__ idx,
                                                     const VT* __restrict__ val,
                                                     const A* __restrict__ x, A* __restrict__ y,
                                                     int base) {
  using S = Semi<SR, A>;
  const int lane = threadIdx.x & (G - 1);
  const int64_t group = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
  for (int64_t col = group; col < ncols; col += ngroups) {
    const A xj = __ldg(x + col);
    if (SR == SR_OA && !xj) continue;  // Bool: a & false adds nothing to any y[i]
    const int64_t p0 = ld_ptr(ptr, col) - base;
    const int64_t p1 = ld_ptr(ptr, col + 1) - base;
    if (p0 >= p1) continue;
    for (int64_t p = p0 + lane; p < p1; p += G) {
      const int i = __ldg(idx + p) - base;
      const A a = PATTERN ? S::one() : to_acc<A>(val[p]);
      AtomicAdd<SR, A>::apply(y + i, S::mul(a, xj));
    }
  }
}

// OR-AND push, warp-cooperative.  Each lane reads x for one column of a
// 32-column tile (four tiles in flight per lane); the warp takes an exclusive
// scan of the true columns' entry counts and spreads those entries over its
// 32 lanes, each finding its column by a binary search of the scan held in
// registers.  A false column costs one byte of x; the warp's lanes stay busy
// whatever the frontier's density.
template <class VT, class PtrT, bool PATTERN>
__global__ void __launch_bounds__(256) spmv_csc_push_oa(int64_t ncols, const PtrT* __restrict__ ptr,
                                                        const int* __restrict__ idx,
                                                        const VT* __restrict__ val,
                                                        const uint8_t* __restrict__ x,
                                                        uint8_t* __restrict__ y, int base) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int U = 4;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c0 = warp * 32 * U; c0 < ncols; c0 += nwarps * 32 * U) {
    uint8_t xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t col = c0 + 32 * u + lane;
      xv[u] = col < ncols ? __ldg(x + col) : uint8_t(0);
    }
#pragma unroll 1
    for (int u = 0; u < U; ++u) {
      const int64_t col = c0 + 32 * u + lane;
      if (!__any_sync(FULL, xv[u] != 0)) continue;
      int64_t p0 = 0, deg = 0;
      if (xv[u]) {
        p0 = ld_ptr(ptr, col) - base;
        deg = ld_ptr(ptr, col + 1) - base - p0;
      }
      int64_t incl = deg;  // inclusive scan of the entry counts over the warp
#pragma unroll
      for (int m = 1; m < 32; m <<= 1) {
        const int64_t t = __shfl_up_sync(FULL, incl, m);
        if (lane >= m) incl += t;
      }
      const int64_t excl = incl - deg;
      const int64_t total = __shfl_sync(FULL, incl, 31);
      for (int64_t k = 0; k < total; k += 32) {
        const int64_t e = k + lane;
        // owner: the largest lane whose scan start is <= e (it has entries)
        int l = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
          const int64_t s = __shfl_sync(FULL, excl, l + step);
          if (s <= e) l += step;
        }
        const int64_t pp = __shfl_sync(FULL, p0, l) + (e - __shfl_sync(FULL, excl, l));
        const uint8_t xj = __shfl_sync(FULL, xv[u], l);
        if (e < total) {
          const int i = __ldg(idx + pp) - base;
          const uint8_t a = PATTERN ? uint8_t(1) : val[pp];
          if (a & xj) *(volatile uint8_t*)(y + i) = 1;
        }
      }
    }
  }
}

template <int SR, class A>
__global__ void fill_identity(A* __restrict__ y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = Semi<SR, A>::identity();
}

// Lanes per fiber chosen by the plan autotuner for the calls it times and
// captures (0 = the heuristic below, 2 = the adaptive pull); set only around
// those calls.
static thread_local int t_group_override = 0;
constexpr int SPMV_ADAPTIVE = 2;

static int pick_group(double avg) {
  if (avg <= 2.0) return 1;
  if (avg <= 8.0) return 4;
  if (avg <= 24.0) return 8;
  return 32;
}

template <int SR, class VT, class A, class PtrT, bool PATTERN>
static int launch_typed(fgb_ctx* ctx, const fgb_sparse* A_, const void* x, void* y, unsigned flags,
                        cudaStream_t s) {
  const int base = A_->index_base;
  const int64_t nf = n_fibers(A_);
  const PtrT* ptr = (const PtrT*)A_->ptr;
  const int* idx = (const int*)A_->idx;
  const VT* val = (const VT*)A_->val;
  const double avg = nf ? (double)A_->nnz / (double)nf : 0.0;
  const int threads = 256;
  if (A_->orient == FGB_CSR) {
    const int accumulate = (flags & FGB_ACCUMULATE) ? 1 : 0;
    int fm = FM_DEFAULT;
    if (flags & FGB_NO_FMA) fm = FM_NOFMA;
    if (flags & FGB_FMA) fm = FM_FMA;
    int G = (flags & FGB_FINCH_ORDER) ? 1 : (t_group_override > 0 ? t_group_override : pick_group(avg));
    // Without a plan, a matrix with rows enough to fill the device at one
    // lane per row takes the adaptive pull: on millions of uniform rows of
    // 2 to 24 entries one lane per row beat 4 or 8 lanes by 30-50 %
    // (GB300, FP64), and its long rows still get a warp each.
    if (!(flags & FGB_FINCH_ORDER) && t_group_override <= 0 && SR != SR_OA &&
        nf >= (int64_t)ctx->num_sms * 2048)
      G = SPMV_ADAPTIVE;
    if (nf == 0) return FGB_OK;
    if constexpr (SR != SR_OA) {
      if (G == SPMV_ADAPTIVE) {
        const int grid = grid_for((nf + 31) / 32 * 32, threads, ctx->num_sms, 8);
        spmv_csr_adaptive<SR, VT, A, PtrT, PATTERN><<<grid, threads, 0, s>>>(nf, ptr, idx, val, (const A*)x,
                                                                             (A*)y, base, accumulate, fm);
        return check_launch("spmv_csr_adaptive");
      }
    }
    int grid = grid_for(nf * G, threads, ctx->num_sms, 8);
#define FGB_PULL(GG)                                                                    \
  spmv_csr_pull<SR, VT, A, PtrT, GG, PATTERN><<<grid, threads, 0, s>>>(                 \
      nf, ptr, idx, val, (const A*)x, (A*)y, base, accumulate, fm)
    switch (G) {
      case 1: FGB_PULL(1); break;
      case 4: FGB_PULL(4); break;
      case 8: FGB_PULL(8); break;
      default: FGB_PULL(32); break;
    }
#undef FGB_PULL
    return check_launch("spmv_csr_pull");
  }
  // CSC push
  const int64_t m = A_->nrows;
  if (!(flags & FGB_ACCUMULATE) && m > 0) {
    fill_identity<SR, A><<<grid_for(m, threads, ctx->num_sms, 4), threads, 0, s>>>((A*)y, m);
    int rc = check_launch("fill_identity");
    if (rc) return rc;
  }
  if (nf == 0) return FGB_OK;
  if constexpr (SR == SR_OA) {
    if (t_group_override <= 0) {  // the plan may still time the lane-group kernels
      const int grid = grid_for((nf + 127) / 128 * 32, threads, ctx->num_sms, 8);
      spmv_csc_push_oa<VT, PtrT, PATTERN><<<grid, threads, 0, s>>>(nf, ptr, idx, val, (const uint8_t*)x,
                                                                  (uint8_t*)y, base);
      return check_launch("spmv_csc_push_oa");
    }
  }
  int G = t_group_override > 0 ? (t_group_override <= 1 ? 1 : t_group_override <= 8 ? 8 : 32)
                               : (avg <= 4.0 ? 1 : (avg <= 16.0 ? 8 : 32));
  int grid = grid_for(nf * G, threads, ctx->num_sms, 8);
#define FGB_PUSH(GG)                                                                    \
  spmv_csc_push<SR, VT, A, PtrT, GG, PATTERN><<<grid, threads, 0, s>>>(nf, ptr, idx, val, \
                                                                      (const A*)x, (A*)y, base)
  switch (G) {
    case 1: FGB_PUSH(1); break;
    case 8: FGB_PUSH(8); break;
    default: FGB_PUSH(32); break;
  }
#undef FGB_PUSH
  return check_launch("spmv_csc_push");
}

template <int SR, class VT, class A, bool PATTERN = false>
static int launch_ptr(fgb_ctx* ctx, const fgb_sparse* A_, const void* x, void* y, unsigned flags,
                      cudaStream_t s) {
  if (A_->ptr_t == FGB_I32)
    return launch_typed<SR, VT, A, int32_t, PATTERN>(ctx, A_, x, y, flags, s);
  return launch_typed<SR, VT, A, int64_t, PATTERN>(ctx, A_, x, y, flags, s);
}

template <int SR>
static int dispatch_numeric(fgb_ctx* ctx, const fgb_sparse* A_, const void* x, int x_t, void* y,
                            int y_t, unsigned flags, cudaStream_t s) {
  const int v = A_->val_t;
  if (x_t != y_t) return set_error(FGB_EUNSUPPORTED, "fgb_spmv: x and y dtypes differ");
  switch (y_t) {
    case FGB_F64:
      if (v == FGB_F64) return launch_ptr<SR, double, double>(ctx, A_, x, y, flags, s);
      break;
    case FGB_F32:
      if (v == FGB_F32) return launch_ptr<SR, float, float>(ctx, A_, x, y, flags, s);
      if (v == FGB_BF16 && SR == SR_PT)
        return launch_ptr<SR_PT, __nv_bfloat16, float>(ctx, A_, x, y, flags, s);
      break;
    case FGB_I32:
      if (v == FGB_I32) return launch_ptr<SR, int32_t, int32_t>(ctx, A_, x, y, flags, s);
      break;
    case FGB_I64:
      if (v == FGB_I64) return launch_ptr<SR, int64_t, int64_t>(ctx, A_, x, y, flags, s);
      break;
    default: break;
  }
  return set_error(FGB_EUNSUPPORTED, "fgb_spmv: no kernel for semiring %d with val %d, x/y %d", SR,
                   v, y_t);
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_spmv(fgb_ctx* ctx, int semiring, const fgb_sparse* A, const void* x, int x_t,
                        void* y, int y_t, unsigned flags, void* stream) {
  if (!ctx) return set_error(FGB_EINVAL, "fgb_spmv: null ctx");
  int rc = check_sparse(A, "fgb_spmv: A", true);
  if (rc) return rc;
  const int64_t n_in = A->ncols, n_out = A->nrows;
  if ((n_in > 0 && !x) || (n_out > 0 && !y)) return set_error(FGB_EINVAL, "fgb_spmv: null x or y");
  if ((flags & FGB_FINCH_ORDER) && A->orient != FGB_CSR)
    return set_error(FGB_EUNSUPPORTED,
                     "fgb_spmv: FGB_FINCH_ORDER needs a CSR matrix (transpose once with "
                     "fgb_transpose)");
  cudaStream_t s = pick_stream(ctx, stream);
  switch (semiring) {
    case FGB_PLUS_TIMES: return dispatch_numeric<SR_PT>(ctx, A, x, x_t, y, y_t, flags, s);
    case FGB_MIN_PLUS: return dispatch_numeric<SR_MINP>(ctx, A, x, x_t, y, y_t, flags, s);
    case FGB_MAX_PLUS: return dispatch_numeric<SR_MAXP>(ctx, A, x, x_t, y, y_t, flags, s);
    case FGB_OR_AND:
      if (x_t != FGB_BOOL || y_t != FGB_BOOL)
        return set_error(FGB_EUNSUPPORTED, "fgb_spmv: OR_AND needs Bool x and y");
      if (A->val_t == FGB_NONE)
        return launch_ptr<SR_OA, uint8_t, uint8_t, true>(ctx, A, x, y, flags, s);
      if (A->val_t == FGB_BOOL)
        return launch_ptr<SR_OA, uint8_t, uint8_t, false>(ctx, A, x, y, flags, s);
      return set_error(FGB_EUNSUPPORTED, "fgb_spmv: OR_AND needs Bool or Pattern values");
    default: return set_error(FGB_EINVAL, "fgb_spmv: unknown semiring %d", semiring);
  }
}

namespace fgb {
// fgb_spmv with the lanes per fiber fixed to `group` (1, 4, 8 or 32).
int spmv_with_group(fgb_ctx* ctx, int semiring, const fgb_sparse* A, const void* x, int x_t,
                    void* y, int y_t, unsigned flags, int group, void* stream) {
  t_group_override = group;
  const int rc = fgb_spmv(ctx, semiring, A, x, x_t, y, y_t, flags, stream);
  t_group_override = 0;
  return rc;
}
}  // namespace fgb
