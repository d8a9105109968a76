/*
 * finch_oracle.c -- TEST INFRASTRUCTURE ONLY.  A CPU restatement, in plain
 * C, of the loop nests Finch.jl v1.2.12 generates for the sparse kernels the
 * GPU library replaces.  The tests, smoke() and the CPU-baseline leg of the
 * benchmark call it to check or time against; the library never does.
 *
 * All sparse inputs are Finch level buffers: 1-based Int64 ptr/idx of a
 * SparseList level (src/tensors/levels/sparse_list_levels.jl:37-53) and the
 * values of its Element child.  Arithmetic is Julia Base: integers wrap;
 * float min/max are the @fastmath forms (new operand wins only when strictly
 * smaller/larger); floats are evaluated either fused (`fma` = 1, what LLVM
 * may emit under @fastmath, src/execute.jl:116-120) or unfused (`fma` = 0).
 * The file is built with -ffp-contract=off, so "unfused" means unfused on
 * every host.
 *
 * Parity of this restatement is pinned against the numeric results printed
 * in Finch's own test fixtures (see tests/golden/make_golden.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { SR_PT = 0, SR_MINP = 1, SR_MAXP = 2, SR_OA = 3 };
enum { T_NONE = -1, T_F64 = 0, T_F32 = 1, T_BF16 = 2, T_I32 = 3, T_I64 = 4, T_BOOL = 5 };

static float bf16_to_f32(uint16_t b) {
  uint32_t u = (uint32_t)b << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

/* Finch.scansearch (src/util/shims.jl:22-44): first position q in [lo, hi]
 * with v[q] >= x, or hi + 1 if there is none.  Exponential steps to the
 * right bracket the answer, then bisection narrows it.  Positions are
 * 1-based; v is a 0-based C array. */
static int64_t scansearch(const int64_t* v, int64_t x, int64_t lo, int64_t hi) {
  int64_t step = 1, p = lo;
  while (p < hi && v[p - 1] < x) {
    step <<= 1;
    p += step;
  }
  int64_t below = p - step;                  /* known: v[below] < x or outside */
  int64_t above = (p < hi ? p : hi) + 1;     /* known: v[above] >= x or outside */
  while (below < above - 1) {
    const int64_t mid = below + ((above - below) >> 1);
    if (v[mid - 1] < x) below = mid; else above = mid;
  }
  return above;
}

/* ---------------------------------------------------------------- scalars */
/* One accumulation step acc <- acc (+) (a (*) x) per semiring and type,
 * written in the operand order of Finch's generated update
 * `y = x * A + y` (typical_spmv_csc.txt:66). */

static double step_f64(int sr, double acc, double a, double x, int fma_on) {
  switch (sr) {
    case SR_PT: return fma_on ? fma(x, a, acc) : (x * a) + acc;
    case SR_MINP: { double t = a + x; return (t < acc) ? t : acc; }
    case SR_MAXP: { double t = a + x; return (t > acc) ? t : acc; }
  }
  return acc;
}
static float step_f32(int sr, float acc, float a, float x, int fma_on) {
  switch (sr) {
    case SR_PT: return fma_on ? fmaf(x, a, acc) : (x * a) + acc;
    case SR_MINP: { float t = a + x; return (t < acc) ? t : acc; }
    case SR_MAXP: { float t = a + x; return (t > acc) ? t : acc; }
  }
  return acc;
}
static int32_t step_i32(int sr, int32_t acc, int32_t a, int32_t x) {
  switch (sr) {
    case SR_PT: return (int32_t)((uint32_t)acc + (uint32_t)x * (uint32_t)a);
    case SR_MINP: { int32_t t = (int32_t)((uint32_t)a + (uint32_t)x); return (t < acc) ? t : acc; }
    case SR_MAXP: { int32_t t = (int32_t)((uint32_t)a + (uint32_t)x); return (t > acc) ? t : acc; }
  }
  return acc;
}
static int64_t step_i64(int sr, int64_t acc, int64_t a, int64_t x) {
  switch (sr) {
    case SR_PT: return (int64_t)((uint64_t)acc + (uint64_t)x * (uint64_t)a);
    case SR_MINP: { int64_t t = (int64_t)((uint64_t)a + (uint64_t)x); return (t < acc) ? t : acc; }
    case SR_MAXP: { int64_t t = (int64_t)((uint64_t)a + (uint64_t)x); return (t > acc) ? t : acc; }
  }
  return acc;
}

/* Identity of (+), Finch's `y .= init` (src/symbolic/symbolic.jl:95-104). */
static void fill_identity(int sr, int at, void* y, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    switch (at) {
      case T_F64: ((double*)y)[i] = sr == SR_MINP ? INFINITY : sr == SR_MAXP ? -INFINITY : 0.0; break;
      case T_F32: ((float*)y)[i] = sr == SR_MINP ? INFINITY : sr == SR_MAXP ? -INFINITY : 0.0f; break;
      case T_I32: ((int32_t*)y)[i] = sr == SR_MINP ? INT32_MAX : sr == SR_MAXP ? INT32_MIN : 0; break;
      case T_I64: ((int64_t*)y)[i] = sr == SR_MINP ? INT64_MAX : sr == SR_MAXP ? INT64_MIN : 0; break;
      case T_BOOL: ((uint8_t*)y)[i] = 0; break;
    }
  }
}

/* y[i] <- y[i] (+) A(q) (*) x[j]  for stored entry q (0-based position). */
static void update(int sr, int vt, int at, void* y, int64_t i, const void* val, int64_t q,
                   const void* x, int64_t j, int fma_on) {
  switch (at) {
    case T_F64: {
      double a = ((const double*)val)[q];
      ((double*)y)[i] = step_f64(sr, ((double*)y)[i], a, ((const double*)x)[j], fma_on);
      break;
    }
    case T_F32: {
      float a = vt == T_BF16 ? bf16_to_f32(((const uint16_t*)val)[q]) : ((const float*)val)[q];
      ((float*)y)[i] = step_f32(sr, ((float*)y)[i], a, ((const float*)x)[j], fma_on);
      break;
    }
    case T_I32:
      ((int32_t*)y)[i] = step_i32(sr, ((int32_t*)y)[i], ((const int32_t*)val)[q], ((const int32_t*)x)[j]);
      break;
    case T_I64:
      ((int64_t*)y)[i] = step_i64(sr, ((int64_t*)y)[i], ((const int64_t*)val)[q], ((const int64_t*)x)[j]);
      break;
    case T_BOOL: {
      uint8_t a = vt == T_NONE ? 1 : ((const uint8_t*)val)[q];
      ((uint8_t*)y)[i] |= (uint8_t)(a & ((const uint8_t*)x)[j]);
      break;
    }
  }
}

/*
 * Serial CSC SpMV, Finch's nest for
 *     y .= init; for j = _, i = _; y[i] <<(+)>>= A[i, j] (*) x[j]; end
 * with A = Dense(SparseList(Element)) (m x n).  The loop follows the
 * generated code of test/reference64/typical/typical_spmv_csc.txt:45-80:
 * per column j read x[j] once, clip the fiber to [1, m] (phase_stop from the
 * last stored coordinate), seek with scansearch when the first coordinate is
 * below 1, then walk the fiber in order.  `init` = 0 keeps y's contents
 * (a nest without `y .= init`).
 */
int orc_spmv_csc(int sr, int vt, int at, int64_t m, int64_t n, const int64_t* ptr,
                 const int64_t* idx, const void* val, const void* x, void* y, int init,
                 int fma_on) {
  if (init) fill_identity(sr, at, y, m);
  for (int64_t j = 1; j <= n; ++j) {
    int64_t q = ptr[j - 1];
    const int64_t q_stop = ptr[j];
    const int64_t i1 = (q < q_stop) ? idx[q_stop - 2] : 0;
    const int64_t phase_stop = (m < i1) ? m : i1;
    if (phase_stop >= 1) {
      if (idx[q - 1] < 1) q = scansearch(idx, 1, q, q_stop - 1);
      for (;;) {
        const int64_t i = idx[q - 1];
        if (i < phase_stop) {
          update(sr, vt, at, y, i - 1, val, q - 1, x, j - 1, fma_on);
          q += 1;
        } else {
          if (i == phase_stop) {
            update(sr, vt, at, y, i - 1, val, q - 1, x, j - 1, fma_on);
            q += 1;
          }
          break;
        }
      }
    }
  }
  return 0;
}

/*
 * Row-pull SpMV over a CSR matrix (swizzle of a CSC of A^T): Finch's nest
 *     y .= init; for i = parallel(_), j = _; y[i] <<(+)>>= A[i, j] (*) x[j]
 * (test/reference64/parallel/parallel_spmv.txt:38-77).  Each row is one
 * running value, j ascending.  Rows are split across `nthreads` threads with
 * Finch's static schedule [fld(m*(t-1), N) + 1, fld(m*t, N)]
 * (src/architecture.jl:689-719).  With one thread this is the serial nest.
 */
int orc_spmv_csr(int sr, int vt, int at, int64_t m, int64_t n, const int64_t* ptr,
                 const int64_t* idx, const void* val, const void* x, void* y, int init,
                 int fma_on, int nthreads) {
  (void)n;
  if (init) fill_identity(sr, at, y, m);
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static, 1) num_threads(nthreads)
  for (int t = 1; t <= nthreads; ++t) {
    const int64_t lo = 1 + (m * (t - 1)) / nthreads;
    const int64_t hi = (m * t) / nthreads;
    for (int64_t i = lo; i <= hi; ++i)
      for (int64_t q = ptr[i - 1]; q < ptr[i]; ++q)
        update(sr, vt, at, y, i - 1, val, q - 1, x, idx[q - 1] - 1, fma_on);
  }
  return 0;
}

/*
 * SpMM  C[i, k] += A[i, j] * B[j, k]  over a CSR A (m x n) and a row-major
 * B (n x nk, leading dimension ldb), Finch's nest for
 * `@einsum C[i,k] += A[i,j]*B[j,k]` with loop order i, j, k: every C[i,k] is
 * one running sum over the row's j ascending.  C (ldc) is zeroed first when
 * `init`.  Threads split rows with the static schedule above.  dtype T_F32
 * (values F32 or BF16) or T_F64.
 */
int orc_spmm_csr(int vt, int at, int64_t m, int64_t n, int64_t nk, const int64_t* ptr,
                 const int64_t* idx, const void* val, const void* B, int64_t ldb, void* C,
                 int64_t ldc, int init, int fma_on, int nthreads) {
  (void)n;
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static, 1) num_threads(nthreads)
  for (int t = 1; t <= nthreads; ++t) {
    const int64_t lo = 1 + (m * (t - 1)) / nthreads;
    const int64_t hi = (m * t) / nthreads;
    for (int64_t i = lo; i <= hi; ++i) {
      if (at == T_F64) {
        double* c = (double*)C + (i - 1) * ldc;
        if (init) for (int64_t k = 0; k < nk; ++k) c[k] = 0.0;
        for (int64_t q = ptr[i - 1]; q < ptr[i]; ++q) {
          const double a = ((const double*)val)[q - 1];
          const double* b = (const double*)B + (idx[q - 1] - 1) * ldb;
          if (fma_on) for (int64_t k = 0; k < nk; ++k) c[k] = fma(b[k], a, c[k]);
          else for (int64_t k = 0; k < nk; ++k) c[k] = b[k] * a + c[k];
        }
      } else {
        float* c = (float*)C + (i - 1) * ldc;
        if (init) for (int64_t k = 0; k < nk; ++k) c[k] = 0.0f;
        for (int64_t q = ptr[i - 1]; q < ptr[i]; ++q) {
          const float a = vt == T_BF16 ? bf16_to_f32(((const uint16_t*)val)[q - 1])
                                       : ((const float*)val)[q - 1];
          const float* b = (const float*)B + (idx[q - 1] - 1) * ldb;
          if (fma_on) for (int64_t k = 0; k < nk; ++k) c[k] = fmaf(b[k], a, c[k]);
          else for (int64_t k = 0; k < nk; ++k) c[k] = b[k] * a + c[k];
        }
      }
    }
  }
  return 0;
}

/*
 * SDDMM  out[q] = A(q) * sum_k X[i,k] * Y[j,k]  for every stored (i, j) of a
 * CSR A, the fused form of compute(lazy(A) .* (lazy(X) * lazy(Y^T)))
 * (benchmark/benchmarks.jl:141-168): the dot is one running sum over k
 * ascending, then multiplied by the stored value.  `acc64` accumulates in
 * double whatever the dtype (the FP64 reference for error reports).
 */
int orc_sddmm_csr(int at, int64_t m, int64_t nk, const int64_t* ptr, const int64_t* idx,
                  const void* val, const void* X, int64_t ldx, const void* Y, int64_t ldy,
                  void* out, int fma_on, int acc64, int nthreads) {
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(static, 1) num_threads(nthreads)
  for (int t = 1; t <= nthreads; ++t) {
    const int64_t lo = 1 + (m * (t - 1)) / nthreads;
    const int64_t hi = (m * t) / nthreads;
    for (int64_t i = lo; i <= hi; ++i)
      for (int64_t q = ptr[i - 1]; q < ptr[i]; ++q) {
        const int64_t j = idx[q - 1];
        if (at == T_F64 || acc64) {
          double acc = 0.0;
          for (int64_t k = 0; k < nk; ++k) {
            double xv = at == T_F64 ? ((const double*)X)[(i - 1) * ldx + k] : ((const float*)X)[(i - 1) * ldx + k];
            double yv = at == T_F64 ? ((const double*)Y)[(j - 1) * ldy + k] : ((const float*)Y)[(j - 1) * ldy + k];
            acc = fma_on ? fma(xv, yv, acc) : xv * yv + acc;
          }
          if (at == T_F64) ((double*)out)[q - 1] = ((const double*)val)[q - 1] * acc;
          else ((double*)out)[q - 1] = (double)((const float*)val)[q - 1] * acc;
        } else {
          float acc = 0.0f;
          for (int64_t k = 0; k < nk; ++k) {
            float xv = ((const float*)X)[(i - 1) * ldx + k];
            float yv = ((const float*)Y)[(j - 1) * ldy + k];
            acc = fma_on ? fmaf(xv, yv, acc) : xv * yv + acc;
          }
          ((float*)out)[q - 1] = ((const float*)val)[q - 1] * acc;
        }
      }
  }
  return 0;
}

/*
 * Two-finger merge of two SparseList fibers, Finch's nest for
 * `z .= 0; for i = _; z[i] = x[i] (op) y[i]` with both operands SparseList
 * (test/reference64/typical/typical_merge_twofinger.txt:31-184): advance the
 * smaller coordinate; `*` stores only where both are stored (0 annihilates),
 * `+` stores the union.  Applied to every fiber of two same-shape matrices.
 * Pass `out_idx` = NULL to count only (out_ptr receives 1-based offsets).
 */
int orc_ewise(int op, int at, int64_t nf, const int64_t* pa, const int64_t* ia, const void* va,
              const int64_t* pb, const int64_t* ib, const void* vb, int64_t* out_ptr,
              int64_t* out_idx, void* out_val) {
  int64_t q = 1;
  out_ptr[0] = 1;
  for (int64_t f = 0; f < nf; ++f) {
    int64_t a = pa[f], ea = pa[f + 1], b = pb[f], eb = pb[f + 1];
    while (a < ea || b < eb) {
      const int64_t ca = a < ea ? ia[a - 1] : INT64_MAX;
      const int64_t cb = b < eb ? ib[b - 1] : INT64_MAX;
      int64_t c = ca < cb ? ca : cb;
      int emit = op == 0 ? (ca == cb) : 1;
      if (emit && out_idx) {
        out_idx[q - 1] = c;
#define EW_CASE(T)                                                                          \
  {                                                                                         \
    T x = ca == c ? ((const T*)va)[a - 1] : (T)0;                                           \
    T y = cb == c ? ((const T*)vb)[b - 1] : (T)0;                                           \
    if (op == 0) ((T*)out_val)[q - 1] = x * y;                                              \
    else if (ca == cb) ((T*)out_val)[q - 1] = x + y;                                        \
    else ((T*)out_val)[q - 1] = ca == c ? x : y;                                            \
  }
        switch (at) {
          case T_F64: EW_CASE(double) break;
          case T_F32: EW_CASE(float) break;
          case T_I32: {
            int32_t x = ca == c ? ((const int32_t*)va)[a - 1] : 0;
            int32_t y = cb == c ? ((const int32_t*)vb)[b - 1] : 0;
            ((int32_t*)out_val)[q - 1] = op == 0 ? (int32_t)((uint32_t)x * (uint32_t)y)
                                                 : (int32_t)((uint32_t)x + (uint32_t)y);
            break;
          }
          case T_I64: {
            int64_t x = ca == c ? ((const int64_t*)va)[a - 1] : 0;
            int64_t y = cb == c ? ((const int64_t*)vb)[b - 1] : 0;
            ((int64_t*)out_val)[q - 1] = op == 0 ? (int64_t)((uint64_t)x * (uint64_t)y)
                                                 : (int64_t)((uint64_t)x + (uint64_t)y);
            break;
          }
        }
#undef EW_CASE
      }
      if (emit) ++q;
      if (ca == c) ++a;
      if (cb == c) ++b;
    }
    out_ptr[f + 1] = q;
  }
  return 0;
}

/*
 * sum(A .* B; dims) for two same-shape CSR matrices (B sparse) or A CSR and
 * B dense row-major (Bd, ldb).  dims 2: per-row sums (length m); dims 1:
 * per-column sums (length n); dims 0: one scalar.  Sums are running sums in
 * storage order (rows ascending, j ascending), evaluated in `double`.
 */
int orc_ewise_reduce(int dims, int at, int64_t m, int64_t n, const int64_t* pa,
                     const int64_t* ia, const void* va, const int64_t* pb, const int64_t* ib,
                     const void* vb, const void* Bd, int64_t ldb, double* y) {
  const int64_t len = dims == 0 ? 1 : dims == 2 ? m : n;
  for (int64_t t = 0; t < len; ++t) y[t] = 0.0;
#define VAL(v, q) (at == T_F64 ? ((const double*)(v))[q] : (double)((const float*)(v))[q])
  for (int64_t i = 0; i < m; ++i) {
    if (pb) {
      int64_t a = pa[i], ea = pa[i + 1], b = pb[i], eb = pb[i + 1];
      while (a < ea && b < eb) {
        const int64_t ca = ia[a - 1], cb = ib[b - 1];
        if (ca == cb) {
          const double p = VAL(va, a - 1) * VAL(vb, b - 1);
          y[dims == 0 ? 0 : dims == 2 ? i : ca - 1] += p;
        }
        if (ca <= cb) ++a;
        if (cb <= ca) ++b;
      }
    } else {
      for (int64_t a = pa[i]; a < pa[i + 1]; ++a) {
        const int64_t c = ia[a - 1];
        const double p = VAL(va, a - 1) * VAL(Bd, i * ldb + (c - 1));
        y[dims == 0 ? 0 : dims == 2 ? i : c - 1] += p;
      }
    }
  }
#undef VAL
  return 0;
}

/*
 * fsparse(I, J, V, (m, n), combine) followed by the copy into
 * Dense(SparseList(Element)) (csc = 1) or its row-major swizzle (csc = 0):
 * the documented contract of src/interface/fsparse.jl:13-100 -- coordinates
 * sorted with the last index most significant (column, then row), duplicates
 * folded left to right in input order (`foldl(combine, V[run])`).  The sort
 * is a stable merge sort on (fiber, coordinate, input position).  1-based
 * coordinates in, 1-based ptr/idx out.  combine: 0 +, 1 |, 2 min, 3 max,
 * 4 last (Julia Base semantics: wrapping integers, NaN-propagating float
 * min/max with -0.0 < +0.0).  Returns the stored count, or -1 if a
 * coordinate is out of range.
 */
static const int64_t* g_coo_key;
static void coo_merge(int64_t* a, int64_t* tmp, int64_t n) {
  if (n < 2) return;
  const int64_t h = n / 2;
  coo_merge(a, tmp, h);
  coo_merge(a + h, tmp, n - h);
  int64_t i = 0, j = h, k = 0;
  while (i < h && j < n) tmp[k++] = g_coo_key[a[j]] < g_coo_key[a[i]] ? a[j++] : a[i++];
  while (i < h) tmp[k++] = a[i++];
  while (j < n) tmp[k++] = a[j++];
  memcpy(a, tmp, (size_t)n * sizeof(int64_t));
}

static double coo_fold_double(int combine, double a, double b) {
  switch (combine) {
    case 0: return a + b;
    case 2:
      if (a != a) return a;
      if (b != b) return b;
      return (b < a || (b == a && signbit(b) && !signbit(a))) ? b : a;
    case 3:
      if (a != a) return a;
      if (b != b) return b;
      return (b > a || (b == a && !signbit(b) && signbit(a))) ? b : a;
    default: return b;
  }
}
static float coo_fold_float(int combine, float a, float b) {
  switch (combine) {
    case 0: return a + b;
    case 2:
      if (a != a) return a;
      if (b != b) return b;
      return (b < a || (b == a && signbit(b) && !signbit(a))) ? b : a;
    case 3:
      if (a != a) return a;
      if (b != b) return b;
      return (b > a || (b == a && !signbit(b) && signbit(a))) ? b : a;
    default: return b;
  }
}
static int32_t coo_fold_int32_t(int combine, int32_t a, int32_t b) {
  switch (combine) {
    case 0: return (int32_t)((uint32_t)a + (uint32_t)b);
    case 1: return a | b;
    case 2: return b < a ? b : a;
    case 3: return b > a ? b : a;
    default: return b;
  }
}
static int64_t coo_fold_int64_t(int combine, int64_t a, int64_t b) {
  switch (combine) {
    case 0: return (int64_t)((uint64_t)a + (uint64_t)b);
    case 1: return a | b;
    case 2: return b < a ? b : a;
    case 3: return b > a ? b : a;
    default: return b;
  }
}
static uint8_t coo_fold_uint8_t(int combine, uint8_t a, uint8_t b) {
  switch (combine) {
    case 0:
    case 1: return (uint8_t)(a | b);
    case 2: return b < a ? b : a;
    case 3: return b > a ? b : a;
    default: return b;
  }
}
int64_t orc_coo_assemble(int csc, int vt, int combine, int64_t m, int64_t n, int64_t nin,
                         const int64_t* I, const int64_t* J, const void* V, int64_t* out_ptr,
                         int64_t* out_idx, void* out_val) {
  const int64_t nfib = csc ? n : m, inner = csc ? m : n;
  int64_t* key = (int64_t*)malloc((size_t)(nin > 0 ? nin : 1) * sizeof(int64_t));
  int64_t* ord = (int64_t*)malloc((size_t)(nin > 0 ? nin : 1) * sizeof(int64_t));
  int64_t* tmp = (int64_t*)malloc((size_t)(nin > 0 ? nin : 1) * sizeof(int64_t));
  for (int64_t k = 0; k < nin; ++k) {
    const int64_t i = I[k] - 1, j = J[k] - 1;
    if (i < 0 || i >= m || j < 0 || j >= n) {
      free(key);
      free(ord);
      free(tmp);
      return -1;
    }
    key[k] = csc ? j * m + i : i * n + j;
    ord[k] = k;
  }
  g_coo_key = key;
  coo_merge(ord, tmp, nin);
  int64_t q = 0, f = 0;
  out_ptr[0] = 1;
  for (int64_t k = 0; k < nin;) {
    int64_t r = k + 1;
    while (r < nin && key[ord[r]] == key[ord[k]]) ++r;
    const int64_t fib = key[ord[k]] / inner;
    while (f < fib) out_ptr[++f] = q + 1;
    out_idx[q] = key[ord[k]] % inner + 1;
#define FOLD(T)                                                      \
  {                                                                  \
    T v = ((const T*)V)[ord[k]];                                     \
    for (int64_t t = k + 1; t < r; ++t) v = coo_fold_##T(combine, v, ((const T*)V)[ord[t]]); \
    ((T*)out_val)[q] = v;                                            \
  }
    switch (vt) {
      case T_F64: FOLD(double) break;
      case T_F32: FOLD(float) break;
      case T_I32: FOLD(int32_t) break;
      case T_I64: FOLD(int64_t) break;
      case T_BOOL: FOLD(uint8_t) break;
      default: break; /* Pattern: no values */
    }
#undef FOLD
    ++q;
    k = r;
  }
  while (f < nfib) out_ptr[++f] = q + 1;
  free(key);
  free(ord);
  free(tmp);
  return q;
}

/*
 * Gustavson's SpGEMM, the nest of docs/examples/spgemm.jl:56-72 in its row
 * form on CSR buffers: for every row r, w .= 0; for k in L[r,:] (stored
 * order), for c in R[k,:]: w[c] += L[r,k] * R[k,c]; then the touched
 * coordinates of w, ascending, are the row of C (stored even when they sum
 * to zero).  Finch's column form on CSC operands is this nest on the
 * transposed problem.  F64 (vt 0) or F32 (vt 1) values, fused (`fma`) or
 * not.  Pass out_idx = NULL to count only.  Returns nnz(C).
 */
int64_t orc_spgemm_csr(int vt, int fma, int64_t m, int64_t n, const int64_t* lp, const int64_t* li,
                       const void* lv, const int64_t* rp, const int64_t* ri, const void* rv,
                       int64_t* out_ptr, int64_t* out_idx, void* out_val) {
  double* wd = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
  float* wf = (float*)calloc((size_t)(n > 0 ? n : 1), sizeof(float));
  unsigned char* seen = (unsigned char*)calloc((size_t)(n > 0 ? n : 1), 1);
  int64_t* list = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  int64_t q = 0;
  out_ptr[0] = 1;
  for (int64_t r = 0; r < m; ++r) {
    int64_t cnt = 0;
    for (int64_t a = lp[r]; a < lp[r + 1]; ++a) {
      const int64_t k = li[a - 1] - 1;
      for (int64_t b = rp[k]; b < rp[k + 1]; ++b) {
        const int64_t c = ri[b - 1] - 1;
        if (!seen[c]) {
          seen[c] = 1;
          list[cnt++] = c;
          wd[c] = 0.0;
          wf[c] = 0.0f;
        }
        if (out_idx) {
          if (vt == T_F64) {
            const double x = ((const double*)lv)[a - 1], y = ((const double*)rv)[b - 1];
            wd[c] = fma ? __builtin_fma(y, x, wd[c]) : wd[c] + y * x;
          } else {
            const float x = ((const float*)lv)[a - 1], y = ((const float*)rv)[b - 1];
            wf[c] = fma ? __builtin_fmaf(y, x, wf[c]) : wf[c] + y * x;
          }
        }
      }
    }
    /* ascending coordinates: counting over the touched list */
    for (int64_t t = 1; t < cnt; ++t) {
      const int64_t v = list[t];
      int64_t u = t - 1;
      while (u >= 0 && list[u] > v) {
        list[u + 1] = list[u];
        --u;
      }
      list[u + 1] = v;
    }
    for (int64_t t = 0; t < cnt; ++t) {
      const int64_t c = list[t];
      if (out_idx) {
        out_idx[q] = c + 1;
        if (vt == T_F64) ((double*)out_val)[q] = wd[c];
        else ((float*)out_val)[q] = wf[c];
      }
      seen[c] = 0;
      ++q;
    }
    out_ptr[r + 1] = q + 1;
  }
  free(wd);
  free(wf);
  free(seen);
  free(list);
  return q;
}

/* Threads available to the OpenMP runtime (1 without OpenMP). */
/* One BFS round of docs/examples/bfs.jl:25-34, as written: j outer over
 * the columns of `edges` (CSC: column j lists the k with edges[k, j]), k
 * inner, and for F[j] && edges[k, j] && !V[k]: nF[k] |= true;
 * P[k] <<choose(fill)>>= j, with choose(z)(a, b) = isequal(a, z) ? b : a
 * (src/util/special_functions.jl:13-34); j is written 1-based.  Then the
 * second loop (bfs.jl:35-42): V[k] |= nF[k]; c += nF[k].  Returns c. */
int64_t orc_bfs_round(int64_t n, const int64_t* ptr, const int64_t* idx, const uint8_t* F, uint8_t* V,
                      int64_t* P, int64_t fill, uint8_t* nF) {
  memset(nF, 0, (size_t)n);
  for (int64_t j = 0; j < n; ++j) {
    if (!F[j]) continue;
    for (int64_t q = ptr[j] - 1; q < ptr[j + 1] - 1; ++q) {
      const int64_t k = idx[q] - 1;
      if (V[k]) continue;
      nF[k] = 1;
      if (P[k] == fill) P[k] = j + 1;
    }
  }
  int64_t c = 0;
  for (int64_t k = 0; k < n; ++k) {
    V[k] |= nF[k];
    c += nF[k];
  }
  return c;
}

/* minby(a, b) = a[1] > b[1] ? b : a (src/util/special_functions.jl:75-88). */
#define MINBY(dd, pp, d, p) \
  do {                      \
    if ((dd) > (d)) {       \
      (dd) = (d);           \
      (pp) = (p);           \
    }                       \
  } while (0)

/* One relaxation round of docs/examples/shortest_paths.jl:22-42 over
 * Float64 distances, as written.  The first loop: for j with active_prev[j],
 * dists[j] <<minby>>= dists_prev[j].  The second: active .= false; for j
 * with active_prev[j], for the stored i of column j of `edges` (CSC; the
 * fill Inf leaves everything unchanged), d = first(dists_prev[j]) +
 * edges[i, j]; dists[i] <<minby>>= (d, j); active[i] |= d <
 * first(dists_prev[i]).  Pairs are (dist, parent) arrays; j is 1-based. */
void orc_minby_round(int64_t n, const int64_t* ptr, const int64_t* idx, const double* w, const double* dprev,
                     const int64_t* pprev, const uint8_t* aprev, double* dist, int64_t* par, uint8_t* active) {
  for (int64_t j = 0; j < n; ++j)
    if (aprev[j]) MINBY(dist[j], par[j], dprev[j], pprev[j]);
  memset(active, 0, (size_t)n);
  for (int64_t j = 0; j < n; ++j) {
    if (!aprev[j]) continue;
    for (int64_t q = ptr[j] - 1; q < ptr[j + 1] - 1; ++q) {
      const int64_t i = idx[q] - 1;
      const double d = dprev[j] + w[q];
      MINBY(dist[i], par[i], d, j + 1);
      active[i] |= (uint8_t)(d < dprev[i]);
    }
  }
}

/* PageRank, docs/examples/pagerank.jl:7-51, as written, over the CSC of
 * `edges` (column j lists the i with edges[i, j]; w NULL for a Pattern,
 * whose stored entries are true = 1).  out_degree[j] += edges[i, j] visits
 * the stored entries (the fill 0 is the identity of +).  The transition
 * matrix is the loop over every (i, j), the fill region included, as `/`
 * has no annihilator (src/symbolic/symbolic.jl:145-153): where
 * out_degree[i] != 0 it stores edges[i, j] / out_degree[j], which is
 * 0 / out_degree[j] where edges stores nothing (NaN for a zero
 * out-degree).  r[j] = 1.0 / n.  Each step: rank .= 0; for j, then the
 * stored i ascending, rank[i] += scaled[i, j] * r[j]; then r[i] = beta +
 * damp * rank[i], beta = (1 - damp) / n; both fused when fma != 0.  Needs
 * n * n doubles of scratch: returns -1 when they cannot be allocated. */
int orc_pagerank(int64_t n, const int64_t* ptr, const int64_t* idx, const double* w, int64_t nsteps, double damp,
                 int fma_on, double* r) {
  double* deg = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
  double* col = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
  double* rank = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
  double* S = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n * n : 1));
  uint8_t* st = (uint8_t*)malloc((size_t)(n > 0 ? n * n : 1));
  if (!deg || !col || !rank || !S || !st) {
    free(deg); free(col); free(rank); free(S); free(st);
    return -1;
  }
  for (int64_t j = 0; j < n; ++j)
    for (int64_t q = ptr[j] - 1; q < ptr[j + 1] - 1; ++q) deg[j] += w ? w[q] : 1.0;
  for (int64_t j = 0; j < n; ++j) {
    for (int64_t i = 0; i < n; ++i) col[i] = 0.0;
    for (int64_t q = ptr[j] - 1; q < ptr[j + 1] - 1; ++q) col[idx[q] - 1] = w ? w[q] : 1.0;
    for (int64_t i = 0; i < n; ++i) {
      st[i + j * n] = deg[i] != 0.0;
      S[i + j * n] = st[i + j * n] ? col[i] / deg[j] : 0.0;
    }
  }
  for (int64_t j = 0; j < n; ++j) r[j] = 1.0 / (double)n;
  const double beta = (1.0 - damp) / (double)n;
  for (int64_t step = 0; step < nsteps; ++step) {
    for (int64_t i = 0; i < n; ++i) rank[i] = 0.0;
    for (int64_t j = 0; j < n; ++j)
      for (int64_t i = 0; i < n; ++i)
        if (st[i + j * n]) rank[i] = fma_on ? fma(S[i + j * n], r[j], rank[i]) : rank[i] + S[i + j * n] * r[j];
    for (int64_t i = 0; i < n; ++i) r[i] = fma_on ? fma(damp, rank[i], beta) : beta + damp * rank[i];
  }
  free(deg); free(col); free(rank); free(S); free(st);
  return 0;
}

/* reduce(max | min, A; dims) as Finch's loop runs it (src/interface/eager.jl:
 * 153-158 lowered like the sum of test/reference64/interface/
 * reduce_default.txt): over the CSC of A, j outer and i inner, every
 * (i, j) folds -- the stored value, or the fill -- with @fastmath's
 * first-operand max/min (the second operand wins only when strictly larger
 * / smaller), from init.  dims 1: y[j] over i; dims 2: y[i] over j; dims 0:
 * y[0] over everything in that order.  Values as doubles. */
void orc_reduce_minmax(int is_max, int dims, int64_t m, int64_t n, const int64_t* ptr, const int64_t* idx,
                       const double* val, double fill, double init, double* y) {
  double* col = (double*)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
  const int64_t ny = dims == 1 ? n : (dims == 2 ? m : 1);
  for (int64_t k = 0; k < ny; ++k) y[k] = init;
  for (int64_t j = 0; j < n; ++j) {
    for (int64_t i = 0; i < m; ++i) col[i] = fill;
    for (int64_t q = ptr[j] - 1; q < ptr[j + 1] - 1; ++q) col[idx[q] - 1] = val[q];
    for (int64_t i = 0; i < m; ++i) {
      double* acc = dims == 1 ? &y[j] : (dims == 2 ? &y[i] : &y[0]);
      const double v = col[i];
      if (is_max ? (v > *acc) : (v < *acc)) *acc = v;
    }
  }
  free(col);
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
