/*
 * finchgb.h -- C ABI of the GB300 (sm_103a) execution backend for the sparse
 * loop nests Finch.jl lowers to SpMV, SpMM, SDDMM, semiring SpMV and fused
 * elementwise+reduce.
 *
 * Every entry point is plain C: opaque handles, raw pointers and sizes, an int
 * status return.  Nothing aborts; the message for the last failure on the
 * calling thread is returned by fgb_last_error().
 *
 * Level buffers follow Finch's SparseList layout
 * (src/tensors/levels/sparse_list_levels.jl:37-53): for each parent position p
 * the stored coordinates are idx[ptr[p]-base .. ptr[p+1]-base) and the values
 * sit at the same positions of the child Element level
 * (src/tensors/levels/element_levels.jl:20-34).  Finch's own buffers are
 * 1-based Int64 (index_base = 1, ptr[1] == 1); 0-based PlusOneVector buffers
 * (src/util/vectors.jl:3-37) are index_base = 0.  Compute kernels read 32-bit
 * idx; fgb_narrow_index() converts Finch's Int64 idx once, at upload.
 *
 * Orientation: FGB_CSC is Finch's Dense(SparseList(Element)) of an m x n
 * matrix A[i,j] (outer level j, ptr has n+1 entries, idx holds rows i).
 * FGB_CSR is swizzle(Tensor(CSC of A^T), 2, 1)
 * (src/tensors/combinators/swizzle.jl:55-58): ptr has m+1 entries and idx
 * holds columns j.
 *
 * Dense operands are row-major with a leading dimension (the last index is
 * fastest), which is how Finch stores swizzle(Tensor(Dense(Dense(Element))) of
 * B^T, 2, 1).
 *
 * Pointers passed to compute entry points are DEVICE pointers (from
 * fgb_malloc, cudaMalloc or another allocator on the same device).  All work
 * is issued on `stream` (a cudaStream_t; NULL = CUDA's default stream) and
 * is asynchronous unless stated otherwise.
 */
#ifndef FINCHGB_H
#define FINCHGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define FGB_API __attribute__((visibility("default")))
#else
#define FGB_API
#endif

#define FGB_VERSION_MAJOR 0
#define FGB_VERSION_MINOR 1

/* Status codes.  The Finch side maps EINVAL to DimensionMismatch /
 * FinchProtocolError, like the checks in Finch's generated code
 * (test/reference64/typical/typical_spmv_csc.txt:42). */
typedef enum {
  FGB_OK = 0,
  FGB_EINVAL = 1,       /* bad shape, format, dtype or argument */
  FGB_ENOMEM = 2,       /* allocation failed or admission refused */
  FGB_ETIMEOUT = 3,     /* a bounded wait ran out */
  FGB_ECUDA = 4,        /* a CUDA runtime call failed */
  FGB_EUNSUPPORTED = 5, /* no kernel for this (semiring, dtype, format) */
  FGB_EBUSY = 6,        /* resource in use / queue full */
  FGB_ECANCELLED = 7    /* request cancelled before it ran */
} fgb_status;

typedef enum {
  FGB_NONE = -1, /* no values: Pattern level (every stored entry is true) */
  FGB_F64 = 0,
  FGB_F32 = 1,
  FGB_BF16 = 2,
  FGB_I32 = 3,
  FGB_I64 = 4,
  FGB_BOOL = 5 /* one byte, 0 or 1 */
} fgb_dtype;

/* Semirings of y[i] <<add>>= mul(A[i,j], x[j]).  Identities follow Finch's
 * algebra traits (src/symbolic/symbolic.jl:95-104); arithmetic follows Julia
 * Base: integers wrap; float min/max are the @fastmath forms Finch runs under
 * (src/execute.jl:116-120): the new operand wins only when strictly smaller
 * (larger). */
typedef enum {
  FGB_PLUS_TIMES = 0, /* y[i] += A[i,j] * x[j]            */
  FGB_MIN_PLUS = 1,   /* y[i] <<min>>= A[i,j] + x[j]      */
  FGB_MAX_PLUS = 2,   /* y[i] <<max>>= A[i,j] + x[j]      */
  FGB_OR_AND = 3      /* y[i] |= A[i,j] & x[j]  (Bool)    */
} fgb_semiring;

typedef enum { FGB_CSR = 0, FGB_CSC = 1 } fgb_orient;

/* Flags for compute calls. */
#define FGB_ACCUMULATE 0x1u /* y/C keep their contents (no `y .= init`)      */
#define FGB_FINCH_ORDER 0x2u /* float sums in Finch's serial order:          \
                                one running sum per output, j ascending       */
#define FGB_FMA 0x4u         /* with FINCH_ORDER: fused a*b+c                */
#define FGB_NO_FMA 0x8u      /* with FINCH_ORDER: rounded product, then add  */

/* A sparse matrix as Finch level buffers (a plain struct; all pointers are
 * device pointers for compute calls). */
typedef struct fgb_sparse {
  int64_t nrows;      /* logical m */
  int64_t ncols;      /* logical n */
  int64_t nnz;        /* stored entries */
  int32_t orient;     /* fgb_orient */
  int32_t index_base; /* 0 or 1 (Finch: 1) */
  int32_t ptr_t;      /* FGB_I32 or FGB_I64 */
  int32_t idx_t;      /* FGB_I32 (compute) or FGB_I64 (input to narrowing) */
  int32_t val_t;      /* fgb_dtype, FGB_NONE for a Pattern level */
  int32_t reserved;
  const void* ptr; /* compressed-dimension + 1 entries */
  const void* idx; /* nnz entries */
  const void* val; /* nnz entries, or NULL for Pattern */
} fgb_sparse;

typedef struct fgb_ctx fgb_ctx;

/* ---- context, errors, memory ------------------------------------------ */

/* Version as MAJOR*1000 + MINOR. */
FGB_API int fgb_version(void);

/* Message of the last failed call on this thread ("" if none). */
FGB_API const char* fgb_last_error(void);

/* Create a context on `device`: records SM count, creates a stream, and
 * lets this process's default stream-ordered memory pool of the device keep
 * up to FGB_POOL_KEEP_BYTES of freed scratch mapped for reuse (it never
 * lowers a larger threshold the caller set).  Replaces the CPU device of
 * src/architecture.jl (AbstractDevice/CPU, architecture.jl:1-60) as the place
 * Finch runs the matched nests. */
#define FGB_POOL_KEEP_BYTES (8ull << 30)
FGB_API int fgb_ctx_create(int device, fgb_ctx** out);
FGB_API int fgb_ctx_destroy(fgb_ctx* ctx);
/* The context's stream (a cudaStream_t). */
FGB_API void* fgb_ctx_stream(fgb_ctx* ctx);
/* Synchronises the device, then returns in *flag whether any kernel of this
 * context gave up a bounded wait since the last call (1) or not (0), and
 * clears the flag.  A kernel that gives up reports here instead of hanging. */
FGB_API int fgb_ctx_device_error(fgb_ctx* ctx, int* flag);
FGB_API int fgb_ctx_num_sms(fgb_ctx* ctx);

/* Device buffers: the storage behind device-resident level buffers (what
 * Finch's transfer(device, lvl) recursion, sparse_list_levels.jl:64-69,
 * element_levels.jl:46-48, would place in HBM). */
FGB_API int fgb_malloc(fgb_ctx* ctx, size_t bytes, void** out);
FGB_API int fgb_free(fgb_ctx* ctx, void* p);
/* Pinned host buffers for copies that overlap compute. */
FGB_API int fgb_host_alloc(fgb_ctx* ctx, size_t bytes, void** out);
FGB_API int fgb_host_free(fgb_ctx* ctx, void* p);
/* Stream-ordered copies (one cudaMemcpyAsync each). */
FGB_API int fgb_upload(fgb_ctx* ctx, void* dst_dev, const void* src_host, size_t bytes, void* stream);
FGB_API int fgb_download(fgb_ctx* ctx, void* dst_host, const void* src_dev, size_t bytes, void* stream);
FGB_API int fgb_stream_sync(fgb_ctx* ctx, void* stream);

/* ---- level-buffer conversion ------------------------------------------ */

/* dst[i] = (int32)(src[i] - delta) for i < n; fails with EINVAL (after the
 * stream finishes) if any value does not fit in int32.  Narrows Finch's Int64
 * ptr/idx buffers (sparse_list_levels.jl:44-49) to the 32-bit form the
 * kernels read.  Synchronous. */
FGB_API int fgb_narrow_index(fgb_ctx* ctx, const int64_t* src, int32_t* dst, int64_t n, int64_t delta,
                     void* stream);

/* Stable transpose of the compressed orientation: CSC <-> CSR of the same
 * logical matrix, with coordinates ascending inside every fiber.  `out`
 * receives ptr (int64, nout+1) / idx (int32, nnz) / val (nnz, same dtype)
 * in caller-allocated device buffers, 0-based.  Replaces Finch's
 * CSC -> CSR copy through dropfills!/copyto! (src/interface/copy.jl:77-113).
 * Synchronous. */
FGB_API int fgb_transpose(fgb_ctx* ctx, const fgb_sparse* A, int64_t* out_ptr, int32_t* out_idx,
                  void* out_val, void* stream);

/* Dense copy of a sparse matrix: out (row-major nrows x ncols, leading
 * dimension ld, elements of A's val_t; one byte 0/1 for a Pattern) holds
 * the stored entries of A and *fill (one host element of val_t) elsewhere
 * -- the copy into Tensor(Dense(Dense(Element(fill))), A) that
 * src/interface/copy.jl makes.  Synchronous. */
FGB_API int fgb_sparse_to_dense(fgb_ctx* ctx, const fgb_sparse* A, const void* fill, void* out, int64_t ld,
                                void* stream);

/* The index a dense vector runs over in fgb_sparse_scale: A[i, j]'s row i
 * or column j. */
typedef enum fgb_axis {
  FGB_AXIS_ROW = 0,
  FGB_AXIS_COL = 1
} fgb_axis;

/* Stored entries of A combined with a dense vector and filtered by another
 * one -- the masked broadcast that builds PageRank's transition matrix
 * (docs/examples/pagerank.jl:17-25):
 *     for j=_, i=_; if keep[k] != 0; out[i, j] = A[i, j] op by[l]; end; end
 * with k and l the row i or column j as keep_axis and by_axis name them
 * (keep NULL keeps every entry).  op is FGB_MAP_MUL or FGB_MAP_DIV.  A's
 * values (F64, F32, I32, I64, BOOL, or NONE: a Pattern's true = 1) and `by`
 * (F64, F32, I32, I64, BOOL) are combined in F32 when one of them is F32
 * and neither is F64 (Julia's promotion for / and *), otherwise in F64
 * (integer products too), and converted to out_t (F64 or F32).  keep: F64,
 * F32, I32, I64 or BOOL (NaN counts as non-zero, as NaN != 0 is true).
 * The result keeps A's orientation and entry order without the dropped
 * entries: out_ptr (int64, n_fibers + 1, 0-based), out_idx (int32) and
 * out_val (out_t) with room for A->nnz entries; *out_nnz (host) receives
 * the kept count.  *n_fill_changed (host, may be NULL) receives how many
 * elements of `by` turn A's fill 0 into something else (0/0 and 0/NaN for
 * DIV, 0*Inf and 0*NaN for MUL): when it is 0, the entries A does not store
 * would all come out 0, so visiting stored entries only is exact -- Finch's
 * nest writes `0 / by[l]` there too, as `/` has no annihilator
 * (src/symbolic/symbolic.jl:145-153).  Synchronous. */
FGB_API int fgb_sparse_scale(fgb_ctx* ctx, const fgb_sparse* A, int op, int by_axis, int by_t,
                             const void* by, int keep_axis, int keep_t, const void* keep, int out_t,
                             int64_t* out_ptr, int32_t* out_idx, void* out_val, int64_t* out_nnz,
                             int64_t* n_fill_changed, void* stream);

/* Duplicate handling of fgb_coo_assemble: Julia's `combine` for fsparse. */
typedef enum fgb_combine {
  FGB_COMBINE_ADD = 0, /* +  (the default; | for Bool values) */
  FGB_COMBINE_OR = 1,  /* |  (Bool) */
  FGB_COMBINE_MIN = 2, /* min (NaN-propagating, -0.0 < +0.0) */
  FGB_COMBINE_MAX = 3, /* max */
  FGB_COMBINE_LAST = 4 /* the last duplicate in input order wins */
} fgb_combine;

/* COO triplets -> SparseList on the device: `fsparse(I, J, V, (m, n),
 * combine)` followed by the copy into Dense(SparseList(Element)) (out->orient
 * CSC) or its row-major swizzle (CSR), replacing the host path through
 * src/interface/fsparse.jl:60-100 and the COO -> CSC copy of
 * src/interface/copy.jl:77-113.  Entries come out sorted by (fiber,
 * coordinate); duplicates are folded left to right in input order with
 * `combine`, so float sums equal foldl's.  I, J: n_in device coordinates
 * (idx_t I32 or I64, base in_base); val: n_in values of val_t, NULL with
 * val_t FGB_NONE for a Pattern.  `out` describes caller buffers: nrows,
 * ncols, orient, index_base, ptr_t (I32/I64) with ptr of n_fibers + 1, idx_t
 * I32 and val_t = val_t, idx/val with room for n_in entries.  On return
 * *nnz_out = out->nnz = the stored count.  A coordinate outside the shape is
 * EINVAL.  Synchronous (the count is returned to the host). */
FGB_API int fgb_coo_assemble(fgb_ctx* ctx, int64_t nrows, int64_t ncols, int64_t n_in, int idx_t,
                             const void* I, const void* J, int in_base, int val_t, const void* val,
                             int combine, fgb_sparse* out, int64_t* nnz_out, void* stream);

/* ---- compute ------------------------------------------------------------ */

/* Semiring SpMV: y[i] <<add>>= mul(A[i,j], x[j]) for A m x n.
 * Replaces the nest `y .= init; for j=_, i=_; y[i] <<op>>= A[i,j] (*) x[j]`
 * (test/reference64/typical/typical_spmv_csc.txt:18-81) and its CSR form.
 * val_t/x_t/y_t combinations:
 *   PLUS_TIMES, MIN_PLUS, MAX_PLUS: F64/F64/F64, F32/F32/F32, BF16/F32/F32
 *                                   (PLUS_TIMES only), I32/I32/I32, I64/I64/I64
 *   OR_AND: BOOL or NONE (Pattern) / BOOL / BOOL
 * CSR runs as a pull (one running value per row); CSC runs as a push with
 * atomic updates of y (order-independent for exact semirings).  With
 * FGB_FINCH_ORDER on a CSR matrix every y[i] is one sequential sum over j
 * ascending, which equals Finch's serial CSC nest bit for bit.  Otherwise a
 * CSR matrix with at least 2048 rows per SM takes the adaptive pull (one
 * lane per row of at most 32 entries, a warp per longer row), and a smaller
 * one a fixed number of lanes per row chosen by its mean row length. */
FGB_API int fgb_spmv(fgb_ctx* ctx, int semiring, const fgb_sparse* A, const void* x, int x_t, void* y,
             int y_t, unsigned flags, void* stream);

/* SpMM: C[i,k] = (C[i,k] +) sum_j A[i,j] * B[j,k], k < nk.  B row-major
 * (ldb), C row-major (ldc).  F32 (A F32 or BF16 values, B/C F32) or F64.
 * Replaces `@einsum C[i,k] += A[i,j]*B[j,k]` = tensordot(A,B,(2,1))
 * (src/interface/lazy.jl:215-257,387-404).  CSR runs load-balanced
 * (merge-path items, deterministic carry fix-up); with FGB_FINCH_ORDER (or
 * an unaligned nk/ldb/ldc) each row is one running sum per column, j
 * ascending, bit-identical to Finch's nest.  CSC runs as a push with
 * atomics. */
FGB_API int fgb_spmm(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk, void* C,
             int64_t ldc, int dtype, unsigned flags, void* stream);

/* Semiring SpMM: C[i,k] <<add>>= mul(A[i,j], B[j,k]) over `semiring` (the
 * fgb_spmv semirings), B row-major (ldb), C row-major (ldc).  MIN_PLUS and
 * MAX_PLUS: values, B and C of `dtype` (F64, F32, I32, I64; integers wrap);
 * OR_AND: Bool (or Pattern) A with Bool B and C; PLUS_TIMES is fgb_spmm.
 * C starts at the semiring's identity unless FGB_ACCUMULATE.  A is CSR.
 * Replaces `@einsum init=-Inf R[i,j] <<max>>= P[i,k] + Q[k,j]`
 * (test/suites/interface_tests.jl:72-82) and its min-plus / or-and forms;
 * results are exact (the reductions are order-free). */
FGB_API int fgb_spmm_semiring(fgb_ctx* ctx, int semiring, const fgb_sparse* A, const void* B, int64_t ldb,
                              int64_t nk, void* C, int64_t ldc, int dtype, unsigned flags, void* stream);

/* Schedule knobs of the load-balanced CSR SpMM (the autotuner's search
 * space).  CSR SpMM walks merge-path items of `path` steps (rows + stored
 * entries) with groups of `lanes` lanes, each lane holding 4 (fp32) or 2
 * (fp64) consecutive columns; columns are processed in slabs of
 * lanes * vector-width, one launch per slab, so the gathered slab of B stays
 * L2-resident.  Zero fields take the defaults. */
typedef struct fgb_spmm_tuning {
  int32_t lanes;   /* 2, 4, 8, 16 or 32 (variants 2 and 3: 2, 4 or 8) */
  int32_t variant; /* 0: B rows gathered into registers; 1: B rows staged into a
                      shared-memory ring by TMA tile::gather4 (fp32); 2: rows
                      cut into virtual rows of at most `path` entries, sorted
                      by length, one launch per column slab of 4 * lanes (fp32);
                      3: variant 2 with the gathers staged in shared memory by
                      cp.async (more warps per SM; identical results) */
  int64_t path;    /* merge-path item length (variants 2, 3: virtual-row length) */
  int32_t bands;   /* variants 2, 3: cut A's columns into this many bands of
                      consecutive columns (0 or 1: none, at most 8), each band's
                      entries in launches of their own, so a launch gathers from
                      1/bands of B's slab; a row's sum still runs over its
                      entries in storage order, band after band */
  int32_t reserved;
} fgb_spmm_tuning;

/* fgb_spmm with an explicit schedule (NULL = defaults).  The result does not
 * depend on the schedule beyond float summation order. */
FGB_API int fgb_spmm_ex(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb, int64_t nk,
                        void* C, int64_t ldc, int dtype, unsigned flags,
                        const fgb_spmm_tuning* tune, void* stream);

/* Size of the fixed device scratch array behind fgb_spmm_noalloc (16 MiB). */
#define FGB_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)

/* fgb_spmm without any memory allocation.  No counterpart in the reference:
 * Finch's CPU kernels allocate nothing on a device, so this exists only for
 * callers of the GPU library that must not allocate device memory -- e.g. a
 * host whose device memory belongs to another pool (CUDA.jl), or a serving
 * loop that cannot afford an allocator call in its latency budget.  Same
 * arguments and results as fgb_spmm; the scratch of the load-balanced
 * schedule comes from one fixed array of FGB_NOALLOC_SCRATCH_BYTES per
 * device, held from first use until the process exits.  The schedule
 * lengthens its merge-path items until its scratch fits; a matrix whose
 * scratch exceeds the array even at the longest items (2^24 steps) is
 * rejected with FGB_EINVAL before any device work.  The context's device must
 * be the current device (FGB_EINVAL otherwise).  The first call on a device
 * looks the array's address up (cudaGetSymbolAddress), which also makes the
 * driver load the array (and the kernels' code) if it has not yet, so make
 * that call before any stream capture and before a region that must see no
 * change in free device memory.  All calls share the array:
 * calls that overlap on the GPU race and must be serialised by the caller. */
FGB_API int fgb_spmm_noalloc(fgb_ctx* ctx, const fgb_sparse* A, const void* B, int64_t ldb,
                             int64_t nk, void* C, int64_t ldc, int dtype, unsigned flags,
                             void* stream);

/* SDDMM: out[e] = A.val[e] * sum_k X[i,k] * Y[j,k] for every stored (i,j)
 * of A (out shares A's pattern).  X is m x k, Y is n x k, both row-major.
 * F32 or F64.  Replaces compute(lazy(A) .* (lazy(X) * lazy(Y^T)))
 * (src/interface/lazy.jl:323-331, benchmark/benchmarks.jl:141-168). */
FGB_API int fgb_sddmm(fgb_ctx* ctx, const fgb_sparse* A, const void* X, int64_t ldx, const void* Y,
              int64_t ldy, int64_t k, void* out_val, int dtype, unsigned flags, void* stream);

/* Schedule knobs of SDDMM (the autotuner's search space).  variant 0: warps
 * own chunks of `chunk` stored entries, `lanes` lanes (4, 8, 16 or 32) per
 * entry, and `slab` columns of k per launch (the dot accumulated across
 * launches; 0 = all of k, -1 = the default: one 128-byte line of Y per launch
 * when Y is far larger than L2).  variant 1 (F32 CSR, k <= 128 and a multiple
 * of 4): sub-groups own virtual rows of at most `chunk` entries, sorted by
 * length, holding the row's slice of X in registers; `slab` > 0 (a multiple
 * of 4) cuts k into launches of that many columns.  variant 2: variant 1
 * with the gathers of Y staged in shared memory by cp.async (identical
 * results).  Zero lanes/chunk take the defaults; NULL, or all fields at their
 * defaults (0, 0, 0, -1), is fgb_sddmm: the library picks the schedule. */
typedef struct fgb_sddmm_tuning {
  int32_t lanes;
  int32_t variant;
  int64_t chunk;
  int64_t slab;
  int32_t bands; /* variants 1, 2: column bands of A as in fgb_spmm_tuning (0 or 1: none) */
  int32_t reserved;
} fgb_sddmm_tuning;

FGB_API int fgb_sddmm_ex(fgb_ctx* ctx, const fgb_sparse* A, const void* X, int64_t ldx,
                         const void* Y, int64_t ldy, int64_t k, void* out_val, int dtype,
                         unsigned flags, const fgb_sddmm_tuning* tune, void* stream);

/* SpGEMM C = A * B (plus-times), Gustavson's algorithm as Finch writes it
 * (docs/examples/spgemm.jl:56-72, test/suites/kernel_tests.jl:89-129): every
 * output accumulates its products in the order of the shared index k, so F64
 * and F32 results equal the serial nest's for the same fused (default) or
 * FGB_NO_FMA choice; touched coordinates are stored even where they sum to
 * zero.  A and B share an orientation (CSR -> CSR, CSC -> CSC), a ptr type
 * and int32 indices.  Two calls: the symbolic one writes C's ptr (int64,
 * n_fibers + 1, in A's index base) and returns nnz(C); the caller allocates
 * C's idx (int32) and values and the numeric one fills them, each fiber's
 * coordinates ascending.  Both synchronous. */
FGB_API int fgb_spgemm_symbolic(fgb_ctx* ctx, const fgb_sparse* A, const fgb_sparse* B,
                                int64_t* c_ptr, int64_t* nnz_c, void* stream);
FGB_API int fgb_spgemm_numeric(fgb_ctx* ctx, const fgb_sparse* A, const fgb_sparse* B, int dtype,
                               unsigned flags, fgb_sparse* C, void* stream);

/* SpGEMM into a dense output: C (row-major A.nrows x B.ncols, leading
 * dimension ldc, dtype F64/F32) = A * B for A, B of one orientation (each
 * with its own ptr type and index base) -- the dense format Galley selects for a product
 * whose estimated density passes one half
 * (src/Galley/PhysicalOptimizer/format-selector.jl:27-65).  Each output sums
 * its products in the order of k as fgb_spgemm_numeric does, so its values
 * equal the sparse product's bit for bit (zero where nothing is stored). */
FGB_API int fgb_spgemm_dense(fgb_ctx* ctx, const fgb_sparse* A, const fgb_sparse* B, int dtype, unsigned flags,
                             void* C, int64_t ldc, void* stream);

/* Elementwise ops of two same-shape CSR/CSC matrices (same orientation). */
typedef enum {
  FGB_EW_MUL = 0, /* C = A .* B   (stored where both are stored) */
  FGB_EW_ADD = 1  /* C = A .+ B   (stored where either is stored) */
} fgb_ewise_op;

/* Pass 1 of a sparse elementwise op: out_ptr (int64, nfibers+1, 0-based)
 * gets the output pattern's fiber offsets and *out_nnz the total.
 * Synchronous (the caller sizes idx/val from *out_nnz).  Follows Finch's
 * two-finger merge of two SparseList fibers
 * (test/reference64/typical/typical_merge_twofinger.txt). */
FGB_API int fgb_ewise_count(fgb_ctx* ctx, int op, const fgb_sparse* A, const fgb_sparse* B,
                    int64_t* out_ptr, int64_t* out_nnz, void* stream);
/* Pass 2: fill idx (int32, 0-based) and val of the output. */
FGB_API int fgb_ewise_fill(fgb_ctx* ctx, int op, const fgb_sparse* A, const fgb_sparse* B,
                   const int64_t* out_ptr, int32_t* out_idx, void* out_val, void* stream);

/* reduce(op, A; dims) for op FGB_MAP_MIN or FGB_MAP_MAX -- maximum(A; dims)
 * and minimum(A; dims) (src/interface/eager.jl:153-158) -- of a sparse A
 * whatever its fill: every output folds its stored entries in coordinate
 * order and the fill `*fill` (one host element of val_t) once where a gap
 * or the end of the fiber leaves coordinates unstored, which is Finch's
 * fold with its fill runs folded once (min and max are idempotent), so the
 * results are Finch's bit for bit, @fastmath's first-operand rule for NaN
 * and signed zeros included.  The fold starts from `*init` (NULL: -Inf or
 * typemin for max, +Inf or typemax for min).  dims 1 reduces over rows
 * (y has ncols elements; A stored CSC), dims 2 over columns (nrows; A
 * stored CSR), dims 0 everything (one element; fibers in storage order).
 * y has A's value type: F64, F32, I64 or I32. */
FGB_API int fgb_reduce_minmax(fgb_ctx* ctx, int op, int dims, const fgb_sparse* A, const void* fill,
                              const void* init, void* y, void* stream);

/* Fused elementwise multiply + reduction:
 *   dims = 2:  y[i] = sum_j A[i,j] * B[i,j]      (length m)
 *   dims = 1:  y[j] = sum_i A[i,j] * B[i,j]      (length n)
 *   dims = 0:  y[0] = sum_ij A[i,j] * B[i,j]     (all dims)
 * B is a sparse matrix of the same shape/orientation (B_dense == NULL), a
 * dense row-major m x n matrix (B == NULL, ld = ldb), or absent (both NULL:
 * B = 1, i.e. reduce(+, A; dims), test/reference64/interface/
 * reduce_default.txt).  F32 or F64; reduce(+, A; dims) of a Pattern or Bool
 * A (val_t FGB_NONE or FGB_BOOL) counts its true entries into I64, as
 * Julia sums Bools into Int64 (dtype FGB_I64).
 * Replaces compute(sum(lazy(A) .* lazy(B); dims)) (src/interface/lazy.jl). */
FGB_API int fgb_ewise_reduce(fgb_ctx* ctx, int dims, const fgb_sparse* A, const fgb_sparse* B,
                     const void* B_dense, int64_t ldb, void* y, int dtype, unsigned flags,
                     void* stream);

/* ---- graph programs: the choose and minby reductions -------------------- */

/* One BFS round of docs/examples/bfs.jl:
 *   _F .= false
 *   for j=_, k=_; if F[j] && edges[k,j] && !(V[k])
 *     _F[k] |= true;  P[k] <<choose(z)>>= j;  end; end
 * with choose(z)(a, b) = isequal(a, z) ? b : a
 * (src/util/special_functions.jl:13-34).  A is the CSR of the adjacency
 * (row k lists the j with edges[k, j] stored; Pattern or any values),
 * frontier has ncols bytes, visited/next nrows bytes (0/1), parent nrows
 * values of parent_t (I32 or I64).  next[k] = the round's _F[k]; for a k
 * reached this round, parent[k] = choose(choose_fill)(parent[k], j1) where
 * j1 is the smallest reaching j (the first the j-ascending loop meets),
 * written as j1 + index_offset (1 for Finch's 1-based vertex numbers).
 * visited is read only (the program's second loop updates it:
 * fgb_or_count).  Bit-exact with the loop nest. */
FGB_API int fgb_bfs_pull(fgb_ctx* ctx, const fgb_sparse* A, const uint8_t* frontier, const uint8_t* visited,
                         void* parent, int parent_t, int64_t choose_fill, int64_t index_offset, uint8_t* next,
                         void* stream);

/* The second loop of a BFS round: for k; let f = next[k]; visited[k] |= f;
 * count[] += f; end.  count is a device int64 added to (exact). */
FGB_API int fgb_or_count(fgb_ctx* ctx, int64_t n, uint8_t* visited, const uint8_t* next, int64_t* count,
                         void* stream);

/* dist[j], parent[j] <<minby>>= (src_dist[j], src_parent[j]) for every j
 * with mask[j] (mask NULL: all j), minby(a, b) = a[1] > b[1] ? b : a
 * (src/util/special_functions.jl:75-88): the first loop of a relaxation
 * round of docs/examples/shortest_paths.jl.  Pairs are held as two arrays,
 * the first components of `dtype` (F64, F32, I32, I64), the second int64. */
FGB_API int fgb_minby_map(fgb_ctx* ctx, int dtype, int64_t n, const uint8_t* mask, const void* src_dist,
                          const int64_t* src_parent, void* dst_dist, int64_t* dst_parent, void* stream);

/* The second loop of that round:
 *   active .= false
 *   for j=_; if active_prev[j]; for i=_
 *     let d = first(dists_prev[j]) + edges[i, j]
 *       dists[i] <<minby>>= (d, j);  active[i] |= d < first(dists_prev[i])
 *   end; end; end; end
 * A is the CSR of the weights (row i lists the j with edges[i, j] stored,
 * ascending; values F64, F32, I32 or I64 -- the distance type); unstored
 * edges are the fill Inf and change nothing.  (dist, parent) are updated
 * in place, active (nrows bytes) written; j is written as j + index_offset.
 * Each row folds its contributions in ascending j, as the nest does, so
 * results are bit-exact.  dist_prev and dist must differ. */
FGB_API int fgb_minby_relax(fgb_ctx* ctx, const fgb_sparse* A, const void* dist_prev, const uint8_t* active_prev,
                            void* dist, int64_t* parent, uint8_t* active, int64_t index_offset, void* stream);

/* ---- dense Element levels and 0-d Scalars ------------------------------ */

typedef enum {
  FGB_MAP_ADD = 0,
  FGB_MAP_SUB = 1,
  FGB_MAP_MUL = 2,
  FGB_MAP_DIV = 3, /* fgb_scalar_op only */
  FGB_MAP_MIN = 4,
  FGB_MAP_MAX = 5
} fgb_map_op;

/* out[0] = sum_i x[i] * y[i] (deterministic: fixed block partials folded in
 * index order).  F32 or F64; out is a device scalar.  Replaces
 * `@einsum s[] += x[i]*y[i]` into a Scalar (src/tensors/scalars.jl:22-93). */
FGB_API int fgb_dense_dot(fgb_ctx* ctx, int dtype, int64_t n, const void* x, const void* y,
                          void* out, void* stream);

/* out[i] = a*x[i] + b*y[i], a and b read from device scalars (NULL = 1;
 * signs bit 0 negates a, bit 1 negates b; y NULL = 0).  F32 or F64. */
FGB_API int fgb_dense_axpby(fgb_ctx* ctx, int dtype, int64_t n, const void* alpha, const void* x,
                            const void* beta, const void* y, void* out, int signs, void* stream);

/* out[i] = alpha*x[i] + beta, or out[i] = beta with x NULL; alpha
 * and beta are device scalars (alpha NULL = 1, beta NULL = 0).  The
 * `r[i] = b + a*x[i]` and `r[j] = c` assignments of Finch programs
 * (docs/examples/pagerank.jl:27-32,43-48); fused (one rounding), as the
 * Finch-order SpMV and fgb_dense_axpby are by default.  F32 or F64. */
FGB_API int fgb_dense_affine(fgb_ctx* ctx, int dtype, int64_t n, const void* alpha, const void* x,
                             const void* beta, void* out, void* stream);

/* out[i] = op(x[i], y[i]) for op in ADD/SUB/MUL/MIN/MAX, the pointwise
 * `x = op.(x, y)` maps of Finch programs.  F64, F32, I32 (wrapping), I64. */
FGB_API int fgb_dense_map(fgb_ctx* ctx, int op, int dtype, int64_t n, const void* x,
                          const void* y, void* out, void* stream);

/* out[0] = op(a[0], b[0]) on device scalars (ADD/SUB/MUL/DIV/MIN/MAX). */
FGB_API int fgb_scalar_op(fgb_ctx* ctx, int op, int dtype, const void* a, const void* b,
                          void* out, void* stream);

/* ---- column panels: SpMM with an L2-resident slice of B ---------------- */

typedef struct fgb_panels fgb_panels;

/* Splits a CSR matrix's columns into `npanels` panels of consecutive
 * columns, built on the device once.  Panel 0 is a CSR over all rows; panels
 * 1.. list only their non-empty rows (a row map over a SparseList of rows,
 * i.e. Finch's SparseList(SparseList(Element)) / DCSR).  Each panel of an
 * SpMM then gathers only its 1/npanels slice of B's rows, which stays in L2;
 * C rows touched by several panels are accumulated panel by panel.  The
 * layout holds a copy of A's idx/val (sorted by panel).  Synchronous. */
FGB_API int fgb_panels_create(fgb_ctx* ctx, const fgb_sparse* A, int32_t npanels,
                              fgb_panels** out);
/* C = (C +) A @ B through the panels (F32 with F32/BF16 values, or F64).
 * nk, ldb, ldc and the B/C pointers must be 4-float (2-double) aligned.
 * The merge-path item boundaries of every panel are computed on the first
 * call and reused while nk and the item length stay the same. */
FGB_API int fgb_panels_spmm(fgb_ctx* ctx, fgb_panels* panels, const void* B, int64_t ldb,
                            int64_t nk, void* C, int64_t ldc, int dtype, unsigned flags,
                            const fgb_spmm_tuning* tune, void* stream);
FGB_API int fgb_panels_destroy(fgb_panels* panels);

/* ---- plans: autotuned, graph-captured operations ------------------------ */

typedef struct fgb_plan fgb_plan;

typedef enum { FGB_PLAN_SPMV = 0, FGB_PLAN_SPMM = 1, FGB_PLAN_SDDMM = 2 } fgb_plan_op;

/* One operation on fixed device operands:
 *   SPMV:  out = A (*) in0 over `semiring`      (dtype of in0/out)
 *   SPMM:  out = A @ in0, in0 n x k (ld_in0), out m x k (ld_out)
 *   SDDMM: out = A .* (in0 @ in1^T), in0 m x k (ld_in0), in1 n x k (ld_in1) */
typedef struct fgb_plan_desc {
  int32_t op;
  int32_t semiring;
  int32_t dtype;
  uint32_t flags;
  const fgb_sparse* A;
  const void* in0;
  const void* in1;
  void* out;
  int64_t ld_in0, ld_in1, ld_out;
  int64_t k;
} fgb_plan_desc;

typedef struct fgb_plan_info {
  int32_t lanes;             /* chosen lanes per fiber / row group / entry; for a
                                CSR SpMV, 2 is the adaptive pull (one lane per row
                                of at most 32 entries, a warp per longer row) */
  int32_t bands;             /* SpMM/SDDMM virtual rows: column bands (1 = none) */
  int64_t path;              /* chosen merge-path item (SpMM) or entry chunk (SDDMM) */
  double tuned_ms;           /* time of the chosen schedule (-1 if not tuned) */
  double first_candidate_ms; /* time of the first schedule tried */
  int32_t candidates;        /* schedules in the search space */
  int32_t from_cache;        /* 1 if the choice came from the tuning cache */
  int32_t panels;            /* SpMM: column panels of the chosen schedule (1 = none) */
  int32_t variant;           /* SpMM: fgb_spmm_tuning.variant; SDDMM: 3 virtual rows, 4 the same
                                with cp.async gathers */
  int32_t launches;          /* kernel launches of one fgb_plan_execute (the captured graph's
                                kernel nodes) */
  int32_t reserved;
} fgb_plan_info;

/* Autotunes (tune_reps timed runs per schedule on these operands; 0 = use
 * the first schedule), precomputes what depends only on A, and captures the
 * chosen launches into a CUDA graph bound to these operand pointers.  The
 * choice is cached per shape class (and appended to the file named by
 * FGB_TUNE_CACHE).  Writes `out` while tuning.  Synchronous. */
FGB_API int fgb_plan_create(fgb_ctx* ctx, const fgb_plan_desc* desc, int32_t tune_reps,
                            fgb_plan** out);
/* Replays the captured operation on `stream`. */
FGB_API int fgb_plan_execute(fgb_plan* plan, void* stream);
FGB_API int fgb_plan_info_get(fgb_plan* plan, fgb_plan_info* out);
FGB_API int fgb_plan_destroy(fgb_plan* plan);

/* ---- seeded inputs ------------------------------------------------------ */

/* Random m x n CSR on the device with fsprand's distribution
 * (src/interface/fsparse.jl:173-290): each (i,j) stored independently with
 * probability p; values N(0,1) (F32) or U[0,1) (F64).  Pass 1 (idx == NULL)
 * writes ptr (int32, 0-based, m+1) and *nnz (synchronous); pass 2 fills idx
 * (int32, ascending per row) and val.  Depends only on (seed, m, n, p). */
FGB_API int fgb_random_csr(fgb_ctx* ctx, uint64_t seed, int64_t m, int64_t n, double p, int val_t,
                           int32_t* ptr, int32_t* idx, void* val, int64_t* nnz, void* stream);

/* ---- serving: continuous batching of many small requests ------------- */

typedef struct fgb_server fgb_server;

typedef enum {
  FGB_REQ_SPMV = 0,      /* y = A x                      (x: ncols, y: nrows)   */
  FGB_REQ_SPMM = 1,      /* C = A B, B ncols x nk        (nk = 4, 8, ..., 128) */
  FGB_REQ_MASKED_MUL = 2 /* A .* B2 on A's pattern       (out: nnz of A)       */
} fgb_request_op;

typedef enum {
  FGB_SERVE_BATCHED = 0, /* persistent device loop, continuous batching */
  FGB_SERVE_PER_CALL = 1 /* one launch + copies + sync per request      */
} fgb_serve_mode;

typedef struct fgb_server_config {
  size_t pool_bytes;     /* HBM budget for in-flight inputs/outputs (admission) */
  int32_t max_inflight;  /* request slots, <= 4096 */
  int32_t rows_per_item; /* rows per work item (default 64): the batched loop's, and per-call
                          * launches' until fgb_server_tune sets them per size class */
  int32_t blocks_per_sm; /* persistent blocks per SM (default 4; capped one below occupancy) */
  int32_t idle_exit_us;  /* device loop exits after this long without work (default 20000) */
  int32_t mode;          /* fgb_serve_mode */
  int32_t reserved;
} fgb_server_config;

typedef struct fgb_request {
  int32_t op;         /* fgb_request_op */
  int32_t matrix;     /* id from fgb_server_register */
  int32_t matrix_b;   /* second operand of FGB_REQ_MASKED_MUL */
  int32_t nk;         /* SpMM width */
  const void* input;  /* host FP32 x or row-major B (NULL for MASKED_MUL) */
  void* output;       /* host FP32 result, written before fgb_server_wait returns */
} fgb_request;

typedef struct fgb_server_stats {
  uint64_t submitted, completed, launches, batches_published, pool_used;
  /* dispatcher time (ns): admitting and staging, scanning for completions,
   * and releasing completed requests; and its loop iterations */
  uint64_t admit_ns, scan_ns, finish_ns, iterations;
  /* summed over completed requests (ns): submit to admission (queueing),
   * admission to completion seen (service) */
  uint64_t queue_ns, service_ns;
} fgb_server_stats;

/* Serving front end for compute() calls on resident tensors.  Admission is by
 * HBM footprint (a request waits until its input and output fit in the pool
 * and a slot is free); admitted requests are published to a device-side loop
 * that overlaps their work; results are identical to running each request
 * alone.  Every device wait is bounded (idle_exit_us). */
FGB_API int fgb_server_create(fgb_ctx* ctx, const fgb_server_config* cfg, fgb_server** out);
/* Registers a resident CSR matrix (device buffers, int32 ptr/idx, F32 values). */
FGB_API int fgb_server_register(fgb_server* srv, const fgb_sparse* A, int32_t* id);
/* Queues a request; returns at once with a ticket.  A page-locked output
 * buffer is written by the device in place (no copy back, no pool memory). */
FGB_API int fgb_server_submit(fgb_server* srv, const fgb_request* req, uint64_t* ticket);
/* Queues n requests under one lock; *n_accepted of them got tickets (all, or
 * those before the first rejected one, whose status is returned). */
FGB_API int fgb_server_submit_batch(fgb_server* srv, const fgb_request* reqs, int32_t n,
                                    uint64_t* tickets, int32_t* n_accepted);
/* Waits for n tickets within one overall timeout; latencies_s may be NULL. */
FGB_API int fgb_server_wait_batch(fgb_server* srv, const uint64_t* tickets, int32_t n,
                                  int32_t timeout_ms, double* latencies_s);
/* Waits up to timeout_ms for a ticket (FGB_ETIMEOUT after that); on success
 * the output is in host memory and *latency_s is submit-to-result time. */
FGB_API int fgb_server_wait(fgb_server* srv, uint64_t ticket, int32_t timeout_ms,
                            double* latency_s);
FGB_API int fgb_server_stats_get(fgb_server* srv, fgb_server_stats* out);

/* Serving shapes per size class.  Registered matrices fall into classes by
 * their mean stored entries per row (class 0: below 1; class c >= 1: in
 * [2^(c-1), 2^c); the last class: everything above).  Each class has its
 * SpMV lanes per row (a power of two <= 32; 32 / lanes rows per warp at
 * once) and rows per work item (the unit the device loop claims). */
#define FGB_SERVER_CLASSES 10
typedef struct fgb_server_class_shape {
  int32_t matrices;      /* registered matrices of the class (tune: output only) */
  int32_t lanes;         /* SpMV lanes per row */
  int32_t rows_per_item; /* rows per work item of per-call launches (the batched
                          * loop keeps the configured value: items only split rows) */
  int32_t reserved;
  double ms;             /* tune: time of the class's sample at the chosen shape (-1: none) */
  double ms_default;     /* tune: the same sample at 32 lanes and the configured rows per item */
} fgb_server_class_shape;
typedef struct fgb_server_tuning {
  fgb_server_class_shape cls[FGB_SERVER_CLASSES];
} fgb_server_tuning;

/* The serving autotuner (no counterpart in Finch): for every size class
 * with registered matrices, times SpMV requests on up to 8 of them through
 * the serving kernel itself at every shape (lanes 2..32, rows per item
 * 32..256), reps timed runs each, keeps the fastest and applies it to the
 * class (its matrices and later registrations).  Both modes sum a row the
 * same way for given lanes, so batched and per-call results stay identical
 * under the same tuning.  A batched server first waits (bounded) for its
 * device loop's idle exit, so the timings have the GPU to themselves.  The
 * server must be idle (FGB_EBUSY
 * otherwise).  Synchronous; allocates its timing buffers. */
FGB_API int fgb_server_tune(fgb_server* srv, int32_t reps, fgb_server_tuning* out);
/* Applies shapes (lanes, rows_per_item per class; other fields ignored),
 * e.g. those another server's fgb_server_tune chose.  Idle server only. */
FGB_API int fgb_server_set_tuning(fgb_server* srv, const fgb_server_tuning* tuning);
/* Stops the device loop (bounded) and frees everything. */
FGB_API int fgb_server_destroy(fgb_server* srv);

/* ---- conjugate gradients ------------------------------------------------ */

typedef struct fgb_cg_options {
  double rtol;           /* stop when ||b - A x|| <= rtol * ||b|| (true residual) */
  int64_t max_iter;      /* iteration cap (rounded up to whole chunks) */
  int32_t chunk;         /* iterations per captured CUDA graph (even) */
  int32_t precision;     /* value type of the iteration SpMV: FGB_F64, FGB_F32 or FGB_BF16 */
  int64_t replace_every; /* FP64 residual replacement period in iterations (0 = only at the end) */
  int32_t accumulate;    /* arithmetic of an FP32/BF16-valued solve: FGB_CG_SUM_* */
  int32_t reserved;
} fgb_cg_options;

/* fgb_cg_options.accumulate (ignored for FP64 values, which sum in FP64) */
#define FGB_CG_SUM_F32 0  /* SpMV: values times an FP32 copy of p, FP32 sums; vectors, dots, updates FP64 */
#define FGB_CG_SUM_F64 1  /* SpMV: values widened to FP64, FP64 sums; vectors, dots, updates FP64 */
#define FGB_CG_SUM_SPMV_PAIR 3 /* SpMV: values times p split into a pair of FP32 numbers (about 48 bits)
                                * by integer operations, each row summed as a pair; vectors, dots and
                                * updates FP64: no FP64 instruction per stored entry */
#define FGB_CG_SUM_PAIR 2 /* SpMV sums, x, r, p, q, dots and updates in pairs of FP32 numbers
                           * (hi + lo, about 48 significant bits), no FP64 arithmetic per row or
                           * stored entry: the fast mode on GPUs whose FP64 rate is far below FP32.
                           * Pairs keep FP32's exponent range: the squares of the residual's
                           * entries must stay above FP32's smallest normal (about 1e-38) down to
                           * the tolerance, so scale b accordingly */

typedef struct fgb_cg_result {
  int64_t iterations;       /* iterations run */
  int64_t replacements;     /* FP64 residual replacements done */
  double true_rel_residual; /* ||b - A x|| / ||b|| at exit, FP64 */
  double seconds;           /* wall time of the solve */
  int32_t converged;
  int32_t compact_index;    /* 1: the iteration SpMV read 16-bit column offsets (a banded matrix) */
} fgb_cg_result;

/* Solves A x = b for SPD CSR A; x holds the initial guess and receives the
 * solution (device FP64 vectors).  A64 carries FP64 values (residual
 * replacement and the FP64 mode); Alow (same pattern) carries the FP32 or
 * BF16 values of the iteration SpMV (NULL when precision is FGB_F64).  The
 * loop is the Finch program `@einsum q[i] += A[i,j]*p[j]`,
 * `@einsum s[] += p[i]*q[i]` and the vector updates, in the arithmetic that
 * opt->accumulate names, with FP64 reliable updates of the residual.
 * Synchronous with respect to `stream`. */
FGB_API int fgb_cg_solve(fgb_ctx* ctx, const fgb_sparse* A64, const fgb_sparse* Alow,
                         const double* b, double* x, const fgb_cg_options* opt,
                         fgb_cg_result* res, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FINCHGB_H */
