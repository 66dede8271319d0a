/*
 * randblas_gb300.h -- C ABI of the GB300 (sm_103a) sketching library.
 *
 * This is the drop-in boundary for RandBLAS's sketching hot path.  Every entry point takes
 * plain pointers and sizes; matrix/vector buffers are DEVICE pointers unless stated
 * otherwise, and every call is asynchronous on the given CUDA stream (NULL = the legacy
 * default stream) unless its comment says it synchronises.  Each declaration names the
 * reference interface it replaces (paths relative to the RandBLAS source tree).
 *
 * Conventions (numeric values shared with the reference's enums' meaning):
 *   layout  RBG_COL_MAJOR / RBG_ROW_MAJOR     blas::Layout
 *   op      RBG_NO_TRANS / RBG_TRANS           blas::Op
 *   family  RBG_GAUSSIAN / RBG_UNIFORM         RandBLAS::ScalarDist (RandBLAS/dense_skops.hh:215-224)
 *   axis    RBG_AXIS_SHORT / RBG_AXIS_LONG     RandBLAS::Axis (RandBLAS/base.hh:306-312)
 *   dtype   RBG_F32 / RBG_F64                  the template parameter T
 *   itype   RBG_I32 / RBG_I64                  the template parameter sint_t
 *
 * Errors: every entry point returns RBG_SUCCESS (0) or a status code; rbg_last_error()
 * returns a thread-local message.  Argument checks that the reference performs with
 * randblas_require (RandBLAS/exceptions.hh:152-162) return RBG_ERROR_INVALID_ARGUMENT
 * with the reference's message text "<cond> was required, but did not hold, in
 * function <f>"; integer overflow of a size product (RandBLAS/base.hh:260-274) returns
 * RBG_ERROR_OVERFLOW.
 */
#ifndef RANDBLAS_GB300_H
#define RANDBLAS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same object as cudaStream_t; declared here so the header needs no CUDA include. */
typedef struct CUstream_st *rbg_stream_t;

enum { RBG_COL_MAJOR = 0, RBG_ROW_MAJOR = 1 };
enum { RBG_NO_TRANS = 0, RBG_TRANS = 1 };
enum { RBG_GAUSSIAN = 0, RBG_UNIFORM = 1 };
enum { RBG_AXIS_SHORT = 0, RBG_AXIS_LONG = 1 };
enum { RBG_F32 = 0, RBG_F64 = 1 };
/* Storage type of A accepted by rbg_lskge3_lowp_ex (precision path only). */
enum { RBG_BF16 = 2 };
enum { RBG_I32 = 0, RBG_I64 = 1 };
enum { RBG_COO = 0, RBG_CSR = 1, RBG_CSC = 2 };
/* NonzeroSort (RandBLAS/sparse_data/base.hh:108-117), with the reference's character values. */
enum { RBG_SORT_CSC = 'C', RBG_SORT_CSR = 'R', RBG_SORT_NONE = 'N' };
enum { RBG_PREC_BF16 = 0, RBG_PREC_FP8_E4M3 = 1 };

enum {
    RBG_SUCCESS = 0,
    RBG_ERROR_INVALID_ARGUMENT = 1, /* RandBLAS::Error from randblas_require */
    RBG_ERROR_OVERFLOW = 2,         /* std::overflow_error from safe_int_product */
    RBG_ERROR_CUDA = 3,             /* a CUDA runtime call or kernel launch failed */
    RBG_ERROR_TIMEOUT = 4,          /* a bounded device-side wait gave up */
    RBG_ERROR_UNSUPPORTED = 5,      /* valid in the reference, not provided by this library */
    RBG_ERROR_ALLOC = 6             /* device memory allocation failed */
};

/* RNGState<Philox4x32> (RandBLAS/base.hh:64-164): 128-bit counter as four little-endian
 * 32-bit words and a 64-bit key as two. */
typedef struct rbg_state {
    uint32_t counter[4];
    uint32_t key[2];
} rbg_state;

/* DenseDist (RandBLAS/dense_skops.hh:231-350). */
typedef struct rbg_dense_dist {
    int64_t n_rows;
    int64_t n_cols;
    int32_t family;     /* RBG_GAUSSIAN (default) or RBG_UNIFORM */
    int32_t major_axis; /* RBG_AXIS_LONG (default) or RBG_AXIS_SHORT */
} rbg_dense_dist;

/* DenseSkOp<T> (RandBLAS/dense_skops.hh:357-478).  buff == NULL means "not materialised":
 * sketching calls then generate the entries they need on the fly, inside the kernel. */
typedef struct rbg_dense_skop {
    rbg_dense_dist dist;
    rbg_state seed_state;
    rbg_state next_state;
    int32_t dtype;  /* RBG_F32 / RBG_F64 */
    int32_t layout; /* layout of buff; the dist's natural layout by default */
    void *buff;     /* device pointer, n_rows * n_cols entries, or NULL */
} rbg_dense_skop;

/* SparseDist (RandBLAS/sparse_skops.hh:131-246). */
typedef struct rbg_sparse_dist {
    int64_t n_rows;
    int64_t n_cols;
    int64_t vec_nnz;    /* default 4 */
    int32_t major_axis; /* RBG_AXIS_SHORT (SASO, default) or RBG_AXIS_LONG (LASO) */
    int32_t reserved;
} rbg_sparse_dist;

/* SparseSkOp<T, RNG, sint_t> (RandBLAS/sparse_skops.hh:289-450).  nnz < 0 means "not
 * sampled": sketching calls then sample it themselves (SASOs inside the kernel). */
typedef struct rbg_sparse_skop {
    rbg_sparse_dist dist;
    rbg_state seed_state;
    rbg_state next_state;
    int64_t nnz;
    int32_t dtype;
    int32_t itype;
    void *vals; /* device pointers, dist.vec_nnz * dim_minor entries each */
    void *rows;
    void *cols;
} rbg_sparse_skop;

/* COOMatrix / CSRMatrix / CSCMatrix views (RandBLAS/sparse_data/coo_matrix.hh:82-308,
 * csr_matrix.hh:73-245, csc_matrix.hh:73-244), zero-based indices, device pointers.
 *   COO: idx_a = rows (nnz),        idx_b = cols (nnz)
 *   CSR: idx_a = rowptr (n_rows+1), idx_b = colidxs (nnz)
 *   CSC: idx_a = colptr (n_cols+1), idx_b = rowidxs (nnz) */
typedef struct rbg_spmat {
    int32_t format; /* RBG_COO / RBG_CSR / RBG_CSC */
    int32_t dtype;
    int32_t itype;
    int32_t reserved;
    int64_t n_rows;
    int64_t n_cols;
    int64_t nnz;
    const void *vals;
    const void *idx_a;
    const void *idx_b;
} rbg_spmat;

/* ------------------------------------------------------------------ library */

/* Message of the last failed call on this host thread ("" if none). */
const char *rbg_last_error(void);
/* 10000 * major + 100 * minor + patch. */
int rbg_version(void);
/* Number of CUDA kernels this library has launched in this process (its own kernels; the
 * radix-sort passes it delegates to CUB are not counted).  No reference counterpart. */
uint64_t rbg_kernel_launches(void);
/* Reproducibility switch, no reference counterpart (process-wide).  On: every path adds in a
 * fixed order, so results are bitwise reproducible run to run.  Off (default): the fused SASO
 * left sketch accumulates with shared-memory reductions whose order depends on scheduling
 * (results agree to FP32 rounding).  rbg_get_deterministic returns the current setting. */
int rbg_set_deterministic(int on);
int rbg_get_deterministic(void);
/* Per-kernel timing, no reference counterpart.  While enabled, the library records CUDA events
 * on the launching stream around its main kernels; rbg_profile_enable also clears what was
 * recorded.  rbg_profile_entry synchronises on the recorded events. */
int rbg_profile_enable(int on);
int rbg_profile_count(int32_t *count);
int rbg_profile_entry(int32_t index, char *name, int32_t name_cap, double *total_ms,
                      int64_t *launches);

/* ------------------------------------------------------------------ host-side logic */

/* RNGState(uint64 k): counter 0, key k (RandBLAS/base.hh:119). */
int rbg_state_from_key(uint64_t k, rbg_state *out);
/* counter.incr(n) on a copy (Random123 r123array4x32::incr, RandBLAS/base.hh:84-97). */
int rbg_state_incr(const rbg_state *in, uint64_t n, rbg_state *out);

/* DenseDist constructor's derived fields (RandBLAS/dense_skops.hh:313-329). */
int rbg_dense_dist_properties(const rbg_dense_dist *D, int64_t *dim_major, int64_t *dim_minor,
                              int32_t *natural_layout, double *isometry_scale);
/* dense::compute_next_state (RandBLAS/dense_skops.hh:172-185). */
int rbg_dense_next_state(const rbg_dense_dist *D, const rbg_state *seed, rbg_state *next);
/* DenseSkOp(dist, seed) (RandBLAS/dense_skops.hh:441-453): fills seed/next state, natural
 * layout and buff = NULL. */
int rbg_dense_skop_init(rbg_dense_skop *S, const rbg_dense_dist *D, const rbg_state *seed,
                        int32_t dtype);

/* SparseDist constructor's derived fields (RandBLAS/sparse_skops.hh:208-224). */
int rbg_sparse_dist_properties(const rbg_sparse_dist *D, int64_t *dim_major,
                               int64_t *dim_minor, int64_t *full_nnz, double *isometry_scale);
/* compute_next_state(SparseDist, state) (RandBLAS/sparse_skops.hh:266-283). */
int rbg_sparse_next_state(const rbg_sparse_dist *D, const rbg_state *seed, rbg_state *next);
/* SparseSkOp(dist, seed) (RandBLAS/sparse_skops.hh:399-407): nnz = -1, no arrays. */
int rbg_sparse_skop_init(rbg_sparse_skop *S, const rbg_sparse_dist *D, const rbg_state *seed,
                         int32_t dtype, int32_t itype);

/* ------------------------------------------------------------------ sampling */

/* fill_dense_unpacked (RandBLAS/dense_skops.hh:563-606): write the n_rows x n_cols
 * submatrix at (ro_s, co_s) of a matrix from D, in `layout`, packed, into buff.  *next gets
 * the state the reference returns (seed + first counter used + rows * stride). */
int rbg_fill_dense_unpacked(int32_t dtype, int32_t layout, const rbg_dense_dist *D,
                            int64_t n_rows, int64_t n_cols, int64_t ro_s, int64_t co_s,
                            void *buff, const rbg_state *seed, rbg_state *next,
                            rbg_stream_t stream);
/* fill_dense(D, buff, seed) (RandBLAS/dense_skops.hh:623-626), natural layout. */
int rbg_fill_dense(int32_t dtype, const rbg_dense_dist *D, void *buff, const rbg_state *seed,
                   rbg_state *next, rbg_stream_t stream);
/* fill_dense(S) (RandBLAS/dense_skops.hh:649-658): S->buff must be a device buffer of
 * n_rows * n_cols entries; written in S->layout. */
int rbg_fill_dense_skop(rbg_dense_skop *S, rbg_stream_t stream);

/* fill_sparse_unpacked_nosub (RandBLAS/sparse_skops.hh:515-565): sample into device COO
 * arrays of length >= vec_nnz * dim_minor.  *nnz is written on return, which makes this
 * call synchronise `stream` for LASOs (their nnz depends on duplicate merging); for SASOs
 * nnz = vec_nnz * dim_minor and the call stays asynchronous.  LASO duplicates are merged
 * as in the reference (sqrt(count) * first sign) and emitted in first-occurrence order
 * (the reference's order there is std::unordered_map's, which is unspecified). */
int rbg_fill_sparse_unpacked_nosub(int32_t dtype, int32_t itype, const rbg_sparse_dist *D,
                                   int64_t *nnz, void *vals, void *rows, void *cols,
                                   const rbg_state *seed, rbg_state *next, rbg_stream_t stream);
/* fill_sparse(S) (RandBLAS/sparse_skops.hh:587-603): S->vals/rows/cols must be device
 * buffers of full_nnz entries; sets S->nnz. */
int rbg_fill_sparse(rbg_sparse_skop *S, rbg_stream_t stream);
/* repeated_fisher_yates(k, n, r, samples, state) (RandBLAS/sparse_skops.hh:259-264):
 * r independent k-subsets of {0..n-1}, int64 samples[k * r]. */
int rbg_repeated_fisher_yates(int64_t k, int64_t n, int64_t r, int64_t *samples,
                              const rbg_state *seed, rbg_state *next, rbg_stream_t stream);

/* ------------------------------------------------------------------ random sparse matrices */

/* random_coo / random_csr / random_csc (RandBLAS/sparse_data/random_matrix.hh:135-355): an
 * m x n sparse matrix whose entries are each present with probability `density`, with
 * Gaussian values, drawn from the sequential stream at `seed` (random_matrix.hh:63-121).
 * Positions, order (CSR order for COO), index arrays and the next state are the reference's;
 * values are its Box-Muller values as rbg_fill_dense computes them.  Two calls, because the
 * number of nonzeros is random:
 *   rbg_random_sparse_create  draws the structure on the GPU, writes *nnz and *next
 *                             (synchronises `stream`); the handle keeps device memory;
 *   rbg_random_sparse_fill    writes device arrays: COO a = rows[nnz], b = cols[nnz];
 *                             CSR a = rowptr[m + 1], b = colidxs[nnz];
 *                             CSC a = colptr[n + 1], b = rowidxs[nnz];
 *   rbg_random_sparse_destroy frees the handle; its device memory is released in stream
 *                             order on the stream of the last create or fill call (which
 *                             must still exist), after the work queued there.
 * density outside [0, 1] fails the reference's check.  Limits of this library: the compressed
 * formats need fewer than 2^30 stream words (about 5e8 nonzeros) and a minor dimension below
 * 2^31 - 1; 0 < density < 2^-53 (where log(1 - density) rounds to 0 and the reference's skip
 * is undefined) returns RBG_ERROR_UNSUPPORTED. */
typedef struct rbg_random_sparse_s *rbg_random_sparse;
int rbg_random_sparse_create(int32_t format, int64_t m, int64_t n, double density,
                             const rbg_state *seed, rbg_random_sparse *out, int64_t *nnz,
                             rbg_state *next, rbg_stream_t stream);
int rbg_random_sparse_fill(rbg_random_sparse h, int32_t dtype, int32_t itype, void *vals,
                           void *a, void *b, rbg_stream_t stream);
/* near_ties: skips of this matrix whose quotient log(1 - u) / log(1 - density) lay within
 * 2^-48 (relative) of an integer, where the device logarithm and the host C library's may floor
 * differently (about 1e-14 per draw; the matrix is the reference's when this is 0);
 * words_drawn: stream words the reference's loop draws.  Either pointer may be NULL. */
int rbg_random_sparse_info(rbg_random_sparse h, int64_t *near_ties, int64_t *words_drawn);
int rbg_random_sparse_destroy(rbg_random_sparse h);

/* ------------------------------------------------------------------ sparse data conversions */

/* The building blocks of RandBLAS's csr_to_coo / csc_to_coo / coo_to_csr / coo_to_csc
 * (RandBLAS/sparse_data/conversions.hh:49-121), on device arrays.  Each performs the
 * reference's checks with its messages and synchronises `stream`.  Index arrays are int32 or
 * int64 (ptr_itype / idx_itype / itype: RBG_I32 or RBG_I64), independently.
 *
 * compressed_ptr_to_sorted_idxs (RandBLAS/sparse_data/base.hh:292-302): idxs[0 ..) gets index j
 * repeated ptr[j + 1] - ptr[j] times, for j < num_comp.  Requires len_idxs >= ptr[num_comp]
 * and no negative segment. */
int rbg_compressed_ptr_to_sorted_idxs(int64_t num_comp, int32_t ptr_itype, const void *ptr,
                                      int64_t len_idxs, int32_t idx_itype, void *idxs,
                                      rbg_stream_t stream);
/* sorted_idxs_to_compressed_ptr (RandBLAS/sparse_data/base.hh:278-290): ptr[0] = 0 and
 * ptr[i + 1] = the number of idxs <= i, for the reference's walk.  A leading negative index
 * leaves every pointer 0, and indices >= num_comp are not counted.  Requires sorted idxs. */
int rbg_sorted_idxs_to_compressed_ptr(int64_t len_idxs, int32_t idx_itype, const void *idxs,
                                      int64_t num_comp, int32_t ptr_itype, void *ptr,
                                      rbg_stream_t stream);
/* coo_arrays_determine_sort (RandBLAS/sparse_data/base.hh:142-167): *sort = RBG_SORT_CSC if the
 * entries are in CSC order (ties allowed), else RBG_SORT_CSR if in CSR order, else
 * RBG_SORT_NONE. */
int rbg_coo_determine_sort(int32_t itype, int64_t nnz, const void *rows, const void *cols,
                           int32_t *sort, rbg_stream_t stream);
/* coo_arrays_apply_sort / COOMatrix::sort_arrays (RandBLAS/sparse_data/base.hh:169-220,
 * coo_matrix.hh:222-226): sorts (vals, rows, cols) in place by (row, col) for RBG_SORT_CSR or
 * (col, row) for RBG_SORT_CSC.  No-op for RBG_SORT_NONE or when the entries are already in that
 * order.  Entries with equal (row, col) keep their relative order (the reference's std::sort
 * leaves it unspecified).  dtype: RBG_F32 or RBG_F64. */
int rbg_coo_apply_sort(int32_t sort, int32_t dtype, int32_t itype, int64_t nnz, void *vals,
                       void *rows, void *cols, rbg_stream_t stream);

/* ------------------------------------------------------------------ dense operators */

/* LSKGE3 / sketch_general left (RandBLAS/skge.hh:154-202, 756-821, 1073-1097):
 *   B = alpha * op(submat(S)) * op(A) + beta * B,  op(submat(S)) d x m at (ro_s, co_s),
 *   op(A) m x n, B d x n; A, B in `layout` with leading dims lda, ldb.
 * T = S->dtype for A, B, alpha, beta.  beta == 0 does not read B; alpha == 0 does not read
 * A.  Generated operators are never materialised: entries are produced in the GEMM. */
int rbg_lskge3(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n, int64_t m,
               double alpha, const rbg_dense_skop *S, int64_t ro_s, int64_t co_s,
               const void *A, int64_t lda, double beta, void *B, int64_t ldb,
               rbg_stream_t stream);
/* RSKGE3 / sketch_general right (RandBLAS/skge.hh:307-355, 928-992, 1175-1199):
 *   B = alpha * op(A) * op(submat(S)) + beta * B,  op(A) m x n, op(submat(S)) n x d. */
int rbg_rskge3(int32_t layout, int32_t opA, int32_t opS, int64_t m, int64_t d, int64_t n,
               double alpha, const void *A, int64_t lda, const rbg_dense_skop *S,
               int64_t ro_s, int64_t co_s, double beta, void *B, int64_t ldb,
               rbg_stream_t stream);
/* Allocation-free variant of rbg_lskge3 -- no counterpart in the reference.  Same arguments
 * and result; it never allocates device memory (no cudaMalloc, cudaMallocAsync or
 * cudaFree), for callers that cannot: code capturing a CUDA graph with a fixed memory plan,
 * or hosts that forbid allocation after start-up.  Its split-K partial sums live in a fixed
 * 32 MiB device array inside the library, which every GPU that loads the library holds until
 * exit; d * n * sizeof(T) may be at most 16 MiB -- a limit that holds for every call, also
 * one whose split plan happens to need no scratch -- and larger sizes return
 * RBG_ERROR_INVALID_ARGUMENT.  The first call on a device looks up that array's address, so
 * make it before any stream capture.  All calls share the array: calls whose kernels can
 * overlap on the GPU race on it. */
int rbg_lskge3_noalloc(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n, int64_t m,
                       double alpha, const rbg_dense_skop *S, int64_t ro_s, int64_t co_s,
                       const void *A, int64_t lda, double beta, void *B, int64_t ldb,
                       rbg_stream_t stream);
/* sketch_vector (RandBLAS/skve.hh:140-164): y = alpha * op(submat(S)) * x + beta * y with
 * strides incx, incy (>= 1); submat(S) is d x m. */
int rbg_sketch_vector(int32_t opS, int64_t d, int64_t m, double alpha, const rbg_dense_skop *S,
                      int64_t ro_s, int64_t co_s, const void *x, int64_t incx, double beta,
                      void *y, int64_t incy, rbg_stream_t stream);

/* ------------------------------------------------------------------ sparse operators */

/* LSKGES / sketch_general left with a SparseSkOp (RandBLAS/skge.hh:465-492, 776-797).
 * An unsampled SASO (nnz < 0) is sampled inside the sketch and never written out. */
int rbg_lskges(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n, int64_t m,
               double alpha, const rbg_sparse_skop *S, int64_t ro_s, int64_t co_s,
               const void *A, int64_t lda, double beta, void *B, int64_t ldb,
               rbg_stream_t stream);
/* RSKGES / sketch_general right with a SparseSkOp (RandBLAS/skge.hh:598-626, 947-968).
 * The reference's rskges has no `return` after sampling an unsampled operator
 * (RandBLAS/skge.hh:616-620) and then fails; this call samples and applies once. */
int rbg_rskges(int32_t layout, int32_t opA, int32_t opS, int64_t m, int64_t d, int64_t n,
               double alpha, const void *A, int64_t lda, const rbg_sparse_skop *S,
               int64_t ro_s, int64_t co_s, double beta, void *B, int64_t ldb,
               rbg_stream_t stream);
/* sketch_vector with a SparseSkOp (RandBLAS/skve.hh:140-164). */
int rbg_sketch_vector_sparse(int32_t opS, int64_t d, int64_t m, double alpha,
                             const rbg_sparse_skop *S, int64_t ro_s, int64_t co_s,
                             const void *x, int64_t incx, double beta, void *y, int64_t incy,
                             rbg_stream_t stream);

/* ------------------------------------------------------------------ symmetric data */

/* require_symmetric (RandBLAS/util.hh:128-146): for i < j,
 * |A(i,j) - A(j,i)| <= (|A(i,j)| + |A(j,i)| + 1) * tol, in precision dtype; no check when
 * tol < 0.  The first failing pair in the reference's loop order is reported with the
 * reference's message ("Symmetry check failed. |A(i,j) - A(j,i)| was ..., which exceeds
 * tolerance of ...").  Synchronises `stream`. */
int rbg_require_symmetric(int32_t dtype, int32_t layout, const void *A, int64_t n, int64_t lda,
                          double tol, rbg_stream_t stream);
/* sketch_symmetric with a dense operator (RandBLAS/sksy.hh:158-529): A is n x n symmetric,
 * checked with sym_check_tol as above, then
 *   side 0:  B (d x n) = alpha * submat(S) * A + beta * B   (sksy.hh:293-311, 513-529),
 *   side 1:  B (n x d) = alpha * A * submat(S) + beta * B   (sksy.hh:158-176, 406-422). */
int rbg_sketch_symmetric(int32_t side, int32_t layout, int64_t d, int64_t n, double alpha,
                         const rbg_dense_skop *S, int64_t ro_s, int64_t co_s, const void *A,
                         int64_t lda, double beta, void *B, int64_t ldb, double sym_check_tol,
                         rbg_stream_t stream);
/* The same with a sparse operator. */
int rbg_sketch_symmetric_sparse(int32_t side, int32_t layout, int64_t d, int64_t n, double alpha,
                                const rbg_sparse_skop *S, int64_t ro_s, int64_t co_s,
                                const void *A, int64_t lda, double beta, void *B, int64_t ldb,
                                double sym_check_tol, rbg_stream_t stream);

/* ------------------------------------------------------------------ sparse data */

/* LSKSP3 / sketch_sparse left (RandBLAS/sparse_data/sksp.hh:132-182, 418-437):
 *   B = alpha * op(submat(S)) * op(A) + beta * B with dense S and sparse A (m x n). */
int rbg_lsksp3(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n, int64_t m,
               double alpha, const rbg_dense_skop *S, int64_t ro_s, int64_t co_s,
               const rbg_spmat *A, double beta, void *B, int64_t ldb, rbg_stream_t stream);
/* RSKSP3 / sketch_sparse right (RandBLAS/sparse_data/sksp.hh:277-326, 520-539):
 *   B = alpha * op(A) * op(submat(S)) + beta * B with sparse A (op(A) m x n). */
int rbg_rsksp3(int32_t layout, int32_t opA, int32_t opS, int64_t m, int64_t d, int64_t n,
               double alpha, const rbg_spmat *A, const rbg_dense_skop *S, int64_t ro_s,
               int64_t co_s, double beta, void *B, int64_t ldb, rbg_stream_t stream);
/* left_spmm (RandBLAS/sparse_data/spmm_dispatch.hh:52-179):
 *   C = alpha * op(submat(A)) * op(B) + beta * C, sparse A, dense B; (ro_a, co_a) are only
 *   allowed for COO, as in the reference. */
int rbg_left_spmm(int32_t layout, int32_t opA, int32_t opB, int64_t d, int64_t n, int64_t m,
                  double alpha, const rbg_spmat *A, int64_t ro_a, int64_t co_a, const void *B,
                  int64_t ldb, double beta, void *C, int64_t ldc, rbg_stream_t stream);
/* right_spmm (RandBLAS/sparse_data/spmm_dispatch.hh:181-219):
 *   C = alpha * op(A) * op(submat(B)) + beta * C, dense A, sparse B. */
int rbg_right_spmm(int32_t layout, int32_t opA, int32_t opB, int64_t m, int64_t d, int64_t n,
                   double alpha, const void *A, int64_t lda, const rbg_spmat *B, int64_t ro_b,
                   int64_t co_b, double beta, void *C, int64_t ldc, rbg_stream_t stream);

/* ------------------------------------------------------------------ precision path */

/* Bytes of device workspace rbg_lskge3_lowp needs for these sizes. */
int rbg_lskge3_lowp_workspace(int32_t precision, int64_t d, int64_t n, int64_t m,
                              size_t *bytes);
/* Left dense sketch on the tensor cores (no reference counterpart; same semantics as
 * rbg_lskge3 with T = float): the entries of submat(S) are generated inside the kernel,
 * rounded to `precision`, multiplied with A rounded the same way, accumulated in FP32 in
 * tensor memory.  RBG_PREC_BF16: both operands BF16.  RBG_PREC_FP8_E4M3: S's entries enter
 * as e4m3 unscaled (|uniform| <= sqrt(3), Gaussians far below e4m3's 448); A is divided, per
 * column and per K slice of the work split, by the power-of-two scale that brings that tile's
 * largest magnitude to <= 448, and the epilogue multiplies the product back (exact).
 * workspace: buffer of rbg_lskge3_lowp_workspace bytes in device memory of the current GPU
 * (cudaMalloc on the device the call runs on; other devices' memory, managed memory and host
 * memory are rejected with RBG_ERROR_INVALID_ARGUMENT), or NULL to let the call allocate
 * (stream-ordered) and free it.  The call runs on one GPU, the current one: its buffers live
 * on that GPU (or in host memory as below).
 * A and B may be device memory or host memory the GPU can read (pinned/registered memory, or
 * any host memory where the device reports cudaDevAttrPageableMemoryAccess); B is then written
 * in place.  For BF16 with pinned A, K >= 2^18, op(A) row- or column-contiguous and no
 * workspace given, the call streams A: 2^16-row chunks (the last 2^16 rows in quarters) are
 * copied by the copy engine on a side stream while the call's stream converts and sketches the
 * previous chunk, so the transfer and the sketch overlap.  Otherwise the
 * conversion pass reads A over the host link.  Pageable memory on systems without that access
 * is rejected with RBG_ERROR_INVALID_ARGUMENT. */
int rbg_lskge3_lowp(int32_t precision, int32_t layout, int32_t opS, int32_t opA, int64_t d,
                    int64_t n, int64_t m, float alpha, const rbg_dense_skop *S, int64_t ro_s,
                    int64_t co_s, const float *A, int64_t lda, float beta, float *B,
                    int64_t ldb, void *workspace, size_t workspace_bytes, rbg_stream_t stream);

/* rbg_lskge3_lowp with A stored as `a_dtype` (RBG_F32 or RBG_BF16); no reference
 * counterpart.  BF16 data enters the tensor cores unchanged. */
int rbg_lskge3_lowp_ex(int32_t precision, int32_t a_dtype, int32_t layout, int32_t opS,
                       int32_t opA, int64_t d, int64_t n, int64_t m, float alpha,
                       const rbg_dense_skop *S, int64_t ro_s, int64_t co_s, const void *A,
                       int64_t lda, float beta, float *B, int64_t ldb, void *workspace,
                       size_t workspace_bytes, rbg_stream_t stream);

/* Device-side status of the precision path (no reference counterpart): RBG_SUCCESS, or
 * RBG_ERROR_TIMEOUT if a bounded wait inside a tensor-core kernel gave up since the last call
 * of this function.  Synchronises the device and clears the status. */
int rbg_lowp_status(int32_t *code);

/* ------------------------------------------------------------------ batching path */

/* One problem of a batch: B_i = alpha_i * submat(S_i) * A_i + beta_i * B_i (left sketch,
 * op = NoTrans) for a generated dense operator S_i with its own state. */
typedef struct rbg_batch_problem {
    int64_t d, n, m;
    rbg_dense_dist dist;
    rbg_state seed;
    int64_t ro_s, co_s;
    const float *A;
    int64_t lda;
    float *B;
    int64_t ldb;
    float alpha, beta;
    int32_t tile_config; /* 0: library's choice; else 1..rbg_batched_tile_configs() */
    int32_t reserved;
} rbg_batch_problem;

/* Sketch `count` independent problems (host array `problems`) in one persistent launch,
 * all in `layout`, T = float, stream-ordered (device memory for the work list comes from
 * cudaMallocAsync on `stream`).  tile_config: 0 = each problem's own tile_config; otherwise
 * one configuration for every problem.  Results do not depend on scheduling: K splits are
 * summed in split order. */
int rbg_lskge3_batched(int32_t layout, const rbg_batch_problem *problems, int64_t count,
                       int32_t tile_config, rbg_stream_t stream);
/* Number of tile configurations the batched kernel offers (ids 1..count). */
int rbg_batched_tile_configs(int32_t *count);
/* Output tile shape (rows x columns) of configuration `config`; columns 0 means a row block
 * over every column of the problem (its operator rows generated once per chunk of k and used
 * by each 128-column pass). */
int rbg_batched_tile_shape(int32_t config, int32_t *rows, int32_t *cols);

/* A reusable batch: validates the problems and uploads the work list once (synchronous);
 * rbg_batched_plan_execute then only zeroes the plan's counters and launches the persistent
 * kernel on `stream`, so it can be captured into a CUDA graph and replayed.  The problems'
 * A and B pointers are baked into the plan. */
typedef struct rbg_batched_plan_s *rbg_batched_plan;
int rbg_batched_plan_create(int32_t layout, const rbg_batch_problem *problems, int64_t count,
                            int32_t tile_config, rbg_batched_plan *plan);
int rbg_batched_plan_execute(rbg_batched_plan plan, rbg_stream_t stream);
/* Work items and device bytes of a plan (either pointer may be NULL). */
int rbg_batched_plan_info(rbg_batched_plan plan, int64_t *work_items, int64_t *device_bytes);
/* Frees the plan (synchronous; no launch of it may be pending). */
int rbg_batched_plan_destroy(rbg_batched_plan plan);

#ifdef __cplusplus
}
#endif

#endif /* RANDBLAS_GB300_H */
