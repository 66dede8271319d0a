// randblas_gb300.hpp -- C++ front end of the GB300 sketching library, shaped like RandBLAS's own
// API so a RandBLAS caller can switch its device-memory code paths over by namespace:
//
//     #include <randblas_gb300.hpp>
//     namespace RB = RandBLAS_GB300;   // instead of RandBLAS, for device buffers
//     RB::DenseDist D(d, m);
//     RB::DenseSkOp<float> S(D, RB::RNGState(42));
//     RB::sketch_general(RB::Layout::RowMajor, RB::Op::NoTrans, RB::Op::NoTrans, d, n, m,
//                        1.0f, S, A_dev, n, 0.0f, B_dev, n);
//
// Types and functions mirror RandBLAS (RNGState base.hh:64-164, DenseDist dense_skops.hh:231-350,
// DenseSkOp 357-478, fill_dense 563-658, SparseDist sparse_skops.hh:131-246, SparseSkOp 289-450,
// fill_sparse 587-603, sketch_general skge.hh:756-1199, sketch_vector skve.hh:140-246,
// sketch_sparse sparse_data/sksp.hh:418-539, random_coo / random_csr / random_csc
// sparse_data/random_matrix.hh:135-355, sparse conversions sparse_data/base.hh:142-302).  Matrix and vector pointers are CUDA device
// pointers; every call is asynchronous on `stream` (default: the legacy default stream).
// Failed argument checks throw RandBLAS_GB300::Error carrying the reference's message text;
// size overflows throw std::overflow_error, as RandBLAS's safe_int_product does.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "randblas_gb300.h"

namespace RandBLAS_GB300 {

enum class Layout : int32_t { ColMajor = RBG_COL_MAJOR, RowMajor = RBG_ROW_MAJOR };
enum class Op : int32_t { NoTrans = RBG_NO_TRANS, Trans = RBG_TRANS };
enum class ScalarDist : int32_t { Gaussian = RBG_GAUSSIAN, Uniform = RBG_UNIFORM };
enum class Axis : int32_t { Short = RBG_AXIS_SHORT, Long = RBG_AXIS_LONG };

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

namespace detail {
inline void check(int rc) {
    if (rc == RBG_SUCCESS) return;
    const std::string msg = rbg_last_error();
    if (rc == RBG_ERROR_OVERFLOW) throw std::overflow_error(msg);
    throw Error(rc, msg);
}
template <typename T>
constexpr int32_t dtype() {
    static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value,
                  "T must be float or double");
    return std::is_same<T, float>::value ? RBG_F32 : RBG_F64;
}
template <typename I>
constexpr int32_t itype() {
    static_assert(std::is_same<I, int32_t>::value || std::is_same<I, int64_t>::value,
                  "sint_t must be int32_t or int64_t");
    return std::is_same<I, int32_t>::value ? RBG_I32 : RBG_I64;
}
}  // namespace detail

// RNGState<Philox4x32>: 128-bit counter, 64-bit key; RNGState(k) has counter 0 and key k.
struct RNGState {
    rbg_state s{};
    RNGState() = default;
    explicit RNGState(uint64_t k) { detail::check(rbg_state_from_key(k, &s)); }
    explicit RNGState(const rbg_state &raw) : s(raw) {}
    RNGState incr(uint64_t n) const {
        rbg_state out;
        detail::check(rbg_state_incr(&s, n, &out));
        return RNGState(out);
    }
    bool operator==(const RNGState &o) const {
        for (int i = 0; i < 4; ++i)
            if (s.counter[i] != o.s.counter[i]) return false;
        return s.key[0] == o.s.key[0] && s.key[1] == o.s.key[1];
    }
    bool operator!=(const RNGState &o) const { return !(*this == o); }
};

struct DenseDist {
    rbg_dense_dist d{};
    int64_t n_rows, n_cols, dim_major, dim_minor;
    ScalarDist family;
    Axis major_axis;
    Layout natural_layout;
    double isometry_scale;
    DenseDist(int64_t rows, int64_t cols, ScalarDist fam = ScalarDist::Gaussian,
              Axis axis = Axis::Long)
        : n_rows(rows), n_cols(cols), family(fam), major_axis(axis) {
        d.n_rows = rows;
        d.n_cols = cols;
        d.family = static_cast<int32_t>(fam);
        d.major_axis = static_cast<int32_t>(axis);
        int32_t nat = 0;
        detail::check(rbg_dense_dist_properties(&d, &dim_major, &dim_minor, &nat,
                                                &isometry_scale));
        natural_layout = static_cast<Layout>(nat);
    }
};

// dense::compute_next_state
inline RNGState compute_next_state(const DenseDist &D, const RNGState &seed) {
    rbg_state out;
    detail::check(rbg_dense_next_state(&D.d, &seed.s, &out));
    return RNGState(out);
}

template <typename T>
struct DenseSkOp {
    DenseDist dist;
    RNGState seed_state, next_state;
    int64_t n_rows, n_cols;
    Layout layout;
    T *buff = nullptr;  // device buffer once filled (fill_dense); the caller owns it
    DenseSkOp(const DenseDist &D, const RNGState &seed)
        : dist(D), seed_state(seed), next_state(compute_next_state(D, seed)),
          n_rows(D.n_rows), n_cols(D.n_cols), layout(D.natural_layout) {}
    rbg_dense_skop c() const {
        rbg_dense_skop s{};
        s.dist = dist.d;
        s.seed_state = seed_state.s;
        s.next_state = next_state.s;
        s.dtype = detail::dtype<T>();
        s.layout = static_cast<int32_t>(layout);
        s.buff = buff;
        return s;
    }
};

struct SparseDist {
    rbg_sparse_dist d{};
    int64_t n_rows, n_cols, vec_nnz, dim_major, dim_minor, full_nnz;
    Axis major_axis;
    double isometry_scale;
    SparseDist(int64_t rows, int64_t cols, int64_t nnz_per_vec = 4, Axis axis = Axis::Short)
        : n_rows(rows), n_cols(cols), vec_nnz(nnz_per_vec), major_axis(axis) {
        d.n_rows = rows;
        d.n_cols = cols;
        d.vec_nnz = nnz_per_vec;
        d.major_axis = static_cast<int32_t>(axis);
        detail::check(rbg_sparse_dist_properties(&d, &dim_major, &dim_minor, &full_nnz,
                                                 &isometry_scale));
    }
};

inline RNGState compute_next_state(const SparseDist &D, const RNGState &seed) {
    rbg_state out;
    detail::check(rbg_sparse_next_state(&D.d, &seed.s, &out));
    return RNGState(out);
}

template <typename T, typename sint_t = int64_t>
struct SparseSkOp {
    SparseDist dist;
    RNGState seed_state, next_state;
    int64_t n_rows, n_cols;
    int64_t nnz = -1;  // -1: not sampled (sketching samples in-kernel)
    T *vals = nullptr;  // device arrays of dist.full_nnz entries for fill_sparse
    sint_t *rows = nullptr;
    sint_t *cols = nullptr;
    SparseSkOp(const SparseDist &D, const RNGState &seed)
        : dist(D), seed_state(seed), next_state(compute_next_state(D, seed)),
          n_rows(D.n_rows), n_cols(D.n_cols) {}
    rbg_sparse_skop c() const {
        rbg_sparse_skop s{};
        s.dist = dist.d;
        s.seed_state = seed_state.s;
        s.next_state = next_state.s;
        s.nnz = nnz;
        s.dtype = detail::dtype<T>();
        s.itype = detail::itype<sint_t>();
        s.vals = vals;
        s.rows = rows;
        s.cols = cols;
        return s;
    }
};

// ------------------------------------------------------------------ sampling
template <typename T>
RNGState fill_dense_unpacked(Layout layout, const DenseDist &D, int64_t n_rows, int64_t n_cols,
                             int64_t ro_s, int64_t co_s, T *buff, const RNGState &seed,
                             rbg_stream_t stream = nullptr) {
    rbg_state next;
    detail::check(rbg_fill_dense_unpacked(detail::dtype<T>(), static_cast<int32_t>(layout), &D.d,
                                          n_rows, n_cols, ro_s, co_s, buff, &seed.s, &next,
                                          stream));
    return RNGState(next);
}

template <typename T>
RNGState fill_dense(const DenseDist &D, T *buff, const RNGState &seed,
                    rbg_stream_t stream = nullptr) {
    rbg_state next;
    detail::check(rbg_fill_dense(detail::dtype<T>(), &D.d, buff, &seed.s, &next, stream));
    return RNGState(next);
}

// fill_dense(S): S.buff must point at n_rows * n_cols device entries.
template <typename T>
void fill_dense(DenseSkOp<T> &S, rbg_stream_t stream = nullptr) {
    rbg_dense_skop c = S.c();
    detail::check(rbg_fill_dense_skop(&c, stream));
}

// fill_sparse(S): S.vals / rows / cols must point at dist.full_nnz device entries.
template <typename T, typename I>
void fill_sparse(SparseSkOp<T, I> &S, rbg_stream_t stream = nullptr) {
    rbg_sparse_skop c = S.c();
    detail::check(rbg_fill_sparse(&c, stream));
    S.nnz = c.nnz;
}

// ------------------------------------------------------------------ sketch_general
// Left, submatrix: B = alpha * op(submat(S)) * op(A) + beta * B.
template <typename T>
void sketch_general(Layout layout, Op opS, Op opA, int64_t d, int64_t n, int64_t m, T alpha,
                    const DenseSkOp<T> &S, int64_t ro_s, int64_t co_s, const T *A, int64_t lda,
                    T beta, T *B, int64_t ldb, rbg_stream_t stream = nullptr) {
    const rbg_dense_skop c = S.c();
    detail::check(rbg_lskge3(static_cast<int32_t>(layout), static_cast<int32_t>(opS),
                             static_cast<int32_t>(opA), d, n, m, alpha, &c, ro_s, co_s, A, lda,
                             beta, B, ldb, stream));
}
// Left, whole operator.
template <typename T>
void sketch_general(Layout layout, Op opS, Op opA, int64_t d, int64_t n, int64_t m, T alpha,
                    const DenseSkOp<T> &S, const T *A, int64_t lda, T beta, T *B, int64_t ldb,
                    rbg_stream_t stream = nullptr) {
    const int64_t rows = opS == Op::NoTrans ? d : m, cols = opS == Op::NoTrans ? m : d;
    if (S.n_rows != rows || S.n_cols != cols)
        throw Error(RBG_ERROR_INVALID_ARGUMENT,
                    "(S.n_rows == " + std::to_string(rows) + " && S.n_cols == " +
                        std::to_string(cols) + ") was required, but did not hold, in function " +
                        "sketch_general");
    sketch_general(layout, opS, opA, d, n, m, alpha, S, 0, 0, A, lda, beta, B, ldb, stream);
}
// Right, submatrix: B = alpha * op(A) * op(submat(S)) + beta * B.
template <typename T>
void sketch_general(Layout layout, Op opA, Op opS, int64_t m, int64_t d, int64_t n, T alpha,
                    const T *A, int64_t lda, const DenseSkOp<T> &S, int64_t ro_s, int64_t co_s,
                    T beta, T *B, int64_t ldb, rbg_stream_t stream = nullptr) {
    const rbg_dense_skop c = S.c();
    detail::check(rbg_rskge3(static_cast<int32_t>(layout), static_cast<int32_t>(opA),
                             static_cast<int32_t>(opS), m, d, n, alpha, A, lda, &c, ro_s, co_s,
                             beta, B, ldb, stream));
}
// Left with a sparse operator (sampled in-kernel when S.nnz < 0).
template <typename T, typename I>
void sketch_general(Layout layout, Op opS, Op opA, int64_t d, int64_t n, int64_t m, T alpha,
                    const SparseSkOp<T, I> &S, int64_t ro_s, int64_t co_s, const T *A,
                    int64_t lda, T beta, T *B, int64_t ldb, rbg_stream_t stream = nullptr) {
    const rbg_sparse_skop c = S.c();
    detail::check(rbg_lskges(static_cast<int32_t>(layout), static_cast<int32_t>(opS),
                             static_cast<int32_t>(opA), d, n, m, alpha, &c, ro_s, co_s, A, lda,
                             beta, B, ldb, stream));
}
// Right with a sparse operator.
template <typename T, typename I>
void sketch_general(Layout layout, Op opA, Op opS, int64_t m, int64_t d, int64_t n, T alpha,
                    const T *A, int64_t lda, const SparseSkOp<T, I> &S, int64_t ro_s,
                    int64_t co_s, T beta, T *B, int64_t ldb, rbg_stream_t stream = nullptr) {
    const rbg_sparse_skop c = S.c();
    detail::check(rbg_rskges(static_cast<int32_t>(layout), static_cast<int32_t>(opA),
                             static_cast<int32_t>(opS), m, d, n, alpha, A, lda, &c, ro_s, co_s,
                             beta, B, ldb, stream));
}

// sketch_vector: y = alpha * op(submat(S)) * x + beta * y.
template <typename T>
void sketch_vector(Op opS, int64_t d, int64_t m, T alpha, const DenseSkOp<T> &S, int64_t ro_s,
                   int64_t co_s, const T *x, int64_t incx, T beta, T *y, int64_t incy,
                   rbg_stream_t stream = nullptr) {
    const rbg_dense_skop c = S.c();
    detail::check(rbg_sketch_vector(static_cast<int32_t>(opS), d, m, alpha, &c, ro_s, co_s, x,
                                    incx, beta, y, incy, stream));
}

// ------------------------------------------------------------------ sketch_symmetric
// (sksy.hh:158-529) A is n x n symmetric, checked with sym_check_tol (no check when < 0).
// Left: B (d x n) = alpha * submat(S) * A + beta * B.
template <typename T>
void sketch_symmetric(Layout layout, int64_t d, int64_t n, T alpha, const DenseSkOp<T> &S,
                      int64_t ro_s, int64_t co_s, const T *A, int64_t lda, T beta, T *B,
                      int64_t ldb, T sym_check_tol = 0, rbg_stream_t stream = nullptr) {
    const rbg_dense_skop c = S.c();
    detail::check(rbg_sketch_symmetric(0, static_cast<int32_t>(layout), d, n, alpha, &c, ro_s,
                                       co_s, A, lda, beta, B, ldb, sym_check_tol, stream));
}
// Right: B (n x d) = alpha * A * submat(S) + beta * B.
template <typename T>
void sketch_symmetric(Layout layout, int64_t n, int64_t d, T alpha, const T *A, int64_t lda,
                      const DenseSkOp<T> &S, int64_t ro_s, int64_t co_s, T beta, T *B,
                      int64_t ldb, T sym_check_tol = 0, rbg_stream_t stream = nullptr) {
    const rbg_dense_skop c = S.c();
    detail::check(rbg_sketch_symmetric(1, static_cast<int32_t>(layout), d, n, alpha, &c, ro_s,
                                       co_s, A, lda, beta, B, ldb, sym_check_tol, stream));
}
// Whole operator, left and right.
template <typename T>
void sketch_symmetric(Layout layout, T alpha, const DenseSkOp<T> &S, const T *A, int64_t lda,
                      T beta, T *B, int64_t ldb, T sym_check_tol = 0,
                      rbg_stream_t stream = nullptr) {
    sketch_symmetric(layout, S.n_rows, S.n_cols, alpha, S, 0, 0, A, lda, beta, B, ldb,
                     sym_check_tol, stream);
}
template <typename T>
void sketch_symmetric(Layout layout, T alpha, const T *A, int64_t lda, const DenseSkOp<T> &S,
                      T beta, T *B, int64_t ldb, T sym_check_tol = 0,
                      rbg_stream_t stream = nullptr) {
    sketch_symmetric(layout, S.n_rows, S.n_cols, alpha, A, lda, S, 0, 0, beta, B, ldb,
                     sym_check_tol, stream);
}

// ------------------------------------------------------------------ sparse data conversions
// NonzeroSort (sparse_data/base.hh:108-117) and the conversion building blocks
// (sparse_data/base.hh:142-220, 278-302) on device arrays; each synchronises `stream`.
enum class NonzeroSort : int32_t { CSC = RBG_SORT_CSC, CSR = RBG_SORT_CSR, None = RBG_SORT_NONE };

template <typename I1, typename I2>
void compressed_ptr_to_sorted_idxs(int64_t num_comp, const I1 *ptr, int64_t len_idxs, I2 *idxs,
                                   rbg_stream_t stream = nullptr) {
    detail::check(rbg_compressed_ptr_to_sorted_idxs(num_comp, detail::itype<I1>(), ptr, len_idxs,
                                                    detail::itype<I2>(), idxs, stream));
}
template <typename I1, typename I2>
void sorted_idxs_to_compressed_ptr(int64_t len_idxs, const I1 *idxs, int64_t num_comp, I2 *ptr,
                                   rbg_stream_t stream = nullptr) {
    detail::check(rbg_sorted_idxs_to_compressed_ptr(len_idxs, detail::itype<I1>(), idxs,
                                                    num_comp, detail::itype<I2>(), ptr, stream));
}
template <typename I>
NonzeroSort coo_arrays_determine_sort(int64_t nnz, const I *rows, const I *cols,
                                      rbg_stream_t stream = nullptr) {
    int32_t s = RBG_SORT_NONE;
    detail::check(rbg_coo_determine_sort(detail::itype<I>(), nnz, rows, cols, &s, stream));
    return static_cast<NonzeroSort>(s);
}
template <typename T, typename I>
void coo_arrays_apply_sort(NonzeroSort s, int64_t nnz, T *vals, I *rows, I *cols,
                           rbg_stream_t stream = nullptr) {
    detail::check(rbg_coo_apply_sort(static_cast<int32_t>(s), detail::dtype<T>(),
                                     detail::itype<I>(), nnz, vals, rows, cols, stream));
}

// ------------------------------------------------------------------ random sparse matrices
// random_coo / random_csr / random_csc (sparse_data/random_matrix.hh:135-355).  The reference
// returns an owning host matrix.  Here the number of nonzeros is known only once the structure
// is drawn, so generation takes two steps:
// - construct: draws the structure on the GPU and synchronises `stream`;
// - fill: writes caller-allocated device arrays of nnz() entries, plus the
//   major dimension + 1 pointers of CSR / CSC.
enum class SparseFormat : int32_t { COO = RBG_COO, CSR = RBG_CSR, CSC = RBG_CSC };

class RandomSparse {
  public:
    RandomSparse(SparseFormat format, int64_t m, int64_t n, double density,
                 const RNGState &state, rbg_stream_t stream = nullptr) {
        detail::check(rbg_random_sparse_create(static_cast<int32_t>(format), m, n, density,
                                               &state.s, &h_, &nnz_, &next_.s, stream));
    }
    ~RandomSparse() {
        if (h_) rbg_random_sparse_destroy(h_);
    }
    RandomSparse(const RandomSparse &) = delete;
    RandomSparse &operator=(const RandomSparse &) = delete;
    int64_t nnz() const { return nnz_; }
    // the state random_csr & co. return beside the matrix
    const RNGState &next_state() const { return next_; }
    // COO: a = rows, b = cols (CSR order); CSR: a = rowptr, b = colidxs;
    // CSC: a = colptr, b = rowidxs.
    template <typename T, typename I>
    void fill(T *vals, I *a, I *b, rbg_stream_t stream = nullptr) const {
        detail::check(rbg_random_sparse_fill(h_, detail::dtype<T>(), detail::itype<I>(), vals, a,
                                             b, stream));
    }
    // skips near a rounding tie of the logarithm (0: the matrix is the reference's)
    int64_t near_ties() const {
        int64_t t = 0;
        detail::check(rbg_random_sparse_info(h_, &t, nullptr));
        return t;
    }

  private:
    rbg_random_sparse h_ = nullptr;
    int64_t nnz_ = 0;
    RNGState next_;
};

// ------------------------------------------------------------------ sparse data and SpMM
// Non-owning views of device arrays shaped like RandBLAS's expert constructors
// (sparse_data/coo_matrix.hh:177-193, csr_matrix.hh, csc_matrix.hh:158-167): zero-based
// indices, int32_t or int64_t.
namespace sparse_data {
template <typename T, typename sint_t = int64_t>
struct COOMatrix {
    using scalar_t = T;
    using index_t = sint_t;
    int64_t n_rows, n_cols, nnz;
    T *vals;
    sint_t *rows, *cols;
    COOMatrix(int64_t n_rows, int64_t n_cols, int64_t nnz, T *vals, sint_t *rows, sint_t *cols)
        : n_rows(n_rows), n_cols(n_cols), nnz(nnz), vals(vals), rows(rows), cols(cols) {}
    rbg_spmat c() const {
        return {RBG_COO, detail::dtype<T>(), detail::itype<sint_t>(), 0, n_rows, n_cols, nnz,
                vals, rows, cols};
    }
};
template <typename T, typename sint_t = int64_t>
struct CSRMatrix {
    using scalar_t = T;
    using index_t = sint_t;
    int64_t n_rows, n_cols, nnz;
    T *vals;
    sint_t *rowptr, *colidxs;
    CSRMatrix(int64_t n_rows, int64_t n_cols, int64_t nnz, T *vals, sint_t *rowptr,
              sint_t *colidxs)
        : n_rows(n_rows), n_cols(n_cols), nnz(nnz), vals(vals), rowptr(rowptr),
          colidxs(colidxs) {}
    rbg_spmat c() const {
        return {RBG_CSR, detail::dtype<T>(), detail::itype<sint_t>(), 0, n_rows, n_cols, nnz,
                vals, rowptr, colidxs};
    }
};
template <typename T, typename sint_t = int64_t>
struct CSCMatrix {
    using scalar_t = T;
    using index_t = sint_t;
    int64_t n_rows, n_cols, nnz;
    T *vals;
    sint_t *rowidxs, *colptr;
    CSCMatrix(int64_t n_rows, int64_t n_cols, int64_t nnz, T *vals, sint_t *rowidxs,
              sint_t *colptr)
        : n_rows(n_rows), n_cols(n_cols), nnz(nnz), vals(vals), rowidxs(rowidxs),
          colptr(colptr) {}
    rbg_spmat c() const {
        return {RBG_CSC, detail::dtype<T>(), detail::itype<sint_t>(), 0, n_rows, n_cols, nnz,
                vals, colptr, rowidxs};
    }
};

// left_spmm (sparse_data/spmm_dispatch.hh:52-179):
//   C (d x n) = alpha * op(submat(A)) * op(B) + beta * C; offsets only for COO data.
template <typename SpMat, typename T = typename SpMat::scalar_t>
void left_spmm(Layout layout, Op opA, Op opB, int64_t d, int64_t n, int64_t m, T alpha,
               const SpMat &A, int64_t ro_a, int64_t co_a, const T *B, int64_t ldb, T beta, T *C,
               int64_t ldc, rbg_stream_t stream = nullptr) {
    const rbg_spmat a = A.c();
    detail::check(rbg_left_spmm(static_cast<int32_t>(layout), static_cast<int32_t>(opA),
                                static_cast<int32_t>(opB), d, n, m, alpha, &a, ro_a, co_a, B, ldb,
                                beta, C, ldc, stream));
}
// right_spmm (sparse_data/spmm_dispatch.hh:181-219):
//   C (m x d) = alpha * op(A) * op(submat(B)) + beta * C.
template <typename SpMat, typename T = typename SpMat::scalar_t>
void right_spmm(Layout layout, Op opA, Op opB, int64_t m, int64_t d, int64_t n, T alpha,
                const T *A, int64_t lda, const SpMat &B, int64_t ro_b, int64_t co_b, T beta,
                T *C, int64_t ldc, rbg_stream_t stream = nullptr) {
    const rbg_spmat b = B.c();
    detail::check(rbg_right_spmm(static_cast<int32_t>(layout), static_cast<int32_t>(opA),
                                 static_cast<int32_t>(opB), m, d, n, alpha, A, lda, &b, ro_b,
                                 co_b, beta, C, ldc, stream));
}
}  // namespace sparse_data

using sparse_data::COOMatrix;
using sparse_data::CSCMatrix;
using sparse_data::CSRMatrix;

// spmm (spmm_dispatch.hh:298-302, 376-380): the sparse operand's position picks the side.
template <typename SpMat, typename T = typename SpMat::scalar_t>
void spmm(Layout layout, Op opA, Op opB, int64_t m, int64_t n, int64_t k, T alpha,
          const SpMat &A, const T *B, int64_t ldb, T beta, T *C, int64_t ldc,
          rbg_stream_t stream = nullptr) {
    sparse_data::left_spmm(layout, opA, opB, m, n, k, alpha, A, 0, 0, B, ldb, beta, C, ldc,
                           stream);
}
template <typename SpMat, typename T = typename SpMat::scalar_t>
void spmm(Layout layout, Op opA, Op opB, int64_t m, int64_t n, int64_t k, T alpha, const T *A,
          int64_t lda, const SpMat &B, T beta, T *C, int64_t ldc,
          rbg_stream_t stream = nullptr) {
    sparse_data::right_spmm(layout, opA, opB, m, n, k, alpha, A, lda, B, 0, 0, beta, C, ldc,
                            stream);
}

// sketch_sparse (sparse_data/sksp.hh:418-539): dense operator, sparse data.
// Left: B (d x n) = alpha * op(submat(S)) * op(A) + beta * B.
template <typename SpMat, typename T>
void sketch_sparse(Layout layout, Op opS, Op opA, int64_t d, int64_t n, int64_t m, T alpha,
                   const DenseSkOp<T> &S, int64_t ro_s, int64_t co_s, const SpMat &A, T beta,
                   T *B, int64_t ldb, rbg_stream_t stream = nullptr) {
    const rbg_dense_skop s = S.c();
    const rbg_spmat a = A.c();
    detail::check(rbg_lsksp3(static_cast<int32_t>(layout), static_cast<int32_t>(opS),
                             static_cast<int32_t>(opA), d, n, m, alpha, &s, ro_s, co_s, &a, beta,
                             B, ldb, stream));
}
// Right: B (m x d) = alpha * op(A) * op(submat(S)) + beta * B.
template <typename SpMat, typename T>
void sketch_sparse(Layout layout, Op opA, Op opS, int64_t m, int64_t d, int64_t n, T alpha,
                   const SpMat &A, const DenseSkOp<T> &S, int64_t ro_s, int64_t co_s, T beta,
                   T *B, int64_t ldb, rbg_stream_t stream = nullptr) {
    const rbg_dense_skop s = S.c();
    const rbg_spmat a = A.c();
    detail::check(rbg_rsksp3(static_cast<int32_t>(layout), static_cast<int32_t>(opA),
                             static_cast<int32_t>(opS), m, d, n, alpha, &a, &s, ro_s, co_s, beta,
                             B, ldb, stream));
}

// Process-wide reproducibility switch (no RandBLAS counterpart).
inline void set_deterministic(bool on) { detail::check(rbg_set_deterministic(on ? 1 : 0)); }

}  // namespace RandBLAS_GB300
