// ref_driver.cc -- C entry points over the reference's own, unmodified RandBLAS headers.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build.py, in the container that has
// the reference source tree, against the project-written stand-ins for Random123 and
// BLAS++ in oracle/shim/ (the two third-party header libraries RandBLAS needs and does
// not vendor).  The output goes to oracle/_ref/ and is used to (1) pin the C restatement
// in oracle/oracle.c and (2) generate the golden fixtures under tests/golden/.  Nothing in
// the product links or calls it.
//
// Each entry point calls the reference's public API:
//   rbref_fill_dense_unpacked ... RandBLAS::fill_dense_unpacked   (RandBLAS/dense_skops.hh:563)
//   rbref_dense_next_state ...... RandBLAS::DenseSkOp::next_state (RandBLAS/dense_skops.hh:441-453)
//   rbref_fill_sparse ........... RandBLAS::fill_sparse_unpacked_nosub (RandBLAS/sparse_skops.hh:515)
//   rbref_sparse_next_state ..... RandBLAS::SparseSkOp::next_state (RandBLAS/sparse_skops.hh:399-407)
//   rbref_sketch_dense .......... RandBLAS::sketch_general, DenseSkOp (RandBLAS/skge.hh:756-1199)
//   rbref_sketch_saso ........... RandBLAS::sketch_general, SparseSkOp (RandBLAS/skge.hh:776,948)
//   rbref_sketch_vector ......... RandBLAS::sketch_vector         (RandBLAS/skve.hh:140-164)
//   rbref_sketch_sparse ......... RandBLAS::sketch_sparse         (RandBLAS/sparse_data/sksp.hh:418-539)
//   rbref_left_spmm, rbref_right_spmm
//                                 RandBLAS::sparse_data::left_spmm / right_spmm
//                                 (RandBLAS/sparse_data/spmm_dispatch.hh:52-219)
//   rbref_compressed_ptr_to_sorted_idxs, rbref_sorted_idxs_to_compressed_ptr,
//   rbref_coo_determine_sort, rbref_coo_apply_sort
//                                 (RandBLAS/sparse_data/base.hh:142-220, 278-302)
//   rbref_random_sparse ......... random_coo / random_csr / random_csc
//                                 (RandBLAS/sparse_data/random_matrix.hh:135-355)
#include <RandBLAS.hh>

#include <cstdint>
#include <cstring>
#include <exception>
#include <string>

namespace {

using RNG = r123::Philox4x32;
using State = RandBLAS::RNGState<RNG>;

thread_local std::string g_err;

State make_state(const uint32_t ctr[4], const uint32_t key[2]) {
    State s;
    for (int i = 0; i < 4; ++i) s.counter.v[i] = ctr[i];
    for (int i = 0; i < 2; ++i) s.key.v[i] = key[i];
    return s;
}

void put_state(const State &s, uint32_t ctr[4], uint32_t key[2]) {
    for (int i = 0; i < 4; ++i) ctr[i] = s.counter.v[i];
    for (int i = 0; i < 2; ++i) key[i] = s.key.v[i];
}

blas::Layout lay(int x) { return x == 0 ? blas::Layout::ColMajor : blas::Layout::RowMajor; }
blas::Op op(int x) { return x == 0 ? blas::Op::NoTrans : blas::Op::Trans; }
RandBLAS::ScalarDist fam(int x) {
    return x == 0 ? RandBLAS::ScalarDist::Gaussian : RandBLAS::ScalarDist::Uniform;
}
RandBLAS::Axis axis(int x) { return x == 0 ? RandBLAS::Axis::Short : RandBLAS::Axis::Long; }

template <typename F>
int guarded(F &&f) {
    try {
        f();
        return 0;
    } catch (const RandBLAS::Error &e) {
        g_err = e.what();
        return 1;
    } catch (const std::overflow_error &e) {
        g_err = e.what();
        return 2;
    } catch (const std::exception &e) {
        g_err = e.what();
        return 3;
    }
}

template <typename T>
void sketch_dense_t(int side, int layout, int opS, int opA, int64_t d, int64_t n, int64_t m,
                    double alpha, int64_t D_rows, int64_t D_cols, int family, int major_axis,
                    const uint32_t ctr[4], const uint32_t key[2], int64_t ro_s, int64_t co_s,
                    const void *A, int64_t lda, double beta, void *B, int64_t ldb, int prefill) {
    RandBLAS::DenseDist D(D_rows, D_cols, fam(family), axis(major_axis));
    RandBLAS::DenseSkOp<T, RNG> S(D, make_state(ctr, key));
    if (prefill) RandBLAS::fill_dense(S);
    if (side == 0) {
        RandBLAS::sketch_general(lay(layout), op(opS), op(opA), d, n, m, (T)alpha, S, ro_s, co_s,
                                 (const T *)A, lda, (T)beta, (T *)B, ldb);
    } else {
        // right sketch: B (d x n here means m x d in the reference's argument names) --
        // callers pass (m, d, n) in the reference's order through (d, n, m).
        RandBLAS::sketch_general(lay(layout), op(opA), op(opS), d, n, m, (T)alpha, (const T *)A,
                                 lda, S, ro_s, co_s, (T)beta, (T *)B, ldb);
    }
}

template <typename T>
void sketch_saso_t(int side, int layout, int opS, int opA, int64_t d, int64_t n, int64_t m,
                   double alpha, int64_t D_rows, int64_t D_cols, int64_t vec_nnz, int major_axis,
                   const uint32_t ctr[4], const uint32_t key[2], int64_t ro_s, int64_t co_s,
                   const void *A, int64_t lda, double beta, void *B, int64_t ldb) {
    RandBLAS::SparseDist D(D_rows, D_cols, vec_nnz, axis(major_axis));
    RandBLAS::SparseSkOp<T, RNG> S(D, make_state(ctr, key));
    // The reference's rskges is missing a `return` after its fill-and-recurse branch
    // (RandBLAS/skge.hh:616-620); sampling the operator first exercises the intended path
    // on both sides.
    RandBLAS::fill_sparse(S);
    if (side == 0) {
        RandBLAS::sketch_general(lay(layout), op(opS), op(opA), d, n, m, (T)alpha, S, ro_s, co_s,
                                 (const T *)A, lda, (T)beta, (T *)B, ldb);
    } else {
        RandBLAS::sketch_general(lay(layout), op(opA), op(opS), d, n, m, (T)alpha, (const T *)A,
                                 lda, S, ro_s, co_s, (T)beta, (T *)B, ldb);
    }
}

}  // namespace

extern "C" {

const char *rbref_last_error() { return g_err.c_str(); }

// 0: Box-Muller with the host libm (default); 1: with the shared float-float functions.
void rbref_set_math(int mode) { r123::boxmuller_math_mode() = mode; }

void rbref_set_cblas(void *sgemm, void *dgemm) {
    blas::shim::sgemm_ptr() = (blas::shim::sgemm_fn)sgemm;
    blas::shim::dgemm_ptr() = (blas::shim::dgemm_fn)dgemm;
}

int rbref_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    RNG g;
    RNG::ctr_type c{};
    RNG::key_type k{};
    for (int i = 0; i < 4; ++i) c.v[i] = ctr[i];
    for (int i = 0; i < 2; ++i) k.v[i] = key[i];
    auto r = g(c, k);
    for (int i = 0; i < 4; ++i) out[i] = r.v[i];
    return 0;
}

int rbref_state_from_key(uint64_t k, uint32_t ctr[4], uint32_t key[2]) {
    State s(k);
    put_state(s, ctr, key);
    return 0;
}

int rbref_counter_incr(uint32_t ctr[4], uint64_t n) {
    State s;
    for (int i = 0; i < 4; ++i) s.counter.v[i] = ctr[i];
    s.counter.incr(n);
    for (int i = 0; i < 4; ++i) ctr[i] = s.counter.v[i];
    return 0;
}

int rbref_fill_dense_unpacked(int dtype, int layout, int64_t D_rows, int64_t D_cols, int family,
                              int major_axis, int64_t n_rows, int64_t n_cols, int64_t ro_s,
                              int64_t co_s, void *buff, const uint32_t ctr[4],
                              const uint32_t key[2], uint32_t next_ctr[4], uint32_t next_key[2]) {
    return guarded([&] {
        RandBLAS::DenseDist D(D_rows, D_cols, fam(family), axis(major_axis));
        State next;
        if (dtype == 0)
            next = RandBLAS::fill_dense_unpacked(lay(layout), D, n_rows, n_cols, ro_s, co_s,
                                                 (float *)buff, make_state(ctr, key));
        else
            next = RandBLAS::fill_dense_unpacked(lay(layout), D, n_rows, n_cols, ro_s, co_s,
                                                 (double *)buff, make_state(ctr, key));
        put_state(next, next_ctr, next_key);
    });
}

int rbref_dense_next_state(int64_t D_rows, int64_t D_cols, int family, int major_axis,
                           const uint32_t ctr[4], const uint32_t key[2], uint32_t next_ctr[4],
                           uint32_t next_key[2], int *natural_layout, int64_t *dim_major) {
    return guarded([&] {
        RandBLAS::DenseDist D(D_rows, D_cols, fam(family), axis(major_axis));
        RandBLAS::DenseSkOp<float, RNG> S(D, make_state(ctr, key));
        put_state(S.next_state, next_ctr, next_key);
        *natural_layout = D.natural_layout == blas::Layout::ColMajor ? 0 : 1;
        *dim_major = D.dim_major;
    });
}

int rbref_fill_sparse(int dtype, int itype, int64_t D_rows, int64_t D_cols, int64_t vec_nnz,
                      int major_axis, void *vals, void *rows, void *cols, int64_t *nnz,
                      const uint32_t ctr[4], const uint32_t key[2], uint32_t next_ctr[4],
                      uint32_t next_key[2]) {
    return guarded([&] {
        RandBLAS::SparseDist D(D_rows, D_cols, vec_nnz, axis(major_axis));
        State seed = make_state(ctr, key);
        State next;
        if (dtype == 0 && itype == 0)
            next = RandBLAS::fill_sparse_unpacked_nosub(D, *nnz, (float *)vals, (int32_t *)rows,
                                                        (int32_t *)cols, seed);
        else if (dtype == 0)
            next = RandBLAS::fill_sparse_unpacked_nosub(D, *nnz, (float *)vals, (int64_t *)rows,
                                                        (int64_t *)cols, seed);
        else if (itype == 0)
            next = RandBLAS::fill_sparse_unpacked_nosub(D, *nnz, (double *)vals, (int32_t *)rows,
                                                        (int32_t *)cols, seed);
        else
            next = RandBLAS::fill_sparse_unpacked_nosub(D, *nnz, (double *)vals, (int64_t *)rows,
                                                        (int64_t *)cols, seed);
        put_state(next, next_ctr, next_key);
    });
}

int rbref_sparse_next_state(int64_t D_rows, int64_t D_cols, int64_t vec_nnz, int major_axis,
                            const uint32_t ctr[4], const uint32_t key[2], uint32_t next_ctr[4],
                            uint32_t next_key[2]) {
    return guarded([&] {
        RandBLAS::SparseDist D(D_rows, D_cols, vec_nnz, axis(major_axis));
        RandBLAS::SparseSkOp<float, RNG> S(D, make_state(ctr, key));
        put_state(S.next_state, next_ctr, next_key);
    });
}

int rbref_repeated_fisher_yates(int64_t k, int64_t n, int64_t r, int64_t *samples,
                                const uint32_t ctr[4], const uint32_t key[2],
                                uint32_t next_ctr[4], uint32_t next_key[2]) {
    return guarded([&] {
        State next = RandBLAS::repeated_fisher_yates(k, n, r, samples, make_state(ctr, key));
        put_state(next, next_ctr, next_key);
    });
}

// side 0: sketch_general(layout, opS, opA, d, n, m, alpha, S, ro_s, co_s, A, lda, beta, B, ldb)
// side 1: sketch_general(layout, opA, opS, d, n, m, alpha, A, lda, S, ro_s, co_s, beta, B, ldb)
//         with (d, n, m) meaning the reference's (m, d, n) of the right-hand overload.
int rbref_sketch_dense(int dtype, int side, int layout, int opS, int opA, int64_t d, int64_t n,
                       int64_t m, double alpha, int64_t D_rows, int64_t D_cols, int family,
                       int major_axis, const uint32_t ctr[4], const uint32_t key[2], int64_t ro_s,
                       int64_t co_s, const void *A, int64_t lda, double beta, void *B,
                       int64_t ldb, int prefill) {
    return guarded([&] {
        if (dtype == 0)
            sketch_dense_t<float>(side, layout, opS, opA, d, n, m, alpha, D_rows, D_cols, family,
                                  major_axis, ctr, key, ro_s, co_s, A, lda, beta, B, ldb, prefill);
        else
            sketch_dense_t<double>(side, layout, opS, opA, d, n, m, alpha, D_rows, D_cols, family,
                                   major_axis, ctr, key, ro_s, co_s, A, lda, beta, B, ldb, prefill);
    });
}

int rbref_sketch_saso(int dtype, int side, int layout, int opS, int opA, int64_t d, int64_t n,
                      int64_t m, double alpha, int64_t D_rows, int64_t D_cols, int64_t vec_nnz,
                      int major_axis, const uint32_t ctr[4], const uint32_t key[2], int64_t ro_s,
                      int64_t co_s, const void *A, int64_t lda, double beta, void *B,
                      int64_t ldb) {
    return guarded([&] {
        if (dtype == 0)
            sketch_saso_t<float>(side, layout, opS, opA, d, n, m, alpha, D_rows, D_cols, vec_nnz,
                                 major_axis, ctr, key, ro_s, co_s, A, lda, beta, B, ldb);
        else
            sketch_saso_t<double>(side, layout, opS, opA, d, n, m, alpha, D_rows, D_cols, vec_nnz,
                                  major_axis, ctr, key, ro_s, co_s, A, lda, beta, B, ldb);
    });
}

int rbref_sketch_vector(int dtype, int opS, int64_t d, int64_t m, double alpha, int64_t D_rows,
                        int64_t D_cols, int family, int major_axis, const uint32_t ctr[4],
                        const uint32_t key[2], int64_t ro_s, int64_t co_s, const void *x,
                        int64_t incx, double beta, void *y, int64_t incy) {
    return guarded([&] {
        RandBLAS::DenseDist D(D_rows, D_cols, fam(family), axis(major_axis));
        if (dtype == 0) {
            RandBLAS::DenseSkOp<float, RNG> S(D, make_state(ctr, key));
            RandBLAS::sketch_vector(op(opS), d, m, (float)alpha, S, ro_s, co_s, (const float *)x,
                                    incx, (float)beta, (float *)y, incy);
        } else {
            RandBLAS::DenseSkOp<double, RNG> S(D, make_state(ctr, key));
            RandBLAS::sketch_vector(op(opS), d, m, alpha, S, ro_s, co_s, (const double *)x, incx,
                                    beta, (double *)y, incy);
        }
    });
}

}  // extern "C"

// fmt: 0 = COO (a = rows, b = cols), 1 = CSR (a = rowptr, b = colidxs), 2 = CSC (a = colptr,
// b = rowidxs); int64 indices, zero-based.
template <typename T>
void sketch_sparse_t(int side, int layout, int opS, int opA, int64_t d, int64_t n, int64_t m,
                     double alpha, int64_t D_rows, int64_t D_cols, int family, int major_axis,
                     const uint32_t ctr[4], const uint32_t key[2], int64_t ro_s, int64_t co_s,
                     int fmt, int64_t A_rows, int64_t A_cols, int64_t nnz, void *vals, int64_t *a,
                     int64_t *b, double beta, void *B, int64_t ldb) {
    using namespace RandBLAS::sparse_data;
    RandBLAS::DenseDist D(D_rows, D_cols, fam(family), axis(major_axis));
    RandBLAS::DenseSkOp<T, RNG> S(D, make_state(ctr, key));
    auto run = [&](auto &Amat) {
        if (side == 0)
            RandBLAS::sketch_sparse(lay(layout), op(opS), op(opA), d, n, m, (T)alpha, S, ro_s,
                                    co_s, Amat, (T)beta, (T *)B, ldb);
        else
            RandBLAS::sketch_sparse(lay(layout), op(opA), op(opS), d, n, m, (T)alpha, Amat, S,
                                    ro_s, co_s, (T)beta, (T *)B, ldb);
    };
    if (fmt == 0) {
        COOMatrix<T, int64_t> Amat(A_rows, A_cols, nnz, (T *)vals, a, b);
        run(Amat);
    } else if (fmt == 1) {
        CSRMatrix<T, int64_t> Amat(A_rows, A_cols, nnz, (T *)vals, a, b);
        run(Amat);
    } else {
        CSCMatrix<T, int64_t> Amat(A_rows, A_cols, nnz, (T *)vals, b, a);
        run(Amat);
    }
}

extern "C" {

int rbref_sketch_sparse(int dtype, int side, int layout, int opS, int opA, int64_t d, int64_t n,
                        int64_t m, double alpha, int64_t D_rows, int64_t D_cols, int family,
                        int major_axis, const uint32_t ctr[4], const uint32_t key[2],
                        int64_t ro_s, int64_t co_s, int fmt, int64_t A_rows, int64_t A_cols,
                        int64_t nnz, void *vals, int64_t *a, int64_t *b, double beta, void *B,
                        int64_t ldb) {
    return guarded([&] {
        if (dtype == 0)
            sketch_sparse_t<float>(side, layout, opS, opA, d, n, m, alpha, D_rows, D_cols, family,
                                   major_axis, ctr, key, ro_s, co_s, fmt, A_rows, A_cols, nnz,
                                   vals, a, b, beta, B, ldb);
        else
            sketch_sparse_t<double>(side, layout, opS, opA, d, n, m, alpha, D_rows, D_cols,
                                    family, major_axis, ctr, key, ro_s, co_s, fmt, A_rows, A_cols,
                                    nnz, vals, a, b, beta, B, ldb);
    });
}

}  // extern "C"

// ------------------------------------------------------------- general sparse x dense
// Same sparse-matrix convention as sketch_sparse_t (fmt 0 COO, 1 CSR, 2 CSC; int64 indices).
template <typename T, typename F>
void with_spmat(int fmt, int64_t n_rows, int64_t n_cols, int64_t nnz, void *vals, int64_t *a,
                int64_t *b, F &&f) {
    using namespace RandBLAS::sparse_data;
    if (fmt == 0) {
        COOMatrix<T, int64_t> M(n_rows, n_cols, nnz, (T *)vals, a, b);
        f(M);
    } else if (fmt == 1) {
        CSRMatrix<T, int64_t> M(n_rows, n_cols, nnz, (T *)vals, a, b);
        f(M);
    } else {
        CSCMatrix<T, int64_t> M(n_rows, n_cols, nnz, (T *)vals, b, a);
        f(M);
    }
}

extern "C" {

// C = alpha * op(submat(A)) * op(B) + beta * C, A sparse (d x m after op), B dense.
int rbref_left_spmm(int dtype, int layout, int opA, int opB, int64_t d, int64_t n, int64_t m,
                    double alpha, int fmt, int64_t A_rows, int64_t A_cols, int64_t nnz,
                    void *vals, int64_t *a, int64_t *b, int64_t ro_a, int64_t co_a,
                    const void *B, int64_t ldb, double beta, void *C, int64_t ldc) {
    return guarded([&] {
        auto go = [&](auto tag) {
            using T = decltype(tag);
            with_spmat<T>(fmt, A_rows, A_cols, nnz, vals, a, b, [&](auto &A) {
                RandBLAS::sparse_data::left_spmm(lay(layout), op(opA), op(opB), d, n, m, (T)alpha,
                                                 A, ro_a, co_a, (const T *)B, ldb, (T)beta,
                                                 (T *)C, ldc);
            });
        };
        if (dtype == 0) go(float{});
        else go(double{});
    });
}

// C = alpha * op(A) * op(submat(B)) + beta * C, A dense (m x n after op), B sparse (n x d).
int rbref_right_spmm(int dtype, int layout, int opA, int opB, int64_t m, int64_t d, int64_t n,
                     double alpha, const void *A, int64_t lda, int fmt, int64_t B_rows,
                     int64_t B_cols, int64_t nnz, void *vals, int64_t *a, int64_t *b,
                     int64_t ro_b, int64_t co_b, double beta, void *C, int64_t ldc) {
    return guarded([&] {
        auto go = [&](auto tag) {
            using T = decltype(tag);
            with_spmat<T>(fmt, B_rows, B_cols, nnz, vals, a, b, [&](auto &B) {
                RandBLAS::sparse_data::right_spmm(lay(layout), op(opA), op(opB), m, d, n,
                                                  (T)alpha, (const T *)A, lda, B, ro_b, co_b,
                                                  (T)beta, (T *)C, ldc);
            });
        };
        if (dtype == 0) go(float{});
        else go(double{});
    });
}

}  // extern "C"

// ------------------------------------------------------------- random sparse matrices
#include <RandBLAS/sparse_data/random_matrix.hh>

namespace {

// Copies min(nnz, cap) entries (and the nmaj + 1 pointers of a compressed format) out of the
// reference's own random_coo / random_csr / random_csc; fmt as in rbref_sketch_sparse.
template <typename T, typename I>
int64_t random_sparse_t(int fmt, int64_t m, int64_t n, double density, const State &seed,
                        int64_t cap, void *vals, void *a, void *b, State &next) {
    using namespace RandBLAS::sparse_data;
    auto out = [&](const T *v, const I *ia, int64_t na, const I *ib, int64_t nnz) {
        const int64_t k = nnz < cap ? nnz : cap;
        if (k > 0) std::memcpy(vals, v, sizeof(T) * k);
        if (ia && na > 0) std::memcpy(a, ia, sizeof(I) * na);
        if (ib && k > 0) std::memcpy(b, ib, sizeof(I) * k);
    };
    if (fmt == 0) {
        auto [A, s] = random_coo<T, I>(m, n, density, seed);
        out(A.vals, A.rows, A.nnz < cap ? A.nnz : cap, A.cols, A.nnz);
        next = s;
        return A.nnz;
    }
    if (fmt == 1) {
        auto [A, s] = random_csr<T, I>(m, n, density, seed);
        out(A.vals, A.rowptr, m + 1, A.colidxs, A.nnz);
        next = s;
        return A.nnz;
    }
    auto [A, s] = random_csc<T, I>(m, n, density, seed);
    out(A.vals, A.colptr, n + 1, A.rowidxs, A.nnz);
    next = s;
    return A.nnz;
}

}  // namespace

extern "C" {

// random_coo / random_csr / random_csc (RandBLAS/sparse_data/random_matrix.hh:135-355).
int rbref_random_sparse(int fmt, int dtype, int itype, int64_t m, int64_t n, double density,
                        const uint32_t ctr[4], const uint32_t key[2], int64_t cap, void *vals,
                        void *a, void *b, int64_t *nnz, uint32_t next_ctr[4],
                        uint32_t next_key[2]) {
    return guarded([&] {
        const State seed = make_state(ctr, key);
        State next;
        if (dtype == 0 && itype == 0)
            *nnz = random_sparse_t<float, int32_t>(fmt, m, n, density, seed, cap, vals, a, b, next);
        else if (dtype == 0)
            *nnz = random_sparse_t<float, int64_t>(fmt, m, n, density, seed, cap, vals, a, b, next);
        else if (itype == 0)
            *nnz = random_sparse_t<double, int32_t>(fmt, m, n, density, seed, cap, vals, a, b, next);
        else
            *nnz = random_sparse_t<double, int64_t>(fmt, m, n, density, seed, cap, vals, a, b, next);
        put_state(next, next_ctr, next_key);
    });
}

}  // extern "C"

// ------------------------------------------------------------------ sparse conversions
namespace {

template <typename F>
int by_itype2(int it1, int it2, F &&f) {
    if (it1 == 0 && it2 == 0) f(int32_t{}, int32_t{});
    else if (it1 == 0) f(int32_t{}, int64_t{});
    else if (it2 == 0) f(int64_t{}, int32_t{});
    else f(int64_t{}, int64_t{});
    return 0;
}

char sort_char(RandBLAS::sparse_data::NonzeroSort s) {
    using RandBLAS::sparse_data::NonzeroSort;
    return s == NonzeroSort::CSC ? 'C' : s == NonzeroSort::CSR ? 'R' : 'N';
}

RandBLAS::sparse_data::NonzeroSort sort_of(int c) {
    using RandBLAS::sparse_data::NonzeroSort;
    return c == 'C' ? NonzeroSort::CSC : c == 'R' ? NonzeroSort::CSR : NonzeroSort::None;
}

}  // namespace

extern "C" {

// compressed_ptr_to_sorted_idxs (RandBLAS/sparse_data/base.hh:292-302)
int rbref_compressed_ptr_to_sorted_idxs(int64_t num_comp, int ptr_itype, void *ptr,
                                        int64_t len_idxs, int idx_itype, void *idxs) {
    return guarded([&] {
        by_itype2(ptr_itype, idx_itype, [&](auto p, auto q) {
            using P = decltype(p);
            using Q = decltype(q);
            RandBLAS::sparse_data::compressed_ptr_to_sorted_idxs(num_comp, (P *)ptr, len_idxs,
                                                                 (Q *)idxs);
        });
    });
}

// sorted_idxs_to_compressed_ptr (RandBLAS/sparse_data/base.hh:278-290)
int rbref_sorted_idxs_to_compressed_ptr(int64_t len_idxs, int idx_itype, const void *idxs,
                                        int64_t num_comp, int ptr_itype, void *ptr) {
    return guarded([&] {
        by_itype2(idx_itype, ptr_itype, [&](auto p, auto q) {
            using P = decltype(p);
            using Q = decltype(q);
            RandBLAS::sparse_data::sorted_idxs_to_compressed_ptr(len_idxs, (const P *)idxs,
                                                                 num_comp, (Q *)ptr);
        });
    });
}

// coo_arrays_determine_sort (RandBLAS/sparse_data/base.hh:142-167): 'C', 'R' or 'N'
int rbref_coo_determine_sort(int itype, int64_t nnz, void *rows, void *cols, int *sort) {
    return guarded([&] {
        if (itype == 0)
            *sort = sort_char(RandBLAS::sparse_data::coo_arrays_determine_sort(
                nnz, (int32_t *)rows, (int32_t *)cols));
        else
            *sort = sort_char(RandBLAS::sparse_data::coo_arrays_determine_sort(
                nnz, (int64_t *)rows, (int64_t *)cols));
    });
}

// coo_arrays_apply_sort (RandBLAS/sparse_data/base.hh:169-220)
int rbref_coo_apply_sort(int sort, int dtype, int itype, int64_t nnz, void *vals, void *rows,
                         void *cols) {
    return guarded([&] {
        const auto s = sort_of(sort);
        if (dtype == 0 && itype == 0)
            RandBLAS::sparse_data::coo_arrays_apply_sort(s, nnz, (float *)vals, (int32_t *)rows,
                                                         (int32_t *)cols);
        else if (dtype == 0)
            RandBLAS::sparse_data::coo_arrays_apply_sort(s, nnz, (float *)vals, (int64_t *)rows,
                                                         (int64_t *)cols);
        else if (itype == 0)
            RandBLAS::sparse_data::coo_arrays_apply_sort(s, nnz, (double *)vals,
                                                         (int32_t *)rows, (int32_t *)cols);
        else
            RandBLAS::sparse_data::coo_arrays_apply_sort(s, nnz, (double *)vals,
                                                         (int64_t *)rows, (int64_t *)cols);
    });
}

}  // extern "C"
