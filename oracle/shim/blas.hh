// Project-written stand-in for the BLAS++ surface the RandBLAS headers use
// (test infrastructure): the Layout/Op/Uplo/Diag/Side enums and gemm, scal, copy, axpy.
//
// gemm forwards to a CBLAS sgemm/dgemm whose addresses the loader installs at run time
// (OpenBLAS as bundled with numpy, 64-bit integer interface) through
// rbref_set_cblas(); when none is installed it runs a plain OpenMP triple loop.
#pragma once
// BLAS++'s header brings in these standard headers; the RandBLAS headers rely on them.
#include <algorithm>
#include <complex>
#include <cstdint>
#include <limits>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace blas {

enum class Layout : char { ColMajor = 'C', RowMajor = 'R' };
enum class Op : char { NoTrans = 'N', Trans = 'T', ConjTrans = 'C' };
enum class Uplo : char { Upper = 'U', Lower = 'L', General = 'G' };
enum class Diag : char { NonUnit = 'N', Unit = 'U' };
enum class Side : char { Left = 'L', Right = 'R' };

namespace shim {
// CBLAS (64-bit ints) function pointer types.
using sgemm_fn = void (*)(int, int, int, int64_t, int64_t, int64_t, float, const float *, int64_t,
                          const float *, int64_t, float, float *, int64_t);
using dgemm_fn = void (*)(int, int, int, int64_t, int64_t, int64_t, double, const double *,
                          int64_t, const double *, int64_t, double, double *, int64_t);
inline sgemm_fn &sgemm_ptr() { static sgemm_fn p = nullptr; return p; }
inline dgemm_fn &dgemm_ptr() { static dgemm_fn p = nullptr; return p; }

template <typename T>
void naive_gemm(Layout layout, Op opA, Op opB, int64_t m, int64_t n, int64_t k, T alpha,
                const T *A, int64_t lda, const T *B, int64_t ldb, T beta, T *C, int64_t ldc) {
    // C(i,j) at C[i*rs + j*cs]; op(A)(i,l) and op(B)(l,j) likewise.
    const bool col = layout == Layout::ColMajor;
    auto at = [&](const T *X, int64_t ld, bool trans, int64_t i, int64_t j) -> T {
        if (trans) { int64_t t = i; i = j; j = t; }
        return col ? X[i + j * ld] : X[i * ld + j];
    };
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t i = 0; i < m; ++i)
        for (int64_t j = 0; j < n; ++j) {
            T acc = 0;
            for (int64_t l = 0; l < k; ++l)
                acc += at(A, lda, opA != Op::NoTrans, i, l) * at(B, ldb, opB != Op::NoTrans, l, j);
            T &c = col ? C[i + j * ldc] : C[i * ldc + j];
            c = (beta == T(0)) ? alpha * acc : alpha * acc + beta * c;
        }
}
}  // namespace shim

template <typename T>
void gemm(Layout layout, Op opA, Op opB, int64_t m, int64_t n, int64_t k, T alpha, const T *A,
          int64_t lda, const T *B, int64_t ldb, T beta, T *C, int64_t ldc) {
    if (m == 0 || n == 0) return;
    const int order = layout == Layout::RowMajor ? 101 : 102;
    const int ta = opA == Op::NoTrans ? 111 : 112;
    const int tb = opB == Op::NoTrans ? 111 : 112;
    if constexpr (std::is_same_v<T, float>) {
        if (shim::sgemm_ptr()) {
            shim::sgemm_ptr()(order, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
            return;
        }
    } else if constexpr (std::is_same_v<T, double>) {
        if (shim::dgemm_ptr()) {
            shim::dgemm_ptr()(order, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
            return;
        }
    }
    shim::naive_gemm(layout, opA, opB, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

template <typename T>
void scal(int64_t n, T alpha, T *x, int64_t incx) {
    for (int64_t i = 0; i < n; ++i) x[i * incx] *= alpha;
}

template <typename T>
void copy(int64_t n, const T *x, int64_t incx, T *y, int64_t incy) {
    for (int64_t i = 0; i < n; ++i) y[i * incy] = x[i * incx];
}

template <typename T>
void axpy(int64_t n, T alpha, const T *x, int64_t incx, T *y, int64_t incy) {
    for (int64_t i = 0; i < n; ++i) y[i * incy] += alpha * x[i * incx];
}

}  // namespace blas
