// symmetric.cu -- sketch_symmetric (RandBLAS/sksy.hh:158-529): a symmetry check of A followed by
// sketch_general with A read as a general matrix.  The check follows require_symmetric
// (RandBLAS/util.hh:128-146): for i < j, |A(i,j) - A(j,i)| <= (|A(i,j)| + |A(j,i)| + 1) * tol,
// skipped when tol < 0; the first failing pair in the reference's loop order (i, then j) is
// reported with the reference's message.
#include <cinttypes>
#include <cstdio>

#include "rbg_internal.h"

namespace rbg {
namespace {

// Smallest linear index i * n + j (i < j) of a failing pair, by atomicMin (none: UINT64_MAX).
template <typename T>
__global__ void symmetry_kernel(const T *__restrict__ A, int64_t n, int64_t rs, int64_t cs, T tol,
                                unsigned long long *first) {
    const int64_t pairs = n * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < pairs;
         t += (int64_t)gridDim.x * blockDim.x) {
        // walk the matrix row by row; only the strict upper triangle is checked
        const int64_t i = t / n, j = t % n;
        if (j <= i) continue;
        const T aij = A[i * rs + j * cs], aji = A[j * rs + i * cs];
        const T viol = aij > aji ? aij - aji : aji - aij;
        const T rel = ((aij < 0 ? -aij : aij) + (aji < 0 ? -aji : aji) + (T)1) * tol;
        if (viol > rel) atomicMin(first, (unsigned long long)t);  // NaNs pass, as in the reference
    }
}

template <typename T>
void check_symmetric(int32_t layout, const void *Ap, int64_t n, int64_t lda, double tol_d,
                     cudaStream_t s) {
    if (tol_d < 0 || n <= 1) return;
    if (!Ap) fail(RBG_ERROR_INVALID_ARGUMENT, "A must not be NULL");
    const T *A = static_cast<const T *>(Ap);
    const int64_t rs = layout == RBG_ROW_MAJOR ? lda : 1, cs = layout == RBG_ROW_MAJOR ? 1 : lda;
    Scratch flag(sizeof(unsigned long long), s);
    RBG_CUDA(cudaMemsetAsync(flag.ptr, 0xFF, sizeof(unsigned long long), s));
    const int64_t work = n * n;
    const int grid = grid_stride_ctas(work, 256);
    symmetry_kernel<T><<<grid, 256, 0, s>>>(A, n, rs, cs, (T)tol_d, flag.as<unsigned long long>());
    RBG_LAUNCHED();
    unsigned long long first = 0;
    RBG_CUDA(cudaMemcpyAsync(&first, flag.ptr, sizeof first, cudaMemcpyDeviceToHost, s));
    RBG_CUDA(cudaStreamSynchronize(s));
    if (first == ~0ull) return;
    const int64_t i = (int64_t)(first / (unsigned long long)n), j = (int64_t)(first % n);
    T aij = 0, aji = 0;
    RBG_CUDA(cudaMemcpy(&aij, A + i * rs + j * cs, sizeof(T), cudaMemcpyDeviceToHost));
    RBG_CUDA(cudaMemcpy(&aji, A + j * rs + i * cs, sizeof(T), cudaMemcpyDeviceToHost));
    const double viol = aij > aji ? (double)(aij - aji) : (double)(aji - aij);
    const double rel = ((aij < 0 ? -(double)aij : (double)aij) +
                        (aji < 0 ? -(double)aji : (double)aji) + 1.0) * tol_d;
    char msg[256];
    std::snprintf(msg, sizeof msg,
                  "Symmetry check failed. |A(%" PRId64 ",%" PRId64 ") - A(%" PRId64 ",%" PRId64
                  ")| was %e, which exceeds tolerance of %e.",
                  i, j, j, i, viol, rel);
    fail(RBG_ERROR_INVALID_ARGUMENT, msg);
}

void require_symmetric_impl(int32_t dtype, int32_t layout, const void *A, int64_t n, int64_t lda,
                            double tol, cudaStream_t s) {
    if (layout != RBG_COL_MAJOR && layout != RBG_ROW_MAJOR)
        fail(RBG_ERROR_INVALID_ARGUMENT, "layout must be RBG_COL_MAJOR or RBG_ROW_MAJOR");
    if (dtype != RBG_F32 && dtype != RBG_F64)
        fail(RBG_ERROR_INVALID_ARGUMENT, "dtype must be RBG_F32 or RBG_F64");
    RBG_REQUIRE("require_symmetric", n >= 0 && lda >= n);
    if (dtype == RBG_F32)
        check_symmetric<float>(layout, A, n, lda, tol, s);
    else
        check_symmetric<double>(layout, A, n, lda, tol, s);
}

}  // namespace
}  // namespace rbg

using namespace rbg;

extern "C" int rbg_require_symmetric(int32_t dtype, int32_t layout, const void *A, int64_t n,
                                     int64_t lda, double tol, rbg_stream_t stream) {
    return guarded([&] { require_symmetric_impl(dtype, layout, A, n, lda, tol, as_cuda(stream)); });
}

extern "C" int rbg_sketch_symmetric(int32_t side, int32_t layout, int64_t d, int64_t n,
                                    double alpha, const rbg_dense_skop *S, int64_t ro_s,
                                    int64_t co_s, const void *A, int64_t lda, double beta,
                                    void *B, int64_t ldb, double sym_check_tol,
                                    rbg_stream_t stream) {
    if (!S) {
        set_last_error("S must not be NULL");
        return RBG_ERROR_INVALID_ARGUMENT;
    }
    if (side != 0 && side != 1) {
        set_last_error("side must be 0 (B = alpha S A + beta B) or 1 (B = alpha A S + beta B)");
        return RBG_ERROR_INVALID_ARGUMENT;
    }
    int rc = rbg_require_symmetric(S->dtype, layout, A, n, lda, sym_check_tol, stream);
    if (rc != RBG_SUCCESS) return rc;
    // sksy.hh:310-311 (left, d x n) and 175-176 (right, n x d)
    if (side == 0)
        return rbg_lskge3(layout, RBG_NO_TRANS, RBG_NO_TRANS, d, n, n, alpha, S, ro_s, co_s, A,
                          lda, beta, B, ldb, stream);
    return rbg_rskge3(layout, RBG_NO_TRANS, RBG_NO_TRANS, n, d, n, alpha, A, lda, S, ro_s, co_s,
                      beta, B, ldb, stream);
}

extern "C" int rbg_sketch_symmetric_sparse(int32_t side, int32_t layout, int64_t d, int64_t n,
                                           double alpha, const rbg_sparse_skop *S, int64_t ro_s,
                                           int64_t co_s, const void *A, int64_t lda,
                                           double beta, void *B, int64_t ldb,
                                           double sym_check_tol, rbg_stream_t stream) {
    if (!S) {
        set_last_error("S must not be NULL");
        return RBG_ERROR_INVALID_ARGUMENT;
    }
    if (side != 0 && side != 1) {
        set_last_error("side must be 0 (B = alpha S A + beta B) or 1 (B = alpha A S + beta B)");
        return RBG_ERROR_INVALID_ARGUMENT;
    }
    int rc = rbg_require_symmetric(S->dtype, layout, A, n, lda, sym_check_tol, stream);
    if (rc != RBG_SUCCESS) return rc;
    if (side == 0)
        return rbg_lskges(layout, RBG_NO_TRANS, RBG_NO_TRANS, d, n, n, alpha, S, ro_s, co_s, A,
                          lda, beta, B, ldb, stream);
    return rbg_rskges(layout, RBG_NO_TRANS, RBG_NO_TRANS, n, d, n, alpha, A, lda, S, ro_s, co_s,
                      beta, B, ldb, stream);
}
