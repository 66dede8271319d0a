// rbg_internal.h -- host-side internals shared by the library's translation units:
// error reporting, argument checks and the kernel launchers each .cu file provides.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <exception>
#include <new>
#include <string>

#include "randblas_gb300.h"
#include "rbg_common.cuh"

namespace rbg {

// Thrown inside the library, caught at the C boundary and turned into a status code.
struct Failure {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const std::string &msg);
void set_last_error(const std::string &msg);

// randblas_require (RandBLAS/exceptions.hh:160-162): same message shape, with the name of
// the reference function whose check this is.
#define RBG_REQUIRE(fn, cond)                                                                  \
    do {                                                                                       \
        if (!(cond))                                                                           \
            ::rbg::fail(RBG_ERROR_INVALID_ARGUMENT,                                            \
                        std::string("(" #cond ") was required, but did not hold, in function ") \
                            + (fn));                                                           \
    } while (0)

// RBG_REQUIRE for a condition evaluated elsewhere (on the device, say): the same message with
// the reference's condition text.
inline void require_as(bool ok, const char *cond_text, const char *fn) {
    if (!ok)
        fail(RBG_ERROR_INVALID_ARGUMENT, std::string("(") + cond_text +
                                             ") was required, but did not hold, in function " + fn);
}

void cuda_check(cudaError_t e, const char *what);
#define RBG_CUDA(call) ::rbg::cuda_check((call), #call)

// Body of every extern "C" entry point: runs f and turns what it throws into a status code
// plus the thread-local message of rbg_last_error.
template <typename F>
int guarded(F &&f) {
    try {
        f();
        return RBG_SUCCESS;
    } catch (const Failure &e) {
        set_last_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc &) {
        set_last_error("host allocation failed");
        return RBG_ERROR_ALLOC;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return RBG_ERROR_INVALID_ARGUMENT;
    }
}

// Call right after each kernel launch of the library: checks the launch and counts it
// (rbg_kernel_launches).
void after_launch(const char *where);
#define RBG_LAUNCHED() ::rbg::after_launch(__func__)

// Optional per-kernel timing (rbg_profile_*): while enabled, a ProfScope records CUDA events
// on the launching stream around the kernel it wraps.
struct ProfScope {
    ProfScope(const char *name, cudaStream_t s);
    ~ProfScope() { finish(); }
    void finish();  // record the stop event now (idempotent)
    int slot = -1;
    cudaStream_t stream = nullptr;
};

// safe_int_product (RandBLAS/base.hh:260-274).
int64_t safe_mul(int64_t a, int64_t b);

inline cudaStream_t as_cuda(rbg_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

int num_sms();

// CTAs for a grid-stride loop over `work` items, `threads` per CTA: enough to cover the work,
// at most 16 per SM.
inline int grid_stride_ctas(int64_t work, int threads) {
    return (int)std::max<int64_t>(
        1, std::min<int64_t>((work + threads - 1) / threads, (int64_t)num_sms() * 16));
}

// Stream-ordered scratch that frees itself (cudaMallocAsync / cudaFreeAsync).
struct Scratch {
    void *ptr = nullptr;
    cudaStream_t stream = nullptr;
    Scratch() = default;
    Scratch(size_t bytes, cudaStream_t s) { alloc(bytes, s); }
    void alloc(size_t bytes, cudaStream_t s);  // frees any previous block first
    ~Scratch();
    Scratch(const Scratch &) = delete;
    Scratch &operator=(const Scratch &) = delete;
    template <typename T>
    T *as() const { return static_cast<T *>(ptr); }
};

// --------------------------------------------------------------- dense operator helpers
struct DenseInfo {
    int64_t dim_major, dim_minor;
    int natural_layout;
    double isometry_scale;
};
DenseInfo dense_info(const rbg_dense_dist &D);
DenseGen make_dense_gen(const rbg_dense_dist &D, const rbg_state &seed);

// --------------------------------------------------------------- fill kernels (fill.cu)
// Natural block R in [R0, R0+nr), C in [C0, C0+nc), written packed, row-major over (R, C)
// (transpose_out = 0) or over (C, R) (transpose_out = 1).
void launch_fill_dense(int dtype, const DenseGen &g, int64_t R0, int64_t C0, int64_t nr,
                       int64_t nc, int transpose_out, void *out, cudaStream_t s);
void launch_fill_saso(int dtype, int itype, const DevState &seed, int64_t vec_nnz,
                      int64_t dim_major, int64_t dim_minor, void *idx_major, void *idx_minor,
                      void *vals, cudaStream_t s);
// LASO into compacted COO; returns nnz (synchronises s).
int64_t launch_fill_laso(int dtype, int itype, const DevState &seed, int64_t vec_nnz,
                         int64_t dim_major, int64_t dim_minor, void *idx_long, void *idx_short,
                         void *vals, cudaStream_t s);
void launch_scale(int dtype, int64_t rows, int64_t cols, int64_t rs, int64_t cs, double beta,
                  void *X, cudaStream_t s);

// --------------------------------------------------------------- dense GEMM (gemm_simt.cu)
// Canonical left problem Out[M x N] = alpha * P[M x K] * Q[K x N] + beta * Out.
struct POperand {
    // generated: natural coordinates R = r0 + (r_on_i ? i : k), C = c0 + (r_on_i ? k : i)
    DenseGen gen;
    int64_t r0, c0;
    int r_on_i;
    // materialised: P(i, k) = buff[base + i * si + k * sk]
    const void *buff;
    int64_t base, si, sk;
};
struct Strided {
    const void *ptr;
    int64_t s0, s1;  // element (a, b) at ptr[a * s0 + b * s1]
};
void gemm_dense_sketch(int dtype, int64_t M, int64_t N, int64_t K, double alpha,
                       const POperand &P, const Strided &Q, double beta, void *out,
                       int64_t os_i, int64_t os_j, cudaStream_t s);

// Argument checks and operand set-up of a left dense sketch (LSKGE3 semantics) for the
// allocation-free entry point in gemm_simt.cu.  Returns false when there is nothing to
// compute (d == 0 or n == 0); throws Failure on invalid arguments.
struct DenseLeftProblem {
    int dtype;
    int64_t M, N, K;
    double alpha, beta;
    POperand P;
    Strided Q;
    void *out;
    int64_t os_i, os_j;
};
bool prepare_dense_left(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n,
                        int64_t m, double alpha, const rbg_dense_skop *S, int64_t ro_s,
                        int64_t co_s, const void *A, int64_t lda, double beta, void *B,
                        int64_t ldb, DenseLeftProblem *out);

// --------------------------------------------------------------- sparse sketch (spmm.cu)
// Sparse operand description for Out[M x N] = alpha * Sp[M x K] * Q[K x N] + beta * Out.
// rbg_set_deterministic: when on, every path sums in a fixed order (bitwise reproducible);
// when off (the default) the fused SASO sketch may add in a scheduling-dependent order.
bool deterministic_mode();

struct SparseOperand {
    enum Kind { SASO_GEN, COO, CSR, CSC } kind;
    // SASO_GEN: S generated in-kernel; Sp = op(submat(S)).
    DevState seed;
    int64_t vec_nnz, dim_major, dim_minor;
    int short_is_row;  // 1: S's short-axis (major) indices are row indices of S
    // COO / CSR / CSC arrays of the (full) sparse matrix X, with Sp = op(submat(X)).
    int dtype, itype;
    int64_t nnz, x_rows, x_cols;
    const void *vals, *idx_a, *idx_b;
    // op and submatrix offsets: Sp(i, k) = X(ro + i, co + k) or, when trans, X(ro + k, co + i)
    int trans;
    int64_t ro, co;
    // COO arrays of a filled SASO operator with all vec_nnz * dim_minor entries: fill_sparse
    // stores the entries of minor index i at [i * vec_nnz, (i + 1) * vec_nnz) (vec_nnz,
    // dim_major, dim_minor and short_is_row are then set as for SASO_GEN).  The arrays may
    // have been changed since; kernels that use this layout check it entry by entry.
    int saso_layout;
};
void spmm_sketch(int dtype, int64_t M, int64_t N, int64_t K, double alpha,
                 const SparseOperand &Sp, const Strided &Q, double beta, void *out,
                 int64_t os_i, int64_t os_j, cudaStream_t s);

// Out[M x N] = alpha * P[M x K] * X[K x N] + beta * Out for a generated operator P and sparse X
// given by its rows: row k's entries are idx[ptr[k] .. ptr[k + 1]) (column j) with values val
// (ptr, idx in itype; nnz bounds the entry arrays).  Nothing of P is materialised; sums are in
// a fixed order.  gen_spmm_applies: whether an output of N columns fits the kernel's tile.
bool gen_spmm_applies(int dtype, int64_t N);
void gen_spmm_sketch(int dtype, int itype, int64_t M, int64_t N, int64_t K, double alpha,
                     const POperand &P, const void *ptr, const void *idx, const void *val,
                     int64_t nnz, double beta, void *out, int64_t os_i, int64_t os_j,
                     cudaStream_t s);

}  // namespace rbg
