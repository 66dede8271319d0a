// capi.cu -- the extern "C" boundary (include/randblas_gb300.h): argument checks with the
// reference's messages, operator bookkeeping (states, natural layouts, submatrix
// addressing) and dispatch to the kernels in fill.cu, gemm_simt.cu and spmm.cu.
#include <atomic>
#include <mutex>
#include <cmath>
#include <cstring>
#include <exception>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "rbg_internal.h"

namespace rbg {

namespace {
thread_local std::string g_last_error;
}

void set_last_error(const std::string &msg) { g_last_error = msg; }

[[noreturn]] void fail(int code, const std::string &msg) { throw Failure{code, msg}; }

void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        cudaGetLastError();  // clear a sticky launch error so later calls start clean
        fail(RBG_ERROR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

namespace {
std::atomic<unsigned long long> g_launches{0};
}

void after_launch(const char *where) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) fail(RBG_ERROR_CUDA, std::string("kernel launch in ") + where + ": " +
                                                   cudaGetErrorString(e));
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

namespace {
struct ProfTable {
    std::mutex mu;
    bool enabled = false;
    std::vector<std::string> names;
    std::vector<std::vector<std::pair<cudaEvent_t, cudaEvent_t>>> events;
};
ProfTable &prof() {
    static ProfTable t;
    return t;
}
}  // namespace

ProfScope::ProfScope(const char *name, cudaStream_t s) : stream(s) {
    ProfTable &t = prof();
    std::lock_guard<std::mutex> g(t.mu);
    if (!t.enabled) return;
    int idx = -1;
    for (size_t i = 0; i < t.names.size(); ++i)
        if (t.names[i] == name) idx = (int)i;
    if (idx < 0) {
        t.names.emplace_back(name);
        t.events.emplace_back();
        idx = (int)t.names.size() - 1;
    }
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) return;
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return;
    }
    cudaEventRecord(a, s);
    t.events[idx].emplace_back(a, b);
    slot = idx;
}

void ProfScope::finish() {
    if (slot < 0) return;
    ProfTable &t = prof();
    std::lock_guard<std::mutex> g(t.mu);
    if (slot < (int)t.events.size() && !t.events[slot].empty())
        cudaEventRecord(t.events[slot].back().second, stream);
    slot = -1;
}

int64_t safe_mul(int64_t a, int64_t b) {
    if (a == 0 || b == 0) return 0;
    int64_t c;
    if (__builtin_mul_overflow(a, b, &c)) {
        std::ostringstream s;
        s << "Overflow when multiplying a (=" << a << ") and b(=" << b << ").";
        fail(RBG_ERROR_OVERFLOW, s.str());
    }
    return c;
}

int num_sms() {
    static int cached[64] = {0};
    int dev = 0;
    RBG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) dev = 0;
    if (!cached[dev]) RBG_CUDA(cudaDeviceGetAttribute(&cached[dev], cudaDevAttrMultiProcessorCount, dev));
    return cached[dev];
}

void Scratch::alloc(size_t bytes, cudaStream_t s) {
    if (ptr) {
        cudaFreeAsync(ptr, stream);
        ptr = nullptr;
    }
    stream = s;
    if (bytes == 0) return;
    const cudaError_t e = cudaMallocAsync(&ptr, bytes, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ptr = nullptr;
        fail(RBG_ERROR_ALLOC, std::string("cudaMallocAsync of ") + std::to_string(bytes) +
                                  " bytes failed: " + cudaGetErrorString(e));
    }
}

Scratch::~Scratch() {
    if (ptr) cudaFreeAsync(ptr, stream);
}

DenseInfo dense_info(const rbg_dense_dist &D) {
    DenseInfo d{};
    const bool is_long = D.major_axis == RBG_AXIS_LONG;
    const int64_t mx = std::max(D.n_rows, D.n_cols), mn = std::min(D.n_rows, D.n_cols);
    d.dim_major = is_long ? mx : mn;
    d.dim_minor = is_long ? mn : mx;
    d.isometry_scale = std::pow((double)d.dim_minor, -0.5);
    // natural_layout (RandBLAS/dense_skops.hh:187-199)
    const bool wide = D.n_rows < D.n_cols;
    if (wide) d.natural_layout = is_long ? RBG_ROW_MAJOR : RBG_COL_MAJOR;
    else d.natural_layout = is_long ? RBG_COL_MAJOR : RBG_ROW_MAJOR;
    return d;
}

DenseGen make_dense_gen(const rbg_dense_dist &D, const rbg_state &seed) {
    const DenseInfo info = dense_info(D);
    DenseGen g{};
    const DevState s = to_dev(seed);
    g.ctr = s.ctr;
    g.key = s.key;
    g.stride = (info.dim_major + 3) / 4;
    g.family = D.family;
    g.natural_col = info.natural_layout == RBG_COL_MAJOR;
    return g;
}

}  // namespace rbg

using namespace rbg;

namespace {

void check_nonnull(const void *p, const char *what) {
    if (!p) fail(RBG_ERROR_INVALID_ARGUMENT, std::string(what) + " must not be NULL");
}

void check_layout(int32_t layout) {
    if (layout != RBG_COL_MAJOR && layout != RBG_ROW_MAJOR)
        fail(RBG_ERROR_INVALID_ARGUMENT, "layout must be RBG_COL_MAJOR or RBG_ROW_MAJOR");
}
void check_op(int32_t op) {
    if (op != RBG_NO_TRANS && op != RBG_TRANS)
        fail(RBG_ERROR_INVALID_ARGUMENT, "op must be RBG_NO_TRANS or RBG_TRANS");
}
void check_dtype(int32_t dtype) {
    if (dtype != RBG_F32 && dtype != RBG_F64)
        fail(RBG_ERROR_INVALID_ARGUMENT, "dtype must be RBG_F32 or RBG_F64");
}
void check_itype(int32_t itype) {
    if (itype != RBG_I32 && itype != RBG_I64)
        fail(RBG_ERROR_INVALID_ARGUMENT, "itype must be RBG_I32 or RBG_I64");
}

void validate_dense_dist(const rbg_dense_dist *D) {
    check_nonnull(D, "dist");
    RBG_REQUIRE("DenseDist", D->n_rows > 0);
    RBG_REQUIRE("DenseDist", D->n_cols > 0);
    if (D->family != RBG_GAUSSIAN && D->family != RBG_UNIFORM)
        fail(RBG_ERROR_INVALID_ARGUMENT, "Unrecognized distribution.");
    if (D->major_axis != RBG_AXIS_SHORT && D->major_axis != RBG_AXIS_LONG)
        fail(RBG_ERROR_INVALID_ARGUMENT, "major_axis must be RBG_AXIS_SHORT or RBG_AXIS_LONG");
}

struct SparseInfo {
    int64_t dim_major, dim_minor, full_nnz;
    double isometry_scale;
};

SparseInfo sparse_info(const rbg_sparse_dist *D) {
    check_nonnull(D, "dist");
    if (D->major_axis != RBG_AXIS_SHORT && D->major_axis != RBG_AXIS_LONG)
        fail(RBG_ERROR_INVALID_ARGUMENT, "major_axis must be RBG_AXIS_SHORT or RBG_AXIS_LONG");
    SparseInfo s{};
    const bool is_short = D->major_axis == RBG_AXIS_SHORT;
    s.dim_major = is_short ? std::min(D->n_rows, D->n_cols) : std::max(D->n_rows, D->n_cols);
    s.dim_minor = D->n_rows + D->n_cols - s.dim_major;
    // sparse::isometry_scale (RandBLAS/sparse_skops.hh:108-114)
    s.isometry_scale = is_short ? std::pow((double)D->vec_nnz, -0.5)
                                : std::sqrt((double)s.dim_major /
                                            ((double)D->vec_nnz * (double)s.dim_minor));
    RBG_REQUIRE("SparseDist", D->n_rows > 0);
    RBG_REQUIRE("SparseDist", D->n_cols > 0);
    RBG_REQUIRE("SparseDist", D->vec_nnz > 0);
    RBG_REQUIRE("SparseDist", D->vec_nnz <= s.dim_major);
    s.full_nnz = safe_mul(D->vec_nnz, s.dim_minor);
    return s;
}

rbg_state state_plus(const rbg_state &s, uint64_t n) {
    const uint4 c = ctr_add(make_uint4(s.counter[0], s.counter[1], s.counter[2], s.counter[3]), n);
    rbg_state out = s;
    out.counter[0] = c.x;
    out.counter[1] = c.y;
    out.counter[2] = c.z;
    out.counter[3] = c.w;
    return out;
}

rbg_state dense_next(const rbg_dense_dist &D, const rbg_state &seed) {
    const DenseInfo info = dense_info(D);
    const int64_t stride = (info.dim_major + 3) / 4;
    return state_plus(seed, (uint64_t)safe_mul(stride, info.dim_minor));
}

rbg_state sparse_next(const rbg_sparse_dist &D, const rbg_state &seed) {
    int64_t num_vec, per_vec;
    if (D.major_axis == RBG_AXIS_SHORT) {
        num_vec = std::max(D.n_rows, D.n_cols);
        per_vec = D.vec_nnz;
    } else {
        num_vec = std::min(D.n_rows, D.n_cols);
        per_vec = (D.vec_nnz + 1) / 2;
    }
    return state_plus(seed, (uint64_t)safe_mul(num_vec, per_vec));
}

struct Dims {
    int64_t rows, cols;
};
Dims dims_before_op(int64_t m, int64_t n, int32_t op) {
    return op == RBG_NO_TRANS ? Dims{m, n} : Dims{n, m};
}

// Element (x, y) of a matrix in `layout` with leading dimension ld sits at x*rs + y*cs.
struct Strides {
    int64_t rs, cs;
};
Strides strides_of(int32_t layout, int64_t ld) {
    return layout == RBG_COL_MAJOR ? Strides{1, ld} : Strides{ld, 1};
}

// fill_dense_unpacked, shared by the C entry points (RandBLAS/dense_skops.hh:563-606).
rbg_state fill_dense_impl(int32_t dtype, int32_t layout, const rbg_dense_dist &D, int64_t n_rows,
                          int64_t n_cols, int64_t ro_s, int64_t co_s, void *buff,
                          const rbg_state &seed, cudaStream_t s) {
    RBG_REQUIRE("fill_dense_unpacked", D.n_rows >= n_rows + ro_s);
    RBG_REQUIRE("fill_dense_unpacked", D.n_cols >= n_cols + co_s);
    RBG_REQUIRE("fill_dense_unpacked", ro_s >= 0 && co_s >= 0 && n_rows >= 0 && n_cols >= 0);
    const DenseInfo info = dense_info(D);
    const int64_t ma_len = info.dim_major;
    const int64_t stride = (ma_len + 3) / 4;
    int64_t nr, nc, R0, C0;
    if (info.natural_layout == RBG_COL_MAJOR) {  // generate the transpose in row-major
        nr = n_cols; nc = n_rows; R0 = co_s; C0 = ro_s;
    } else {
        nr = n_rows; nc = n_cols; R0 = ro_s; C0 = co_s;
    }
    safe_mul(R0, ma_len);
    const int64_t first_ctr = safe_mul(R0, stride) + C0 / 4;
    const int64_t next_off = first_ctr + safe_mul(nr, stride);
    if (nr > 0 && nc > 0) {
        check_nonnull(buff, "buff");
        const DenseGen g = make_dense_gen(D, seed);
        launch_fill_dense(dtype, g, R0, C0, nr, nc, layout != info.natural_layout, buff, s);
    }
    return state_plus(seed, (uint64_t)next_off);
}

// The P operand of the canonical GEMM for submat(S) at (ro_s, co_s):
// P(i, k) = S(ro_s + i, co_s + k), or S(ro_s + k, co_s + i) when eff_trans.
POperand make_p(const rbg_dense_skop &S, int eff_trans, int64_t ro_s, int64_t co_s) {
    POperand P{};
    if (S.buff) {
        const Strides st = strides_of(S.layout, S.layout == RBG_COL_MAJOR ? S.dist.n_rows
                                                                          : S.dist.n_cols);
        P.buff = S.buff;
        P.base = ro_s * st.rs + co_s * st.cs;
        P.si = eff_trans ? st.cs : st.rs;
        P.sk = eff_trans ? st.rs : st.cs;
    } else {
        const DenseInfo info = dense_info(S.dist);
        P.gen = make_dense_gen(S.dist, S.seed_state);
        if (info.natural_layout == RBG_ROW_MAJOR) {
            P.r_on_i = !eff_trans;
            P.r0 = ro_s;
            P.c0 = co_s;
        } else {
            P.r_on_i = eff_trans;
            P.r0 = co_s;
            P.c0 = ro_s;
        }
        P.buff = nullptr;
    }
    return P;
}

void validate_dense_skop(const rbg_dense_skop *S) {
    check_nonnull(S, "S");
    validate_dense_dist(&S->dist);
    check_dtype(S->dtype);
    if (S->buff) check_layout(S->layout);
}

// Q(k, j) = op(A)(k, j) for A in `layout` with leading dim lda.
Strided q_of(const void *A, int32_t layout, int64_t lda, int32_t opA) {
    const Strides a = strides_of(layout, lda);
    return opA == RBG_NO_TRANS ? Strided{A, a.rs, a.cs} : Strided{A, a.cs, a.rs};
}
// Q(k, j) = op(A)(j, k).
Strided q_of_transposed(const void *A, int32_t layout, int64_t lda, int32_t opA) {
    const Strides a = strides_of(layout, lda);
    return opA == RBG_NO_TRANS ? Strided{A, a.cs, a.rs} : Strided{A, a.rs, a.cs};
}

void lskge3_impl(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n, int64_t m,
                 double alpha, const rbg_dense_skop *S, int64_t ro_s, int64_t co_s,
                 const void *A, int64_t lda, double beta, void *B, int64_t ldb, cudaStream_t s) {
    check_layout(layout);
    check_op(opS);
    check_op(opA);
    validate_dense_skop(S);
    const Dims sub = dims_before_op(d, m, opS);
    RBG_REQUIRE("lskge3", S->dist.n_rows >= sub.rows + ro_s);
    RBG_REQUIRE("lskge3", S->dist.n_cols >= sub.cols + co_s);
    RBG_REQUIRE("lskge3", ro_s >= 0 && co_s >= 0 && d >= 0 && n >= 0 && m >= 0);
    const Dims a = dims_before_op(m, n, opA);
    if (layout == RBG_COL_MAJOR) {
        RBG_REQUIRE("lskge3", lda >= a.rows);
        RBG_REQUIRE("lskge3", ldb >= d);
    } else {
        RBG_REQUIRE("lskge3", lda >= a.cols);
        RBG_REQUIRE("lskge3", ldb >= n);
    }
    if (d == 0 || n == 0) return;
    check_nonnull(B, "B");
    if (alpha != 0.0 && m > 0) check_nonnull(A, "A");
    const POperand P = make_p(*S, opS == RBG_TRANS, ro_s, co_s);
    const Strides b = strides_of(layout, ldb);
    gemm_dense_sketch(S->dtype, d, n, m, alpha, P, q_of(A, layout, lda, opA), beta, B, b.rs,
                      b.cs, s);
}

void rskge3_impl(int32_t layout, int32_t opA, int32_t opS, int64_t m, int64_t d, int64_t n,
                 double alpha, const void *A, int64_t lda, const rbg_dense_skop *S,
                 int64_t ro_s, int64_t co_s, double beta, void *B, int64_t ldb, cudaStream_t s) {
    check_layout(layout);
    check_op(opS);
    check_op(opA);
    validate_dense_skop(S);
    const Dims sub = dims_before_op(n, d, opS);
    RBG_REQUIRE("rskge3", S->dist.n_rows >= sub.rows + ro_s);
    RBG_REQUIRE("rskge3", S->dist.n_cols >= sub.cols + co_s);
    RBG_REQUIRE("rskge3", ro_s >= 0 && co_s >= 0 && d >= 0 && n >= 0 && m >= 0);
    const Dims a = dims_before_op(m, n, opA);
    if (layout == RBG_COL_MAJOR) {
        RBG_REQUIRE("rskge3", lda >= a.rows);
        RBG_REQUIRE("rskge3", ldb >= m);
    } else {
        RBG_REQUIRE("rskge3", lda >= a.cols);
        RBG_REQUIRE("rskge3", ldb >= d);
    }
    if (d == 0 || m == 0) return;
    check_nonnull(B, "B");
    if (alpha != 0.0 && n > 0) check_nonnull(A, "A");
    // B^T (d x m) = op(submat(S))^T * op(A)^T: P(i, k) = op(submat(S))(k, i).
    const POperand P = make_p(*S, opS == RBG_NO_TRANS, ro_s, co_s);
    const Strides b = strides_of(layout, ldb);
    gemm_dense_sketch(S->dtype, d, m, n, alpha, P, q_of_transposed(A, layout, lda, opA), beta, B,
                      b.cs, b.rs, s);
}

void validate_sparse_skop(const rbg_sparse_skop *S) {
    check_nonnull(S, "S");
    sparse_info(&S->dist);
    check_dtype(S->dtype);
    check_itype(S->itype);
}

// Sparse operand for op(submat(S)) or its transpose; samples unsampled operators as needed
// into `tmp` (kept alive by the caller).
SparseOperand sparse_operand_of(const rbg_sparse_skop &S, int trans, int64_t ro, int64_t co,
                                Scratch tmp[3], cudaStream_t s) {
    SparseOperand op{};
    op.trans = trans;
    op.ro = ro;
    op.co = co;
    op.dtype = S.dtype;
    op.itype = S.itype;
    op.x_rows = S.dist.n_rows;
    op.x_cols = S.dist.n_cols;
    const SparseInfo info = sparse_info(&S.dist);
    const int short_is_row = S.dist.n_rows <= S.dist.n_cols;
    if (S.nnz >= 0) {
        op.kind = SparseOperand::COO;
        op.nnz = S.nnz;
        op.vals = S.vals;
        op.idx_a = S.rows;
        op.idx_b = S.cols;
        if (S.nnz > 0) {
            check_nonnull(S.vals, "S.vals");
            check_nonnull(S.rows, "S.rows");
            check_nonnull(S.cols, "S.cols");
        }
        if (S.dist.major_axis == RBG_AXIS_SHORT && S.nnz > 0 && S.nnz == info.full_nnz) {
            op.saso_layout = 1;
            op.vec_nnz = S.dist.vec_nnz;
            op.dim_major = info.dim_major;
            op.dim_minor = info.dim_minor;
            op.short_is_row = short_is_row;
        }
        return op;
    }
    if (S.dist.major_axis == RBG_AXIS_SHORT && S.dist.vec_nnz <= 64) {
        op.kind = SparseOperand::SASO_GEN;
        op.seed = to_dev(S.seed_state);
        op.vec_nnz = S.dist.vec_nnz;
        op.dim_major = info.dim_major;
        op.dim_minor = info.dim_minor;
        op.short_is_row = short_is_row;
        return op;
    }
    // sample into temporaries (same semantics as fill_sparse on a shallow copy,
    // RandBLAS/skge.hh:483-487), 64-bit indices
    const size_t esz = S.dtype == RBG_F32 ? 4 : 8;
    tmp[0].alloc((size_t)info.full_nnz * esz, s);
    tmp[1].alloc((size_t)info.full_nnz * 8, s);
    tmp[2].alloc((size_t)info.full_nnz * 8, s);
    void *rows = tmp[1].ptr, *cols = tmp[2].ptr;
    void *idx_short = short_is_row ? rows : cols, *idx_long = short_is_row ? cols : rows;
    int64_t nnz;
    if (S.dist.major_axis == RBG_AXIS_SHORT) {
        launch_fill_saso(S.dtype, RBG_I64, to_dev(S.seed_state), S.dist.vec_nnz, info.dim_major,
                         info.dim_minor, idx_short, idx_long, tmp[0].ptr, s);
        nnz = info.full_nnz;
    } else {
        nnz = launch_fill_laso(S.dtype, RBG_I64, to_dev(S.seed_state), S.dist.vec_nnz,
                               info.dim_major, info.dim_minor, idx_long, idx_short, tmp[0].ptr, s);
    }
    op.kind = SparseOperand::COO;
    op.itype = RBG_I64;
    op.nnz = nnz;
    op.vals = tmp[0].ptr;
    op.idx_a = rows;
    op.idx_b = cols;
    return op;
}

void lskges_impl(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n, int64_t m,
                 double alpha, const rbg_sparse_skop *S, int64_t ro_s, int64_t co_s,
                 const void *A, int64_t lda, double beta, void *B, int64_t ldb, cudaStream_t s) {
    check_layout(layout);
    check_op(opS);
    check_op(opA);
    validate_sparse_skop(S);
    // left_spmm's checks (RandBLAS/sparse_data/spmm_dispatch.hh:73-135)
    const Dims sx = opS == RBG_NO_TRANS ? Dims{S->dist.n_rows, S->dist.n_cols}
                                        : Dims{S->dist.n_cols, S->dist.n_rows};
    RBG_REQUIRE("left_spmm", sx.rows >= d);
    RBG_REQUIRE("left_spmm", sx.cols >= m);
    RBG_REQUIRE("left_spmm", ro_s >= 0 && co_s >= 0 && d >= 0 && n >= 0 && m >= 0);
    const Dims a = dims_before_op(m, n, opA);
    if (layout == RBG_COL_MAJOR) {
        RBG_REQUIRE("left_spmm", lda >= a.rows);
        RBG_REQUIRE("left_spmm", ldb >= d);
    } else {
        RBG_REQUIRE("left_spmm", ldb >= n);
        RBG_REQUIRE("left_spmm", lda >= a.cols);
    }
    if (d == 0 || n == 0) return;
    check_nonnull(B, "B");
    const Strides b = strides_of(layout, ldb);
    if (alpha == 0.0 || m == 0) {
        launch_scale(S->dtype, d, n, b.rs, b.cs, beta, B, s);
        return;
    }
    check_nonnull(A, "A");
    Scratch tmp[3];
    const SparseOperand sp = sparse_operand_of(*S, opS == RBG_TRANS, ro_s, co_s, tmp, s);
    spmm_sketch(S->dtype, d, n, m, alpha, sp, q_of(A, layout, lda, opA), beta, B, b.rs, b.cs, s);
}

void rskges_impl(int32_t layout, int32_t opA, int32_t opS, int64_t m, int64_t d, int64_t n,
                 double alpha, const void *A, int64_t lda, const rbg_sparse_skop *S,
                 int64_t ro_s, int64_t co_s, double beta, void *B, int64_t ldb, cudaStream_t s) {
    check_layout(layout);
    check_op(opS);
    check_op(opA);
    validate_sparse_skop(S);
    // right_spmm reduces to left_spmm on op(submat(S))^T (RandBLAS/sparse_data/spmm_dispatch.hh:181-219)
    const Dims sx = opS == RBG_NO_TRANS ? Dims{S->dist.n_cols, S->dist.n_rows}
                                        : Dims{S->dist.n_rows, S->dist.n_cols};
    RBG_REQUIRE("left_spmm", sx.rows >= d);
    RBG_REQUIRE("left_spmm", sx.cols >= n);
    RBG_REQUIRE("left_spmm", ro_s >= 0 && co_s >= 0 && d >= 0 && n >= 0 && m >= 0);
    const Dims a = dims_before_op(m, n, opA);
    if (layout == RBG_COL_MAJOR) {
        RBG_REQUIRE("left_spmm", lda >= a.rows);
        RBG_REQUIRE("left_spmm", ldb >= m);
    } else {
        RBG_REQUIRE("left_spmm", lda >= a.cols);
        RBG_REQUIRE("left_spmm", ldb >= d);
    }
    if (d == 0 || m == 0) return;
    check_nonnull(B, "B");
    const Strides b = strides_of(layout, ldb);
    if (alpha == 0.0 || n == 0) {
        launch_scale(S->dtype, m, d, b.rs, b.cs, beta, B, s);
        return;
    }
    check_nonnull(A, "A");
    Scratch tmp[3];
    // Out(i, j) = B(j, i); Sp(i, k) = op(submat(S))(k, i)
    const SparseOperand sp = sparse_operand_of(*S, opS == RBG_NO_TRANS, ro_s, co_s, tmp, s);
    spmm_sketch(S->dtype, d, m, n, alpha, sp, q_of_transposed(A, layout, lda, opA), beta, B,
                b.cs, b.rs, s);
}

// ---------------------------------------------------------------- sparse data matrices
void validate_spmat(const rbg_spmat *A, int32_t dtype) {
    check_nonnull(A, "A");
    if (A->format != RBG_COO && A->format != RBG_CSR && A->format != RBG_CSC)
        fail(RBG_ERROR_INVALID_ARGUMENT, "format must be RBG_COO, RBG_CSR or RBG_CSC");
    check_dtype(A->dtype);
    check_itype(A->itype);
    if (A->dtype != dtype)
        fail(RBG_ERROR_INVALID_ARGUMENT, "sparse matrix and operator scalar types differ");
    RBG_REQUIRE("SparseMatrix", A->n_rows >= 0 && A->n_cols >= 0 && A->nnz >= 0);
    if (A->format != RBG_COO) check_nonnull(A->idx_a, "A.idx_a");
    if (A->nnz > 0) {
        check_nonnull(A->vals, "A.vals");
        check_nonnull(A->idx_b, "A.idx_b");
        if (A->format == RBG_COO) check_nonnull(A->idx_a, "A.idx_a");
    }
}

SparseOperand operand_of_spmat(const rbg_spmat &A, int trans, int64_t ro, int64_t co) {
    SparseOperand op{};
    op.kind = A.format == RBG_COO ? SparseOperand::COO
              : A.format == RBG_CSR ? SparseOperand::CSR
                                    : SparseOperand::CSC;
    op.dtype = A.dtype;
    op.itype = A.itype;
    op.nnz = A.nnz;
    op.x_rows = A.n_rows;
    op.x_cols = A.n_cols;
    op.vals = A.vals;
    op.idx_a = A.idx_a;
    op.idx_b = A.idx_b;
    op.trans = trans;
    op.ro = ro;
    op.co = co;
    return op;
}

// left_spmm checks on op(A) (d x m at (ro_a, co_a)): COO may be larger, CSR/CSC must match
// exactly with zero offsets (RandBLAS/sparse_data/spmm_dispatch.hh:99-107).  The reference
// applies a transposed A by recursing on A.transpose() with the offsets swapped
// (spmm_dispatch.hh:73-90), so its checks -- and their messages -- name the transposed
// matrix and offsets; these do the same.
void check_left_spmm_dims(const rbg_spmat &X, int32_t opA, int64_t d, int64_t m, int64_t ro,
                          int64_t co) {
    struct Shape {
        int64_t n_rows, n_cols;
    };
    const bool nt = opA == RBG_NO_TRANS;
    const Shape A = nt ? Shape{X.n_rows, X.n_cols} : Shape{X.n_cols, X.n_rows};
    const int64_t ro_a = nt ? ro : co, co_a = nt ? co : ro;
    RBG_REQUIRE("left_spmm", ro_a >= 0 && co_a >= 0);
    if (X.format == RBG_COO) {
        RBG_REQUIRE("left_spmm", A.n_rows >= d);
        RBG_REQUIRE("left_spmm", A.n_cols >= m);
    } else {
        RBG_REQUIRE("left_spmm", A.n_rows == d);
        RBG_REQUIRE("left_spmm", A.n_cols == m);
        RBG_REQUIRE("left_spmm", ro_a == 0);
        RBG_REQUIRE("left_spmm", co_a == 0);
    }
}

// left_spmm's leading-dimension checks (spmm_dispatch.hh:110-135), in its names: the dense
// operand B (op(B) m x n) and C (d x n), both read in `layout`.
void check_left_spmm_lds(int32_t layout, int32_t opB, int64_t d, int64_t n, int64_t m,
                         int64_t ldb, int64_t ldc) {
    const int64_t rows_B = opB == RBG_NO_TRANS ? m : n;
    const int64_t cols_B = opB == RBG_NO_TRANS ? n : m;
    if (layout == RBG_COL_MAJOR) {
        RBG_REQUIRE("left_spmm", ldb >= rows_B);
        RBG_REQUIRE("left_spmm", ldc >= d);
    } else {
        RBG_REQUIRE("left_spmm", ldc >= n);
        RBG_REQUIRE("left_spmm", ldb >= cols_B);
    }
}

void left_spmm_impl(int32_t layout, int32_t opA, int32_t opB, int64_t d, int64_t n, int64_t m,
                    double alpha, const rbg_spmat *A, int64_t ro_a, int64_t co_a, const void *B,
                    int64_t ldb, double beta, void *C, int64_t ldc, cudaStream_t s) {
    check_layout(layout);
    check_op(opA);
    check_op(opB);
    check_nonnull(A, "A");
    validate_spmat(A, A->dtype);
    check_left_spmm_dims(*A, opA, d, m, ro_a, co_a);
    check_left_spmm_lds(layout, opB, d, n, m, ldb, ldc);
    if (d == 0 || n == 0) return;
    check_nonnull(C, "C");
    const Strides c = strides_of(layout, ldc);
    if (alpha == 0.0 || m == 0) {
        launch_scale(A->dtype, d, n, c.rs, c.cs, beta, C, s);
        return;
    }
    check_nonnull(B, "B");
    spmm_sketch(A->dtype, d, n, m, alpha, operand_of_spmat(*A, opA == RBG_TRANS, ro_a, co_a),
                q_of(B, layout, ldb, opB), beta, C, c.rs, c.cs, s);
}

void right_spmm_impl(int32_t layout, int32_t opA, int32_t opB, int64_t m, int64_t d, int64_t n,
                     double alpha, const void *A, int64_t lda, const rbg_spmat *B, int64_t ro_b,
                     int64_t co_b, double beta, void *C, int64_t ldc, cudaStream_t s) {
    check_layout(layout);
    check_op(opA);
    check_op(opB);
    check_nonnull(B, "B");
    validate_spmat(B, B->dtype);
    // C^T = op(submat(B))^T op(A)^T: the reference's reduction to left_spmm with the layout
    // and B's op flipped (spmm_dispatch.hh:181-219), and its checks in that problem's names
    check_left_spmm_dims(*B, opB == RBG_NO_TRANS ? RBG_TRANS : RBG_NO_TRANS, d, n, ro_b, co_b);
    check_left_spmm_lds(layout == RBG_COL_MAJOR ? RBG_ROW_MAJOR : RBG_COL_MAJOR, opA, d, m, n,
                        lda, ldc);
    if (d == 0 || m == 0) return;
    check_nonnull(C, "C");
    const Strides c = strides_of(layout, ldc);
    if (alpha == 0.0 || n == 0) {
        launch_scale(B->dtype, m, d, c.rs, c.cs, beta, C, s);
        return;
    }
    check_nonnull(A, "A");
    spmm_sketch(B->dtype, d, m, n, alpha, operand_of_spmat(*B, opB == RBG_NO_TRANS, ro_b, co_b),
                q_of_transposed(A, layout, lda, opA), beta, C, c.cs, c.rs, s);
}

// Materialise submat(S) (rows x cols at (ro_s, co_s)) in S's natural layout, packed, unless
// S already holds a buffer.  Returns the strides of submat(S)(x, y) = base[x*rs + y*cs].
struct SubmatView {
    const void *base;
    Strides st;
};
SubmatView submat_view(const rbg_dense_skop &S, int64_t rows, int64_t cols, int64_t ro_s,
                       int64_t co_s, Scratch &tmp, cudaStream_t s) {
    const size_t esz = S.dtype == RBG_F32 ? 4 : 8;
    if (S.buff) {
        const Strides st = strides_of(S.layout, S.layout == RBG_COL_MAJOR ? S.dist.n_rows
                                                                          : S.dist.n_cols);
        const char *base = (const char *)S.buff + (ro_s * st.rs + co_s * st.cs) * (int64_t)esz;
        return SubmatView{base, st};
    }
    const int32_t nat = dense_info(S.dist).natural_layout;
    tmp.alloc((size_t)safe_mul(rows, cols) * esz, s);
    fill_dense_impl(S.dtype, nat, S.dist, rows, cols, ro_s, co_s, tmp.ptr, S.seed_state, s);
    return SubmatView{tmp.ptr, strides_of(nat, nat == RBG_COL_MAJOR ? rows : cols)};
}

void lsksp3_impl(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n, int64_t m,
                 double alpha, const rbg_dense_skop *S, int64_t ro_s, int64_t co_s,
                 const rbg_spmat *A, double beta, void *B, int64_t ldb, cudaStream_t s) {
    check_layout(layout);
    check_op(opS);
    check_op(opA);
    validate_dense_skop(S);
    validate_spmat(A, S->dtype);
    const Dims sub = dims_before_op(d, m, opS);
    const Dims asub = dims_before_op(m, n, opA);
    RBG_REQUIRE("lsksp3", A->n_rows >= asub.rows);
    RBG_REQUIRE("lsksp3", A->n_cols >= asub.cols);
    RBG_REQUIRE("lsksp3", S->dist.n_rows >= sub.rows + ro_s);
    RBG_REQUIRE("lsksp3", S->dist.n_cols >= sub.cols + co_s);
    RBG_REQUIRE("lsksp3", ro_s >= 0 && co_s >= 0 && d >= 0 && n >= 0 && m >= 0);
    if (layout == RBG_COL_MAJOR) RBG_REQUIRE("lsksp3", ldb >= d);
    else RBG_REQUIRE("lsksp3", ldb >= n);
    // B^T = op(A)^T op(submat(S))^T goes through left_spmm on op(A)^T (n x m)
    check_left_spmm_dims(*A, opA == RBG_NO_TRANS ? RBG_TRANS : RBG_NO_TRANS, n, m, 0, 0);
    if (d == 0 || n == 0) return;
    check_nonnull(B, "B");
    const Strides b = strides_of(layout, ldb);
    if (alpha == 0.0 || m == 0) {
        launch_scale(S->dtype, d, n, b.rs, b.cs, beta, B, s);
        return;
    }
    // a generated operator against CSR rows of op(A): generate and apply in one kernel
    const bool rows_of_opA = (A->format == RBG_CSR && opA == RBG_NO_TRANS) ||
                             (A->format == RBG_CSC && opA == RBG_TRANS);
    if (!S->buff && rows_of_opA && gen_spmm_applies(S->dtype, n)) {
        gen_spmm_sketch(S->dtype, A->itype, d, n, m, alpha,
                        make_p(*S, opS == RBG_TRANS, ro_s, co_s), A->idx_a, A->idx_b, A->vals,
                        A->nnz, beta, B, b.rs, b.cs, s);
        return;
    }
    Scratch tmp;
    const SubmatView sv = submat_view(*S, sub.rows, sub.cols, ro_s, co_s, tmp, s);
    // Q(k, j) = op(submat(S))(j, k)
    const Strided q = opS == RBG_NO_TRANS ? Strided{sv.base, sv.st.cs, sv.st.rs}
                                          : Strided{sv.base, sv.st.rs, sv.st.cs};
    spmm_sketch(S->dtype, n, d, m, alpha, operand_of_spmat(*A, opA == RBG_NO_TRANS, 0, 0), q,
                beta, B, b.cs, b.rs, s);
}

void rsksp3_impl(int32_t layout, int32_t opA, int32_t opS, int64_t m, int64_t d, int64_t n,
                 double alpha, const rbg_spmat *A, const rbg_dense_skop *S, int64_t ro_s,
                 int64_t co_s, double beta, void *B, int64_t ldb, cudaStream_t s) {
    check_layout(layout);
    check_op(opS);
    check_op(opA);
    validate_dense_skop(S);
    validate_spmat(A, S->dtype);
    const Dims sub = dims_before_op(n, d, opS);
    const Dims asub = dims_before_op(m, n, opA);
    RBG_REQUIRE("rsksp3", A->n_rows >= asub.rows);
    RBG_REQUIRE("rsksp3", A->n_cols >= asub.cols);
    RBG_REQUIRE("rsksp3", S->dist.n_rows >= sub.rows + ro_s);
    RBG_REQUIRE("rsksp3", S->dist.n_cols >= sub.cols + co_s);
    RBG_REQUIRE("rsksp3", ro_s >= 0 && co_s >= 0 && d >= 0 && n >= 0 && m >= 0);
    if (layout == RBG_COL_MAJOR) RBG_REQUIRE("rsksp3", ldb >= m);
    else RBG_REQUIRE("rsksp3", ldb >= d);
    check_left_spmm_dims(*A, opA, m, n, 0, 0);
    if (d == 0 || m == 0) return;
    check_nonnull(B, "B");
    const Strides b = strides_of(layout, ldb);
    if (alpha == 0.0 || n == 0) {
        launch_scale(S->dtype, m, d, b.rs, b.cs, beta, B, s);
        return;
    }
    // B^T = op(S)^T op(A)^T: a generated operator against the rows of op(A)^T (the columns of
    // op(A)) when they are stored directly
    const bool cols_of_opA = (A->format == RBG_CSC && opA == RBG_NO_TRANS) ||
                             (A->format == RBG_CSR && opA == RBG_TRANS);
    if (!S->buff && cols_of_opA && gen_spmm_applies(S->dtype, m)) {
        gen_spmm_sketch(S->dtype, A->itype, d, m, n, alpha,
                        make_p(*S, opS == RBG_NO_TRANS, ro_s, co_s), A->idx_a, A->idx_b, A->vals,
                        A->nnz, beta, B, b.cs, b.rs, s);
        return;
    }
    Scratch tmp;
    const SubmatView sv = submat_view(*S, sub.rows, sub.cols, ro_s, co_s, tmp, s);
    // Q(k, j) = op(submat(S))(k, j)
    const Strided q = opS == RBG_NO_TRANS ? Strided{sv.base, sv.st.rs, sv.st.cs}
                                          : Strided{sv.base, sv.st.cs, sv.st.rs};
    spmm_sketch(S->dtype, m, d, n, alpha, operand_of_spmat(*A, opA == RBG_TRANS, 0, 0), q, beta,
                B, b.rs, b.cs, s);
}

}  // namespace

namespace rbg {

bool prepare_dense_left(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n,
                        int64_t m, double alpha, const rbg_dense_skop *S, int64_t ro_s,
                        int64_t co_s, const void *A, int64_t lda, double beta, void *B,
                        int64_t ldb, DenseLeftProblem *out) {
    check_layout(layout);
    check_op(opS);
    check_op(opA);
    validate_dense_skop(S);
    const Dims sub = dims_before_op(d, m, opS);
    RBG_REQUIRE("lskge3", S->dist.n_rows >= sub.rows + ro_s);
    RBG_REQUIRE("lskge3", S->dist.n_cols >= sub.cols + co_s);
    RBG_REQUIRE("lskge3", ro_s >= 0 && co_s >= 0 && d >= 0 && n >= 0 && m >= 0);
    const Dims a = dims_before_op(m, n, opA);
    if (layout == RBG_COL_MAJOR) {
        RBG_REQUIRE("lskge3", lda >= a.rows);
        RBG_REQUIRE("lskge3", ldb >= d);
    } else {
        RBG_REQUIRE("lskge3", lda >= a.cols);
        RBG_REQUIRE("lskge3", ldb >= n);
    }
    if (d == 0 || n == 0) return false;
    check_nonnull(B, "B");
    if (alpha != 0.0 && m > 0) check_nonnull(A, "A");
    const Strides b = strides_of(layout, ldb);
    out->dtype = S->dtype;
    out->M = d;
    out->N = n;
    out->K = m;
    out->alpha = alpha;
    out->beta = beta;
    out->P = make_p(*S, opS == RBG_TRANS, ro_s, co_s);
    out->Q = q_of(A, layout, lda, opA);
    out->out = B;
    out->os_i = b.rs;
    out->os_j = b.cs;
    return true;
}

namespace {
std::atomic<int> g_deterministic{0};
}  // namespace

bool deterministic_mode() { return g_deterministic.load(std::memory_order_relaxed) != 0; }

}  // namespace rbg

extern "C" {

const char *rbg_last_error(void) { return g_last_error.c_str(); }

int rbg_set_deterministic(int on) {
    rbg::g_deterministic.store(on ? 1 : 0, std::memory_order_relaxed);
    return RBG_SUCCESS;
}

int rbg_get_deterministic(void) { return rbg::deterministic_mode() ? 1 : 0; }

int rbg_version(void) { return 10100; }

uint64_t rbg_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int rbg_profile_enable(int on) {
    return guarded([&] {
        ProfTable &t = prof();
        std::lock_guard<std::mutex> g(t.mu);
        for (auto &v : t.events)
            for (auto &p : v) {
                cudaEventDestroy(p.first);
                cudaEventDestroy(p.second);
            }
        t.names.clear();
        t.events.clear();
        t.enabled = on != 0;
    });
}

int rbg_profile_count(int32_t *count) {
    return guarded([&] {
        check_nonnull(count, "count");
        ProfTable &t = prof();
        std::lock_guard<std::mutex> g(t.mu);
        *count = (int32_t)t.names.size();
    });
}

int rbg_profile_entry(int32_t index, char *name, int32_t name_cap, double *total_ms,
                      int64_t *launches) {
    return guarded([&] {
        ProfTable &t = prof();
        std::lock_guard<std::mutex> g(t.mu);
        if (index < 0 || index >= (int32_t)t.names.size())
            fail(RBG_ERROR_INVALID_ARGUMENT, "profile index out of range");
        double ms = 0.0;
        for (auto &p : t.events[index]) {
            RBG_CUDA(cudaEventSynchronize(p.second));
            float x = 0.f;
            RBG_CUDA(cudaEventElapsedTime(&x, p.first, p.second));
            ms += x;
        }
        if (name && name_cap > 0) {
            std::strncpy(name, t.names[index].c_str(), (size_t)name_cap - 1);
            name[name_cap - 1] = 0;
        }
        if (total_ms) *total_ms = ms;
        if (launches) *launches = (int64_t)t.events[index].size();
    });
}

int rbg_state_from_key(uint64_t k, rbg_state *out) {
    return guarded([&] {
        check_nonnull(out, "out");
        std::memset(out, 0, sizeof *out);
        out->key[0] = (uint32_t)k;
        out->key[1] = (uint32_t)(k >> 32);
    });
}

int rbg_state_incr(const rbg_state *in, uint64_t n, rbg_state *out) {
    return guarded([&] {
        check_nonnull(in, "in");
        check_nonnull(out, "out");
        *out = state_plus(*in, n);
    });
}

int rbg_dense_dist_properties(const rbg_dense_dist *D, int64_t *dim_major, int64_t *dim_minor,
                              int32_t *natural_layout, double *isometry_scale) {
    return guarded([&] {
        validate_dense_dist(D);
        const DenseInfo info = dense_info(*D);
        if (dim_major) *dim_major = info.dim_major;
        if (dim_minor) *dim_minor = info.dim_minor;
        if (natural_layout) *natural_layout = info.natural_layout;
        if (isometry_scale) *isometry_scale = info.isometry_scale;
    });
}

int rbg_dense_next_state(const rbg_dense_dist *D, const rbg_state *seed, rbg_state *next) {
    return guarded([&] {
        validate_dense_dist(D);
        check_nonnull(seed, "seed");
        check_nonnull(next, "next");
        *next = dense_next(*D, *seed);
    });
}

int rbg_dense_skop_init(rbg_dense_skop *S, const rbg_dense_dist *D, const rbg_state *seed,
                        int32_t dtype) {
    return guarded([&] {
        check_nonnull(S, "S");
        validate_dense_dist(D);
        check_nonnull(seed, "seed");
        check_dtype(dtype);
        S->dist = *D;
        S->seed_state = *seed;
        S->next_state = dense_next(*D, *seed);
        S->dtype = dtype;
        S->layout = dense_info(*D).natural_layout;
        S->buff = nullptr;
    });
}

int rbg_sparse_dist_properties(const rbg_sparse_dist *D, int64_t *dim_major,
                               int64_t *dim_minor, int64_t *full_nnz, double *isometry_scale) {
    return guarded([&] {
        const SparseInfo info = sparse_info(D);
        if (dim_major) *dim_major = info.dim_major;
        if (dim_minor) *dim_minor = info.dim_minor;
        if (full_nnz) *full_nnz = info.full_nnz;
        if (isometry_scale) *isometry_scale = info.isometry_scale;
    });
}

int rbg_sparse_next_state(const rbg_sparse_dist *D, const rbg_state *seed, rbg_state *next) {
    return guarded([&] {
        sparse_info(D);
        check_nonnull(seed, "seed");
        check_nonnull(next, "next");
        *next = sparse_next(*D, *seed);
    });
}

int rbg_sparse_skop_init(rbg_sparse_skop *S, const rbg_sparse_dist *D, const rbg_state *seed,
                         int32_t dtype, int32_t itype) {
    return guarded([&] {
        check_nonnull(S, "S");
        sparse_info(D);
        check_nonnull(seed, "seed");
        check_dtype(dtype);
        check_itype(itype);
        S->dist = *D;
        S->seed_state = *seed;
        S->next_state = sparse_next(*D, *seed);
        S->nnz = -1;
        S->dtype = dtype;
        S->itype = itype;
        S->vals = S->rows = S->cols = nullptr;
    });
}

int rbg_fill_dense_unpacked(int32_t dtype, int32_t layout, const rbg_dense_dist *D,
                            int64_t n_rows, int64_t n_cols, int64_t ro_s, int64_t co_s,
                            void *buff, const rbg_state *seed, rbg_state *next,
                            rbg_stream_t stream) {
    return guarded([&] {
        check_dtype(dtype);
        check_layout(layout);
        validate_dense_dist(D);
        check_nonnull(seed, "seed");
        const rbg_state nx =
            fill_dense_impl(dtype, layout, *D, n_rows, n_cols, ro_s, co_s, buff, *seed,
                            as_cuda(stream));
        if (next) *next = nx;
    });
}

int rbg_fill_dense(int32_t dtype, const rbg_dense_dist *D, void *buff, const rbg_state *seed,
                   rbg_state *next, rbg_stream_t stream) {
    return guarded([&] {
        check_dtype(dtype);
        validate_dense_dist(D);
        check_nonnull(seed, "seed");
        const rbg_state nx = fill_dense_impl(dtype, dense_info(*D).natural_layout, *D, D->n_rows,
                                             D->n_cols, 0, 0, buff, *seed, as_cuda(stream));
        if (next) *next = nx;
    });
}

int rbg_fill_dense_skop(rbg_dense_skop *S, rbg_stream_t stream) {
    return guarded([&] {
        validate_dense_skop(S);
        RBG_REQUIRE("fill_dense", S->buff != nullptr);
        check_layout(S->layout);
        fill_dense_impl(S->dtype, S->layout, S->dist, S->dist.n_rows, S->dist.n_cols, 0, 0,
                        S->buff, S->seed_state, as_cuda(stream));
    });
}

int rbg_fill_sparse_unpacked_nosub(int32_t dtype, int32_t itype, const rbg_sparse_dist *D,
                                   int64_t *nnz, void *vals, void *rows, void *cols,
                                   const rbg_state *seed, rbg_state *next,
                                   rbg_stream_t stream) {
    return guarded([&] {
        check_dtype(dtype);
        check_itype(itype);
        const SparseInfo info = sparse_info(D);
        check_nonnull(nnz, "nnz");
        check_nonnull(seed, "seed");
        check_nonnull(vals, "vals");
        check_nonnull(rows, "rows");
        check_nonnull(cols, "cols");
        const bool short_is_row = D->n_rows <= D->n_cols;
        void *idx_short = short_is_row ? rows : cols;
        void *idx_long = short_is_row ? cols : rows;
        const cudaStream_t s = as_cuda(stream);
        if (D->major_axis == RBG_AXIS_SHORT) {
            launch_fill_saso(dtype, itype, to_dev(*seed), D->vec_nnz, info.dim_major,
                             info.dim_minor, idx_short, idx_long, vals, s);
            *nnz = info.full_nnz;
        } else {
            *nnz = launch_fill_laso(dtype, itype, to_dev(*seed), D->vec_nnz, info.dim_major,
                                    info.dim_minor, idx_long, idx_short, vals, s);
        }
        if (next) *next = sparse_next(*D, *seed);
    });
}

int rbg_fill_sparse(rbg_sparse_skop *S, rbg_stream_t stream) {
    return guarded([&] {
        validate_sparse_skop(S);
        RBG_REQUIRE("fill_sparse", S->rows != nullptr);
        RBG_REQUIRE("fill_sparse", S->cols != nullptr);
        RBG_REQUIRE("fill_sparse", S->vals != nullptr);
        const int rc = rbg_fill_sparse_unpacked_nosub(S->dtype, S->itype, &S->dist, &S->nnz,
                                                      S->vals, S->rows, S->cols, &S->seed_state,
                                                      nullptr, stream);
        if (rc) fail(rc, g_last_error);
    });
}

int rbg_repeated_fisher_yates(int64_t k, int64_t n, int64_t r, int64_t *samples,
                              const rbg_state *seed, rbg_state *next, rbg_stream_t stream) {
    return guarded([&] {
        check_nonnull(seed, "seed");
        if (k > n)
            fail(RBG_ERROR_INVALID_ARGUMENT,
                 "vec_nnz > dim_major was required, but did not hold, in function "
                 "repeated_fisher_yates");
        RBG_REQUIRE("repeated_fisher_yates", k >= 0 && n >= 0 && r >= 0);
        if (k > 0 && r > 0) {
            check_nonnull(samples, "samples");
            launch_fill_saso(RBG_F32, RBG_I64, to_dev(*seed), k, n, r, samples, nullptr, nullptr,
                             as_cuda(stream));
        }
        if (next) *next = state_plus(*seed, (uint64_t)safe_mul(r, k));
    });
}

int rbg_lskge3(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n, int64_t m,
               double alpha, const rbg_dense_skop *S, int64_t ro_s, int64_t co_s,
               const void *A, int64_t lda, double beta, void *B, int64_t ldb,
               rbg_stream_t stream) {
    return guarded([&] {
        lskge3_impl(layout, opS, opA, d, n, m, alpha, S, ro_s, co_s, A, lda, beta, B, ldb,
                    as_cuda(stream));
    });
}

int rbg_rskge3(int32_t layout, int32_t opA, int32_t opS, int64_t m, int64_t d, int64_t n,
               double alpha, const void *A, int64_t lda, const rbg_dense_skop *S,
               int64_t ro_s, int64_t co_s, double beta, void *B, int64_t ldb,
               rbg_stream_t stream) {
    return guarded([&] {
        rskge3_impl(layout, opA, opS, m, d, n, alpha, A, lda, S, ro_s, co_s, beta, B, ldb,
                    as_cuda(stream));
    });
}

int rbg_sketch_vector(int32_t opS, int64_t d, int64_t m, double alpha, const rbg_dense_skop *S,
                      int64_t ro_s, int64_t co_s, const void *x, int64_t incx, double beta,
                      void *y, int64_t incy, rbg_stream_t stream) {
    return guarded([&] {
        check_op(opS);
        // skve.hh:154-163: RowMajor, n = 1, lda = incx, ldb = incy
        const int64_t dd = opS == RBG_TRANS ? m : d;
        const int64_t mm = opS == RBG_TRANS ? d : m;
        lskge3_impl(RBG_ROW_MAJOR, opS, RBG_NO_TRANS, dd, 1, mm, alpha, S, ro_s, co_s, x, incx,
                    beta, y, incy, as_cuda(stream));
    });
}

int rbg_lskges(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n, int64_t m,
               double alpha, const rbg_sparse_skop *S, int64_t ro_s, int64_t co_s,
               const void *A, int64_t lda, double beta, void *B, int64_t ldb,
               rbg_stream_t stream) {
    return guarded([&] {
        lskges_impl(layout, opS, opA, d, n, m, alpha, S, ro_s, co_s, A, lda, beta, B, ldb,
                    as_cuda(stream));
    });
}

int rbg_rskges(int32_t layout, int32_t opA, int32_t opS, int64_t m, int64_t d, int64_t n,
               double alpha, const void *A, int64_t lda, const rbg_sparse_skop *S,
               int64_t ro_s, int64_t co_s, double beta, void *B, int64_t ldb,
               rbg_stream_t stream) {
    return guarded([&] {
        rskges_impl(layout, opA, opS, m, d, n, alpha, A, lda, S, ro_s, co_s, beta, B, ldb,
                    as_cuda(stream));
    });
}

int rbg_sketch_vector_sparse(int32_t opS, int64_t d, int64_t m, double alpha,
                             const rbg_sparse_skop *S, int64_t ro_s, int64_t co_s,
                             const void *x, int64_t incx, double beta, void *y, int64_t incy,
                             rbg_stream_t stream) {
    return guarded([&] {
        check_op(opS);
        const int64_t dd = opS == RBG_TRANS ? m : d;
        const int64_t mm = opS == RBG_TRANS ? d : m;
        lskges_impl(RBG_ROW_MAJOR, opS, RBG_NO_TRANS, dd, 1, mm, alpha, S, ro_s, co_s, x, incx,
                    beta, y, incy, as_cuda(stream));
    });
}

int rbg_lsksp3(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n, int64_t m,
               double alpha, const rbg_dense_skop *S, int64_t ro_s, int64_t co_s,
               const rbg_spmat *A, double beta, void *B, int64_t ldb, rbg_stream_t stream) {
    return guarded([&] {
        lsksp3_impl(layout, opS, opA, d, n, m, alpha, S, ro_s, co_s, A, beta, B, ldb,
                    as_cuda(stream));
    });
}

int rbg_rsksp3(int32_t layout, int32_t opA, int32_t opS, int64_t m, int64_t d, int64_t n,
               double alpha, const rbg_spmat *A, const rbg_dense_skop *S, int64_t ro_s,
               int64_t co_s, double beta, void *B, int64_t ldb, rbg_stream_t stream) {
    return guarded([&] {
        rsksp3_impl(layout, opA, opS, m, d, n, alpha, A, S, ro_s, co_s, beta, B, ldb,
                    as_cuda(stream));
    });
}

int rbg_left_spmm(int32_t layout, int32_t opA, int32_t opB, int64_t d, int64_t n, int64_t m,
                  double alpha, const rbg_spmat *A, int64_t ro_a, int64_t co_a, const void *B,
                  int64_t ldb, double beta, void *C, int64_t ldc, rbg_stream_t stream) {
    return guarded([&] {
        left_spmm_impl(layout, opA, opB, d, n, m, alpha, A, ro_a, co_a, B, ldb, beta, C, ldc,
                       as_cuda(stream));
    });
}

int rbg_right_spmm(int32_t layout, int32_t opA, int32_t opB, int64_t m, int64_t d, int64_t n,
                   double alpha, const void *A, int64_t lda, const rbg_spmat *B, int64_t ro_b,
                   int64_t co_b, double beta, void *C, int64_t ldc, rbg_stream_t stream) {
    return guarded([&] {
        right_spmm_impl(layout, opA, opB, m, d, n, alpha, A, lda, B, ro_b, co_b, beta, C, ldc,
                        as_cuda(stream));
    });
}

}  // extern "C"
