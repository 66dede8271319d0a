// spmm.cu -- sparse sketching and sparse-times-dense products:
//   LSKGES / RSKGES (RandBLAS/skge.hh:465-492, 598-626), left_spmm / right_spmm
//   (RandBLAS/sparse_data/spmm_dispatch.hh:52-219) and the SpMM inside LSKSP3 / RSKSP3.
//
// Canonical problem: Out[M x N] = alpha * Sp[M x K] * Q[K x N] + beta * Out with Sp sparse.
//
// 1. Row lists.  The nonzeros of Sp (after the submatrix filter and the transpose that
//    op() asks for) are sorted by (row, k) with a stable radix sort, giving CSR-like row
//    lists whose entries are in increasing k.  A SASO that has not been sampled is sampled
//    right here (Fisher-Yates per minor index, RandBLAS/sparse_skops.hh:51-106) and never
//    written out as COO.
// 2. SpMM.  A CTA owns 1024 output rows x 32 output columns x one K range.  It walks the K
//    range in blocks: the block of Q (KB x 32) is staged in shared memory once, then each
//    warp adds, for each of its 32 rows, the row's entries that fall in the block -- lane
//    = output column, accumulators in registers, entries in k order.  Each CTA writes a
//    partial result for its K range and a second kernel adds the ranges in a fixed order,
//    so results are deterministic.  Reads of Q are coalesced and happen once per CTA.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>

#include "rbg_internal.h"
#include "simt_tiles.cuh"
#include "tc_ptx.cuh"

namespace rbg {
namespace {

constexpr int kSliceCols = 32;
// Rows per warp: 32 accumulators per lane for float, 16 for double (register budget of a
// 1024-thread CTA).
template <typename T>
constexpr int rows_per_warp() { return sizeof(T) == 4 ? 32 : 16; }

int bits_for(uint64_t x) {  // bits needed to store values in [0, x]
    int b = 0;
    while (b < 64 && (x >> b) != 0) ++b;
    return std::max(b, 1);
}

// ------------------------------------------------------------------ entry extraction
// Writes one slot per potential nonzero: key = (row << kbits) | k (or row alone when the
// entries are known to arrive in increasing k per row); entries outside the submatrix get
// key M << kbits, which sorts after every valid key; kcol[slot] = k; val[slot] = value.
struct KeySpec {
    int64_t M, K, ro, co;
    int trans;
    int kbits;        // 0: key = row only
};

template <typename V>
__device__ __forceinline__ void emit(const KeySpec &ks, int64_t slot, int64_t x, int64_t y, V v,
                                     uint64_t *key, int32_t *kcol, V *val) {
    // Sp(i, k) = X(ro + i, co + k), or X(ro + k, co + i) when transposed.
    const int64_t i = ks.trans ? y - ks.co : x - ks.ro;
    const int64_t k = ks.trans ? x - ks.ro : y - ks.co;
    const bool ok = i >= 0 && i < ks.M && k >= 0 && k < ks.K;
    key[slot] = ok ? (((uint64_t)i << ks.kbits) | (ks.kbits ? (uint64_t)k : 0ull))
                   : ((uint64_t)ks.M << ks.kbits);
    kcol[slot] = ok ? (int32_t)k : 0;
    val[slot] = v;
}

// Generated SASO: same steps as the sampling kernel in fill.cu (vec_nnz Fisher-Yates steps
// per minor index, counter seed + i*vec_nnz + j), emitted straight into sort slots.
template <typename V>
__global__ void saso_entries_kernel(DevState s, int64_t vec_nnz, int64_t dim_major,
                                    int64_t dim_minor, int short_is_row, KeySpec ks,
                                    uint64_t *key, int32_t *kcol, V *val) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    int64_t mp[64], mv[64];  // vec_nnz <= 64 on this path (checked by the host)
    for (int64_t i = tid; i < dim_minor; i += nthreads) {
        int msize = 0;
        const int64_t off = i * vec_nnz;
        for (int64_t j = 0; j < vec_nnz; ++j) {
            const uint4 r = philox(ctr_add(s.ctr, (uint64_t)(off + j)), s.key);
            const int64_t ell = j + (int64_t)((uint64_t)r.x % (uint64_t)(dim_major - j));
            int64_t vj = j, vl = ell;
            int sj = -1, sl = -1;
            for (int q = 0; q < msize; ++q) {
                if (mp[q] == j) { vj = mv[q]; sj = q; }
                if (mp[q] == ell) { vl = mv[q]; sl = q; }
            }
            if (ell != j) {
                if (sl >= 0) {
                    mv[sl] = vj;
                } else {
                    mp[msize] = ell;
                    mv[msize] = vj;
                    ++msize;
                }
            }
            if (sj >= 0) {
                --msize;
                mp[sj] = mp[msize];
                mv[sj] = mv[msize];
            }
            const V v = (r.y % 2u == 0u) ? (V)1 : (V)-1;
            const int64_t x = short_is_row ? vl : i;
            const int64_t y = short_is_row ? i : vl;
            emit(ks, off + j, x, y, v, key, kcol, val);
        }
    }
}

template <typename V, typename I>
__global__ void coo_entries_kernel(int64_t nnz, const I *rows, const I *cols, const V *vals,
                                   KeySpec ks, uint64_t *key, int32_t *kcol, V *val) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz;
         e += (int64_t)gridDim.x * blockDim.x)
        emit(ks, e, (int64_t)rows[e], (int64_t)cols[e], vals[e], key, kcol, val);
}

// CSR (compressed over rows, by_rows = 1) or CSC (compressed over columns): one thread per
// compressed line.
template <typename V, typename I>
__global__ void compressed_entries_kernel(int64_t lines, const I *ptr, const I *idx,
                                          const V *vals, int by_rows, KeySpec ks, uint64_t *key,
                                          int32_t *kcol, V *val) {
    for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < lines;
         l += (int64_t)gridDim.x * blockDim.x) {
        for (int64_t e = (int64_t)ptr[l]; e < (int64_t)ptr[l + 1]; ++e) {
            const int64_t other = (int64_t)idx[e];
            emit(ks, e, by_rows ? l : other, by_rows ? other : l, vals[e], key, kcol, val);
        }
    }
}

template <typename V>
__global__ void gather_entries_kernel(int64_t n, const int32_t *perm, const int32_t *kcol_in,
                                      const V *val_in, int32_t *kcol_out, V *val_out) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t e = perm[p];
        kcol_out[p] = kcol_in[e];
        val_out[p] = val_in[e];
    }
}

__global__ void iota_kernel(int64_t n, int32_t *p) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        p[i] = (int32_t)i;
}

// rowptr[r] = first sorted position whose row is >= r, for r in [0, M]; entries outside the
// submatrix carry row M and sort last.
__global__ void rowptr_kernel(int64_t n, const uint64_t *skey, int kbits, int64_t M,
                              int64_t *rowptr) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p <= n;
         p += (int64_t)gridDim.x * blockDim.x) {
        auto row_of = [&](int64_t q) -> int64_t {
            if (q >= n) return M;
            return (int64_t)(skey[q] >> kbits);
        };
        const int64_t hi = row_of(p);
        const int64_t lo = p == 0 ? -1 : row_of(p - 1);
        for (int64_t r = lo + 1; r <= hi && r <= M; ++r) rowptr[r] = p;
    }
}

// ------------------------------------------------------------------ SpMM
template <typename T>
struct SpmmArgs {
    int64_t M, N, K;
    const int64_t *rowptr;
    const int32_t *kcol;
    const T *val;
    const T *Q;
    int64_t qs0, qs1;     // Q(k, c) = Q[k*qs0 + c*qs1]
    int64_t k_per_split;  // multiple of KB
    T *partial;           // [split][M][N], or nullptr when writing `out` directly
    T *out;
    int64_t os_i, os_j;
    T alpha, beta;
};

template <typename T, int KB>
__global__ void __launch_bounds__(1024, 1) spmm_rows_kernel(SpmmArgs<T> a) {
    constexpr int RPW = rows_per_warp<T>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T(*Qs)[kSliceCols + 1] = reinterpret_cast<T(*)[kSliceCols + 1]>(smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t c0 = (int64_t)blockIdx.x * kSliceCols;
    const int64_t row_base = (int64_t)blockIdx.y * (32 * RPW) + warp * RPW;
    const int64_t ka = (int64_t)blockIdx.z * a.k_per_split;
    const int64_t kz = min(a.K, ka + a.k_per_split);

    // lane l < RPW tracks row row_base + l: cursor = first entry with k >= block start
    const int64_t my_row = row_base + lane;
    int64_t cur = 0, end = 0;
    if (lane < RPW && my_row < a.M) {
        int64_t lo = a.rowptr[my_row], hi = a.rowptr[my_row + 1];
        end = hi;
        while (lo < hi) {  // lower_bound of ka
            const int64_t mid = (lo + hi) >> 1;
            if (a.kcol[mid] < ka) lo = mid + 1;
            else hi = mid;
        }
        cur = lo;
    }

    T acc[RPW];
#pragma unroll
    for (int r = 0; r < RPW; ++r) acc[r] = (T)0;
    const int64_t col = c0 + lane;
    const bool col_ok = col < a.N;

    for (int64_t kb = ka; kb < kz; kb += KB) {
        const int kn = (int)min((int64_t)KB, kz - kb);
        __syncthreads();
        if (a.qs1 == 1 || a.qs0 != 1) {
            for (int w = threadIdx.x; w < KB * kSliceCols; w += blockDim.x) {
                const int k = w / kSliceCols, c = w % kSliceCols;
                Qs[k][c] = (k < kn && c0 + c < a.N) ? a.Q[(kb + k) * a.qs0 + (c0 + c) * a.qs1]
                                                     : (T)0;
            }
        } else {
            for (int w = threadIdx.x; w < KB * kSliceCols; w += blockDim.x) {
                const int c = w / KB, k = w % KB;
                Qs[k][c] = (k < kn && c0 + c < a.N) ? a.Q[(kb + k) * a.qs0 + (c0 + c) * a.qs1]
                                                     : (T)0;
            }
        }
        __syncthreads();
        const int64_t kend = kb + kn;
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
            int64_t c = __shfl_sync(0xffffffffu, cur, r);
            const int64_t e = __shfl_sync(0xffffffffu, end, r);
            while (true) {
                const int64_t idx = c + lane;
                const bool valid = idx < e;
                const int32_t kk = valid ? a.kcol[idx] : INT32_MAX;
                const T vv = valid ? a.val[idx] : (T)0;
                const unsigned in_blk = __ballot_sync(0xffffffffu, valid && kk < kend);
                const int cnt = __popc(in_blk);  // entries are k-sorted: a prefix
                for (int t = 0; t < cnt; ++t) {
                    const int32_t kt = __shfl_sync(0xffffffffu, kk, t);
                    const T vt = __shfl_sync(0xffffffffu, vv, t);
                    const int64_t off = kt - kb;  // in [0, kn) for k-sorted lists
                    if ((uint64_t)off < (uint64_t)kn) acc[r] = fma(vt, Qs[off][lane], acc[r]);
                }
                c += cnt;
                if (cnt < 32) break;
            }
            if (lane == r) cur = c;
        }
    }

    if (!col_ok) return;
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
        const int64_t i = row_base + r;
        if (i >= a.M) break;
        if (a.partial) {
            a.partial[((int64_t)blockIdx.z * a.M + i) * a.N + col] = acc[r];
        } else {
            T &o = a.out[i * a.os_i + col * a.os_j];
            o = (a.beta == (T)0) ? a.alpha * acc[r] : fma(a.alpha, acc[r], a.beta * o);
        }
    }
}

template <typename T>
__global__ void spmm_reduce_kernel(int64_t M, int64_t N, int splits, const T *partial, T alpha,
                                   T beta, T *out, int64_t os_i, int64_t os_j) {
    const int64_t total = M * N;
    const bool j_fast = os_j <= os_i;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = j_fast ? t / N : t % M;
        const int64_t j = j_fast ? t % N : t / M;
        T sum = (T)0;
        for (int s = 0; s < splits; ++s) sum += partial[((int64_t)s * M + i) * N + j];
        T &o = out[i * os_i + j * os_j];
        o = (beta == (T)0) ? alpha * sum : fma(alpha, sum, beta * o);
    }
}

// ------------------------------------------------------------------ fused SASO scatter
// Left sketch by a SASO operator whose sparse vectors are the columns of S (short axis =
// columns, no transpose), the shape RandBLAS's LSKGES gives a wide SparseDist
// (RandBLAS/sparse_skops.hh:131-246, skge.hh:465-492):  B(r, :) += S(r, k) op(A)(k, :).
// Instead of building row lists, a pre-pass samples each column's vec_nnz (row, sign) pairs
// once into 32-bit words that are ready to use in the scatter: the byte offset of the row in
// the shared-memory B slice, with the sign in bit 31 (entries outside submat(S) point at a
// spare row past the slice).  Every CTA then keeps a d x 32 slice of B in shared memory and
// streams its share of A's rows exactly once, adding each row into the vec_nnz rows of the
// slice with shared-memory reductions (one mask, one add, one sign flip and the reduction per
// entry), and the chunks' slices are summed in chunk order.  Additions into one slice entry
// arrive in a scheduling-dependent order, so the last bits can vary between runs;
// rbg_set_deterministic(1) selects the row-list path instead.
#ifndef RBG_FUSED_THREADS
#define RBG_FUSED_THREADS 1024
#endif
constexpr int kFusedCols = 32;
constexpr int kFusedRowBytes = kFusedCols * 4;
constexpr int kFusedThreads = RBG_FUSED_THREADS;
constexpr int kFusedMaxNnz = 16;
constexpr uint32_t kSignBit = 0x80000000u;

// Column c of submat(S) (minor index co + c) as kp words (vec_nnz entries, then spare-row
// padding).
__global__ void saso_pack_kernel(DevState s, int vec_nnz, int kp, uint32_t dim_major,
                                 int64_t co, int64_t K, int64_t ro, int64_t M,
                                 uint32_t *__restrict__ packed) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    const uint32_t spare = (uint32_t)M * kFusedRowBytes;
    for (int64_t c = tid; c < K; c += nthreads) {
        uint32_t w[kFusedMaxNnz];
        saso_column(s, (uint64_t)(co + c), vec_nnz, dim_major,
                    [&](int j, uint32_t major, bool neg) {
                        const int64_t row = (int64_t)major - ro;
                        w[j] = (row >= 0 && row < M)
                                   ? ((uint32_t)row * kFusedRowBytes) | (neg ? kSignBit : 0u)
                                   : spare;
                    });
        for (int j = vec_nnz; j < kp; ++j) w[j] = spare;
        uint4 *dst = reinterpret_cast<uint4 *>(packed + c * kp);
        for (int q = 0; q < kp / 4; ++q)
            dst[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
    }
}

__device__ __forceinline__ void red_shared_add_bits(uint32_t addr, uint32_t bits) {
    asm volatile("red.shared.add.f32 [%0], %1;" ::"r"(addr), "f"(__uint_as_float(bits))
                 : "memory");
}

// staging buffer of saso_scatter_kernel<kp> (entry words of 32 rows per warp) and the
// largest dynamic shared memory the kernel may use
constexpr size_t fused_stage_bytes(int kp) { return (size_t)(kFusedThreads / 32) * 32 * 4 * kp; }
constexpr size_t kFusedMaxDynamic = (size_t)220 * 1024;

// grid (ceil(N / 32), chunks); dynamic shared memory: the (M + 1) x 32 float slice of B (the
// last row absorbs entries outside submat(S)), then the staging buffer.
template <int KP>
__global__ void __launch_bounds__(kFusedThreads, 1)
    saso_scatter_kernel(int64_t M, int64_t N, int64_t K, const uint32_t *__restrict__ packed,
                        const float *__restrict__ Q, int64_t qs0, int64_t qs1, int64_t k_per_chunk,
                        float alpha, float beta, float *out, int64_t os_i, int64_t os_j,
                        float *partial) {
    extern __shared__ float bs[];
    uint4 *stage = reinterpret_cast<uint4 *>(bs + (M + 1) * kFusedCols);  // 16-byte aligned
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t j0 = (int64_t)blockIdx.x * kFusedCols;
    const int64_t k_begin = (int64_t)blockIdx.y * k_per_chunk;
    const int64_t k_end = min(K, k_begin + k_per_chunk);
    for (int64_t t = threadIdx.x; t < (M + 1) * kFusedCols; t += kFusedThreads) bs[t] = 0.f;
    __syncthreads();
    const uint32_t lane_base = (uint32_t)__cvta_generic_to_shared(bs) + 4u * (uint32_t)lane;
    const bool col_ok = j0 + lane < N;
    const float *qcol = Q + (col_ok ? (j0 + lane) * qs1 : 0);
    for (int64_t base = k_begin + (int64_t)warp * 32; base < k_end;
         base += (int64_t)kFusedThreads) {
        const int64_t kr = base + lane;
#pragma unroll
        for (int q = 0; q < KP / 4; ++q)
            stage[(warp * 32 + lane) * (KP / 4) + q] =
                kr < k_end ? reinterpret_cast<const uint4 *>(packed + kr * KP)[q]
                           : make_uint4(0u, 0u, 0u, 0u);  // a zero row adds 0.0 to row 0
        uint32_t a[32];
#pragma unroll
        for (int t = 0; t < 32; ++t)
            a[t] = (col_ok && base + t < k_end) ? __float_as_uint(__ldcs(qcol + (base + t) * qs0))
                                                : 0u;
        __syncwarp();
#pragma unroll
        for (int t = 0; t < 32; ++t) {
#pragma unroll
            for (int q = 0; q < KP / 4; ++q) {
                const uint4 w = stage[(warp * 32 + t) * (KP / 4) + q];
                red_shared_add_bits(lane_base + (w.x & ~kSignBit), a[t] ^ (w.x & kSignBit));
                red_shared_add_bits(lane_base + (w.y & ~kSignBit), a[t] ^ (w.y & kSignBit));
                red_shared_add_bits(lane_base + (w.z & ~kSignBit), a[t] ^ (w.z & kSignBit));
                red_shared_add_bits(lane_base + (w.w & ~kSignBit), a[t] ^ (w.w & kSignBit));
            }
        }
        __syncwarp();
    }
    __syncthreads();
    for (int64_t t = threadIdx.x; t < M * kFusedCols; t += kFusedThreads) {
        const int64_t r = t / kFusedCols, j = j0 + t % kFusedCols;
        if (j >= N) continue;
        if (partial) {
            partial[((int64_t)blockIdx.y * M + r) * N + j] = bs[t];
        } else {
            float &o = out[r * os_i + j * os_j];
            o = beta == 0.f ? alpha * bs[t] : fmaf(alpha, bs[t], beta * o);
        }
    }
}

// The fused path applies: float data, SASO columns as the sparse vectors, no transpose, and
// the B slice (plus the spare row) fits in shared memory next to the staging buffer.
size_t fused_smem_bytes(int64_t M) { return (size_t)(M + 1) * kFusedCols * sizeof(float); }

bool fused_saso_applies(int dtype, int64_t M, int64_t K, const SparseOperand &Sp) {
    if (deterministic_mode() || dtype != RBG_F32) return false;
    if (Sp.kind != SparseOperand::SASO_GEN || !Sp.short_is_row || Sp.trans) return false;
    if (Sp.vec_nnz < 1 || Sp.vec_nnz > kFusedMaxNnz || Sp.vec_nnz > Sp.dim_major) return false;
    if (Sp.dim_major >= (int64_t)UINT32_MAX || M >= 32768 || K > INT32_MAX) return false;
    return fused_smem_bytes(M) + fused_stage_bytes(Sp.vec_nnz > 8 ? 16 : 8) <= kFusedMaxDynamic;
}

void fused_saso(int64_t M, int64_t N, int64_t K, double alpha, const SparseOperand &Sp,
                const Strided &Q, double beta, float *out, int64_t os_i, int64_t os_j,
                cudaStream_t s) {
    const int kp = Sp.vec_nnz > 8 ? 16 : 8;  // entries per column, padded with spare-row words
    Scratch packed((size_t)K * kp * sizeof(uint32_t), s);
    {
        ProfScope prof("saso_pack", s);
        saso_pack_kernel<<<grid_stride_ctas(K, 128), 128, 0, s>>>(
            Sp.seed, (int)Sp.vec_nnz, kp, (uint32_t)Sp.dim_major, Sp.co, K, Sp.ro, M,
            packed.as<uint32_t>());
        RBG_LAUNCHED();
    }
    const int64_t slices = (N + kFusedCols - 1) / kFusedCols;
    const int64_t sms = num_sms();
    int64_t chunks = std::max<int64_t>(1, sms / slices);
    chunks = std::min<int64_t>(chunks, (K + 1023) / 1024);
    while (chunks > 1 && (double)chunks * M * N * 4 > (double)(1ll << 30)) --chunks;
    const int64_t k_per_chunk = (K + chunks - 1) / chunks;
    chunks = (K + k_per_chunk - 1) / k_per_chunk;
    if (slices > INT32_MAX || chunks > 65535)
        fail(RBG_ERROR_UNSUPPORTED, "sparse sketch too large");
    Scratch part;
    float *partial = nullptr;
    if (chunks > 1) {
        part.alloc((size_t)chunks * M * N * sizeof(float), s);
        partial = part.as<float>();
    }
    const size_t smem = fused_smem_bytes(M) + fused_stage_bytes(kp);
    static bool attr_set[2] = {false, false};
    const dim3 grid((unsigned)slices, (unsigned)chunks);
    {
        ProfScope prof("saso_scatter", s);
        if (kp == 8) {
            if (!attr_set[0]) {
                RBG_CUDA(cudaFuncSetAttribute(saso_scatter_kernel<8>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)kFusedMaxDynamic));
                attr_set[0] = true;
            }
            saso_scatter_kernel<8><<<grid, kFusedThreads, smem, s>>>(
                M, N, K, packed.as<uint32_t>(), static_cast<const float *>(Q.ptr), Q.s0, Q.s1,
                k_per_chunk, (float)alpha, (float)beta, out, os_i, os_j, partial);
        } else {
            if (!attr_set[1]) {
                RBG_CUDA(cudaFuncSetAttribute(saso_scatter_kernel<16>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)kFusedMaxDynamic));
                attr_set[1] = true;
            }
            saso_scatter_kernel<16><<<grid, kFusedThreads, smem, s>>>(
                M, N, K, packed.as<uint32_t>(), static_cast<const float *>(Q.ptr), Q.s0, Q.s1,
                k_per_chunk, (float)alpha, (float)beta, out, os_i, os_j, partial);
        }
        RBG_LAUNCHED();
    }
    if (chunks > 1) {
        spmm_reduce_kernel<float><<<grid_stride_ctas(M * N, 256), 256, 0, s>>>(
            M, N, (int)chunks, partial, (float)alpha, (float)beta, out, os_i, os_j);
        RBG_LAUNCHED();
    }
}


// ------------------------------------------------------------------ row-bucketed SASO
// The same left sketch as the scatter above (wide SASO, sparse vectors = columns of S, no
// transpose), with B accumulated in registers instead of shared-memory reductions:
//  1. saso_bucket_kernel: S's columns are cut into sub-chunks of C columns (C <= 256).  Per
//     sub-chunk one CTA samples the columns (saso_column), counting sorts the entries by row
//     of B and writes a record: the entry words (byte offset of the column's row in the staged
//     A tile, sign in bit 31), in row order and by column within a row, then the u16 row
//     offsets.  The fixed order makes the sums reproducible.
//  2. saso_rows_kernel: a CTA owns 512 rows x 64 columns of B and a range of sub-chunks.  Per
//     sub-chunk one TMA tile load brings the C x 64 block of A and one bulk copy the record
//     into a 3-stage shared-memory ring.  Each warp owns 16 rows, taken as 8 pairs (r, r + 8):
//     the two half-warps walk the two rows' entry lists side by side, lane l keeping columns
//     4 (l & 15) .. 4 (l & 15) + 3 in registers.  There are no atomics: an entry costs one
//     word load, one 16-byte load per lane and four FMAs with +-1.  The CTAs' ranges are
//     summed in range order.
constexpr int kRowsCols = 64;
constexpr int kRowsRowBytes = kRowsCols * 4;
constexpr int kRowsPerWarp = 16;
constexpr int kRowsWarps = 32;
constexpr int kRowsPerCta = kRowsPerWarp * kRowsWarps;
constexpr int kRowsStages = 3;
constexpr int kRowsMaxM = 2048;
constexpr int kBucketThreads = 256;
constexpr int kBucketWarps = kBucketThreads / 32;
constexpr size_t kRowsMaxDynamic = (size_t)226 * 1024;  // leaves room for static shared memory

struct RowsPlan {
    int C = 0;                // columns of S (rows of A) per sub-chunk
    int ew = 1;               // words per entry: 1 (offset | sign) or 2 (offset, value)
    uint32_t ent_cap = 0;     // vec_nnz * C entries per record
    uint32_t ent_words = 0;   // ent_cap * ew
    uint32_t rec_bytes = 0;   // entry words + (M + 1) u16 offsets, padded to 16 bytes
    uint32_t tile_bytes = 0;  // C x 64 floats of A
    uint32_t stage_bytes = 0; // tile, then record (128-byte aligned)
    size_t smem = 0;          // rows kernel dynamic shared memory
    size_t bucket_smem = 0;   // bucket kernel dynamic shared memory
};

// words before the bucket list in shared memory: M + 1 row counters, rounded up to 16 bytes
__host__ __device__ __forceinline__ uint32_t bucket_head_words(int M) {
    return (uint32_t)(M + 4) & ~3u;
}

bool rows_plan(int64_t M, int vec_nnz, int ew, RowsPlan &pl) {
    for (int C = 256; C >= 32; C -= 32) {
        pl.C = C;
        pl.ew = ew;
        pl.ent_cap = (uint32_t)(vec_nnz * C);
        pl.ent_words = pl.ent_cap * (uint32_t)ew;
        pl.rec_bytes = (uint32_t)((pl.ent_words * 4 + (M + 1) * 2 + 15) & ~(int64_t)15);
        pl.tile_bytes = (uint32_t)(C * kRowsRowBytes);
        pl.stage_bytes = (pl.tile_bytes + pl.rec_bytes + 127u) & ~127u;
        pl.smem = 128 + 128 + (size_t)kRowsStages * pl.stage_bytes;  // barriers, alignment
        pl.bucket_smem = ((size_t)bucket_head_words((int)M) + pl.ent_words) * 4;
        if (pl.smem <= kRowsMaxDynamic) return true;
    }
    return false;
}

template <typename I>
struct BucketArgs {
    DevState seed;  // generated operators
    RoundKeys rk;   // seed.key's round keys
    int vec_nnz;
    uint32_t dim_major;
    int64_t co, K, ro;
    int M, C;
    uint32_t ent_words, rec_words;
    uint32_t *rec;
    // filled operators: COO arrays in fill_sparse's layout, and the list of entries that are
    // not where that layout puts them (left to saso_overflow_kernel)
    const I *rows, *cols;
    const float *vals;
    unsigned long long *ovf_count;
    int64_t *ovf;
};

// kFilled: read each column's entries from the COO arrays (two words per entry: offset,
// value); otherwise sample them (one word: offset | sign).
template <int KP, bool kFilled, typename I>
__global__ void __launch_bounds__(kBucketThreads) saso_bucket_kernel(BucketArgs<I> a) {
    constexpr int EW = kFilled ? 2 : 1;
    extern __shared__ __align__(16) uint32_t bsm[];
    __shared__ uint32_t wtot[kBucketWarps + 1];
    const int M = a.M, vec_nnz = a.vec_nnz;
    const uint32_t head = bucket_head_words(M);
    uint32_t *start = bsm;        // [M + 1]: counts, then first positions
    uint32_t *list = bsm + head;  // [ent_words]
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    // counts and list start at zero (a list slot that is never written holds offset 0)
    for (uint32_t i = t; i < head + a.ent_words; i += kBucketThreads) bsm[i] = 0u;
    __syncthreads();

    const int64_t sub = blockIdx.x;
    const int64_t c = sub * a.C + t;
    uint32_t row[KP], word[KP], val[KP], rank[KP];
#pragma unroll
    for (int q = 0; q < KP; ++q) row[q] = (uint32_t)M;  // M: no entry
    if (t < a.C && c < a.K) {
        if constexpr (kFilled) {
            const int64_t g = a.co + c;  // minor index of this column
#pragma unroll
            for (int q = 0; q < KP; ++q) {
                if (q >= vec_nnz) break;
                const int64_t e = g * vec_nnz + q;
                const int64_t col = (int64_t)__ldg(a.cols + e);
                if (col != g) {  // not where fill_sparse puts it
                    const unsigned long long slot = atomicAdd(a.ovf_count, 1ull);
                    a.ovf[slot] = e;
                    continue;
                }
                const int64_t r = (int64_t)__ldg(a.rows + e) - a.ro;
                if (r >= 0 && r < M) {
                    row[q] = (uint32_t)r;
                    word[q] = (uint32_t)t * kRowsRowBytes;
                    val[q] = __float_as_uint(__ldg(a.vals + e));
                }
            }
        } else {
            saso_column(a.seed, a.rk, (uint64_t)(a.co + c), vec_nnz, a.dim_major,
                        [&](int j, uint32_t major, bool neg) {
                            const int64_t r = (int64_t)major - a.ro;
#pragma unroll
                            for (int q = 0; q < KP; ++q)
                                if (q == j) {
                                    row[q] = (r >= 0 && r < M) ? (uint32_t)r : (uint32_t)M;
                                    word[q] = ((uint32_t)t * kRowsRowBytes) |
                                              (neg ? kSignBit : 0u);
                                }
                        });
        }
    }
#pragma unroll
    for (int q = 0; q < KP; ++q)
        if (q < vec_nnz && row[q] < (uint32_t)M) rank[q] = atomicAdd(&start[row[q]], 1u);
    __syncthreads();
    // exclusive scan of the row counts, each thread a contiguous run of rows
    const int per = (M + kBucketThreads - 1) / kBucketThreads;
    const int r0 = min(M, t * per), r1 = min(M, r0 + per);
    uint32_t local = 0;
    for (int r = r0; r < r1; ++r) local += start[r];
    uint32_t incl = local;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    if (lane == 31) wtot[warp] = incl;
    __syncthreads();
    if (t == 0) {
        uint32_t run = 0;
        for (int w = 0; w < kBucketWarps; ++w) {
            const uint32_t v = wtot[w];
            wtot[w] = run;
            run += v;
        }
        wtot[kBucketWarps] = run;
        start[M] = run;
    }
    __syncthreads();
    uint32_t run = wtot[warp] + incl - local;
    for (int r = r0; r < r1; ++r) {
        const uint32_t v = start[r];
        start[r] = run;
        run += v;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < KP; ++q)
        if (q < vec_nnz && row[q] < (uint32_t)M) {
            const uint32_t pos = (start[row[q]] + rank[q]) * EW;
            list[pos] = word[q];
            if constexpr (kFilled) list[pos + 1] = val[q];
        }
    __syncthreads();
    // the atomics hand out ranks in any order: sort each row's entries by column, which fixes
    // the order of the sums
    for (int r = t; r < M; r += kBucketThreads) {
        const uint32_t b = start[r], e = start[r + 1];
        for (uint32_t p = b + 1; p < e; ++p) {
            const uint32_t w = list[p * EW];
            const uint32_t v = kFilled ? list[p * EW + EW - 1] : 0u;
            uint32_t q = p;
            while (q > b && (list[(q - 1) * EW] & ~kSignBit) > (w & ~kSignBit)) {
                list[q * EW] = list[(q - 1) * EW];
                if constexpr (kFilled) list[q * EW + 1] = list[(q - 1) * EW + 1];
                --q;
            }
            list[q * EW] = w;
            if constexpr (kFilled) list[q * EW + 1] = v;
        }
    }
    __syncthreads();
    // record: entry words (zeros past the total), then u16 offsets (the total from row M on)
    const uint32_t total = start[M];
    uint32_t *dst = a.rec + sub * (int64_t)a.rec_words;
    for (uint32_t p = t; p < a.ent_words; p += kBucketThreads) dst[p] = list[p];
    uint16_t *offs = reinterpret_cast<uint16_t *>(dst + a.ent_words);
    for (uint32_t p = t; p < 2 * (a.rec_words - a.ent_words); p += kBucketThreads)
        offs[p] = (uint16_t)(p < (uint32_t)M ? start[p] : total);
}

// Entries of a filled operator that are not where fill_sparse puts them: out(r, :) +=
// alpha * v * Q(k, :) with shared-memory-free atomics, after the main result is written.
template <typename I>
__global__ void saso_overflow_kernel(const unsigned long long *count, const int64_t *ovf,
                                     const I *rows, const I *cols, const float *vals,
                                     int64_t ro, int64_t co, int64_t M, int64_t K, int64_t N,
                                     const float *Q, int64_t qs0, float alpha, float *out,
                                     int64_t os_i, int64_t os_j) {
    const int64_t n = (int64_t)*count;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * N;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = ovf[t / N], j = t % N;
        const int64_t r = (int64_t)rows[e] - ro, k = (int64_t)cols[e] - co;
        if (r < 0 || r >= M || k < 0 || k >= K) continue;
        atomicAdd(out + r * os_i + j * os_j, alpha * vals[e] * Q[k * qs0 + j]);
    }
}

struct RowsParams {
    int M, N, C;
    int64_t nsub, spc;  // sub-chunks, sub-chunks per CTA range
    uint32_t ent_cap, ent_words, rec_bytes, tile_bytes, stage_bytes;
    const unsigned char *rec;
    float alpha, beta;
    float *out;
    int64_t os_i, os_j;
    float *partial;  // [range][M][N], or nullptr when writing `out` directly
    int *err;
};

// One slot of a row's entry list: when i < n, load the entry word at shared address `ea`,
// then this lane's 4 floats of the A row it names (byte offset in the tile at `tile`), and
// add them times +-1 into acc.  The word load and the adds are predicated on i < n; a slot
// past the list reads row 0 of the tile (every temporary stays defined, which keeps register
// pressure down) and adds nothing.
__device__ __forceinline__ void saso_slot(float4 &acc, uint32_t ea, uint32_t tile, int i, int n) {
    asm volatile(
        "{\n\t"
        ".reg .pred p;\n\t"
        ".reg .b32 w, o, sg;\n\t"
        ".reg .f32 a0, a1, a2, a3;\n\t"
        "setp.lt.s32 p, %6, %7;\n\t"
        "mov.b32 w, 0;\n\t"
        "@p ld.shared.u32 w, [%4];\n\t"
        "and.b32 o, w, 0x7fffffff;\n\t"
        "add.u32 o, o, %5;\n\t"
        "ld.shared.v4.f32 {a0, a1, a2, a3}, [o];\n\t"
        "and.b32 sg, w, 0x80000000;\n\t"
        "or.b32 sg, sg, 0x3f800000;\n\t"
        "@p fma.rn.f32 %0, a0, sg, %0;\n\t"
        "@p fma.rn.f32 %1, a1, sg, %1;\n\t"
        "@p fma.rn.f32 %2, a2, sg, %2;\n\t"
        "@p fma.rn.f32 %3, a3, sg, %3;\n\t"
        "}"
        : "+f"(acc.x), "+f"(acc.y), "+f"(acc.z), "+f"(acc.w)
        : "r"(ea), "r"(tile), "r"(i), "r"(n));
}

// Refill ring slot `slot` with sub-chunk `sub`: the C x 64 tile of A by TMA, the record by a
// bulk copy, both completing on the slot's full barrier.
__device__ __forceinline__ void rows_issue(const CUtensorMap *qmap, const RowsParams &p,
                                           uint32_t base, int slot, int64_t sub) {
    const uint32_t st = base + 128u + (uint32_t)slot * p.stage_bytes;
    const uint32_t bar = base + 8u * (uint32_t)slot;
    tc::mbar_arrive_expect_tx_at(bar, p.tile_bytes + p.rec_bytes);
    tc::tma_load_2d_at(st, qmap, bar, (int)blockIdx.x * kRowsCols, (int)(sub * p.C));
    tc::bulk_load_at(st + p.tile_bytes, p.rec + sub * p.rec_bytes, p.rec_bytes, bar);
}

// The same slot for records with two words per entry (byte offset, FP32 value): `ea` is the
// entry's address, and the value replaces the +-1.
__device__ __forceinline__ void saso_slot_valued(float4 &acc, uint32_t ea, uint32_t tile, int i,
                                                 int n) {
    asm volatile(
        "{\n\t"
        ".reg .pred p;\n\t"
        ".reg .b32 w, o, v;\n\t"
        ".reg .f32 a0, a1, a2, a3;\n\t"
        "setp.lt.s32 p, %6, %7;\n\t"
        "mov.b32 w, 0;\n\t"
        "mov.b32 v, 0;\n\t"
        "@p ld.shared.v2.u32 {w, v}, [%4];\n\t"
        "add.u32 o, w, %5;\n\t"
        "ld.shared.v4.f32 {a0, a1, a2, a3}, [o];\n\t"
        "@p fma.rn.f32 %0, a0, v, %0;\n\t"
        "@p fma.rn.f32 %1, a1, v, %1;\n\t"
        "@p fma.rn.f32 %2, a2, v, %2;\n\t"
        "@p fma.rn.f32 %3, a3, v, %3;\n\t"
        "}"
        : "+f"(acc.x), "+f"(acc.y), "+f"(acc.z), "+f"(acc.w)
        : "r"(ea), "r"(tile), "r"(i), "r"(n));
}

// Warp shuffles kept in program order (volatile), so the per-row values of the unrolled row
// loop are not all computed up front, which would cost registers.
__device__ __forceinline__ uint32_t shfl_idx_ordered(uint32_t v, int src) {
    uint32_t r;
    asm volatile("shfl.sync.idx.b32 %0, %1, %2, 0x1f, 0xffffffff;" : "=r"(r) : "r"(v), "r"(src));
    return r;
}

__device__ __forceinline__ int shfl_xor_ordered(int v, int mask) {
    int r;
    asm volatile("shfl.sync.bfly.b32 %0, %1, %2, 0x1f, 0xffffffff;" : "=r"(r) : "r"(v), "r"(mask));
    return r;
}

// grid (ceil(N / 64), ceil(M / 512), ranges), 1024 threads.  Shared memory: full barriers at
// base, empty barriers at base + 24, the ring of stages from base + 128.  kValued: records
// with (offset, value) entries.
template <bool kValued>
__global__ void __launch_bounds__(kRowsWarps * 32, 1)
    saso_rows_kernel(const __grid_constant__ CUtensorMap qmap, RowsParams p) {
    constexpr uint32_t kEntryBytes = kValued ? 8u : 4u;
    extern __shared__ __align__(128) unsigned char rsm_raw[];
    const uint32_t raw = tc::smem_addr(rsm_raw);
    const uint32_t base = (raw + 127u) & ~127u;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wrow = blockIdx.y * kRowsPerCta + warp * kRowsPerWarp;
    const int nloc = (int)(min(p.nsub, (int64_t)blockIdx.z * p.spc + p.spc) -
                           (int64_t)blockIdx.z * p.spc);
    if (threadIdx.x == 0) {
        uint64_t *bars = reinterpret_cast<uint64_t *>(rsm_raw + (base - raw));
        for (int q = 0; q < kRowsStages; ++q) {
            tc::mbar_init(&bars[q], 1);
            tc::mbar_init(&bars[kRowsStages + q], kRowsWarps);
        }
        tc::fence_barrier_init();
        tc::prefetch_tensormap(&qmap);
    }
    __syncthreads();
    int issued = 0;
    if (threadIdx.x == 0)
        for (; issued < min(kRowsStages, nloc); ++issued)
            rows_issue(&qmap, p, base, issued, (int64_t)blockIdx.z * p.spc + issued);

    // half-warp h works on row r + 8h of the pair (r, r + 8); lane l holds columns
    // 4 (l & 15) .. 4 (l & 15) + 3 of its rows
    const int half = lane >> 4;
    constexpr int kAcc = kRowsPerWarp / 2;
    float4 acc[kAcc];
#pragma unroll
    for (int r = 0; r < kAcc; ++r) acc[r] = make_float4(0.f, 0.f, 0.f, 0.f);
    // lane l <= 16 reads the offset of row wrow + l (rows past M read the total)
    const uint32_t off_byte = 2u * (uint32_t)min(wrow + min(lane, kRowsPerWarp), p.M);
    bool ok = true;
    int it = 0;
    for (; it < nloc; ++it) {
        const int slot = it % kRowsStages;
        const uint32_t ph = (uint32_t)(it / kRowsStages) & 1u;
        if (!__all_sync(0xffffffffu, tc::mbar_wait_at(base + 8u * slot, ph, p.err))) {
            ok = false;
            break;
        }
        const uint32_t st = base + 128u + (uint32_t)slot * p.stage_bytes;
        const uint32_t tile = st + 16u * (uint32_t)(lane & 15);
        const uint32_t ents = st + p.tile_bytes;
        const uint32_t o = tc::lds_u16(ents + 4u * p.ent_words + off_byte);
        uint32_t b = __shfl_sync(0xffffffffu, o, 8 * half);
#pragma unroll
        for (int r = 0; r < kAcc; ++r) {
            const uint32_t e = min(shfl_idx_ordered(o, r + 1 + 8 * half), p.ent_cap);
            const int n = (int)e - (int)b;  // entries of this half's row
            const int nmax = max(n, shfl_xor_ordered(n, 16));
            // both halves run nmax slots (rounded up to even) in step
            uint32_t ea = ents + kEntryBytes * b;
#pragma unroll 1
            for (int i = 0; i < nmax; i += 2, ea += 2u * kEntryBytes) {
                if constexpr (kValued) {
                    saso_slot_valued(acc[r], ea, tile, i, n);
                    saso_slot_valued(acc[r], ea + kEntryBytes, tile, i + 1, n);
                } else {
                    saso_slot(acc[r], ea, tile, i, n);
                    saso_slot(acc[r], ea + kEntryBytes, tile, i + 1, n);
                }
            }
            b = e;
        }
        __syncwarp();
        if (lane == 0) tc::mbar_arrive_at(base + 24u + 8u * slot);
        if (warp == 0 && it + kRowsStages < nloc) {
            bool freed = true;
            if (lane == 0) {
                freed = tc::mbar_wait_at(base + 24u + 8u * slot, ph, p.err);
                if (freed) {
                    rows_issue(&qmap, p, base, slot,
                               (int64_t)blockIdx.z * p.spc + it + kRowsStages);
                    ++issued;
                }
            }
            if (!__shfl_sync(0xffffffffu, freed, 0)) {
                ok = false;
                ++it;  // this sub-chunk was consumed
                break;
            }
        }
    }
    if (threadIdx.x == 0) {
        // after an early exit, wait (bounded, whatever the error word says) for loads still in
        // flight into the ring
        __shared__ int drain_err;
        drain_err = 0;
        for (int j = it; j < issued; ++j)
            tc::mbar_wait_at(base + 8u * (j % kRowsStages), (uint32_t)(j / kRowsStages) & 1u,
                             &drain_err, 200000000ll);
    }
    if (!ok) return;

    const int col = (int)blockIdx.x * kRowsCols + 4 * (lane & 15);
    constexpr int kCols = 4;
#pragma unroll
    for (int r = 0; r < kAcc; ++r) {
        const int row = wrow + r + 8 * half;
        const float v4[4] = {acc[r].x, acc[r].y, acc[r].z, acc[r].w};
        if (row >= p.M) break;
#pragma unroll
        for (int h = 0; h < kCols; ++h) {
            const int cc = col + h;
            if (cc >= p.N) break;
            if (p.partial) {
                p.partial[((int64_t)blockIdx.z * p.M + row) * p.N + cc] = v4[h];
            } else {
                float &o = p.out[row * p.os_i + cc * p.os_j];
                o = p.beta == 0.f ? p.alpha * v4[h] : fmaf(p.alpha, v4[h], p.beta * o);
            }
        }
    }
}

// The row-bucketed path applies to the scatter's operators (a sampled wide SASO, no
// transpose) and to filled SASO operators in fill_sparse's layout (outside deterministic
// mode: entries moved out of that layout are added with atomics), with M <= 2048, row-major
// op(A) with 16-byte aligned rows (TMA), at least 64 columns and 256 rows.
bool saso_rows_applies(int dtype, int64_t M, int64_t N, int64_t K, const SparseOperand &Sp,
                       const Strided &Q) {
    if (dtype != RBG_F32) return false;
    const bool filled = Sp.kind == SparseOperand::COO && Sp.saso_layout;
    if (Sp.kind != SparseOperand::SASO_GEN && !filled) return false;
    if (filled && (deterministic_mode() || (Sp.itype != RBG_I32 && Sp.itype != RBG_I64)))
        return false;
    if (!Sp.short_is_row || Sp.trans) return false;
    if (Sp.vec_nnz < 1 || Sp.vec_nnz > kFusedMaxNnz || Sp.vec_nnz > Sp.dim_major) return false;
    if (Sp.dim_major >= (int64_t)UINT32_MAX || M > kRowsMaxM || N < kRowsCols || K < 256 ||
        K > INT32_MAX || N > INT32_MAX)
        return false;
    if (Q.s1 != 1 || Q.s0 < N || (Q.s0 * 4) % 16 != 0 ||
        (reinterpret_cast<uintptr_t>(Q.ptr) & 15) != 0)
        return false;
    RowsPlan pl;
    return rows_plan(M, (int)Sp.vec_nnz, filled ? 2 : 1, pl);
}

template <bool kFilled, typename I>
void launch_bucket(const RowsPlan &pl, int64_t nsub, const BucketArgs<I> &a, int vec_nnz,
                   cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        RBG_CUDA(cudaFuncSetAttribute(saso_bucket_kernel<8, kFilled, I>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
        RBG_CUDA(cudaFuncSetAttribute(saso_bucket_kernel<16, kFilled, I>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
        attr = true;
    }
    if (pl.bucket_smem > 64 * 1024) fail(RBG_ERROR_UNSUPPORTED, "SASO bucket plan");
    if (vec_nnz <= 8)
        saso_bucket_kernel<8, kFilled, I>
            <<<(unsigned)nsub, kBucketThreads, pl.bucket_smem, s>>>(a);
    else
        saso_bucket_kernel<16, kFilled, I>
            <<<(unsigned)nsub, kBucketThreads, pl.bucket_smem, s>>>(a);
    RBG_LAUNCHED();
}

template <bool kValued>
void launch_rows(dim3 grid, size_t smem, const CUtensorMap &map, const RowsParams &p,
                 cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        RBG_CUDA(cudaFuncSetAttribute(saso_rows_kernel<kValued>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kRowsMaxDynamic));
        attr = true;
    }
    saso_rows_kernel<kValued><<<grid, kRowsWarps * 32, smem, s>>>(map, p);
    RBG_LAUNCHED();
}

int64_t gcd64(int64_t a, int64_t b) {
    while (b) {
        const int64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

template <typename I>
void saso_rows(int64_t M, int64_t N, int64_t K, double alpha, const SparseOperand &Sp,
               const Strided &Q, double beta, float *out, int64_t os_i, int64_t os_j,
               cudaStream_t s) {
    const bool filled = Sp.kind == SparseOperand::COO;
    RowsPlan pl;
    if (!rows_plan(M, (int)Sp.vec_nnz, filled ? 2 : 1, pl))
        fail(RBG_ERROR_UNSUPPORTED, "SASO row plan");
    const int64_t nsub = (K + pl.C - 1) / pl.C;
    Scratch rec((size_t)nsub * pl.rec_bytes, s);
    Scratch ovf_count, ovf;
    BucketArgs<I> a{};
    a.seed = Sp.seed;
    a.rk = round_keys(Sp.seed.key);
    a.vec_nnz = (int)Sp.vec_nnz;
    a.dim_major = (uint32_t)Sp.dim_major;
    a.co = Sp.co; a.K = K; a.ro = Sp.ro;
    a.M = (int)M; a.C = pl.C;
    a.ent_words = pl.ent_words;
    a.rec_words = pl.rec_bytes / 4;
    a.rec = rec.as<uint32_t>();
    if (filled) {
        ovf_count.alloc(sizeof(unsigned long long), s);
        ovf.alloc((size_t)Sp.nnz * sizeof(int64_t), s);
        RBG_CUDA(cudaMemsetAsync(ovf_count.ptr, 0, sizeof(unsigned long long), s));
        a.rows = static_cast<const I *>(Sp.idx_a);
        a.cols = static_cast<const I *>(Sp.idx_b);
        a.vals = static_cast<const float *>(Sp.vals);
        a.ovf_count = ovf_count.as<unsigned long long>();
        a.ovf = ovf.as<int64_t>();
    }
    {
        ProfScope prof("saso_bucket", s);
        if (filled) launch_bucket<true, I>(pl, nsub, a, (int)Sp.vec_nnz, s);
        else launch_bucket<false, I>(pl, nsub, a, (int)Sp.vec_nnz, s);
    }
    const int64_t slices = (N + kRowsCols - 1) / kRowsCols;
    const int64_t rblocks = (M + kRowsPerCta - 1) / kRowsPerCta;
    const int64_t base = slices * rblocks;
    const int64_t sms = num_sms();
    // K ranges: a whole number of waves over the SMs when that takes few ranges
    int64_t ranges = sms / gcd64(base, sms);
    if (ranges > 32) ranges = std::max<int64_t>(1, sms / base);
    ranges = std::min(ranges, nsub);
    while (ranges > 1 && (double)ranges * M * N * 4 > (double)(1ll << 30)) --ranges;
    const int64_t spc = (nsub + ranges - 1) / ranges;
    ranges = (nsub + spc - 1) / spc;
    if (slices > INT32_MAX || rblocks > 65535 || ranges > 65535)
        fail(RBG_ERROR_UNSUPPORTED, "sparse sketch too large");
    Scratch part;
    float *partial = nullptr;
    if (ranges > 1) {
        part.alloc((size_t)ranges * M * N * sizeof(float), s);
        partial = part.as<float>();
    }
    CUtensorMap map;
    const cuuint64_t dims[2] = {(cuuint64_t)N, (cuuint64_t)K};
    const cuuint64_t strides[1] = {(cuuint64_t)Q.s0 * 4};
    const cuuint32_t box[2] = {(cuuint32_t)kRowsCols, (cuuint32_t)pl.C};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult cr = tc::tensor_map_encoder()(
        &map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(Q.ptr), dims, strides, box,
        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) fail(RBG_ERROR_CUDA, "cuTensorMapEncodeTiled failed (SASO rows)");
    RowsParams p{};
    p.M = (int)M; p.N = (int)N; p.C = pl.C;
    p.nsub = nsub; p.spc = spc;
    p.ent_cap = pl.ent_cap; p.ent_words = pl.ent_words; p.rec_bytes = pl.rec_bytes;
    p.tile_bytes = pl.tile_bytes; p.stage_bytes = pl.stage_bytes;
    p.rec = rec.as<unsigned char>();
    p.alpha = (float)alpha; p.beta = (float)beta;
    p.out = out; p.os_i = os_i; p.os_j = os_j;
    p.partial = partial;
    p.err = tc::wait_error_flag();
    {
        ProfScope prof("saso_rows", s);
        const dim3 grid((unsigned)slices, (unsigned)rblocks, (unsigned)ranges);
        if (filled) launch_rows<true>(grid, pl.smem, map, p, s);
        else launch_rows<false>(grid, pl.smem, map, p, s);
    }
    if (ranges > 1) {
        spmm_reduce_kernel<float><<<grid_stride_ctas(M * N, 256), 256, 0, s>>>(
            M, N, (int)ranges, partial, (float)alpha, (float)beta, out, os_i, os_j);
        RBG_LAUNCHED();
    }
    if (filled) {
        // entries moved out of fill_sparse's layout (none for an operator as sampled)
        saso_overflow_kernel<I><<<(unsigned)num_sms() * 4, 256, 0, s>>>(
            ovf_count.as<unsigned long long>(), ovf.as<int64_t>(), a.rows, a.cols, a.vals,
            Sp.ro, Sp.co, M, K, N, static_cast<const float *>(Q.ptr), Q.s0, (float)alpha, out,
            os_i, os_j);
        RBG_LAUNCHED();
    }
}

template <typename T>
void run(int64_t M, int64_t N, int64_t K, double alpha, const SparseOperand &Sp,
         const Strided &Q, double beta, void *out, int64_t os_i, int64_t os_j, cudaStream_t s) {
    if (K > INT32_MAX) fail(RBG_ERROR_UNSUPPORTED, "sparse sketch: inner dimension >= 2^31");
    // ---- 1. entries into sort slots
    int64_t slots = 0;
    bool k_ordered = false;  // entries of each row already arrive in increasing k
    if (Sp.kind == SparseOperand::SASO_GEN) {
        slots = safe_mul(Sp.vec_nnz, Sp.dim_minor);
        // minor index i runs over S's columns (short_is_row) or rows; within one row of Sp
        // the entries then come in increasing k exactly when k follows the minor index.
        k_ordered = (Sp.short_is_row && !Sp.trans) || (!Sp.short_is_row && Sp.trans);
    } else {
        slots = Sp.nnz;
    }
    if (slots > INT32_MAX) fail(RBG_ERROR_UNSUPPORTED, "sparse sketch: more than 2^31 nonzeros");
    KeySpec ks{M, K, Sp.ro, Sp.co, Sp.trans, 0};
    const int rbits = bits_for((uint64_t)M);
    if (!k_ordered) ks.kbits = bits_for((uint64_t)K);
    if (rbits + ks.kbits > 64) fail(RBG_ERROR_UNSUPPORTED, "sparse sketch: sort key too wide");
    const int end_bit = rbits + ks.kbits;

    Scratch keys(std::max<int64_t>(slots, 1) * 8, s), skeys(std::max<int64_t>(slots, 1) * 8, s);
    Scratch kc(std::max<int64_t>(slots, 1) * 4, s), vv(std::max<int64_t>(slots, 1) * sizeof(T), s);
    Scratch perm(std::max<int64_t>(slots, 1) * 4, s), sperm(std::max<int64_t>(slots, 1) * 4, s);
    Scratch rowptr((M + 1) * 8, s);
    const int th = 256;
    ProfScope prof_lists("spmm_row_lists", s);
    if (slots > 0) {
        if (Sp.kind == SparseOperand::SASO_GEN) {
            if (Sp.vec_nnz > 64)
                fail(RBG_ERROR_UNSUPPORTED, "in-kernel SASO sampling needs vec_nnz <= 64");
            saso_entries_kernel<T><<<grid_stride_ctas(Sp.dim_minor, 128), 128, 0, s>>>(
                Sp.seed, Sp.vec_nnz, Sp.dim_major, Sp.dim_minor, Sp.short_is_row, ks,
                keys.as<uint64_t>(), kc.as<int32_t>(), vv.as<T>());
        } else if (Sp.kind == SparseOperand::COO) {
            if (Sp.itype == RBG_I32)
                coo_entries_kernel<T, int32_t><<<grid_stride_ctas(slots, th), th, 0, s>>>(
                    slots, (const int32_t *)Sp.idx_a, (const int32_t *)Sp.idx_b,
                    (const T *)Sp.vals, ks, keys.as<uint64_t>(), kc.as<int32_t>(), vv.as<T>());
            else
                coo_entries_kernel<T, int64_t><<<grid_stride_ctas(slots, th), th, 0, s>>>(
                    slots, (const int64_t *)Sp.idx_a, (const int64_t *)Sp.idx_b,
                    (const T *)Sp.vals, ks, keys.as<uint64_t>(), kc.as<int32_t>(), vv.as<T>());
        } else {
            const int by_rows = Sp.kind == SparseOperand::CSR;
            const int64_t lines = by_rows ? Sp.x_rows : Sp.x_cols;
            if (Sp.itype == RBG_I32)
                compressed_entries_kernel<T, int32_t><<<grid_stride_ctas(lines, th), th, 0, s>>>(
                    lines, (const int32_t *)Sp.idx_a, (const int32_t *)Sp.idx_b,
                    (const T *)Sp.vals, by_rows, ks, keys.as<uint64_t>(), kc.as<int32_t>(),
                    vv.as<T>());
            else
                compressed_entries_kernel<T, int64_t><<<grid_stride_ctas(lines, th), th, 0, s>>>(
                    lines, (const int64_t *)Sp.idx_a, (const int64_t *)Sp.idx_b,
                    (const T *)Sp.vals, by_rows, ks, keys.as<uint64_t>(), kc.as<int32_t>(),
                    vv.as<T>());
        }
        RBG_LAUNCHED();
        iota_kernel<<<grid_stride_ctas(slots, th), th, 0, s>>>(slots, perm.as<int32_t>());
        RBG_LAUNCHED();
        // ---- 2. stable sort by key (invalid keys have every bit set and sort last)
        size_t tmp_bytes = 0;
        RBG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.as<uint64_t>(),
                                                 skeys.as<uint64_t>(), perm.as<int32_t>(),
                                                 sperm.as<int32_t>(), (int)slots, 0, end_bit,
                                                 s));
        Scratch tmp(tmp_bytes, s);
        RBG_CUDA(cub::DeviceRadixSort::SortPairs(tmp.ptr, tmp_bytes, keys.as<uint64_t>(),
                                                 skeys.as<uint64_t>(), perm.as<int32_t>(),
                                                 sperm.as<int32_t>(), (int)slots, 0, end_bit,
                                                 s));
        // sorted entries go back into the `keys` buffer's neighbours: reuse perm/kc storage
        gather_entries_kernel<T><<<grid_stride_ctas(slots, th), th, 0, s>>>(
            slots, sperm.as<int32_t>(), kc.as<int32_t>(), vv.as<T>(), perm.as<int32_t>(),
            reinterpret_cast<T *>(keys.ptr));
        RBG_LAUNCHED();
    }
    rowptr_kernel<<<grid_stride_ctas(slots + 1, th), th, 0, s>>>(slots, skeys.as<uint64_t>(),
                                                        ks.kbits, M, rowptr.as<int64_t>());
    RBG_LAUNCHED();
    prof_lists.finish();

    // ---- 3. SpMM
    constexpr int KB = sizeof(T) == 4 ? 1024 : 512;
    const int64_t slices = (N + kSliceCols - 1) / kSliceCols;
    constexpr int rows_per_cta = 32 * rows_per_warp<T>();
    const int64_t rblocks = (M + rows_per_cta - 1) / rows_per_cta;
    const int64_t kblocks = (K + KB - 1) / KB;
    const int64_t base = slices * rblocks;
    const int64_t sms = num_sms();
    int64_t splits = 1;
    if (base < sms) {
        splits = std::max<int64_t>(1, sms / base);
        splits = std::min<int64_t>(splits, kblocks);
        while (splits > 1 && (double)splits * M * N * sizeof(T) > (double)(1ll << 30)) --splits;
    }
    const int64_t kb_per_split = (kblocks + splits - 1) / splits;
    splits = (kblocks + kb_per_split - 1) / kb_per_split;
    if (splits > 65535 || rblocks > 65535) fail(RBG_ERROR_UNSUPPORTED, "sparse sketch too large");
    Scratch part;
    SpmmArgs<T> args{};
    args.M = M; args.N = N; args.K = K;
    args.rowptr = rowptr.as<int64_t>();
    args.kcol = perm.as<int32_t>();
    args.val = reinterpret_cast<const T *>(keys.ptr);
    args.Q = static_cast<const T *>(Q.ptr);
    args.qs0 = Q.s0; args.qs1 = Q.s1;
    args.k_per_split = kb_per_split * KB;
    args.out = (T *)out; args.os_i = os_i; args.os_j = os_j;
    args.alpha = (T)alpha; args.beta = (T)beta;
    if (splits > 1) {
        part.alloc((size_t)splits * M * N * sizeof(T), s);
        args.partial = part.as<T>();
    }
    const size_t smem = (size_t)KB * (kSliceCols + 1) * sizeof(T);
    static bool attr_set[2] = {false, false};
    if (!attr_set[sizeof(T) == 8]) {
        RBG_CUDA(cudaFuncSetAttribute(spmm_rows_kernel<T, KB>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set[sizeof(T) == 8] = true;
    }
    {
        ProfScope prof("spmm_rows", s);
        spmm_rows_kernel<T, KB><<<dim3((unsigned)slices, (unsigned)rblocks, (unsigned)splits),
                                  1024, smem, s>>>(args);
        RBG_LAUNCHED();
    }
    if (splits > 1) {
        spmm_reduce_kernel<T><<<grid_stride_ctas(M * N, 256), 256, 0, s>>>(
            M, N, (int)splits, args.partial, (T)alpha, (T)beta, (T *)out, os_i, os_j);
        RBG_LAUNCHED();
    }
}

// --------------------------------------------------------- generated operator x sparse data
// LSKSP3 / RSKSP3 (RandBLAS/sparse_data/sksp.hh:132-539) when the dense operator holds no
// buffer: Out[M x N] = alpha * P[M x K] * X[K x N] + beta * Out with P = op(submat(S)) generated
// from its counters and X sparse, its rows stored directly (CSR rows, or the CSC columns of a
// transpose).  The reference fills submat(S) into a temporary and then runs the SpMM; here every
// operator entry is generated once and used where it is generated.
//   A CTA owns 32 output rows x all N columns (a shared-memory tile, column stride 33) and a K
// range, walked 32 k's at a time.  Per iteration:
//  1. every thread issues the loads of one nonzero of the iteration (and of the next
//     iteration's row starts), which stay in flight during generation;
//  2. all 256 threads generate the 32 x 32 operator tile, one Philox block each, with the plain
//     path's generator (simt::gen_p_tile_by, two 16-wide halves);
//  3. the nonzeros are staged in shared memory; warp w takes, in entry order, those with
//     column j = w (mod 8), lane l adding P(l, k) * v to row l of column j.  Iterations with
//     more than 256 nonzeros read the rest directly.
// Each output has a single owner that adds in k order, and K ranges are summed in order by
// spmm_reduce_kernel, so results do not depend on scheduling.
constexpr int kGenRows = 32;
constexpr int kGenK = 2 * simt::BK;         // k's per iteration
constexpr int kGenWarps = simt::NT / 32;
constexpr int kGenStage = simt::NT;         // nonzeros staged per iteration
constexpr size_t kGenSpmmMaxSmem = 200 * 1024;

template <typename T>
size_t gen_spmm_smem(int64_t N) {
    return sizeof(T) * ((size_t)kGenK * (kGenRows + 4) + (size_t)N * (kGenRows + 1)) +
           (sizeof(int32_t) + sizeof(T) + 1) * kGenStage + 2 * sizeof(int64_t) * (kGenK + 1) +
           8;  // alignment of the row starts
}

// Row (within the iteration) of entry e: the last q in [0, kn) with rs[q] <= e.
__device__ __forceinline__ int row_in_iteration(const int64_t *rs, int kn, int64_t e) {
    int lo = 0, hi = kn;  // rs[lo] <= e < rs[hi] for a well-formed row range
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (rs[mid] <= e) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <typename T, typename I>
__global__ void __launch_bounds__(simt::NT)
    gen_spmm_kernel(int64_t M, int64_t N, int64_t K, POperand P,
                    const __grid_constant__ RoundKeys rk, const I *__restrict__ ptr,
                    const I *__restrict__ idx, const T *__restrict__ val, int64_t nnz,
                    int64_t k_per_split, T alpha, T beta, T *out, int64_t os_i, int64_t os_j,
                    T *partial) {
    extern __shared__ __align__(16) unsigned char gen_smem[];
    using PsRow = T[kGenRows + 4];
    PsRow *Ps = reinterpret_cast<PsRow *>(gen_smem);  // kGenK rows
    T *tile = reinterpret_cast<T *>(gen_smem + sizeof(T) * kGenK * (kGenRows + 4));
    T *st_v = tile + N * (kGenRows + 1);
    int32_t *st_j = reinterpret_cast<int32_t *>(st_v + kGenStage);
    uint8_t *st_k = reinterpret_cast<uint8_t *>(st_j + kGenStage);
    int64_t *rs_all = reinterpret_cast<int64_t *>(
        (reinterpret_cast<uintptr_t>(st_k + kGenStage) + 7) & ~uintptr_t(7));  // [2][kGenK + 1]
    const int64_t i0 = (int64_t)blockIdx.x * kGenRows;
    const int64_t kb = (int64_t)blockIdx.y * k_per_split;
    const int64_t ke = min(K, kb + k_per_split);
    const int64_t iters = (ke - kb + kGenK - 1) / kGenK;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // row starts, clamped to the entry arrays (a malformed range then holds no entries)
    auto row_start = [&](int64_t k) {
        return max((int64_t)0, min((int64_t)ptr[k], nnz));
    };
    for (int64_t t = tid; t < N * (kGenRows + 1); t += simt::NT) tile[t] = (T)0;
    if (tid <= kGenK && kb + tid <= ke) rs_all[tid] = row_start(kb + tid);
    __syncthreads();
    for (int64_t it = 0; it < iters; ++it) {
        const int64_t k0 = kb + it * kGenK;
        const int kn = (int)min((int64_t)kGenK, ke - k0);
        const int64_t *rs = rs_all + (it & 1) * (kGenK + 1);
        int64_t *rs_next = rs_all + ((it + 1) & 1) * (kGenK + 1);
        const int64_t e_begin = rs[0], e_end = max(rs[kn], e_begin);
        // 1. loads in flight during generation
        const int64_t e = e_begin + tid;
        const bool have = e < e_end;
        int64_t j = -1;
        T v = (T)0;
        if (have) {
            j = (int64_t)idx[e];
            v = val[e];
        }
        int64_t rn = 0;
        const bool next_rs = tid <= kGenK && k0 + kGenK + tid <= ke;
        if (next_rs) rn = row_start(k0 + kGenK + tid);
        // 2. the 32 x 32 operator tile, one 16-wide half per 128 threads
        const int half = tid >> 7;
        simt::gen_p_tile_by<T, kGenRows, simt::NT / 2>(Ps + half * simt::BK, P, M, K, i0,
                                                       k0 + half * simt::BK, tid & 127, rk);
        // 3. stage, then apply
        if (have) {
            st_j[tid] = (j >= 0 && j < N) ? (int32_t)j : -1;
            st_v[tid] = v;
            st_k[tid] = (uint8_t)row_in_iteration(rs, kn, e);
        }
        if (next_rs) rs_next[tid] = rn;
        __syncthreads();
        const int64_t staged = min(e_end - e_begin, (int64_t)kGenStage);
        for (int64_t b = 0; b < staged; b += 32) {
            const int64_t q = b + lane;
            const int32_t jq = q < staged ? st_j[q] : -1;
            unsigned mask = __ballot_sync(0xffffffffu, jq >= 0 && (jq & (kGenWarps - 1)) == warp);
            while (mask) {
                const int src = __ffs(mask) - 1;
                mask &= mask - 1;
                const int64_t slot = b + src;
                T &o = tile[(int64_t)st_j[slot] * (kGenRows + 1) + lane];
                o = fma(Ps[st_k[slot]][lane], st_v[slot], o);
            }
        }
        for (int64_t eb = e_begin + kGenStage; eb < e_end; eb += 32) {  // beyond the stage
            const int64_t eq = eb + lane;
            const bool in = eq < e_end;
            const int64_t jq = in ? (int64_t)idx[eq] : -1;
            const T vq = in ? val[eq] : (T)0;
            const int kq = in ? row_in_iteration(rs, kn, eq) : 0;
            unsigned mask = __ballot_sync(
                0xffffffffu, in && jq >= 0 && jq < N && (int)(jq & (kGenWarps - 1)) == warp);
            while (mask) {
                const int src = __ffs(mask) - 1;
                mask &= mask - 1;
                const int64_t jj = __shfl_sync(0xffffffffu, jq, src);
                const T vv = __shfl_sync(0xffffffffu, vq, src);
                const int kk = __shfl_sync(0xffffffffu, kq, src);
                T &o = tile[jj * (kGenRows + 1) + lane];
                o = fma(Ps[kk][lane], vv, o);
            }
        }
        __syncthreads();  // Ps, the stage and rs are rewritten next iteration
    }
    const int64_t rows = min((int64_t)kGenRows, M - i0);
    if (partial) {
        T *dst = partial + ((int64_t)blockIdx.y * M + i0) * N;
        for (int64_t t = tid; t < rows * N; t += simt::NT) {
            const int64_t i = t / N, jc = t % N;
            dst[i * N + jc] = tile[jc * (kGenRows + 1) + i];
        }
        return;
    }
    const bool j_fast = os_j <= os_i;
    for (int64_t t = tid; t < rows * N; t += simt::NT) {
        const int64_t i = j_fast ? t / N : t % rows;
        const int64_t jc = j_fast ? t % N : t / rows;
        T &o = out[(i0 + i) * os_i + jc * os_j];
        const T acc = tile[jc * (kGenRows + 1) + i];
        o = (beta == (T)0) ? alpha * acc : fma(alpha, acc, beta * o);
    }
}

template <typename T, typename I>
void gen_spmm_rows(int64_t M, int64_t N, int64_t K, double alpha, const POperand &P,
                   const void *ptr, const void *idx, const void *val, int64_t nnz, double beta,
                   void *out, int64_t os_i, int64_t os_j, cudaStream_t s) {
    const size_t smem = gen_spmm_smem<T>(N);
    auto kernel = gen_spmm_kernel<T, I>;
    RBG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    int per_sm = 0;
    RBG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, simt::NT, smem));
    const int64_t tiles = (M + kGenRows - 1) / kGenRows;
    const int64_t steps = (K + kGenK - 1) / kGenK;
    const int64_t slots = (int64_t)num_sms() * std::max(1, per_sm);
    // fill the resident slots, keeping at least 8 iterations per split and the partials
    // <= 1 GiB
    int64_t splits = std::max<int64_t>(1, slots / tiles);
    splits = std::min<int64_t>(splits, std::max<int64_t>(1, steps / 8));
    splits = std::min<int64_t>(splits, std::max<int64_t>(1, (int64_t(1) << 30) /
                                                               (M * N * (int64_t)sizeof(T))));
    const int64_t k_per_split = ((steps + splits - 1) / splits) * kGenK;
    splits = (K + k_per_split - 1) / k_per_split;
    Scratch ws;
    T *partial = nullptr;
    if (splits > 1) {
        ws.alloc(sizeof(T) * (size_t)(splits * M * N), s);
        partial = ws.as<T>();
    }
    {
        ProfScope prof("gen_spmm", s);
        kernel<<<dim3((unsigned)tiles, (unsigned)splits), simt::NT, smem, s>>>(
            M, N, K, P, round_keys(P.gen.key), static_cast<const I *>(ptr),
            static_cast<const I *>(idx),
            static_cast<const T *>(val), nnz, k_per_split, (T)alpha, (T)beta,
            static_cast<T *>(out), os_i, os_j, partial);
        RBG_LAUNCHED();
    }
    if (splits > 1) {
        ProfScope prof("gen_spmm_reduce", s);
        spmm_reduce_kernel<T><<<grid_stride_ctas(M * N, 256), 256, 0, s>>>(
            M, N, (int)splits, partial, (T)alpha, (T)beta, static_cast<T *>(out), os_i, os_j);
        RBG_LAUNCHED();
    }
}

}  // namespace

bool gen_spmm_applies(int dtype, int64_t N) {
    return N >= 1 && (dtype == RBG_F32 ? gen_spmm_smem<float>(N) : gen_spmm_smem<double>(N)) <=
                         kGenSpmmMaxSmem;
}

void gen_spmm_sketch(int dtype, int itype, int64_t M, int64_t N, int64_t K, double alpha,
                     const POperand &P, const void *ptr, const void *idx, const void *val,
                     int64_t nnz, double beta, void *out, int64_t os_i, int64_t os_j,
                     cudaStream_t s) {
    if (M <= 0 || N <= 0) return;
    if (K <= 0 || alpha == 0.0) {
        launch_scale(dtype, M, N, os_i, os_j, beta, out, s);
        return;
    }
    if (dtype == RBG_F32 && itype == RBG_I32)
        gen_spmm_rows<float, int32_t>(M, N, K, alpha, P, ptr, idx, val, nnz, beta, out, os_i,
                                      os_j, s);
    else if (dtype == RBG_F32)
        gen_spmm_rows<float, int64_t>(M, N, K, alpha, P, ptr, idx, val, nnz, beta, out, os_i,
                                      os_j, s);
    else if (itype == RBG_I32)
        gen_spmm_rows<double, int32_t>(M, N, K, alpha, P, ptr, idx, val, nnz, beta, out, os_i,
                                       os_j, s);
    else
        gen_spmm_rows<double, int64_t>(M, N, K, alpha, P, ptr, idx, val, nnz, beta, out, os_i,
                                       os_j, s);
}

void spmm_sketch(int dtype, int64_t M, int64_t N, int64_t K, double alpha,
                 const SparseOperand &Sp, const Strided &Q, double beta, void *out,
                 int64_t os_i, int64_t os_j, cudaStream_t s) {
    if (M <= 0 || N <= 0) return;
    if (K <= 0 || alpha == 0.0) {
        launch_scale(dtype, M, N, os_i, os_j, beta, out, s);
        return;
    }
    if (saso_rows_applies(dtype, M, N, K, Sp, Q)) {
        if (Sp.kind == SparseOperand::COO && Sp.itype == RBG_I32)
            saso_rows<int32_t>(M, N, K, alpha, Sp, Q, beta, static_cast<float *>(out), os_i,
                               os_j, s);
        else
            saso_rows<int64_t>(M, N, K, alpha, Sp, Q, beta, static_cast<float *>(out), os_i,
                               os_j, s);
    }
    else if (fused_saso_applies(dtype, M, K, Sp))
        fused_saso(M, N, K, alpha, Sp, Q, beta, static_cast<float *>(out), os_i, os_j, s);
    else if (dtype == RBG_F32)
        run<float>(M, N, K, alpha, Sp, Q, beta, out, os_i, os_j, s);
    else
        run<double>(M, N, K, alpha, Sp, Q, beta, out, os_i, os_j, s);
}

}  // namespace rbg
