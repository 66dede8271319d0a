// gemm_simt.cu -- the plain (FP32 / FP64) dense sketch: LSKGE3 / RSKGE3 semantics
// (RandBLAS/skge.hh:154-202, 307-355) as one CUDA-core GEMM whose S operand is produced
// tile by tile inside the kernel (or read from a materialised DenseSkOp buffer).
//
// Canonical problem: Out[M x N] = alpha * P[M x K] * Q[K x N] + beta * Out, with
// P = op(submat(S)) (left sketch) or its transpose (right sketch, solved as B^T), Q a
// strided view of op(A).  The reference materialises submat(S) with new[] and calls
// blas::gemm; here S never touches HBM.  Accumulation is in T (float or double), like the
// reference's BLAS call; K is split across CTAs when the output has too few tiles, with a
// fixed-order reduction so results do not depend on timing.
#include <algorithm>
#include <exception>
#include <mutex>

#include "rbg_internal.h"
#include "simt_tiles.cuh"

namespace rbg {
namespace {

using simt::BM;
using simt::BN;
using simt::BK;
using simt::NT;
using simt::gen_p_tile;
using simt::load_tile;
using simt::load_tile_regs;
using simt::store_tile_regs;

// TN: output columns per CTA (128, or 64 for narrow problems); each thread owns 8 rows x TN/16
// columns, in two halves TN/2 apart.  CL > 1 (FP32, generated operator): the CL CTAs of a
// thread-block cluster hold CL consecutive column tiles of the same row block and share its
// operator tiles, each generating 1/CL of every interior tile (one cluster barrier per k step
// instead of __syncthreads); results are the same bits as with CL = 1.  CL must divide BM / 4.
template <typename T, bool GEN, int TN, int CL = 1>
__global__ void __launch_bounds__(NT, (sizeof(T) == 4 || TN < BN) ? 2 : 1)
    dense_sketch_kernel(int64_t M, int64_t N, int64_t K, POperand P,
                        const __grid_constant__ RoundKeys rk, Strided Q, T alpha, T beta,
                        T *__restrict__ out, int64_t os_i, int64_t os_j, int64_t kt_per_split,
                        T *__restrict__ partial) {
    static_assert(CL == 1 || (GEN && sizeof(T) == 4), "clusters: FP32, generated operator");
    constexpr int CPT = TN / 16, CH = CPT / 2;
    // two stages for FP32 (the next k step's data tile is loaded into registers while the
    // current one is computed); one for FP64 (two would exceed 48 KB of static shared memory)
    constexpr int NBUF = sizeof(T) == 4 ? 2 : 1;
    __shared__ __align__(16) T Ps[NBUF][BK][BM + 4];
    __shared__ __align__(16) T Qs[NBUF][BK][TN + 4];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int64_t tiles_n = (N + TN - 1) / TN;
    const int64_t i0 = (blockIdx.x / tiles_n) * BM;
    const int64_t j0 = (blockIdx.x % tiles_n) * TN;
    const int64_t kt_total = (K + BK - 1) / BK;
    const int64_t kt_begin = blockIdx.y * kt_per_split;
    const int64_t kt_end = min(kt_total, kt_begin + kt_per_split);

    T acc[8][CPT];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < CPT; ++b) acc[a][b] = (T)0;

    const T *Qp = static_cast<const T *>(Q.ptr);
    T qr[BK * TN / NT];  // this thread's share of the next data tile
    if (kt_begin < kt_end) load_tile_regs<T, TN>(qr, Qp, Q.s0, Q.s1, K, N, kt_begin * BK, j0);
    uint32_t remote[CL];  // the operator tiles of the cluster's CTAs
    uint32_t rank = 0;
    if constexpr (CL > 1) {
        rank = simt::cluster_rank();
        const uint32_t local = (uint32_t)__cvta_generic_to_shared(&Ps[0][0][0]);
#pragma unroll
        for (int q = 0; q < CL; ++q) remote[q] = simt::cluster_map(local, (uint32_t)q);
        simt::cluster_arrive();  // every CTA of the cluster runs before any stores into it
        simt::cluster_wait();
    }
    for (int64_t kt = kt_begin; kt < kt_end; ++kt) {
        const int64_t k0 = kt * BK;
        const int buf = NBUF == 2 ? (int)((kt - kt_begin) & 1) : 0;
        if constexpr (GEN) {
            if constexpr (CL > 1) {
                // the same decision in every CTA of the cluster (same row block, same k)
                const bool aligned = ((P.r_on_i ? P.c0 + k0 : P.c0 + i0) & 3) == 0;
                if (aligned && i0 + BM <= M && k0 + BK <= K)
                    simt::gen_p_tile_shared<BM, CL>(
                        remote, (uint32_t)(buf * BK * (BM + 4) * sizeof(float)), P, i0, k0,
                        rank, rk);
                else
                    gen_p_tile<T, BM>(Ps[buf], P, M, K, i0, k0, rk);
            } else {
                gen_p_tile<T, BM>(Ps[buf], P, M, K, i0, k0, rk);
            }
        } else {
            // P(i, k) = buff[base + i*si + k*sk]
            load_tile<T, BM>(Ps[buf], static_cast<const T *>(P.buff) + P.base, P.sk, P.si, K, M,
                             k0, i0);
        }
        store_tile_regs<T, TN>(Qs[buf], qr, Q.s0, Q.s1);
        // with two stages, this barrier also retires the reads of the stage written next (in
        // every CTA of the cluster)
        if constexpr (CL > 1) {
            simt::cluster_arrive();
            if (kt + 1 < kt_end) load_tile_regs<T, TN>(qr, Qp, Q.s0, Q.s1, K, N, k0 + BK, j0);
            simt::cluster_wait();
        } else {
            __syncthreads();
            if (kt + 1 < kt_end) load_tile_regs<T, TN>(qr, Qp, Q.s0, Q.s1, K, N, k0 + BK, j0);
        }
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            T a[8], b[CPT];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a[q] = Ps[buf][kk][ty * 4 + q];
                a[4 + q] = Ps[buf][kk][64 + ty * 4 + q];
            }
#pragma unroll
            for (int q = 0; q < CH; ++q) {
                b[q] = Qs[buf][kk][tx * CH + q];
                b[CH + q] = Qs[buf][kk][TN / 2 + tx * CH + q];
            }
#pragma unroll
            for (int x = 0; x < 8; ++x)
#pragma unroll
                for (int y = 0; y < CPT; ++y) acc[x][y] = fma(a[x], b[y], acc[x][y]);
        }
        if (NBUF == 1) __syncthreads();
    }

#pragma unroll
    for (int x = 0; x < 8; ++x) {
        const int64_t i = i0 + (x < 4 ? ty * 4 + x : 64 + ty * 4 + (x - 4));
        if (i >= M) continue;
#pragma unroll
        for (int y = 0; y < CPT; ++y) {
            const int64_t j = j0 + (y < CH ? tx * CH + y : TN / 2 + tx * CH + (y - CH));
            if (j >= N) continue;
            if (partial) {
                partial[((int64_t)blockIdx.y * M + i) * N + j] = acc[x][y];
            } else {
                T &o = out[i * os_i + j * os_j];
                o = (beta == (T)0) ? alpha * acc[x][y] : fma(alpha, acc[x][y], beta * o);
            }
        }
    }
}

// out = alpha * sum_s partial[s] + beta * out, splits summed in order 0..S-1.
template <typename T>
__global__ void reduce_splits_kernel(int64_t M, int64_t N, int splits, const T *partial, T alpha,
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

// ------------------------------------------------------------------ one output column
// Out(i) = sum_k P(i, k) Q(k) with P generated (sketch_vector, and any sketch with n = 1): no
// tile padding, so the cost is the generation of P.  partial[split][i] holds each K range's
// sum, added in split order by reduce_splits_kernel.
//  * r_on_i (a natural row of S per output i): one warp per output, lanes walking the row's
//    counter blocks (4 entries each) in turn; the warp's lane sums are combined by a fixed
//    shuffle tree.
//  * otherwise (a natural row per k): one thread per counter block along the natural row,
//    i.e. 4 consecutive outputs, walking k.
template <typename T>
__device__ __forceinline__ void load4(const T *q, int64_t qs0, bool vec, T out[4]) {
    if (vec) {  // four consecutive, 16-byte aligned values
        if constexpr (sizeof(T) == 4) {
            const float4 w = __ldg(reinterpret_cast<const float4 *>(q));
            out[0] = w.x; out[1] = w.y; out[2] = w.z; out[3] = w.w;
        } else {
            const double2 w0 = __ldg(reinterpret_cast<const double2 *>(q));
            const double2 w1 = __ldg(reinterpret_cast<const double2 *>(q) + 1);
            out[0] = w0.x; out[1] = w0.y; out[2] = w1.x; out[3] = w1.y;
        }
    } else {
#pragma unroll
        for (int l = 0; l < 4; ++l) out[l] = __ldg(q + l * qs0);
    }
}

// Philox's round keys come precomputed in the parameters (rk); a lane's counter advances by
// its stride instead of being recomputed from the entry's coordinates.  vec: Q has unit stride
// and every counter block's four values start on a 16-byte boundary.
template <typename T>
__global__ void __launch_bounds__(256) gemv_gen_kernel(int64_t M, int64_t K, POperand P,
                                                       const __grid_constant__ RoundKeys rk,
                                                       const T *__restrict__ Q, int64_t qs0,
                                                       int vec, int64_t k_per_split,
                                                       T *partial) {
    const DenseGen &g = P.gen;
    const int64_t kb = (int64_t)blockIdx.y * k_per_split;
    const int64_t ke = min(K, kb + k_per_split);
    if (P.r_on_i) {
        const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
        const int lane = threadIdx.x & 31;
        if (i >= M) return;
        const int64_t R = P.r0 + i, cb = P.c0 + kb, ce = P.c0 + ke;  // natural columns
        // blocks [b_in, b_out) hold four columns inside [cb, ce) each
        const int64_t b_in = (cb + 3) / 4, b_out = ce / 4;
        T acc = (T)0;
        int64_t b = cb / 4 + lane;
        uint4 c = g.counter_of(R, b);
        for (; 4 * b < ce; b += 32, c = ctr_add(c, 32)) {
            float v[4];
            gen4(g.family, c, rk, v);
            if (b >= b_in && b < b_out) {
                T q[4];
                load4(Q + (4 * b - P.c0) * qs0, qs0, vec != 0, q);
#pragma unroll
                for (int l = 0; l < 4; ++l) acc = fma(finish_entry<T>(g.family, v[l]), q[l], acc);
            } else {
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    const int64_t C = 4 * b + l;
                    if (C >= cb && C < ce)
                        acc = fma(finish_entry<T>(g.family, v[l]), __ldg(Q + (C - P.c0) * qs0),
                                  acc);
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) partial[(int64_t)blockIdx.y * M + i] = acc;
    } else {
        const int64_t b = P.c0 / 4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
        const int64_t i0 = 4 * b - P.c0;  // output of lane 0 of the block (may be negative)
        if (i0 >= M) return;
        T acc[4] = {(T)0, (T)0, (T)0, (T)0};
        uint4 c = g.counter_of(P.r0 + kb, b);
        for (int64_t k = kb; k < ke; ++k, c = ctr_add(c, (uint64_t)g.stride)) {
            float v[4];
            gen4(g.family, c, rk, v);
            const T q = __ldg(Q + k * qs0);
#pragma unroll
            for (int l = 0; l < 4; ++l) acc[l] = fma(finish_entry<T>(g.family, v[l]), q, acc[l]);
        }
#pragma unroll
        for (int l = 0; l < 4; ++l)
            if (i0 + l >= 0 && i0 + l < M) partial[(int64_t)blockIdx.y * M + i0 + l] = acc[l];
    }
}

template <typename T>
void run_gemv(int64_t M, int64_t K, double alpha, const POperand &P, const Strided &Q,
              double beta, void *out, int64_t os_i, cudaStream_t s) {
    // threads of one K range: a warp per output (r_on_i), else a thread per counter block
    const int64_t threads = P.r_on_i ? M * 32 : (M + 3) / 4 + 1;
    const int64_t blocks = (threads + 255) / 256;
    // K splits: at least one full wave of resident blocks, then the count whose last wave is
    // fullest (ties to fewer splits), with K ranges of >= 4096 columns (r_on_i) or 64 rows
    int per_sm = 0;
    RBG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gemv_gen_kernel<T>, 256, 0));
    const int64_t slots = (int64_t)num_sms() * std::max(1, per_sm);
    const int64_t max_splits = std::max<int64_t>(
        1, std::min<int64_t>(P.r_on_i ? (K + 4095) / 4096 : (K + 63) / 64, 65535));
    int64_t splits = 1;
    double best = -1.0;
    for (int64_t c = 1; c <= std::min<int64_t>(max_splits, 256); ++c) {
        const int64_t ctas = blocks * c;
        const int64_t waves = (ctas + slots - 1) / slots;
        const double eff = (double)ctas / (double)(waves * slots);
        if (eff > best + 1e-3) {
            best = eff;
            splits = c;
        }
        if (ctas >= 8 * slots && eff > 0.95) break;
    }
    const int64_t k_per_split = (K + splits - 1) / splits;
    splits = (K + k_per_split - 1) / k_per_split;
    Scratch ws((size_t)splits * M * sizeof(T), s);
    if (blocks > INT32_MAX) fail(RBG_ERROR_UNSUPPORTED, "sketch with n = 1: too many rows");
    {
        ProfScope prof("dense_sketch_gemv_generated", s);
        // 16-byte aligned blocks: Q + (4 b - c0) on a 16-byte boundary for every b
        const int vec = Q.s0 == 1 && ((reinterpret_cast<uintptr_t>(Q.ptr) -
                                       (uintptr_t)(P.c0 % 4) * sizeof(T)) & 15) == 0;
        gemv_gen_kernel<T><<<dim3((unsigned)blocks, (unsigned)splits), 256, 0, s>>>(
            M, K, P, round_keys(P.gen.key), static_cast<const T *>(Q.ptr), Q.s0, vec,
            k_per_split, ws.as<T>());
        RBG_LAUNCHED();
    }
    const int grid_r = grid_stride_ctas(M, 256);
    reduce_splits_kernel<T><<<grid_r, 256, 0, s>>>(M, 1, (int)splits, ws.as<T>(), (T)alpha,
                                                   (T)beta, (T *)out, os_i, 1);
    RBG_LAUNCHED();
}

// Pick a split of K so that tiles * splits fills whole waves of `per_sm` resident CTAs per SM
// (1 for FP64: co-resident FP64 CTAs share the SM's FP64 pipe, so a second CTA on an SM
// doubles that SM's time).
int choose_splits(int64_t tiles, int64_t kt_total, int64_t out_elems, size_t esz,
                  int per_sm = 2) {
    const int64_t slots = (int64_t)num_sms() * per_sm;
    if (tiles >= 4 * slots || kt_total < 16) return 1;
    int best = 1;
    double best_eff = -1.0;
    for (int s = 1; s <= 128; ++s) {
        if (kt_total / s < 8) break;
        if ((double)s * out_elems * esz > (double)(1ll << 30)) break;
        const int64_t ctas = tiles * s;
        const int64_t waves = (ctas + slots - 1) / slots;
        const double eff = (double)ctas / (double)(waves * slots) - 0.002 * s;
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = s;
        }
    }
    return best;
}

// Output columns per CTA: 64 when the problem is at most 64 wide (half the wasted columns of
// a 128-wide tile), else 128.
int tile_n_for(int64_t N) { return N <= 64 ? 64 : BN; }

template <typename T, bool GEN>
void launch_dense(int tn, dim3 grid, cudaStream_t s, int64_t M, int64_t N, int64_t K,
                  const POperand &P, const Strided &Q, double alpha, double beta, void *out,
                  int64_t os_i, int64_t os_j, int64_t kt_per_split, T *partial) {
    if constexpr (GEN && sizeof(T) == 4) {
        // Gaussian operators: pairs of column tiles of a row block share the generated operator
        // tiles (measured on GB300: +28-30 % at 2048 x 2^18 x 512 and 1024 x 2^17 x 256).
        // Larger clusters cost more in cluster barriers than they save, and uniform entries
        // are too cheap to generate for sharing to pay.
        const int64_t tiles_n = (N + tn - 1) / tn;
        const int cl = (P.gen.family == RBG_GAUSSIAN && tiles_n % 2 == 0) ? 2 : 1;
        if (cl > 1) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = grid;
            cfg.blockDim = dim3(NT);
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = (unsigned)cl;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            const float a = (float)alpha, b = (float)beta;
            float *o = static_cast<float *>(out);
            float *pt = reinterpret_cast<float *>(partial);
            const RoundKeys rk = round_keys(P.gen.key);
#define RBG_DENSE_CLUSTER(TNV, CLV)                                                          \
    RBG_CUDA(cudaLaunchKernelEx(&cfg, dense_sketch_kernel<float, true, TNV, CLV>, M, N, K, P, \
                                rk, Q, a, b, o, os_i, os_j, kt_per_split, pt))
            if (tn == 64) RBG_DENSE_CLUSTER(64, 2);
            else RBG_DENSE_CLUSTER(BN, 2);
#undef RBG_DENSE_CLUSTER
            return;
        }
    }
    // Philox's round keys in the parameters (unused for a materialised operator)
    const RoundKeys rk = round_keys(P.gen.key);
    if (tn == 64)
        dense_sketch_kernel<T, GEN, 64><<<grid, NT, 0, s>>>(M, N, K, P, rk, Q, (T)alpha,
                                                            (T)beta, (T *)out, os_i, os_j,
                                                            kt_per_split, partial);
    else
        dense_sketch_kernel<T, GEN, BN><<<grid, NT, 0, s>>>(M, N, K, P, rk, Q, (T)alpha,
                                                            (T)beta, (T *)out, os_i, os_j,
                                                            kt_per_split, partial);
}

template <typename T>
void run(int64_t M, int64_t N, int64_t K, double alpha, const POperand &P, const Strided &Q,
         double beta, void *out, int64_t os_i, int64_t os_j, cudaStream_t s) {
    if (N == 1 && !P.buff) {
        run_gemv<T>(M, K, alpha, P, Q, beta, out, os_i, s);
        return;
    }
    const int tn = tile_n_for(N);
    const int64_t tiles = ((M + BM - 1) / BM) * ((N + tn - 1) / tn);
    const int64_t kt_total = (K + BK - 1) / BK;
    const int splits = choose_splits(tiles, kt_total, M * N, sizeof(T), sizeof(T) == 8 ? 1 : 2);
    const int64_t kt_per_split = (kt_total + splits - 1) / splits;
    Scratch ws;
    T *partial = nullptr;
    if (splits > 1) {
        ws.alloc((size_t)splits * M * N * sizeof(T), s);
        partial = ws.as<T>();
    }
    const dim3 grid((unsigned)tiles, (unsigned)splits);
    {
        ProfScope prof(P.buff ? "dense_sketch_simt_loaded" : "dense_sketch_simt_generated", s);
        if (P.buff)
            launch_dense<T, false>(tn, grid, s, M, N, K, P, Q, alpha, beta, out, os_i, os_j,
                                   kt_per_split, partial);
        else
            launch_dense<T, true>(tn, grid, s, M, N, K, P, Q, alpha, beta, out, os_i, os_j,
                                  kt_per_split, partial);
        RBG_LAUNCHED();
    }
    if (splits > 1) {
        const int64_t work = M * N;
        const int grid_r = grid_stride_ctas(work, 256);
        reduce_splits_kernel<T><<<grid_r, 256, 0, s>>>(M, N, splits, partial, (T)alpha,
                                                       (T)beta, (T *)out, os_i, os_j);
        RBG_LAUNCHED();
    }
}

}  // namespace

void gemm_dense_sketch(int dtype, int64_t M, int64_t N, int64_t K, double alpha,
                       const POperand &P, const Strided &Q, double beta, void *out,
                       int64_t os_i, int64_t os_j, cudaStream_t s) {
    if (M <= 0 || N <= 0) return;
    if (K <= 0 || alpha == 0.0) {
        // B = beta * B; A and S are not read (BLAS gemm semantics at alpha == 0).
        launch_scale(dtype, M, N, os_i, os_j, beta, out, s);
        return;
    }
    if (dtype == RBG_F32)
        run<float>(M, N, K, alpha, P, Q, beta, out, os_i, os_j, s);
    else
        run<double>(M, N, K, alpha, P, Q, beta, out, os_i, os_j, s);
}

}  // namespace rbg

// ------------------------------------------------------------------ allocation-free variant
// For callers that cannot allocate device memory -- code running inside a CUDA graph being
// captured with a fixed memory plan, an allocator hook, or a host that forbids allocation
// after start-up -- rbg_lskge3_noalloc runs the left dense sketch above with its split-K
// partial sums in this file-scope device array instead of stream-ordered allocations.
// Every GPU that loads this library holds the array until the process exits.
namespace rbg {
namespace {

constexpr size_t kNoallocScratchBytes = size_t(32) << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Device address of g_noalloc_scratch, looked up once per device (with that device current).
void *noalloc_scratch_address() {
    static std::mutex mu;
    static void *addr[64] = {nullptr};
    int dev = 0;
    RBG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) fail(RBG_ERROR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> g(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        RBG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        addr[dev] = p;
    }
    return addr[dev];
}

template <typename T>
void run_noalloc(const DenseLeftProblem &pb, cudaStream_t s) {
    const int64_t M = pb.M, N = pb.N, K = pb.K;
    const size_t slice = (size_t)M * (size_t)N * sizeof(T);
    // the limit holds whether or not this call's split plan needs the scratch, so whether a
    // size is accepted never depends on the GPU's SM count
    if (slice > kNoallocScratchBytes / 2)
        fail(RBG_ERROR_INVALID_ARGUMENT,
             "rbg_lskge3_noalloc: d * n * sizeof(T) = " + std::to_string(slice) +
                 " bytes exceeds its limit of " + std::to_string(kNoallocScratchBytes / 2) +
                 " bytes (half of its fixed 32 MiB scratch); use rbg_lskge3");
    const int tn = tile_n_for(N);
    const int64_t tiles = ((M + BM - 1) / BM) * ((N + tn - 1) / tn);
    const int64_t kt_total = (K + BK - 1) / BK;
    int splits = choose_splits(tiles, kt_total, M * N, sizeof(T), sizeof(T) == 8 ? 1 : 2);
    while (splits > 1 && (size_t)splits * slice > kNoallocScratchBytes) --splits;
    const int64_t kt_per_split = (kt_total + splits - 1) / splits;
    T *partial = splits > 1 ? static_cast<T *>(noalloc_scratch_address()) : nullptr;
    const dim3 grid((unsigned)tiles, (unsigned)splits);
    // every partial element is written by exactly one CTA before the reduction reads it, so
    // the scratch needs no clearing between calls
    if (pb.P.buff)
        launch_dense<T, false>(tn, grid, s, M, N, K, pb.P, pb.Q, pb.alpha, pb.beta, pb.out,
                               pb.os_i, pb.os_j, kt_per_split, partial);
    else
        launch_dense<T, true>(tn, grid, s, M, N, K, pb.P, pb.Q, pb.alpha, pb.beta, pb.out,
                              pb.os_i, pb.os_j, kt_per_split, partial);
    RBG_LAUNCHED();
    if (splits > 1) {
        const int64_t work = M * N;
        const int grid_r = grid_stride_ctas(work, 256);
        reduce_splits_kernel<T><<<grid_r, 256, 0, s>>>(M, N, splits, partial, (T)pb.alpha,
                                                       (T)pb.beta, (T *)pb.out, pb.os_i, pb.os_j);
        RBG_LAUNCHED();
    }
}

}  // namespace
}  // namespace rbg

// The first call on a device looks up the scratch array's device address; make that first
// call before capturing the stream into a CUDA graph.  Calls share the one array: two calls
// whose kernels overlap on the GPU (different streams, no ordering) race on it.
extern "C" int rbg_lskge3_noalloc(int32_t layout, int32_t opS, int32_t opA, int64_t d, int64_t n,
                                  int64_t m, double alpha, const rbg_dense_skop *S, int64_t ro_s,
                                  int64_t co_s, const void *A, int64_t lda, double beta, void *B,
                                  int64_t ldb, rbg_stream_t stream) {
    using namespace rbg;
    return guarded([&] {
        DenseLeftProblem pb{};
        if (!prepare_dense_left(layout, opS, opA, d, n, m, alpha, S, ro_s, co_s, A, lda, beta, B,
                                ldb, &pb))
            return;
        const cudaStream_t s = as_cuda(stream);
        if (pb.K <= 0 || pb.alpha == 0.0) {
            launch_scale(pb.dtype, pb.M, pb.N, pb.os_i, pb.os_j, pb.beta, pb.out, s);
            return;
        }
        if (pb.dtype == RBG_F32)
            run_noalloc<float>(pb, s);
        else
            run_noalloc<double>(pb, s);
    });
}
