// lowp_tc.cu -- the tensor-core precision path: B = alpha * op(submat(S)) * op(A) + beta * B
// with S's entries generated inside the kernel, rounded to BF16, and multiplied on the 5th
// generation tensor cores (tcgen05.mma, FP32 accumulators in tensor memory).  No reference
// counterpart: the reference's LSKGE3 (RandBLAS/skge.hh:154-202) materialises S in FP32/FP64
// and calls blas::gemm; this path keeps its semantics with BF16 operands.
//
// Three launches per call:
//  1. convert: op(A) (FP32, any layout) -> At, BF16, K-major ([n][m], m contiguous), the
//     layout the tensor core reads through TMA with the 128-byte swizzle.
//  2. sketch: persistent, one CTA per SM, 16 warps with fixed roles --
//       warp 0      TMA producer: A tiles (512 n-rows x 64 k) into a 2-stage ring;
//       warp 1      MMA issuer (one thread) and tensor-memory owner (512 columns);
//       warps 4-7   epilogue: tensor memory -> registers -> FP32 partial tile in HBM;
//       warps 8-15  S producers: Philox4x32-10 + transform for a 128 x 64 tile of S per stage,
//                   written as BF16 in the same swizzled K-major layout.
//     A work unit is one 128 x 512 output tile over one slice of the K range; every unit's
//     partial goes to its own slot, so the final sum has a fixed order.  S is never written
//     to HBM.
//  3. reduce: B = alpha * sum over K slices (in order) + beta * B.
// All waits on mbarriers are bounded (clock64 budget); a timeout sets the device error word
// that the host reads through rbg_lowp_status().
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "rbg_internal.h"
#include "tc_ptx.cuh"

namespace rbg {
namespace {

constexpr int BM = 128;          // rows of S per tile (tensor-memory lanes)
constexpr int BN = 512;          // columns of A per tile (tensor-memory columns)
constexpr int BK = 64;           // k per stage: 64 BF16 = one 128-byte swizzle row
constexpr int STAGES = 2;
constexpr int S_STAGE_BYTES = BM * BK * 2;  // 16 KiB
constexpr int A_STAGE_BYTES = BN * BK * 2;  // 64 KiB
constexpr int NUM_THREADS = 512;
constexpr int EPI_WARP0 = 4;
constexpr int GEN_WARP0 = 8;
constexpr int GEN_WARPS = 8;
constexpr int GEN_THREADS = GEN_WARPS * 32;
constexpr uint32_t TMEM_COLS = 512;
constexpr int SMEM_BYTES = STAGES * (S_STAGE_BYTES + A_STAGE_BYTES) + 1024 /*align*/ + 256;

struct LowpParams {
    int64_t M, N, K;       // d, n, m
    DenseGen gen;          // operator entries
    int64_t r0, c0;        // natural coordinates of submat(S)(0, 0)
    int r_on_i;            // 1: natural row follows the output row i
    int64_t k_steps;       // ceil(K / BK)
    int64_t tiles_n;       // ceil(N / BN)
    int64_t tiles;         // ceil(M / BM) * tiles_n
    int64_t ks_per_group;  // k-steps per K slice
    int64_t units;         // tiles * groups
    float *partial;        // [groups][M][N]
    int *err;
};

__device__ __forceinline__ float finish_bf16_input(int family, float v) {
    return family == RBG_UNIFORM ? __fmul_rn(v, 1.7320508075688772f) : v;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// Eight consecutive natural-column entries C = Cs .. Cs+7 of natural row R (transformed,
// uniform entries scaled).  kAligned: Cs % 4 == 0 (two Philox calls instead of three).
template <bool kAligned>
__device__ __forceinline__ void gen8(const DenseGen &g, int64_t R, int64_t Cs, float out[8]) {
    const int64_t b0 = Cs >> 2;
    float v[12];
    gen4<true>(g.family, g.counter_of(R, b0), g.key, v);
    gen4<true>(g.family, g.counter_of(R, b0 + 1), g.key, v + 4);
    if (kAligned) {
#pragma unroll
        for (int e = 0; e < 8; ++e) out[e] = finish_bf16_input(g.family, v[e]);
    } else {
        const int sh = (int)(Cs & 3);
        if (sh) gen4<true>(g.family, g.counter_of(R, b0 + 2), g.key, v + 8);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const float x = sh == 0 ? v[e] : sh == 1 ? v[e + 1] : sh == 2 ? v[e + 2] : v[e + 3];
            out[e] = finish_bf16_input(g.family, x);
        }
    }
}

// S tile (BM rows x BK k, BF16, K-major, 128-byte swizzle) for rows i0.., k-step k0...
// Row i occupies bytes [128 i, 128 i + 128); its 16-byte chunk c sits at chunk c ^ (i % 8).
template <bool kAligned>
__device__ __forceinline__ void produce_s_tile(uint8_t *tile, const LowpParams &p, int64_t i0,
                                               int64_t k0, int gt) {
    if (p.r_on_i) {
        // natural row follows i: thread unit = (row i, 8-wide k chunk c), one 16-byte store
        for (int u = gt; u < BM * 8; u += GEN_THREADS) {
            const int i = u >> 3, c = u & 7;
            const int64_t gi = i0 + i, gk = k0 + 8 * c;
            uint4 w = make_uint4(0, 0, 0, 0);
            if (gi < p.M && gk < p.K) {
                float v[8];
                gen8<kAligned>(p.gen, p.r0 + gi, p.c0 + gk, v);
                if (gk + 8 > p.K) {
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        if (gk + e >= p.K) v[e] = 0.f;
                }
                w = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]),
                               pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
            }
            *reinterpret_cast<uint4 *>(tile + i * 128 + ((c ^ (i & 7)) << 4)) = w;
        }
    } else {
        // natural row follows k: thread unit = (k index kk, 8 consecutive rows i = 8q..8q+7)
        for (int u = gt; u < BK * (BM / 8); u += GEN_THREADS) {
            const int kk = u / (BM / 8), q = u % (BM / 8);
            const int64_t gk = k0 + kk, gi = i0 + 8 * q;
            float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (gk < p.K && gi < p.M) {
                gen8<kAligned>(p.gen, p.r0 + gk, p.c0 + gi, v);
#pragma unroll
                for (int e = 0; e < 8; ++e)
                    if (gi + e >= p.M) v[e] = 0.f;
            }
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int i = 8 * q + e;
                *reinterpret_cast<__nv_bfloat16 *>(tile + i * 128 + (((kk >> 3) ^ (i & 7)) << 4) +
                                                   (kk & 7) * 2) = __float2bfloat16_rn(v[e]);
            }
        }
    }
}

template <bool kAligned>
__global__ void __launch_bounds__(NUM_THREADS, 1)
    sketch_bf16_kernel(const __grid_constant__ CUtensorMap tmap_a, LowpParams p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *s_tiles = smem;                                 // STAGES x 16 KiB
    uint8_t *a_tiles = smem + STAGES * S_STAGE_BYTES;        // STAGES x 64 KiB
    uint64_t *bars = reinterpret_cast<uint64_t *>(a_tiles + STAGES * A_STAGE_BYTES);
    uint64_t *full_a = bars;
    uint64_t *full_s = bars + STAGES;
    uint64_t *empty = bars + 2 * STAGES;
    uint64_t *acc_full = bars + 3 * STAGES;
    uint64_t *acc_empty = acc_full + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_empty + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            tc::mbar_init(&full_a[s], 1);
            tc::mbar_init(&full_s[s], GEN_WARPS);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(acc_full, 1);
        tc::mbar_init(acc_empty, 4);
        tc::fence_barrier_init();
        tc::prefetch_tensormap(&tmap_a);
    }
    if (warp == 1) {
        tc::tmem_alloc(tmem_slot, TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        // ---------------- TMA producer
        if (lane == 0) {
            int64_t it = 0;
            for (int64_t u = blockIdx.x; u < p.units; u += gridDim.x) {
                const int64_t tile = u % p.tiles, g = u / p.tiles;
                const int64_t n0 = (tile % p.tiles_n) * BN;
                const int64_t ks0 = g * p.ks_per_group;
                const int64_t ks1 = min(p.k_steps, ks0 + p.ks_per_group);
                for (int64_t ks = ks0; ks < ks1; ++ks, ++it) {
                    const int s = (int)(it % STAGES);
                    const uint32_t ph = (uint32_t)((it / STAGES) & 1);
                    if (!tc::mbar_wait(&empty[s], ph ^ 1, p.err)) goto done;
                    tc::mbar_arrive_expect_tx(&full_a[s], A_STAGE_BYTES);
                    uint8_t *dst = a_tiles + s * A_STAGE_BYTES;
                    tc::tma_load_2d(dst, &tmap_a, &full_a[s], (int)(ks * BK), (int)n0);
                    tc::tma_load_2d(dst + A_STAGE_BYTES / 2, &tmap_a, &full_a[s], (int)(ks * BK),
                                    (int)(n0 + BN / 2));
                }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer
        if (lane == 0) {
            constexpr uint32_t idesc = tc::idesc_bf16_f32(BM, BN / 2);
            int64_t it = 0, uc = 0;
            for (int64_t u = blockIdx.x; u < p.units; u += gridDim.x, ++uc) {
                const int64_t g = u / p.tiles;
                const int64_t ks0 = g * p.ks_per_group;
                const int64_t ks1 = min(p.k_steps, ks0 + p.ks_per_group);
                if (!tc::mbar_wait(acc_empty, (uint32_t)((uc & 1) ^ 1), p.err)) goto done;
                tc::tc_fence_after();
                for (int64_t ks = ks0; ks < ks1; ++ks, ++it) {
                    const int s = (int)(it % STAGES);
                    const uint32_t ph = (uint32_t)((it / STAGES) & 1);
                    if (!tc::mbar_wait(&full_a[s], ph, p.err)) goto done;
                    if (!tc::mbar_wait(&full_s[s], ph, p.err)) goto done;
                    tc::tc_fence_after();
                    const uint64_t adesc =
                        tc::sw128_kmajor_desc(tc::smem_addr(s_tiles + s * S_STAGE_BYTES));
                    const uint64_t bdesc0 =
                        tc::sw128_kmajor_desc(tc::smem_addr(a_tiles + s * A_STAGE_BYTES));
                    const uint64_t bdesc1 = tc::sw128_kmajor_desc(
                        tc::smem_addr(a_tiles + s * A_STAGE_BYTES + A_STAGE_BYTES / 2));
#pragma unroll
                    for (int kk = 0; kk < BK / 16; ++kk) {
                        const uint32_t acc = (ks > ks0 || kk > 0) ? 1u : 0u;
                        // advancing 16 BF16 along k = 32 bytes = 2 in the encoded address
                        tc::mma_f16(tmem, adesc + 2 * kk, bdesc0 + 2 * kk, idesc, acc);
                        tc::mma_f16(tmem + BN / 2, adesc + 2 * kk, bdesc1 + 2 * kk, idesc, acc);
                    }
                    tc::mma_commit(&empty[s]);
                }
                tc::mma_commit(acc_full);
            }
        }
    } else if (warp >= EPI_WARP0 && warp < EPI_WARP0 + 4) {
        // ---------------- epilogue: tensor memory -> FP32 partial tile
        const int q = warp - EPI_WARP0;  // tensor-memory lanes 32q .. 32q+31
        int64_t uc = 0;
        for (int64_t u = blockIdx.x; u < p.units; u += gridDim.x, ++uc) {
            const int64_t tile = u % p.tiles, g = u / p.tiles;
            const int64_t m0 = (tile / p.tiles_n) * BM, n0 = (tile % p.tiles_n) * BN;
            if (!tc::mbar_wait(acc_full, (uint32_t)(uc & 1), p.err)) goto done;
            tc::tc_fence_after();
            const int64_t row = m0 + 32 * q + lane;
            float *dst = p.partial + (g * p.M + row) * p.N;
#pragma unroll 1
            for (int c = 0; c < BN / 32; ++c) {
                uint32_t r[32];
                tc::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(c * 32), r);
                tc::tmem_ld_wait();
                const int64_t col = n0 + c * 32;
                if (row < p.M && col < p.N) {
                    if (col + 32 <= p.N && (p.N & 3) == 0) {
#pragma unroll
                        for (int v = 0; v < 8; ++v)
                            *reinterpret_cast<float4 *>(dst + col + 4 * v) =
                                make_float4(__uint_as_float(r[4 * v]), __uint_as_float(r[4 * v + 1]),
                                            __uint_as_float(r[4 * v + 2]),
                                            __uint_as_float(r[4 * v + 3]));
                    } else {
#pragma unroll
                        for (int v = 0; v < 32; ++v)
                            if (col + v < p.N) dst[col + v] = __uint_as_float(r[v]);
                    }
                }
            }
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(acc_empty);
        }
    } else if (warp >= GEN_WARP0) {
        // ---------------- S producers
        const int gt = threadIdx.x - GEN_WARP0 * 32;
        int64_t it = 0;
        for (int64_t u = blockIdx.x; u < p.units; u += gridDim.x) {
            const int64_t tile = u % p.tiles, g = u / p.tiles;
            const int64_t m0 = (tile / p.tiles_n) * BM;
            const int64_t ks0 = g * p.ks_per_group;
            const int64_t ks1 = min(p.k_steps, ks0 + p.ks_per_group);
            for (int64_t ks = ks0; ks < ks1; ++ks, ++it) {
                const int s = (int)(it % STAGES);
                const uint32_t ph = (uint32_t)((it / STAGES) & 1);
                if (!tc::mbar_wait(&empty[s], ph ^ 1, p.err)) goto done;
                produce_s_tile<kAligned>(s_tiles + s * S_STAGE_BYTES, p, m0, ks * BK, gt);
                tc::fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&full_s[s]);
            }
        }
    }
done:
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// op(A)(k, j) -> At[j * pitch + k] in BF16, through a 64 x 64 shared-memory tile.
__global__ void convert_a_kernel(const float *__restrict__ A, int64_t sk, int64_t sj, int64_t K,
                                 int64_t N, __nv_bfloat16 *__restrict__ At, int64_t pitch) {
    __shared__ float tile[64][65];
    const int64_t tk = (K + 63) / 64, tj = (N + 63) / 64;
    for (int64_t t = blockIdx.x; t < tk * tj; t += gridDim.x) {
        const int64_t k0 = (t % tk) * 64, j0 = (t / tk) * 64;
        if (sj == 1 || sk != 1) {
            for (int w = threadIdx.x; w < 64 * 64; w += blockDim.x) {
                const int kk = w / 64, jj = w % 64;
                tile[kk][jj] = (k0 + kk < K && j0 + jj < N) ? A[(k0 + kk) * sk + (j0 + jj) * sj]
                                                             : 0.f;
            }
        } else {
            for (int w = threadIdx.x; w < 64 * 64; w += blockDim.x) {
                const int jj = w / 64, kk = w % 64;
                tile[kk][jj] = (k0 + kk < K && j0 + jj < N) ? A[(k0 + kk) * sk + (j0 + jj) * sj]
                                                             : 0.f;
            }
        }
        __syncthreads();
        // each thread writes two consecutive k (one 32-bit BF16 pair) of one row j
        for (int w = threadIdx.x; w < 64 * 32; w += blockDim.x) {
            const int jj = w / 32, kp = (w % 32) * 2;
            if (j0 + jj < N && k0 + kp < K) {
                const __nv_bfloat162 h = __floats2bfloat162_rn(tile[kp][jj], tile[kp + 1][jj]);
                if (k0 + kp + 1 < K)
                    *reinterpret_cast<__nv_bfloat162 *>(At + (j0 + jj) * pitch + k0 + kp) = h;
                else
                    At[(j0 + jj) * pitch + k0 + kp] = h.x;
            }
        }
        __syncthreads();
    }
}

// B = alpha * sum_g partial[g] + beta * B, slices summed in order.
__global__ void lowp_reduce_kernel(int64_t M, int64_t N, int64_t groups, const float *partial,
                                   float alpha, float beta, float *out, int64_t os_i,
                                   int64_t os_j) {
    const int64_t total = M * N;
    const bool j_fast = os_j <= os_i;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = j_fast ? t / N : t % M;
        const int64_t j = j_fast ? t % N : t / M;
        float sum = 0.f;
        for (int64_t g = 0; g < groups; ++g) sum += partial[(g * M + i) * N + j];
        float &o = out[i * os_i + j * os_j];
        o = beta == 0.f ? alpha * sum : fmaf(alpha, sum, beta * o);
    }
}

__device__ int g_lowp_error = 0;

struct Plan {
    int64_t k_steps, tiles_n, tiles, groups, ks_per_group, units, pitch;
    size_t at_bytes, partial_bytes, total;
};

Plan make_plan(int64_t M, int64_t N, int64_t K, int sms) {
    Plan pl{};
    pl.k_steps = (K + BK - 1) / BK;
    pl.tiles_n = (N + BN - 1) / BN;
    pl.tiles = ((M + BM - 1) / BM) * pl.tiles_n;
    pl.pitch = (K + 7) / 8 * 8;  // TMA: row pitch a multiple of 16 bytes
    // K slices: fill whole waves of one CTA per SM, keep slices >= 16 k-steps, bound the
    // partial buffer at 1 GiB
    int64_t best_g = 1;
    double best = -1.0;
    const int64_t gmax = std::max<int64_t>(1, std::min<int64_t>(pl.k_steps / 16, 64));
    for (int64_t g = 1; g <= gmax; ++g) {
        if ((double)g * M * N * 4 > (double)(1ll << 30)) break;
        const int64_t units = pl.tiles * g;
        const int64_t waves = (units + sms - 1) / sms;
        const double eff = (double)units / (double)(waves * sms) - 0.001 * (double)g;
        if (eff > best + 1e-12) {
            best = eff;
            best_g = g;
        }
    }
    pl.ks_per_group = (pl.k_steps + best_g - 1) / best_g;
    pl.groups = (pl.k_steps + pl.ks_per_group - 1) / pl.ks_per_group;
    pl.units = pl.tiles * pl.groups;
    pl.at_bytes = ((size_t)N * pl.pitch * 2 + 1023) / 1024 * 1024;
    pl.partial_bytes = (size_t)pl.groups * M * N * 4;
    pl.total = pl.at_bytes + pl.partial_bytes;
    return pl;
}

using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                              const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                              const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
    static EncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(p);
    });
    if (!fn) fail(RBG_ERROR_CUDA, "cuTensorMapEncodeTiled is not available");
    return fn;
}

void lowp_bf16(int64_t M, int64_t N, int64_t K, float alpha, const DenseGen &gen, int64_t r0,
               int64_t c0, int r_on_i, const Strided &Q, float beta, float *out, int64_t os_i,
               int64_t os_j, void *workspace, size_t ws_bytes, cudaStream_t s) {
    const int sms = num_sms();
    const Plan pl = make_plan(M, N, K, sms);
    Scratch own;
    uint8_t *ws = static_cast<uint8_t *>(workspace);
    if (!ws) {
        own.alloc(pl.total, s);
        ws = own.as<uint8_t>();
    } else if (ws_bytes < pl.total) {
        fail(RBG_ERROR_INVALID_ARGUMENT, "workspace smaller than rbg_lskge3_lowp_workspace()");
    } else if ((reinterpret_cast<uintptr_t>(ws) & 1023) != 0) {
        fail(RBG_ERROR_INVALID_ARGUMENT, "workspace must be 1024-byte aligned");
    }
    __nv_bfloat16 *At = reinterpret_cast<__nv_bfloat16 *>(ws);
    float *partial = reinterpret_cast<float *>(ws + pl.at_bytes);

    {
        ProfScope prof("lowp_convert_a", s);
        const int64_t tiles = ((K + 63) / 64) * ((N + 63) / 64);
        const int grid = (int)std::min<int64_t>(tiles, (int64_t)sms * 16);
        convert_a_kernel<<<grid, 256, 0, s>>>(static_cast<const float *>(Q.ptr), Q.s0, Q.s1, K, N,
                                              At, pl.pitch);
        RBG_LAUNCHED();
    }

    CUtensorMap map;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)N};
    const cuuint64_t strides[1] = {(cuuint64_t)pl.pitch * 2};
    const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)(BN / 2)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult cr = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, At, dims, strides,
                                    box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                    CU_TENSOR_MAP_SWIZZLE_128B,
                                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) fail(RBG_ERROR_CUDA, "cuTensorMapEncodeTiled failed");

    int *err = nullptr;
    RBG_CUDA(cudaGetSymbolAddress((void **)&err, g_lowp_error));
    LowpParams p{};
    p.M = M; p.N = N; p.K = K;
    p.gen = gen; p.r0 = r0; p.c0 = c0; p.r_on_i = r_on_i;
    p.k_steps = pl.k_steps; p.tiles_n = pl.tiles_n; p.tiles = pl.tiles;
    p.ks_per_group = pl.ks_per_group; p.units = pl.units;
    p.partial = partial; p.err = err;
    const bool aligned = (c0 % 4) == 0;
    static bool attr[2] = {false, false};
    if (!attr[aligned]) {
        if (aligned)
            RBG_CUDA(cudaFuncSetAttribute(sketch_bf16_kernel<true>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        else
            RBG_CUDA(cudaFuncSetAttribute(sketch_bf16_kernel<false>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        attr[aligned] = true;
    }
    const int grid = (int)std::min<int64_t>(pl.units, sms);
    {
        ProfScope prof("lowp_sketch_bf16_tc", s);
        if (aligned)
            sketch_bf16_kernel<true><<<grid, NUM_THREADS, SMEM_BYTES, s>>>(map, p);
        else
            sketch_bf16_kernel<false><<<grid, NUM_THREADS, SMEM_BYTES, s>>>(map, p);
        RBG_LAUNCHED();
    }
    {
        ProfScope prof("lowp_reduce", s);
        const int64_t work = M * N;
        const int g = (int)std::max<int64_t>(1, std::min<int64_t>((work + 255) / 256,
                                                                  (int64_t)sms * 16));
        lowp_reduce_kernel<<<g, 256, 0, s>>>(M, N, pl.groups, partial, alpha, beta, out, os_i,
                                             os_j);
        RBG_LAUNCHED();
    }
}

}  // namespace
}  // namespace rbg

using namespace rbg;

namespace {
template <typename F>
int guarded_lowp(F &&f) {
    try {
        f();
        return RBG_SUCCESS;
    } catch (const Failure &e) {
        set_last_error(e.msg);
        return e.code;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return RBG_ERROR_INVALID_ARGUMENT;
    }
}
}  // namespace

extern "C" int rbg_lskge3_lowp_workspace(int32_t precision, int64_t d, int64_t n, int64_t m,
                                         size_t *bytes) {
    return guarded_lowp([&] {
        if (!bytes) fail(RBG_ERROR_INVALID_ARGUMENT, "bytes must not be NULL");
        if (precision != RBG_PREC_BF16)
            fail(RBG_ERROR_UNSUPPORTED, "only RBG_PREC_BF16 is provided");
        RBG_REQUIRE("lskge3_lowp", d > 0 && n > 0 && m > 0);
        int sms = 148;
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess)
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        else
            cudaGetLastError();
        *bytes = make_plan(d, n, m, sms).total;
    });
}

extern "C" int rbg_lowp_status(int32_t *code) {
    return guarded_lowp([&] {
        if (!code) fail(RBG_ERROR_INVALID_ARGUMENT, "code must not be NULL");
        int v = 0;
        RBG_CUDA(cudaMemcpyFromSymbol(&v, g_lowp_error, sizeof v));
        const int zero = 0;
        RBG_CUDA(cudaMemcpyToSymbol(g_lowp_error, &zero, sizeof zero));
        *code = v;
    });
}

extern "C" int rbg_lskge3_lowp(int32_t precision, int32_t layout, int32_t opS, int32_t opA,
                               int64_t d, int64_t n, int64_t m, float alpha,
                               const rbg_dense_skop *S, int64_t ro_s, int64_t co_s, const float *A,
                               int64_t lda, float beta, float *B, int64_t ldb, void *workspace,
                               size_t workspace_bytes, rbg_stream_t stream) {
    return guarded_lowp([&] {
        if (precision != RBG_PREC_BF16)
            fail(RBG_ERROR_UNSUPPORTED, "only RBG_PREC_BF16 is provided");
        if (layout != RBG_COL_MAJOR && layout != RBG_ROW_MAJOR)
            fail(RBG_ERROR_INVALID_ARGUMENT, "layout must be RBG_COL_MAJOR or RBG_ROW_MAJOR");
        if ((opS != RBG_NO_TRANS && opS != RBG_TRANS) || (opA != RBG_NO_TRANS && opA != RBG_TRANS))
            fail(RBG_ERROR_INVALID_ARGUMENT, "op must be RBG_NO_TRANS or RBG_TRANS");
        if (!S) fail(RBG_ERROR_INVALID_ARGUMENT, "S must not be NULL");
        if (S->dtype != RBG_F32) fail(RBG_ERROR_INVALID_ARGUMENT, "the precision path takes FP32 data");
        if (S->buff)
            fail(RBG_ERROR_UNSUPPORTED, "the precision path generates S; pass an unfilled operator");
        RBG_REQUIRE("DenseDist", S->dist.n_rows > 0);
        RBG_REQUIRE("DenseDist", S->dist.n_cols > 0);
        const int64_t sub_rows = opS == RBG_NO_TRANS ? d : m;
        const int64_t sub_cols = opS == RBG_NO_TRANS ? m : d;
        RBG_REQUIRE("lskge3", S->dist.n_rows >= sub_rows + ro_s);
        RBG_REQUIRE("lskge3", S->dist.n_cols >= sub_cols + co_s);
        RBG_REQUIRE("lskge3", ro_s >= 0 && co_s >= 0 && d >= 0 && n >= 0 && m >= 0);
        const int64_t a_rows = opA == RBG_NO_TRANS ? m : n, a_cols = opA == RBG_NO_TRANS ? n : m;
        if (layout == RBG_COL_MAJOR) {
            RBG_REQUIRE("lskge3", lda >= a_rows);
            RBG_REQUIRE("lskge3", ldb >= d);
        } else {
            RBG_REQUIRE("lskge3", lda >= a_cols);
            RBG_REQUIRE("lskge3", ldb >= n);
        }
        if (d == 0 || n == 0) return;
        if (!B) fail(RBG_ERROR_INVALID_ARGUMENT, "B must not be NULL");
        const cudaStream_t s = as_cuda(stream);
        const int64_t brs = layout == RBG_COL_MAJOR ? 1 : ldb;
        const int64_t bcs = layout == RBG_COL_MAJOR ? ldb : 1;
        if (m == 0 || alpha == 0.f) {
            launch_scale(RBG_F32, d, n, brs, bcs, beta, B, s);
            return;
        }
        if (!A) fail(RBG_ERROR_INVALID_ARGUMENT, "A must not be NULL");
        if (m > (int64_t)INT32_MAX - 64 || n > (int64_t)INT32_MAX - BN)
            fail(RBG_ERROR_UNSUPPORTED, "dimension too large for 32-bit TMA coordinates");
        const int64_t ars = layout == RBG_COL_MAJOR ? 1 : lda;
        const int64_t acs = layout == RBG_COL_MAJOR ? lda : 1;
        const Strided Q = opA == RBG_NO_TRANS ? Strided{A, ars, acs} : Strided{A, acs, ars};
        // P(i, k) = op(submat(S))(i, k), in natural coordinates (as make_p in capi.cu)
        const DenseInfo info = dense_info(S->dist);
        const int eff_trans = opS == RBG_TRANS;
        int r_on_i;
        int64_t r0, c0;
        if (info.natural_layout == RBG_ROW_MAJOR) {
            r_on_i = !eff_trans;
            r0 = ro_s;
            c0 = co_s;
        } else {
            r_on_i = eff_trans;
            r0 = co_s;
            c0 = ro_s;
        }
        lowp_bf16(d, n, m, alpha, make_dense_gen(S->dist, S->seed_state), r0, c0, r_on_i, Q, beta,
                  B, brs, bcs, workspace, workspace_bytes, s);
    });
}
