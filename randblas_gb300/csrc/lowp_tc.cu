// lowp_tc.cu -- the tensor-core precision path: B = alpha * op(submat(S)) * op(A) + beta * B
// with S's entries generated inside the kernel, rounded to BF16 (or FP8 e4m3), and multiplied
// on the 5th-generation tensor cores (tcgen05.mma, FP32 accumulators in tensor memory).  No
// reference counterpart: the reference's LSKGE3 (RandBLAS/skge.hh:154-202) materialises S in
// FP32/FP64 and calls blas::gemm; this path keeps its semantics with reduced-precision operands.
//
// Three launches per call (four for FP8):
//  0. (FP8) amax: the largest |op(A)(k, j)| of every column j within every K slice.
//  1. convert: op(A) (FP32 or BF16, any layout) -> At, k-blocked ([k / 64 bytes][n][64 bytes]),
//     so every stage's TMA box is one contiguous block; BF16, or e4m3 after dividing by the
//     power-of-two scale of its (K slice, column).
//  2. sketch: persistent clusters of CN CTAs (one per SM), 16 or 24 warps with fixed roles --
//       warp 0      TMA producer: A tiles (512 n-rows x 64 bytes of k) into a 5-stage ring;
//       warp 1      MMA issuer (one elected lane issues) and tensor-memory owner (512 columns);
//       warps 4-7   epilogue: tensor memory -> registers -> FP32 partial tile (or, with one
//                   K slice, B itself), through a shared-memory staging buffer and tensor
//                   stores where the layout allows (plain stores otherwise);
//       warps 8-    S producers (8 or 16 warps) in 4 groups taking stages in turn:
//                   Philox4x32-10 (round keys from the kernel parameters) + transform for
//                   their half of a 128-row S stage (the N-peer makes the other half and copies
//                   it over with a bulk shared-memory copy), stored in the 64-byte swizzled
//                   K-major layout the tensor core reads.
//     A work unit is one 128 x 512 output tile over one slice of the K range; every unit's
//     partial goes to its own slot, so the final sum has a fixed order.  S is never written
//     to HBM.
//  3. reduce: B = alpha * sum over K slices (in order) + beta * B.
// All waits on mbarriers are bounded (clock64 budget); a timeout sets the device error word
// that the host reads through rbg_lowp_status().
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "rbg_internal.h"
#include "tc_ptx.cuh"

namespace rbg {
namespace {

constexpr int BM = 128;          // rows of S per tile (tensor-memory lanes)
constexpr int BN = 512;          // columns of A per tile (tensor-memory columns)
constexpr int ROW_BYTES = 64;    // one swizzled row of a stage: 32 BF16 or 64 e4m3 values of k
constexpr int CHUNKS = ROW_BYTES / 16;      // 16-byte chunks per row
constexpr int STAGES = 5;
constexpr int S_STAGE_BYTES = BM * ROW_BYTES;  // 8 KiB
constexpr int A_STAGE_BYTES = BN * ROW_BYTES;  // 32 KiB

// Element traits: k values per stage and per 16-byte chunk.
template <bool kFp8>
struct Elem {
    static constexpr int BYTES = kFp8 ? 1 : 2;
    static constexpr int BK = ROW_BYTES / BYTES;  // 32 (BF16) or 64 (e4m3)
    static constexpr int PER_CHUNK = 16 / BYTES;  // 8 or 16
};
// Warp roles: 0 TMA, 1 MMA, 4-7 epilogue (one per tensor-memory lane quarter), kGenWarps
// generator warps from 8 on, in GEN_GROUPS groups of consecutive warps; a warp runs on
// sub-partition id % 4.  Generator warps share the sub-partitions' issue slots with the MMA
// and TMA threads: 16 suit launches that generation bounds (e4m3, Gaussian entries, operators
// not shared by a cluster pair), 8 the uniform BF16 sketch of a cluster pair, whose MMA issue
// is the tighter limit (measured at 4096 x 2^20 x 1024: 5.77 ms against 5.97 with 16).
constexpr int EPI_WARP0 = 4;
constexpr int GEN_WARP0 = 8;
constexpr int GEN_GROUPS = 4;  // groups take stages in turn
template <int kGenWarps>
struct GenLayout {
    static constexpr int THREADS = 32 * (GEN_WARP0 + kGenWarps);
    static constexpr int GROUP_WARPS = kGenWarps / GEN_GROUPS;
    static constexpr int GROUP_THREADS = 32 * GROUP_WARPS;
    static_assert(kGenWarps % GEN_GROUPS == 0, "generator groups of whole warps");
};
// A group's previous stage (it - GEN_GROUPS) guarantees only that the MMAs up to
// it - GEN_GROUPS - STAGES have completed.  Its parity wait on the empty barrier of stage it
// is unambiguous only if the phase before the awaited one (the MMAs of it - STAGES) is
// already complete, so GEN_GROUPS must not exceed STAGES; with more groups a wait can pass a
// phase early, merging two phases of the stage's barriers.
static_assert(GEN_GROUPS <= STAGES, "generator groups must not outnumber the stages");
// group gi synchronises on named barrier 1 + gi; the hardware has barriers 0 .. 15
static_assert(GEN_GROUPS + 1 <= 16, "one named barrier per generator group");
constexpr uint32_t TMEM_COLS = 512;
// Epilogue staging for tensor stores: per epilogue warp two buffers of 32 rows x 16 FP32
// columns (64-byte rows, 64-byte swizzle), so one store reads a buffer while the warp fills
// the other.
constexpr int EPI_COLS = 16;
constexpr int EPI_BUF_BYTES = 32 * EPI_COLS * 4;               // 2 KiB
constexpr int EPI_BUFS = 2;
constexpr int EPI_STAGE_BYTES = 4 * EPI_BUFS * EPI_BUF_BYTES;  // 16 KiB
constexpr int SMEM_BYTES =
    STAGES * (S_STAGE_BYTES + A_STAGE_BYTES) + EPI_STAGE_BYTES + 1024 /*align*/ + 256;

struct LowpParams {
    int64_t M, N, K;       // d, n, m
    DenseGen gen;          // operator entries
    RoundKeys rk;          // gen.key's round keys (the fast producers' Philox)
    int64_t r0, c0;        // natural coordinates of submat(S)(0, 0)
    int r_on_i;            // 1: natural row follows the output row i
    int64_t k_steps;       // ceil(K / k per stage)
    int64_t m_groups;      // row tiles of BM rows
    int64_t n_groups;      // column groups, each CN tiles of BN columns
    int64_t ks_per_group;  // k-steps per K slice
    int64_t units;         // m_groups * n_groups * k_groups
    int64_t npad;          // rows per k-block of the converted A (multiple of BN)
    float *partial;        // [k_groups][M][N]
    const uint32_t *amax;  // FP8: [k_groups][npad] column maxima (float bits); else null
    int *err;
    // 0: the epilogue writes with plain stores; 1: tensor stores of alpha * acc into out (one
    // K slice, beta = 0, out_map over out); 2: tensor stores into the partial buffer (out_map
    // over [k_groups][M][N])
    int out_tma;
    // one K slice: the epilogue writes B = alpha * acc + beta * B itself (no partials, no
    // reduce pass)
    int direct;
    float *out;
    int64_t os_i, os_j;
    float alpha, beta;
};

__device__ __forceinline__ float finish_bf16_input(int family, float v) {
    return family == RBG_UNIFORM ? __fmul_rn(v, 1.7320508075688772f) : v;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// 128-bit counter + small increment (add with carry through all four words).
__device__ __forceinline__ uint4 ctr_add_u32(uint4 c, uint32_t v) {
    asm("add.cc.u32 %0, %0, %4;\n\t"
        "addc.cc.u32 %1, %1, 0;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.u32 %3, %3, 0;"
        : "+r"(c.x), "+r"(c.y), "+r"(c.z), "+r"(c.w)
        : "r"(v));
    return c;
}


// Four e4m3 values (round to nearest, saturating to +-448) in one word, first value lowest.
__device__ __forceinline__ uint32_t pack_e4m3x4(float a, float b, float c, float d) {
    const uint32_t lo = __nv_cvt_float2_to_fp8x2(make_float2(a, b), __NV_SATFINITE, __NV_E4M3);
    const uint32_t hi = __nv_cvt_float2_to_fp8x2(make_float2(c, d), __NV_SATFINITE, __NV_E4M3);
    return lo | (hi << 16);
}

// Power-of-two scale of one (K slice, column) of A on the FP8 path: the smallest 2^e with
// amax / 2^e <= 448 (the largest finite e4m3), from amax's float bits; 1 for an all-zero
// column.  Dividing by it and multiplying the product back are exact.
__device__ __forceinline__ float e4m3_scale(uint32_t amax_bits) {
    const float amax = __uint_as_float(amax_bits);
    if (!(amax > 0.f)) return 1.0f;
    const uint32_t xb = __float_as_uint(__fdiv_rn(amax, 448.0f));
    int e = (int)((xb >> 23) & 0xFFu) - 127;
    if (e < -126) return 0x1p-126f;
    if (xb & 0x7FFFFFu) ++e;
    e = min(e, 127);
    return __uint_as_float((uint32_t)(e + 127) << 23);
}

// One 16-byte chunk of Elem<kFp8>::PER_CHUNK finished entries.
template <bool kFp8>
__device__ __forceinline__ uint4 pack_chunk(const float *v) {
    if (kFp8)
        return make_uint4(pack_e4m3x4(v[0], v[1], v[2], v[3]), pack_e4m3x4(v[4], v[5], v[6], v[7]),
                          pack_e4m3x4(v[8], v[9], v[10], v[11]),
                          pack_e4m3x4(v[12], v[13], v[14], v[15]));
    return make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                      pack_bf16(v[6], v[7]));
}

// PER_CHUNK consecutive natural-column entries starting at a block-aligned counter `c`
// (PER_CHUNK / 4 Philox calls), finished (uniform entries scaled) and packed.
template <bool kFp8>
__device__ __forceinline__ uint4 gen_chunk_aligned(int family, uint4 c, const RoundKeys &key) {
    constexpr int E = Elem<kFp8>::PER_CHUNK;
    float v[E];
    if (family == RBG_UNIFORM) {
#pragma unroll
        for (int q = 0; q < E / 4; ++q) {
            const uint4 r = philox(q == 0 ? c : ctr_add_u32(c, (uint32_t)q), key);
            v[4 * q] = uneg11(r.x);
            v[4 * q + 1] = uneg11(r.y);
            v[4 * q + 2] = uneg11(r.z);
            v[4 * q + 3] = uneg11(r.w);
        }
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = __fmul_rn(v[e], 1.7320508075688772f);
    } else {
#pragma unroll
        for (int q = 0; q < E / 4; ++q)
            gen4<true>(family, q == 0 ? c : ctr_add_u32(c, (uint32_t)q), key, v + 4 * q);
    }
    return pack_chunk<kFp8>(v);
}

// Eight consecutive natural-column entries C = Cs .. Cs+7 of natural row R, any alignment.
__device__ __forceinline__ void gen8_any(const DenseGen &g, int64_t R, int64_t Cs, float out[8]) {
    const int64_t b0 = Cs >> 2;
    const int sh = (int)(Cs & 3);
    float v[12];
    gen4<true>(g.family, g.counter_of(R, b0), g.key, v);
    gen4<true>(g.family, g.counter_of(R, b0 + 1), g.key, v + 4);
    if (sh) gen4<true>(g.family, g.counter_of(R, b0 + 2), g.key, v + 8);
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const float x = sh == 0 ? v[e] : sh == 1 ? v[e + 1] : sh == 2 ? v[e + 2] : v[e + 3];
        out[e] = finish_bf16_input(g.family, x);
    }
}

// Byte offset of byte kb of row i in a BM-row tile stored K-major with the 64-byte swizzle:
// row i occupies bytes [64 i, 64 i + 64); its 16-byte chunk c sits at chunk c ^ ((i / 2) % 4)
// (address bits 4-5 XOR bits 7-8).
__device__ __forceinline__ uint32_t sw_byte(int i, int kb) {
    return (uint32_t)(i * ROW_BYTES + ((((kb >> 4) ^ ((i >> 1) & 3))) << 4) + (kb & 15));
}

// The part of one S stage this CTA produces: rows [row_lo, row_lo + rows) of the stage, by
// `nth` threads (thread index gt).  Generic path: any operator orientation and submatrix
// offset.
template <bool kFp8>
__device__ __forceinline__ void produce_s_generic(uint8_t *tile, const LowpParams &p, int64_t i0,
                                                  int64_t k0, int row_lo, int rows, int gt,
                                                  int nth) {
    constexpr int E = Elem<kFp8>::PER_CHUNK;
    constexpr int BKE = Elem<kFp8>::BK;
    if (p.r_on_i) {
        for (int u = gt; u < rows * CHUNKS; u += nth) {
            const int i = row_lo + u / CHUNKS, c = u % CHUNKS;
            const int64_t gi = i0 + i, gk = k0 + E * c;
            uint4 w = make_uint4(0, 0, 0, 0);
            if (gi < p.M && gk < p.K) {
                float v[E];
#pragma unroll
                for (int h = 0; h < E / 8; ++h) gen8_any(p.gen, p.r0 + gi, p.c0 + gk + 8 * h, v + 8 * h);
#pragma unroll
                for (int e = 0; e < E; ++e)
                    if (gk + e >= p.K) v[e] = 0.f;
                w = pack_chunk<kFp8>(v);
            }
            *reinterpret_cast<uint4 *>(tile + sw_byte(i, 16 * c)) = w;
        }
    } else {
        for (int u = gt; u < BKE * (rows / 8); u += nth) {
            const int kk = u / (rows / 8), q = u % (rows / 8);
            const int64_t gk = k0 + kk, gi = i0 + row_lo + 8 * q;
            float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (gk < p.K && gi < p.M) {
                gen8_any(p.gen, p.r0 + gk, p.c0 + gi, v);
#pragma unroll
                for (int e = 0; e < 8; ++e)
                    if (gi + e >= p.M) v[e] = 0.f;
            }
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                uint8_t *dst = tile + sw_byte(row_lo + 8 * q + e, kk * Elem<kFp8>::BYTES);
                if (kFp8)
                    *dst = (uint8_t)(pack_e4m3x4(v[e], 0.f, 0.f, 0.f) & 0xFFu);
                else
                    *reinterpret_cast<__nv_bfloat16 *>(dst) = __float2bfloat16_rn(v[e]);
            }
        }
    }
}

// Four consecutive natural-column entries at a block-aligned counter, finished as the
// reduced-precision paths take them (uniform entries scaled by sqrt(3)).
__device__ __forceinline__ void gen4_finished(int family, uint4 c, const RoundKeys &key,
                                              float v[4]) {
    if (family == RBG_UNIFORM) {
        const uint4 r = philox(c, key);
        v[0] = __fmul_rn(uneg11(r.x), 1.7320508075688772f);
        v[1] = __fmul_rn(uneg11(r.y), 1.7320508075688772f);
        v[2] = __fmul_rn(uneg11(r.z), 1.7320508075688772f);
        v[3] = __fmul_rn(uneg11(r.w), 1.7320508075688772f);
    } else {
        gen4<true>(family, c, key, v);
    }
}

// The part of one S stage this CTA produces when the operator enters transposed (natural
// row = k, natural column = output row i) and the column offset is a multiple of 4: one
// Philox call gives the entries of 4 consecutive output rows at one k.  A work item is an
// i-quad by KC consecutive k: KC calls, then one KC-value store into each of the 4 rows of
// the K-major tile.  The stage must lie inside K (the caller falls back to the generic
// producer for a last, partial one); rows past M are zero.
template <bool kFp8, int KC>
__device__ __forceinline__ void produce_s_transposed(uint8_t *tile, const LowpParams &p,
                                                     int64_t i0, int64_t k0, int row_lo,
                                                     int rows, int gt, int nth) {
    constexpr int BKE = Elem<kFp8>::BK;
    constexpr int BYTES = Elem<kFp8>::BYTES;
    static_assert(KC * BYTES == 8 || KC * BYTES == 16, "one 8- or 16-byte store per row");
    constexpr int KCS = BKE / KC;
    for (int u = gt; u < (rows / 4) * KCS; u += nth) {
        const int kc = u % KCS, q4 = u / KCS;
        const int64_t gi = i0 + row_lo + 4 * q4;  // first of the 4 output rows
        const int64_t gk = k0 + kc * KC;
        uint4 c = ctr_add(p.gen.ctr, (uint64_t)((p.r0 + gk) * p.gen.stride + (p.c0 + gi) / 4));
        float v[KC][4];
#pragma unroll
        for (int kk = 0; kk < KC; ++kk) {
            gen4_finished(p.gen.family, c, p.rk, v[kk]);
            if (kk + 1 < KC) c = ctr_add(c, (uint64_t)p.gen.stride);
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const bool ok = gi + e < p.M;
            uint8_t *dst = tile + sw_byte(row_lo + 4 * q4 + e, kc * KC * BYTES);
            if constexpr (KC * BYTES == 16) {
                uint4 w;
                if constexpr (kFp8)
                    w = make_uint4(pack_e4m3x4(v[0][e], v[1][e], v[2][e], v[3][e]),
                                   pack_e4m3x4(v[4][e], v[5][e], v[6][e], v[7][e]),
                                   pack_e4m3x4(v[8][e], v[9][e], v[10][e], v[11][e]),
                                   pack_e4m3x4(v[12][e], v[13][e], v[14][e], v[15][e]));
                else
                    w = make_uint4(pack_bf16(v[0][e], v[1][e]), pack_bf16(v[2][e], v[3][e]),
                                   pack_bf16(v[4][e], v[5][e]), pack_bf16(v[6][e], v[7][e]));
                *reinterpret_cast<uint4 *>(dst) = ok ? w : make_uint4(0, 0, 0, 0);
            } else {
                uint2 w;
                if constexpr (kFp8)
                    w = make_uint2(pack_e4m3x4(v[0][e], v[1][e], v[2][e], v[3][e]),
                                   pack_e4m3x4(v[4][e], v[5][e], v[6][e], v[7][e]));
                else
                    w = make_uint2(pack_bf16(v[0][e], v[1][e]), pack_bf16(v[2][e], v[3][e]));
                *reinterpret_cast<uint2 *>(dst) = ok ? w : make_uint2(0, 0);
            }
        }
    }
}

// One CTA computes a BM x BN output tile over one K slice per work unit.  The CN CTAs of a
// cluster hold the same BM rows of S and different BN-column tiles of A: each produces BM / CN
// rows of every S stage and copies them into its peer with a bulk shared-memory copy.  Each
// CTA loads its own A tiles (no multicast: clusters of two CTAs tile every SM, and CTAs whose
// A loads do not wait on each other measured faster than pairs sharing them).
// kMode: 0 the generic producer only; 1 natural row follows i and the operator's column
// offset is a multiple of 4, so every k chunk starts on a counter block; 2 natural row follows
// k and the column offset is a multiple of 4, so every i-quad starts on a counter block.  kFp8: e4m3 operands (kind::f8f6f4, 64 k per stage) and
// the epilogue multiplies each column by its K slice's scale; else BF16 (kind::f16, 32 k).
template <int CN, int kMode, bool kFp8, int kGenWarps>
__global__ void __launch_bounds__(GenLayout<kGenWarps>::THREADS, 1)
    sketch_tc_kernel(const __grid_constant__ CUtensorMap tmap_a,
                     const __grid_constant__ CUtensorMap tmap_out,
                     const __grid_constant__ LowpParams p) {
    constexpr int BKE = Elem<kFp8>::BK;
    constexpr int PER_CHUNK = Elem<kFp8>::PER_CHUNK;
    constexpr int CS = CN;
    constexpr int ROWS = BM / CN;                        // S rows this CTA produces per stage
    constexpr uint32_t PART_BYTES = ROWS * ROW_BYTES;    // their bytes in a stage
    constexpr int GROUP_THREADS = GenLayout<kGenWarps>::GROUP_THREADS;
    constexpr int ROW_SLOTS = GROUP_THREADS / CHUNKS;    // rows a generator group covers at once
    constexpr int FAST_ROWS = ROWS / ROW_SLOTS;          // rows per generator thread per stage
    static_assert(ROWS % ROW_SLOTS == 0, "generator mapping");
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *s_tiles = smem;                                 // STAGES x S_STAGE_BYTES
    uint8_t *a_tiles = smem + STAGES * S_STAGE_BYTES;        // STAGES x A_STAGE_BYTES
    uint8_t *out_stage = a_tiles + STAGES * A_STAGE_BYTES;   // 4 warps x 2 x EPI_BUF_BYTES
    uint64_t *bars = reinterpret_cast<uint64_t *>(out_stage + EPI_STAGE_BYTES);
    // full[s]: two arrivals (TMA thread, producing generator group) plus the bytes of the A
    // tile and, with CN = 2, of the peer's S rows; empty[s]: one MMA commit per cluster CTA
    uint64_t *full = bars;
    uint64_t *empty = bars + STAGES;
    uint64_t *acc_full = bars + 2 * STAGES;
    uint64_t *acc_empty = acc_full + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_empty + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = CS > 1 ? tc::cluster_ctarank() : 0u;
    const uint32_t n_idx = rank;
    const int64_t cluster_id = blockIdx.x / CS;
    const int64_t num_clusters = gridDim.x / CS;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            tc::mbar_init(&full[s], 2);
            tc::mbar_init(&empty[s], CS);
        }
        tc::mbar_init(acc_full, 1);
        tc::mbar_init(acc_empty, 4);
        tc::fence_barrier_init();
        tc::prefetch_tensormap(&tmap_a);
        if (p.out_tma) tc::prefetch_tensormap(&tmap_out);
    }
    if (warp == 1) {
        tc::tmem_alloc(tmem_slot, TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    if (CS > 1) tc::cluster_sync();  // peers' barriers are initialised before any signal
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // The TMA and MMA roles run their loops on the whole warp, issuing from one elected lane,
    // with 16 generator warps (measured 3-5% faster there); with 8, lane 0 alone runs them
    // (1% faster there).
    constexpr bool kWarpLoops = kGenWarps == 16;
    auto role_sync = [] {
        if constexpr (kWarpLoops) __syncwarp();
    };
    auto role_lead = [] {
        if constexpr (kWarpLoops) return tc::elect_one();
        else return true;
    };

    auto unit_tiles = [&](int64_t u, int64_t &m0, int64_t &n0, int64_t &ks0, int64_t &ks1) {
        const int64_t mg = u % p.m_groups;
        const int64_t ng = (u / p.m_groups) % p.n_groups;
        const int64_t g = u / (p.m_groups * p.n_groups);
        m0 = mg * BM;
        n0 = (ng * CN + n_idx) * BN;
        ks0 = g * p.ks_per_group;
        ks1 = min(p.k_steps, ks0 + p.ks_per_group);
        return g;
    };

    if (warp == 0) {
        // ---------------- TMA producer: the whole warp runs the loop and one elected lane
        // issues the loads (kWarpLoops), or lane 0 alone runs it
        if (kWarpLoops || lane == 0) {
            int s = 0;
            uint32_t ph = 0;
            for (int64_t u = cluster_id; u < p.units; u += num_clusters) {
                int64_t m0, n0, ks0, ks1;
                unit_tiles(u, m0, n0, ks0, ks1);
                for (int64_t ks = ks0; ks < ks1; ++ks) {
                    if (!tc::mbar_wait(&empty[s], ph ^ 1, p.err)) goto done;
                    role_sync();
                    if (role_lead()) {
                        tc::mbar_arrive_expect_tx(&full[s], A_STAGE_BYTES);
                        uint8_t *dst = a_tiles + s * A_STAGE_BYTES;
                        const int64_t row0 = ks * p.npad + n0;  // k-blocked layout
                        tc::tma_load_2d(dst, &tmap_a, &full[s], 0, (int)row0);
                        tc::tma_load_2d(dst + A_STAGE_BYTES / 2, &tmap_a, &full[s], 0,
                                        (int)(row0 + BN / 2));
                    }
                    role_sync();
                    if (++s == STAGES) {
                        s = 0;
                        ph ^= 1u;
                    }
                }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer: the whole warp runs the loop (its counters and
        // descriptors stay warp-uniform) and one elected lane issues the MMAs and commits
        // (kWarpLoops), or lane 0 alone runs it
        if (kWarpLoops || lane == 0) {
            constexpr uint32_t idesc =
                kFp8 ? tc::idesc_e4m3_f32(BM, BN / 2) : tc::idesc_bf16_f32(BM, BN / 2);
            // Stage index and phase advance by increment (no 64-bit division), and the
            // shared-memory descriptors of stage s are the stage-0 ones plus s stage strides in
            // their 16-byte address field (addresses stay below 2^18, so the field never
            // overflows): this warp's instructions are few, which matters because it shares
            // its sub-partition's issue slots with generator warps.
            const uint64_t adesc0 = tc::kmajor_desc(tc::smem_addr(s_tiles), ROW_BYTES);
            const uint64_t bdesc00 = tc::kmajor_desc(tc::smem_addr(a_tiles), ROW_BYTES);
            const uint64_t bdesc10 =
                tc::kmajor_desc(tc::smem_addr(a_tiles + A_STAGE_BYTES / 2), ROW_BYTES);
            int s = 0;
            uint32_t ph = 0;
            int64_t it = 0, uc = 0;
            for (int64_t u = cluster_id; u < p.units; u += num_clusters, ++uc) {
                int64_t m0, n0, ks0, ks1;
                unit_tiles(u, m0, n0, ks0, ks1);
                if (!tc::mbar_wait(acc_empty, (uint32_t)((uc & 1) ^ 1), p.err, 256)) goto done;
                role_sync();
                tc::tc_fence_after();
                uint32_t acc = 0;
                for (int64_t ks = ks0; ks < ks1; ++ks, ++it) {
                    if (!tc::mbar_wait(&full[s], ph, p.err)) goto done;
                    role_sync();
                    tc::tc_fence_after();
                    const uint64_t adesc = adesc0 + (uint64_t)(s * (S_STAGE_BYTES >> 4));
                    const uint64_t bdesc0 = bdesc00 + (uint64_t)(s * (A_STAGE_BYTES >> 4));
                    const uint64_t bdesc1 = bdesc10 + (uint64_t)(s * (A_STAGE_BYTES >> 4));
                    if (role_lead()) {
#pragma unroll
                        for (int kk = 0; kk < ROW_BYTES / 32; ++kk) {
                            // one MMA takes 32 bytes of k (16 BF16 or 32 e4m3) = 2 in the
                            // encoded address; the first MMA of a unit overwrites the
                            // accumulator
                            const uint32_t accum = kk == 0 ? acc : 1u;
                            if (kFp8) {
                                tc::mma_f8(tmem, adesc + 2 * kk, bdesc0 + 2 * kk, idesc, accum);
                                tc::mma_f8(tmem + BN / 2, adesc + 2 * kk, bdesc1 + 2 * kk, idesc,
                                           accum);
                            } else {
                                tc::mma_f16(tmem, adesc + 2 * kk, bdesc0 + 2 * kk, idesc, accum);
                                tc::mma_f16(tmem + BN / 2, adesc + 2 * kk, bdesc1 + 2 * kk,
                                            idesc, accum);
                            }
                        }
                        // stage s of every CTA in the cluster may be rewritten by any of them,
                        // so each CTA's MMA completion is signalled to all of them
                        if (CS > 1)
                            tc::mma_commit_multicast(&empty[s], (uint16_t)((1u << CS) - 1));
                        else
                            tc::mma_commit(&empty[s]);
                    }
                    role_sync();
                    acc = 1u;
                    if (++s == STAGES) {
                        s = 0;
                        ph ^= 1u;
                    }
                }
                if (role_lead()) tc::mma_commit(acc_full);
                role_sync();
            }
            // wait until the last arrivals on this CTA's stage barriers -- including the
            // peers' -- have landed, so nothing targets this CTA after it exits
            const int64_t last = it;
            for (int64_t j = 0; j < STAGES && j < last; ++j) {
                const int64_t idx = last - 1 - j;
                if (!tc::mbar_wait(&empty[idx % STAGES],
                                             (uint32_t)((idx / STAGES) & 1), p.err))
                    goto done;
            }
        }
    } else if (warp >= EPI_WARP0 && warp < EPI_WARP0 + 4) {
        // ---------------- epilogue: tensor memory -> FP32 partial tile
        const int q = warp - EPI_WARP0;  // tensor-memory lanes 32q .. 32q+31
        int64_t uc = 0;
        if (p.out_tma) {
            // tensor stores: 32 columns of tensor memory at a time, in two 16-column halves
            // that each go registers -> a staging buffer (this lane's row, 64-byte swizzle) ->
            // one tensor store issued by lane 0; tensor memory is handed back as soon as the
            // last columns are loaded, while the stores drain.  (Loading 16 columns at a time
            // measured 1.5% slower on the 2^18 x 512 output; a third buffer gained nothing.)
            const uint32_t stage0 =
                tc::smem_addr(out_stage) + (uint32_t)(q * EPI_BUFS * EPI_BUF_BYTES);
            const uint32_t row_off = (uint32_t)lane * (EPI_COLS * 4);
            const uint32_t sw = (uint32_t)((lane >> 1) & 3);
            uint32_t cnt = 0;
            for (int64_t u = cluster_id; u < p.units; u += num_clusters, ++uc) {
                int64_t m0, n0, ks0, ks1;
                const int64_t g = unit_tiles(u, m0, n0, ks0, ks1);
                if (!tc::mbar_wait(acc_full, (uint32_t)(uc & 1), p.err, 512)) goto done;
                tc::tc_fence_after();
                const int y = (int)(m0 + 32 * q);
#pragma unroll 1
                for (int c = 0; c < BN / 32; ++c) {
                    uint32_t r[32];
                    tc::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(c * 32), r);
                    tc::tmem_ld_wait();
                    if (n0 + c * 32 >= p.N) break;
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int64_t col = n0 + c * 32 + h * EPI_COLS;
                        if (col >= p.N) break;
                        float v[EPI_COLS];
#pragma unroll
                        for (int j = 0; j < EPI_COLS; ++j) {
                            float x = __uint_as_float(r[h * EPI_COLS + j]);
                            if (kFp8) x *= e4m3_scale(p.amax[g * p.npad + col + j]);
                            v[j] = p.out_tma == 1 ? p.alpha * x : x;
                        }
                        const uint32_t buf = stage0 + cnt * EPI_BUF_BYTES;
                        // the store issued from this buffer two halves ago has read it
                        if (lane == 0) tc::bulk_wait_read<EPI_BUFS - 1>();
                        __syncwarp();
#pragma unroll
                        for (int j = 0; j < EPI_COLS / 4; ++j)
                            tc::sts_v4(buf + row_off + ((((uint32_t)j) ^ sw) << 4), v[4 * j],
                                       v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                        tc::fence_proxy_async_smem();
                        __syncwarp();
                        if (lane == 0) {
                            if (p.out_tma == 1) tc::tma_store_2d(&tmap_out, buf, (int)col, y);
                            else tc::tma_store_3d(&tmap_out, buf, (int)col, y, (int)g);
                            tc::bulk_commit();
                        }
                        cnt ^= 1u;
                    }
                }
                tc::tc_fence_before();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(acc_empty);
            }
        } else {
            for (int64_t u = cluster_id; u < p.units; u += num_clusters, ++uc) {
                int64_t m0, n0, ks0, ks1;
                const int64_t g = unit_tiles(u, m0, n0, ks0, ks1);
                if (!tc::mbar_wait(acc_full, (uint32_t)(uc & 1), p.err, 512)) goto done;
                tc::tc_fence_after();
                const int64_t row = m0 + 32 * q + lane;
                float *dst = p.partial + (g * p.M + row) * p.N;
#pragma unroll 1
                for (int c = 0; c < BN / 32; ++c) {
                    uint32_t r[32];
                    tc::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(c * 32), r);
                    tc::tmem_ld_wait();
                    const int64_t col = n0 + c * 32;
                    if (kFp8) {
                        // undo the (K slice, column) scales of A (powers of two: exact)
                        const uint32_t *am = p.amax + g * p.npad + col;
#pragma unroll
                        for (int v = 0; v < 32; ++v)
                            r[v] = __float_as_uint(__uint_as_float(r[v]) * e4m3_scale(am[v]));
                    }
                    if (p.direct) {
                        if (row < p.M && col < p.N) {
                            float *o = p.out + row * p.os_i;
                            if (col + 32 <= p.N && p.os_j == 1 &&
                                ((reinterpret_cast<uintptr_t>(o + col)) & 15) == 0) {
#pragma unroll
                                for (int v = 0; v < 8; ++v) {
                                    float4 *o4 = reinterpret_cast<float4 *>(o + col + 4 * v);
                                    float4 b = make_float4(0.f, 0.f, 0.f, 0.f);
                                    if (p.beta != 0.f) b = *o4;
                                    const float a0 = __uint_as_float(r[4 * v]);
                                    const float a1 = __uint_as_float(r[4 * v + 1]);
                                    const float a2 = __uint_as_float(r[4 * v + 2]);
                                    const float a3 = __uint_as_float(r[4 * v + 3]);
                                    const bool b0 = p.beta == 0.f;
                                    float4 w;
                                    w.x = b0 ? p.alpha * a0 : fmaf(p.alpha, a0, p.beta * b.x);
                                    w.y = b0 ? p.alpha * a1 : fmaf(p.alpha, a1, p.beta * b.y);
                                    w.z = b0 ? p.alpha * a2 : fmaf(p.alpha, a2, p.beta * b.z);
                                    w.w = b0 ? p.alpha * a3 : fmaf(p.alpha, a3, p.beta * b.w);
                                    *o4 = w;
                                }
                            } else {
#pragma unroll
                                for (int v = 0; v < 32; ++v)
                                    if (col + v < p.N) {
                                        float &x = o[(col + v) * p.os_j];
                                        const float a = __uint_as_float(r[v]);
                                        x = p.beta == 0.f ? p.alpha * a
                                                          : fmaf(p.alpha, a, p.beta * x);
                                    }
                            }
                        }
                    } else if (row < p.M && col < p.N) {
                        if (col + 32 <= p.N && (p.N & 3) == 0) {
#pragma unroll
                            for (int v = 0; v < 8; ++v)
                                *reinterpret_cast<float4 *>(dst + col + 4 * v) = make_float4(
                                    __uint_as_float(r[4 * v]), __uint_as_float(r[4 * v + 1]),
                                    __uint_as_float(r[4 * v + 2]), __uint_as_float(r[4 * v + 3]));
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
        }
    } else if (warp >= GEN_WARP0) {
        // ---------------- S producers: GEN_GROUPS groups, group gi takes the stages with
        // it % GEN_GROUPS == gi
        const int gw = warp - GEN_WARP0;
        const int gi = gw / GenLayout<kGenWarps>::GROUP_WARPS;
        const int tg = (gw % GenLayout<kGenWarps>::GROUP_WARPS) * 32 + lane;
        const int row_lo = (int)n_idx * ROWS;
        // the N-peer's copies of the full barriers and S tiles (stage s at + 8 s and
        // + s * S_STAGE_BYTES): shared::cluster addresses, computed rather than kept in an
        // array indexed by the stage, which would live in local memory
        uint32_t peer_full0 = 0, peer_tiles = 0;
        if (CN > 1) {
            peer_full0 = tc::map_to_rank(tc::smem_addr(&full[0]), rank ^ 1u);
            peer_tiles = tc::map_to_rank(tc::smem_addr(s_tiles), rank ^ 1u);
        }
        const int fc = tg % CHUNKS;
        int64_t it_unit = 0;  // the iteration count (shared by every role) at the unit's start
        for (int64_t u = cluster_id; u < p.units; u += num_clusters) {
            int64_t m0, n0, ks0, ks1;
            unit_tiles(u, m0, n0, ks0, ks1);
            // this group's first k-step of the unit, then every GEN_GROUPS-th; its stage and
            // phase advance by increment (no division per step)
            const int64_t skip = ((int64_t)gi - it_unit % GEN_GROUPS + GEN_GROUPS) % GEN_GROUPS;
            int64_t it = it_unit + skip;
            int s = (int)(it % STAGES);
            uint32_t ph = (uint32_t)((it / STAGES) & 1);
            it_unit += ks1 - ks0;
            const int64_t ks_first = ks0 + skip;
            // fast path: the counter of each owned row's chunk at the group's first k-step,
            // advanced by GEN_GROUPS stages of counters per step
            uint4 ctr[FAST_ROWS > 0 ? FAST_ROWS : 1];
            bool row_ok[FAST_ROWS > 0 ? FAST_ROWS : 1];
            if (kMode == 1) {
#pragma unroll
                for (int t = 0; t < FAST_ROWS; ++t) {
                    const int64_t gi_row = m0 + row_lo + tg / CHUNKS + t * ROW_SLOTS;
                    row_ok[t] = gi_row < p.M;
                    ctr[t] = ctr_add(p.gen.ctr,
                                     (uint64_t)((p.r0 + gi_row) * p.gen.stride + p.c0 / 4 +
                                                (PER_CHUNK / 4) * fc + ks_first * (BKE / 4)));
                }
            }
            for (int64_t ks = ks_first; ks < ks1; ks += GEN_GROUPS) {
                if (!tc::mbar_wait(&empty[s], ph ^ 1, p.err)) goto done;
                uint8_t *tile = s_tiles + s * S_STAGE_BYTES;
                const int64_t gk = ks * BKE + PER_CHUNK * fc;
                if (kMode == 1 && gk + PER_CHUNK <= p.K) {
#pragma unroll
                    for (int t = 0; t < FAST_ROWS; ++t) {
                        const int i = row_lo + tg / CHUNKS + t * ROW_SLOTS;
                        const uint4 w = row_ok[t]
                                            ? gen_chunk_aligned<kFp8>(p.gen.family, ctr[t],
                                                                      p.rk)
                                            : make_uint4(0, 0, 0, 0);
                        *reinterpret_cast<uint4 *>(tile + sw_byte(i, 16 * fc)) = w;
                    }
                } else if (kMode == 2 && (ks + 1) * BKE <= p.K) {
                    // KC: k values per work item, so that a group's 128 threads get one item
                    // each (BF16) or two (e4m3: 8 values, one 8-byte store per row)
                    constexpr int KC = kFp8 ? 8 : (ROWS == 64 ? 4 : 8);
                    produce_s_transposed<kFp8, KC>(tile, p, m0, ks * BKE, row_lo, ROWS, tg,
                                                   GROUP_THREADS);
                } else {
                    produce_s_generic<kFp8>(tile, p, m0, ks * BKE, row_lo, ROWS, tg,
                                            GROUP_THREADS);
                }
                tc::fence_proxy_async_smem();
                tc::named_barrier(1 + gi, GROUP_THREADS);
                if (tg == 0) {
                    if (CN > 1) {
                        // the peer's share of this stage arrives by bulk copy
                        tc::mbar_arrive_expect_tx(&full[s], PART_BYTES);
                        const uint32_t off = (uint32_t)(s * S_STAGE_BYTES + row_lo * ROW_BYTES);
                        tc::bulk_copy_to_peer(peer_tiles + off, s_tiles + off, PART_BYTES,
                                              peer_full0 + 8u * (uint32_t)s);
                    } else {
                        tc::mbar_arrive(&full[s]);
                    }
                }
                if (kMode == 1) {
#pragma unroll
                    for (int t = 0; t < FAST_ROWS; ++t)
                        ctr[t] = ctr_add_u32(ctr[t], (uint32_t)(GEN_GROUPS * (BKE / 4)));
                }
                // GEN_GROUPS <= STAGES: at most one wrap of the ring per step
                s += GEN_GROUPS;
                if (s >= STAGES) {
                    s -= STAGES;
                    ph ^= 1u;
                }
            }
        }
    }
done:
    // tensor stores still reading the staging buffers finish before the CTA exits
    if (p.out_tma && warp >= EPI_WARP0 && warp < EPI_WARP0 + 4 && lane == 0) tc::bulk_wait_all();
    tc::tc_fence_before();
    __syncwarp();
    __syncthreads();
    if (CS > 1) tc::cluster_sync();  // no CTA leaves while a peer may still signal it
    if (warp == 1) {
        __syncwarp();
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// op(A)(k, j) -> At, k-blocked with BKE values of k per block: element (k, j) at
// ((k / BKE) * npad + j) * BKE + k % BKE, so the TMA box of a stage (BKE consecutive k of 256
// consecutive j, 64 bytes each) is one contiguous block.  Rows j in [N, npad) and k in
// [K, kpad) are written as zeros.  When j has unit stride the kernels transpose a 64 (k) x 128
// (j) tile through shared memory (vector reads along j, 16-byte writes along k); when k has
// unit stride they convert in order.
__device__ __forceinline__ int64_t blocked_index(int64_t k, int64_t j, int64_t npad, int bke) {
    return ((k / bke) * npad + j) * bke + (k % bke);
}

// Loads of A in its storage type (FP32 or BF16), widened to float.
__device__ __forceinline__ float load_a(const float *p) { return *p; }
__device__ __forceinline__ float load_a(const __nv_bfloat16 *p) { return __bfloat162float(*p); }

// Four consecutive elements; `p` must be 16-byte (FP32) or 8-byte (BF16) aligned.
__device__ __forceinline__ float4 load_a4(const float *p) {
    return *reinterpret_cast<const float4 *>(p);
}
__device__ __forceinline__ float4 load_a4(const __nv_bfloat16 *p) {
    const uint2 w = *reinterpret_cast<const uint2 *>(p);
    return make_float4(__uint_as_float(w.x << 16), __uint_as_float(w.x & 0xFFFF0000u),
                       __uint_as_float(w.y << 16), __uint_as_float(w.y & 0xFFFF0000u));
}

template <typename TA>
__global__ void __launch_bounds__(256) convert_a_kernel(const TA *__restrict__ A, int64_t sk,
                                                        int64_t sj, int64_t K, int64_t N,
                                                        int64_t kpad, int64_t npad,
                                                        __nv_bfloat16 *__restrict__ At) {
    constexpr uintptr_t VEC_ALIGN = 4 * sizeof(TA) - 1;
    __shared__ float tile[64][129];
    if (sk == 1 && sj != 1) {
        // direct: 4 consecutive k of one row j per thread
        const int64_t kq = kpad / 4;
        for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < kq * npad;
             t += (int64_t)gridDim.x * blockDim.x) {
            const int64_t j = t / kq, k = (t % kq) * 4;
            float v[4] = {0.f, 0.f, 0.f, 0.f};
            if (j < N) {
                const TA *src = A + j * sj + k;
                if (k + 4 <= K && ((reinterpret_cast<uintptr_t>(src) & VEC_ALIGN) == 0)) {
                    const float4 f = load_a4(src);
                    v[0] = f.x; v[1] = f.y; v[2] = f.z; v[3] = f.w;
                } else {
                    for (int e = 0; e < 4; ++e) v[e] = k + e < K ? load_a(src + e) : 0.f;
                }
            }
            uint2 w;
            w.x = pack_bf16(v[0], v[1]);
            w.y = pack_bf16(v[2], v[3]);
            *reinterpret_cast<uint2 *>(At + blocked_index(k, j, npad, Elem<false>::BK)) = w;
        }
        return;
    }
    const int64_t tk = (kpad + 63) / 64, tj = (npad + 127) / 128;
    const bool vec = sj == 1 && (N % 4) == 0 && (sk % 4) == 0 &&
                     (reinterpret_cast<uintptr_t>(A) & VEC_ALIGN) == 0;
    for (int64_t t = blockIdx.x; t < tk * tj; t += gridDim.x) {
        const int64_t k0 = (t % tk) * 64, j0 = (t / tk) * 128;
        if (vec) {
            // 32 groups of 4 per k-row of the tile; 8 rows per pass of 256 threads
            for (int w = threadIdx.x; w < 64 * 32; w += 256) {
                const int kk = w / 32, jq = (w % 32) * 4;
                float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
                if (k0 + kk < K && j0 + jq < N) f = load_a4(A + (k0 + kk) * sk + j0 + jq);
                tile[kk][jq] = f.x;
                tile[kk][jq + 1] = f.y;
                tile[kk][jq + 2] = f.z;
                tile[kk][jq + 3] = f.w;
            }
        } else {
            for (int w = threadIdx.x; w < 64 * 128; w += 256) {
                const int kk = w / 128, jj = w % 128;
                tile[kk][jj] = (k0 + kk < K && j0 + jj < N)
                                   ? load_a(A + (k0 + kk) * sk + (j0 + jj) * sj)
                                   : 0.f;
            }
        }
        __syncthreads();
        // 128 rows j x 8 chunks of 8 k: one 16-byte store each (zeros outside K x N)
        for (int w = threadIdx.x; w < 128 * 8; w += 256) {
            const int jj = w / 8, c = w % 8;
            const int64_t k = k0 + 8 * c;
            if (j0 + jj >= npad || k >= kpad) continue;
            uint4 q;
            q.x = pack_bf16(tile[8 * c][jj], tile[8 * c + 1][jj]);
            q.y = pack_bf16(tile[8 * c + 2][jj], tile[8 * c + 3][jj]);
            q.z = pack_bf16(tile[8 * c + 4][jj], tile[8 * c + 5][jj]);
            q.w = pack_bf16(tile[8 * c + 6][jj], tile[8 * c + 7][jj]);
            *reinterpret_cast<uint4 *>(At + blocked_index(k, j0 + jj, npad, Elem<false>::BK)) = q;
        }
        __syncthreads();
    }
}

// FP8 path, pass 0: amax[g * npad + j] = max |op(A)(k, j)| over k in K slice g (float bits,
// atomicMax; the array starts zeroed).  grid.x: blocks of 256 columns (j unit stride) or of 8
// columns (otherwise, one warp per column); grid.y: chunks of at most 2048 k inside one slice.
template <typename TA>
__global__ void __launch_bounds__(256) amax_kernel(const TA *__restrict__ A, int64_t sk,
                                                   int64_t sj, int64_t K, int64_t N,
                                                   int64_t k_per_group, int64_t chunks_per_group,
                                                   uint32_t *__restrict__ amax, int64_t npad) {
    constexpr int64_t CH = 2048;
    const int64_t g = blockIdx.y / chunks_per_group;
    const int64_t kb = g * k_per_group + (blockIdx.y % chunks_per_group) * CH;
    const int64_t ke = min(min(kb + CH, (g + 1) * k_per_group), K);
    if (sj == 1) {
        const int64_t j = blockIdx.x * 256 + threadIdx.x;
        if (j >= N) return;
        float m = 0.f;
        for (int64_t k = kb; k < ke; ++k) m = fmaxf(m, fabsf(load_a(A + k * sk + j)));
        if (m > 0.f) atomicMax(amax + g * npad + j, __float_as_uint(m));
    } else {
        const int64_t j = blockIdx.x * 8 + (threadIdx.x >> 5);
        if (j >= N) return;
        const int lane = threadIdx.x & 31;
        float m = 0.f;
        for (int64_t k = kb + lane; k < ke; k += 32) m = fmaxf(m, fabsf(load_a(A + k * sk + j * sj)));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
        if (lane == 0 && m > 0.f) atomicMax(amax + g * npad + j, __float_as_uint(m));
    }
}

// FP8 path, pass 1: op(A)(k, j) / scale(g, j) -> e4m3, k-blocked with 64 k per block.
template <typename TA>
__global__ void __launch_bounds__(256) convert_a_fp8_kernel(const TA *__restrict__ A, int64_t sk,
                                                            int64_t sj, int64_t K, int64_t N,
                                                            int64_t kpad, int64_t npad,
                                                            int64_t k_per_group,
                                                            const uint32_t *__restrict__ amax,
                                                            uint8_t *__restrict__ At) {
    constexpr int BKE = Elem<true>::BK;
    constexpr uintptr_t VEC_ALIGN = 4 * sizeof(TA) - 1;
    __shared__ float tile[64][129];
    __shared__ float inv_s[128];  // 1 / scale of the tile's columns (K slice g)
    if (sk == 1 && sj != 1) {
        // direct: 16 consecutive k of one row j per thread
        const int64_t kq = kpad / 16;
        for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < kq * npad;
             t += (int64_t)gridDim.x * blockDim.x) {
            const int64_t j = t / kq, k = (t % kq) * 16;
            float v[16];
#pragma unroll
            for (int e = 0; e < 16; ++e) v[e] = 0.f;
            if (j < N) {
                const float inv = __fdiv_rn(1.0f, e4m3_scale(amax[(k / k_per_group) * npad + j]));
                const TA *src = A + j * sj + k;
                for (int e = 0; e < 16; ++e) v[e] = k + e < K ? load_a(src + e) * inv : 0.f;
            }
            *reinterpret_cast<uint4 *>(At + blocked_index(k, j, npad, BKE)) = pack_chunk<true>(v);
        }
        return;
    }
    const int64_t tk = kpad / 64, tj = (npad + 127) / 128;
    const bool vec = sj == 1 && (N % 4) == 0 && (sk % 4) == 0 &&
                     (reinterpret_cast<uintptr_t>(A) & VEC_ALIGN) == 0;
    for (int64_t t = blockIdx.x; t < tk * tj; t += gridDim.x) {
        const int64_t k0 = (t % tk) * 64, j0 = (t / tk) * 128;
        if (vec) {
            for (int w = threadIdx.x; w < 64 * 32; w += 256) {
                const int kk = w / 32, jq = (w % 32) * 4;
                float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
                if (k0 + kk < K && j0 + jq < N) f = load_a4(A + (k0 + kk) * sk + j0 + jq);
                tile[kk][jq] = f.x;
                tile[kk][jq + 1] = f.y;
                tile[kk][jq + 2] = f.z;
                tile[kk][jq + 3] = f.w;
            }
        } else {
            for (int w = threadIdx.x; w < 64 * 128; w += 256) {
                const int kk = w / 128, jj = w % 128;
                tile[kk][jj] = (k0 + kk < K && j0 + jj < N)
                                   ? load_a(A + (k0 + kk) * sk + (j0 + jj) * sj)
                                   : 0.f;
            }
        }
        // one K slice per tile (slices are whole multiples of 64 k): each column's reciprocal
        // scale once per tile, not once per 16-k chunk
        const int64_t g = k0 / k_per_group;
        if (threadIdx.x < 128 && j0 + threadIdx.x < npad)
            inv_s[threadIdx.x] = __fdiv_rn(1.0f, e4m3_scale(amax[g * npad + j0 + threadIdx.x]));
        __syncthreads();
        // 128 rows j x 4 chunks of 16 k: one 16-byte store each
        for (int w = threadIdx.x; w < 128 * 4; w += 256) {
            const int jj = w / 4, c = w % 4;
            if (j0 + jj >= npad) continue;
            const float inv = inv_s[jj];
            float v[16];
#pragma unroll
            for (int e = 0; e < 16; ++e) v[e] = tile[16 * c + e][jj] * inv;
            *reinterpret_cast<uint4 *>(At + blocked_index(k0 + 16 * c, j0 + jj, npad, BKE)) =
                pack_chunk<true>(v);
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
    bool fp8;
    int bke;  // k values per stage
    int64_t k_steps, tiles_m, tiles_n, m_groups, n_groups, groups, ks_per_group, units, kpad,
        npad;
    int cn;
    size_t at_bytes, amax_bytes, partial_bytes, total;
};

int resident_clusters(int cs);

Plan make_plan(int64_t M, int64_t N, int64_t K, bool fp8) {
    Plan pl{};
    pl.fp8 = fp8;
    pl.bke = fp8 ? Elem<true>::BK : Elem<false>::BK;
    pl.k_steps = (K + pl.bke - 1) / pl.bke;
    pl.tiles_m = (M + BM - 1) / BM;
    pl.tiles_n = (N + BN - 1) / BN;
    pl.cn = pl.tiles_n >= 2 ? 2 : 1;
    pl.m_groups = pl.tiles_m;
    pl.n_groups = (pl.tiles_n + pl.cn - 1) / pl.cn;
    const int slots = std::max(1, resident_clusters(pl.cn));
    pl.kpad = pl.k_steps * pl.bke;
    pl.npad = pl.tiles_n * BN;
    // K slices: the fewest estimated seconds -- waves of resident clusters times the k-steps of
    // a slice (about 0.3 us per k-step of a unit on GB300), plus, for more than one slice,
    // writing the partials and reading them back in the reduce pass at ~6 TB/s -- with slices
    // of >= 32 k-steps and the partial buffer at most 1 GiB
    const int64_t tiles = pl.m_groups * pl.n_groups;
    int64_t best_g = 1;
    double best = 0.0;
    const int64_t gmax = std::max<int64_t>(1, std::min<int64_t>(pl.k_steps / 32, 64));
    for (int64_t g = 1; g <= gmax; ++g) {
        if ((double)g * M * N * 4 > (double)(1ll << 30)) break;
        const int64_t units = tiles * g;
        const int64_t waves = (units + slots - 1) / slots;
        const double t = (double)waves * (double)((pl.k_steps + g - 1) / g) * 0.3e-6 +
                         (g > 1 ? (2.0 * g + 1.0) * (double)M * N * 4.0 / 6.0e12 : 0.0);
        if (g == 1 || t < best * (1.0 - 1e-9)) {
            best = t;
            best_g = g;
        }
    }
    pl.ks_per_group = (pl.k_steps + best_g - 1) / best_g;
    pl.groups = (pl.k_steps + pl.ks_per_group - 1) / pl.ks_per_group;
    pl.units = tiles * pl.groups;
    pl.at_bytes = ((size_t)pl.npad * pl.kpad * (fp8 ? 1 : 2) + 1023) / 1024 * 1024;
    pl.amax_bytes = fp8 ? ((size_t)pl.groups * pl.npad * 4 + 1023) / 1024 * 1024 : 0;
    pl.partial_bytes = pl.groups == 1 ? 0 : (size_t)pl.groups * M * N * 4;  // 1: written directly
    pl.total = pl.at_bytes + pl.amax_bytes + pl.partial_bytes;
    return pl;
}

template <int CN, int kMode, bool kFp8, int kGenWarps>
void set_smem_attr() {
    static bool done = false;
    if (!done) {
        RBG_CUDA(cudaFuncSetAttribute(sketch_tc_kernel<CN, kMode, kFp8, kGenWarps>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
        done = true;
    }
}

// One launch configuration of clusters of CN CTAs (one CTA per SM, shared memory decides).
template <int CN>
cudaLaunchConfig_t cluster_config(int clusters, int threads, cudaLaunchAttribute *attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(clusters * CN));
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = SMEM_BYTES;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CN;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

template <int CN>
int query_resident_clusters() {
    set_smem_attr<CN, 1, false, 16>();
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = cluster_config<CN>(256, GenLayout<16>::THREADS, attr);
    int n = 0;
    const cudaError_t e =
        cudaOccupancyMaxActiveClusters(&n, sketch_tc_kernel<CN, 1, false, 16>, &cfg);
    if (e != cudaSuccess || n <= 0) {
        cudaGetLastError();
        n = num_sms() / CN;
    }
    return n;
}

// Clusters of `cs` CTAs (one CTA per SM) that fit on the current device at once.
int resident_clusters(int cs) {
    static std::mutex mu;
    static int cached[64][3] = {};
    int dev = 0;
    RBG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) dev = 0;
    std::lock_guard<std::mutex> g(mu);
    int &c = cached[dev][cs];
    if (!c) c = cs == 1 ? query_resident_clusters<1>() : query_resident_clusters<2>();
    return c;
}

template <int CN, int kMode, bool kFp8, int kGenWarps>
void launch_sketch(int clusters, const CUtensorMap &map, const CUtensorMap &out_map,
                   const LowpParams &p, cudaStream_t s) {
    set_smem_attr<CN, kMode, kFp8, kGenWarps>();
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cluster_config<CN>(clusters, GenLayout<kGenWarps>::THREADS, attr);
    cfg.stream = s;
    RBG_CUDA(cudaLaunchKernelEx(&cfg, sketch_tc_kernel<CN, kMode, kFp8, kGenWarps>, map, out_map,
                                p));
    RBG_LAUNCHED();
}

// Cluster pairs sharing uniform BF16 operator rows that start on counter blocks take the
// 8-generator-warp form; everything else 16 generator warps.
template <int kMode, bool kFp8>
void launch_for(const Plan &pl, const CUtensorMap &map, const CUtensorMap &out_map,
                const LowpParams &p, cudaStream_t s) {
    const int clusters = (int)std::min<int64_t>(pl.units, resident_clusters(pl.cn));
    if constexpr (kMode == 1 && !kFp8) {
        if (pl.cn == 2 && p.gen.family == RBG_UNIFORM) {
            launch_sketch<2, kMode, kFp8, 8>(clusters, map, out_map, p, s);
            return;
        }
    }
    if (pl.cn == 2) launch_sketch<2, kMode, kFp8, 16>(clusters, map, out_map, p, s);
    else launch_sketch<1, kMode, kFp8, 16>(clusters, map, out_map, p, s);
}


CUtensorMap encode_at_map(const Plan &pl, const void *At) {
    CUtensorMap map;
    // rows of 64 bytes (bke values): row r = (k / bke) * npad + j
    const cuuint64_t dims[2] = {(cuuint64_t)pl.bke, (cuuint64_t)pl.npad * pl.k_steps};
    const cuuint64_t strides[1] = {(cuuint64_t)ROW_BYTES};
    const cuuint32_t box[2] = {(cuuint32_t)pl.bke, (cuuint32_t)(BN / 2)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult cr = tc::tensor_map_encoder()(
        &map, pl.fp8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
        const_cast<void *>(At), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
        CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) fail(RBG_ERROR_CUDA, "cuTensorMapEncodeTiled failed");
    return map;
}

bool device_memory_here(const void *ptr) {
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    int dev = -1;
    RBG_CUDA(cudaGetDevice(&dev));
    return pa.type == cudaMemoryTypeDevice && pa.device == dev;
}

// The epilogue's tensor-store target, set in p.out_tma: with one K slice, B itself when
// beta = 0 and B is device memory of this GPU with contiguous rows at a 16-byte pitch and a
// 16-byte aligned base (2D map over [M][os_i]); with several slices, the partial buffer when N
// is a multiple of 4 (3D map over [k_groups][M][N], so a box's rows past M are clipped rather
// than written into the next slice).  Otherwise the epilogue keeps plain stores.
CUtensorMap out_tensor_map(const Plan &pl, LowpParams &p) {
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    p.out_tma = 0;
    const cuuint32_t box[3] = {(cuuint32_t)EPI_COLS, 32, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult cr;
    int kind;
    if (pl.groups == 1) {
        if (p.beta != 0.f || p.os_j != 1 || (p.os_i & 3) != 0 ||
            (reinterpret_cast<uintptr_t>(p.out) & 15) != 0 || !device_memory_here(p.out))
            return map;
        const cuuint64_t dims[2] = {(cuuint64_t)p.N, (cuuint64_t)p.M};
        const cuuint64_t strides[1] = {(cuuint64_t)p.os_i * 4};
        cr = tc::tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, p.out, dims,
                                      strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                      CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        kind = 1;
    } else {
        if ((p.N & 3) != 0) return map;
        const cuuint64_t dims[3] = {(cuuint64_t)p.N, (cuuint64_t)p.M, (cuuint64_t)pl.groups};
        const cuuint64_t strides[2] = {(cuuint64_t)p.N * 4, (cuuint64_t)p.M * p.N * 4};
        cr = tc::tensor_map_encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, p.partial, dims,
                                      strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                      CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        kind = 2;
    }
    if (cr != CUDA_SUCCESS) {
        std::memset(&map, 0, sizeof map);
        return map;
    }
    p.out_tma = kind;
    return map;
}

// BF16 with A in pinned host memory: K is cut into chunks of kStreamChunk rows of op(A).  The
// copy engine brings chunk c + 1 into one of two FP32 staging buffers (cudaMemcpy2DAsync:
// op(A) row- or column-contiguous) on its own stream while the main stream converts chunk c to
// BF16 (full grid, from HBM) and sketches it on the tensor cores (all clusters).  Chunk c adds
// into B (beta for the first chunk, 1 after) with its operator columns (or rows) offset by
// c * kStreamChunk.  The host link then sets the time instead of the sum of the transfer and
// the sketch.  (Converting beside the sketch instead, on a small grid, made the sketch's
// clusters wait for SMs and the whole step 30-50 % slower and erratic.)  The last
// kStreamChunk rows go in quarter chunks: the work left after the last copy (that chunk's
// conversion and sketch) is then a quarter as long.
constexpr int64_t kStreamChunk = 1 << 16;
constexpr int64_t kStreamTail = kStreamChunk / 4;

// (first row, rows) of each chunk of K rows
std::vector<std::pair<int64_t, int64_t>> stream_chunks(int64_t K) {
    std::vector<std::pair<int64_t, int64_t>> ch;
    int64_t k0 = 0;
    for (; K - k0 > kStreamChunk; k0 += kStreamChunk) ch.emplace_back(k0, kStreamChunk);
    for (int64_t kc; k0 < K; k0 += kc) {
        kc = std::min(kStreamTail, K - k0);
        ch.emplace_back(k0, kc);
    }
    return ch;
}

bool lowp_streams(bool fp8, int64_t K, const void *A, const Strided &Q, const void *workspace) {
    if (fp8 || workspace || K < 4 * kStreamChunk || (Q.s1 != 1 && Q.s0 != 1)) return false;
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, A) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return pa.type == cudaMemoryTypeHost;  // pinned (the copy engine reads it at full rate)
}

cudaStream_t copy_stream() {
    static cudaStream_t st = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            st = nullptr;
        }
    });
    if (!st) fail(RBG_ERROR_CUDA, "could not create the copy stream");
    return st;
}

void lowp_run_streamed(int64_t M, int64_t N, int64_t K, float alpha, const DenseGen &gen,
                       int64_t r0, int64_t c0, int r_on_i, const Strided &Q, bool a_bf16,
                       float beta, float *out, int64_t os_i, int64_t os_j, cudaStream_t s) {
    const cudaStream_t cps = copy_stream();
    const int sms = num_sms();
    const auto chunks = stream_chunks(K);
    const int64_t nch = (int64_t)chunks.size();
    // one plan per chunk length (at most four distinct lengths)
    std::vector<std::pair<int64_t, Plan>> plans;
    plans.reserve(4);  // every length is planned below, before any reference is kept
    auto plan_for = [&](int64_t kc) -> const Plan & {
        for (const auto &q : plans)
            if (q.first == kc) return q.second;
        plans.emplace_back(kc, make_plan(M, N, kc, false));
        return plans.back().second;
    };
    size_t at_b = 0, part_b = 0;
    for (const auto &c : chunks) {
        const Plan &q = plan_for(c.second);
        at_b = std::max(at_b, q.at_bytes);
        part_b = std::max(part_b, q.partial_bytes);
    }
    const size_t esz = a_bf16 ? 2 : 4;
    const size_t stage_b = ((size_t)kStreamChunk * N * esz + 1023) / 1024 * 1024;
    // B in host memory: the chunks accumulate into a device copy of it (B's orientation,
    // tight pitch), which goes back once at the end.  Reading and writing host B for every
    // chunk would take the host link's H2D direction from A's copies.
    cudaPointerAttributes pb_attr{};
    bool b_host = false;
    if (cudaPointerGetAttributes(&pb_attr, out) == cudaSuccess)
        b_host = pb_attr.type == cudaMemoryTypeHost;
    else
        cudaGetLastError();
    const bool b_rows = os_j == 1;  // rows of B contiguous (else columns)
    const size_t bdev_b = b_host ? ((size_t)M * N * sizeof(float) + 1023) / 1024 * 1024 : 0;
    Scratch buf(2 * stage_b + at_b + part_b + bdev_b + 1024, s);
    uint8_t *base = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(buf.ptr) + 1023) & ~uintptr_t(1023));
    uint8_t *Af[2] = {base, base + stage_b};
    uint8_t *At = base + 2 * stage_b;
    float *partial = reinterpret_cast<float *>(base + 2 * stage_b + at_b);
    float *const out_host = out;
    const int64_t os_i_host = os_i, os_j_host = os_j;
    if (b_host) {
        out = reinterpret_cast<float *>(base + 2 * stage_b + at_b + part_b);
        os_i = b_rows ? N : 1;
        os_j = b_rows ? 1 : M;
        if (beta != 0.f)  // the first chunk reads beta * B
            RBG_CUDA(cudaMemcpy2DAsync(
                out, (size_t)(b_rows ? N : M) * sizeof(float), out_host,
                (size_t)(b_rows ? os_i_host : os_j_host) * sizeof(float),
                (size_t)(b_rows ? N : M) * sizeof(float), (size_t)(b_rows ? M : N),
                cudaMemcpyHostToDevice, s));
    }
    cudaEvent_t ready, copied[2], converted[2];
    RBG_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    for (int q = 0; q < 2; ++q) {
        RBG_CUDA(cudaEventCreateWithFlags(&copied[q], cudaEventDisableTiming));
        RBG_CUDA(cudaEventCreateWithFlags(&converted[q], cudaEventDisableTiming));
    }
    RBG_CUDA(cudaEventRecord(ready, s));  // the staging memory and earlier work on s
    RBG_CUDA(cudaStreamWaitEvent(cps, ready, 0));
    int *err = tc::wait_error_flag();
    const bool rows = Q.s1 == 1;  // op(A) rows contiguous (else columns)
    auto copy_chunk = [&](int64_t c) -> Strided {
        const int b = (int)(c & 1);
        const int64_t k0 = chunks[c].first, kc = chunks[c].second;
        // Af[b] is free once chunk c - 2 has been converted
        if (c >= 2) RBG_CUDA(cudaStreamWaitEvent(cps, converted[b], 0));
        const uint8_t *src = static_cast<const uint8_t *>(Q.ptr) + (size_t)k0 * Q.s0 * esz;
        Strided q_dev;
        q_dev.ptr = Af[b];
        if (rows) {  // [kc][N], rows of op(A) at pitch s0
            RBG_CUDA(cudaMemcpy2DAsync(Af[b], (size_t)N * esz, src, (size_t)Q.s0 * esz,
                                       (size_t)N * esz, (size_t)kc, cudaMemcpyHostToDevice,
                                       cps));
            q_dev.s0 = N;
            q_dev.s1 = 1;
        } else {     // [N][kc], columns of op(A) at pitch s1
            RBG_CUDA(cudaMemcpy2DAsync(Af[b], (size_t)kc * esz, src, (size_t)Q.s1 * esz,
                                       (size_t)kc * esz, (size_t)N, cudaMemcpyHostToDevice,
                                       cps));
            q_dev.s0 = 1;
            q_dev.s1 = kc;
        }
        RBG_CUDA(cudaEventRecord(copied[b], cps));
        return q_dev;
    };
    Strided q_next = copy_chunk(0);
    for (int64_t c = 0; c < nch; ++c) {
        const int b = (int)(c & 1);
        const int64_t k0 = chunks[c].first, kc = chunks[c].second;
        const Plan &pl = plan_for(kc);
        const Strided q_dev = q_next;
        if (c + 1 < nch) q_next = copy_chunk(c + 1);  // in flight during this chunk's work
        RBG_CUDA(cudaStreamWaitEvent(s, copied[b], 0));
        {
            ProfScope prof("lowp_convert_a", s);
            if (a_bf16)
                convert_a_kernel<<<sms * 8, 256, 0, s>>>(
                    static_cast<const __nv_bfloat16 *>(q_dev.ptr), q_dev.s0, q_dev.s1, kc, N,
                    pl.kpad, pl.npad, reinterpret_cast<__nv_bfloat16 *>(At));
            else
                convert_a_kernel<<<sms * 8, 256, 0, s>>>(
                    static_cast<const float *>(q_dev.ptr), q_dev.s0, q_dev.s1, kc, N, pl.kpad,
                    pl.npad, reinterpret_cast<__nv_bfloat16 *>(At));
            RBG_LAUNCHED();
        }
        RBG_CUDA(cudaEventRecord(converted[b], s));
        const CUtensorMap map = encode_at_map(pl, At);
        LowpParams p{};
        p.M = M; p.N = N; p.K = kc;
        p.gen = gen;
        p.rk = round_keys(gen.key);
        p.r0 = r_on_i ? r0 : r0 + k0;
        p.c0 = r_on_i ? c0 + k0 : c0;
        p.r_on_i = r_on_i;
        p.k_steps = pl.k_steps; p.m_groups = pl.m_groups; p.n_groups = pl.n_groups;
        p.ks_per_group = pl.ks_per_group; p.units = pl.units; p.npad = pl.npad;
        p.partial = partial; p.amax = nullptr; p.err = err;
        p.direct = pl.groups == 1;
        p.out = out; p.os_i = os_i; p.os_j = os_j;
        p.alpha = alpha; p.beta = c == 0 ? beta : 1.f;
        const CUtensorMap out_map = out_tensor_map(pl, p);
        {
            ProfScope prof("lowp_sketch_bf16_tc", s);
            const int mode = (p.c0 % 4) != 0 ? 0 : r_on_i ? 1 : 2;
            if (mode == 1) launch_for<1, false>(pl, map, out_map, p, s);
            else if (mode == 2) launch_for<2, false>(pl, map, out_map, p, s);
            else launch_for<0, false>(pl, map, out_map, p, s);
        }
        if (!p.direct) {
            ProfScope prof("lowp_reduce", s);
            const int64_t work = M * N;
            const int g = (int)std::max<int64_t>(
                1, std::min<int64_t>((work + 255) / 256, (int64_t)sms * 16));
            lowp_reduce_kernel<<<g, 256, 0, s>>>(M, N, pl.groups, partial, alpha, p.beta, out,
                                                 os_i, os_j);
            RBG_LAUNCHED();
        }
    }
    if (b_host)
        RBG_CUDA(cudaMemcpy2DAsync(
            out_host, (size_t)(b_rows ? os_i_host : os_j_host) * sizeof(float), out,
            (size_t)(b_rows ? N : M) * sizeof(float), (size_t)(b_rows ? N : M) * sizeof(float),
            (size_t)(b_rows ? M : N), cudaMemcpyDeviceToHost, s));
    RBG_CUDA(cudaEventDestroy(ready));
    for (int q = 0; q < 2; ++q) {
        RBG_CUDA(cudaEventDestroy(copied[q]));
        RBG_CUDA(cudaEventDestroy(converted[q]));
    }
}

void lowp_run(bool fp8, int64_t M, int64_t N, int64_t K, float alpha, const DenseGen &gen,
              int64_t r0, int64_t c0, int r_on_i, const Strided &Q, bool a_bf16, float beta,
              float *out, int64_t os_i, int64_t os_j, void *workspace, size_t ws_bytes,
              cudaStream_t s) {
    const int sms = num_sms();
    const Plan pl = make_plan(M, N, K, fp8);
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
    uint8_t *At = ws;
    uint32_t *amax = fp8 ? reinterpret_cast<uint32_t *>(ws + pl.at_bytes) : nullptr;
    float *partial = reinterpret_cast<float *>(ws + pl.at_bytes + pl.amax_bytes);

    if (fp8) {
        ProfScope prof("lowp_amax", s);
        RBG_CUDA(cudaMemsetAsync(amax, 0, pl.amax_bytes, s));
        const int64_t kpg = pl.ks_per_group * pl.bke;
        const int64_t cpg = (kpg + 2047) / 2048;
        const dim3 grid((unsigned)(Q.s1 == 1 ? (N + 255) / 256 : (N + 7) / 8),
                        (unsigned)(pl.groups * cpg));
        if (grid.y > 65535) fail(RBG_ERROR_UNSUPPORTED, "FP8 path: too many K chunks");
        if (a_bf16)
            amax_kernel<<<grid, 256, 0, s>>>(static_cast<const __nv_bfloat16 *>(Q.ptr), Q.s0,
                                             Q.s1, K, N, kpg, cpg, amax, pl.npad);
        else
            amax_kernel<<<grid, 256, 0, s>>>(static_cast<const float *>(Q.ptr), Q.s0, Q.s1, K,
                                             N, kpg, cpg, amax, pl.npad);
        RBG_LAUNCHED();
    }
    {
        ProfScope prof("lowp_convert_a", s);
        const int64_t kpg = pl.ks_per_group * pl.bke;
        if (fp8 && a_bf16)
            convert_a_fp8_kernel<<<sms * 8, 256, 0, s>>>(
                static_cast<const __nv_bfloat16 *>(Q.ptr), Q.s0, Q.s1, K, N, pl.kpad, pl.npad,
                kpg, amax, At);
        else if (fp8)
            convert_a_fp8_kernel<<<sms * 8, 256, 0, s>>>(static_cast<const float *>(Q.ptr), Q.s0,
                                                         Q.s1, K, N, pl.kpad, pl.npad, kpg, amax,
                                                         At);
        else if (a_bf16)
            convert_a_kernel<<<sms * 8, 256, 0, s>>>(static_cast<const __nv_bfloat16 *>(Q.ptr),
                                                     Q.s0, Q.s1, K, N, pl.kpad, pl.npad,
                                                     reinterpret_cast<__nv_bfloat16 *>(At));
        else
            convert_a_kernel<<<sms * 8, 256, 0, s>>>(static_cast<const float *>(Q.ptr), Q.s0,
                                                     Q.s1, K, N, pl.kpad, pl.npad,
                                                     reinterpret_cast<__nv_bfloat16 *>(At));
        RBG_LAUNCHED();
    }

    const CUtensorMap map = encode_at_map(pl, At);

    int *err = tc::wait_error_flag();
    LowpParams p{};
    p.M = M; p.N = N; p.K = K;
    p.gen = gen; p.rk = round_keys(gen.key); p.r0 = r0; p.c0 = c0; p.r_on_i = r_on_i;
    p.k_steps = pl.k_steps; p.m_groups = pl.m_groups; p.n_groups = pl.n_groups;
    p.ks_per_group = pl.ks_per_group; p.units = pl.units; p.npad = pl.npad;
    p.partial = partial; p.amax = amax; p.err = err;
    p.direct = pl.groups == 1;
    p.out = out; p.os_i = os_i; p.os_j = os_j;
    p.alpha = alpha; p.beta = beta;
    const CUtensorMap out_map = out_tensor_map(pl, p);
    // fast producers: the operator's natural column offset is a multiple of 4, so chunks
    // (natural row follows i: mode 1) or i-quads (it follows k: mode 2) start on counter blocks
    const int mode = (c0 % 4) != 0 ? 0 : r_on_i ? 1 : 2;
    {
        ProfScope prof(fp8 ? "lowp_sketch_fp8_tc" : "lowp_sketch_bf16_tc", s);
        if (fp8) {
            if (mode == 1) launch_for<1, true>(pl, map, out_map, p, s);
            else if (mode == 2) launch_for<2, true>(pl, map, out_map, p, s);
            else launch_for<0, true>(pl, map, out_map, p, s);
        } else {
            if (mode == 1) launch_for<1, false>(pl, map, out_map, p, s);
            else if (mode == 2) launch_for<2, false>(pl, map, out_map, p, s);
            else launch_for<0, false>(pl, map, out_map, p, s);
        }
    }
    if (!p.direct) {
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

namespace tc {
EncodeFn tensor_map_encoder() {
    static EncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        // cuTensorMapEncodeTiled as introduced in CUDA 12.0 (the version its ABI dates from)
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(p);
    });
    if (!fn) fail(RBG_ERROR_CUDA, "cuTensorMapEncodeTiled is not available");
    return fn;
}

int *wait_error_flag() {
    int *err = nullptr;
    RBG_CUDA(cudaGetSymbolAddress((void **)&err, g_lowp_error));
    return err;
}
}  // namespace tc
}  // namespace rbg

using namespace rbg;

extern "C" int rbg_lskge3_lowp_workspace(int32_t precision, int64_t d, int64_t n, int64_t m,
                                         size_t *bytes) {
    return guarded([&] {
        if (!bytes) fail(RBG_ERROR_INVALID_ARGUMENT, "bytes must not be NULL");
        if (precision != RBG_PREC_BF16 && precision != RBG_PREC_FP8_E4M3)
            fail(RBG_ERROR_INVALID_ARGUMENT, "precision must be RBG_PREC_BF16 or RBG_PREC_FP8_E4M3");
        RBG_REQUIRE("lskge3_lowp", d > 0 && n > 0 && m > 0);
        *bytes = make_plan(d, n, m, precision == RBG_PREC_FP8_E4M3).total;
    });
}

extern "C" int rbg_lowp_status(int32_t *code) {
    return guarded([&] {
        if (!code) fail(RBG_ERROR_INVALID_ARGUMENT, "code must not be NULL");
        int v = 0;
        RBG_CUDA(cudaMemcpyFromSymbol(&v, g_lowp_error, sizeof v));
        const int zero = 0;
        RBG_CUDA(cudaMemcpyToSymbol(g_lowp_error, &zero, sizeof zero));
        *code = v;
    });
}

namespace {
// Device memory, pinned (registered) host memory, or -- on systems where the GPU can access
// pageable memory (address translation over the host link) -- any host memory.
void require_gpu_accessible(const void *p, const char *name) {
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    if (pa.type != cudaMemoryTypeUnregistered) return;
    int dev = 0, pageable = 0;
    RBG_CUDA(cudaGetDevice(&dev));
    RBG_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
    if (!pageable)
        fail(RBG_ERROR_INVALID_ARGUMENT,
             std::string(name) + " is pageable host memory, which this GPU cannot read; pin it "
                                 "(cudaHostRegister / cudaMallocHost) or pass device memory");
}

// A caller's workspace holds the converted copy of A that the tensor-core kernel streams
// through TMA at HBM rate: it must be memory of the current GPU itself -- not another GPU's
// memory, managed memory, or host memory mapped into this GPU.
void require_current_device_memory(const void *p, const char *name) {
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
        cudaGetLastError();
        fail(RBG_ERROR_INVALID_ARGUMENT,
             std::string(name) + " must be device memory of the current GPU (its pointer "
                                 "attributes could not be read)");
    }
    int dev = -1;
    RBG_CUDA(cudaGetDevice(&dev));
    if (pa.type != cudaMemoryTypeDevice || pa.device != dev)
        fail(RBG_ERROR_INVALID_ARGUMENT,
             std::string(name) + " must be device memory of the current GPU (cudaMalloc on "
                                 "device " + std::to_string(dev) + ")");
}

int lowp_entry(int32_t precision, int32_t a_dtype, int32_t layout, int32_t opS, int32_t opA,
               int64_t d, int64_t n, int64_t m, float alpha, const rbg_dense_skop *S,
               int64_t ro_s, int64_t co_s, const void *A, int64_t lda, float beta, float *B,
               int64_t ldb, void *workspace, size_t workspace_bytes, rbg_stream_t stream) {
    return guarded([&] {
        if (precision != RBG_PREC_BF16 && precision != RBG_PREC_FP8_E4M3)
            fail(RBG_ERROR_INVALID_ARGUMENT, "precision must be RBG_PREC_BF16 or RBG_PREC_FP8_E4M3");
        if (a_dtype != RBG_F32 && a_dtype != RBG_BF16)
            fail(RBG_ERROR_INVALID_ARGUMENT, "a_dtype must be RBG_F32 or RBG_BF16");
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
        if (workspace) require_current_device_memory(workspace, "workspace");
        const cudaStream_t s = as_cuda(stream);
        const int64_t brs = layout == RBG_COL_MAJOR ? 1 : ldb;
        const int64_t bcs = layout == RBG_COL_MAJOR ? ldb : 1;
        if (m == 0 || alpha == 0.f) {
            launch_scale(RBG_F32, d, n, brs, bcs, beta, B, s);
            return;
        }
        if (!A) fail(RBG_ERROR_INVALID_ARGUMENT, "A must not be NULL");
        // A and B may live in host memory the GPU can read: the A conversion pass then reads
        // A over the host link, and B is written in place
        require_gpu_accessible(A, "A");
        require_gpu_accessible(B, "B");
        if ((double)((m + 31) / 32) * (double)((n + BN - 1) / BN * BN) > (double)INT32_MAX)
            fail(RBG_ERROR_UNSUPPORTED, "dimensions too large for 32-bit TMA coordinates");
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
        const bool fp8 = precision == RBG_PREC_FP8_E4M3;
        if (lowp_streams(fp8, m, A, Q, workspace))
            lowp_run_streamed(d, n, m, alpha, make_dense_gen(S->dist, S->seed_state), r0, c0,
                              r_on_i, Q, a_dtype == RBG_BF16, beta, B, brs, bcs, s);
        else
            lowp_run(fp8, d, n, m, alpha, make_dense_gen(S->dist, S->seed_state), r0, c0,
                     r_on_i, Q, a_dtype == RBG_BF16, beta, B, brs, bcs, workspace,
                     workspace_bytes, s);
    });
}
}  // namespace

extern "C" int rbg_lskge3_lowp(int32_t precision, int32_t layout, int32_t opS, int32_t opA,
                               int64_t d, int64_t n, int64_t m, float alpha,
                               const rbg_dense_skop *S, int64_t ro_s, int64_t co_s, const float *A,
                               int64_t lda, float beta, float *B, int64_t ldb, void *workspace,
                               size_t workspace_bytes, rbg_stream_t stream) {
    return lowp_entry(precision, RBG_F32, layout, opS, opA, d, n, m, alpha, S, ro_s, co_s, A, lda,
                      beta, B, ldb, workspace, workspace_bytes, stream);
}

extern "C" int rbg_lskge3_lowp_ex(int32_t precision, int32_t a_dtype, int32_t layout,
                                  int32_t opS, int32_t opA, int64_t d, int64_t n, int64_t m,
                                  float alpha, const rbg_dense_skop *S, int64_t ro_s,
                                  int64_t co_s, const void *A, int64_t lda, float beta, float *B,
                                  int64_t ldb, void *workspace, size_t workspace_bytes,
                                  rbg_stream_t stream) {
    return lowp_entry(precision, a_dtype, layout, opS, opA, d, n, m, alpha, S, ro_s, co_s, A, lda,
                      beta, B, ldb, workspace, workspace_bytes, stream);
}
