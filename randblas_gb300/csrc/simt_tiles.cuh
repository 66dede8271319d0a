// simt_tiles.cuh -- tile routines of the CUDA-core dense sketch, shared by the single-problem
// kernel (gemm_simt.cu) and the persistent batched kernel (batched.cu): the operator tile
// generated from its counters, and strided loads of the data tile into shared memory.
#pragma once

#include "rbg_internal.h"

namespace rbg {
namespace simt {

constexpr int BM = 128, BN = 128, BK = 16, NT = 256;  // tile M, max tile N, k step, threads

// P tile, k-major: Ps[k][i] for i in [0, TM), k in [0, BK).  Entries outside M x K are 0.
// Generated by THREADS threads of the CTA, this one being number tid, with Philox keyed by
// `key`: the operator's key (uint2), or its round keys (RoundKeys) when the caller has them in
// its kernel parameters.
template <typename T, int TM, int THREADS, typename Key>
__device__ __forceinline__ void gen_p_tile_by(T (*Ps)[TM + 4], const POperand &P, int64_t M,
                                              int64_t K, int64_t i0, int64_t k0, int tid,
                                              const Key &key) {
    const DenseGen &g = P.gen;
    if (P.r_on_i && ((P.c0 + k0) & 3) == 0 && i0 + TM <= M && k0 + BK <= K) {
        // interior tile, block-aligned: TM rows x BK / 4 whole counter blocks, no bounds
        const int64_t b0 = (P.c0 + k0) >> 2;
        for (int w = tid; w < TM * (BK / 4); w += THREADS) {
            const int i = w / (BK / 4), b = w % (BK / 4);
            float v[4];
            gen4(g.family, g.counter_of(P.r0 + i0 + i, b0 + b), key, v);
#pragma unroll
            for (int l = 0; l < 4; ++l) Ps[4 * b + l][i] = finish_entry<T>(g.family, v[l]);
        }
        return;
    }
    if (!P.r_on_i && ((P.c0 + i0) & 3) == 0 && i0 + TM <= M && k0 + BK <= K) {
        const int64_t b0 = (P.c0 + i0) >> 2;
        for (int w = tid; w < BK * (TM / 4); w += THREADS) {
            const int k = w / (TM / 4), b = w % (TM / 4);
            float v[4];
            gen4(g.family, g.counter_of(P.r0 + k0 + k, b0 + b), key, v);
#pragma unroll
            for (int l = 0; l < 4; ++l) Ps[k][4 * b + l] = finish_entry<T>(g.family, v[l]);
        }
        return;
    }
    if (P.r_on_i) {
        // R follows i, C follows k: each of the TM rows needs the counter blocks covering
        // columns [c0 + k0, c0 + k0 + BK).
        const int64_t cfirst = P.c0 + k0;
        const int64_t b0 = cfirst / 4;
        const int nb = (int)((cfirst + BK - 1) / 4 - b0 + 1);
        for (int w = tid; w < TM * nb; w += THREADS) {
            const int i = w / nb, b = w % nb;
            const bool row_ok = i0 + i < M;
            float v[4] = {0.f, 0.f, 0.f, 0.f};
            if (row_ok) gen4(g.family, g.counter_of(P.r0 + i0 + i, b0 + b), key, v);
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const int64_t k = (b0 + b) * 4 + l - cfirst;
                if (k >= 0 && k < BK)
                    Ps[k][i] = (row_ok && k0 + k < K) ? finish_entry<T>(g.family, v[l]) : (T)0;
            }
        }
    } else {
        // R follows k, C follows i: each of the BK rows needs the blocks covering columns
        // [c0 + i0, c0 + i0 + TM).
        const int64_t cfirst = P.c0 + i0;
        const int64_t b0 = cfirst / 4;
        const int nb = (int)((cfirst + TM - 1) / 4 - b0 + 1);
        for (int w = tid; w < BK * nb; w += THREADS) {
            const int k = w / nb, b = w % nb;
            const bool k_ok = k0 + k < K;
            float v[4] = {0.f, 0.f, 0.f, 0.f};
            if (k_ok) gen4(g.family, g.counter_of(P.r0 + k0 + k, b0 + b), key, v);
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const int64_t i = (b0 + b) * 4 + l - cfirst;
                if (i >= 0 && i < TM)
                    Ps[k][i] = (k_ok && i0 + i < M) ? finish_entry<T>(g.family, v[l]) : (T)0;
            }
        }
    }
}

// gen_p_tile_by with all NT threads of the CTA, keyed by the operator's key or by `key`.
template <typename T, int TM = BM>
__device__ __forceinline__ void gen_p_tile(T (*Ps)[TM + 4], const POperand &P, int64_t M,
                                           int64_t K, int64_t i0, int64_t k0) {
    gen_p_tile_by<T, TM, NT>(Ps, P, M, K, i0, k0, (int)threadIdx.x, P.gen.key);
}
template <typename T, int TM, typename Key>
__device__ __forceinline__ void gen_p_tile(T (*Ps)[TM + 4], const POperand &P, int64_t M,
                                           int64_t K, int64_t i0, int64_t k0, const Key &key) {
    gen_p_tile_by<T, TM, NT>(Ps, P, M, K, i0, k0, (int)threadIdx.x, key);
}

// ------------------------------------------------------------------ thread-block clusters
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// the shared::cluster address of the same location in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t cluster_map(uint32_t local, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}
__device__ __forceinline__ void st_cluster(uint32_t addr, float v) {
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}
__device__ __forceinline__ void st_cluster(uint32_t addr, unsigned long long v) {
    asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}
// barrier over all threads of all CTAs of the cluster, split into arrive and wait
__device__ __forceinline__ void cluster_arrive() {
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// *key when given, else the operator's own key (for callers without round keys).
template <typename Key>
__device__ __forceinline__ const Key &key_or(const Key *key, const uint2 &) { return *key; }
__device__ __forceinline__ const uint2 &key_or(const uint2 *key, const uint2 &own) {
    return key ? *key : own;
}

// An interior FP32 operator tile [BK][TM + 4] (whole, block-aligned counter blocks, as in
// gen_p_tile's fast path) generated by the CL CTAs of a cluster together: CTA `rank`
// generates 1/CL of it and stores every entry into all CL CTAs' tiles, at remote[q] + off in
// CTA q.  The caller then runs a cluster barrier before any CTA reads the tile.  `key` as in
// gen_p_tile_by.
template <int TM, int CL, typename Key>
__device__ __forceinline__ void gen_p_tile_shared(const uint32_t (&remote)[CL], uint32_t off0,
                                                  const POperand &P, int64_t i0, int64_t k0,
                                                  uint32_t rank, const Key &key) {
    const DenseGen &g = P.gen;
    constexpr uint32_t kRowB = (TM + 4) * sizeof(float);
    if (P.r_on_i) {
        constexpr int ROWS = TM / CL;  // rows of the tile per CTA
        const int64_t b0 = (P.c0 + k0) >> 2;
        for (int w = threadIdx.x; w < ROWS * (BK / 4); w += NT) {
            const int i = (int)rank * ROWS + w / (BK / 4), b = w % (BK / 4);
            float v[4];
            gen4(g.family, g.counter_of(P.r0 + i0 + i, b0 + b), key, v);
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const float e = finish_entry<float>(g.family, v[l]);
                const uint32_t off = off0 + (4 * b + l) * kRowB + i * 4u;
#pragma unroll
                for (int q = 0; q < CL; ++q) st_cluster(remote[q] + off, e);
            }
        }
    } else {
        constexpr int BLOCKS = TM / 4 / CL;  // counter blocks of a natural row per CTA
        const int64_t b0 = (P.c0 + i0) >> 2;
        for (int w = threadIdx.x; w < BK * BLOCKS; w += NT) {
            const int k = w / BLOCKS, b = (int)rank * BLOCKS + w % BLOCKS;
            float v[4];
            gen4(g.family, g.counter_of(P.r0 + k0 + k, b0 + b), key, v);
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const float e = finish_entry<float>(g.family, v[l]);
                const uint32_t off = off0 + k * kRowB + (4 * b + l) * 4u;
#pragma unroll
                for (int q = 0; q < CL; ++q) st_cluster(remote[q] + off, e);
            }
        }
    }
}

// Strided tile load into a k-major SMEM tile: dst[k][x] = src(k0 + k, x0 + x), x in [0, W).
// Threads walk the unit-stride dimension when there is one.  The data matrix is read-only
// during a sketch, so loads go through the read-only data path (also when the pointer reaches
// the kernel through memory rather than as a parameter).
template <typename T, int W>
__device__ __forceinline__ void load_tile(T (*dst)[W + 4], const T *__restrict__ src,
                                          int64_t sk, int64_t sx, int64_t K, int64_t X,
                                          int64_t k0, int64_t x0) {
    if (k0 + BK <= K && x0 + W <= X) {  // interior: no bounds
        const T *base = src + k0 * sk + x0 * sx;
        const bool x_fast = sx == 1 || sk != 1;
#pragma unroll 4
        for (int w = threadIdx.x; w < BK * W; w += NT) {
            const int k = x_fast ? w / W : w % BK, x = x_fast ? w % W : w / BK;
            dst[k][x] = __ldg(base + k * sk + x * sx);
        }
        return;
    }
    if (sx == 1 || sk != 1) {
        for (int w = threadIdx.x; w < BK * W; w += NT) {
            const int k = w / W, x = w % W;
            dst[k][x] = (k0 + k < K && x0 + x < X) ? __ldg(src + (k0 + k) * sk + (x0 + x) * sx)
                                                   : (T)0;
        }
    } else {
        for (int w = threadIdx.x; w < BK * W; w += NT) {
            const int x = w / BK, k = w % BK;
            dst[k][x] = (k0 + k < K && x0 + x < X) ? __ldg(src + (k0 + k) * sk + (x0 + x) * sx)
                                                   : (T)0;
        }
    }
}

// load_tile split in two, so the global loads of the next k step can be in flight while the
// current one is computed: load_tile_regs reads this thread's BK * W / NT elements (the same
// elements load_tile would store) into registers; store_tile_regs writes them to the tile.
template <typename T, int W>
__device__ __forceinline__ void load_tile_regs(T (&r)[BK * W / NT], const T *__restrict__ src,
                                               int64_t sk, int64_t sx, int64_t K, int64_t X,
                                               int64_t k0, int64_t x0) {
    const bool x_fast = sx == 1 || sk != 1;
    if (k0 + BK <= K && x0 + W <= X) {  // interior: no bounds
        const T *base = src + k0 * sk + x0 * sx;
#pragma unroll
        for (int e = 0; e < BK * W / NT; ++e) {
            const int w = threadIdx.x + e * NT;
            const int k = x_fast ? w / W : w % BK, x = x_fast ? w % W : w / BK;
            r[e] = __ldg(base + k * sk + x * sx);
        }
        return;
    }
#pragma unroll
    for (int e = 0; e < BK * W / NT; ++e) {
        const int w = threadIdx.x + e * NT;
        const int k = x_fast ? w / W : w % BK, x = x_fast ? w % W : w / BK;
        r[e] = (k0 + k < K && x0 + x < X) ? __ldg(src + (k0 + k) * sk + (x0 + x) * sx) : (T)0;
    }
}

template <typename T, int W>
__device__ __forceinline__ void store_tile_regs(T (*dst)[W + 4], const T (&r)[BK * W / NT],
                                                int64_t sk, int64_t sx) {
    const bool x_fast = sx == 1 || sk != 1;
#pragma unroll
    for (int e = 0; e < BK * W / NT; ++e) {
        const int w = threadIdx.x + e * NT;
        const int k = x_fast ? w / W : w % BK, x = x_fast ? w % W : w / BK;
        dst[k][x] = r[e];
    }
}

}  // namespace simt
}  // namespace rbg
