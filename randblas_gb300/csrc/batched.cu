// batched.cu -- the batching path: many independent left dense sketches
// B_i = alpha_i * submat(S_i) * A_i + beta_i * B_i (LSKGE3 semantics, RandBLAS/skge.hh:154-202,
// op = NoTrans, T = float) of uneven shapes in ONE persistent launch.  No reference
// counterpart: the reference sketches problems one call at a time.
//
// Design.  The host turns the batch into a list of work items (problem, output tile, K split),
// sorted by decreasing cost (longest-processing-time first), and uploads it with one
// descriptor per problem.  A persistent grid of two CTAs per SM takes items from an atomic
// counter.  Each item runs the CUDA-core tile of the plain path (simt_tiles.cuh: operator
// entries generated from the RNG counters, data tile staged in shared memory, 8 x (BN/16)
// FP32 accumulators per thread).  Problems with long K are split so no item dominates the
// tail; the CTA that finishes a tile's last split (an atomic per tile, no waiting) sums the
// splits' partial tiles in split order, so results do not depend on scheduling.
// The tile is chosen per problem -- by the caller (an autotuner), or here: Gaussian problems
// take row blocks (128 rows over all columns, the operator rows generated once per chunk of
// 128 k's and used by every 128-column pass, the pass accumulators parked in a per-CTA scratch
// area between chunks), so each operator entry is generated once per problem; uniform ones
// take a 128 x (128, 64 or 32) or 64 x 256 tile by a cost model.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "rbg_internal.h"
#include "simt_tiles.cuh"

namespace rbg {
namespace {

using simt::BK;
using simt::BM;
using simt::NT;

constexpr int kConfigs = 5;
// config id -> output tile (rows x columns); every configuration is 256 threads with 8 x TN
// accumulators each.  The operator tile (rows x 16 per k step) is generated once per output
// tile, so wider tiles spend less on generation per FLOP and narrower ones waste less on
// padding columns.  Configuration 5 (kRowBlock) is a row block of 128 rows over ALL of the
// problem's columns: its operator rows are generated once per chunk of kChunkK k's into shared
// memory and used by every 128-column pass, whose accumulators wait between chunks in a
// per-CTA scratch area (L2-resident), so each generated entry serves all n columns.
constexpr int kRowBlock = 5;
constexpr int kTileRows[kConfigs + 1] = {0, 128, 128, 128, 64, 128};
constexpr int kTileWidth[kConfigs + 1] = {0, 128, 64, 32, 256, 128};  // 5: width of one pass
constexpr int kMaxSplits = 64;
constexpr int kChunkK = 8 * BK;            // row-block configuration: k's per generated chunk
constexpr int kPsFloats = BK * (BM + 4);   // one operator stage (largest tile)
constexpr int kQsFloats = BK * (256 + 4);  // one data stage (largest tile)
constexpr size_t kBatchedSmem =
    sizeof(float) * (size_t)std::max(2 * (kPsFloats + kQsFloats),
                                     kChunkK * (BM + 4) + 2 * BK * (BM + 4));

struct ProbDev {
    POperand P;       // generated operator
    Strided Q;        // Q(k, j) = A(k, j)
    float *out;       // B(i, j) = out[i * os_i + j * os_j]
    int64_t os_i, os_j;
    int64_t M, N, K;  // d, n, m (K = 0 when alpha == 0 or m == 0)
    float alpha, beta;
    int32_t bm, bn;   // output tile rows and columns
    int32_t splits;
    int64_t kt_per_split;
    int64_t tiles_n;
    int64_t partial_off;  // floats into the partial buffer ([splits][M][N])
    int64_t counter_off;  // ints into the tile counters
    int32_t paired;       // column tiles taken two at a time by a cluster pair
    int32_t passes;       // row-block configuration: 128-column passes (else 0)
};

struct WorkItem {
    int32_t prob;
    int32_t split;
    int64_t tile;
};

// W consecutive floats from shared memory at a W * 4-byte aligned address, in one load.
template <int W>
__device__ __forceinline__ void load_row(const float *p, float *out) {
    if constexpr (W == 4) {
        const float4 v = *reinterpret_cast<const float4 *>(p);
        out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = v.w;
    } else if constexpr (W == 2) {
        const float2 v = *reinterpret_cast<const float2 *>(p);
        out[0] = v.x; out[1] = v.y;
    } else {
        out[0] = p[0];
    }
}

// One output tile (or one K split of it) of problem `pb`: BMT x BNT, TN columns per thread.
// kPair: the two CTAs of a cluster take column tiles `tile` and `tile + 1` (same row block,
// same split) and share the generated operator tiles, each generating half of every interior
// tile into both CTAs' stages (remote[q]: CTA q's operator stages), with one cluster barrier
// per k step.
template <int BMT, int BNT, int TN, bool kPair>
__device__ __forceinline__ void batched_tile(const ProbDev &pb, int64_t tile, int split,
                                             float *ps_raw, float *qs_raw, float *partial,
                                             int *counters, int *s_flag, uint32_t rank,
                                             const uint32_t (&remote)[2]) {
    if constexpr (kPair) tile += rank;
    constexpr int TX = BNT / TN;  // thread columns
    static_assert(TX * (BMT / 8) == NT, "one 8 x TN block per thread");
    // two stages each: stage s of the operator tile at ps_raw + s * kPsStage, of the data tile
    // at qs_raw + s * kQsStage; the next data tile is loaded into registers while the current
    // one is computed
    using PsTile = float[BK][BMT + 4];
    using QsTile = float[BK][BNT + 4];
    PsTile *Ps2 = reinterpret_cast<PsTile *>(ps_raw);
    QsTile *Qs2 = reinterpret_cast<QsTile *>(qs_raw);
    const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
    const int64_t i0 = (tile / pb.tiles_n) * BMT, j0 = (tile % pb.tiles_n) * BNT;
    const int64_t kt_total = (pb.K + BK - 1) / BK;
    const int64_t kb = (int64_t)split * pb.kt_per_split;
    const int64_t ke = min(kt_total, kb + pb.kt_per_split);
    const float *Qp = static_cast<const float *>(pb.Q.ptr);

    float acc[8][TN];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) acc[a][b] = 0.f;

    // register prefetch of the data tile up to 128 columns (the 256-wide tile would spill)
    constexpr bool kPrefetch = BNT <= 128;
    float qr[kPrefetch ? BK * BNT / NT : 1];
    if constexpr (kPrefetch)
        if (kb < ke)
            simt::load_tile_regs<float, BNT>(qr, Qp, pb.Q.s0, pb.Q.s1, pb.K, pb.N, kb * BK, j0);
    for (int64_t kt = kb; kt < ke; ++kt) {
        const int64_t k0 = kt * BK;
        const int st = (int)((kt - kb) & 1);
        float(*Ps)[BMT + 4] = Ps2[st];
        float(*Qs)[BNT + 4] = Qs2[st];
        if constexpr (kPair) {
            // the same decision in both CTAs (same row block, same k)
            const bool aligned = ((pb.P.r_on_i ? pb.P.c0 + k0 : pb.P.c0 + i0) & 3) == 0;
            if (aligned && i0 + BMT <= pb.M && k0 + BK <= pb.K)
                simt::gen_p_tile_shared<BMT, 2>(
                    remote, (uint32_t)(st * BK * (BMT + 4) * sizeof(float)), pb.P, i0, k0, rank,
                    pb.P.gen.key);
            else
                simt::gen_p_tile<float, BMT>(Ps, pb.P, pb.M, pb.K, i0, k0);
        } else {
            simt::gen_p_tile<float, BMT>(Ps, pb.P, pb.M, pb.K, i0, k0);
        }
        if constexpr (kPrefetch)
            simt::store_tile_regs<float, BNT>(Qs, qr, pb.Q.s0, pb.Q.s1);
        else
            simt::load_tile<float, BNT>(Qs, Qp, pb.Q.s0, pb.Q.s1, pb.K, pb.N, k0, j0);
        // this barrier also retires the reads of the stage written next (in both CTAs of a
        // pair)
        if constexpr (kPair) simt::cluster_arrive();
        else __syncthreads();
        if constexpr (kPrefetch)
            if (kt + 1 < ke)
                simt::load_tile_regs<float, BNT>(qr, Qp, pb.Q.s0, pb.Q.s1, pb.K, pb.N, k0 + BK,
                                                 j0);
        if constexpr (kPair) simt::cluster_wait();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            // explicit vector loads: the tiles are views of flat shared arrays, so the compiler
            // cannot prove the 16-byte alignment it would need to vectorise on its own (rows are
            // (width + 4) floats, a multiple of 16 bytes)
            float a[8], b[TN];
            const float4 a0 = *reinterpret_cast<const float4 *>(&Ps[kk][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4 *>(&Ps[kk][BMT / 2 + ty * 4]);
            a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
            a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
            load_row<TN / 2>(&Qs[kk][tx * (TN / 2)], b);
            load_row<TN / 2>(&Qs[kk][BNT / 2 + tx * (TN / 2)], b + TN / 2);
#pragma unroll
            for (int x = 0; x < 8; ++x)
#pragma unroll
                for (int y = 0; y < TN; ++y) acc[x][y] = fmaf(a[x], b[y], acc[x][y]);
        }
    }
    __syncthreads();  // the stages are free for the next item

    auto row_of = [&](int x) { return i0 + (x < 4 ? ty * 4 + x : BMT / 2 + ty * 4 + (x - 4)); };
    auto col_of = [&](int y) {
        return j0 + (y < TN / 2 ? tx * (TN / 2) + y : BNT / 2 + tx * (TN / 2) + (y - TN / 2));
    };
    if (pb.splits == 1) {
#pragma unroll
        for (int x = 0; x < 8; ++x) {
            const int64_t i = row_of(x);
            if (i >= pb.M) continue;
#pragma unroll
            for (int y = 0; y < TN; ++y) {
                const int64_t j = col_of(y);
                if (j >= pb.N) continue;
                float &o = pb.out[i * pb.os_i + j * pb.os_j];
                o = pb.beta == 0.f ? pb.alpha * acc[x][y] : fmaf(pb.alpha, acc[x][y], pb.beta * o);
            }
        }
        return;
    }
    // K split: publish this split's partial tile; the last split to finish reduces the tile
    float *mine = partial + pb.partial_off + (int64_t)split * pb.M * pb.N;
#pragma unroll
    for (int x = 0; x < 8; ++x) {
        const int64_t i = row_of(x);
        if (i >= pb.M) continue;
#pragma unroll
        for (int y = 0; y < TN; ++y) {
            const int64_t j = col_of(y);
            if (j < pb.N) mine[i * pb.N + j] = acc[x][y];
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const int done = atomicAdd(counters + pb.counter_off + tile, 1);
        *s_flag = done == pb.splits - 1;
    }
    __syncthreads();
    if (!*s_flag) return;
    __threadfence();
    const float *base = partial + pb.partial_off;
    for (int w = threadIdx.x; w < BMT * BNT; w += NT) {
        const int64_t i = i0 + w / BNT, j = j0 + w % BNT;
        if (i >= pb.M || j >= pb.N) continue;
        float sum = 0.f;
        for (int s = 0; s < pb.splits; ++s) sum += __ldcg(base + ((int64_t)s * pb.M + i) * pb.N + j);
        float &o = pb.out[i * pb.os_i + j * pb.os_j];
        o = pb.beta == 0.f ? pb.alpha * sum : fmaf(pb.alpha, sum, pb.beta * o);
    }
}

// Configuration kRowBlock: one item is a row block (128 rows) of problem `pb` over one K split
// and all of its columns, in pb.passes passes of 128 columns.  Per chunk of kChunkK k's the
// operator rows are generated once into shared memory (chunk[k][i]); each pass then loads its
// accumulators (8 x 8 per thread) from this CTA's scratch area -- zeros in the first chunk --,
// runs the chunk's k steps against staged 16 x 128 data tiles (the next tile's loads in flight
// in registers) and stores the accumulators back, or in the last chunk writes them out as the
// other configurations do (the output directly with one split, else its split slot, the last
// split summing the slots in split order).
__device__ __forceinline__ void batched_rowblock(const ProbDev &pb, int64_t tile, int split,
                                                 float *smem, float *partial, int *counters,
                                                 int *s_flag, float *scratch) {
    constexpr int BMT = 128, BNT = 128, TN = 8, TX = BNT / TN;
    static_assert(TX * (BMT / 8) == NT, "one 8 x TN block per thread");
    using ChunkRow = float[BMT + 4];
    using QsTile = float[BK][BNT + 4];
    ChunkRow *chunk = reinterpret_cast<ChunkRow *>(smem);                    // [kChunkK]
    QsTile *Qs2 = reinterpret_cast<QsTile *>(smem + kChunkK * (BMT + 4));     // [2]
    const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
    const int64_t i0 = tile * BMT;
    const int64_t kt_total = (pb.K + BK - 1) / BK;
    const int64_t kb = (int64_t)split * pb.kt_per_split;
    const int64_t ke = min(kt_total, kb + pb.kt_per_split);
    const float *Qp = static_cast<const float *>(pb.Q.ptr);
    constexpr int QR = BK * BNT / NT;
    float qr[QR];
    // the data tiles in (chunk, pass, k step) order; prefetch the first
    if (kb < ke) simt::load_tile_regs<float, BNT>(qr, Qp, pb.Q.s0, pb.Q.s1, pb.K, pb.N, kb * BK, 0);
    int stage = 0;
    auto row_of = [&](int x) { return i0 + (x < 4 ? ty * 4 + x : BMT / 2 + ty * 4 + (x - 4)); };
    if (kb >= ke) {
        // nothing to multiply (alpha == 0 or m == 0; one split): B = beta * B
        for (int w = threadIdx.x; w < BMT * pb.passes * BNT; w += NT) {
            const int64_t i = i0 + w / (pb.passes * BNT), j = w % (pb.passes * BNT);
            if (i >= pb.M || j >= pb.N) continue;
            float &o = pb.out[i * pb.os_i + j * pb.os_j];
            o = pb.beta == 0.f ? 0.f : pb.beta * o;
        }
        __syncthreads();
        return;
    }
    for (int64_t c0 = kb; c0 < ke; c0 += kChunkK / BK) {
        const int steps = (int)min((int64_t)(kChunkK / BK), ke - c0);
        const bool first = c0 == kb, last = c0 + steps == ke;
        for (int q = 0; q < steps; ++q)
            simt::gen_p_tile<float, BMT>(chunk + q * BK, pb.P, pb.M, pb.K, i0, (c0 + q) * BK);
        // (the chunk is published by the first k step's barrier below)
        for (int pass = 0; pass < pb.passes; ++pass) {
            const int64_t j0 = (int64_t)pass * BNT;
            float acc[8][TN];
            float *sc = scratch + (int64_t)pass * 64 * NT + threadIdx.x;
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int b = 0; b < TN; ++b) acc[a][b] = first ? 0.f : sc[(a * TN + b) * NT];
            for (int q = 0; q < steps; ++q) {
                float(*Qs)[BNT + 4] = Qs2[stage];
                simt::store_tile_regs<float, BNT>(Qs, qr, pb.Q.s0, pb.Q.s1);
                __syncthreads();  // the chunk (first step) and this data tile are complete
                // the next data tile in (chunk, pass, step) order
                int64_t nk = c0 + q + 1, nj = j0;
                if (q + 1 == steps) {
                    nk = c0;
                    nj = j0 + BNT;
                    if (pass + 1 == pb.passes) {
                        nk = c0 + steps;
                        nj = 0;
                    }
                }
                if (nk < ke)
                    simt::load_tile_regs<float, BNT>(qr, Qp, pb.Q.s0, pb.Q.s1, pb.K, pb.N,
                                                     nk * BK, nj);
                const float(*Ps)[BMT + 4] = chunk + q * BK;
#pragma unroll
                for (int kk = 0; kk < BK; ++kk) {
                    float a[8], b[TN];
                    const float4 a0 = *reinterpret_cast<const float4 *>(&Ps[kk][ty * 4]);
                    const float4 a1 = *reinterpret_cast<const float4 *>(&Ps[kk][BMT / 2 + ty * 4]);
                    a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
                    a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
                    const float4 b0 = *reinterpret_cast<const float4 *>(&Qs[kk][tx * 4]);
                    const float4 b1 = *reinterpret_cast<const float4 *>(&Qs[kk][BNT / 2 + tx * 4]);
                    b[0] = b0.x; b[1] = b0.y; b[2] = b0.z; b[3] = b0.w;
                    b[4] = b1.x; b[5] = b1.y; b[6] = b1.z; b[7] = b1.w;
#pragma unroll
                    for (int x = 0; x < 8; ++x)
#pragma unroll
                        for (int y = 0; y < TN; ++y) acc[x][y] = fmaf(a[x], b[y], acc[x][y]);
                }
                stage ^= 1;
            }
            if (!last) {
#pragma unroll
                for (int a = 0; a < 8; ++a)
#pragma unroll
                    for (int b = 0; b < TN; ++b) sc[(a * TN + b) * NT] = acc[a][b];
                continue;
            }
            auto col_of = [&](int y) {
                return j0 + (y < TN / 2 ? tx * (TN / 2) + y : BNT / 2 + tx * (TN / 2) + (y - TN / 2));
            };
            if (pb.splits == 1) {
#pragma unroll
                for (int x = 0; x < 8; ++x) {
                    const int64_t i = row_of(x);
                    if (i >= pb.M) continue;
#pragma unroll
                    for (int y = 0; y < TN; ++y) {
                        const int64_t j = col_of(y);
                        if (j >= pb.N) continue;
                        float &o = pb.out[i * pb.os_i + j * pb.os_j];
                        o = pb.beta == 0.f ? pb.alpha * acc[x][y]
                                           : fmaf(pb.alpha, acc[x][y], pb.beta * o);
                    }
                }
                continue;
            }
            float *mine = partial + pb.partial_off + (int64_t)split * pb.M * pb.N;
#pragma unroll
            for (int x = 0; x < 8; ++x) {
                const int64_t i = row_of(x);
                if (i >= pb.M) continue;
#pragma unroll
                for (int y = 0; y < TN; ++y) {
                    const int64_t j = col_of(y);
                    if (j < pb.N) mine[i * pb.N + j] = acc[x][y];
                }
            }
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) {
                const int done =
                    atomicAdd(counters + pb.counter_off + tile * pb.passes + pass, 1);
                *s_flag = done == pb.splits - 1;
            }
            __syncthreads();
            if (*s_flag) {
                __threadfence();
                const float *base = partial + pb.partial_off;
                for (int w = threadIdx.x; w < BMT * BNT; w += NT) {
                    const int64_t i = i0 + w / BNT, j = j0 + w % BNT;
                    if (i >= pb.M || j >= pb.N) continue;
                    float sum = 0.f;
                    for (int sp = 0; sp < pb.splits; ++sp)
                        sum += __ldcg(base + ((int64_t)sp * pb.M + i) * pb.N + j);
                    float &o = pb.out[i * pb.os_i + j * pb.os_j];
                    o = pb.beta == 0.f ? pb.alpha * sum : fmaf(pb.alpha, sum, pb.beta * o);
                }
            }
            __syncthreads();  // s_flag is rewritten by the next pass
        }
        __syncthreads();  // every pass is done with the chunk before it is regenerated
    }
    __syncthreads();  // the stages are free for the next item
}

template <bool kPair>
__device__ __forceinline__ void batched_dispatch(const ProbDev &pb, const WorkItem &item,
                                                 float *Ps, float *Qs, float *partial,
                                                 int *counters, int *s_flag, uint32_t rank,
                                                 const uint32_t (&remote)[2], float *scratch) {
    if (!kPair && pb.passes > 0)
        batched_rowblock(pb, item.tile, item.split, Ps, partial, counters, s_flag, scratch);
    else if (pb.bm == 64)
        batched_tile<64, 256, 8, kPair>(pb, item.tile, item.split, Ps, Qs, partial, counters,
                                        s_flag, rank, remote);
    else if (pb.bn == 128)
        batched_tile<128, 128, 8, kPair>(pb, item.tile, item.split, Ps, Qs, partial, counters,
                                         s_flag, rank, remote);
    else if (pb.bn == 64)
        batched_tile<128, 64, 4, kPair>(pb, item.tile, item.split, Ps, Qs, partial, counters,
                                        s_flag, rank, remote);
    else
        batched_tile<128, 32, 2, kPair>(pb, item.tile, item.split, Ps, Qs, partial, counters,
                                        s_flag, rank, remote);
}

// Launched in clusters of two.  Phase 1: pair items (items[0, n_pairs)), both CTAs of a
// cluster on the same item -- rank 0 takes it from counter 0 and stores its index into rank
// 1's shared memory before the cluster barrier.  Phase 2: single items
// (items[n_pairs, n_items)) from counter 1, each CTA on its own.
__global__ void __launch_bounds__(NT, 2)
    batched_sketch_kernel(const ProbDev *__restrict__ probs, const WorkItem *__restrict__ items,
                          int64_t n_pairs, int64_t n_items, unsigned long long *work_counter,
                          float *__restrict__ partial, int *__restrict__ counters,
                          float *__restrict__ scratch, int64_t scratch_stride) {
    extern __shared__ __align__(16) float bsm_tiles[];  // 2 operator stages, 2 data stages
    float *Ps = bsm_tiles;
    float *Qs = bsm_tiles + 2 * kPsFloats;
    __shared__ ProbDev s_pb;
    __shared__ WorkItem s_item;
    __shared__ int s_flag;
    __shared__ unsigned long long s_w;
    const uint32_t rank = simt::cluster_rank();
    const uint32_t ps_local = (uint32_t)__cvta_generic_to_shared(Ps);
    const uint32_t remote[2] = {simt::cluster_map(ps_local, 0), simt::cluster_map(ps_local, 1)};
    const uint32_t peer_w =
        simt::cluster_map((uint32_t)__cvta_generic_to_shared(&s_w), rank ^ 1u);
    simt::cluster_arrive();  // both CTAs run before any store into the other
    simt::cluster_wait();
    for (;;) {
        if (rank == 0 && threadIdx.x == 0) {
            const unsigned long long w = atomicAdd(work_counter, 1ull);
            s_w = w;
            simt::st_cluster(peer_w, w);
        }
        simt::cluster_arrive();
        simt::cluster_wait();
        if (s_w >= (unsigned long long)n_pairs) break;  // the same in both CTAs
        if (threadIdx.x == 0) {
            s_item = items[s_w];
            s_pb = probs[s_item.prob];
        }
        __syncthreads();
        batched_dispatch<true>(s_pb, s_item, Ps, Qs, partial, counters, &s_flag, rank, remote,
                               nullptr);
        // both CTAs are done with this item's stages and with s_w before the next fetch
        simt::cluster_arrive();
        simt::cluster_wait();
    }
    for (;;) {
        if (threadIdx.x == 0) {
            s_w = (unsigned long long)n_pairs + atomicAdd(work_counter + 1, 1ull);
            if (s_w < (unsigned long long)n_items) {
                s_item = items[s_w];
                s_pb = probs[s_item.prob];
            }
        }
        __syncthreads();
        if (s_w >= (unsigned long long)n_items) break;
        batched_dispatch<false>(s_pb, s_item, Ps, Qs, partial, counters, &s_flag, rank, remote,
                                scratch + (int64_t)blockIdx.x * scratch_stride);
        __syncthreads();  // s_pb / s_item / s_w are rewritten by the next fetch
    }
}

void set_batched_smem_attr() {
    static bool done = false;
    if (done) return;
    RBG_CUDA(cudaFuncSetAttribute(batched_sketch_kernel,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kBatchedSmem));
    done = true;
}

int resident_batched_ctas() {
    int per_sm = 0;
    set_batched_smem_attr();
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_sketch_kernel, NT,
                                                      kBatchedSmem) !=
            cudaSuccess ||
        per_sm <= 0) {
        cudaGetLastError();
        per_sm = 1;
    }
    return per_sm * num_sms();
}

// Tile for a problem the caller left to the library.  Gaussian operators take row blocks.
// Uniform ones take the cheapest tile by a cost model, per k step of 16 and in thread
// instructions: FMAs over the whole (padded) tile, plus generating its operator rows, plus
// staging the data tile.  The 64 x 256 tile runs about 1.3x slower per FMA than the 128-row
// tiles (two more shared-memory wavefronts per k step for its data rows, no register
// prefetch).
int default_config(int64_t m_rows, int64_t n, int family) {
    // Gaussian operators: row blocks, whose entries are generated once for all columns
    // (measured faster than every other configuration in each n class of 16..512, up to 1.25x
    // for n > 256)
    if (family == RBG_GAUSSIAN) return kRowBlock;
    int best = 1;
    double best_cost = 0.0;
    for (int c = 1; c < kRowBlock; ++c) {
        const double bm = kTileRows[c], bn = kTileWidth[c];
        const int64_t tiles_n = (n + kTileWidth[c] - 1) / kTileWidth[c];
        const double gen = 10.0;  // uniform entries
        const double tiles = (double)((m_rows + kTileRows[c] - 1) / kTileRows[c]) * tiles_n;
        const double cost = tiles * (bm * bn * (bm == 64 ? 1.3 : 1.0) + bm * gen + 2.0 * bn);
        if (c == 1 || cost < best_cost * 0.999) {
            best_cost = cost;
            best = c;
        }
    }
    return best;
}

}  // namespace
}  // namespace rbg

// The device memory and launch shape of one batch (the opaque rbg_batched_plan of the C ABI).
struct rbg_batched_plan_s {
    int64_t n_items = 0;
    int64_t n_pairs = 0;  // pair items at the front of the item list
    int grid = 0;
    int64_t scratch_stride = 0;  // floats of row-block accumulator scratch per CTA
    bool stream_ordered = false;  // memory from cudaMallocAsync (freed on a stream)
    void *mem = nullptr;
    rbg::ProbDev *probs = nullptr;
    rbg::WorkItem *items = nullptr;
    unsigned long long *work_counter = nullptr;  // pair and single counters, then the tile counters
    int *counters = nullptr;
    size_t counter_bytes = 0;  // work counter + tile counters, zeroed before each run
    float *partial = nullptr;
    float *scratch = nullptr;  // grid x scratch_stride floats
    size_t bytes = 0;
};

namespace rbg {
namespace {
using BatchedPlan = rbg_batched_plan_s;

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// Validate the problems and build the descriptors and the sorted work list (host only).
// Columns an item of problem `pd` covers: its tile width, or every pass of a row block.
int64_t item_width(const ProbDev &pd) { return pd.passes ? (int64_t)pd.passes * pd.bn : pd.bn; }

void build_plan(int32_t layout, const rbg_batch_problem *problems, int64_t count,
                int32_t tile_config, std::vector<ProbDev> &descs, std::vector<WorkItem> &items,
                int64_t &n_pairs, int64_t &partial_floats, int64_t &tile_counters, int &grid,
                int64_t &scratch_stride) {
    if (layout != RBG_COL_MAJOR && layout != RBG_ROW_MAJOR)
        fail(RBG_ERROR_INVALID_ARGUMENT, "layout must be RBG_COL_MAJOR or RBG_ROW_MAJOR");
    if (count < 0) fail(RBG_ERROR_INVALID_ARGUMENT, "count must be >= 0");
    if (count > 0 && !problems) fail(RBG_ERROR_INVALID_ARGUMENT, "problems must not be NULL");
    if (count > INT32_MAX) fail(RBG_ERROR_INVALID_ARGUMENT, "too many problems");
    if (tile_config < 0 || tile_config > kConfigs)
        fail(RBG_ERROR_INVALID_ARGUMENT, "tile_config must be 0 or a listed configuration");
    descs.clear();
    items.clear();
    std::vector<WorkItem> pairs;
    n_pairs = 0;
    partial_floats = 0;
    tile_counters = 0;
    scratch_stride = 0;
    std::vector<int64_t> kt(count, 0);
    double total_cost = 0.0;
    descs.resize(count);
    for (int64_t p = 0; p < count; ++p) {
        const rbg_batch_problem &q = problems[p];
        ProbDev &pd = descs[p];
        std::memset(&pd, 0, sizeof pd);
        RBG_REQUIRE("lskge3_batched", q.d >= 0 && q.n >= 0 && q.m >= 0);
        RBG_REQUIRE("lskge3_batched", q.ro_s >= 0 && q.co_s >= 0);
        RBG_REQUIRE("DenseDist", q.dist.n_rows > 0);
        RBG_REQUIRE("DenseDist", q.dist.n_cols > 0);
        if (q.dist.family != RBG_GAUSSIAN && q.dist.family != RBG_UNIFORM)
            fail(RBG_ERROR_INVALID_ARGUMENT, "Unrecognized ScalarDist.");
        RBG_REQUIRE("lskge3_batched", q.dist.n_rows >= q.d + q.ro_s);
        RBG_REQUIRE("lskge3_batched", q.dist.n_cols >= q.m + q.co_s);
        if (layout == RBG_COL_MAJOR) {
            RBG_REQUIRE("lskge3_batched", q.lda >= q.m);
            RBG_REQUIRE("lskge3_batched", q.ldb >= q.d);
        } else {
            RBG_REQUIRE("lskge3_batched", q.lda >= q.n);
            RBG_REQUIRE("lskge3_batched", q.ldb >= q.n);
        }
        const int32_t cfg = tile_config ? tile_config : q.tile_config;
        if (cfg < 0 || cfg > kConfigs)
            fail(RBG_ERROR_INVALID_ARGUMENT, "tile_config must be 0 or a listed configuration");
        pd.M = q.d;
        pd.N = q.n;
        pd.K = (q.alpha == 0.f) ? 0 : q.m;  // alpha == 0: A and S are not read
        pd.alpha = q.alpha;
        pd.beta = q.beta;
        if (pd.M == 0 || pd.N == 0) continue;
        if (!q.B) fail(RBG_ERROR_INVALID_ARGUMENT, "B must not be NULL");
        if (pd.K > 0 && !q.A) fail(RBG_ERROR_INVALID_ARGUMENT, "A must not be NULL");
        const DenseInfo info = dense_info(q.dist);
        pd.P.gen = make_dense_gen(q.dist, q.seed);
        if (info.natural_layout == RBG_ROW_MAJOR) {
            pd.P.r_on_i = 1;
            pd.P.r0 = q.ro_s;
            pd.P.c0 = q.co_s;
        } else {
            pd.P.r_on_i = 0;
            pd.P.r0 = q.co_s;
            pd.P.c0 = q.ro_s;
        }
        pd.P.buff = nullptr;
        pd.Q = layout == RBG_ROW_MAJOR ? Strided{q.A, q.lda, 1} : Strided{q.A, 1, q.lda};
        pd.out = q.B;
        pd.os_i = layout == RBG_ROW_MAJOR ? q.ldb : 1;
        pd.os_j = layout == RBG_ROW_MAJOR ? 1 : q.ldb;
        const int c = cfg ? cfg : default_config(pd.M, pd.N, q.dist.family);
        pd.bm = kTileRows[c];
        pd.bn = kTileWidth[c];
        pd.tiles_n = (pd.N + pd.bn - 1) / pd.bn;
        if (c == kRowBlock) {
            // one item per row block, covering every column in passes
            pd.passes = (int32_t)pd.tiles_n;
            pd.tiles_n = 1;
            scratch_stride = std::max<int64_t>(scratch_stride, (int64_t)pd.passes * 64 * NT);
        }
        kt[p] = (pd.K + BK - 1) / BK;
        const int64_t tiles = ((pd.M + pd.bm - 1) / pd.bm) * pd.tiles_n;
        total_cost += (double)tiles * (double)std::max<int64_t>(kt[p], 1) * pd.bm *
                      (double)item_width(pd);
    }
    // split long K so that no item costs more than ~1/8 of a CTA's fair share (the device is
    // queried only after every argument has been checked)
    grid = std::max(2, resident_batched_ctas() & ~1);  // clusters of two
    const double cap = std::max(total_cost / (8.0 * std::max(grid, 1)), 128.0 * 128.0 * 64.0);
    for (int64_t p = 0; p < count; ++p) {
        ProbDev &pd = descs[p];
        if (pd.M == 0 || pd.N == 0) continue;
        const int64_t tiles = ((pd.M + pd.bm - 1) / pd.bm) * pd.tiles_n;
        const int64_t cap_kt =
            std::max<int64_t>(32, (int64_t)(cap / ((double)pd.bm * (double)item_width(pd))));
        int64_t splits = kt[p] > 0 ? (kt[p] + cap_kt - 1) / cap_kt : 1;
        splits = std::min<int64_t>(splits, kMaxSplits);
        pd.kt_per_split = kt[p] > 0 ? (kt[p] + splits - 1) / splits : 0;
        splits = kt[p] > 0 ? (kt[p] + pd.kt_per_split - 1) / pd.kt_per_split : 1;
        pd.splits = (int32_t)splits;
        if (splits > 1) {
            pd.partial_off = partial_floats;
            partial_floats += splits * pd.M * pd.N;
            pd.counter_off = tile_counters;
            tile_counters += tiles * std::max<int64_t>(1, pd.passes);
        }
        // split-major: the items running at the same time share a K range, so each slab of A
        // is read from HBM once and reused from L2 by every output tile that needs it
        // Gaussian operators over two or more column tiles: column tiles (2j, 2j + 1) of a row
        // block go to a cluster pair that shares the generated operator tiles (a last odd
        // column tile stays a single item)
        pd.paired = pd.P.gen.family == RBG_GAUSSIAN && pd.tiles_n >= 2 && pd.passes == 0;
        const int64_t tm = (pd.M + pd.bm - 1) / pd.bm;
        for (int64_t sp = 0; sp < splits; ++sp)
            for (int64_t it = 0; it < tm; ++it)
                for (int64_t jt = 0; jt < pd.tiles_n; ++jt) {
                    const int64_t t = it * pd.tiles_n + jt;
                    if (pd.paired && jt + 1 < pd.tiles_n && jt % 2 == 0)
                        pairs.push_back(WorkItem{(int32_t)p, (int32_t)sp, t});
                    else if (!pd.paired || jt % 2 == 0)
                        items.push_back(WorkItem{(int32_t)p, (int32_t)sp, t});
                }
    }
    // longest processing time first; ties keep problem order (and the split-major order)
    auto lpt = [&](const WorkItem &a, const WorkItem &b) {
        const ProbDev &pa = descs[a.prob], &pb = descs[b.prob];
        return (double)pa.kt_per_split * pa.bm * (double)item_width(pa) >
               (double)pb.kt_per_split * pb.bm * (double)item_width(pb);
    };
    std::stable_sort(pairs.begin(), pairs.end(), lpt);
    std::stable_sort(items.begin(), items.end(), lpt);
    n_pairs = (int64_t)pairs.size();
    items.insert(items.begin(), pairs.begin(), pairs.end());
}

void execute_plan(const BatchedPlan &pl, cudaStream_t s) {
    if (pl.n_items == 0) return;
    RBG_CUDA(cudaMemsetAsync(pl.work_counter, 0, pl.counter_bytes, s));
    ProfScope prof("batched_sketch", s);
    set_batched_smem_attr();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)pl.grid);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = kBatchedSmem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    RBG_CUDA(cudaLaunchKernelEx(&cfg, batched_sketch_kernel, (const ProbDev *)pl.probs,
                                (const WorkItem *)pl.items, pl.n_pairs, pl.n_items,
                                pl.work_counter, pl.partial, pl.counters, pl.scratch,
                                pl.scratch_stride));
    RBG_LAUNCHED();
}

// Lay the plan's device memory out and upload descriptors and items.
void upload_plan(BatchedPlan &pl, const std::vector<ProbDev> &descs,
                 const std::vector<WorkItem> &items, int64_t n_pairs, int64_t partial_floats,
                 int64_t tile_counters, cudaStream_t s, bool stream_ordered) {
    const size_t probs_b = align256(descs.size() * sizeof(ProbDev));
    const size_t items_b = align256(items.size() * sizeof(WorkItem));
    const size_t ctr_b =
        align256(2 * sizeof(unsigned long long) + (size_t)tile_counters * sizeof(int));
    const size_t part_b = align256((size_t)partial_floats * sizeof(float));
    const size_t scr_b = align256((size_t)pl.grid * (size_t)pl.scratch_stride * sizeof(float));
    pl.bytes = probs_b + items_b + ctr_b + part_b + scr_b;
    pl.stream_ordered = stream_ordered;
    if (stream_ordered)
        RBG_CUDA(cudaMallocAsync(&pl.mem, std::max<size_t>(pl.bytes, 256), s));
    else
        RBG_CUDA(cudaMalloc(&pl.mem, std::max<size_t>(pl.bytes, 256)));
    uint8_t *base = static_cast<uint8_t *>(pl.mem);
    pl.probs = reinterpret_cast<ProbDev *>(base);
    pl.items = reinterpret_cast<WorkItem *>(base + probs_b);
    pl.work_counter = reinterpret_cast<unsigned long long *>(base + probs_b + items_b);
    pl.counters = reinterpret_cast<int *>(pl.work_counter + 2);
    pl.counter_bytes = 2 * sizeof(unsigned long long) + (size_t)tile_counters * sizeof(int);
    pl.partial = reinterpret_cast<float *>(base + probs_b + items_b + ctr_b);
    pl.scratch = reinterpret_cast<float *>(base + probs_b + items_b + ctr_b + part_b);
    pl.n_items = (int64_t)items.size();
    pl.n_pairs = n_pairs;
    if (!descs.empty())
        RBG_CUDA(cudaMemcpyAsync(pl.probs, descs.data(), descs.size() * sizeof(ProbDev),
                                 cudaMemcpyHostToDevice, s));
    if (!items.empty())
        RBG_CUDA(cudaMemcpyAsync(pl.items, items.data(), items.size() * sizeof(WorkItem),
                                 cudaMemcpyHostToDevice, s));
    if (!stream_ordered) RBG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace
}  // namespace rbg

using namespace rbg;

extern "C" int rbg_batched_tile_configs(int32_t *count) {
    if (!count) {
        set_last_error("count must not be NULL");
        return RBG_ERROR_INVALID_ARGUMENT;
    }
    *count = kConfigs;
    return RBG_SUCCESS;
}

extern "C" int rbg_batched_tile_shape(int32_t config, int32_t *rows, int32_t *cols) {
    return guarded([&] {
        if (!rows || !cols) fail(RBG_ERROR_INVALID_ARGUMENT, "rows and cols must not be NULL");
        if (config < 1 || config > kConfigs)
            fail(RBG_ERROR_INVALID_ARGUMENT, "config must be one of the listed configurations");
        *rows = kTileRows[config];
        *cols = config == kRowBlock ? 0 : kTileWidth[config];  // 0: every column
    });
}

extern "C" int rbg_batched_plan_create(int32_t layout, const rbg_batch_problem *problems,
                                       int64_t count, int32_t tile_config,
                                       rbg_batched_plan *plan) {
    return guarded([&] {
        if (!plan) fail(RBG_ERROR_INVALID_ARGUMENT, "plan must not be NULL");
        *plan = nullptr;
        std::vector<ProbDev> descs;
        std::vector<WorkItem> items;
        int64_t partial_floats = 0, tile_counters = 0;
        int grid = 0;
        int64_t n_pairs = 0;
        int64_t scratch_stride = 0;
        build_plan(layout, problems, count, tile_config, descs, items, n_pairs, partial_floats,
                   tile_counters, grid, scratch_stride);
        auto *pl = new BatchedPlan();
        pl->grid = grid;
        pl->scratch_stride = scratch_stride;
        try {
            upload_plan(*pl, descs, items, n_pairs, partial_floats, tile_counters, nullptr,
                        false);
        } catch (...) {
            if (pl->mem) cudaFree(pl->mem);
            delete pl;
            throw;
        }
        *plan = pl;
    });
}

extern "C" int rbg_batched_plan_execute(rbg_batched_plan plan, rbg_stream_t stream) {
    return guarded([&] {
        if (!plan) fail(RBG_ERROR_INVALID_ARGUMENT, "plan must not be NULL");
        execute_plan(*plan, as_cuda(stream));
    });
}

extern "C" int rbg_batched_plan_info(rbg_batched_plan plan, int64_t *work_items,
                                     int64_t *device_bytes) {
    return guarded([&] {
        if (!plan) fail(RBG_ERROR_INVALID_ARGUMENT, "plan must not be NULL");
        if (work_items) *work_items = plan->n_items;
        if (device_bytes) *device_bytes = (int64_t)plan->bytes;
    });
}

extern "C" int rbg_batched_plan_destroy(rbg_batched_plan plan) {
    return guarded([&] {
        if (!plan) return;
        if (plan->mem) RBG_CUDA(cudaFree(plan->mem));
        delete plan;
    });
}

extern "C" int rbg_lskge3_batched(int32_t layout, const rbg_batch_problem *problems,
                                  int64_t count, int32_t tile_config, rbg_stream_t stream) {
    return guarded([&] {
        const cudaStream_t s = as_cuda(stream);
        std::vector<ProbDev> descs;
        std::vector<WorkItem> items;
        int64_t partial_floats = 0, tile_counters = 0;
        int grid = 0;
        int64_t n_pairs = 0;
        int64_t scratch_stride = 0;
        build_plan(layout, problems, count, tile_config, descs, items, n_pairs, partial_floats,
                   tile_counters, grid, scratch_stride);
        if (items.empty()) return;
        BatchedPlan pl;
        pl.grid = grid;
        pl.scratch_stride = scratch_stride;
        upload_plan(pl, descs, items, n_pairs, partial_floats, tile_counters, s, true);
        execute_plan(pl, s);
        RBG_CUDA(cudaFreeAsync(pl.mem, s));
    });
}
