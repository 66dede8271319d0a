// fill.cu -- sampling kernels: dense operators (fill_dense), SASOs (repeated Fisher-Yates)
// and LASOs (iid indices with duplicate merging), plus the beta-scaling kernel.
#include <algorithm>
#include <vector>

#include "rbg_internal.h"

namespace rbg {
namespace {

// ------------------------------------------------------------------ fill_dense
// One CTA fills a 32 (R) x 128 (C) tile of the natural block: 32 x 33 Philox calls (the C
// window is not aligned to counter blocks), staged in shared memory, then written out
// coalesced in either orientation.  Every entry is a function of (R, C) alone, so the
// result does not depend on the launch shape (the reference's thread-count invariance,
// RandBLAS/DevNotes.md:12-14).
constexpr int kFillTR = 32;
constexpr int kFillTC = 128;

template <typename T>
__global__ void __launch_bounds__(256) fill_dense_kernel(DenseGen g,
                                                         const __grid_constant__ RoundKeys rk,
                                                         int64_t R0, int64_t C0,
                                                         int64_t nr, int64_t nc, int transpose_out,
                                                         T *__restrict__ out) {
    __shared__ T tile[kFillTR][kFillTC + 1];
    const int64_t tiles_c = (nc + kFillTC - 1) / kFillTC;
    const int64_t tiles_r = (nr + kFillTR - 1) / kFillTR;
    for (int64_t t = blockIdx.x; t < tiles_c * tiles_r; t += gridDim.x) {
        const int64_t tr = t / tiles_c, tc = t % tiles_c;
        const int64_t rb = tr * kFillTR;                  // first local row
        const int64_t cb = tc * kFillTC;                  // first local column
        const int64_t cabs = C0 + cb;                     // first natural column
        const int64_t blk0 = cabs / 4;                    // first counter block
        const int nblk = (int)((cabs + kFillTC - 1) / 4 - blk0 + 1);
        for (int w = threadIdx.x; w < kFillTR * nblk; w += blockDim.x) {
            const int lr = w / nblk, b = w % nblk;
            const int64_t R = R0 + rb + lr;
            if (rb + lr >= nr) continue;
            float v[4];
            gen4(g.family, g.counter_of(R, blk0 + b), rk, v);
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const int64_t lc = (blk0 + b) * 4 + l - cabs;  // column inside the tile
                if (lc >= 0 && lc < kFillTC) tile[lr][lc] = finish_entry<T>(g.family, v[l]);
            }
        }
        __syncthreads();
        if (!transpose_out) {
            for (int w = threadIdx.x; w < kFillTR * kFillTC; w += blockDim.x) {
                const int lr = w / kFillTC, lc = w % kFillTC;
                if (rb + lr < nr && cb + lc < nc) out[(rb + lr) * nc + cb + lc] = tile[lr][lc];
            }
        } else {
            for (int w = threadIdx.x; w < kFillTR * kFillTC; w += blockDim.x) {
                const int lc = w / kFillTR, lr = w % kFillTR;
                if (rb + lr < nr && cb + lc < nc) out[(cb + lc) * nr + rb + lr] = tile[lr][lc];
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ SASO
// One thread per minor index i runs the vec_nnz steps of a partial Fisher-Yates shuffle of
// the identity over [0, dim_major) (RandBLAS/sparse_skops.hh:51-106).  Step j uses counter
// seed + i*vec_nnz + j and swaps positions j and ell = j + x0 mod (dim_major - j).  Only
// positions >= j can still change, so the thread keeps a small map from "touched
// positions" to their values instead of the O(dim_major) workspace.
constexpr int kSasoLocalCap = 64;

template <typename V, typename I>
__device__ __forceinline__ void saso_vector(const DevState &s, int64_t vec_nnz,
                                            int64_t dim_major, int64_t i, I *idx_major,
                                            I *idx_minor, V *vals, int64_t *map_pos,
                                            int64_t *map_val) {
    int msize = 0;
    const int64_t off = i * vec_nnz;
    for (int64_t j = 0; j < vec_nnz; ++j) {
        const uint4 r = philox(ctr_add(s.ctr, (uint64_t)(off + j)), s.key);
        const int64_t span = dim_major - j;
        const int64_t ell = j + (int64_t)((uint64_t)r.x % (uint64_t)span);
        // current values at positions j and ell
        int64_t vj = j, vl = ell;
        int sj = -1, sl = -1;
        for (int q = 0; q < msize; ++q) {
            if (map_pos[q] == j) { vj = map_val[q]; sj = q; }
            if (map_pos[q] == ell) { vl = map_val[q]; sl = q; }
        }
        // position j becomes final (value vl); position ell takes vj
        if (ell != j) {
            if (sl >= 0) {
                map_val[sl] = vj;
            } else {
                map_pos[msize] = ell;
                map_val[msize] = vj;
                ++msize;
            }
        }
        if (sj >= 0) {  // j is final now: drop it from the map
            --msize;
            map_pos[sj] = map_pos[msize];
            map_val[sj] = map_val[msize];
        }
        idx_major[off + j] = (I)vl;
        if (idx_minor) idx_minor[off + j] = (I)i;
        if (vals) vals[off + j] = (r.y % 2u == 0u) ? (V)1 : (V)-1;
    }
}

template <typename V, typename I>
__global__ void saso_kernel(DevState s, int64_t vec_nnz, int64_t dim_major, int64_t dim_minor,
                            I *idx_major, I *idx_minor, V *vals, int64_t *scratch) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    int64_t lpos[kSasoLocalCap], lval[kSasoLocalCap];
    int64_t *mp = lpos, *mv = lval;
    if (vec_nnz > kSasoLocalCap) {
        mp = scratch + tid * 2 * vec_nnz;
        mv = mp + vec_nnz;
    }
    for (int64_t i = tid; i < dim_minor; i += nthreads)
        saso_vector(s, vec_nnz, dim_major, i, idx_major, idx_minor, vals, mp, mv);
}

// dim_major < 2^32 and vec_nnz <= kSasoFastMaxNnz (operators of any practical size): the
// 32-bit sampler (saso_column), 128 minor indices per block, with the block's entries staged
// in shared memory so that the stores of all three arrays are contiguous.
template <typename V, typename I>
__global__ void __launch_bounds__(128) saso_fast_kernel(DevState s,
                                                        const __grid_constant__ RoundKeys rk,
                                                        int vec_nnz, uint32_t dim_major,
                                                        int64_t dim_minor, I *idx_major,
                                                        I *idx_minor, V *vals) {
    __shared__ I smaj[128 * kSasoFastMaxNnz];
    __shared__ V sval[128 * kSasoFastMaxNnz];
    for (int64_t base = blockIdx.x * 128ll; base < dim_minor; base += gridDim.x * 128ll) {
        const int64_t i = base + threadIdx.x;
        if (i < dim_minor)
            saso_column(s, rk, (uint64_t)i, vec_nnz, dim_major,
                        [&](int j, uint32_t major, bool neg) {
                            smaj[threadIdx.x * vec_nnz + j] = (I)major;
                            sval[threadIdx.x * vec_nnz + j] = neg ? (V)-1 : (V)1;
                        });
        __syncthreads();
        const int64_t n = min((int64_t)128, dim_minor - base) * vec_nnz, off = base * vec_nnz;
        for (int64_t t = threadIdx.x; t < n; t += 128) {
            idx_major[off + t] = smaj[t];
            if (idx_minor) idx_minor[off + t] = (I)(base + t / vec_nnz);
            if (vals) vals[off + t] = sval[t];
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ LASO
// One thread per minor index i: vec_nnz iid samples over [0, dim_major) with Rademacher
// signs (RandBLAS/util.hh:516-546: sample j of the vector uses counter
// seed + i*ceil(vec_nnz/2) + j/2, lanes 2*(j%2) and 2*(j%2)+1), then duplicate merging
// to sqrt(count) * first sign (RandBLAS/sparse_skops.hh:453-491) in first-occurrence order.
// Pass 1 writes each vector at slot i*vec_nnz of a temporary and its distinct count.
template <typename V>
__global__ void laso_sample_kernel(DevState s, int64_t vec_nnz, int64_t dim_major,
                                   int64_t dim_minor, int64_t *tmp_idx, V *tmp_val,
                                   int64_t *counts, int64_t *cnt_scratch) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    const int64_t per_vec = (vec_nnz + 1) / 2;
    const double dn = (double)dim_major;
    for (int64_t i = tid; i < dim_minor; i += nthreads) {
        int64_t *idx = tmp_idx + i * vec_nnz;
        V *val = tmp_val + i * vec_nnz;
        int64_t *cnt = cnt_scratch + i * vec_nnz;
        const uint4 base = ctr_add(s.ctr, (uint64_t)(i * per_vec));
        int64_t distinct = 0;
        uint4 r = make_uint4(0, 0, 0, 0);
        for (int64_t j = 0; j < vec_nnz; ++j) {
            if ((j & 1) == 0) r = philox(ctr_add(base, (uint64_t)(j / 2)), s.key);
            const uint32_t xi = (j & 1) ? r.z : r.x;
            const uint32_t xs = (j & 1) ? r.w : r.y;
            const double u = __ddiv_rn(__dadd_rn((double)uneg11(xi), 1.0), 2.0);
            const int64_t k = (int64_t)__dmul_rn(dn, u);
            const V sign = uneg11(xs) >= 0.0f ? (V)1 : (V)-1;
            int64_t found = -1;
            for (int64_t q = 0; q < distinct; ++q)
                if (idx[q] == k) { found = q; break; }
            if (found >= 0) {
                cnt[found] += 1;
            } else {
                idx[distinct] = k;
                val[distinct] = sign;
                cnt[distinct] = 1;
                ++distinct;
            }
        }
        for (int64_t q = 0; q < distinct; ++q) {
            if (cnt[q] > 1) val[q] = (V)(sqrt((V)cnt[q]) * val[q]);
        }
        counts[i] = distinct;
    }
}

template <typename V, typename I>
__global__ void laso_compact_kernel(int64_t vec_nnz, int64_t dim_minor, const int64_t *tmp_idx,
                                    const V *tmp_val, const int64_t *counts,
                                    const int64_t *offsets, I *idx_long, I *idx_short,
                                    V *vals) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = tid; i < dim_minor; i += nthreads) {
        const int64_t o = offsets[i];
        for (int64_t q = 0; q < counts[i]; ++q) {
            idx_long[o + q] = (I)tmp_idx[i * vec_nnz + q];
            idx_short[o + q] = (I)i;
            vals[o + q] = tmp_val[i * vec_nnz + q];
        }
    }
}

// Exclusive prefix sum of n int64 values with one CTA (n is a vector count here).
__global__ void exclusive_scan_1cta(const int64_t *in, int64_t *out, int64_t n, int64_t *total) {
    __shared__ int64_t carry;
    __shared__ int64_t warp_sums[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t base = 0; base < n; base += blockDim.x) {
        const int64_t i = base + threadIdx.x;
        int64_t v = i < n ? in[i] : 0;
        int64_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int64_t w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_sums[lane] = w;
        }
        __syncthreads();
        const int64_t before = (warp > 0 ? warp_sums[warp - 1] : 0) + carry;
        if (i < n) out[i] = before + x - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + x;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

// ------------------------------------------------------------------ beta scaling
// X = beta * X over a rows x cols strided matrix; beta == 0 writes exact zeros without
// reading X (util::safe_scal, RandBLAS/util.hh:55-62).
template <typename T>
__global__ void scale_kernel(int64_t rows, int64_t cols, int64_t rs, int64_t cs, T beta, T *X) {
    const int64_t n = rows * cols;
    const bool rows_fast = rs <= cs;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = rows_fast ? t % rows : t / cols;
        const int64_t b = rows_fast ? t / rows : t % cols;
        T &x = X[a * rs + b * cs];
        x = beta == (T)0 ? (T)0 : beta * x;
    }
}

}  // namespace

void launch_fill_dense(int dtype, const DenseGen &g, int64_t R0, int64_t C0, int64_t nr,
                       int64_t nc, int transpose_out, void *out, cudaStream_t s) {
    if (nr <= 0 || nc <= 0) return;
    const int64_t tiles = ((nr + kFillTR - 1) / kFillTR) * ((nc + kFillTC - 1) / kFillTC);
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)num_sms() * 8);
    const RoundKeys rk = round_keys(g.key);  // Philox's round keys in the parameters
    if (dtype == RBG_F32)
        fill_dense_kernel<float><<<grid, 256, 0, s>>>(g, rk, R0, C0, nr, nc, transpose_out,
                                                      (float *)out);
    else
        fill_dense_kernel<double><<<grid, 256, 0, s>>>(g, rk, R0, C0, nr, nc, transpose_out,
                                                       (double *)out);
    RBG_LAUNCHED();
}

void launch_fill_saso(int dtype, int itype, const DevState &seed, int64_t vec_nnz,
                      int64_t dim_major, int64_t dim_minor, void *idx_major, void *idx_minor,
                      void *vals, cudaStream_t s) {
    if (dim_minor <= 0 || vec_nnz <= 0) return;
    const int threads = 128;
    int grid = grid_stride_ctas(dim_minor, threads);
    if (dim_major < (int64_t)UINT32_MAX && vec_nnz <= kSasoFastMaxNnz) {
#define RBG_SASO_FAST(V, I)                                                                  \
    saso_fast_kernel<V, I><<<grid, 128, 0, s>>>(seed, round_keys(seed.key), (int)vec_nnz,   \
                                                (uint32_t)dim_major,                         \
                                                dim_minor, (I *)idx_major, (I *)idx_minor,   \
                                                (V *)vals)
        if (dtype == RBG_F32 && itype == RBG_I32) RBG_SASO_FAST(float, int32_t);
        else if (dtype == RBG_F32) RBG_SASO_FAST(float, int64_t);
        else if (itype == RBG_I32) RBG_SASO_FAST(double, int32_t);
        else RBG_SASO_FAST(double, int64_t);
#undef RBG_SASO_FAST
        RBG_LAUNCHED();
        return;
    }
    int64_t *scratch = nullptr;
    Scratch buf;
    if (vec_nnz > kSasoLocalCap) {
        // bound the concurrent threads so the per-thread maps stay under 256 MiB
        const int64_t per_thread = 2 * vec_nnz * (int64_t)sizeof(int64_t);
        const int64_t max_threads = std::max<int64_t>(threads, (256ll << 20) / per_thread);
        grid = (int)std::max<int64_t>(1, std::min<int64_t>(grid, max_threads / threads));
        buf.alloc((size_t)grid * threads * per_thread, s);
        scratch = buf.as<int64_t>();
    }
#define RBG_SASO(V, I)                                                                       \
    saso_kernel<V, I><<<grid, threads, 0, s>>>(seed, vec_nnz, dim_major, dim_minor,          \
                                               (I *)idx_major, (I *)idx_minor, (V *)vals,    \
                                               scratch)
    if (dtype == RBG_F32 && itype == RBG_I32) RBG_SASO(float, int32_t);
    else if (dtype == RBG_F32) RBG_SASO(float, int64_t);
    else if (itype == RBG_I32) RBG_SASO(double, int32_t);
    else RBG_SASO(double, int64_t);
#undef RBG_SASO
    RBG_LAUNCHED();
}

int64_t launch_fill_laso(int dtype, int itype, const DevState &seed, int64_t vec_nnz,
                         int64_t dim_major, int64_t dim_minor, void *idx_long, void *idx_short,
                         void *vals, cudaStream_t s) {
    if (dim_minor <= 0 || vec_nnz <= 0) return 0;
    const size_t esz = dtype == RBG_F32 ? 4 : 8;
    const int64_t full = safe_mul(vec_nnz, dim_minor);
    Scratch tmp_idx((size_t)full * 8, s), tmp_val((size_t)full * esz, s),
        tmp_cnt((size_t)full * 8, s), counts((size_t)dim_minor * 8, s),
        offsets((size_t)(dim_minor + 1) * 8, s);
    const int threads = 128;
    const int grid = grid_stride_ctas(dim_minor, threads);
    if (dtype == RBG_F32)
        laso_sample_kernel<float><<<grid, threads, 0, s>>>(seed, vec_nnz, dim_major, dim_minor,
                                                           tmp_idx.as<int64_t>(),
                                                           tmp_val.as<float>(),
                                                           counts.as<int64_t>(),
                                                           tmp_cnt.as<int64_t>());
    else
        laso_sample_kernel<double><<<grid, threads, 0, s>>>(seed, vec_nnz, dim_major,
                                                            dim_minor, tmp_idx.as<int64_t>(),
                                                            tmp_val.as<double>(),
                                                            counts.as<int64_t>(),
                                                            tmp_cnt.as<int64_t>());
    RBG_LAUNCHED();
    int64_t *total = offsets.as<int64_t>() + dim_minor;
    exclusive_scan_1cta<<<1, 1024, 0, s>>>(counts.as<int64_t>(), offsets.as<int64_t>(),
                                           dim_minor, total);
    RBG_LAUNCHED();
#define RBG_LASO(V, I)                                                                         \
    laso_compact_kernel<V, I><<<grid, threads, 0, s>>>(vec_nnz, dim_minor, tmp_idx.as<int64_t>(), \
                                                       tmp_val.as<V>(), counts.as<int64_t>(),   \
                                                       offsets.as<int64_t>(), (I *)idx_long,    \
                                                       (I *)idx_short, (V *)vals)
    if (dtype == RBG_F32 && itype == RBG_I32) RBG_LASO(float, int32_t);
    else if (dtype == RBG_F32) RBG_LASO(float, int64_t);
    else if (itype == RBG_I32) RBG_LASO(double, int32_t);
    else RBG_LASO(double, int64_t);
#undef RBG_LASO
    RBG_LAUNCHED();
    int64_t nnz = 0;
    RBG_CUDA(cudaMemcpyAsync(&nnz, total, sizeof nnz, cudaMemcpyDeviceToHost, s));
    RBG_CUDA(cudaStreamSynchronize(s));
    return nnz;
}

void launch_scale(int dtype, int64_t rows, int64_t cols, int64_t rs, int64_t cs, double beta,
                  void *X, cudaStream_t s) {
    if (rows <= 0 || cols <= 0 || beta == 1.0) return;
    const int grid = grid_stride_ctas(rows * cols, 256);
    if (dtype == RBG_F32)
        scale_kernel<float><<<grid, 256, 0, s>>>(rows, cols, rs, cs, (float)beta, (float *)X);
    else
        scale_kernel<double><<<grid, 256, 0, s>>>(rows, cols, rs, cs, beta, (double *)X);
    RBG_LAUNCHED();
}

}  // namespace rbg
