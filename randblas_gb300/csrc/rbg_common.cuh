// rbg_common.cuh -- device building blocks shared by every kernel of the library:
// Philox4x32-10, 128-bit counter arithmetic, the float transforms RandBLAS applies to
// Philox output, and the entry-generation rule of a dense sketching operator.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "randblas_gb300.h"
#include "rbg_ffmath.cuh"

namespace rbg {

// ------------------------------------------------------------------ Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As Easy as 1, 2, 3" (SC'11),
// section 4: Philox-4x32 with 10 rounds.  This is the generator behind RandBLAS's
// DefaultRNG (RandBLAS/base.hh:53).
constexpr uint32_t kMulA = 0xD2511F53u;
constexpr uint32_t kMulB = 0xCD9E8D57u;
constexpr uint32_t kWeylA = 0x9E3779B9u;
constexpr uint32_t kWeylB = 0xBB67AE85u;

__device__ __forceinline__ uint4 philox(uint4 c, uint2 k) {
#pragma unroll
    for (int round = 0; round < 10; ++round) {
        if (round > 0) {
            k.x += kWeylA;
            k.y += kWeylB;
        }
        const uint32_t hi_a = __umulhi(kMulA, c.x), lo_a = kMulA * c.x;
        const uint32_t hi_b = __umulhi(kMulB, c.z), lo_b = kMulB * c.z;
        c = make_uint4(hi_b ^ c.y ^ k.x, lo_b, hi_a ^ c.w ^ k.y, lo_a);
    }
    return c;
}

// The ten round keys of one key (key + r * Weyl, r = 0 .. 9), computed once on the host and
// passed in kernel parameters: the rounds then read them as constant operands instead of
// advancing the key in registers on every call.
struct RoundKeys {
    uint2 k[10];
};
__host__ __device__ inline RoundKeys round_keys(uint2 key) {
    RoundKeys rk;
    for (int r = 0; r < 10; ++r)
        rk.k[r] = make_uint2(key.x + (uint32_t)r * kWeylA, key.y + (uint32_t)r * kWeylB);
    return rk;
}
__device__ __forceinline__ uint4 philox(uint4 c, const RoundKeys &rk) {
#pragma unroll
    for (int round = 0; round < 10; ++round) {
        const uint32_t hi_a = __umulhi(kMulA, c.x), lo_a = kMulA * c.x;
        const uint32_t hi_b = __umulhi(kMulB, c.z), lo_b = kMulB * c.z;
        c = make_uint4(hi_b ^ c.y ^ rk.k[round].x, lo_b, hi_a ^ c.w ^ rk.k[round].y, lo_a);
    }
    return c;
}

// counter + n, the counter read as a little-endian 128-bit integer
// (Random123's r123array4x32::incr, asserted by test/test_basic_rng/test_r123.cc:705-797).
__host__ __device__ __forceinline__ uint4 ctr_add(uint4 c, uint64_t n) {
    const uint64_t lo = ((uint64_t)c.y << 32 | c.x);
    const uint64_t sum = lo + n;
    const uint64_t carry = sum < lo ? 1u : 0u;
    uint64_t hi = ((uint64_t)c.w << 32 | c.z) + carry;
    return make_uint4((uint32_t)sum, (uint32_t)(sum >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
}

struct DevState {
    uint4 ctr;
    uint2 key;
};

__host__ __device__ __forceinline__ DevState to_dev(const rbg_state &s) {
    return DevState{make_uint4(s.counter[0], s.counter[1], s.counter[2], s.counter[3]),
                    make_uint2(s.key[0], s.key[1])};
}

// ------------------------------------------------------------------ transforms
// Random123's documented transforms, as RandBLAS uses them (RandBLAS/random_gen.hh:60-137):
//   uneg11(x) = (int32)x * 2^-31 + 2^-32, u01(x) = x * 2^-32 + 2^-33 (float),
//   boxmuller(u0, u1) = (sin(pi*uneg11(u0)) * r, cos(pi*uneg11(u0)) * r),
//   r = sqrt(-2 log(u01(u1))).
// The products by powers of two are exact, so each transform rounds once, after the addition;
// one FMA computes exactly that (the same value as a multiply followed by a rounded add).
__device__ __forceinline__ float uneg11(uint32_t x) {
    return __fmaf_rn(__int2float_rn((int32_t)x), 0x1p-31f, 0x1p-32f);
}

__device__ __forceinline__ float u01(uint32_t x) {
    return __fmaf_rn(__uint2float_rn(x), 0x1p-32f, 0x1p-33f);
}

// Box-Muller for the plain paths and the explicit fills: sin, cos and log are evaluated in
// float-float arithmetic (rbg_ffmath.cuh: FP32 instructions only) and rounded once to float,
// which gives the correctly rounded float except in vanishingly rare cases; then
// r = sqrtf(-2 * log) and the two products are rounded in float exactly as the reference's
// host code does.  Against glibc's float sincosf / logf (which are not correctly rounded) the
// results agree bit for bit in about 98.5% of cases and otherwise by one or two ulp (three in
// about 7 of 10^6, when the sine and the logarithm both round the other way).
__device__ __forceinline__ void boxmuller(uint32_t u0, uint32_t u1, float &first,
                                          float &second) {
    const float theta = __fmul_rn(3.14159265358979323846f, uneg11(u0));
    float s, c;
    ff::sincosf_ff(theta, s, c);
    const float l = ff::logf_ff(u01(u1));
    const float r = __fsqrt_rn(__fmul_rn(-2.0f, l));
    first = __fmul_rn(s, r);
    second = __fmul_rn(c, r);
}

// Box-Muller for the reduced-precision tensor-core paths, whose entries are rounded to BF16 /
// FP8 afterwards: the hardware's approximate sine, cosine, base-2 logarithm and square root
// (one instruction each), with -2 ln(u) taken as log2(u) * (-2 ln 2).  The angle lies in
// (-pi, pi) and u01 in (0, 1], where their errors (about 1e-6 relative) are far below a BF16
// ulp (3.9e-3 relative), so at most a BF16 rounding of the entry changes.  The uniform inputs
// are the exact transforms (each an FMA whose product is exact: one rounding, as above).
// The logarithm and square root take their flush-to-zero forms: u01 lies in [2^-33, 1] and
// the square root's argument is 0 or at least 1e-7, so no subnormal ever reaches them, the
// results are those of the plain forms, and the subnormal handling those forms carry (about
// 6% of the Gaussian tensor-core producers' time) is gone.
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float lg2_approx(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ void boxmuller_fast(uint32_t u0, uint32_t u1, float &first,
                                               float &second) {
    float s, c;
    __sincosf(__fmul_rn(3.14159265358979323846f, uneg11(u0)), &s, &c);
    const float r = sqrt_approx(__fmul_rn(lg2_approx(u01(u1)), -1.3862943611198906f));
    first = __fmul_rn(s, r);
    second = __fmul_rn(c, r);
}

// Four operator entries from one Philox call: Gaussian pairs (lanes 0,1) and (2,3), or
// four uniforms on (-1, 1).  Uniform entries are NOT scaled here (see scale_uniform).
template <bool kFast = false, typename Key = uint2>
__device__ __forceinline__ void gen4(int family, uint4 ctr, const Key &key, float v[4]) {
    const uint4 r = philox(ctr, key);
    if (family == RBG_GAUSSIAN) {
        if (kFast) {
            boxmuller_fast(r.x, r.y, v[0], v[1]);
            boxmuller_fast(r.z, r.w, v[2], v[3]);
        } else {
            boxmuller(r.x, r.y, v[0], v[1]);
            boxmuller(r.z, r.w, v[2], v[3]);
        }
    } else {
        v[0] = uneg11(r.x);
        v[1] = uneg11(r.y);
        v[2] = uneg11(r.z);
        v[3] = uneg11(r.w);
    }
}

// RandBLAS scales uniform entries by (T)sqrt(3) in the operator's precision T after the
// float transform (RandBLAS/dense_skops.hh:589).
template <typename T>
__device__ __forceinline__ T scale_uniform(float v);
template <>
__device__ __forceinline__ float scale_uniform<float>(float v) {
    return __fmul_rn(v, 1.7320508075688772f);
}
template <>
__device__ __forceinline__ double scale_uniform<double>(float v) {
    return __dmul_rn((double)v, 1.7320508075688772);
}

template <typename T>
__device__ __forceinline__ T finish_entry(int family, float v) {
    return family == RBG_UNIFORM ? scale_uniform<T>(v) : (T)v;
}

// ------------------------------------------------------------------ SASO columns
constexpr int kSasoFastMaxNnz = 16;

// Minor index i of a SASO with vec_nnz <= kSasoFastMaxNnz: the partial Fisher-Yates shuffle
// of sparse_skops.hh:51-106 with 32-bit arithmetic (exact: dim_major < 2^32, x0 % span <
// span).  emit(j, major, negative) is called for j = 0 .. vec_nnz - 1 in order; counters run
// seed + i * vec_nnz + j.  Philox is keyed by `key`: s.key, or its round keys when the caller
// has them in its kernel parameters.
template <typename Key, typename F>
__device__ __forceinline__ void saso_column(const DevState &s, const Key &key, uint64_t i,
                                            int vec_nnz, uint32_t dim_major, F &&emit) {
    uint32_t mp[kSasoFastMaxNnz], mv[kSasoFastMaxNnz];
    int msize = 0;
    const uint64_t off = i * (uint64_t)vec_nnz;
    for (int j = 0; j < vec_nnz; ++j) {
        const uint4 r = philox(ctr_add(s.ctr, off + (uint64_t)j), key);
        const uint32_t ell = (uint32_t)j + r.x % (dim_major - (uint32_t)j);
        uint32_t vj = (uint32_t)j, vl = ell;
        int sj = -1, sl = -1;
        for (int q = 0; q < msize; ++q) {
            if (mp[q] == (uint32_t)j) { vj = mv[q]; sj = q; }
            if (mp[q] == ell) { vl = mv[q]; sl = q; }
        }
        if (ell != (uint32_t)j) {
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
        emit(j, vl, (r.y & 1u) != 0u);
    }
}
template <typename F>
__device__ __forceinline__ void saso_column(const DevState &s, uint64_t i, int vec_nnz,
                                            uint32_t dim_major, F &&emit) {
    saso_column(s, s.key, i, vec_nnz, dim_major, emit);
}

// ------------------------------------------------------------------ dense operators
// A dense operator entry S(x, y) (0 <= x < n_rows, 0 <= y < n_cols) lives at "natural"
// coordinates (R, C): R = x, C = y when the natural layout is RowMajor, R = y, C = x when
// it is ColMajor.  Row R owns counters seed + [R*stride, (R+1)*stride) with
// stride = ceil(dim_major / 4); entry C is lane C % 4 of counter C / 4 of its row
// (RandBLAS/dense_skops.hh:96-170, 563-606).
struct DenseGen {
    uint4 ctr;        // seed counter
    uint2 key;        // seed key
    int64_t stride;   // counters per natural row
    int family;       // RBG_GAUSSIAN / RBG_UNIFORM
    int natural_col;  // 1 when the natural layout is ColMajor

    __device__ __forceinline__ uint4 counter_of(int64_t R, int64_t block) const {
        return ctr_add(ctr, (uint64_t)(R * stride + block));
    }
};

// Per-launch error word (device-side bounds checks and bounded waits report here).
struct DevError {
    int *flag;  // nullable
    __device__ __forceinline__ void raise(int code) const {
        if (flag) atomicCAS(flag, 0, code);
    }
};

}  // namespace rbg
