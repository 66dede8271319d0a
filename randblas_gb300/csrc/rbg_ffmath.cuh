// rbg_ffmath.cuh -- sin, cos and log of float arguments evaluated in float-float arithmetic
// (a value carried as an unevaluated sum hi + lo of two floats, about 44 significant bits)
// and rounded once to float.  Used by the plain paths' Box-Muller transform, whose entries
// must agree with the reference's float sincosf / logf (RandBLAS/random_gen.hh:60-109) to
// within 2 ulp: evaluating these three functions this way gives the correctly rounded float
// except when the exact value lies within ~2^-40 relative of a rounding boundary, using only
// FP32 instructions (GB300's FP64 rate is 1/64 of its FP32 rate).
//
// Methods (all published; constants derived for this file from the mathematics, not copied):
// * error-free transformations: two-sum (Knuth, TAOCP vol. 2, 4.2.2), fast two-sum and
//   FMA-based two-product (Dekker, "A floating-point technique for extending the available
//   precision", Numer. Math. 18, 1971);
// * sin / cos: Cody-Waite reduction by pi/2 split into three pieces (Cody & Waite, Software
//   Manual for the Elementary Functions, 1980), then the Taylor series of sin and cos on
//   |r| <= pi/4, the leading terms in float-float and the tail in float;
// * log: x = 2^e m with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s), s = (m - 1) / (m + 1),
//   by its Taylor series, plus e log 2 with log 2 split so that e * hi is exact.
// The coefficients are 1/n! and 2/k rounded to float-float pairs, pi/2 split into 20-bit
// pieces (k * piece is exact for |k| <= 2), log 2 split at 18 bits.
//
// Compiles as CUDA device code (arithmetic through the _rn intrinsics, so no contraction) and
// as host C++ (built with -ffp-contract=off for the host-side accuracy test).
#pragma once

#include <cstdint>
#include <cstring>
#if !defined(__CUDACC__)
#include <cmath>
#endif

#if defined(__CUDACC__)
#define RBG_FF_FN __host__ __device__ __forceinline__
#else
#define RBG_FF_FN inline
#endif

namespace rbg {
namespace ff {

RBG_FF_FN float add(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
RBG_FF_FN float sub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
RBG_FF_FN float mul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
RBG_FF_FN float fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}
RBG_FF_FN float div(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
RBG_FF_FN uint32_t bits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return u;
#endif
}
RBG_FF_FN float from_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    std::memcpy(&x, &u, 4);
    return x;
#endif
}

struct F2 {
    float hi, lo;
};

// s + e = a + b exactly (any magnitudes)
RBG_FF_FN F2 two_sum(float a, float b) {
    const float s = add(a, b);
    const float bb = sub(s, a);
    const float e = add(sub(a, sub(s, bb)), sub(b, bb));
    return {s, e};
}
// s + e = a + b exactly when |a| >= |b| (or a == 0)
RBG_FF_FN F2 fast_two_sum(float a, float b) {
    const float s = add(a, b);
    return {s, sub(b, sub(s, a))};
}
RBG_FF_FN F2 ff_add(F2 a, F2 b) {
    F2 s = two_sum(a.hi, b.hi);
    s.lo = add(s.lo, add(a.lo, b.lo));
    return fast_two_sum(s.hi, s.lo);
}
RBG_FF_FN F2 ff_add(F2 a, float b) {
    F2 s = two_sum(a.hi, b);
    s.lo = add(s.lo, a.lo);
    return fast_two_sum(s.hi, s.lo);
}
RBG_FF_FN F2 ff_mul(F2 a, F2 b) {
    const float p = mul(a.hi, b.hi);
    float e = fma(a.hi, b.hi, -p);
    e = fma(a.hi, b.lo, fma(a.lo, b.hi, e));
    return fast_two_sum(p, e);
}
RBG_FF_FN F2 ff_sqr(F2 a) {
    const float p = mul(a.hi, a.hi);
    float e = fma(a.hi, a.hi, -p);
    e = fma(add(a.hi, a.hi), a.lo, e);
    return fast_two_sum(p, e);
}

// pi/2 = C1 + C2 + C3 (C1, C2: 20 significant bits)
constexpr float kC1 = 0x1.921fcp+0f;
constexpr float kC2 = -0x1.5777ap-21f;
constexpr float kC3 = -0x1.73dcb4p-43f;
constexpr float kTwoOverPi = 0x1.45f306p-1f;
constexpr float kRoundMagic = 12582912.0f;  // 1.5 * 2^23: adding it rounds to an integer

// sin r, cos r for |r| <= pi/4 (plus rounding), r = r.hi + r.lo
RBG_FF_FN void sincos_reduced(F2 r, F2 &s, F2 &c) {
    const F2 r2 = ff_sqr(r);
    const float x = r2.hi;
    // sin r = r + r * r2 * (-1/3! + r2 (1/5! + r2 (-1/7! + r2 (1/9! - r2/11! + r2^2/13!))))
    const float ts = mul(x, fma(x, fma(x, 0x1.612462p-33f, -0x1.ae6456p-26f), 0x1.71de3ap-19f));
    F2 p = ff_add(F2{-0x1.a01a02p-13f, 0x1.7f97fap-39f}, ts);
    p = ff_add(F2{0x1.111112p-7f, -0x1.dddddep-32f}, ff_mul(r2, p));
    p = ff_add(F2{-0x1.555556p-3f, 0x1.555556p-28f}, ff_mul(r2, p));
    s = ff_add(r, ff_mul(r, ff_mul(r2, p)));
    // cos r = 1 + r2 (-1/2 + r2 (1/4! + r2 (-1/6! + r2 (1/8! - r2/10! + ... + r2^4/16!))))
    const float tc = mul(
        x, fma(x, fma(x, fma(x, fma(x, 0x1.ae7f3ep-45f, -0x1.93974ap-37f), 0x1.1eed8ep-29f),
                      -0x1.27e4fcp-22f),
               0x1.a01a02p-16f));
    F2 q = ff_add(F2{-0x1.6c16c2p-10f, 0x1.27d27ep-35f}, tc);
    q = ff_add(F2{0x1.555556p-5f, -0x1.555556p-30f}, ff_mul(r2, q));
    q = ff_add(F2{-0.5f, 0.0f}, ff_mul(r2, q));
    c = ff_add(F2{1.0f, 0.0f}, ff_mul(r2, q));
}

// sin(theta), cos(theta) for a float |theta| <= 4, each rounded to float.
RBG_FF_FN void sincosf_ff(float theta, float &sin_out, float &cos_out) {
    const float y = fma(theta, kTwoOverPi, kRoundMagic);
    const float k = sub(y, kRoundMagic);       // nearest integer to theta * 2/pi, |k| <= 3
    const uint32_t quadrant = bits(y) & 3u;   // k mod 4 (the magic's low bits are zero)
    const float t = fma(-k, kC1, theta);      // exact: k * C1 has <= 22 bits, t is small
    F2 r = two_sum(t, mul(-k, kC2));          // k * C2 exact
    r.lo = fma(-k, kC3, r.lo);
    r = fast_two_sum(r.hi, r.lo);
    F2 s, c;
    sincos_reduced(r, s, c);
    const float sv = s.hi, cv = c.hi;
    switch (quadrant) {
        case 0: sin_out = sv; cos_out = cv; break;
        case 1: sin_out = cv; cos_out = -sv; break;
        case 2: sin_out = -sv; cos_out = -cv; break;
        default: sin_out = -cv; cos_out = sv; break;
    }
}

// log(x) for a positive normal float x, rounded to float.
RBG_FF_FN float logf_ff(float x) {
    const uint32_t b = bits(x);
    int e = (int)((b >> 23) & 0xFFu) - 127;
    float m = from_bits((b & 0x7FFFFFu) | 0x3F800000u);  // [1, 2)
    if (m > 0x1.6a09e6p+0f) {                            // sqrt(2)
        m = mul(m, 0.5f);
        e += 1;
    }
    const float f = sub(m, 1.0f);  // exact
    // s = f / (2 + f) in float-float
    const F2 den = fast_two_sum(2.0f, f);
    const float sh = div(f, den.hi);
    float res = fma(-sh, den.hi, f);  // exact remainder of the rounded division
    res = fma(-sh, den.lo, res);
    const F2 s = fast_two_sum(sh, div(res, den.hi));
    const F2 s2 = ff_sqr(s);
    const float z = s2.hi;
    // log m = 2 s + s^3 (2/3 + s2 (2/5 + s2 (2/7 + ... + s2^4 2/15)))
    const float tl = mul(
        z, fma(z, fma(z, fma(z, fma(z, 0x1.111112p-3f, 0x1.3b13b2p-3f), 0x1.745d18p-3f),
                      0x1.c71c72p-3f),
               0x1.24924ap-2f));
    F2 q = ff_add(F2{0x1.99999ap-2f, -0x1.99999ap-28f}, tl);
    q = ff_add(F2{0x1.555556p-1f, -0x1.555556p-26f}, ff_mul(s2, q));
    const F2 lm = ff_add(F2{add(s.hi, s.hi), add(s.lo, s.lo)}, ff_mul(ff_mul(s, s2), q));
    // + e log 2, log 2 = LN2_HI + LN2_LO with e * LN2_HI exact
    const float ef = (float)e;
    const F2 el = fast_two_sum(mul(ef, 0x1.62e4p-1f), mul(ef, 0x1.7f7d1cp-20f));
    return ff_add(el, lm).hi;
}

}  // namespace ff
}  // namespace rbg
