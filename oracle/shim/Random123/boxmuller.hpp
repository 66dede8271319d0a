// Project-written Box-Muller transform (test infrastructure), following the documented
// Random123 definition used by RandBLAS/random_gen.hh:60-74: for 32-bit inputs (u0, u1),
//   theta = pi * uneg11<float>(u0), r = sqrt(-2 log(u01<float>(u1))),
//   result = (sin(theta) * r, cos(theta) * r), all in float.
//
// The sine, cosine and logarithm come from the host libm (glibc's sincosf / logf, what the
// reference gets on Linux) unless boxmuller_math_mode() is set to 1: then from the project's
// float-float specification (rbg_ffmath.cuh), the functions the GPU evaluates, so that the
// reference's own code and the GPU can be compared bit for bit ("shared math" mode).
#pragma once
#include <cmath>
#include <cstdint>
#include "rbg_ffmath.cuh"
#include "uniform.hpp"

namespace r123 {

struct float2 { float x, y; };
struct double2 { double x, y; };

inline int &boxmuller_math_mode() {
    static int mode = 0;
    return mode;
}

inline float2 boxmuller(std::uint32_t u0, std::uint32_t u1) {
    float s, c, l;
    const float theta = 3.14159265358979323846f * uneg11<float>(u0);
    if (boxmuller_math_mode() == 1) {
        rbg::ff::sincosf_ff(theta, s, c);
        l = rbg::ff::logf_ff(u01<float>(u1));
    } else {
        ::sincosf(theta, &s, &c);
        l = std::log(u01<float>(u1));
    }
    float r = std::sqrt(-2.0f * l);
    return float2{s * r, c * r};
}

inline double2 boxmuller(std::uint64_t u0, std::uint64_t u1) {
    double s, c;
    ::sincos(3.14159265358979323846 * uneg11<double>(u0), &s, &c);
    double r = std::sqrt(-2.0 * std::log(u01<double>(u1)));
    return double2{s * r, c * r};
}

}  // namespace r123
