// Project-written Philox4x32-R (test infrastructure), restated from the published
// description: Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As Easy as 1, 2, 3",
// SC'11, section 4.  Checked against the known-answer vectors the reference ships
// (test/test_basic_rng/r123_kat_vectors.txt:19-21).
#pragma once
#include <cstdint>
#include "array.h"

namespace r123 {

template <unsigned R>
struct Philox4x32_R {
    using ctr_type = r123array4x32;
    using key_type = r123array2x32;
    using ukey_type = r123array2x32;
    static constexpr unsigned rounds = R;

    ctr_type operator()(ctr_type in, key_type k) const {
        constexpr std::uint32_t mul_a = 0xD2511F53u, mul_b = 0xCD9E8D57u;
        constexpr std::uint32_t weyl_a = 0x9E3779B9u, weyl_b = 0xBB67AE85u;
        std::uint32_t x0 = in.v[0], x1 = in.v[1], x2 = in.v[2], x3 = in.v[3];
        std::uint32_t ka = k.v[0], kb = k.v[1];
        for (unsigned round = 0; round < R; ++round) {
            if (round > 0) { ka += weyl_a; kb += weyl_b; }
            std::uint64_t pa = (std::uint64_t)mul_a * x0;
            std::uint64_t pb = (std::uint64_t)mul_b * x2;
            std::uint32_t n0 = (std::uint32_t)(pb >> 32) ^ x1 ^ ka;
            std::uint32_t n1 = (std::uint32_t)pb;
            std::uint32_t n2 = (std::uint32_t)(pa >> 32) ^ x3 ^ kb;
            std::uint32_t n3 = (std::uint32_t)pa;
            x0 = n0; x1 = n1; x2 = n2; x3 = n3;
        }
        ctr_type out{};
        out.v[0] = x0; out.v[1] = x1; out.v[2] = x2; out.v[3] = x3;
        return out;
    }
};

using Philox4x32 = Philox4x32_R<10>;

}  // namespace r123
