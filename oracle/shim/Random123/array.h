// Project-written stand-in for Random123's counter/key array types (test infrastructure).
//
// RandBLAS (RandBLAS/base.hh:64-164) needs, of an array type A:
//   A::value_type, A::static_size, a public C array `v`, operator[], aggregate
//   brace-initialisation, and incr(uint64) / incr() that add to the array read as a
//   little-endian multi-word unsigned integer (asserted by the reference's
//   test/test_basic_rng/test_r123.cc:705-797).
#pragma once
#include <cstddef>
#include <cstdint>
#include "features/compilerfeatures.h"

namespace r123 {

template <typename W, std::size_t N>
struct wide_uint_array {
    using value_type = W;
    static constexpr std::size_t static_size = N;
    W v[N];

    W &operator[](std::size_t i) { return v[i]; }
    const W &operator[](std::size_t i) const { return v[i]; }
    W *begin() { return v; }
    W *end() { return v + N; }
    const W *begin() const { return v; }
    const W *end() const { return v + N; }
    constexpr std::size_t size() const { return N; }

    // Add n to the array read as a little-endian integer with N words of W bits.
    wide_uint_array &incr(unsigned long long n = 1) {
        constexpr unsigned bits = 8 * sizeof(W);
        unsigned long long carry = 0;
        for (std::size_t i = 0; i < N; ++i) {
            unsigned long long add_lo;
            if (bits >= 64) {
                add_lo = n;
                n = 0;
            } else {
                add_lo = n & ((1ull << bits) - 1);
                n >>= bits;
            }
            W before = v[i];
            W sum = (W)(before + (W)add_lo);
            W sum2 = (W)(sum + (W)carry);
            unsigned long long c1 = (sum < before) ? 1 : 0;
            unsigned long long c2 = (sum2 < sum) ? 1 : 0;
            v[i] = sum2;
            carry = c1 + c2;
            if (n == 0 && carry == 0) break;
        }
        return *this;
    }
};

template <typename W, std::size_t N>
inline bool operator==(const wide_uint_array<W, N> &a, const wide_uint_array<W, N> &b) {
    for (std::size_t i = 0; i < N; ++i)
        if (a.v[i] != b.v[i]) return false;
    return true;
}
template <typename W, std::size_t N>
inline bool operator!=(const wide_uint_array<W, N> &a, const wide_uint_array<W, N> &b) {
    return !(a == b);
}

using r123array4x32 = wide_uint_array<std::uint32_t, 4>;
using r123array2x32 = wide_uint_array<std::uint32_t, 2>;

}  // namespace r123
