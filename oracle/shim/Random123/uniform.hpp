// Project-written integer -> float transforms (test infrastructure), following the
// documented Random123 definitions used by RandBLAS/random_gen.hh:112-137 and
// RandBLAS/util.hh:516-546:
//   u01<F>(x)    = x * 2^-W + 2^-(W+1)            in (0, 1)
//   uneg11<F>(x) = (signed)x * 2^-(W-1) + 2^-W    in (-1, 1)
// for a W-bit unsigned x.
#pragma once
#include <array>
#include <cstdint>
#include <limits>
#include <type_traits>

namespace r123 {

template <typename F, typename U>
inline F u01(U in) {
    using UU = typename std::make_unsigned<U>::type;
    const F scale = F(1) / (F(std::numeric_limits<UU>::max()) + F(1));
    return F(UU(in)) * scale + F(0.5) * scale;
}

template <typename F, typename U>
inline F uneg11(U in) {
    using SS = typename std::make_signed<U>::type;
    const F scale = F(1) / (F(std::numeric_limits<SS>::max()) + F(1));
    return F(SS(in)) * scale + F(0.5) * scale;
}

template <typename F, typename A>
inline std::array<F, A::static_size> uneg11all(const A &in) {
    std::array<F, A::static_size> out;
    for (std::size_t i = 0; i < A::static_size; ++i) out[i] = uneg11<F>(in[i]);
    return out;
}

template <typename F, typename A>
inline std::array<F, A::static_size> u01all(const A &in) {
    std::array<F, A::static_size> out;
    for (std::size_t i = 0; i < A::static_size; ++i) out[i] = u01<F>(in[i]);
    return out;
}

}  // namespace r123
