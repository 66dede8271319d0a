// Project-written stand-in for Random123's compiler-feature header (test infrastructure).
// The RandBLAS headers include it only for the macros below.
#pragma once
#ifndef R123_CUDA_DEVICE
#define R123_CUDA_DEVICE
#endif
#ifndef R123_STATIC_INLINE
#define R123_STATIC_INLINE static inline
#endif
#ifndef R123_FORCE_INLINE
#define R123_FORCE_INLINE(decl) decl __attribute__((always_inline))
#endif
#ifndef R123_ASSERT
#include <cassert>
#define R123_ASSERT(x) assert(x)
#endif
