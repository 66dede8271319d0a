// shared_math.cc -- TEST INFRASTRUCTURE ONLY.  The oracle's "shared math" mode: the float
// sine, cosine and logarithm of the Box-Muller transform taken from the project's own
// specification of them (randblas_gb300/csrc/rbg_ffmath.cuh: float-float evaluation, one
// final rounding), compiled here as host C++ without contraction, so that the oracle and the
// GPU evaluate Box-Muller with the same math functions and can be compared bit for bit.
// In its default mode the oracle uses the host libm (glibc's sincosf / logf), as the
// reference does (Random123's boxmuller, RandBLAS/random_gen.hh:60-109); the distance between
// the two modes is that libm's rounding error.
#include "rbg_ffmath.cuh"

extern "C" {
void orc_ffm_sincosf(float theta, float *s, float *c) { rbg::ff::sincosf_ff(theta, *s, *c); }
float orc_ffm_logf(float x) { return rbg::ff::logf_ff(x); }
}
