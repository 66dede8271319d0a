// Host-side accuracy check of randblas_gb300/csrc/rbg_ffmath.cuh: its float-float sin, cos and
// log against the correctly rounded values (double evaluation rounded to float) and against
// glibc's sincosf / logf, and the Box-Muller transform built on them against the oracle's
// (glibc-based) transform.  Built by tests/test_ffmath.py with -ffp-contract=off.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "rbg_ffmath.cuh"

extern "C" float orc_uneg11(uint32_t u);
extern "C" float orc_u01(uint32_t u);
extern "C" void orc_boxmuller(uint32_t u0, uint32_t u1, float *first, float *second);

static int64_t ulp(float a, float b) {
    int32_t ia, ib;
    std::memcpy(&ia, &a, 4);
    std::memcpy(&ib, &b, 4);
    int64_t x = ia < 0 ? -(int64_t)(ia & 0x7FFFFFFF) : ia;
    int64_t y = ib < 0 ? -(int64_t)(ib & 0x7FFFFFFF) : ib;
    return x > y ? x - y : y - x;
}

struct Tally {
    int64_t n = 0, exact = 0, one = 0, two = 0, more = 0, maxd = 0;
    void add(int64_t d) {
        ++n;
        if (d == 0) ++exact;
        else if (d == 1) ++one;
        else if (d == 2) ++two;
        else ++more;
        if (d > maxd) maxd = d;
    }
    void print(const char *name) const {
        std::printf("\"%s\": {\"n\": %lld, \"exact\": %lld, \"one\": %lld, \"two\": %lld, "
                    "\"more\": %lld, \"max\": %lld}",
                    name, (long long)n, (long long)exact, (long long)one, (long long)two,
                    (long long)more, (long long)maxd);
    }
};

static uint64_t state = 0x9E3779B97F4A7C15ull;
static uint32_t next32() {
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return (uint32_t)(state >> 16);
}

int main(int argc, char **argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 1 << 22;
    Tally sin_cr, cos_cr, log_cr, sin_g, cos_g, log_g, bm;
    static const uint32_t edges[] = {0u, 1u, 2u, 0x7FFFFFFFu, 0x80000000u, 0x80000001u,
                                     0xFFFFFFFFu, 0xFFFFFFFEu, 0x40000000u, 0xC0000000u,
                                     0x20000000u, 0xE0000000u, 0xB504F333u, 0x5A827999u,
                                     0x3FFFFFFFu, 0xBFFFFFFFu};
    const long ne = sizeof(edges) / sizeof(edges[0]);
    for (long i = 0; i < n + ne * ne; ++i) {
        uint32_t u0, u1;
        if (i < ne * ne) {
            u0 = edges[i / ne];
            u1 = edges[i % ne];
        } else {
            u0 = next32();
            u1 = next32();
        }
        const float theta = 3.14159265358979323846f * orc_uneg11(u0);
        const float x = orc_u01(u1);
        float s, c;
        rbg::ff::sincosf_ff(theta, s, c);
        const float l = rbg::ff::logf_ff(x);
        sin_cr.add(ulp(s, (float)std::sin((double)theta)));
        cos_cr.add(ulp(c, (float)std::cos((double)theta)));
        log_cr.add(ulp(l, (float)std::log((double)x)));
        float gs, gc;
        sincosf(theta, &gs, &gc);
        sin_g.add(ulp(s, gs));
        cos_g.add(ulp(c, gc));
        log_g.add(ulp(l, logf(x)));
        const float r = std::sqrt(-2.0f * l);
        float f0, f1;
        orc_boxmuller(u0, u1, &f0, &f1);
        bm.add(ulp(s * r, f0));
        bm.add(ulp(c * r, f1));
    }
    std::printf("{");
    sin_cr.print("sin_vs_correctly_rounded"); std::printf(", ");
    cos_cr.print("cos_vs_correctly_rounded"); std::printf(", ");
    log_cr.print("log_vs_correctly_rounded"); std::printf(", ");
    sin_g.print("sin_vs_glibc"); std::printf(", ");
    cos_g.print("cos_vs_glibc"); std::printf(", ");
    log_g.print("log_vs_glibc"); std::printf(", ");
    bm.print("boxmuller_vs_oracle");
    std::printf("}\n");
    return 0;
}
