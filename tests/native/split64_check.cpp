// Host check of shamrock_gb300/csrc/split64.cuh: the integer hi/lo split must equal the
// FP64 conversions (hi = fl32(v), lo = fl32(v - hi)) bit for bit, including ties to even,
// the all-ones mantissa rounding into the next binade, and the FP64 fallback range.
#include "../../shamrock_gb300/csrc/split64.cuh"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

static long bad = 0, n = 0;

static void chk(double v) {
    float hi, lo;
    gbsph::split64(v, hi, lo);
    const float h2 = (float) v;
    const float l2 = (float) (v - (double) h2);
    uint32_t a, b, c, d;
    std::memcpy(&a, &hi, 4);
    std::memcpy(&b, &h2, 4);
    std::memcpy(&c, &lo, 4);
    std::memcpy(&d, &l2, 4);
    n++;
    if (a != b || c != d) {
        if (bad < 5) std::printf("mismatch v=%.17g\n", v);
        bad++;
    }
}

int main(int argc, char **argv) {
    const long count = argc > 1 ? std::atol(argv[1]) : 2000000;
    std::mt19937_64 g(1);
    std::uniform_real_distribution<double> u(-1, 1);
    std::uniform_int_distribution<int> ex(-80, 130);
    for (long i = 0; i < count; i++) {
        const double v = std::ldexp(u(g), ex(g));
        chk(v);
        if (i % 4 == 0) { // values a fraction of an ulp around a float, incl. the halfway points
            const float f    = (float) v;
            const double ulp = std::ldexp(1.0, std::ilogb(f) - 23);
            for (int k = -4; k <= 4; k++) chk((double) f + k * ulp / 8);
        }
    }
    const double specials[] = {0.0, -0.0, 1.0, -1.0, 1e-30, 1e30, 3e38, 1e-40, 5e-324,
                               INFINITY, -INFINITY, 16777216.0, 16777217.0, 0.1};
    for (double v : specials) chk(v);
    for (int e = -74; e <= 126; e++) {
        const double v = std::ldexp(2.0 - std::ldexp(1.0, -52), e);
        chk(v);
        chk(-v);
    }
    std::printf("checked %ld, mismatches %ld\n", n, bad);
    return bad != 0;
}
