// Checks the integer-only fixed-point read-out of fixed_point.h against
// IEEE-754 rounding done by the C library in FP64:
//   fixed_to_float(F) == (float)((double)F * 2^-32) for |F| < 2^53
// argv[1] = number of random fixed-point samples.  Exit status 0 when every
// case agrees.
#include "fixed_point.h"

#include <cfenv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

using namespace ocm;

int main(int argc, char** argv) {
    std::fesetround(FE_TONEAREST);
    const long long samples = argc > 1 ? std::atoll(argv[1]) : 1000000;
    long long bad = 0, n = 0;
    std::mt19937_64 g(12345);
    for (long long k = 0; k < samples; ++k, ++n) {
        const int sh = (int)(g() % 64);
        long long F = (long long)(g() >> sh);
        if (F >= (1ll << 53)) F >>= 11;
        if (g() & 1) F = -F;
        const float a = fixed_to_float(F);
        const float b = (float)((double)F * (1.0 / 4294967296.0));
        if (a != b && bad++ < 15) std::printf("fixed_to_float %lld: %.9g != %.9g\n", F, a, b);
    }
    // exact halfway cases of the FP32 rounding
    for (int msb = 24; msb < 53; ++msb)
        for (long long q = (1ll << 23); q < (1ll << 23) + 64; ++q) {
            const int s = msb - 23;
            const long long F = (q << s) | (1ll << (s - 1));
            for (long long v : {F, -F, F + 1, F - 1}) {
                const float a = fixed_to_float(v);
                const float b = (float)((double)v * (1.0 / 4294967296.0));
                if (a != b && bad++ < 20) std::printf("fixed_to_float %lld\n", v);
                ++n;
            }
        }
    // fixed_from_float against the C library's round-half-even of f * 2^32
    std::uniform_real_distribution<double> mag(-30.0, 30.5);
    for (long long k = 0; k < samples; ++k, ++n) {
        float f = (float)std::ldexp(1.0 + (double)(g() % (1ull << 23)) / 8388608.0, (int)std::floor(mag(g)));
        if (g() & 1) f = -f;
        if (!(std::fabs(f) < 2147483648.0f)) continue;
        const long long a = (long long)fixed_from_float(f);
        const long long b = std::llrint((double)f * 4294967296.0);
        if (a != b && bad++ < 40) std::printf("fixed_from_float %.9g: %lld != %lld\n", f, a, b);
    }
    // values whose low word is an exact tie, integers, tiny values, zeros
    for (float f : {0.0f, -0.0f, 1.0f, -1.0f, 0.5f, -0.5f, 1e-12f, -1e-12f, 2.3283064e-10f, -2.3283064e-10f,
                    3.4924597e-10f, -3.4924597e-10f, 1.0e9f, -1.0e9f, 2147483520.0f, -2147483648.0f}) {
        const long long a = (long long)fixed_from_float(f);
        const long long b = std::llrint((double)f * 4294967296.0);
        if (a != b && bad++ < 60) std::printf("fixed_from_float %.9g: %lld != %lld\n", f, a, b);
        ++n;
    }
    std::printf("checked %lld cases, %lld mismatches\n", n, bad);
    return bad == 0 ? 0 : 1;
}
