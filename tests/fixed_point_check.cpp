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
    std::printf("checked %lld cases, %lld mismatches\n", n, bad);
    return bad == 0 ? 0 : 1;
}
