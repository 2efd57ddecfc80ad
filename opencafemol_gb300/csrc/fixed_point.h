// fixed_point.h - read-out of the 64-bit fixed-point force accumulator
// (2^32 units per kJ/mol/nm) as FP32, written with integer operations only.
//
// On GB300 FP64 arithmetic runs on a narrow pipe; the integrators read every
// bead's force once per step, and going through a double there
// ((float)((double)F * 2^-32): an int64->f64 conversion, a multiply and an
// f64->f32 conversion) costs more than the integer version below, which
// measured ~2% faster on the batched kernel.  (The other direction,
// f * 2^32 -> int64, stays one FMUL plus one hardware conversion: an
// integer restatement of it measured slower.)
//
//   fixed_to_float(F) == F * 2^-32 correctly rounded to FP32
//                        (round-half-even), equal to
//                        (float)((double)F * 2^-32) whenever |F| < 2^53.
//
// The function compiles for host and device so the CPU tests can check it
// against the C library's rounding.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define OCM_HD __host__ __device__ __forceinline__
#else
#define OCM_HD inline
#endif

namespace ocm {

OCM_HD int clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

OCM_HD uint32_t f32_bits(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    __builtin_memcpy(&u, &f, 4);
    return u;
#endif
}

OCM_HD float f32_from_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    __builtin_memcpy(&f, &u, 4);
    return f;
#endif
}

// F * 2^-32 correctly rounded to FP32.
OCM_HD float fixed_to_float(long long F) {
    const bool neg = F < 0;
    uint64_t a = neg ? (uint64_t)0 - (uint64_t)F : (uint64_t)F;
    if (a == 0) return 0.f;
    int msb = 63 - clz64(a);                  // value = a * 2^-32 in [2^(msb-32), 2^(msb-31))
    uint32_t m;
    if (msb <= 23) {
        m = (uint32_t)(a << (23 - msb));      // exact
    } else {
        const int s = msb - 23;               // 1..40
        uint64_t q = a >> s;
        const uint64_t rem = a & ((1ull << s) - 1ull);
        const uint64_t half = 1ull << (s - 1);
        q += (rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull;
        if (q == (1ull << 24)) {              // rounded up to the next binade
            q >>= 1;
            ++msb;
        }
        m = (uint32_t)q;
    }
    const uint32_t be = (uint32_t)(msb + 95);  // biased exponent of 2^(msb - 32)
    return f32_from_bits((neg ? 0x80000000u : 0u) | (be << 23) | (m & 0x7FFFFFu));
}

}  // namespace ocm
