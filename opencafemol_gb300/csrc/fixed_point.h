// fixed_point.h - conversions between FP32 forces and the 64-bit fixed-point
// force accumulator (2^32 units per kJ/mol/nm), written with 32-bit
// operations only.
//
// On GB300 FP64 arithmetic runs on a narrow pipe; the integrators read every
// bead's force once per step, and going through a double there
// ((float)((double)F * 2^-32): an int64->f64 conversion, a multiply and an
// f64->f32 conversion) costs more than the integer version below, which
// measured ~2% faster on the batched kernel.  The other direction,
// fixed_from_float, splits the value at the binary point into two 32-bit
// conversions.
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

// f * 2^32 rounded to the nearest int64 (ties to even), for |f| < 2^31,
// with 32-bit operations only.  With a = |f|, a = fl + r where fl =
// floor(a) and r = a - fl are exact (Sterbenz), so round(a * 2^32) =
// fl * 2^32 + round(r * 2^32), where r * 2^32 < 2^32 - 128 cannot round up
// to 2^32 and the tie parity is the low word's; rounding half to even is
// symmetric, so the sign is applied to the integer.  On GB300 a float ->
// int64 conversion runs on the narrow FP64 pipe; the two float -> uint32
// conversions here do not.  Out of range (|f| >= 2^31) or NaN give an
// unspecified value: the engines flag such forces before they matter.
OCM_HD unsigned long long fixed_from_float(float f) {
#if defined(__CUDA_ARCH__)
    const float a = fabsf(f);
    const float fl = floorf(a);
    const unsigned int hi = __float2uint_rz(fl);
    const unsigned int lo = __float2uint_rn((a - fl) * 4294967296.0f);
#else
    const float a = __builtin_fabsf(f);
    const float fl = __builtin_floorf(a);
    const unsigned int hi = (unsigned int)fl;
    const unsigned int lo = (unsigned int)__builtin_llrintf((a - fl) * 4294967296.0f);
#endif
    const unsigned long long v = ((unsigned long long)hi << 32) + (unsigned long long)lo;
    return f < 0.f ? (unsigned long long)0 - v : v;
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
