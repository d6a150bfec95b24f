/* fp_exact.h - float arithmetic with double-precision semantics, without FP64 instructions.
 *
 * The reference's SVGF multiplies a float by the double literal 0.0001 (applyFilterKernel,
 * lib/CUDA/shared_kernel_code/finalize_shared.h:382): the product is formed in double and rounded back to float.
 * GB300 executes FP64 on a narrow pipe, and inside the a-trous loop that product became the filter's busiest
 * pipe. mul_float_by_double() returns the same float, bit for bit, from exact integer arithmetic: the 24-bit
 * by 53-bit significand product (at most 77 bits, held in 128 bits) is rounded to nearest-even at 53 bits (the
 * double) and then at 24 bits or at the float denormal quantum (the float), exactly as the two conversions do.
 *
 * Host and device share the code; the host instantiation is checked against real double arithmetic over
 * millions of inputs by the CPU tests.
 */
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define LH2G_HD __host__ __device__ __forceinline__
#else
#define LH2G_HD static inline
#endif

namespace lh2g {

LH2G_HD int clz64_hd(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

LH2G_HD uint32_t float_bits_hd(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

LH2G_HD float bits_float_hd(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

/* v >> s rounded to nearest, ties to even, for 0 < s < 128 */
LH2G_HD unsigned __int128 shift_round_even(unsigned __int128 v, int s) {
    const unsigned __int128 q = v >> s;
    const unsigned __int128 rem = v - (q << s);
    const unsigned __int128 half = (unsigned __int128)1 << (s - 1);
    return (rem > half || (rem == half && (q & 1))) ? q + 1 : q;
}

/* (float)((double)w * C) for w >= 0 (including +0 and +inf) and a positive normal double C = mc * 2^ec with
 * mc in [2^52, 2^53). NaN and negative w are not expected by the caller and are passed through unchanged. */
LH2G_HD float mul_float_by_double(const float w, const uint64_t mc, const int ec) {
    const uint32_t b = float_bits_hd(w);
    if (b == 0u || b >= 0x7f800000u) return w;   /* +0, +inf, NaN, negative values */
    const uint32_t E = b >> 23;
    const uint64_t m = E ? (uint64_t)((b & 0x7fffffu) | 0x800000u) : (uint64_t)(b & 0x7fffffu);
    const int e = E ? (int)E - 150 : -149;
    /* exact product, below 2^77 */
    unsigned __int128 P = (unsigned __int128)m * mc;
    const uint64_t hi = (uint64_t)(P >> 64), lo = (uint64_t)P;
    const int L = hi ? 128 - clz64_hd(hi) : 64 - clz64_hd(lo);   /* bit length */
    /* round to the 53-bit double significand (no double denormals occur: |w C| > 2^-160) */
    int exp2 = e + ec;                    /* value = P * 2^exp2 */
    if (L > 53) {
        P = shift_round_even(P, L - 53);
        exp2 += L - 53;
        if ((uint64_t)(P >> 53)) P >>= 1, exp2 += 1;   /* rounding carried into a new bit (the low bit was 0) */
    } else {
        P <<= (53 - L);
        exp2 -= 53 - L;
    }
    const uint64_t q = (uint64_t)P;       /* in [2^52, 2^53) */
    const int msb = exp2 + 52;            /* exponent of the leading bit */
    if (msb > 127) return bits_float_hd(0x7f800000u);
    /* float: 24 significant bits, or the fixed 2^-149 quantum below 2^-126 */
    const int s = msb >= -126 ? 29 : 29 + (-126 - msb);
    if (s > 60) return 0.0f;              /* below half the smallest denormal */
    const uint64_t r = (uint64_t)shift_round_even((unsigned __int128)q, s);
    if (msb >= -126) return bits_float_hd(((uint32_t)(msb + 126) << 23) + (uint32_t)r);   /* r in [2^23, 2^24]: a carry bumps the exponent */
    return bits_float_hd((uint32_t)r);    /* denormal, or the smallest normal when rounding carried */
}

/* the double 0.0001 = 0x1.a36e2eb1c432dp-14 */
constexpr uint64_t DBL_1EM4_MANT = 0x1a36e2eb1c432dull;
constexpr int DBL_1EM4_EXP = -66;

}  // namespace lh2g
