// FP32 <-> FP64 conversions and the finiteness test on the integer pipe.
//
// On GB300 the FP64 pipe is the scarce one (1.19 TFLOP/s against 72.6 FP32), and the
// conversion instructions between FP32 and FP64 issue to it.  The stage-3 epilogue of the
// mixed RK3 (u64 += (double)delta; uhi = (float)u64; non-finite check) issued three or four
// FP64-pipe instructions per value, which made stage 3 nearly twice as long as stages 1-2.
// These routines do the same conversions from the IEEE 754 binary32 / binary64 encodings
// with integer instructions, leaving the FP64 pipe one add per value:
//  * binary32 -> binary64 is exact: sign kept, exponent rebiased (127 -> 1023), mantissa
//    widened; subnormal inputs are normalised; infinities and NaNs keep their class.
//  * binary64 -> binary32 rounds to nearest, ties to even (the default rounding of the
//    conversion instruction), including the carry into the exponent, overflow to infinity
//    and subnormal results; NaNs stay NaN (quiet), infinities stay infinite.
// They are checked value by value against the hardware conversions.
#pragma once

#include <cstdint>

namespace dgx {

__device__ __forceinline__ double f32_to_f64_bits(float x) {
    const uint32_t b = __float_as_uint(x);
    const uint64_t s = (uint64_t)(b & 0x80000000u) << 32;
    const uint32_t e = (b >> 23) & 0xFFu;
    const uint32_t m = b & 0x7FFFFFu;
    uint64_t r;
    if (e == 0xFFu) {  // infinity or NaN (a NaN keeps a nonzero payload)
        r = s | (0x7FFull << 52) | ((uint64_t)m << 29);
    } else if (e != 0) {  // normal
        r = s | ((uint64_t)(e + (1023 - 127)) << 52) | ((uint64_t)m << 29);
    } else if (m == 0) {  // signed zero
        r = s;
    } else {  // subnormal: m * 2^-149 with the leading one at bit t
        const int t = 31 - __clz(m);
        const uint64_t frac = (uint64_t)(m & ((1u << t) - 1u));
        r = s | ((uint64_t)(t - 149 + 1023) << 52) | (frac << (52 - t));
    }
    return __longlong_as_double((long long)r);
}

__device__ __forceinline__ float f64_to_f32_bits(double x) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const uint32_t s = (uint32_t)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7FFu);
    const uint64_t m = b & 0xFFFFFFFFFFFFFull;
    if (e == 0x7FF) return __uint_as_float(s | 0x7F800000u | (m ? 0x400000u : 0u));
    const int fe = e - (1023 - 127);  // biased binary32 exponent
    if (fe >= 0xFF) return __uint_as_float(s | 0x7F800000u);
    if (fe > 0) {  // normal range: keep 23 mantissa bits, round the 29 dropped ones
        const uint32_t mant = (uint32_t)(m >> 29);
        const uint32_t rem = (uint32_t)(m & 0x1FFFFFFFu);
        uint32_t r = s | ((uint32_t)fe << 23) | mant;
        if (rem > 0x10000000u || (rem == 0x10000000u && (mant & 1u))) ++r;  // a carry may reach infinity
        return __uint_as_float(r);
    }
    // subnormal or zero result: value = M * 2^(e - 1075) with M the 53-bit significand;
    // binary32 subnormals count units of 2^-149, so q = M * 2^(e - 926), rounded
    if (e == 0) return __uint_as_float(s);  // binary64 subnormals are far below 2^-150
    const uint64_t M = m | (1ull << 52);
    const int shift = 926 - e;  // >= 30
    if (shift > 54) return __uint_as_float(s);  // below half the smallest subnormal
    const uint64_t q = M >> shift;
    const uint64_t rem = M & ((1ull << shift) - 1ull);
    const uint64_t half = 1ull << (shift - 1);
    uint32_t r = s | (uint32_t)q;
    if (rem > half || (rem == half && (q & 1ull))) ++r;  // may carry into the smallest normal
    return __uint_as_float(r);
}

__device__ __forceinline__ bool finite_bits(double x) {
    return (((uint64_t)__double_as_longlong(x) >> 52) & 0x7FFu) != 0x7FFu;
}

}  // namespace dgx
