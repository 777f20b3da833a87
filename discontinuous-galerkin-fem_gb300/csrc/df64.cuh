// Double-float arithmetic ("df64") for the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with |lo| <= ulp(hi)/2,
// about 48 significant bits.  GB300 runs FP32 about 60x faster than FP64 (72.6 against
// 1.19 TFLOP/s measured), so an operation costing 6-11 FP32 instructions still beats
// the FP64 pipe.  The exponent range is FP32's.
//
// Building blocks are the error-free transformations of the literature:
//   TwoSum (Knuth, TAOCP vol. 2), FastTwoSum (Dekker 1971, requires |a| >= |b|), and the
//   product error a*b - fl(a*b) = fma(a, b, -fl(a*b)).
// Addition is the cheaper ("sloppy") double-word addition analysed by Joldes, Muller and
// Popescu (ACM TOMS 2017, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic"): its error is bounded relative to |a| + |b| rather than to
// |a + b|, the same form of bound as a chain of FP64 additions.  Multiplication uses one
// TwoProd and the two cross terms; division one refinement step of the quotient; square
// root one Newton step (Karp and Markstein 1997) from the FP32 square root.
#pragma once

#include <cmath>

namespace dgx {

struct f2 {
    float hi, lo;
    f2() = default;
    __host__ __device__ constexpr f2(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ explicit f2(double x) {
#ifdef __CUDA_ARCH__
        split(x);
#else
        hi = (float)x;
        lo = (float)(x - (double)hi);
#endif
    }
    __host__ __device__ explicit f2(int x) : f2((double)x) {}
    __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }

#ifdef __CUDA_ARCH__
    // double -> (hi, lo) with integer operations only (the FP64 pipe is the scarce one):
    // hi = the sign, exponent and top 23 mantissa bits; lo = the other 29 mantissa bits,
    // normalised by their leading one.  hi + lo equals x to about 2^-53 relative.  Values
    // outside FP32's normal range go through the hardware conversion with lo = 0.
    __device__ __forceinline__ void split(double x) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(x);
        const unsigned hw = (unsigned)(b >> 32);
        const int e = (int)((hw >> 20) & 0x7ffu);
        const int fe = e - 896;  // FP32 biased exponent of hi
        if (fe <= 0 || fe >= 255) {
            hi = __double2float_rn(x);
            lo = 0.f;
            return;
        }
        const unsigned sign = hw & 0x80000000u;
        const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
        hi = __uint_as_float(sign | ((unsigned)fe << 23) | (unsigned)(m >> 29));
        const unsigned low = (unsigned)(m & 0x1FFFFFFFull);  // value low * 2^(e - 1075)
        lo = 0.f;
        if (low) {
            const int lead = 31 - __clz(low);
            const int lexp = lead + e - 1075 + 127;
            if (lexp > 0) {
                const unsigned mant = lead >= 23 ? low >> (lead - 23) : low << (23 - lead);
                lo = __uint_as_float(sign | ((unsigned)lexp << 23) | (mant & 0x7FFFFFu));
            }
        }
    }
#endif
};

__device__ __forceinline__ f2 df_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return f2(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ f2 df_fast_two_sum(float a, float b) {  // |a| >= |b| (or a == 0)
    const float s = a + b;
    return f2(s, b - (s - a));
}

__device__ __forceinline__ f2 operator+(f2 a, f2 b) {
    const f2 s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ f2 operator-(f2 a) { return f2(-a.hi, -a.lo); }
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return a + (-b); }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return df_fast_two_sum(p, e);
}
__device__ __forceinline__ f2 operator/(f2 a, f2 b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const f2 r = a - b * f2(q1, 0.f);
    const float q2 = __fdiv_rn(r.hi, b.hi);
    return df_fast_two_sum(q1, q2);
}
__device__ __forceinline__ f2& operator+=(f2& a, f2 b) { return a = a + b; }
__device__ __forceinline__ f2& operator-=(f2& a, f2 b) { return a = a - b; }
__device__ __forceinline__ f2& operator*=(f2& a, f2 b) { return a = a * b; }

__device__ __forceinline__ bool operator<(f2 a, f2 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(f2 a, f2 b) { return b < a; }
__device__ __forceinline__ f2 fabs(f2 a) { return a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f) ? -a : a; }

// acc + a*b with the sum kept lazily normalised: hi + lo is the value, |lo| may grow to a
// few ulps of hi over a contraction; settle() restores the invariant before nonlinear use.
__device__ __forceinline__ f2 mac(f2 acc, f2 a, f2 b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    const f2 s = df_two_sum(acc.hi, p);
    return f2(s.hi, acc.lo + (s.lo + e));
}
__device__ __forceinline__ f2 settle(f2 x) { return df_two_sum(x.hi, x.lo); }

__device__ __forceinline__ f2 df_sqrt(f2 a) {
    if (!(a.hi > 0.f)) return f2(__fsqrt_rn(a.hi), 0.f);  // 0, negative or NaN: as FP32 does
    const float s = __fsqrt_rn(a.hi);
    // one Newton step on s: sqrt(a) ~ s + (a - s^2) / (2 s)
    const float p = s * s;
    const float pe = fmaf(s, s, -p);
    const float r = ((a.hi - p) - pe) + a.lo;
    return df_fast_two_sum(s, __fdiv_rn(r, 2.0f * s));
}

}  // namespace dgx
