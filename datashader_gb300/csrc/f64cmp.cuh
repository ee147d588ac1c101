// f64cmp.cuh -- float64 comparisons and small conversions by integer
// operations on the bit patterns.
//
// The antialiased line kernels are bound by the float64 pipe, which on this
// part issues one warp instruction per 16 SM cycles; a float64 compare or
// min / max there costs as much as an add.  The integer pipes are nearly
// idle, so the comparisons of the per-pixel loop are done on the IEEE bit
// patterns instead.  Each helper states the inputs for which it returns the
// IEEE result; the ones marked "every input" include NaNs, infinities and
// both zeros.
#pragma once

#include <cstdint>
#include <cstring>

// Host and device: the host copy lets a CPU test compare each helper with
// the IEEE operation over special and random values.
#define F64CMP_FN __host__ __device__ __forceinline__

namespace dsgb {

constexpr unsigned long long F64_SIGN = 0x8000000000000000ull;
constexpr unsigned long long F64_INF = 0x7FF0000000000000ull;
constexpr unsigned long long F64_ONE = 0x3FF0000000000000ull;
constexpr unsigned long long F64_MAG = 0x7FFFFFFFFFFFFFFFull;

F64CMP_FN unsigned long long f64_bits(double v) {
#ifdef __CUDA_ARCH__
    return (unsigned long long)__double_as_longlong(v);
#else
    unsigned long long b;
    std::memcpy(&b, &v, 8);
    return b;
#endif
}

// v < 0.0, every input: the negative non-zero non-NaN patterns are
// [SIGN + 1, SIGN | INF].
F64CMP_FN bool f64_lt0(double v) {
    return f64_bits(v) - (F64_SIGN + 1) <= F64_INF - 1;
}

// v > 0.0, every input: [1, INF].
F64CMP_FN bool f64_gt0(double v) {
    return f64_bits(v) - 1 < F64_INF;
}

// a > b for b >= +0.0 or NaN (sign bit clear unless NaN), every a.  Non-NaN
// patterns with the sign bit clear order as their values; a negative a or
// -0.0 (pattern above INF) is never greater, nor is anything against NaN.
F64CMP_FN bool f64_gt_nonneg(double a, double b) {
    const unsigned long long A = f64_bits(a), B = f64_bits(b);
    return A > B && A <= F64_INF && B <= F64_INF;
}

// a <= b for a, b in [+0.0, +inf] (sign bit clear, no NaN).
F64CMP_FN bool f64_le_nonneg(double a, double b) {
    return f64_bits(a) <= f64_bits(b);
}

// |v| <= m for m in [+0.0, +inf], every v (a NaN's magnitude is above INF).
F64CMP_FN bool f64_abs_le(double v, double m) {
    return (f64_bits(v) & F64_MAG) <= f64_bits(m);
}

// -m <= v && v <= 0.0 for m in [+0.0, +inf], every v: v is +0.0 or has the
// sign bit set, and its magnitude is at most m (which excludes NaN).
F64CMP_FN bool f64_in_neg_range(double v, double m) {
    const unsigned long long V = f64_bits(v);
    return (V == 0 || (long long)V < 0) && (V & F64_MAG) <= f64_bits(m);
}

// v is a NaN, every input.
F64CMP_FN bool f64_isnan(double v) {
    return (f64_bits(v) & F64_MAG) > F64_INF;
}

// Order-preserving int64 image of a non-NaN float64, both zeros at 0:
// f64_okey(a) < f64_okey(b) <=> a < b, and == <=> a == b.
F64CMP_FN long long f64_okey(double v) {
    const unsigned long long V = f64_bits(v);
    return (long long)V < 0 ? -(long long)(V & F64_MAG) : (long long)V;
}

// a < b, every input.
F64CMP_FN bool f64_lt(double a, double b) {
    return !f64_isnan(a) && !f64_isnan(b) && f64_okey(a) < f64_okey(b);
}

// a == b, every input: the same non-NaN pattern, or both zeros.
F64CMP_FN bool f64_eq(double a, double b) {
    const unsigned long long A = f64_bits(a), B = f64_bits(b);
    return (A == B && (A & F64_MAG) <= F64_INF) || ((A | B) & F64_MAG) == 0;
}

// |a| < |b|, every input (a NaN's magnitude is above INF).
F64CMP_FN bool f64_abs_lt(double a, double b) {
    const unsigned long long MA = f64_bits(a) & F64_MAG, MB = f64_bits(b) & F64_MAG;
    return MA < MB && MB <= F64_INF;
}

// a > b for a in [+0.0, +inf], every b: against a b with the sign bit set,
// true unless b is a NaN or both are zeros.
F64CMP_FN bool f64_nonneg_gt(double a, double b) {
    const unsigned long long A = f64_bits(a), B = f64_bits(b);
    return (long long)B < 0 ? (B <= (F64_SIGN | F64_INF) && (A != 0 || B != F64_SIGN)) : A > B;
}

// max(0, min((long long)ceil(v), hi)) and max(0, min((long long)floor(v), hi))
// for hi < 2^31, every v, with the float64 -> int64 conversion of the device
// (NaN -> 0, saturating): a NaN or v <= 0 (ceil) / v < 1 (floor) gives 0,
// v >= 2^31 gives max(0, hi), and between them the integer part is the
// mantissa shifted right by 52 - exponent, plus one for ceil when any
// fraction bit is set.
F64CMP_FN long long f64_ceil_clamp(double v, long long hi) {
    const unsigned long long V = f64_bits(v);
    if ((long long)V <= 0 || V > F64_INF) return 0;
    const int e = (int)(V >> 52) - 1023;
    long long c;
    if (e >= 31) c = 1ll << 31;
    else if (e < 0) c = 1;
    else {
        const unsigned long long m = (V & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
        const int sh = 52 - e;
        c = (long long)(m >> sh) + ((m & ((1ull << sh) - 1)) != 0);
    }
    c = c < hi ? c : hi;
    return c > 0 ? c : 0;
}
F64CMP_FN long long f64_floor_clamp(double v, long long hi) {
    const unsigned long long V = f64_bits(v);
    if ((long long)V <= 0 || V > F64_INF) return 0;
    const int e = (int)(V >> 52) - 1023;
    long long c;
    if (e >= 31) c = 1ll << 31;
    else if (e < 0) c = 0;
    else c = (long long)((((V & 0x000FFFFFFFFFFFFFull) | (1ull << 52))) >> (52 - e));
    c = c < hi ? c : hi;
    return c > 0 ? c : 0;
}

// 1.0 - max(0.0, min(t, 1.0)) with the comparisons of
//     m = t < 1.0 ? t : 1.0;  c = 0.0 > m ? 0.0 : m;  return 1.0 - c;
// for every t.  The clamp sends t in [+0, 1] to itself, t > 1 and NaN
// (either sign) to 1.0, negative t and -0.0 to zero (-0.0 for -0.0 itself,
// which 1.0 - c does not distinguish from +0.0).  One float64 subtraction.
F64CMP_FN double f64_one_minus_clamp01(double t) {
    const unsigned long long T = f64_bits(t);
    const bool negative_or_zero = T - F64_SIGN <= F64_INF;        // [-inf, -0.0]
    const double c = T <= F64_ONE ? t : (negative_or_zero ? 0.0 : 1.0);
    return 1.0 - c;
}

// (double)x for every uint32 x, without the float64 conversion: the
// leading one is shifted out and the 31 bits below it left-aligned
// (shifted in two steps, so no shift count reaches 32), exponent
// 1023 + 31 - clz(x); exact, as every uint32 fits the 52-bit mantissa.
F64CMP_FN double f64_from_u32(unsigned x) {
#ifdef __CUDA_ARCH__
    const int lz = __clz((int)x);
#else
    const int lz = x ? __builtin_clz(x) : 32;
#endif
    const unsigned m = (x << (lz & 31)) << 1;
    const unsigned hi = x ? ((1054u - (unsigned)lz) << 20) | (m >> 12) : 0u;
    const unsigned lo = m << 20;
#ifdef __CUDA_ARCH__
    return __hiloint2double((int)hi, (int)lo);
#else
    const unsigned long long b = ((unsigned long long)hi << 32) | lo;
    double d;
    std::memcpy(&d, &b, 8);
    return d;
#endif
}

}  // namespace dsgb
