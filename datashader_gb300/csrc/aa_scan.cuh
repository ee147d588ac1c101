// aa_scan.cuh -- the pixel span of one scanline of the antialiased line's
// rectangle (line.py:814-821 x_intercept, and the ceil / floor that follow it
// at line.py:921-926) without a float64 division in the common case, and
// the case of each scanned pixel decided in float32 where that is exact.
//
// The span ends are ceil(x) and floor(x) of the float64 intercept
//     x = cx0 + ((y - cy0) / (cy1 - cy0)) * (cx1 - cx0).
// Only the integers next to x matter.  The intercept is first computed in
// float32, with a bound B on its distance from the float64 value (first-
// order error analysis of each float32 rounding, each conversion of an input
// and the float64 result's own roundings, times a margin of 4); when the
// float32 value lies farther than B from every integer, the integer on
// either side of it is the float64 value's too.  Otherwise, or when an input
// is not finite, the float64 expression is evaluated as the reference does.
// The float32 work runs on the FMA pipe; the float64 division it replaces
// takes several passes through the float64 pipe, which bounds the kernels.
#pragma once

#include "f64cmp.cuh"

#include <cmath>

namespace dsgb {

// x_intercept in float64, the reference's operations in order (compiled
// without multiply-add contraction).
F64CMP_FN double aa_x_intercept(double y, double cx0, double cy0, double cx1, double cy1) {
    if (f64_eq(cy0, cy1)) return cx1;
    const double frac = (y - cy0) / (cy1 - cy0);
    return cx0 + frac * (cx1 - cx0);
}

// The float32 intercept xf for scanline y (an integer below 2^24, exact in
// float32) and whether it is provably on the same side of every integer as
// aa_x_intercept (cy0 != cy1 is the caller's case).
//
// Error terms (u = 2^-24, R = the exact real value of each quantity):
//   Nf = y - Y0f:        |Nf - N_R| <= u (|Y0| + |Nf|)
//   Df = Y1f - Y0f:      |Df - D_R| <= u (|Y0| + |Y1| + |Df|) <= |Df| / 8  (checked)
//   Xd = X1f - X0f:      |Xd - X_R| <= u (|X0| + |X1| + |Xd|)
//   Ff = Nf * (1 / Df):  |Ff - F_R| <= (|Nf - N_R| + |F_R| |Df - D_R|) / |Df| + 2 u |Ff|
//   Pf = Ff * Xd:        |Pf - P_R| <= |Ff - F_R| |Xd| + |F_R| |Xd - X_R| + u |Pf|
//   xf = X0f + Pf:       |xf - x_R| <= u |X0| + |Pf - P_R| + u |xf|
// with |F_R| <= |Ff| + 1 under the checked bound on Df.  The float64 value's
// own error is below 2^-50 of the same magnitudes, inside the margin.
F64CMP_FN bool aa_x_intercept_f32(unsigned y, double cx0, double cy0, double cx1, double cy1, float &xf) {
    const float u = 5.9604645e-08f;                       // 2^-24
    if (y >= (1u << 24)) return false;
    const float yf = (float)y;
    const float X0 = (float)cx0, X1 = (float)cx1, Y0 = (float)cy0, Y1 = (float)cy1;
    const float Nf = yf - Y0, Df = Y1 - Y0, Xd = X1 - X0;
    const float aX0 = fabsf(X0), aX1 = fabsf(X1), aY0 = fabsf(Y0), aY1 = fabsf(Y1);
    const float aDf = fabsf(Df), aXd = fabsf(Xd), aNf = fabsf(Nf);
    const float eD = u * (aY0 + aY1 + aDf);
    if (!(8.0f * eD <= aDf)) return false;                // also Df == 0, NaN, infinities
    const float If = 1.0f / Df;
    const float Ff = Nf * If;
    const float Pf = Ff * Xd;
    xf = X0 + Pf;
    const float aIf = fabsf(If), aFf = fabsf(Ff), Fr = aFf + 1.0f;
    const float eF = (u * (aY0 + aNf) + Fr * eD) * aIf + 2.0f * u * aFf;
    const float eP = eF * aXd + Fr * u * (aX0 + aX1 + aXd) + u * fabsf(Pf);
    const float e = u * aX0 + eP + u * fabsf(xf);
    const float bound = 4.0f * e + u;
    const float dist = fminf(xf - floorf(xf), ceilf(xf) - xf);
    return dist > bound;                                  // false for NaN
}

// The float64 fallback, out of line on the device (OUT_OF_LINE): it runs for
// about one scanline end in a hundred, and inlined twice into a scan loop it
// costs instruction-cache room; where the call's register saves cost more
// (the adjoint's dual-number loop spills around it), it stays inline.
#if defined(__CUDACC__)
#define AA_COLD_FN __host__ __device__ __noinline__
#else
#define AA_COLD_FN inline
#endif
template <bool CEIL>
AA_COLD_FN long long aa_scan_bound_f64(double yd, double cx0, double cy0, double cx1, double cy1, long long hi) {
    const double x = aa_x_intercept(yd, cx0, cy0, cx1, cy1);
    return CEIL ? f64_ceil_clamp(x, hi) : f64_floor_clamp(x, hi);
}

// max(0, min(ceil(x), hi)) (CEIL) or max(0, min(floor(x), hi)) of the
// intercept x, for hi < 2^31 and y < 2^31: integer operations for a
// horizontal edge, the float32 intercept when it is decisive, the float64
// expression otherwise.
template <bool CEIL, bool OUT_OF_LINE = false>
F64CMP_FN long long aa_scan_bound(unsigned y, double yd, double cx0, double cy0, double cx1, double cy1,
                                  long long hi) {
    if (f64_eq(cy0, cy1)) return CEIL ? f64_ceil_clamp(cx1, hi) : f64_floor_clamp(cx1, hi);
    float xf;
    if (aa_x_intercept_f32(y, cx0, cy0, cx1, cy1, xf)) {   // |xf| < 2^23 here
        long long c = (long long)(CEIL ? ceilf(xf) : floorf(xf));
        c = c < hi ? c : hi;
        return c > 0 ? c : 0;
    }
    if (OUT_OF_LINE) return aa_scan_bound_f64<CEIL>(yd, cx0, cy0, cx1, cy1, hi);
    const double x = aa_x_intercept(yd, cx0, cy0, cx1, cy1);
    return CEIL ? f64_ceil_clamp(x, hi) : f64_floor_clamp(x, hi);
}

// ---- the case of a scanned pixel, decided in float32 (the queued line
// kernel).  along = (x - x0) * ax + (y - y0) * ay against 0 and the length,
// and for a start cap the previous direction's dot (x - x0) * pax +
// (y - y0) * pay against 0 (line.py:930-950).  Each test is decided only
// when the float32 value is farther from its threshold than four times its
// first-order error bound: u = 2^-24 for each of the conversions of x0, y0,
// the direction and the length, the differences, the products and the sum
// (|x0| + 3 |dx|) |ax| + (|y0| + 3 |dy|) |ay| + |along|; the float64 value's
// own roundings are 2^-29 of that.  Otherwise the answer is AAC_EXACT and
// the float64 tests decide.
struct AAClassF {                          // float32 images of the segment's float64 values
    float x0, y0, ax, ay, len, pax, pay;
};

enum { AAC_NONE = 0, AAC_CAP_BEFORE = 1, AAC_CAP_AFTER = 2, AAC_SIDE = 3, AAC_EXACT = 4 };

// x, y below 2^24 (exact in float32).  cap_before: the start cap is drawn
// whatever the previous direction (overwrite or a segment start); cap_after:
// the end cap is drawn (overwrite or a segment end).
F64CMP_FN int aa_classify(unsigned x, unsigned y, const AAClassF &k, bool cap_before, bool cap_after) {
    const float u = 5.9604645e-08f;                       // 2^-24
    const float dx = (float)x - k.x0, dy = (float)y - k.y0;
    const float mx = fabsf(k.x0) + 3.0f * fabsf(dx), my = fabsf(k.y0) + 3.0f * fabsf(dy);
    const float along = dx * k.ax + dy * k.ay;
    const float ba = 4.0f * u * (mx * fabsf(k.ax) + my * fabsf(k.ay) + fabsf(along)) + 1e-30f;
    if (along < -ba) {
        if (cap_before) return AAC_CAP_BEFORE;
        const float pd = dx * k.pax + dy * k.pay;
        const float bp = 4.0f * u * (mx * fabsf(k.pax) + my * fabsf(k.pay) + fabsf(pd)) + 1e-30f;
        if (pd > bp) return AAC_CAP_BEFORE;
        if (pd < -bp) return AAC_NONE;
        return AAC_EXACT;
    }
    if (along > ba) {
        const float dl = along - k.len;
        const float bl = ba + 4.0f * u * (k.len + fabsf(dl));
        if (dl > bl) return cap_after ? AAC_CAP_AFTER : AAC_NONE;
        if (dl < -bl) return AAC_SIDE;
    }
    return AAC_EXACT;                                     // also NaN and infinite values
}

}  // namespace dsgb
