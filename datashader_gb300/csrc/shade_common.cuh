// shade_common.cuh -- device helpers shared by the shading kernels
// (eq_hist.cu, shade.cu): an order-preserving key of a double, and
// numpy.interp restated (numpy/_core/src/multiarray/compiled_base.c: binary
// search, slope = (fp[j+1]-fp[j]) / (xp[j+1]-xp[j]), slope*(x-xp[j]) + fp[j],
// the NaN fallbacks), float64 throughout without contraction.
#pragma once

#include "dsgb_internal.cuh"

namespace dsgb {

__device__ __forceinline__ unsigned long long ord64(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double unord64(unsigned long long u) {
    unsigned long long b = (u >> 63) ? (u & 0x7fffffffffffffffull) : ~u;
    return __longlong_as_double((long long)b);
}
__device__ __forceinline__ double dnan() { return __longlong_as_double(0x7ff8000000000000ll); }

// np.interp(x, xp, fp) for sorted xp (left = fp[0], right = fp[-1]).
__device__ __forceinline__ double np_interp(double x, const double *xp, const double *fp, int len,
                                            double left, double right) {
    if (x != x) return x;
    if (x > xp[len - 1]) return right;
    if (x < xp[0]) return left;
    int lo = 0, hi = len - 1;          // invariant xp[lo] <= x, and x < xp[hi] or hi = len-1
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (xp[mid] <= x) lo = mid; else hi = mid;
    }
    int j = lo;
    if (x >= xp[len - 1]) j = len - 1;
    if (j == len - 1) return fp[j];
    if (xp[j] == x) return fp[j];
    double slope = __ddiv_rn(__dsub_rn(fp[j + 1], fp[j]), __dsub_rn(xp[j + 1], xp[j]));
    double r = __dadd_rn(__dmul_rn(slope, __dsub_rn(x, xp[j])), fp[j]);
    if (r != r) {
        r = __dadd_rn(__dmul_rn(slope, __dsub_rn(x, xp[j + 1])), fp[j + 1]);
        if (r != r && fp[j] == fp[j + 1]) r = fp[j];
    }
    return r;
}

}  // namespace dsgb
