// binning.cuh -- exact Point binning (datashader/glyphs/points.py:190-204).
//
// Reference semantics: a row is kept when xmin <= x <= xmax and
// ymin <= y <= ymax (float64 compares); xx = int(x*sx + tx) with the product
// and the sum each rounded in float64 (numba emits no FMA) and int()
// truncating toward zero; xx >= width maps to width-1; a negative index
// wraps like a numba array index.
//
// GB300 has little float64 throughput, so the common case runs in float32
// and is proven: E (binning_error_bound, host) bounds |float32 result -
// float64 result|.  When the float32 value v = fma(x, (float)s, (float)t)
// lies farther than E from every integer, truncating v gives the same bin as
// the float64 formula; otherwise the float64 formula runs (about one
// coordinate in 500 on a 1024-px axis).  Bit-identical to the reference.
#pragma once

#include <cmath>
#include <float.h>
#include <stdint.h>
#include <string.h>

namespace dsgb {

struct BinAxis {
    double s, t;          // scale / translate (core.py:62-81)
    float sf, tf;         // their float32 images
    float e;              // proven error bound of the float32 path (pixels)
    int n;                // number of bins
};

// Exact float64 binning of one mapped coordinate.
__device__ __forceinline__ int bin_exact64_st(double m, double s, double t, int n) {
    const double v = __dadd_rn(__dmul_rn(m, s), t);
    long long xx = __double2ll_rz(v);
    if (xx >= n) xx = n - 1;
    if (xx < 0) xx += n;              // numba indexes negative positions from the end
    if (xx < 0) xx = 0;               // unreachable after the bounds test; memory safety
    return (int)xx;
}
__device__ __forceinline__ int bin_exact64(double m, const BinAxis &a) { return bin_exact64_st(m, a.s, a.t, a.n); }

// float32 binning of a coordinate whose float64 value is `exact` (a float
// promoted exactly, or the original double).  `xf` is a float32 image of it
// within the error budget of E.
//
// The integer part comes from the 1.5 * 2^23 magic addition (FADD/IADD only,
// no float<->int conversion): for 0 <= v < 2^22, t = v + 1.5*2^23 is v
// rounded to the nearest integer k (ulp 1), k = bits(t) - bits(1.5*2^23),
// fr = v - k exactly, and floor(v) = k - (fr < 0).  |fr| is the distance to
// the nearest integer, so |fr| > E proves the float64 result has the same
// floor.  v < 0.5 (within half a pixel of the lower edge) takes the float64
// path, which keeps the negative-index rule of the reference in one place.
template <typename T>
__device__ __forceinline__ int bin_fast32(float xf, T exact, const BinAxis &a) {
    const float v = __fmaf_rn(xf, a.sf, a.tf);
    if (v >= 0.5f && v < 4194304.0f) {
        const float t = __fadd_rn(v, 12582912.0f);
        const float fr = __fsub_rn(v, __fsub_rn(t, 12582912.0f));
        if (fabsf(fr) > a.e) {
            int r = (__float_as_int(t) - 0x4B400000) - (fr < 0.0f ? 1 : 0);
            return r >= a.n ? a.n - 1 : r;
        }
    }
    return bin_exact64((double)exact, a);
}

// Float32 image of a double by mantissa truncation (integer ops only);
// false outside the normal float32 range.
__device__ __forceinline__ bool f64_to_f32_trunc(double x, float &out) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if ((b << 1) == 0) { out = 0.0f; return true; }
    const int e = (int)((b >> 52) & 0x7ff) - 1023 + 127;
    if (e <= 0 || e >= 255) return false;
    out = __uint_as_float(((unsigned)(b >> 63) << 31) | ((unsigned)e << 23) |
                          (unsigned)((b >> 29) & 0x7fffffu));
    return true;
}

// Order-preserving int64 key of a double with -0.0 folded onto +0.0; NaN
// keys fall outside every [key(lo), key(hi)] interval.
__host__ __device__ __forceinline__ long long bound_key(double v) {
#ifdef __CUDA_ARCH__
    long long b = __double_as_longlong(v);
#else
    long long b;
    memcpy(&b, &v, 8);
#endif
    if (b == (long long)0x8000000000000000ull) b = 0;
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}

struct BinBounds {
    float xminf, xmaxf, yminf, ymaxf;     // exact float images of the inclusive bounds
    long long kxmin, kxmax, kymin, kymax; // keys of the float64 bounds
};

// Hot-loop form: the float32 fast path only.  Returns 0 (outside the
// bounds), 1 (inside, xi/yi decided) or 2 (inside, one coordinate within E
// of a pixel edge: call bin_exact_f32).  Keeping the float64 code out of
// the unrolled loop keeps the loop small.
__device__ __forceinline__ int fast_coord(float v, const BinAxis &a, int &r) {
    if (!(v >= 0.5f && v < 4194304.0f)) return 0;
    const float t = __fadd_rn(v, 12582912.0f);
    const float fr = __fsub_rn(v, __fsub_rn(t, 12582912.0f));
    r = (__float_as_int(t) - 0x4B400000) - (fr < 0.0f ? 1 : 0);
    r = r >= a.n ? a.n - 1 : r;
    return fabsf(fr) > a.e ? 1 : 0;
}

__device__ __forceinline__ int bin_try_f32(float x, float y, const BinBounds &bb, const BinAxis &ax,
                                           const BinAxis &ay, int &xi, int &yi) {
    if (!(x >= bb.xminf && x <= bb.xmaxf && y >= bb.yminf && y <= bb.ymaxf)) return 0;
    const int okx = fast_coord(__fmaf_rn(x, ax.sf, ax.tf), ax, xi);
    const int oky = fast_coord(__fmaf_rn(y, ay.sf, ay.tf), ay, yi);
    return (okx & oky) ? 1 : 2;
}

// The exact float64 binning of an in-bounds float32 point: one out-of-line
// copy, kept out of the unrolled hot loops.  Scalars go in by value and the
// pair comes back packed in one 64-bit register: reference arguments would
// force the caller's bins and the axis structs into local memory.
static __device__ __noinline__ unsigned long long bin_exact_pair(float x, float y, double sx, double tx, int nx,
                                                                 double sy, double ty, int ny) {
    const unsigned xi = (unsigned)bin_exact64_st((double)x, sx, tx, nx);
    const unsigned yi = (unsigned)bin_exact64_st((double)y, sy, ty, ny);
    return (unsigned long long)xi | ((unsigned long long)yi << 32);
}
__device__ __forceinline__ void bin_exact_f32(float x, float y, const BinAxis &ax, const BinAxis &ay,
                                              int &xi, int &yi) {
    const unsigned long long r = bin_exact_pair(x, y, ax.s, ax.t, ax.n, ay.s, ay.t, ay.n);
    xi = (int)(unsigned)r;
    yi = (int)(unsigned)(r >> 32);
}

__device__ __forceinline__ bool bin_point_f32(float x, float y, const BinBounds &bb, const BinAxis &ax,
                                              const BinAxis &ay, int &xi, int &yi) {
    if (!(x >= bb.xminf && x <= bb.xmaxf && y >= bb.yminf && y <= bb.ymaxf)) return false;
    xi = bin_fast32<float>(x, x, ax);
    yi = bin_fast32<float>(y, y, ay);
    return true;
}

__device__ __forceinline__ bool bin_point_f64(double x, double y, const BinBounds &bb, const BinAxis &ax,
                                              const BinAxis &ay, int &xi, int &yi) {
    const long long kx = bound_key(x), ky = bound_key(y);
    if (!(kx >= bb.kxmin && kx <= bb.kxmax && ky >= bb.kymin && ky <= bb.kymax)) return false;
    float xf, yf;
    xi = f64_to_f32_trunc(x, xf) ? bin_fast32<double>(xf, x, ax) : bin_exact64(x, ax);
    yi = f64_to_f32_trunc(y, yf) ? bin_fast32<double>(yf, y, ay) : bin_exact64(y, ay);
    return true;
}

// ---------------------------------------------------------------- host side

// Smallest float >= v (as a double compare) / largest float <= v.
static inline float float_ceil_of(double v) {
    if (std::isnan(v)) return NAN;
    float f = (float)v;
    if ((double)f < v) f = nextafterf(f, INFINITY);
    return f;
}
static inline float float_floor_of(double v) {
    if (std::isnan(v)) return NAN;
    float f = (float)v;
    if ((double)f > v) f = nextafterf(f, -INFINITY);
    return f;
}

// Bound E on |fma32(x', sf, tf) - fl64(fl64(x*s) + t)| over lo <= x <= hi,
// with sf = (float)s, tf = (float)t and x' = x or its float32 truncation:
//   |x|max * |s - sf| + |t - tf|           representation of s and t
//   2^-23 * |x|max * |sf|                  truncation of a float64 x
//   2^-24 * (|x|max * |sf| + |tf|)         rounding of the float32 fma
//   2^-52 * (|x|max * |s| + |t|)           the two float64 roundings
// summed and doubled for margin.  +inf disables the fast path (non-finite
// values, or magnitudes at which float32 cannot resolve a pixel).
static inline double binning_error_bound(double lo, double hi, double s, double t, int n) {
    if (!std::isfinite(lo) || !std::isfinite(hi) || !std::isfinite(s) || !std::isfinite(t))
        return INFINITY;
    const double xm = std::fmax(std::fabs(lo), std::fabs(hi));
    const double sf = (double)(float)s, tf = (double)(float)t;
    const double mag = xm * std::fabs(s) + std::fabs(t) + (double)n + 1.0;
    if (!(mag < 1e6) || std::fabs(s) > 1e30 || xm > 1e30 || !std::isfinite(sf) || !std::isfinite(tf))
        return INFINITY;
    const double e = xm * std::fabs(s - sf) + std::fabs(t - tf) + ldexp(1.0, -23) * xm * std::fabs(sf) +
                     ldexp(1.0, -24) * (xm * std::fabs(sf) + std::fabs(tf)) +
                     ldexp(1.0, -52) * (xm * std::fabs(s) + std::fabs(t));
    return 2.0 * e + 1e-30;
}

static inline BinAxis make_axis(double s, double t, double lo, double hi, int n) {
    BinAxis a;
    a.s = s; a.t = t; a.sf = (float)s; a.tf = (float)t; a.n = n;
    a.e = (float)binning_error_bound(lo, hi, s, t, n);
    return a;
}

static inline BinBounds make_bounds(double xmin, double xmax, double ymin, double ymax) {
    BinBounds b;
    b.xminf = float_ceil_of(xmin); b.xmaxf = float_floor_of(xmax);
    b.yminf = float_ceil_of(ymin); b.ymaxf = float_floor_of(ymax);
    b.kxmin = bound_key(xmin); b.kxmax = bound_key(xmax);
    b.kymin = bound_key(ymin); b.kymax = bound_key(ymax);
    return b;
}

static inline bool fast_path_ok(const BinAxis &ax, const BinAxis &ay) {
    return std::isfinite(ax.e) && std::isfinite(ay.e) && ax.e < 0.01f && ay.e < 0.01f;
}

// The float64 image fl(fl(v * s) + t) of a float32 value, each operation
// rounded (volatile keeps the host compiler from fusing them).
static inline double image64(float v, double s, double t) {
    volatile double a = (double)v * s;
    volatile double b = a + t;
    return b;
}

// Precondition of the integer classification (bins from the float32 image
// alone: both in [0, n) with the fraction inside the window is inside the
// bounds; a bin outside [-1, n] is outside them; the rest take the float64
// formula): the smallest in-bounds float maps to >= 0 and the float below it
// to <= 0; the largest in-bounds float below n + 0.5 and the float above it
// to >= n.  The canvas relation of core.py:62-81 (t = -lo * s) gives this;
// other descriptors take the general binning.
static inline bool edges_ok(float lo, float hi, double s, double t, int n) {
    if (!(s > 0.0) || !std::isfinite(lo) || !std::isfinite(hi) || !(hi >= lo)) return false;
    return image64(nextafterf(lo, -INFINITY), s, t) <= 0.0 && image64(lo, s, t) >= 0.0 &&
           image64(hi, s, t) < n + 0.5 && image64(nextafterf(hi, INFINITY), s, t) >= (double)n;
}

}  // namespace dsgb
