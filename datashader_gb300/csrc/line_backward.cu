// line_backward.cu -- adjoints of the aggregation (no reference counterpart).
//
// dsgb_line_axis0_backward: the adjoint of the antialiased LineAxis0 sum('v')
// aggregate (self-intersecting form, overwrite == False: every pixel of
// segment i receives v_i * (aa - prev_aa), line.py:826-981 with
// reductions.py:1065-1075).  For a loss L with dL/dagg = g:
//
//   dL/dv_i  = sum over the pixels p that segment i appends of g[p] * (aa - prev_aa)
//   dL/dy_k  = sum over segments i-1, i, i+1 touching y_k of g[p] * v_i * d(aa - prev_aa)/dy_k
//
// Segment i depends on y_{i-1} (the previous vertex, used by the previous-
// segment correction), y_i and y_{i+1}.  The coverage is recomputed, never
// stored: each thread re-runs the segment's scan conversion in forward-mode
// dual arithmetic (a value and its three tangents), through the pixel
// mapping, Liang-Barsky clipping and _full_antialias.  Every branch is taken
// on the value, computed with the same operations as the forward kernel
// (this file is compiled without FMA contraction), so the pixels and
// decisions are exactly the forward pass's; the gradient is the derivative
// almost everywhere (clamps, abs, the integer scanline limits and the
// "value <= prev_value" choice are kinks with one-sided derivatives).
//
// dsgb_points_backward: the gather adjoint of points sum / mean with respect
// to the value column: dL/dv_i = g[p(i)] (sum) or g[p(i)] / count[p(i)] (mean)
// for rows that land on a pixel with a non-NaN value, 0 otherwise.
#include "dsgb_internal.cuh"
#include "binning.cuh"
#include "f64cmp.cuh"
#include "aa_scan.cuh"

#include <cmath>

namespace dsgb {

// ---------------------------------------------------------------- duals
//
// The value is float64 and computed with exactly the forward kernel's
// operations (it decides every pixel and branch).  The three tangents are
// float32: they only feed dL/dy, whose contract is agreement with float64
// finite differences to 1e-4 relative, and GB300 issues float64 at a small
// fraction of its float32 rate, so each dual operation costs one float64
// operation instead of seven.

struct D3 {
    double v;
    float g0, g1, g2;
};
__device__ __forceinline__ float f32(double v) { return __double2float_rn(v); }
__device__ __forceinline__ D3 dc(double v) { return D3{v, 0.0f, 0.0f, 0.0f}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return D3{a.v + b.v, a.g0 + b.g0, a.g1 + b.g1, a.g2 + b.g2}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return D3{a.v - b.v, a.g0 - b.g0, a.g1 - b.g1, a.g2 - b.g2}; }
__device__ __forceinline__ D3 operator-(D3 a) { return D3{-a.v, -a.g0, -a.g1, -a.g2}; }
__device__ __forceinline__ D3 operator*(D3 a, D3 b) {
    const float af = f32(a.v), bf = f32(b.v);
    return D3{a.v * b.v, a.g0 * bf + af * b.g0, a.g1 * bf + af * b.g1, a.g2 * bf + af * b.g2};
}
__device__ __forceinline__ D3 operator/(D3 a, D3 b) {
    const double q = a.v / b.v;
    const float qf = f32(q), rb = 1.0f / f32(b.v);
    return D3{q, (a.g0 - qf * b.g0) * rb, (a.g1 - qf * b.g1) * rb, (a.g2 - qf * b.g2) * rb};
}
__device__ __forceinline__ D3 dsqrt(D3 a) {
    const double r = sqrt(a.v);
    const float k = f64_gt0(r) ? 0.5f / f32(r) : 0.0f;
    return D3{r, a.g0 * k, a.g1 * k, a.g2 * k};
}
__device__ __forceinline__ D3 dabs(D3 a) { return f64_lt0(a.v) ? -a : a; }
__device__ __forceinline__ D3 dsq(D3 a) { return a * a; }
// max(0, min(x, 1)) with the comparisons m = x < 1 ? x : 1, 0 > m ? 0 : m,
// classified on the bit pattern (f64cmp.cuh): x itself (with its tangents)
// for [+0, 1) and -0.0, a constant 0 for negative x, a constant 1 for
// [1, inf] and NaN.
__device__ __forceinline__ D3 dclamp01(D3 x) {
    const unsigned long long T = f64_bits(x.v);
    if (T < F64_ONE || T == F64_SIGN) return x;
    return f64_lt0(x.v) ? dc(0.0) : dc(1.0);
}
// den = edge1 - edge0, computed once per segment; exactly 1.0 skips the
// division (x / 1.0 == x, and the constant divisor has no tangents), as in
// the forward kernel.
__device__ __forceinline__ D3 dlinearstep(double e0, double den, bool unit_den, D3 x) {
    const D3 d = x - dc(e0);
    return dclamp01(unit_den ? d : d / dc(den));
}
// element i (0..3) of four scalars, by selects
__device__ __forceinline__ double pick4_b(int i, double a0, double a1, double a2, double a3) {
    const double lo = (i & 1) ? a1 : a0, hi = (i & 1) ? a3 : a2;
    return (i & 2) ? hi : lo;
}

// line.py:783-800 in duals
__device__ __forceinline__ bool dclipt(D3 p, D3 q, D3 &t0, D3 &t1) {
    bool accept = true;
    if (f64_lt0(p.v) && f64_lt0(q.v)) {
        const D3 r = q / p;
        if (f64_lt(t1.v, r.v)) accept = false;
        else if (f64_lt(t0.v, r.v)) t0 = r;
    } else if (f64_gt0(p.v) && f64_lt(q.v, p.v)) {
        const D3 r = q / p;
        if (f64_lt(r.v, t0.v)) accept = false;
        else if (f64_lt(r.v, t1.v)) t1 = r;
    } else if (f64_lt0(q.v)) {
        accept = false;
    }
    return accept;
}

struct BwdParams {
    ColumnRef X, Y, V;
    int64_t n;
    int32_t width, height;
    double sx, tx, sy, ty;
    double xmin, xmax, ymin, ymax;
    double line_width;
    int64_t aa_nx, aa_ny;   // round((xmax - xmin) * sx), round((ymax - ymin) * sy), on the host
    int32_t plot_start;
    const double *grad;
    const uint8_t *any;
    double *grad_v, *grad_y;
};

// The appends of one segment: accumulates dL/dv_i and the three y tangents.
__device__ void segment_backward(const BwdParams &p, int64_t i, D3 x0, D3 x1, D3 y0, D3 y1,
                                 bool segment_start, bool segment_end, D3 xm, D3 ym,
                                 long long nx, long long ny, double field,
                                 double &gv, double &gy0, double &gy1, double &gy2) {
    double line_width = p.line_width;
    bool overwrite = false;
    if (f64_eq(x0.v, x1.v) && f64_eq(y0.v, y1.v)) return;
    const bool flip_xy = f64_abs_lt(x0.v - x1.v, y0.v - y1.v);
    if (flip_xy) {
        D3 t;
        t = x0; x0 = y0; y0 = t;
        t = x1; x1 = y1; y1 = t;
        t = xm; xm = ym; ym = t;
    }
    double scale = 1.0;
    if (line_width < 1.0) { scale *= line_width; line_width = 1.0; }
    const bool unit_scale = scale == 1.0;
    const double aa = 1.0;
    const double halfwidth = 0.5 * (line_width + aa);
    const bool flip_order = f64_lt(y1.v, y0.v) || (f64_eq(y1.v, y0.v) && f64_lt(x1.v, x0.v));
    D3 alongx = x1 - x0, alongy = y1 - y0;
    const D3 length = dsqrt(dsq(alongx) + dsq(alongy));
    alongx = alongx / length;
    alongy = alongy / length;
    const D3 rightx = alongy, righty = -alongx;
    // the corners only bound the scan (integers): plain float64 values, as
    // the forward kernel computes them (+-ca, +-cb shared)
    double bx0, bx1, bx2, bx3, by0, by1, by2, by3;
    const double ca = halfwidth * (rightx.v - alongx.v), cb = halfwidth * (rightx.v + alongx.v);
    if (flip_order) {
        bx0 = x1.v - ca; bx1 = x1.v + cb; bx2 = x0.v + ca; bx3 = x0.v - cb;
        by0 = y1.v + cb; by1 = y1.v + ca; by2 = y0.v - cb; by3 = y0.v - ca;
    } else {
        bx0 = x0.v + ca; bx1 = x0.v - cb; bx2 = x1.v - ca; bx3 = x1.v + cb;
        by0 = y0.v - cb; by1 = y0.v - ca; by2 = y1.v + cb; by3 = y1.v + ca;
    }
    long long xmaxi = nx - 1, ymaxi = ny - 1;
    if (flip_xy) { long long t = xmaxi; xmaxi = ymaxi; ymaxi = t; }
    const int lowindex = flip_order ? (f64_lt(x1.v, x0.v) ? 0 : 1) : (f64_lt(x0.v, x1.v) ? 0 : 1);
    D3 prev_alongx = dc(0), prev_alongy = dc(0), prev_length = dc(0), prev_rightx = dc(0), prev_righty = dc(0);
    if (!overwrite && !segment_start) {
        prev_alongx = x0 - xm;
        prev_alongy = y0 - ym;
        prev_length = dsqrt(dsq(prev_alongx) + dsq(prev_alongy));
        if (f64_gt0(prev_length.v)) {
            prev_alongx = prev_alongx / prev_length;
            prev_alongy = prev_alongy / prev_length;
            prev_rightx = prev_alongy;
            prev_righty = -prev_alongx;
        } else {
            overwrite = true;
        }
    }
    const long long ystart = f64_ceil_clamp(pick4_b(lowindex, by0, by1, by2, by3), ymaxi);
    const long long yend = f64_floor_clamp(pick4_b((lowindex + 2) % 4, by0, by1, by2, by3), ymaxi);
    int ll = lowindex, lu = (ll + 1) % 4, rl = lowindex, ru = (rl + 3) % 4;
    const double lw_lo = 0.5 * (line_width - aa);
    const double ls_den = halfwidth - lw_lo;
    const bool unit_den = ls_den == 1.0;
    // cap pixels at distance >= halfwidth append nothing (as in the forward kernel)
    const unsigned long long cap_far = f64_bits(__dmul_ru(halfwidth, halfwidth));
    float ty0 = 0.0f, ty1 = 0.0f, ty2 = 0.0f;     // the y tangents of this segment, in float32
    for (long long y = ystart; y <= yend; ++y) {
        const double yd = f64_from_u32((unsigned)y);
        if (ll == lowindex && f64_nonneg_gt(yd, pick4_b(lu, by0, by1, by2, by3))) { ll = lu; lu = (ll + 1) % 4; }
        if (rl == lowindex && f64_nonneg_gt(yd, pick4_b(ru, by0, by1, by2, by3))) { rl = ru; ru = (rl + 3) % 4; }
        // the span ends are integers: only the intercept's value matters (aa_scan.cuh)
        const long long xleft = aa_scan_bound<true>((unsigned)y, yd, pick4_b(ll, bx0, bx1, bx2, bx3),
            pick4_b(ll, by0, by1, by2, by3), pick4_b(lu, bx0, bx1, bx2, bx3), pick4_b(lu, by0, by1, by2, by3), xmaxi);
        const long long xright = aa_scan_bound<false>((unsigned)y, yd, pick4_b(rl, bx0, bx1, bx2, bx3),
            pick4_b(rl, by0, by1, by2, by3), pick4_b(ru, bx0, bx1, bx2, bx3), pick4_b(ru, by0, by1, by2, by3), xmaxi);
        for (long long x = xleft; x <= xright; ++x) {
            const D3 xd = dc(f64_from_u32((unsigned)x)), ydd = dc(yd);
            const D3 along = (xd - x0) * alongx + (ydd - y0) * alongy;
            bool prev_correction = false;
            D3 distance;
            if (f64_lt0(along.v)) {
                if (!(overwrite || segment_start || f64_gt0(((xd - x0) * prev_alongx + (ydd - y0) * prev_alongy).v)))
                    continue;
                const D3 d2 = dsq(xd - x0) + dsq(ydd - y0);
                if (f64_bits(d2.v) >= cap_far) continue;
                distance = dsqrt(d2);
            } else if (f64_gt_nonneg(along.v, length.v)) {
                if (!(overwrite || segment_end)) continue;
                const D3 d2 = dsq(xd - x1) + dsq(ydd - y1);
                if (f64_bits(d2.v) >= cap_far) continue;
                distance = dsqrt(d2);
            } else {
                distance = dabs((xd - x0) * rightx + (ydd - y0) * righty);
                if (!overwrite && !segment_start) {
                    const D3 pd = (xd - x0) * prev_alongx + (ydd - y0) * prev_alongy;
                    if (f64_in_neg_range(pd.v, prev_length.v) &&
                        f64_abs_le(((xd - x0) * prev_rightx + (ydd - y0) * prev_righty).v, halfwidth))
                        prev_correction = true;
                }
            }
            D3 value = dc(1.0) - dlinearstep(lw_lo, ls_den, unit_den, distance);
            if (!unit_scale) value = value * dc(scale);      // x * 1.0 == x
            D3 prev_value = dc(0.0);
            if (prev_correction) {
                const D3 prev_distance = dabs((xd - x0) * prev_rightx + (ydd - y0) * prev_righty);
                prev_value = dc(1.0) - dlinearstep(lw_lo, ls_den, unit_den, prev_distance);
                if (!unit_scale) prev_value = prev_value * dc(scale);
                if (f64_le_nonneg(value.v, prev_value.v)) value = dc(0.0);
            }
            if (f64_gt0(value.v)) {
                const long long xx = flip_xy ? y : x, yy = flip_xy ? x : y;
                if (xx < 0 || yy < 0 || xx >= p.width || yy >= p.height) continue;
                const int64_t pix = yy * (int64_t)p.width + xx;
                if (p.any && !p.any[pix]) continue;
                const double g = p.grad[pix];
                const D3 d = value - prev_value;
                gv += g * d.v;
                const float gf = f32(g * field);
                ty0 += gf * d.g0;
                ty1 += gf * d.g1;
                ty2 += gf * d.g2;
            }
        }
    }
    gy0 += (double)ty0;
    gy1 += (double)ty1;
    gy2 += (double)ty2;
}

// `order` (may be null) lists the segments in work order (see
// build_line_work_order): the lanes of a warp then recompute segments of
// similar pixel counts.  Each segment's results go to its own rows, so the
// order changes only the order of the grad_y atomics.
__global__ void __launch_bounds__(256, 1) line_backward_kernel(const BwdParams p, const unsigned *order) {
    for (int64_t k = gtid(); k + 1 < p.n; k += gstride()) {
        const int64_t i = order ? (int64_t)order[k] : k;
        const double field = load_f64(p.V, i);
        const double xv0 = load_f64(p.X, i), yv0 = load_f64(p.Y, i);
        const double xv1 = load_f64(p.X, i + 1), yv1 = load_f64(p.Y, i + 1);
        // the previous row, with numba's wrap of index -1 onto the last row
        const int64_t im = i > 0 ? i - 1 : p.n - 1;
        bool segment_start = (i == 0) ? (p.plot_start != 0)
                                      : (isnull(load_f64(p.X, im)) || isnull(load_f64(p.Y, im)));
        const bool segment_end = (i == p.n - 2) || isnull(load_f64(p.X, i + 2)) || isnull(load_f64(p.Y, i + 2));
        double xmv = 0.0, ymv = 0.0;
        if (!segment_start) { xmv = load_f64(p.X, im); ymv = load_f64(p.Y, im); }
        if (isnull(field) || isnull(xv0) || isnull(yv0) || isnull(xv1) || isnull(yv1)) continue;
        // tangents: g0 = d/dy_{i-1}, g1 = d/dy_i, g2 = d/dy_{i+1}
        D3 x0 = dc(xv0), x1 = dc(xv1);
        D3 y0 = D3{yv0, 0.0f, 1.0f, 0.0f}, y1 = D3{yv1, 0.0f, 0.0f, 1.0f};
        // line.py:734-780 (Liang-Barsky) in duals
        bool skip = false;
        if (f64_lt(x0.v, p.xmin) && f64_lt(x1.v, p.xmin)) skip = true;
        else if (f64_lt(p.xmax, x0.v) && f64_lt(p.xmax, x1.v)) skip = true;
        else if (f64_lt(y0.v, p.ymin) && f64_lt(y1.v, p.ymin)) skip = true;
        else if (f64_lt(p.ymax, y0.v) && f64_lt(p.ymax, y1.v)) skip = true;
        D3 t0 = dc(0.0), t1 = dc(1.0);
        const D3 dx1 = x1 - x0;
        if (!dclipt(-dx1, x0 - dc(p.xmin), t0, t1)) skip = true;
        if (!dclipt(dx1, dc(p.xmax) - x0, t0, t1)) skip = true;
        const D3 dy1 = y1 - y0;
        if (!dclipt(-dy1, y0 - dc(p.ymin), t0, t1)) skip = true;
        if (!dclipt(dy1, dc(p.ymax) - y0, t0, t1)) skip = true;
        if (skip) continue;
        bool cs = false;
        if (f64_lt(t1.v, 1.0)) { x1 = x0 + t1 * dx1; y1 = y0 + t1 * dy1; }
        if (f64_gt0(t0.v)) { cs = true; x0 = x0 + t0 * dx1; y0 = y0 + t0 * dy1; }
        segment_start = segment_start || cs;
        // line.py:723-726 (no snap) in duals
        const D3 sxd = dc(p.sx), txd = dc(p.tx), syd = dc(p.sy), tyd = dc(p.ty), half = dc(0.5);
        const D3 px0 = x0 * sxd + txd - half, py0 = y0 * syd + tyd - half;
        const D3 px1 = x1 * sxd + txd - half, py1 = y1 * syd + tyd - half;
        D3 pxm = dc(0.0), pym = dc(0.0);
        if (!segment_start) {
            pxm = dc(xmv) * sxd + txd - half;
            pym = D3{ymv, 1.0f, 0.0f, 0.0f} * syd + tyd - half;
        }
        const long long nx = p.aa_nx, ny = p.aa_ny;
        double gv = 0.0, gy0 = 0.0, gy1 = 0.0, gy2 = 0.0;
        segment_backward(p, i, px0, px1, py0, py1, segment_start, segment_end, pxm, pym, nx, ny, field,
                         gv, gy0, gy1, gy2);
        p.grad_v[i] = gv;   // only segment i appends row i's value
        if (f64_bits(gy0) & F64_MAG) atomicAdd(&p.grad_y[im], gy0);      // gy != 0.0 (NaN included)
        if (f64_bits(gy1) & F64_MAG) atomicAdd(&p.grad_y[i], gy1);
        if (f64_bits(gy2) & F64_MAG) atomicAdd(&p.grad_y[i + 1], gy2);
    }
}

// ---- the adjoint with pixels queued by case (as aa_queued_kernel, line.cu):
// each lane scans its segment and classifies the pixels in float32
// (aa_classify, the value's float64 tests reproduced), the warp works off its
// per-case queues 32 pixels at a time with every lane on one dual-number
// path.  A pixel's dL/dv term goes to a shared-memory slot indexed by (its
// segment, the working lane), summed per segment in lane order at the end of
// the batch; its three float32 tangent terms are staged per round and summed
// by the segment's lane in round order.  Both orders are fixed by the work,
// so the results repeat run to run; they differ from the per-segment scan's
// order by rounding only.
constexpr int BQ_WARPS = 4;
constexpr int BQ_BLOCKS_PER_SM = 3;               // 72 KB of shared memory each

struct AASegB {                            // a segment in the flipped frame, dual values
    D3 x0, y0, x1, y1, ax, ay, len, pax, pay, plen;
    double field;
    unsigned flags;                        // AAF_* (line.cu)
};
constexpr unsigned BAF_OVERWRITE = 1u, BAF_START = 2u, BAF_END = 4u, BAF_FLIP = 8u, BAF_PREV = 16u;

struct BQShared {
    AASegB seg[BQ_WARPS][32];
    double gslot[BQ_WARPS][32][32];        // [segment lane][working lane]
    unsigned long long q[BQ_WARPS][3][64];
    float4 tstage[BQ_WARPS][32];           // a round's tangent terms; w = the segment lane (as float bits), -1: none
};

struct BQConsts {
    double halfwidth, lw_lo, ls_den, scale;
    bool unit_den, unit_scale;
    unsigned long long cap_far;
};

__device__ __forceinline__ D3 bq_ramp(const BQConsts &c, D3 d) {
    D3 v = dc(1.0) - dlinearstep(c.lw_lo, c.ls_den, c.unit_den, d);
    if (!c.unit_scale) v = v * dc(c.scale);
    return v;
}

// value and prev_value of one queued pixel (which: 0 cap, 1 side, 2 exact);
// false when nothing is appended
__device__ __forceinline__ bool bq_pixel(const BQConsts &c, const AASegB &S, int which, bool before, long long x,
                                         long long y, D3 &value, D3 &prev_value) {
    const D3 xd = dc(f64_from_u32((unsigned)x)), ydd = dc(f64_from_u32((unsigned)y));
    const bool overwrite = S.flags & BAF_OVERWRITE, start = S.flags & BAF_START, end = S.flags & BAF_END;
    prev_value = dc(0.0);
    bool prev_correction = false;
    D3 distance;
    if (which == 2) {                                     // the per-segment body, all cases
        const D3 along = (xd - S.x0) * S.ax + (ydd - S.y0) * S.ay;
        if (f64_lt0(along.v)) {
            if (!(overwrite || start || f64_gt0(((xd - S.x0) * S.pax + (ydd - S.y0) * S.pay).v))) return false;
            which = 0; before = true;
        } else if (f64_gt_nonneg(along.v, S.len.v)) {
            if (!(overwrite || end)) return false;
            which = 0; before = false;
        } else {
            which = 1;
        }
    }
    if (which == 0) {
        const D3 d2 = before ? dsq(xd - S.x0) + dsq(ydd - S.y0) : dsq(xd - S.x1) + dsq(ydd - S.y1);
        if (f64_bits(d2.v) >= c.cap_far) return false;
        distance = dsqrt(d2);
    } else {
        distance = dabs((xd - S.x0) * S.ay + (ydd - S.y0) * -S.ax);
        if (S.flags & BAF_PREV) {
            const D3 pd = (xd - S.x0) * S.pax + (ydd - S.y0) * S.pay;
            if (f64_in_neg_range(pd.v, S.plen.v) &&
                f64_abs_le(((xd - S.x0) * S.pay + (ydd - S.y0) * -S.pax).v, c.halfwidth))
                prev_correction = true;
        }
    }
    value = bq_ramp(c, distance);
    if (prev_correction) {
        prev_value = bq_ramp(c, dabs((xd - S.x0) * S.pay + (ydd - S.y0) * -S.pax));
        if (f64_le_nonneg(value.v, prev_value.v)) value = dc(0.0);
    }
    return f64_gt0(value.v);
}

__global__ void __launch_bounds__(BQ_WARPS * 32) line_backward_queued_kernel(const BwdParams p, const unsigned *order) {
    extern __shared__ __align__(16) unsigned char bq_smem[];
    BQShared &sh = *reinterpret_cast<BQShared *>(bq_smem);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    AASegB *segs = sh.seg[warp];
    BQConsts c;
    {
        double lw = p.line_width;
        c.scale = 1.0;
        if (lw < 1.0) { c.scale *= lw; lw = 1.0; }
        c.unit_scale = c.scale == 1.0;
        c.halfwidth = 0.5 * (lw + 1.0);
        c.lw_lo = 0.5 * (lw - 1.0);
        c.ls_den = c.halfwidth - c.lw_lo;
        c.unit_den = c.ls_den == 1.0;
        c.cap_far = f64_bits(__dmul_ru(c.halfwidth, c.halfwidth));
    }
    for (int j = 0; j < 32; ++j) sh.gslot[warp][lane][j] = 0.0;
    const int64_t nseg = p.n - 1;
    const int64_t nbatches = (nseg + 31) / 32;
    const int64_t warps_total = (int64_t)gridDim.x * BQ_WARPS;
    for (int64_t b = (int64_t)blockIdx.x * BQ_WARPS + warp; b < nbatches; b += warps_total) {
        const int64_t k = b * 32 + lane;
        bool set_up = false, active = false;
        int64_t i = 0, im = 0;
        AASegB S;
        long long cy = 0, cyend = -1, cx = 1, cxr = 0, xmaxi = 0;
        int ll = 0, lu = 1, rl = 0, ru = 3, lowindex = 0;
        double bx0 = 0, bx1 = 0, bx2 = 0, bx3 = 0, by0 = 0, by1 = 0, by2 = 0, by3 = 0;
        AAClassF kf = AAClassF{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (k < nseg) {
            // ---- line_backward_kernel's prologue and segment_backward's set-up
            i = order ? (int64_t)order[k] : k;
            const double field = load_f64(p.V, i);
            const double xv0 = load_f64(p.X, i), yv0 = load_f64(p.Y, i);
            const double xv1 = load_f64(p.X, i + 1), yv1 = load_f64(p.Y, i + 1);
            im = i > 0 ? i - 1 : p.n - 1;
            bool segment_start = (i == 0) ? (p.plot_start != 0)
                                          : (isnull(load_f64(p.X, im)) || isnull(load_f64(p.Y, im)));
            const bool segment_end = (i == p.n - 2) || isnull(load_f64(p.X, i + 2)) || isnull(load_f64(p.Y, i + 2));
            double xmv = 0.0, ymv = 0.0;
            if (!segment_start) { xmv = load_f64(p.X, im); ymv = load_f64(p.Y, im); }
            bool skip = isnull(field) || isnull(xv0) || isnull(yv0) || isnull(xv1) || isnull(yv1);
            D3 x0 = dc(xv0), x1 = dc(xv1);
            D3 y0 = D3{yv0, 0.0f, 1.0f, 0.0f}, y1 = D3{yv1, 0.0f, 0.0f, 1.0f};
            if (f64_lt(x0.v, p.xmin) && f64_lt(x1.v, p.xmin)) skip = true;
            else if (f64_lt(p.xmax, x0.v) && f64_lt(p.xmax, x1.v)) skip = true;
            else if (f64_lt(y0.v, p.ymin) && f64_lt(y1.v, p.ymin)) skip = true;
            else if (f64_lt(p.ymax, y0.v) && f64_lt(p.ymax, y1.v)) skip = true;
            D3 t0 = dc(0.0), t1 = dc(1.0);
            const D3 dx1 = x1 - x0;
            if (!dclipt(-dx1, x0 - dc(p.xmin), t0, t1)) skip = true;
            if (!dclipt(dx1, dc(p.xmax) - x0, t0, t1)) skip = true;
            const D3 dy1 = y1 - y0;
            if (!dclipt(-dy1, y0 - dc(p.ymin), t0, t1)) skip = true;
            if (!dclipt(dy1, dc(p.ymax) - y0, t0, t1)) skip = true;
            if (!skip) {
                bool cs = false;
                if (f64_lt(t1.v, 1.0)) { x1 = x0 + t1 * dx1; y1 = y0 + t1 * dy1; }
                if (f64_gt0(t0.v)) { cs = true; x0 = x0 + t0 * dx1; y0 = y0 + t0 * dy1; }
                segment_start = segment_start || cs;
                const D3 sxd = dc(p.sx), txd = dc(p.tx), syd = dc(p.sy), tyd = dc(p.ty), half = dc(0.5);
                D3 px0 = x0 * sxd + txd - half, py0 = y0 * syd + tyd - half;
                D3 px1 = x1 * sxd + txd - half, py1 = y1 * syd + tyd - half;
                D3 pxm = dc(0.0), pym = dc(0.0);
                if (!segment_start) {
                    pxm = dc(xmv) * sxd + txd - half;
                    pym = D3{ymv, 1.0f, 0.0f, 0.0f} * syd + tyd - half;
                }
                set_up = true;
                if (!(f64_eq(px0.v, px1.v) && f64_eq(py0.v, py1.v))) {
                    bool overwrite = false;
                    const bool flip_xy = f64_abs_lt(px0.v - px1.v, py0.v - py1.v);
                    if (flip_xy) {
                        D3 t;
                        t = px0; px0 = py0; py0 = t;
                        t = px1; px1 = py1; py1 = t;
                        t = pxm; pxm = pym; pym = t;
                    }
                    const bool flip_order = f64_lt(py1.v, py0.v) || (f64_eq(py1.v, py0.v) && f64_lt(px1.v, px0.v));
                    D3 alongx = px1 - px0, alongy = py1 - py0;
                    const D3 length = dsqrt(dsq(alongx) + dsq(alongy));
                    alongx = alongx / length;
                    alongy = alongy / length;
                    const double ca = c.halfwidth * (alongy.v - alongx.v), cb = c.halfwidth * (alongy.v + alongx.v);
                    if (flip_order) {
                        bx0 = px1.v - ca; bx1 = px1.v + cb; bx2 = px0.v + ca; bx3 = px0.v - cb;
                        by0 = py1.v + cb; by1 = py1.v + ca; by2 = py0.v - cb; by3 = py0.v - ca;
                    } else {
                        bx0 = px0.v + ca; bx1 = px0.v - cb; bx2 = px1.v - ca; bx3 = px1.v + cb;
                        by0 = py0.v - cb; by1 = py0.v - ca; by2 = py1.v + cb; by3 = py1.v + ca;
                    }
                    xmaxi = p.aa_nx - 1;
                    long long ymaxi = p.aa_ny - 1;
                    if (flip_xy) { const long long t = xmaxi; xmaxi = ymaxi; ymaxi = t; }
                    lowindex = flip_order ? (f64_lt(px1.v, px0.v) ? 0 : 1) : (f64_lt(px0.v, px1.v) ? 0 : 1);
                    D3 pax = dc(0.0), pay = dc(0.0), plen = dc(0.0);
                    if (!segment_start) {
                        pax = px0 - pxm;
                        pay = py0 - pym;
                        plen = dsqrt(dsq(pax) + dsq(pay));
                        if (f64_gt0(plen.v)) {
                            pax = pax / plen;
                            pay = pay / plen;
                        } else {
                            overwrite = true;
                        }
                    }
                    S.x0 = px0; S.y0 = py0; S.x1 = px1; S.y1 = py1;
                    S.ax = alongx; S.ay = alongy; S.len = length;
                    S.pax = pax; S.pay = pay; S.plen = plen;
                    S.field = field;
                    S.flags = (overwrite ? BAF_OVERWRITE : 0u) | (segment_start ? BAF_START : 0u) |
                              (segment_end ? BAF_END : 0u) | (flip_xy ? BAF_FLIP : 0u) |
                              (!overwrite && !segment_start ? BAF_PREV : 0u);
                    cy = f64_ceil_clamp(pick4_b(lowindex, by0, by1, by2, by3), ymaxi) - 1;
                    cyend = f64_floor_clamp(pick4_b((lowindex + 2) % 4, by0, by1, by2, by3), ymaxi);
                    ll = lowindex; lu = (ll + 1) % 4; rl = lowindex; ru = (rl + 3) % 4;
                    kf = AAClassF{(float)px0.v, (float)py0.v, (float)alongx.v, (float)alongy.v, (float)length.v,
                                  (float)pax.v, (float)pay.v};
                    active = true;
                    segs[lane] = S;
                }
            }
        }
        __syncwarp();
        const bool cap_before = active && (S.flags & (BAF_OVERWRITE | BAF_START));
        const bool cap_after = active && (S.flags & (BAF_OVERWRITE | BAF_END));
        float ta0 = 0.0f, ta1 = 0.0f, ta2 = 0.0f;      // this lane's segment's tangent sums
        int nq[3] = {0, 0, 0};
        while (true) {
            // ---- one pixel per lane from its scan, classified (as the forward kernel)
            int kind = -1;
            bool before = false;
            long long px = 0, py = 0;
            while (active) {
                if (cx <= cxr) { px = cx; py = cy; ++cx; kind = 2; break; }
                if (++cy > cyend) { active = false; break; }
                const double yd = f64_from_u32((unsigned)cy);
                if (ll == lowindex && f64_nonneg_gt(yd, pick4_b(lu, by0, by1, by2, by3))) { ll = lu; lu = (ll + 1) % 4; }
                if (rl == lowindex && f64_nonneg_gt(yd, pick4_b(ru, by0, by1, by2, by3))) { rl = ru; ru = (rl + 3) % 4; }
                cx = aa_scan_bound<true>((unsigned)cy, yd, pick4_b(ll, bx0, bx1, bx2, bx3), pick4_b(ll, by0, by1, by2, by3),
                                         pick4_b(lu, bx0, bx1, bx2, bx3), pick4_b(lu, by0, by1, by2, by3), xmaxi);
                cxr = aa_scan_bound<false>((unsigned)cy, yd, pick4_b(rl, bx0, bx1, bx2, bx3), pick4_b(rl, by0, by1, by2, by3),
                                           pick4_b(ru, bx0, bx1, bx2, bx3), pick4_b(ru, by0, by1, by2, by3), xmaxi);
            }
            if (kind == 2) {
                switch (aa_classify((unsigned)px, (unsigned)py, kf, cap_before, cap_after)) {
                case AAC_NONE: kind = -1; break;
                case AAC_CAP_BEFORE: kind = 0; before = true; break;
                case AAC_CAP_AFTER: kind = 0; break;
                case AAC_SIDE: kind = 1; break;
                default: break;
                }
            }
            const unsigned long long item = (unsigned long long)px | ((unsigned long long)py << 24) |
                                            ((unsigned long long)lane << 48) | ((unsigned long long)before << 53);
#pragma unroll
            for (int w = 0; w < 3; ++w) {
                const unsigned m = __ballot_sync(0xffffffffu, kind == w);
                if (kind == w) sh.q[warp][w][nq[w] + __popc(m & lt_mask)] = item;
                nq[w] += __popc(m);
            }
            __syncwarp();
            const bool last = !__any_sync(0xffffffffu, active);
            // ---- work off rounds of 32 (all of them after the last pixels)
            while (true) {
                int which;
                if (nq[0] >= 32 || (last && nq[0] > 0)) which = 0;
                else if (nq[1] >= 32 || (last && nq[1] > 0)) which = 1;
                else if (nq[2] >= 32 || (last && nq[2] > 0)) which = 2;
                else break;
                const int cnt = nq[which];
                const int take = cnt < 32 ? cnt : 32;
                const int from = cnt - take;
                nq[which] = from;
                float4 st = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
                if (lane < take) {
                    const unsigned long long it = sh.q[warp][which][from + lane];
                    const int sl = (int)((it >> 48) & 31u);
                    const AASegB &T = segs[sl];
                    const long long x = (long long)(it & 0xFFFFFFu), y = (long long)((it >> 24) & 0xFFFFFFu);
                    D3 value, prev_value;
                    if (bq_pixel(c, T, which, (it >> 53) & 1u, x, y, value, prev_value)) {
                        const long long xx = (T.flags & BAF_FLIP) ? y : x, yy = (T.flags & BAF_FLIP) ? x : y;
                        if (xx >= 0 && yy >= 0 && xx < p.width && yy < p.height) {
                            const int64_t pix = yy * (int64_t)p.width + xx;
                            if (!p.any || p.any[pix]) {
                                const double g = p.grad[pix];
                                const D3 d = value - prev_value;
                                sh.gslot[warp][sl][lane] += g * d.v;
                                const float gf = f32(g * T.field);
                                st = make_float4(gf * d.g0, gf * d.g1, gf * d.g2, __int_as_float(sl));
                            }
                        }
                    }
                }
                if (__any_sync(0xffffffffu, __float_as_int(st.w) >= 0)) {
                    sh.tstage[warp][lane] = st;
                    __syncwarp();
                    for (int j = 0; j < 32; ++j) {                // this round's terms of this lane's segment, in lane order
                        const float4 t = sh.tstage[warp][j];
                        if (__float_as_int(t.w) == lane) { ta0 += t.x; ta1 += t.y; ta2 += t.z; }
                    }
                    __syncwarp();
                }
            }
            __syncwarp();
            if (last) break;
        }
        // ---- the batch's results, one segment a lane
        if (set_up) {
            double gv = 0.0;
            for (int j = 0; j < 32; ++j) {
                gv += sh.gslot[warp][lane][j];
                sh.gslot[warp][lane][j] = 0.0;
            }
            p.grad_v[i] = gv;                                  // only segment i appends row i's value
            const double gy0 = (double)ta0, gy1 = (double)ta1, gy2 = (double)ta2;
            if (f64_bits(gy0) & F64_MAG) atomicAdd(&p.grad_y[im], gy0);
            if (f64_bits(gy1) & F64_MAG) atomicAdd(&p.grad_y[i], gy1);
            if (f64_bits(gy2) & F64_MAG) atomicAdd(&p.grad_y[i + 1], gy2);
        }
        __syncwarp();
    }
}

// ---- points sum / mean gather adjoint
struct PBwdParams {
    ColumnRef X, Y, V;
    int64_t n;
    BinAxis ax, ay;
    double xmin, xmax, ymin, ymax;
    int32_t width;
    const double *grad;
    const uint32_t *counts;
    double *grad_v;
};

__global__ void __launch_bounds__(256) points_backward_kernel(const PBwdParams p) {
    for (int64_t i = gtid(); i < p.n; i += gstride()) {
        const double x = load_f64(p.X, i), y = load_f64(p.Y, i), v = load_f64(p.V, i);
        double g = 0.0;
        if (!isnull(v) && (p.xmin <= x && x <= p.xmax) && (p.ymin <= y && y <= p.ymax)) {
            const int xi = bin_exact64(x, p.ax), yi = bin_exact64(y, p.ay);
            const int64_t pix = (int64_t)yi * p.width + xi;
            g = p.grad[pix];
            if (p.counts) g = g / (double)p.counts[pix];
        }
        p.grad_v[i] = g;
    }
}


}  // namespace dsgb

using namespace dsgb;

extern "C" int dsgb_line_axis0_backward_ws(const dsgb_column *cols, int32_t ncols, int64_t n,
                                           int32_t x_col, int32_t y_col, int32_t v_col,
                                           const dsgb_canvas *canvas, double line_width,
                                           int32_t plot_start, const double *grad_agg,
                                           const uint8_t *agg_any, double *grad_v, double *grad_y,
                                           void *workspace, size_t workspace_bytes, void *stream) {
    if (!cols || !canvas || !grad_agg || !grad_v || !grad_y || n < 0 || x_col < 0 || y_col < 0 || v_col < 0 ||
        x_col >= ncols || y_col >= ncols || v_col >= ncols || canvas->width <= 0 || canvas->height <= 0) {
        set_error("dsgb_line_axis0_backward: invalid arguments");
        return DSGB_E_INVALID;
    }
    if (!(line_width > 0.0) || canvas->x_log || canvas->y_log) {
        set_error("dsgb_line_axis0_backward: needs an antialiased line (line_width > 0) on linear axes");
        return DSGB_E_UNSUPPORTED;
    }
    BwdParams p;
    memset(&p, 0, sizeof(p));
    p.X = ColumnRef{cols[x_col].data, cols[x_col].dtype};
    p.Y = ColumnRef{cols[y_col].data, cols[y_col].dtype};
    p.V = ColumnRef{cols[v_col].data, cols[v_col].dtype};
    p.n = n; p.width = canvas->width; p.height = canvas->height;
    p.sx = canvas->sx; p.tx = canvas->tx; p.sy = canvas->sy; p.ty = canvas->ty;
    p.xmin = canvas->xmin; p.xmax = canvas->xmax; p.ymin = canvas->ymin; p.ymax = canvas->ymax;
    p.line_width = line_width; p.plot_start = plot_start;
    const double span_x = (p.xmax - p.xmin) * p.sx, span_y = (p.ymax - p.ymin) * p.sy;
    if (!(std::fabs(span_x) < 2147483648.0) || !(std::fabs(span_y) < 2147483648.0)) {
        set_error("dsgb_line_axis0_backward: the canvas spans (xmax - xmin) * sx and (ymax - ymin) * sy must be below 2^31 pixels");
        return DSGB_E_INVALID;
    }
    p.aa_nx = (int64_t)std::rint(span_x);     // Python round: half to even, as rint
    p.aa_ny = (int64_t)std::rint(span_y);
    p.grad = grad_agg; p.any = agg_any; p.grad_v = grad_v; p.grad_y = grad_y;
    cudaStream_t st = as_stream(stream);
    cudaError_t e = cudaMemsetAsync(grad_y, 0, (size_t)n * 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(grad_v, 0, (size_t)n * 8, st);
    if (e != cudaSuccess) return cuda_status(e, "dsgb_line_axis0_backward memset");
    if (n > 1) {
        LineWorkArgs a;
        a.X = p.X; a.Y = p.Y; a.n = n; a.sx = p.sx; a.sy = p.sy; a.line_width = line_width;
        const unsigned *order = build_line_work_order(a, workspace, workspace_bytes, st);
        if (p.aa_nx <= (1 << 24) && p.aa_ny <= (1 << 24)) {
            // pixels queued by case (24-bit pixel coordinates in the queue items)
            e = cudaFuncSetAttribute(line_backward_queued_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(BQShared));
            if (e != cudaSuccess) return cuda_status(e, "dsgb_line_axis0_backward smem attribute");
            int sms = sm_count();
            if (sms <= 0) sms = 148;
            line_backward_queued_kernel<<<(unsigned)(sms * BQ_BLOCKS_PER_SM), BQ_WARPS * 32, sizeof(BQShared), st>>>(p, order);
        } else {
            line_backward_kernel<<<grid_of(n), 256, 0, st>>>(p, order);
        }
    }
    DSGB_CHECK_LAUNCH("dsgb_line_axis0_backward");
    return DSGB_OK;
}

extern "C" int dsgb_line_axis0_backward(const dsgb_column *cols, int32_t ncols, int64_t n,
                                        int32_t x_col, int32_t y_col, int32_t v_col,
                                        const dsgb_canvas *canvas, double line_width,
                                        int32_t plot_start, const double *grad_agg,
                                        const uint8_t *agg_any, double *grad_v, double *grad_y,
                                        void *stream) {
    return dsgb_line_axis0_backward_ws(cols, ncols, n, x_col, y_col, v_col, canvas, line_width, plot_start,
                                       grad_agg, agg_any, grad_v, grad_y, nullptr, 0, stream);
}

extern "C" int dsgb_points_backward(const dsgb_column *cols, int32_t ncols, int64_t n,
                                    int32_t x_col, int32_t y_col, int32_t v_col,
                                    const dsgb_canvas *canvas, const double *grad_agg,
                                    const uint32_t *counts, double *grad_v, uint32_t flags, void *stream) {
    (void)flags;
    if (!cols || !canvas || !grad_agg || !grad_v || n < 0 || x_col < 0 || y_col < 0 || v_col < 0 ||
        x_col >= ncols || y_col >= ncols || v_col >= ncols || canvas->width <= 0 || canvas->height <= 0) {
        set_error("dsgb_points_backward: invalid arguments");
        return DSGB_E_INVALID;
    }
    if (canvas->x_log || canvas->y_log) {
        set_error("dsgb_points_backward: log axes are not supported");
        return DSGB_E_UNSUPPORTED;
    }
    PBwdParams p;
    memset(&p, 0, sizeof(p));
    p.X = ColumnRef{cols[x_col].data, cols[x_col].dtype};
    p.Y = ColumnRef{cols[y_col].data, cols[y_col].dtype};
    p.V = ColumnRef{cols[v_col].data, cols[v_col].dtype};
    p.n = n;
    p.ax = make_axis(canvas->sx, canvas->tx, canvas->xmin, canvas->xmax, canvas->width);
    p.ay = make_axis(canvas->sy, canvas->ty, canvas->ymin, canvas->ymax, canvas->height);
    p.xmin = canvas->xmin; p.xmax = canvas->xmax; p.ymin = canvas->ymin; p.ymax = canvas->ymax;
    p.width = canvas->width;
    p.grad = grad_agg; p.counts = counts; p.grad_v = grad_v;
    if (n > 0) points_backward_kernel<<<grid_of(n), 256, 0, as_stream(stream)>>>(p);
    DSGB_CHECK_LAUNCH("dsgb_points_backward");
    return DSGB_OK;
}
