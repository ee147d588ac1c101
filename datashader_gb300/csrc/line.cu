// line.cu -- Canvas.line, LineAxis0 glyph, on GB300.
//
// Replaces LineAxis0._internal_build_extend / _build_extend_line_axis0
// (datashader/glyphs/line.py:59-103, 1099-1149) with draw_segment
// (1033-1097), Liang-Barsky clipping (734-800), pixel mapping (688-731),
// Bresenham (986-1031) and the antialiased wide-line scan conversion
// _full_antialias (826-981).
//
// One thread draws one segment (rows i, i+1); the pixel appends are
// atomics on the caller's bases.  This file is compiled with -fmad=false:
// numba contracts no multiply-adds, so every product and sum is rounded
// separately and the coverage values are bit-identical to the reference's.
// Only the order of the floating-point accumulation differs (atomics).
#include "dsgb_internal.cuh"
#include "f64cmp.cuh"
#include "aa_scan.cuh"

#include <cmath>

namespace dsgb {

struct LineParams {
    ColumnRef cols[MAX_COLS];
    BaseDev bases[MAX_BASES];
    int32_t ncols, nbases;
    int64_t n, row_offset;
    int32_t x_col, y_col;
    int32_t width, height;
    double sx, tx, sy, ty;
    double xmin, xmax, ymin, ymax;
    double line_width;
    int64_t aa_nx, aa_ny;   // round((xmax - xmin) * sx), round((ymax - ymin) * sy) (line.py:1070-1071)
    int32_t plot_start, overwrite, use_2_stage;
    int64_t field_mod;      // > 0: appends carry a visit key (row = key % field_mod); 0: the row itself
    int32_t debug;          // DSGB_FLAG_DEBUG_CHECKS
};

// One append of row i (field row = segment start) at pixel (x, y).
// aa / pa are aa_factor / prev_aa_factor (1, 0 for Bresenham lines).  KEYED:
// `key` is a visit key (line j, row r: j * p.field_mod + r) that orders the
// row-index bases as the reference visits the appends, and the fields are
// read at row r; otherwise `key` is the row.
template <bool KEYED>
__device__ void line_append(const LineParams &p, int64_t key, long long x, long long y,
                            double aa, double pa) {
    if (x < 0 || y < 0 || x >= p.width || y >= p.height) {   // memory safety only
        if (p.debug) raise_status(DSGB_STATUS_INDEX);
        return;
    }
    const int64_t pix = (int64_t)y * p.width + x;
    const int64_t i = KEYED ? key % p.field_mod : key;
    const long long row = (long long)(key + p.row_offset);
#pragma unroll 1
    for (int b = 0; b < p.nbases; ++b) {
        const BaseDev &B = p.bases[b];
        int64_t cell = pix;
        if (B.cat_col >= 0) {
            long long c = load_i64(p.cols[B.cat_col], i);
            if (c < 0) c += B.ncat;
            if (c < 0 || c >= B.ncat) {
                if (p.debug) raise_status(DSGB_STATUS_INDEX);
                continue;
            }
            cell = pix * B.ncat + c;
        }
        double field = 1.0;
        bool has = true;
        if (B.col >= 0) {
            field = load_f64(p.cols[B.col], i);
            has = !isnull(field);
        }
        const bool unweighted = (B.flags & DSGB_BASEF_UNWEIGHTED) || B.col < 0;
        switch (B.op) {
        case DSGB_BASE_COUNT: if (has) atomicAdd((unsigned *)B.agg + cell, 1u); break;
        case DSGB_BASE_ANY: if (has) ((volatile uint8_t *)B.agg)[cell] = 1; break;
        case DSGB_BASE_SUM: if (has) atomicAdd((double *)B.agg + cell, field); break;
        case DSGB_BASE_MAX: if (has) atomic_max_key((long long *)B.agg + cell, f64_key(field)); break;
        case DSGB_BASE_MIN: if (has) atomic_min_key((long long *)B.agg + cell, f64_key(field)); break;
        case DSGB_BASE_MIN_ROW: if (has) atomic_min_key((long long *)B.agg + cell, row); break;
        case DSGB_BASE_MAX_ROW: if (has) atomic_max_key((long long *)B.agg + cell, row); break;
        case DSGB_BASE_ARGMAX: if (has) pair_update<true>((long long *)B.agg + 2 * cell, f64_key(field), row); break;
        case DSGB_BASE_ARGMIN: if (has) pair_update<false>((long long *)B.agg + 2 * cell, f64_key(field), row); break;
        case DSGB_BASE_AA_SUM: {
            // reductions.py:966-973, 1065-1075, 560-569: value = field*(aa - prev)
            if (!has) break;
            double d = aa - pa;
            double value = unweighted ? d : field * d;
            if (!isnull(value)) atomicAdd((double *)B.agg + cell, value);
            break; }
        case DSGB_BASE_AA_CNT0:
            // reductions.py:680-685: count once per row (prev_aa_factor == 0)
            if (has && pa == 0.0) atomicAdd((unsigned *)B.agg + cell, 1u);
            break;
        case DSGB_BASE_AA_MAX: {
            // reductions.py:1186-1192 and siblings: keep the largest field*aa
            if (!has) break;
            double value = unweighted ? aa : field * aa;
            if (!isnull(value)) atomic_max_key((long long *)B.agg + cell, f64_key(value));
            break; }
        case DSGB_BASE_AA_ARGMAX: {
            if (!has) break;
            double value = unweighted ? aa : field * aa;
            if (!isnull(value)) pair_update<true>((long long *)B.agg + 2 * cell, f64_key(value), row);
            break; }
        default: break;
        }
    }
}

// line.py:783-800.  Comparisons by integer operations (f64cmp.cuh), IEEE
// results for every input.
__device__ __forceinline__ bool clipt(double p, double q, double &t0, double &t1) {
    bool accept = true;
    if (f64_lt0(p) && f64_lt0(q)) {
        double r = q / p;
        if (f64_lt(t1, r)) accept = false;
        else if (f64_lt(t0, r)) t0 = r;
    } else if (f64_gt0(p) && f64_lt(q, p)) {
        double r = q / p;
        if (f64_lt(r, t0)) accept = false;
        else if (f64_lt(r, t1)) t1 = r;
    } else if (f64_lt0(q)) {
        accept = false;
    }
    return accept;
}

// line.py:734-780
__device__ __forceinline__ void liang_barsky(double xmin, double xmax, double ymin, double ymax,
                                             double &x0, double &x1, double &y0, double &y1,
                                             bool &skip, bool &cs, bool &ce) {
    if (f64_lt(x0, xmin) && f64_lt(x1, xmin)) skip = true;
    else if (f64_lt(xmax, x0) && f64_lt(xmax, x1)) skip = true;
    else if (f64_lt(y0, ymin) && f64_lt(y1, ymin)) skip = true;
    else if (f64_lt(ymax, y0) && f64_lt(ymax, y1)) skip = true;
    double t0 = 0, t1 = 1;
    double dx1 = x1 - x0;
    if (!clipt(-dx1, x0 - xmin, t0, t1)) skip = true;
    if (!clipt(dx1, xmax - x0, t0, t1)) skip = true;
    double dy1 = y1 - y0;
    if (!clipt(-dy1, y0 - ymin, t0, t1)) skip = true;
    if (!clipt(dy1, ymax - y0, t0, t1)) skip = true;
    if (f64_lt(t1, 1.0)) { ce = true; x1 = x0 + t1 * dx1; y1 = y0 + t1 * dy1; } else ce = false;
    if (f64_gt0(t0)) { cs = true; x0 = x0 + t0 * dx1; y0 = y0 + t0 * dy1; } else cs = false;
}

__device__ __forceinline__ double sq(double v) { return v * v; }
// element i (0..3) of four scalars, by selects
__device__ __forceinline__ double pick4(int i, double a0, double a1, double a2, double a3) {
    const double lo = (i & 1) ? a1 : a0, hi = (i & 1) ? a3 : a2;
    return (i & 2) ? hi : lo;
}

// line.py:826-981 -- _full_antialias.
template <bool KEYED>
__device__ void full_antialias(const LineParams &p, double line_width, bool overwrite, int64_t i,
                               double x0, double x1, double y0, double y1,
                               bool segment_start, bool segment_end, double xm, double ym,
                               long long nx, long long ny) {
    if (f64_eq(x0, x1) && f64_eq(y0, y1)) return;
    const bool flip_xy = f64_abs_lt(x0 - x1, y0 - y1);
    if (flip_xy) {
        double t;
        t = x0; x0 = y0; y0 = t;
        t = x1; x1 = y1; y1 = t;
        t = xm; xm = ym; ym = t;
    }
    double scale = 1.0;
    if (line_width < 1.0) { scale *= line_width; line_width = 1.0; }
    const double aa = 1.0;
    const double halfwidth = 0.5 * (line_width + aa);
    const bool flip_order = f64_lt(y1, y0) || (f64_eq(y1, y0) && f64_lt(x1, x0));
    double alongx = x1 - x0;
    double alongy = y1 - y0;
    const double length = sqrt(sq(alongx) + sq(alongy));
    alongx /= length;
    alongy /= length;
    const double rightx = alongy;
    const double righty = -alongx;
    // the four corners (bx[k], by[k]) as scalars: they are picked by a run-time
    // index per scanline, which an array would leave in local memory.  With
    // rightx = alongy and righty = -alongx the eight products
    // halfwidth * (+-right +- along) are +-ca and +-cb (round to nearest is
    // symmetric, so each is the same value; only the sign of a zero may
    // differ, which the corners' one use, the scan bounds, does not see).
    double bx0, bx1, bx2, bx3, by0, by1, by2, by3;
    const double ca = halfwidth * (rightx - alongx), cb = halfwidth * (rightx + alongx);
    if (flip_order) {
        bx0 = x1 - ca; bx1 = x1 + cb; bx2 = x0 + ca; bx3 = x0 - cb;
        by0 = y1 + cb; by1 = y1 + ca; by2 = y0 - cb; by3 = y0 - ca;
    } else {
        bx0 = x0 + ca; bx1 = x0 - cb; bx2 = x1 - ca; bx3 = x1 + cb;
        by0 = y0 - cb; by1 = y0 - ca; by2 = y1 + cb; by3 = y1 + ca;
    }
    long long xmaxi = nx - 1, ymaxi = ny - 1;
    if (flip_xy) { long long t = xmaxi; xmaxi = ymaxi; ymaxi = t; }
    const int lowindex = flip_order ? (f64_lt(x1, x0) ? 0 : 1) : (f64_lt(x0, x1) ? 0 : 1);
    double prev_alongx = 0, prev_alongy = 0, prev_length = 0, prev_rightx = 0, prev_righty = 0;
    if (!overwrite && !segment_start) {
        prev_alongx = x0 - xm;
        prev_alongy = y0 - ym;
        prev_length = sqrt(sq(prev_alongx) + sq(prev_alongy));
        if (f64_gt0(prev_length)) {
            prev_alongx /= prev_length;
            prev_alongy /= prev_length;
            prev_rightx = prev_alongy;
            prev_righty = -prev_alongx;
        } else {
            overwrite = true;
        }
    }
    // clampi((long long)ceil / floor(.), 0, max) by integer operations (nx, ny < 2^31)
    const long long ystart = f64_ceil_clamp(pick4(lowindex, by0, by1, by2, by3), ymaxi);
    const long long yend = f64_floor_clamp(pick4((lowindex + 2) % 4, by0, by1, by2, by3), ymaxi);
    int ll = lowindex, lu = (ll + 1) % 4, rl = lowindex, ru = (rl + 3) % 4;
    const double lw_lo = 0.5 * (line_width - aa);
    const double ls_den = halfwidth - lw_lo;           // linearstep's edge1 - edge0
    const bool unit_den = ls_den == 1.0;               // x / 1.0 == x: the division is skipped
    // A cap pixel whose squared distance d2 (>= +0 or NaN) is at least
    // halfwidth^2 rounded up has sqrt(d2) >= halfwidth (the square root and
    // its rounding are monotone; halfwidth is a float64), so linearstep is 1
    // and its coverage 0: it appends nothing and the square root is skipped.
    const unsigned long long cap_far = f64_bits(__dmul_ru(halfwidth, halfwidth));
    // The comparisons, the float64 pixel coordinates and the ceil / floor
    // conversions are integer operations on the bit patterns (f64cmp.cuh),
    // each with the IEEE result for the values that reach it: the float64
    // pipe, which bounds this loop, then issues only the products, sums,
    // square roots and divisions (none for the ramp when its denominator is
    // exactly 1.0).  length >= +0 (or NaN), prev_length in (0, inf],
    // halfwidth in [1, inf], and the coverage values lie in [+0, 1].
    for (long long y = ystart; y <= yend; ++y) {
        const double yd = f64_from_u32((unsigned)y);
        if (ll == lowindex && f64_nonneg_gt(yd, pick4(lu, by0, by1, by2, by3))) { ll = lu; lu = (ll + 1) % 4; }
        if (rl == lowindex && f64_nonneg_gt(yd, pick4(ru, by0, by1, by2, by3))) { rl = ru; ru = (rl + 3) % 4; }
        // clampi(ceil / floor(x_intercept(...)), 0, max), line.py:921-926 (aa_scan.cuh)
        const long long xleft = aa_scan_bound<true>((unsigned)y, yd, pick4(ll, bx0, bx1, bx2, bx3),
            pick4(ll, by0, by1, by2, by3), pick4(lu, bx0, bx1, bx2, bx3), pick4(lu, by0, by1, by2, by3), xmaxi);
        const long long xright = aa_scan_bound<false>((unsigned)y, yd, pick4(rl, bx0, bx1, bx2, bx3),
            pick4(rl, by0, by1, by2, by3), pick4(ru, bx0, bx1, bx2, bx3), pick4(ru, by0, by1, by2, by3), xmaxi);
        for (long long x = xleft; x <= xright; ++x) {
            const double xd = f64_from_u32((unsigned)x);         // 0 <= x < 2^31
            const double along = (xd - x0) * alongx + (yd - y0) * alongy;
            bool prev_correction = false;
            double distance;
            if (f64_lt0(along)) {
                if (!(overwrite || segment_start || f64_gt0((xd - x0) * prev_alongx + (yd - y0) * prev_alongy)))
                    continue;
                const double d2 = sq(xd - x0) + sq(yd - y0);
                if (f64_bits(d2) >= cap_far) continue;
                distance = sqrt(d2);
            } else if (f64_gt_nonneg(along, length)) {
                if (!(overwrite || segment_end)) continue;
                const double d2 = sq(xd - x1) + sq(yd - y1);
                if (f64_bits(d2) >= cap_far) continue;
                distance = sqrt(d2);
            } else {
                distance = fabs((xd - x0) * rightx + (yd - y0) * righty);
                if (!overwrite && !segment_start) {
                    const double pd = (xd - x0) * prev_alongx + (yd - y0) * prev_alongy;
                    if (f64_in_neg_range(pd, prev_length) &&
                        f64_abs_le((xd - x0) * prev_rightx + (yd - y0) * prev_righty, halfwidth))
                        prev_correction = true;
                }
            }
            // 1 - linearstep(lw_lo, halfwidth, distance), line.py:808-811
            double value = f64_one_minus_clamp01(unit_den ? distance - lw_lo : (distance - lw_lo) / ls_den);
            value *= scale;
            double prev_value = 0.0;
            if (prev_correction) {
                const double prev_distance = fabs((xd - x0) * prev_rightx + (yd - y0) * prev_righty);
                prev_value = f64_one_minus_clamp01(unit_den ? prev_distance - lw_lo : (prev_distance - lw_lo) / ls_den);
                prev_value *= scale;
                if (f64_le_nonneg(value, prev_value)) value = 0.0;
            }
            if (f64_gt0(value)) {
                if (flip_xy) line_append<KEYED>(p, i, y, x, value, prev_value);
                else line_append<KEYED>(p, i, x, y, value, prev_value);
            }
        }
    }
}

// line.py:986-1031 -- integer Bresenham.
template <bool KEYED>
__device__ void bresenham(const LineParams &p, int64_t i, bool segment_start, long long x0, long long x1,
                          long long y0, long long y1, bool clipped) {
    long long dx = x1 - x0;
    const long long ix = (dx > 0) - (dx < 0);
    dx = (dx < 0 ? -dx : dx) * 2;
    long long dy = y1 - y0;
    const long long iy = (dy > 0) - (dy < 0);
    dy = (dy < 0 ? -dy : dy) * 2;
    if (!clipped && !(dx | dy)) { line_append<KEYED>(p, i, x0, y0, 1.0, 0.0); return; }
    if (segment_start) line_append<KEYED>(p, i, x0, y0, 1.0, 0.0);
    if (dx >= dy) {
        long long error = 2 * dy - dx;
        while (x0 != x1) {
            if (error >= 0 && (error || ix > 0)) { error -= 2 * dx; y0 += iy; }
            error += 2 * dy;
            x0 += ix;
            line_append<KEYED>(p, i, x0, y0, 1.0, 0.0);
        }
    } else {
        long long error = 2 * dx - dy;
        while (y0 != y1) {
            if (error >= 0 && (error || iy > 0)) { error -= 2 * dy; x0 += ix; }
            error += 2 * dx;
            y0 += iy;
            line_append<KEYED>(p, i, x0, y0, 1.0, 0.0);
        }
    }
}

__device__ __forceinline__ long long pyround(double v) { return (long long)rint(v); }

// line.py:688-721 -- map_onto_pixel_snap
__device__ __forceinline__ void map_snap(const LineParams &p, double x, double y, long long &xo, long long &yo) {
    long long xx = (long long)(x * p.sx + p.tx);
    long long yy = (long long)(y * p.sy + p.ty);
    long long xxmax = pyround(p.xmax * p.sx + p.tx);
    long long yymax = pyround(p.ymax * p.sy + p.ty);
    xo = xx == xxmax ? xx - 1 : xx;
    yo = yy == yymax ? yy - 1 : yy;
}

// line.py:1104-1124 + 1045-1095, one segment.
// One segment of a line (rows' vertices (x0, y0) -> (x1, y1), previous
// vertex (xm, ym)): clip, map, antialiased coverage or Bresenham
// (line.py:1033-1097 _build_draw_segment).  `row` is the row whose fields
// the appends use.
template <bool KEYED = false>
__device__ void draw_segment(const LineParams &p, int64_t row, double x0, double y0, double x1, double y1,
                             bool segment_start, bool segment_end, double xm, double ym) {
    const bool antialias = p.line_width > 0.0;
    bool skip = isnull(x0) || isnull(y0) || isnull(x1) || isnull(y1);
    bool cs = false, ce = false;
    liang_barsky(p.xmin, p.xmax, p.ymin, p.ymax, x0, x1, y0, y1, skip, cs, ce);
    if (skip) return;
    const bool clipped = cs || ce;
    segment_start = segment_start || cs;
    if (antialias) {
        // line.py:723-726 map_onto_pixel_no_snap
        const double px0 = x0 * p.sx + p.tx - 0.5, py0 = y0 * p.sy + p.ty - 0.5;
        const double px1 = x1 * p.sx + p.tx - 0.5, py1 = y1 * p.sy + p.ty - 0.5;
        double pxm = 0.0, pym = 0.0;
        if (!segment_start) { pxm = xm * p.sx + p.tx - 0.5; pym = ym * p.sy + p.ty - 0.5; }
        const long long nx = p.aa_nx, ny = p.aa_ny;          // pyround((xmax - xmin) * sx), on the host
        full_antialias<KEYED>(p, p.line_width, p.overwrite != 0, row, px0, px1, py0, py1,
                       segment_start, segment_end, pxm, pym, nx, ny);
    } else {
        long long ix0, iy0, ix1, iy1;
        map_snap(p, x0, y0, ix0, iy0);
        map_snap(p, x1, y1, ix1, iy1);
        bresenham<KEYED>(p, row, segment_start, ix0, ix1, iy0, iy1, clipped);
    }
}

__global__ void __launch_bounds__(256, 1) line_axis0_kernel(const LineParams p) {
    const ColumnRef X = p.cols[p.x_col], Y = p.cols[p.y_col];
    for (int64_t i = gtid(); i + 1 < p.n; i += gstride()) {
        const double x0 = load_f64(X, i), y0 = load_f64(Y, i);
        const double x1 = load_f64(X, i + 1), y1 = load_f64(Y, i + 1);
        // the previous row, with numba's wrap of index -1 onto the last row
        const int64_t im = i > 0 ? i - 1 : p.n - 1;
        const bool segment_start = (i == 0) ? (p.plot_start != 0)
                                            : (isnull(load_f64(X, im)) || isnull(load_f64(Y, im)));
        const bool segment_end = (i == p.n - 2) || isnull(load_f64(X, i + 2)) || isnull(load_f64(Y, i + 2));
        double xm = 0.0, ym = 0.0;
        if (!(segment_start || p.use_2_stage)) { xm = load_f64(X, im); ym = load_f64(Y, im); }
        draw_segment(p, i, x0, y0, x1, y1, segment_start, segment_end, xm, ym);
    }
}

// ---- antialiased LineAxis0 in work order.  One thread per segment leaves
// most lanes idle when the segments of a warp cover different numbers of
// pixels (the float64 pipe issues each instruction for the whole warp).
// Segments are first bucketed by an estimate of their pixel work (the area
// of their padded bounding box in pixels), counting-sorted by bucket, and
// drawn in that order, so the lanes of a warp do similar work.
constexpr int LINE_WORK_BUCKETS = 64;
constexpr int LINE_ORDER_TILE = 4096;

static size_t line_ws_align(size_t v) { return (v + 255) / 256 * 256; }

// The estimate only orders the segments (any deterministic one draws the
// same pixels): float32 after the two float64 differences, off the float64
// pipe that bounds the drawing kernels.
__device__ __forceinline__ int line_work_bucket(const LineWorkArgs &p, int64_t i) {
    const double x0 = load_f64(p.X, i), y0 = load_f64(p.Y, i), x1 = load_f64(p.X, i + 1), y1 = load_f64(p.Y, i + 1);
    if (isnull(x0) || isnull(y0) || isnull(x1) || isnull(y1)) return 0;
    const float pad = (float)p.line_width + 2.0f;
    const float w = (fabsf((float)(x1 - x0) * (float)p.sx) + pad) * (fabsf((float)(y1 - y0) * (float)p.sy) + pad);
    if (!(w < 2.0f * (LINE_WORK_BUCKETS - 1))) return LINE_WORK_BUCKETS - 1;
    return (int)(w * 0.5f);
}

__global__ void __launch_bounds__(256) line_work_hist(const LineWorkArgs p, unsigned *hist) {
    __shared__ unsigned h[LINE_WORK_BUCKETS];
    if (threadIdx.x < LINE_WORK_BUCKETS) h[threadIdx.x] = 0;
    __syncthreads();
    for (int64_t i = gtid(); i + 1 < p.n; i += gstride()) atomicAdd(&h[line_work_bucket(p, i)], 1u);
    __syncthreads();
    if (threadIdx.x < LINE_WORK_BUCKETS && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

__global__ void line_work_scan(const unsigned *hist, unsigned *cursor) {
    if (threadIdx.x != 0) return;
    unsigned o = 0;
    for (int b = 0; b < LINE_WORK_BUCKETS; ++b) { cursor[b] = o; o += hist[b]; }
}

__global__ void __launch_bounds__(256) line_work_order(const LineWorkArgs p, unsigned *cursor, unsigned *order) {
    __shared__ unsigned h[LINE_WORK_BUCKETS];
    __shared__ unsigned char bk[LINE_ORDER_TILE];      // each segment's bucket, computed once
    if (threadIdx.x < LINE_WORK_BUCKETS) h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t s0 = (int64_t)blockIdx.x * LINE_ORDER_TILE;
    const int64_t s1 = s0 + LINE_ORDER_TILE < p.n - 1 ? s0 + LINE_ORDER_TILE : p.n - 1;
    for (int64_t i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
        const int b = line_work_bucket(p, i);
        bk[i - s0] = (unsigned char)b;
        atomicAdd(&h[b], 1u);
    }
    __syncthreads();
    if (threadIdx.x < LINE_WORK_BUCKETS && h[threadIdx.x])
        h[threadIdx.x] = atomicAdd(&cursor[threadIdx.x], h[threadIdx.x]);
    __syncthreads();
    for (int64_t i = s0 + threadIdx.x; i < s1; i += blockDim.x)
        order[atomicAdd(&h[bk[i - s0]], 1u)] = (unsigned)i;
}

size_t line_work_order_bytes(int64_t n) {
    if (n < 2) return 0;
    return line_ws_align((size_t)LINE_WORK_BUCKETS * 8) + line_ws_align((size_t)(n - 1) * 4);
}

const unsigned *build_line_work_order(const LineWorkArgs &a, void *workspace, size_t ws_bytes, cudaStream_t st) {
    if (a.n < 2 || !workspace || ws_bytes < line_work_order_bytes(a.n) || ((uintptr_t)workspace & 255u))
        return nullptr;
    unsigned *hist = (unsigned *)workspace;
    unsigned *cursor = hist + LINE_WORK_BUCKETS;
    unsigned *order = (unsigned *)((char *)workspace + line_ws_align((size_t)LINE_WORK_BUCKETS * 8));
    if (cudaMemsetAsync(hist, 0, (size_t)LINE_WORK_BUCKETS * 4, st) != cudaSuccess) return nullptr;
    line_work_hist<<<grid_of(a.n - 1), 256, 0, st>>>(a, hist);
    line_work_scan<<<1, 32, 0, st>>>(hist, cursor);
    const int64_t tiles = (a.n - 1 + LINE_ORDER_TILE - 1) / LINE_ORDER_TILE;
    line_work_order<<<(unsigned)tiles, 256, 0, st>>>(a, cursor, order);
    return order;
}

__global__ void __launch_bounds__(256, 1) line_axis0_ordered_kernel(const LineParams p, const unsigned *order) {
    const ColumnRef X = p.cols[p.x_col], Y = p.cols[p.y_col];
    for (int64_t k = gtid(); k + 1 < p.n; k += gstride()) {
        const int64_t i = order[k];
        const double x0 = load_f64(X, i), y0 = load_f64(Y, i);
        const double x1 = load_f64(X, i + 1), y1 = load_f64(Y, i + 1);
        const int64_t im = i > 0 ? i - 1 : p.n - 1;
        const bool segment_start = (i == 0) ? (p.plot_start != 0)
                                            : (isnull(load_f64(X, im)) || isnull(load_f64(Y, im)));
        const bool segment_end = (i == p.n - 2) || isnull(load_f64(X, i + 2)) || isnull(load_f64(Y, i + 2));
        double xm = 0.0, ym = 0.0;
        if (!(segment_start || p.use_2_stage)) { xm = load_f64(X, im); ym = load_f64(Y, im); }
        draw_segment(p, i, x0, y0, x1, y1, segment_start, segment_end, xm, ym);
    }
}

// The vertex arrays of the multi-line layouts and of ragged rows (see
// lines_kernel and lines_ragged_kernel below).
struct RaggedGeom {
    const double *xf, *yf;
    const int64_t *xs, *ys;
    int64_t nrows, nx, ny;
};
struct LinesGeom {
    const double *xs, *ys;
    int64_t nrows, nv;      // LAYOUT 1: nv = lines; LAYOUT 2: nv = vertices per line
    int64_t xrow, yrow;     // LAYOUT 2: row strides of xs and ys (0 = shared by all rows)
    int64_t only_line;      // >= 0: draw this line alone (two-stage plans); -1: every line
};

// ---- antialiased LineAxis0, pixels queued by case.  In the kernels above a
// warp's 32 segments scan their pixels together, and each pixel takes one of
// three float64 paths (before the segment, after it, beside it) or none, so
// the float64 pipe issues every path for the whole warp with half the lanes
// idle.  Here each lane scans its segment's pixels and classifies them in
// float32 with an error bound; the pixels go to per-warp queues in shared
// memory by case (cap, side, or exact when the bound does not decide), and
// the warp works off each queue 32 pixels at a time, every lane on the same
// float64 path.  Same arithmetic as full_antialias on the same values.
constexpr int AAQ_CAP = 64;                // per queue and warp: < 32 queued + 32 added in one round

struct AASeg {                             // a segment in the flipped frame (line.py:840-906)
    double x0, y0, x1, y1;
    double ax, ay, len;                    // alongx, alongy, length
    double pax, pay, plen;                 // prev_alongx, prev_alongy, prev_length
    long long row;
    unsigned flags;                        // AAF_*
};
constexpr unsigned AAF_OVERWRITE = 1u, AAF_START = 2u, AAF_END = 4u, AAF_FLIP = 8u, AAF_PREV = 16u;

struct AAConsts {                          // uniform per launch
    double halfwidth, lw_lo, ls_den, scale;
    bool unit_den;
    unsigned long long cap_far;
};

__device__ __forceinline__ AAConsts aa_consts(double line_width) {
    AAConsts c;
    c.scale = 1.0;
    if (line_width < 1.0) { c.scale *= line_width; line_width = 1.0; }
    c.halfwidth = 0.5 * (line_width + 1.0);
    c.lw_lo = 0.5 * (line_width - 1.0);
    c.ls_den = c.halfwidth - c.lw_lo;
    c.unit_den = c.ls_den == 1.0;
    c.cap_far = f64_bits(__dmul_ru(c.halfwidth, c.halfwidth));
    return c;
}

// 1 - linearstep(lw_lo, halfwidth, d), times scale
__device__ __forceinline__ double aa_ramp(const AAConsts &c, double d) {
    return f64_one_minus_clamp01(c.unit_den ? d - c.lw_lo : (d - c.lw_lo) / c.ls_den) * c.scale;
}

// The pixel of full_antialias's inner loop, all cases (the exact queue):
// value and prev_value (value 0: nothing appended).
static __device__ __noinline__ double2 aa_pixel_exact(const AAConsts c, const AASeg &S, long long x, long long y) {
    const double xd = f64_from_u32((unsigned)x), yd = f64_from_u32((unsigned)y);
    const bool overwrite = S.flags & AAF_OVERWRITE, start = S.flags & AAF_START, end = S.flags & AAF_END;
    const double along = (xd - S.x0) * S.ax + (yd - S.y0) * S.ay;
    bool prev_correction = false;
    double distance;
    if (f64_lt0(along)) {
        if (!(overwrite || start || f64_gt0((xd - S.x0) * S.pax + (yd - S.y0) * S.pay))) return make_double2(0.0, 0.0);
        const double d2 = sq(xd - S.x0) + sq(yd - S.y0);
        if (f64_bits(d2) >= c.cap_far) return make_double2(0.0, 0.0);
        distance = sqrt(d2);
    } else if (f64_gt_nonneg(along, S.len)) {
        if (!(overwrite || end)) return make_double2(0.0, 0.0);
        const double d2 = sq(xd - S.x1) + sq(yd - S.y1);
        if (f64_bits(d2) >= c.cap_far) return make_double2(0.0, 0.0);
        distance = sqrt(d2);
    } else {
        distance = fabs((xd - S.x0) * S.ay + (yd - S.y0) * -S.ax);
        if (S.flags & AAF_PREV) {
            const double pd = (xd - S.x0) * S.pax + (yd - S.y0) * S.pay;
            if (f64_in_neg_range(pd, S.plen) && f64_abs_le((xd - S.x0) * S.pay + (yd - S.y0) * -S.pax, c.halfwidth))
                prev_correction = true;
        }
    }
    double value = aa_ramp(c, distance);
    double prev_value = 0.0;
    if (prev_correction) {
        prev_value = aa_ramp(c, fabs((xd - S.x0) * S.pay + (yd - S.y0) * -S.pax));
        if (f64_le_nonneg(value, prev_value)) value = 0.0;
    }
    return make_double2(value, prev_value);
}

// A cap pixel (classified before or after the segment, with the cap drawn).
__device__ __forceinline__ double2 aa_pixel_cap(const AAConsts &c, const AASeg &S, long long x, long long y,
                                                bool before) {
    const double xd = f64_from_u32((unsigned)x), yd = f64_from_u32((unsigned)y);
    const double d2 = before ? sq(xd - S.x0) + sq(yd - S.y0) : sq(xd - S.x1) + sq(yd - S.y1);
    if (f64_bits(d2) >= c.cap_far) return make_double2(0.0, 0.0);
    return make_double2(aa_ramp(c, sqrt(d2)), 0.0);
}

// A pixel beside the segment (0 <= along <= length).
__device__ __forceinline__ double2 aa_pixel_side(const AAConsts &c, const AASeg &S, long long x, long long y) {
    const double xd = f64_from_u32((unsigned)x), yd = f64_from_u32((unsigned)y);
    double value = aa_ramp(c, fabs((xd - S.x0) * S.ay + (yd - S.y0) * -S.ax));
    double prev_value = 0.0;
    if (S.flags & AAF_PREV) {
        const double pd = (xd - S.x0) * S.pax + (yd - S.y0) * S.pay;
        const double q = (xd - S.x0) * S.pay + (yd - S.y0) * -S.pax;
        if (f64_in_neg_range(pd, S.plen) && f64_abs_le(q, c.halfwidth)) {
            prev_value = aa_ramp(c, fabs(q));
            if (f64_le_nonneg(value, prev_value)) value = 0.0;
        }
    }
    return make_double2(value, prev_value);
}

// One queue item of kind `which` (0 cap, 1 side, 2 exact), appended when its
// value is positive: the queue drains share this one append site.
template <bool KEYED>
__device__ __forceinline__ void aa_item_work(const LineParams &p, const AAConsts &c, const AASeg *segs, int which,
                                             unsigned long long it) {
    const AASeg &S = segs[(it >> 48) & 31u];
    const long long x = (long long)(it & 0xFFFFFFu), y = (long long)((it >> 24) & 0xFFFFFFu);
    double2 v;
    if (which == 0) v = aa_pixel_cap(c, S, x, y, (it >> 53) & 1u);
    else if (which == 1) v = aa_pixel_side(c, S, x, y);
    else v = aa_pixel_exact(c, S, x, y);
    if (f64_gt0(v.x)) {
        const bool flip = S.flags & AAF_FLIP;
        line_append<KEYED>(p, S.row, flip ? y : x, flip ? x : y, v.x, v.y);
    }
}

// Queue items: x (24 bits), y (24 bits), the warp lane of the segment (5
// bits), before / after for caps (1 bit).
__device__ __forceinline__ unsigned long long aa_item(long long x, long long y, int lane, bool before) {
    return (unsigned long long)x | ((unsigned long long)y << 24) | ((unsigned long long)lane << 48) |
           ((unsigned long long)before << 53);
}

enum { AAK_NONE = 0, AAK_CAP = 1, AAK_SIDE = 2, AAK_EXACT = 3 };

// SRC 0: LineAxis0 rows (line_axis0_kernel's segments, in `order` or row
// order); SRC 1 / 2: the multi-line layouts of lines_kernel (every line),
// KEYED appends carrying LineAxis0Multi's visit keys; SRC 3: ragged rows
// (lines_ragged_kernel's segments, one a flat x vertex, `rg`).
template <int SRC, bool KEYED>
__global__ void __launch_bounds__(256, 3) aa_queued_kernel(const LineParams p, const unsigned *order, const LinesGeom g,
                                                           const RaggedGeom rg, const int64_t nseg) {
    __shared__ AASeg seg_s[8][32];
    __shared__ unsigned long long q_s[8][3][AAQ_CAP];
    const ColumnRef X = p.cols[p.x_col], Y = p.cols[p.y_col];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    AASeg *segs = seg_s[warp];
    unsigned long long *qcap = q_s[warp][0], *qside = q_s[warp][1], *qexact = q_s[warp][2];
    const AAConsts c = aa_consts(p.line_width);
    const int64_t nbatches = (nseg + 31) / 32;
    const int64_t warps_total = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t b = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp; b < nbatches; b += warps_total) {
        const int64_t k = b * 32 + lane;
        // ---- set-up: draw_segment (line.py:1033-1097) and full_antialias up to the scan
        bool active = false;
        AASeg S;
        long long cy = 0, cyend = -1, cx = 1, cxr = 0, xmaxi = 0;
        int ll = 0, lu = 1, rl = 0, ru = 3, lowindex = 0;
        double bx0 = 0, bx1 = 0, bx2 = 0, bx3 = 0, by0 = 0, by1 = 0, by2 = 0, by3 = 0;
        AAClassF kf = AAClassF{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (k < nseg) {
            // the segment, its neighbours' NaN tests and its previous vertex,
            // as line_axis0_kernel / lines_kernel read them
            int64_t i = 0;                                   // the append key (row, or visit key)
            double x0 = 0.0, y0 = 0.0, x1 = 0.0, y1 = 0.0, xm = 0.0, ym = 0.0;
            bool segment_start = false, segment_end = false, have_seg = true;
            if (SRC == 0) {
                i = order ? (int64_t)order[k] : k;           // no order: row order
                x0 = load_f64(X, i); y0 = load_f64(Y, i);
                x1 = load_f64(X, i + 1); y1 = load_f64(Y, i + 1);
                const int64_t im = i > 0 ? i - 1 : p.n - 1;
                segment_start = (i == 0) ? (p.plot_start != 0) : (isnull(load_f64(X, im)) || isnull(load_f64(Y, im)));
                segment_end = (i == p.n - 2) || isnull(load_f64(X, i + 2)) || isnull(load_f64(Y, i + 2));
                if (!(segment_start || p.use_2_stage)) { xm = load_f64(X, im); ym = load_f64(Y, im); }
            } else if (SRC == 1) {                           // line j down the rows (line.py:1152-1242)
                const bool one = g.only_line >= 0;           // one line alone (two-stage plans)
                const int64_t r = one ? k : k / g.nv, j = one ? g.only_line : k - r * g.nv;
                const double *Xp = g.xs + j, *Yp = g.ys + j;
                const int64_t st = g.nv;
                x0 = Xp[r * st]; y0 = Yp[r * st]; x1 = Xp[(r + 1) * st]; y1 = Yp[(r + 1) * st];
                const int64_t rm = r > 0 ? r - 1 : g.nrows - 1;
                segment_start = (r == 0) ? (p.plot_start != 0) : (isnull(Xp[rm * st]) || isnull(Yp[rm * st]));
                segment_end = (r == g.nrows - 2) || isnull(Xp[(r + 2) * st]) || isnull(Yp[(r + 2) * st]);
                if (!(segment_start || p.use_2_stage)) { xm = Xp[rm * st]; ym = Yp[rm * st]; }
                i = KEYED ? j * p.field_mod + r : r;        // line j's appends after lines 0 .. j-1
            } else if (SRC == 3) {                           // ragged row (line.py:1538-1612)
                int64_t lo = 0, hi = rg.nrows - 1;
                while (lo < hi) {
                    const int64_t mid = (lo + hi + 1) >> 1;
                    if (rg.xs[mid] <= k) lo = mid; else hi = mid - 1;
                }
                const bool last = lo == rg.nrows - 1;
                const int64_t xa = min(max(rg.xs[lo], (int64_t)0), rg.nx);
                const int64_t xb = max(min(last ? rg.nx : rg.xs[lo + 1], rg.nx), xa);
                const int64_t ya = min(max(rg.ys[lo], (int64_t)0), rg.ny);
                const int64_t yb = max(min(last ? rg.ny : rg.ys[lo + 1], rg.ny), ya);
                const int64_t len = min(xb - xa, yb - ya);
                const int64_t j = k - xa;
                have_seg = j >= 0 && j + 1 < len;
                if (have_seg) {
                    const double *Xp = rg.xf + xa, *Yp = rg.yf + ya;
                    x0 = Xp[j]; y0 = Yp[j]; x1 = Xp[j + 1]; y1 = Yp[j + 1];
                    segment_start = (j == 0) || isnull(Xp[j - 1]) || isnull(Yp[j - 1]);
                    segment_end = (j == len - 2) || isnull(Xp[j + 2]) || isnull(Yp[j + 2]);
                    if (!(segment_start || p.use_2_stage)) { xm = Xp[j - 1]; ym = Yp[j - 1]; }
                }
                i = lo;
            } else {                                         // row r along its vertices (line.py:1244-1437)
                const bool one = g.only_line >= 0;
                const int64_t r = one ? g.only_line : k / (g.nv - 1), j = one ? k : k - r * (g.nv - 1);
                const double *Xp = g.xs + r * g.xrow, *Yp = g.ys + r * g.yrow;
                x0 = Xp[j]; x1 = Xp[j + 1]; y0 = Yp[j]; y1 = Yp[j + 1];
                segment_start = (j == 0) || isnull(Xp[j - 1]) || isnull(Yp[j - 1]);
                segment_end = (j == g.nv - 2) || isnull(Xp[j + 2]) || isnull(Yp[j + 2]);
                if (!(segment_start || p.use_2_stage)) { xm = Xp[j - 1]; ym = Yp[j - 1]; }
                i = r;
            }
            bool skip = !have_seg || isnull(x0) || isnull(y0) || isnull(x1) || isnull(y1);
            bool cs = false, ce = false;
            liang_barsky(p.xmin, p.xmax, p.ymin, p.ymax, x0, x1, y0, y1, skip, cs, ce);
            segment_start = segment_start || cs;
            double px0 = x0 * p.sx + p.tx - 0.5, py0 = y0 * p.sy + p.ty - 0.5;
            double px1 = x1 * p.sx + p.tx - 0.5, py1 = y1 * p.sy + p.ty - 0.5;
            double pxm = 0.0, pym = 0.0;
            if (!segment_start) { pxm = xm * p.sx + p.tx - 0.5; pym = ym * p.sy + p.ty - 0.5; }
            if (!skip && !(f64_eq(px0, px1) && f64_eq(py0, py1))) {
                bool overwrite = p.overwrite != 0;
                const bool flip_xy = f64_abs_lt(px0 - px1, py0 - py1);
                if (flip_xy) {
                    double t;
                    t = px0; px0 = py0; py0 = t;
                    t = px1; px1 = py1; py1 = t;
                    t = pxm; pxm = pym; pym = t;
                }
                const bool flip_order = f64_lt(py1, py0) || (f64_eq(py1, py0) && f64_lt(px1, px0));
                double alongx = px1 - px0, alongy = py1 - py0;
                const double length = sqrt(sq(alongx) + sq(alongy));
                alongx /= length;
                alongy /= length;
                const double ca = c.halfwidth * (alongy - alongx), cb = c.halfwidth * (alongy + alongx);
                if (flip_order) {
                    bx0 = px1 - ca; bx1 = px1 + cb; bx2 = px0 + ca; bx3 = px0 - cb;
                    by0 = py1 + cb; by1 = py1 + ca; by2 = py0 - cb; by3 = py0 - ca;
                } else {
                    bx0 = px0 + ca; bx1 = px0 - cb; bx2 = px1 - ca; bx3 = px1 + cb;
                    by0 = py0 - cb; by1 = py0 - ca; by2 = py1 + cb; by3 = py1 + ca;
                }
                xmaxi = p.aa_nx - 1;
                long long ymaxi = p.aa_ny - 1;
                if (flip_xy) { const long long t = xmaxi; xmaxi = ymaxi; ymaxi = t; }
                lowindex = flip_order ? (f64_lt(px1, px0) ? 0 : 1) : (f64_lt(px0, px1) ? 0 : 1);
                double pax = 0.0, pay = 0.0, plen = 0.0;
                if (!overwrite && !segment_start) {
                    pax = px0 - pxm;
                    pay = py0 - pym;
                    plen = sqrt(sq(pax) + sq(pay));
                    if (f64_gt0(plen)) {
                        pax /= plen;
                        pay /= plen;
                    } else {
                        overwrite = true;
                    }
                }
                S.x0 = px0; S.y0 = py0; S.x1 = px1; S.y1 = py1;
                S.ax = alongx; S.ay = alongy; S.len = length;
                S.pax = pax; S.pay = pay; S.plen = plen;
                S.row = i;
                S.flags = (overwrite ? AAF_OVERWRITE : 0u) | (segment_start ? AAF_START : 0u) |
                          (segment_end ? AAF_END : 0u) | (flip_xy ? AAF_FLIP : 0u) |
                          (!overwrite && !segment_start ? AAF_PREV : 0u);
                cy = f64_ceil_clamp(pick4(lowindex, by0, by1, by2, by3), ymaxi) - 1;
                cyend = f64_floor_clamp(pick4((lowindex + 2) % 4, by0, by1, by2, by3), ymaxi);
                ll = lowindex; lu = (ll + 1) % 4; rl = lowindex; ru = (rl + 3) % 4;
                kf = AAClassF{(float)px0, (float)py0, (float)alongx, (float)alongy, (float)length, (float)pax, (float)pay};
                active = true;
                segs[lane] = S;
            }
        }
        __syncwarp();
        const bool cap_before = active && (S.flags & (AAF_OVERWRITE | AAF_START));
        const bool cap_after = active && (S.flags & (AAF_OVERWRITE | AAF_END));
        int ncap = 0, nside = 0, nexact = 0;          // warp-uniform queue lengths
        while (__any_sync(0xffffffffu, active)) {
            // ---- one pixel per lane: the next of its scan (line.py:908-981 loop order)
            int kind = AAK_NONE;
            long long px = 0, py = 0;
            bool before = false;
            while (active) {
                if (cx <= cxr) { px = cx; py = cy; ++cx; kind = AAK_EXACT; break; }
                if (++cy > cyend) { active = false; break; }
                const double yd = f64_from_u32((unsigned)cy);
                if (ll == lowindex && f64_nonneg_gt(yd, pick4(lu, by0, by1, by2, by3))) { ll = lu; lu = (ll + 1) % 4; }
                if (rl == lowindex && f64_nonneg_gt(yd, pick4(ru, by0, by1, by2, by3))) { rl = ru; ru = (rl + 3) % 4; }
                cx = aa_scan_bound<true, true>((unsigned)cy, yd, pick4(ll, bx0, bx1, bx2, bx3), pick4(ll, by0, by1, by2, by3),
                                         pick4(lu, bx0, bx1, bx2, bx3), pick4(lu, by0, by1, by2, by3), xmaxi);
                cxr = aa_scan_bound<false, true>((unsigned)cy, yd, pick4(rl, bx0, bx1, bx2, bx3), pick4(rl, by0, by1, by2, by3),
                                           pick4(ru, bx0, bx1, bx2, bx3), pick4(ru, by0, by1, by2, by3), xmaxi);
            }
            if (kind != AAK_NONE) {
                switch (aa_classify((unsigned)px, (unsigned)py, kf, cap_before, cap_after)) {
                case AAC_NONE: kind = AAK_NONE; break;
                case AAC_CAP_BEFORE: kind = AAK_CAP; before = true; break;
                case AAC_CAP_AFTER: kind = AAK_CAP; break;
                case AAC_SIDE: kind = AAK_SIDE; break;
                default: kind = AAK_EXACT; break;
                }
            }
            // ---- append to the queues (lane order within a round)
            const unsigned long long item = aa_item(px, py, lane, before);
            unsigned m = __ballot_sync(0xffffffffu, kind == AAK_CAP);
            if (kind == AAK_CAP) qcap[ncap + __popc(m & lt_mask)] = item;
            ncap += __popc(m);
            m = __ballot_sync(0xffffffffu, kind == AAK_SIDE);
            if (kind == AAK_SIDE) qside[nside + __popc(m & lt_mask)] = item;
            nside += __popc(m);
            m = __ballot_sync(0xffffffffu, kind == AAK_EXACT);
            if (kind == AAK_EXACT) qexact[nexact + __popc(m & lt_mask)] = item;
            nexact += __popc(m);
            __syncwarp();
            // ---- work off full rounds of 32, every lane on the same path (one
            // round a pass; after the last pixels, the partial rounds too)
            const bool last = !__any_sync(0xffffffffu, active);
            while (true) {
                int which, cnt;
                if (ncap >= 32 || (last && ncap > 0)) { which = 0; cnt = ncap; }
                else if (nside >= 32 || (last && nside > 0)) { which = 1; cnt = nside; }
                else if (nexact >= 32 || (last && nexact > 0)) { which = 2; cnt = nexact; }
                else break;
                const int take = cnt < 32 ? cnt : 32;
                const int from = cnt - take;
                if (which == 0) ncap = from; else if (which == 1) nside = from; else nexact = from;
                if (lane < take) aa_item_work<KEYED>(p, c, segs, which, q_s[warp][which][from + lane]);
            }
            __syncwarp();
        }
    }
}

// Multi-line layouts over float64 vertex arrays.
//   LAYOUT 1, LineAxis0Multi (line.py:1152-1242): xs, ys [nrows][nlines];
//       line j runs down the rows; segment (i, j) appends row i; the
//       segment start and the previous vertex follow LineAxis0.
//   LAYOUT 2, the LinesAxis1 family (line.py:1244-1437): line i runs along
//       the nv columns of row i, vertex (i, j) = (xs[i * xrow + j],
//       ys[i * yrow + j]); xrow = 0 is LinesAxis1XConstant (one x array for
//       every line), yrow = 0 LinesAxis1YConstant, both nv LinesAxis1;
//       segment (i, j) appends row i; a segment starts at j == 0 or after a
//       NaN.
// Consecutive threads take consecutive array elements (coalesced loads).

template <int LAYOUT>
__global__ void __launch_bounds__(256, 1) lines_kernel(const LineParams p, const LinesGeom g) {
    const bool one = g.only_line >= 0;
    const int64_t nseg = one ? (LAYOUT == 1 ? g.nrows - 1 : g.nv - 1)
                             : (LAYOUT == 1 ? (g.nrows - 1) * g.nv : g.nrows * (g.nv - 1));
    for (int64_t s = gtid(); s < nseg; s += gstride()) {
        if (LAYOUT == 1) {
            const int64_t i = one ? s : s / g.nv, j = one ? g.only_line : s - i * g.nv;
            const double *X = g.xs + j, *Y = g.ys + j;
            const int64_t st = g.nv;
            const double x0 = X[i * st], y0 = Y[i * st], x1 = X[(i + 1) * st], y1 = Y[(i + 1) * st];
            const int64_t im = i > 0 ? i - 1 : g.nrows - 1;
            const bool segment_start = (i == 0) ? (p.plot_start != 0) : (isnull(X[im * st]) || isnull(Y[im * st]));
            const bool segment_end = (i == g.nrows - 2) || isnull(X[(i + 2) * st]) || isnull(Y[(i + 2) * st]);
            double xm = 0.0, ym = 0.0;
            if (!(segment_start || p.use_2_stage)) { xm = X[im * st]; ym = Y[im * st]; }
            // line j's appends come after every append of lines 0 .. j-1 (line.py:1190-1194)
            if (p.field_mod > 0)
                draw_segment<true>(p, j * p.field_mod + i, x0, y0, x1, y1, segment_start, segment_end, xm, ym);
            else
                draw_segment(p, i, x0, y0, x1, y1, segment_start, segment_end, xm, ym);
        } else {
            const int64_t i = one ? g.only_line : s / (g.nv - 1), j = one ? s : s - i * (g.nv - 1);
            const double *X = g.xs + i * g.xrow, *Y = g.ys + i * g.yrow;
            const double x0 = X[j], x1 = X[j + 1], y0 = Y[j], y1 = Y[j + 1];
            const bool segment_start = (j == 0) || isnull(X[j - 1]) || isnull(Y[j - 1]);
            const bool segment_end = (j == g.nv - 2) || isnull(X[j + 2]) || isnull(Y[j + 2]);
            double xm = 0.0, ym = 0.0;
            if (!(segment_start || p.use_2_stage)) { xm = X[j - 1]; ym = Y[j - 1]; }
            draw_segment(p, i, x0, y0, x1, y1, segment_start, segment_end, xm, ym);
        }
    }
}

// LinesAxis1Ragged (line.py:457-523, 1538-1612): row i runs over its own
// slices of the flat x and y arrays, [xs[i], xs[i+1]) and [ys[i], ys[i+1])
// (the last row to the flat lengths), through the shorter of the two.  One
// thread per flat x vertex finds its row by bisection over the starts (non-
// decreasing); the slices are clamped to the arrays, so malformed starts
// cannot read outside them.

__global__ void __launch_bounds__(256, 1) lines_ragged_kernel(const LineParams p, const RaggedGeom g) {
    for (int64_t k = gtid(); k < g.nx; k += gstride()) {
        int64_t lo = 0, hi = g.nrows - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (g.xs[mid] <= k) lo = mid; else hi = mid - 1;
        }
        const int64_t i = lo;
        const bool last = i == g.nrows - 1;
        const int64_t xa = min(max(g.xs[i], (int64_t)0), g.nx);
        const int64_t xb = max(min(last ? g.nx : g.xs[i + 1], g.nx), xa);
        const int64_t ya = min(max(g.ys[i], (int64_t)0), g.ny);
        const int64_t yb = max(min(last ? g.ny : g.ys[i + 1], g.ny), ya);
        const int64_t len = min(xb - xa, yb - ya);
        const int64_t j = k - xa;
        if (j < 0 || j + 1 >= len) continue;
        const double *X = g.xf + xa, *Y = g.yf + ya;
        const bool segment_start = (j == 0) || isnull(X[j - 1]) || isnull(Y[j - 1]);
        const bool segment_end = (j == len - 2) || isnull(X[j + 2]) || isnull(Y[j + 2]);
        double xm = 0.0, ym = 0.0;
        if (!(segment_start || p.use_2_stage)) { xm = X[j - 1]; ym = Y[j - 1]; }
        draw_segment(p, i, X[j], Y[j], X[j + 1], Y[j + 1], segment_start, segment_end, xm, ym);
    }
}

// One ragged row alone (two-stage plans, line.py:1616-1693): the row's slice
// bounds are read on the device, its segments split over a small grid; the
// previous vertex is never read.
__global__ void __launch_bounds__(256, 1) lines_ragged_row_kernel(const LineParams p, const RaggedGeom g, int64_t i) {
    const bool last = i == g.nrows - 1;
    const int64_t xa = min(max(g.xs[i], (int64_t)0), g.nx);
    const int64_t xb = max(min(last ? g.nx : g.xs[i + 1], g.nx), xa);
    const int64_t ya = min(max(g.ys[i], (int64_t)0), g.ny);
    const int64_t yb = max(min(last ? g.ny : g.ys[i + 1], g.ny), ya);
    const int64_t len = min(xb - xa, yb - ya);
    const double *X = g.xf + xa, *Y = g.yf + ya;
    for (int64_t j = gtid(); j + 1 < len; j += gstride()) {
        const bool segment_start = (j == 0) || isnull(X[j - 1]) || isnull(Y[j - 1]);
        const bool segment_end = (j == len - 2) || isnull(X[j + 2]) || isnull(Y[j + 2]);
        draw_segment(p, i, X[j], Y[j], X[j + 1], Y[j + 1], segment_start, segment_end, 0.0, 0.0);
    }
}

// Visit keys (j * nrows + r, plus the row offset) held by the row-index
// bases back to rows (r plus the row offset); empty cells keep their marker.
__global__ void unkey_rows_kernel(int op, void *agg, int64_t n, int64_t nrows, int64_t row_offset) {
    for (int64_t c = gtid(); c < n; c += gstride()) {
        long long *v = (long long *)agg;
        long long *r = (op == DSGB_BASE_MIN_ROW || op == DSGB_BASE_MAX_ROW) ? v + c : v + 2 * c + 1;
        const long long k = *r;
        if (k == ROW_EMPTY_MIN || k < row_offset) continue;             // empty (max-row empty is -1)
        *r = row_offset + (k - row_offset) % nrows;
    }
}

int bases_init(const dsgb_base *bases, int32_t nbases, int64_t ncells, cudaStream_t st);
int finalize_outputs(const dsgb_column *cols, int32_t ncols, int64_t row_offset,
                     const dsgb_base *bases, int32_t nbases, const dsgb_output *outs, int32_t nouts,
                     int64_t ncells, cudaStream_t st);

int build_line_params(LineParams &p, const dsgb_column *cols, int32_t ncols, int64_t n,
                      int64_t row_offset, int32_t x_col, int32_t y_col, const dsgb_canvas *cv,
                      const dsgb_base *bases, int32_t nbases) {
    if (!cols || !cv || ncols <= 0 || ncols > MAX_COLS || n < 0 || nbases < 0 || nbases > MAX_BASES ||
        (nbases > 0 && !bases) || x_col < 0 || x_col >= ncols || y_col < 0 || y_col >= ncols ||
        cv->width <= 0 || cv->height <= 0) {
        set_error("dsgb_line_axis0: invalid arguments");
        return DSGB_E_INVALID;
    }
    if (cv->x_log || cv->y_log) {
        set_error("dsgb_line_axis0: log axes are not supported for lines");
        return DSGB_E_UNSUPPORTED;
    }
    memset(&p, 0, sizeof(p));
    for (int c = 0; c < ncols; ++c) {
        if (dtype_size(cols[c].dtype) == 0 || (n > 0 && !cols[c].data)) {
            set_error("dsgb_line_axis0: column %d invalid", c);
            return DSGB_E_INVALID;
        }
        p.cols[c].data = cols[c].data;
        p.cols[c].dtype = cols[c].dtype;
    }
    for (int b = 0; b < nbases; ++b) {
        const dsgb_base &B = bases[b];
        if (!B.agg || B.col >= ncols || B.cat_col >= ncols || B.ncat < 1 || B.op < DSGB_BASE_COUNT ||
            B.op > DSGB_BASE_AA_ARGMAX) {
            set_error("dsgb_line_axis0: base %d invalid", b);
            return DSGB_E_INVALID;
        }
        p.bases[b] = BaseDev{B.op, B.col, B.cat_col < 0 ? -1 : B.cat_col, B.ncat, B.flags, B.agg};
    }
    p.ncols = ncols; p.nbases = nbases; p.n = n; p.row_offset = row_offset;
    p.x_col = x_col; p.y_col = y_col; p.width = cv->width; p.height = cv->height;
    p.sx = cv->sx; p.tx = cv->tx; p.sy = cv->sy; p.ty = cv->ty;
    p.xmin = cv->xmin; p.xmax = cv->xmax; p.ymin = cv->ymin; p.ymax = cv->ymax;
    // The antialiased scan's pixel counts (line.py:1070-1071, Python round:
    // half to even, as rint), once here instead of per segment.  The
    // kernels' integer ceil / floor take pixel indexes below 2^31.
    const double span_x = (p.xmax - p.xmin) * p.sx, span_y = (p.ymax - p.ymin) * p.sy;
    if (!(std::fabs(span_x) < 2147483648.0) || !(std::fabs(span_y) < 2147483648.0)) {
        set_error("dsgb_line_axis0: the canvas spans (xmax - xmin) * sx and (ymax - ymin) * sy must be below 2^31 pixels");
        return DSGB_E_INVALID;
    }
    p.aa_nx = (int64_t)std::rint(span_x);
    p.aa_ny = (int64_t)std::rint(span_y);
    return DSGB_OK;
}

}  // namespace dsgb

namespace dsgb {
DSGB_STATUS_READER(status_line)
}

using namespace dsgb;

extern "C" size_t dsgb_line_workspace_size(int64_t n) { return line_work_order_bytes(n); }

static int line_axis0_impl(const dsgb_column *cols, int32_t ncols, int64_t n, int64_t row_offset,
                           int32_t x_col, int32_t y_col, const dsgb_canvas *canvas,
                           double line_width, int32_t plot_start, int32_t overwrite,
                           int32_t use_2_stage_agg,
                           const dsgb_base *bases, int32_t nbases,
                           const dsgb_output *outs, int32_t nouts,
                           void *workspace, size_t ws_bytes, uint32_t flags, void *stream);

extern "C" int dsgb_line_axis0_ws(const dsgb_column *cols, int32_t ncols, int64_t n, int64_t row_offset,
                                  int32_t x_col, int32_t y_col, const dsgb_canvas *canvas,
                                  double line_width, int32_t plot_start, int32_t overwrite,
                                  int32_t use_2_stage_agg,
                                  const dsgb_base *bases, int32_t nbases,
                                  const dsgb_output *outs, int32_t nouts,
                                  void *workspace, size_t workspace_bytes, uint32_t flags, void *stream) {
    return line_axis0_impl(cols, ncols, n, row_offset, x_col, y_col, canvas, line_width, plot_start, overwrite,
                           use_2_stage_agg, bases, nbases, outs, nouts, workspace, workspace_bytes, flags, stream);
}

extern "C" int dsgb_line_axis0(const dsgb_column *cols, int32_t ncols, int64_t n, int64_t row_offset,
                               int32_t x_col, int32_t y_col, const dsgb_canvas *canvas,
                               double line_width, int32_t plot_start, int32_t overwrite,
                               int32_t use_2_stage_agg,
                               const dsgb_base *bases, int32_t nbases,
                               const dsgb_output *outs, int32_t nouts,
                               uint32_t flags, void *stream) {
    return line_axis0_impl(cols, ncols, n, row_offset, x_col, y_col, canvas, line_width, plot_start, overwrite,
                           use_2_stage_agg, bases, nbases, outs, nouts, nullptr, 0, flags, stream);
}

static int line_axis0_impl(const dsgb_column *cols, int32_t ncols, int64_t n, int64_t row_offset,
                           int32_t x_col, int32_t y_col, const dsgb_canvas *canvas,
                           double line_width, int32_t plot_start, int32_t overwrite,
                           int32_t use_2_stage_agg,
                           const dsgb_base *bases, int32_t nbases,
                           const dsgb_output *outs, int32_t nouts,
                           void *workspace, size_t ws_bytes, uint32_t flags, void *stream) {
    NvtxRange range("dsgb_line_axis0");
    LineParams p;
    int rc = build_line_params(p, cols, ncols, n, row_offset, x_col, y_col, canvas, bases, nbases);
    if (rc) return rc;
    p.debug = (flags & DSGB_FLAG_DEBUG_CHECKS) != 0;
    if (!(line_width >= 0.0)) { set_error("dsgb_line_axis0: line_width must be >= 0"); return DSGB_E_INVALID; }
    p.line_width = line_width;
    p.plot_start = plot_start;
    p.overwrite = overwrite;
    p.use_2_stage = use_2_stage_agg;
    cudaStream_t st = as_stream(stream);
    const int64_t ncells = (int64_t)canvas->width * canvas->height;
    if (!(flags & DSGB_FLAG_NO_INIT)) {
        rc = bases_init(bases, nbases, ncells, st);
        if (rc) return rc;
    }
    if (n > 1 && nbases > 0) {
        int sms = sm_count();
        if (sms <= 0) sms = 148;
        int64_t blocks = (n + 255) / 256;
        if (blocks > (int64_t)sms * 16) blocks = (int64_t)sms * 16;
        const unsigned *order = nullptr;
        if (line_width > 0.0) {
            LineWorkArgs a;
            a.X = p.cols[p.x_col]; a.Y = p.cols[p.y_col]; a.n = n;
            a.sx = p.sx; a.sy = p.sy; a.line_width = line_width;
            order = build_line_work_order(a, workspace, ws_bytes, st);
        }
        // antialiased: pixels queued by case, segments in work order when the
        // workspace holds it (else in row order); canvases past 2^24 pixels a
        // side, or DSGB_FLAG_EXACT_BIN, scan per segment
        if (line_width > 0.0 && p.aa_nx <= (1 << 24) && p.aa_ny <= (1 << 24) && !(flags & DSGB_FLAG_EXACT_BIN)) {
            // three blocks an SM (80 registers)
            aa_queued_kernel<0, false><<<(unsigned)((int64_t)sms * 3), 256, 0, st>>>(p, order, LinesGeom{}, RaggedGeom{},
                                                                                     n - 1);
        } else if (order) {
            line_axis0_ordered_kernel<<<(unsigned)blocks, 256, 0, st>>>(p, order);
        } else {
            line_axis0_kernel<<<(unsigned)blocks, 256, 0, st>>>(p);
        }
        DSGB_CHECK_LAUNCH("line_axis0 kernel");
    }
    if (!(flags & DSGB_FLAG_NO_FINALIZE) && nouts > 0)
        rc = finalize_outputs(cols, ncols, row_offset, bases, nbases, outs, nouts, ncells, st);
    return rc;
}

extern "C" int dsgb_lines(const dsgb_column *cols, int32_t ncols, int64_t nrows, int64_t row_offset,
                          int32_t layout, const double *xs, const double *ys, int64_t nv, int64_t x_row_stride,
                          int64_t y_row_stride, const dsgb_canvas *canvas, double line_width, int32_t plot_start,
                          int32_t overwrite,
                          const dsgb_base *bases, int32_t nbases, const dsgb_output *outs, int32_t nouts,
                          uint32_t flags, void *stream) {
    if (layout != 1 && layout != 2) {
        set_error("dsgb_lines: layout must be 1 (LineAxis0Multi) or 2 (LinesAxis1 family)");
        return DSGB_E_INVALID;
    }
    if (layout == 2 && ((x_row_stride != 0 && x_row_stride != nv) || (y_row_stride != 0 && y_row_stride != nv))) {
        set_error("dsgb_lines: row strides must be 0 (shared) or nv");
        return DSGB_E_INVALID;
    }
    if (nrows < 0 || nv < 1 || (nrows > 0 && (!xs || !ys))) {
        set_error("dsgb_lines: invalid vertex arrays");
        return DSGB_E_INVALID;
    }
    LineParams p;
    // the field columns are indexed by row; x/y come from xs / ys
    int rc = build_line_params(p, cols, ncols, nrows, row_offset, 0, 0, canvas, bases, nbases);
    if (rc) return rc;
    p.debug = (flags & DSGB_FLAG_DEBUG_CHECKS) != 0;
    if (!(line_width >= 0.0)) { set_error("dsgb_lines: line_width must be >= 0"); return DSGB_E_INVALID; }
    p.line_width = line_width;
    p.plot_start = plot_start;
    p.overwrite = overwrite;
    p.use_2_stage = 0;
    if (layout == 1 && nv > 1 && !(flags & DSGB_FLAG_ROW_ORDER)) p.field_mod = nrows;
    LinesGeom g;
    g.xs = xs; g.ys = ys; g.nrows = nrows; g.nv = nv;
    g.xrow = layout == 1 ? nv : x_row_stride;
    g.yrow = layout == 1 ? nv : y_row_stride;
    g.only_line = -1;
    cudaStream_t st = as_stream(stream);
    const int64_t ncells = (int64_t)canvas->width * canvas->height;
    if (!(flags & DSGB_FLAG_NO_INIT)) {
        rc = bases_init(bases, nbases, ncells, st);
        if (rc) return rc;
    }
    const int64_t nseg = layout == 1 ? (nrows > 0 ? (nrows - 1) * nv : 0) : nrows * (nv - 1);
    if (nseg > 0 && nbases > 0) {
        int sms = sm_count();
        if (sms <= 0) sms = 148;
        int64_t blocks = (nseg + 255) / 256;
        if (blocks > (int64_t)sms * 16) blocks = (int64_t)sms * 16;
        if (line_width > 0.0 && p.aa_nx <= (1 << 24) && p.aa_ny <= (1 << 24) && !(flags & DSGB_FLAG_EXACT_BIN)) {
            // antialiased: pixels queued by case (the LineAxis0 kernel's machinery)
            const unsigned qblocks = (unsigned)((int64_t)sms * 3);
            if (layout == 2) aa_queued_kernel<2, false><<<qblocks, 256, 0, st>>>(p, nullptr, g, RaggedGeom{}, nseg);
            else if (p.field_mod > 0) aa_queued_kernel<1, true><<<qblocks, 256, 0, st>>>(p, nullptr, g, RaggedGeom{}, nseg);
            else aa_queued_kernel<1, false><<<qblocks, 256, 0, st>>>(p, nullptr, g, RaggedGeom{}, nseg);
        } else if (layout == 1) {
            lines_kernel<1><<<(unsigned)blocks, 256, 0, st>>>(p, g);
        } else {
            lines_kernel<2><<<(unsigned)blocks, 256, 0, st>>>(p, g);
        }
        DSGB_CHECK_LAUNCH("lines kernel");
    }
    if (p.field_mod > 0) {
        // visit keys -> rows; a key of one call does not order against a row of another
        for (int32_t b = 0; b < nbases; ++b) {
            const int op = bases[b].op;
            if (op != DSGB_BASE_MIN_ROW && op != DSGB_BASE_MAX_ROW && op != DSGB_BASE_ARGMAX && op != DSGB_BASE_ARGMIN)
                continue;
            if (flags & DSGB_FLAG_NO_INIT) {
                set_error("dsgb_lines: row-index bases over several axis=0 lines cannot accumulate across calls");
                return DSGB_E_INVALID;
            }
            const int64_t n = ncells * (bases[b].cat_col >= 0 ? bases[b].ncat : 1);
            int64_t blocks = (n + 255) / 256;
            if (blocks > 4096) blocks = 4096;
            if (blocks > 0)
                unkey_rows_kernel<<<(unsigned)blocks, 256, 0, st>>>(op, bases[b].agg, n, nrows, row_offset);
            DSGB_CHECK_LAUNCH("unkey rows");
        }
    }
    if (!(flags & DSGB_FLAG_NO_FINALIZE) && nouts > 0)
        rc = finalize_outputs(cols, ncols, row_offset, bases, nbases, outs, nouts, ncells, st);
    return rc;
}

namespace dsgb {

// Stage-2 fold of one line's aggregate into the accumulator (compiler.py:
// 198-268 with utils.py:615-923), on the int64 storage of the bases:
// AA_MAX keys (empty = KEY_EMPTY_MAX, below every key), MIN_ROW rows (empty
// = ROW_EMPTY_MIN, above every row), MAX_ROW rows (empty = -1).
__global__ void stage2_fold_kernel(int fold, long long *acc, const long long *part, int64_t n) {
    for (int64_t c = gtid(); c < n; c += gstride()) {
        long long a = acc[c];
        const long long o = part[c];
        switch (fold) {
        case DSGB_FOLD_MAX: if (o > a) a = o; break;                 // nanmax_in_place / row_max_in_place
        case DSGB_FOLD_ROW_MIN: if (o < a) a = o; break;             // row_min_in_place
        case DSGB_FOLD_MIN:                                           // nanmin_in_place
            if (o != KEY_EMPTY_MAX && (a == KEY_EMPTY_MAX || o < a)) a = o;
            break;
        case DSGB_FOLD_FIRST: if (a == KEY_EMPTY_MAX) a = o; break;  // nanfirst_in_place
        case DSGB_FOLD_LAST: if (o != KEY_EMPTY_MAX) a = o; break;   // nanlast_in_place
        case DSGB_FOLD_SUM:                                           // nansum_in_place, float64
            if (o != KEY_EMPTY_MAX) a = a == KEY_EMPTY_MAX ? o : f64_key(__dadd_rn(key_f64(a), key_f64(o)));
            break;
        case DSGB_FOLD_SUM_F32:                                       // nansum_in_place on a float32 aggregate
            if (o != KEY_EMPTY_MAX)
                a = a == KEY_EMPTY_MAX ? o
                    : f64_key((double)__fadd_rn((float)key_f64(a), (float)key_f64(o)));
            break;
        default: break;
        }
        acc[c] = a;
    }
}

// where's stage-2 combine (reductions.py:1992-2018) on the {key, row} pairs
// of AA_ARGMAX (empty key KEY_EMPTY_MAX): the other line's selector key, when
// present, replaces the accumulated pair where the selector's own
// non-antialiased append would update (max / min strict, first only into an
// empty cell, last always), carrying that line's row.
__global__ void stage2_fold_pairs_kernel(int fold, long long *acc, const long long *part, int64_t n) {
    for (int64_t c = gtid(); c < n; c += gstride()) {
        const long long ok = part[2 * c];
        if (ok == KEY_EMPTY_MAX) continue;
        const long long ak = acc[2 * c];
        bool take = false;
        switch (fold) {
        case DSGB_FOLD_WHERE_MAX: take = ok > ak; break;
        case DSGB_FOLD_WHERE_MIN: take = ak == KEY_EMPTY_MAX || ok < ak; break;
        case DSGB_FOLD_WHERE_FIRST: take = ak == KEY_EMPTY_MAX; break;
        case DSGB_FOLD_WHERE_LAST: take = true; break;
        default: break;
        }
        if (take) { acc[2 * c] = ok; acc[2 * c + 1] = part[2 * c + 1]; }
    }
}

static bool fold_fits(int op, int fold) {
    if (op == DSGB_BASE_AA_ARGMAX)
        return fold == DSGB_FOLD_WHERE_MAX || fold == DSGB_FOLD_WHERE_MIN || fold == DSGB_FOLD_WHERE_FIRST ||
               fold == DSGB_FOLD_WHERE_LAST;
    if (op == DSGB_BASE_AA_SUM || op == DSGB_BASE_AA_CNT0 || op == DSGB_BASE_COUNT) return fold == DSGB_FOLD_ADD;
    if (op == DSGB_BASE_AA_MAX)
        return fold == DSGB_FOLD_MAX || fold == DSGB_FOLD_MIN || fold == DSGB_FOLD_FIRST || fold == DSGB_FOLD_LAST ||
               fold == DSGB_FOLD_SUM || fold == DSGB_FOLD_SUM_F32;
    if (op == DSGB_BASE_MIN_ROW) return fold == DSGB_FOLD_ROW_MIN;
    if (op == DSGB_BASE_MAX_ROW) return fold == DSGB_FOLD_MAX;
    return false;
}

}  // namespace dsgb

namespace dsgb {

// The stage-2 driver shared by the two-stage entry points: draw(params, L)
// draws line L alone; line 0 goes into the bases, every later line into the
// re-initialised per-line aggregates, folded in line order (additive bases
// keep drawing into their accumulators).
template <class DrawLine>
static int run_two_stage(LineParams &p, const dsgb_base *bases, int32_t nbases, const int32_t *folds,
                         void *const *line_aggs, int64_t nlines, int64_t ncells, cudaStream_t st, DrawLine draw) {
    if (nbases > 0 && (!folds || !line_aggs)) { set_error("two-stage lines: folds / line_aggs missing"); return DSGB_E_INVALID; }
    dsgb_base line_bases[MAX_BASES];      // the per-line aggregates to re-initialise for every line
    int32_t nline_bases = 0;
    for (int32_t b = 0; b < nbases; ++b) {
        if (!fold_fits(bases[b].op, folds[b]) || (folds[b] != DSGB_FOLD_ADD && !line_aggs[b])) {
            set_error("two-stage lines: base %d (op %d) has no stage-2 fold %d", b, bases[b].op, folds[b]);
            return DSGB_E_UNSUPPORTED;
        }
        if (folds[b] == DSGB_FOLD_ADD) continue;
        line_bases[nline_bases] = bases[b];
        line_bases[nline_bases].agg = line_aggs[b];
        ++nline_bases;
    }
    p.use_2_stage = 1;                     // the previous vertex is not read (line.py:1170, 1266)
    // the same plan drawing into the per-line aggregates; additive bases (the
    // zero-initialised sums and counts of mean, _sum_zero and
    // _count_ignore_antialiasing, whose stage-2 nansum is a plain sum) keep
    // drawing into their accumulators
    LineParams pl = p;
    for (int32_t b = 0; b < nbases; ++b)
        if (folds[b] != DSGB_FOLD_ADD) pl.bases[b].agg = line_aggs[b];
    int rc = bases_init(bases, nbases, ncells, st);
    if (rc) return rc;
    for (int64_t L = 0; L < nlines && nbases > 0; ++L) {
        if (L > 0 && nline_bases > 0) {
            rc = bases_init(line_bases, nline_bases, ncells, st);
            if (rc) return rc;
        }
        draw(L > 0 ? pl : p, L);
        DSGB_CHECK_LAUNCH("two-stage lines kernel");
        for (int32_t b = 0; b < nbases && L > 0; ++b) {
            if (folds[b] == DSGB_FOLD_ADD) continue;
            const int64_t n = ncells * (bases[b].ncat < 1 ? 1 : bases[b].ncat);
            const unsigned fb = (unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
            if (fb == 0) continue;
            if (bases[b].op == DSGB_BASE_AA_ARGMAX)
                stage2_fold_pairs_kernel<<<fb, 256, 0, st>>>(folds[b], (long long *)bases[b].agg,
                                                            (const long long *)line_aggs[b], n);
            else
                stage2_fold_kernel<<<fb, 256, 0, st>>>(folds[b], (long long *)bases[b].agg,
                                                      (const long long *)line_aggs[b], n);
            DSGB_CHECK_LAUNCH("stage-2 fold");
        }
    }
    return DSGB_OK;
}

}  // namespace dsgb

extern "C" int dsgb_lines_2stage(const dsgb_column *cols, int32_t ncols, int64_t nrows, int64_t row_offset,
                                 int32_t layout, const double *xs, const double *ys, int64_t nv,
                                 int64_t x_row_stride, int64_t y_row_stride, const dsgb_canvas *canvas,
                                 double line_width, int32_t overwrite, const dsgb_base *bases, int32_t nbases,
                                 const int32_t *folds, void *const *line_aggs, const dsgb_output *outs,
                                 int32_t nouts, uint32_t flags, void *stream) {
    if (layout != 1 && layout != 2) {
        set_error("dsgb_lines_2stage: layout must be 1 (LineAxis0Multi) or 2 (LinesAxis1 family)");
        return DSGB_E_INVALID;
    }
    if (layout == 2 && ((x_row_stride != 0 && x_row_stride != nv) || (y_row_stride != 0 && y_row_stride != nv))) {
        set_error("dsgb_lines_2stage: row strides must be 0 (shared) or nv");
        return DSGB_E_INVALID;
    }
    if (nrows < 0 || nv < 1 || (nrows > 0 && (!xs || !ys))) {
        set_error("dsgb_lines_2stage: invalid vertex arrays");
        return DSGB_E_INVALID;
    }
    if (!(line_width > 0.0)) { set_error("dsgb_lines_2stage: two-stage plans are antialiased (line_width > 0)"); return DSGB_E_INVALID; }
    if (flags & DSGB_FLAG_NO_INIT) {
        set_error("dsgb_lines_2stage: a two-stage plan cannot accumulate across calls");
        return DSGB_E_INVALID;
    }
    LineParams p;
    int rc = build_line_params(p, cols, ncols, nrows, row_offset, 0, 0, canvas, bases, nbases);
    if (rc) return rc;
    p.debug = (flags & DSGB_FLAG_DEBUG_CHECKS) != 0;
    p.line_width = line_width;
    p.plot_start = 1;
    p.overwrite = overwrite;
    LinesGeom g;
    g.xs = xs; g.ys = ys; g.nrows = nrows; g.nv = nv;
    g.xrow = layout == 1 ? nv : x_row_stride;
    g.yrow = layout == 1 ? nv : y_row_stride;
    g.only_line = -1;
    cudaStream_t st = as_stream(stream);
    const int64_t ncells = (int64_t)canvas->width * canvas->height;
    const int64_t nseg = layout == 1 ? nrows - 1 : nv - 1;   // segments of one line
    int sms = sm_count();
    if (sms <= 0) sms = 148;
    int64_t blocks = (nseg + 255) / 256;
    if (blocks > (int64_t)sms * 16) blocks = (int64_t)sms * 16;
    if (blocks < 1) blocks = 1;
    // antialiased (always, in a two-stage plan): pixels queued by case, one
    // line a launch, the grid sized to the line's 32-segment batches
    const bool queued = p.aa_nx <= (1 << 24) && p.aa_ny <= (1 << 24) && !(flags & DSGB_FLAG_EXACT_BIN);
    int64_t qblocks = ((nseg + 31) / 32 + 7) / 8;
    if (qblocks > (int64_t)sms * 3) qblocks = (int64_t)sms * 3;
    if (qblocks < 1) qblocks = 1;
    rc = run_two_stage(p, bases, nbases, folds, line_aggs, nseg > 0 ? (layout == 1 ? nv : nrows) : 0, ncells, st,
                       [&](const LineParams &pp, int64_t L) {
                           g.only_line = L;
                           if (queued && layout == 1)
                               aa_queued_kernel<1, false><<<(unsigned)qblocks, 256, 0, st>>>(pp, nullptr, g, RaggedGeom{}, nseg);
                           else if (queued)
                               aa_queued_kernel<2, false><<<(unsigned)qblocks, 256, 0, st>>>(pp, nullptr, g, RaggedGeom{}, nseg);
                           else if (layout == 1)
                               lines_kernel<1><<<(unsigned)blocks, 256, 0, st>>>(pp, g);
                           else
                               lines_kernel<2><<<(unsigned)blocks, 256, 0, st>>>(pp, g);
                       });
    if (rc) return rc;
    if (!(flags & DSGB_FLAG_NO_FINALIZE) && nouts > 0)
        rc = finalize_outputs(cols, ncols, row_offset, bases, nbases, outs, nouts, ncells, st);
    return rc;
}

extern "C" int dsgb_lines_ragged_2stage(const dsgb_column *cols, int32_t ncols, int64_t nrows, int64_t row_offset,
                                        const double *x_flat, int64_t nx, const int64_t *x_start,
                                        const double *y_flat, int64_t ny, const int64_t *y_start,
                                        const dsgb_canvas *canvas, double line_width, int32_t overwrite,
                                        const dsgb_base *bases, int32_t nbases, const int32_t *folds,
                                        void *const *line_aggs, const dsgb_output *outs, int32_t nouts,
                                        uint32_t flags, void *stream) {
    if (nrows < 0 || nx < 0 || ny < 0 || (nrows > 0 && (!x_start || !y_start)) || (nx > 0 && !x_flat) ||
        (ny > 0 && !y_flat)) {
        set_error("dsgb_lines_ragged_2stage: invalid vertex arrays");
        return DSGB_E_INVALID;
    }
    if (!(line_width > 0.0)) {
        set_error("dsgb_lines_ragged_2stage: two-stage plans are antialiased (line_width > 0)");
        return DSGB_E_INVALID;
    }
    if (flags & DSGB_FLAG_NO_INIT) {
        set_error("dsgb_lines_ragged_2stage: a two-stage plan cannot accumulate across calls");
        return DSGB_E_INVALID;
    }
    LineParams p;
    int rc = build_line_params(p, cols, ncols, nrows, row_offset, 0, 0, canvas, bases, nbases);
    if (rc) return rc;
    p.debug = (flags & DSGB_FLAG_DEBUG_CHECKS) != 0;
    p.line_width = line_width;
    p.plot_start = 1;
    p.overwrite = overwrite;
    RaggedGeom g;
    g.xf = x_flat; g.yf = y_flat; g.xs = x_start; g.ys = y_start; g.nrows = nrows; g.nx = nx; g.ny = ny;
    cudaStream_t st = as_stream(stream);
    const int64_t ncells = (int64_t)canvas->width * canvas->height;
    // a row's length is known on the device only: a small grid strides over its segments
    rc = run_two_stage(p, bases, nbases, folds, line_aggs, nx > 1 ? nrows : 0, ncells, st,
                       [&](const LineParams &pp, int64_t L) {
                           lines_ragged_row_kernel<<<32, 256, 0, st>>>(pp, g, L);
                       });
    if (rc) return rc;
    if (!(flags & DSGB_FLAG_NO_FINALIZE) && nouts > 0)
        rc = finalize_outputs(cols, ncols, row_offset, bases, nbases, outs, nouts, ncells, st);
    return rc;
}

extern "C" int dsgb_lines_ragged(const dsgb_column *cols, int32_t ncols, int64_t nrows, int64_t row_offset,
                                 const double *x_flat, int64_t nx, const int64_t *x_start,
                                 const double *y_flat, int64_t ny, const int64_t *y_start,
                                 const dsgb_canvas *canvas, double line_width, int32_t overwrite,
                                 const dsgb_base *bases, int32_t nbases, const dsgb_output *outs, int32_t nouts,
                                 uint32_t flags, void *stream) {
    if (nrows < 0 || nx < 0 || ny < 0 || (nrows > 0 && (!x_start || !y_start)) || (nx > 0 && !x_flat) ||
        (ny > 0 && !y_flat)) {
        set_error("dsgb_lines_ragged: invalid vertex arrays");
        return DSGB_E_INVALID;
    }
    LineParams p;
    int rc = build_line_params(p, cols, ncols, nrows, row_offset, 0, 0, canvas, bases, nbases);
    if (rc) return rc;
    p.debug = (flags & DSGB_FLAG_DEBUG_CHECKS) != 0;
    if (!(line_width >= 0.0)) { set_error("dsgb_lines_ragged: line_width must be >= 0"); return DSGB_E_INVALID; }
    p.line_width = line_width;
    p.plot_start = 1;
    p.overwrite = overwrite;
    p.use_2_stage = 0;
    RaggedGeom g;
    g.xf = x_flat; g.yf = y_flat; g.xs = x_start; g.ys = y_start; g.nrows = nrows; g.nx = nx; g.ny = ny;
    cudaStream_t st = as_stream(stream);
    const int64_t ncells = (int64_t)canvas->width * canvas->height;
    if (!(flags & DSGB_FLAG_NO_INIT)) {
        rc = bases_init(bases, nbases, ncells, st);
        if (rc) return rc;
    }
    if (nrows > 0 && nx > 1 && nbases > 0) {
        if (p.line_width > 0.0 && p.aa_nx <= (1 << 24) && p.aa_ny <= (1 << 24) && !(flags & DSGB_FLAG_EXACT_BIN)) {
            // antialiased: pixels queued by case (one segment a flat x vertex)
            int sms = sm_count();
            if (sms <= 0) sms = 148;
            aa_queued_kernel<3, false><<<(unsigned)((int64_t)sms * 3), 256, 0, st>>>(p, nullptr, LinesGeom{}, g, nx);
        } else {
            lines_ragged_kernel<<<grid_of(nx), 256, 0, st>>>(p, g);
        }
        DSGB_CHECK_LAUNCH("lines ragged kernel");
    }
    if (!(flags & DSGB_FLAG_NO_FINALIZE) && nouts > 0)
        rc = finalize_outputs(cols, ncols, row_offset, bases, nbases, outs, nouts, ncells, st);
    return rc;
}
