// points_params.cuh -- the parameters and per-row device code shared by the
// Canvas.points kernels (points.cu) and the deterministic sum path
// (points_det.cu): exact binning of a row and the fused append of every base.
#pragma once

#include "dsgb_internal.cuh"
#include "binning.cuh"

namespace dsgb {

struct PointsParams {
    ColumnRef cols[MAX_COLS];
    BaseDev bases[MAX_BASES];
    int32_t ncols, nbases;
    int64_t n, row_offset;
    int32_t x_col, y_col;
    int32_t width, height;
    int32_t x_log, y_log;
    double sx, tx, sy, ty;
    double xmin, xmax, ymin, ymax;
    BinAxis ax, ay;                    // float32 fast path (binning.cuh)
    BinBounds bb;
    int32_t debug;                     // DSGB_FLAG_DEBUG_CHECKS
};

// ------------------------------------------------------------------ binning

__device__ __forceinline__ bool bin_f32_fast(const PointsParams &p, float x, float y, int &xi, int &yi) {
    return bin_point_f32(x, y, p.bb, p.ax, p.ay, xi, yi);
}

__device__ __forceinline__ bool bin_f64_fast(const PointsParams &p, double x, double y, int &xi, int &yi) {
    return bin_point_f64(x, y, p.bb, p.ax, p.ay, xi, yi);
}

__device__ __forceinline__ bool bin_exact_xy(const PointsParams &p, double x, double y, int &xi, int &yi) {
    if (!((p.xmin <= x && x <= p.xmax) && (p.ymin <= y && y <= p.ymax))) return false;
    double mx = p.x_log ? log10(x) : x;   // LogAxis.mapper (core.py:131-134)
    double my = p.y_log ? log10(y) : y;
    xi = bin_exact64(mx, p.ax);
    yi = bin_exact64(my, p.ay);
    return true;
}

// ---------------------------------------------------------------- appends

// The GPU form of the fused append: one pass over the bases for row i.
__device__ __forceinline__ void accumulate(const PointsParams &p, int64_t i, int64_t pix) {
    const long long row = (long long)(i + p.row_offset);
#pragma unroll 1
    for (int b = 0; b < p.nbases; ++b) {
        const BaseDev &B = p.bases[b];
        int64_t cell = pix;
        if (B.cat_col >= 0) {
            // compiler.py:379-390 -- agg[:, :, int(code)], negative codes wrap
            long long c = load_i64(p.cols[B.cat_col], i);
            if (c < 0) c += B.ncat;
            if (c < 0 || c >= B.ncat) {
                if (p.debug) raise_status(DSGB_STATUS_INDEX);
                continue;
            }
            cell = pix * B.ncat + c;
        }
        double field = 0.0;
        bool has = true;
        if (B.col >= 0) {
            field = load_f64(p.cols[B.col], i);
            has = !isnull(field);
        }
        if (!has) continue;
        switch (B.op) {
        case DSGB_BASE_COUNT: atomicAdd((unsigned *)B.agg + cell, 1u); break;
        case DSGB_BASE_ANY: ((volatile uint8_t *)B.agg)[cell] = 1; break;
        case DSGB_BASE_SUM: atomicAdd((double *)B.agg + cell, field); break;
        case DSGB_BASE_MAX: atomic_max_key((long long *)B.agg + cell, f64_key(field)); break;
        case DSGB_BASE_MIN: atomic_min_key((long long *)B.agg + cell, f64_key(field)); break;
        case DSGB_BASE_MIN_ROW: atomic_min_key((long long *)B.agg + cell, row); break;
        case DSGB_BASE_MAX_ROW: atomic_max_key((long long *)B.agg + cell, row); break;
        case DSGB_BASE_ARGMAX: pair_update<true>((long long *)B.agg + 2 * cell, f64_key(field), row); break;
        case DSGB_BASE_ARGMIN: pair_update<false>((long long *)B.agg + 2 * cell, f64_key(field), row); break;
        default: break;
        }
    }
}

enum Mode { MODE_GENERIC = 0, MODE_COUNT = 1, MODE_MEAN = 2 };

// Per-row work of one kernel instantiation.  MEAN: bases[0] = SUM(v), bases[1] = COUNT(v).
template <int MODE>
__device__ __forceinline__ void emit(const PointsParams &p, int64_t i, int xi, int yi, double v) {
    if (p.debug && ((unsigned)xi >= (unsigned)p.width || (unsigned)yi >= (unsigned)p.height)) {
        raise_status(DSGB_STATUS_INDEX);
        return;
    }
    int64_t pix = (int64_t)yi * p.width + xi;
    if (MODE == MODE_COUNT) {
        atomicAdd((unsigned *)p.bases[0].agg + pix, 1u);
    } else if (MODE == MODE_MEAN) {
        if (!isnull(v)) {
            atomicAdd((double *)p.bases[0].agg + pix, v);
            atomicAdd((unsigned *)p.bases[1].agg + pix, 1u);
        }
    } else {
        accumulate(p, i, pix);
    }
}

template <int MODE>
__device__ __forceinline__ double mean_value(const PointsParams &p, int64_t i) {
    if (MODE != MODE_MEAN) return 0.0;
    return load_f64(p.cols[p.bases[0].col], i);
}

}  // namespace dsgb
