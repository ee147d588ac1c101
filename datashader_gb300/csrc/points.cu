// points.cu -- Canvas.points on GB300: projection + fused aggregation.
//
// Replaces Point._build_extend (datashader/glyphs/points.py:182-242) and the
// per-reduction append functions that compiler.make_append fuses
// (datashader/compiler.py:321-475).
//
// Binning is exact (binning.cuh): a float32 fast path proven against the
// float64 formula of points.py:199-203, with a float64 fallback.
#include "points_params.cuh"

namespace dsgb {


// float32 coordinates, 4 rows per thread per iteration (float4 streaming loads).
template <int MODE, bool FAST, bool WARPAGG>
__global__ void __launch_bounds__(256, 4) points_f32_kernel(const PointsParams p) {
    const float *xs = (const float *)p.cols[p.x_col].data;
    const float *ys = (const float *)p.cols[p.y_col].data;
    const int64_t n4 = p.n >> 2;
    const float4 *x4 = (const float4 *)xs;
    const float4 *y4 = (const float4 *)ys;
    const int lane = threadIdx.x & 31;
    // Warp-uniform trip count so that the warp-level match below is legal.
    for (int64_t base = gtid() - lane; base < n4; base += gstride()) {
        const int64_t v = base + lane;
        const bool live = v < n4;
        float4 a = make_float4(0, 0, 0, 0), b = a;
        if (live) { a = __ldcs(x4 + v); b = __ldcs(y4 + v); }
        float xa[4] = {a.x, a.y, a.z, a.w};
        float ya[4] = {b.x, b.y, b.z, b.w};
        double va[4] = {0, 0, 0, 0};
        if (MODE == MODE_MEAN && live) {
#pragma unroll
            for (int k = 0; k < 4; ++k) va[k] = mean_value<MODE>(p, 4 * v + k);
        }
        int xs_[4], ys_[4];
        unsigned inm = 0;
        if (FAST) {
            unsigned need = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int r = live ? bin_try_f32(xa[k], ya[k], p.bb, p.ax, p.ay, xs_[k], ys_[k]) : 0;
                inm |= (unsigned)(r != 0) << k;
                need |= (unsigned)(r == 2) << k;
            }
            if (need) {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if ((need >> k) & 1u) bin_exact_f32(xa[k], ya[k], p.ax, p.ay, xs_[k], ys_[k]);
            }
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                inm |= (unsigned)(live && bin_exact_xy(p, (double)xa[k], (double)ya[k], xs_[k], ys_[k])) << k;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const bool in = (inm >> k) & 1u;
            const int xi = in ? xs_[k] : 0, yi = in ? ys_[k] : 0;
            if (WARPAGG && MODE == MODE_COUNT) {
                unsigned key = in ? (unsigned)(yi * p.width + xi) : (0x80000000u | (unsigned)lane);
                unsigned peers = __match_any_sync(0xffffffffu, key);
                if (in && lane == __ffs(peers) - 1)
                    atomicAdd((unsigned *)p.bases[0].agg + key, (unsigned)__popc(peers));
            } else if (in) {
                emit<MODE>(p, 4 * v + k, xi, yi, va[k]);
            }
        }
    }
    // tail rows (n not a multiple of 4)
    for (int64_t i = 4 * n4 + gtid(); i < p.n; i += gstride()) {
        int xi, yi;
        float x = xs[i], y = ys[i];
        bool in = FAST ? bin_f32_fast(p, x, y, xi, yi) : bin_exact_xy(p, (double)x, (double)y, xi, yi);
        if (in) emit<MODE>(p, i, xi, yi, mean_value<MODE>(p, i));
    }
}

// float64 coordinates, 2 rows per thread per iteration (double2 streaming loads).
template <int MODE, bool FAST>
__global__ void __launch_bounds__(256, 4) points_f64_kernel(const PointsParams p) {
    const double *xs = (const double *)p.cols[p.x_col].data;
    const double *ys = (const double *)p.cols[p.y_col].data;
    const int64_t n2 = p.n >> 1;
    const double2 *x2 = (const double2 *)xs;
    const double2 *y2 = (const double2 *)ys;
    for (int64_t v = gtid(); v < n2; v += gstride()) {
        double2 a = __ldcs(x2 + v), b = __ldcs(y2 + v);
        double xa[2] = {a.x, a.y}, ya[2] = {b.x, b.y};
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            int xi, yi;
            bool in = FAST ? bin_f64_fast(p, xa[k], ya[k], xi, yi) : bin_exact_xy(p, xa[k], ya[k], xi, yi);
            if (in) emit<MODE>(p, 2 * v + k, xi, yi, mean_value<MODE>(p, 2 * v + k));
        }
    }
    for (int64_t i = 2 * n2 + gtid(); i < p.n; i += gstride()) {
        int xi, yi;
        bool in = FAST ? bin_f64_fast(p, xs[i], ys[i], xi, yi) : bin_exact_xy(p, xs[i], ys[i], xi, yi);
        if (in) emit<MODE>(p, i, xi, yi, mean_value<MODE>(p, i));
    }
}

// Any coordinate dtype (integers, unaligned columns): scalar loads, exact binning.
template <int MODE>
__global__ void __launch_bounds__(256) points_any_kernel(const PointsParams p) {
    for (int64_t i = gtid(); i < p.n; i += gstride()) {
        int xi, yi;
        double x = load_f64(p.cols[p.x_col], i), y = load_f64(p.cols[p.y_col], i);
        if (bin_exact_xy(p, x, y, xi, yi)) emit<MODE>(p, i, xi, yi, mean_value<MODE>(p, i));
    }
}

// Rows given as segments [begin, end) of the columns (a viewport over a
// spatially sorted store): blockIdx.y is the segment, blockIdx.x strides it.
constexpr int MAX_SEGMENTS = 256;
struct SegList {
    int64_t begin[MAX_SEGMENTS];
    int64_t end[MAX_SEGMENTS];
};

template <int MODE, bool F32, bool FAST>
__global__ void __launch_bounds__(256) points_seg_kernel(const PointsParams p, const SegList s) {
    const int64_t b = s.begin[blockIdx.y], e = s.end[blockIdx.y];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = b + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < e; i += stride) {
        int xi, yi;
        bool in;
        if (F32) {
            const float x = ((const float *)p.cols[p.x_col].data)[i];
            const float y = ((const float *)p.cols[p.y_col].data)[i];
            in = FAST ? bin_f32_fast(p, x, y, xi, yi) : bin_exact_xy(p, (double)x, (double)y, xi, yi);
        } else {
            in = bin_exact_xy(p, load_f64(p.cols[p.x_col], i), load_f64(p.cols[p.y_col], i), xi, yi);
        }
        if (in) emit<MODE>(p, i, xi, yi, mean_value<MODE>(p, i));
    }
}

// ------------------------------------------------------------- host side

static int build_params(PointsParams &p, const dsgb_column *cols, int32_t ncols, int64_t n,
                        int64_t row_offset, int32_t x_col, int32_t y_col,
                        const dsgb_canvas *cv, const dsgb_base *bases, int32_t nbases) {
    if (!cols || !cv || ncols <= 0 || ncols > MAX_COLS || n < 0 || nbases < 0 || nbases > MAX_BASES ||
        (nbases > 0 && !bases)) {
        set_error("dsgb_points: invalid arguments (ncols=%d, n=%lld, nbases=%d)", ncols, (long long)n, nbases);
        return DSGB_E_INVALID;
    }
    if (x_col < 0 || x_col >= ncols || y_col < 0 || y_col >= ncols) {
        set_error("dsgb_points: x_col/y_col out of range");
        return DSGB_E_INVALID;
    }
    if (cv->width <= 0 || cv->height <= 0) {
        set_error("dsgb_points: invalid canvas size %dx%d", cv->width, cv->height);
        return DSGB_E_INVALID;
    }
    memset(&p, 0, sizeof(p));
    for (int c = 0; c < ncols; ++c) {
        if (dtype_size(cols[c].dtype) == 0 || (n > 0 && !cols[c].data)) {
            set_error("dsgb_points: column %d has bad dtype %d or null data", c, cols[c].dtype);
            return DSGB_E_INVALID;
        }
        p.cols[c].data = cols[c].data;
        p.cols[c].dtype = cols[c].dtype;
    }
    for (int b = 0; b < nbases; ++b) {
        const dsgb_base &B = bases[b];
        if (!B.agg || B.col >= ncols || B.cat_col >= ncols || B.ncat < 1 ||
            B.op < DSGB_BASE_COUNT || B.op > DSGB_BASE_ARGMIN) {
            set_error("dsgb_points: base %d invalid (op=%d col=%d cat=%d ncat=%d)", b, B.op, B.col,
                      B.cat_col, B.ncat);
            return DSGB_E_INVALID;
        }
        p.bases[b] = BaseDev{B.op, B.col, B.cat_col < 0 ? -1 : B.cat_col, B.ncat, B.flags, B.agg};
    }
    p.ncols = ncols; p.nbases = nbases; p.n = n; p.row_offset = row_offset;
    p.x_col = x_col; p.y_col = y_col;
    p.width = cv->width; p.height = cv->height; p.x_log = cv->x_log; p.y_log = cv->y_log;
    p.sx = cv->sx; p.tx = cv->tx; p.sy = cv->sy; p.ty = cv->ty;
    p.xmin = cv->xmin; p.xmax = cv->xmax; p.ymin = cv->ymin; p.ymax = cv->ymax;
    p.ax = make_axis(cv->sx, cv->tx, cv->xmin, cv->xmax, cv->width);
    p.ay = make_axis(cv->sy, cv->ty, cv->ymin, cv->ymax, cv->height);
    p.bb = make_bounds(cv->xmin, cv->xmax, cv->ymin, cv->ymax);
    return DSGB_OK;
}

static bool aligned16(const void *ptr) { return ((uintptr_t)ptr & 15u) == 0; }

int launch_points(const PointsParams &p, uint32_t flags, cudaStream_t st) {
    if (p.n == 0 || p.nbases == 0) return DSGB_OK;
    int mode = MODE_GENERIC;
    if (p.nbases == 1 && p.bases[0].op == DSGB_BASE_COUNT && p.bases[0].col < 0 && p.bases[0].cat_col < 0)
        mode = MODE_COUNT;
    else if (p.nbases == 2 && p.bases[0].op == DSGB_BASE_SUM && p.bases[1].op == DSGB_BASE_COUNT &&
             p.bases[0].col >= 0 && p.bases[0].col == p.bases[1].col &&
             p.bases[0].cat_col < 0 && p.bases[1].cat_col < 0)
        mode = MODE_MEAN;
    const int xdt = p.cols[p.x_col].dtype, ydt = p.cols[p.y_col].dtype;
    const void *xp = p.cols[p.x_col].data, *yp = p.cols[p.y_col].data;
    const bool fast = !(flags & DSGB_FLAG_EXACT_BIN) && !p.x_log && !p.y_log && fast_path_ok(p.ax, p.ay);
    const bool warpagg = (flags & DSGB_FLAG_WARP_AGG) != 0;
    const int threads = 256;
    int sms = sm_count();
    if (sms <= 0) sms = 148;
    int64_t blocks = (int64_t)sms * 8;
    if (xdt == DSGB_F32 && ydt == DSGB_F32 && aligned16(xp) && aligned16(yp)) {
        int64_t need = ((p.n >> 2) + threads - 1) / threads;
        if (need < 1) need = 1;
        if (blocks > need) blocks = need;
#define DSGB_L32(M, F, W) points_f32_kernel<M, F, W><<<(unsigned)blocks, threads, 0, st>>>(p)
        if (mode == MODE_COUNT) {
            if (fast) { if (warpagg) DSGB_L32(MODE_COUNT, true, true); else DSGB_L32(MODE_COUNT, true, false); }
            else { if (warpagg) DSGB_L32(MODE_COUNT, false, true); else DSGB_L32(MODE_COUNT, false, false); }
        } else if (mode == MODE_MEAN) {
            if (fast) DSGB_L32(MODE_MEAN, true, false); else DSGB_L32(MODE_MEAN, false, false);
        } else {
            if (fast) DSGB_L32(MODE_GENERIC, true, false); else DSGB_L32(MODE_GENERIC, false, false);
        }
#undef DSGB_L32
    } else if (xdt == DSGB_F64 && ydt == DSGB_F64 && aligned16(xp) && aligned16(yp)) {
        int64_t need = ((p.n >> 1) + threads - 1) / threads;
        if (need < 1) need = 1;
        if (blocks > need) blocks = need;
#define DSGB_L64(M, F) points_f64_kernel<M, F><<<(unsigned)blocks, threads, 0, st>>>(p)
        if (mode == MODE_COUNT) { if (fast) DSGB_L64(MODE_COUNT, true); else DSGB_L64(MODE_COUNT, false); }
        else if (mode == MODE_MEAN) { if (fast) DSGB_L64(MODE_MEAN, true); else DSGB_L64(MODE_MEAN, false); }
        else { if (fast) DSGB_L64(MODE_GENERIC, true); else DSGB_L64(MODE_GENERIC, false); }
#undef DSGB_L64
    } else {
        int64_t need = (p.n + threads - 1) / threads;
        if (blocks > need) blocks = need;
        if (mode == MODE_COUNT) points_any_kernel<MODE_COUNT><<<(unsigned)blocks, threads, 0, st>>>(p);
        else if (mode == MODE_MEAN) points_any_kernel<MODE_MEAN><<<(unsigned)blocks, threads, 0, st>>>(p);
        else points_any_kernel<MODE_GENERIC><<<(unsigned)blocks, threads, 0, st>>>(p);
    }
    DSGB_CHECK_LAUNCH("points kernel launch");
    return DSGB_OK;
}

static int launch_points_segments(const PointsParams &p, const SegList &s, int nseg, int64_t maxlen,
                                  uint32_t flags, cudaStream_t st) {
    if (nseg == 0 || maxlen == 0 || p.nbases == 0) return DSGB_OK;
    int mode = MODE_GENERIC;
    if (p.nbases == 1 && p.bases[0].op == DSGB_BASE_COUNT && p.bases[0].col < 0 && p.bases[0].cat_col < 0)
        mode = MODE_COUNT;
    else if (p.nbases == 2 && p.bases[0].op == DSGB_BASE_SUM && p.bases[1].op == DSGB_BASE_COUNT &&
             p.bases[0].col >= 0 && p.bases[0].col == p.bases[1].col &&
             p.bases[0].cat_col < 0 && p.bases[1].cat_col < 0)
        mode = MODE_MEAN;
    const bool f32 = p.cols[p.x_col].dtype == DSGB_F32 && p.cols[p.y_col].dtype == DSGB_F32;
    const bool fast = f32 && !(flags & DSGB_FLAG_EXACT_BIN) && !p.x_log && !p.y_log && fast_path_ok(p.ax, p.ay);
    int sms = sm_count();
    if (sms <= 0) sms = 148;
    int64_t gx = (maxlen + 255) / 256;
    const int64_t cap = ((int64_t)sms * 8 + nseg - 1) / nseg;
    if (gx > cap) gx = cap;
    if (gx < 1) gx = 1;
    const dim3 grid((unsigned)gx, (unsigned)nseg);
#define DSGB_LSEG(M)                                                                        \
    do {                                                                                    \
        if (fast) points_seg_kernel<M, true, true><<<grid, 256, 0, st>>>(p, s);            \
        else if (f32) points_seg_kernel<M, true, false><<<grid, 256, 0, st>>>(p, s);       \
        else points_seg_kernel<M, false, false><<<grid, 256, 0, st>>>(p, s);               \
    } while (0)
    if (mode == MODE_COUNT) DSGB_LSEG(MODE_COUNT);
    else if (mode == MODE_MEAN) DSGB_LSEG(MODE_MEAN);
    else DSGB_LSEG(MODE_GENERIC);
#undef DSGB_LSEG
    DSGB_CHECK_LAUNCH("points segments kernel launch");
    return DSGB_OK;
}

int bases_init(const dsgb_base *bases, int32_t nbases, int64_t ncells, cudaStream_t st);
size_t cached_workspace_size(int64_t n, int width, int height);
int launch_points_hot(const ColumnRef &xc, const ColumnRef &yc, int64_t n, const dsgb_canvas *cv,
                      const BinAxis &ax, const BinAxis &ay, const BinBounds &bb, uint32_t *out, bool accumulate,
                      cudaStream_t st);
int launch_points_hot_mean(const ColumnRef &xc, const ColumnRef &yc, const ColumnRef &vc, int64_t n,
                           const dsgb_canvas *cv, const BinAxis &ax, const BinAxis &ay, const BinBounds &bb,
                           double *sum, uint32_t *count, bool accumulate, cudaStream_t st);
int launch_points_cached(const ColumnRef &xc, const ColumnRef &yc, int64_t n, const dsgb_canvas *cv,
                         const BinAxis &ax, const BinAxis &ay, const BinBounds &bb,
                         uint32_t *out, bool accumulate, void *ws, size_t ws_bytes, cudaStream_t st);
int launch_points_cached_mean(const ColumnRef &xc, const ColumnRef &yc, const ColumnRef &vc, int64_t n,
                              const dsgb_canvas *cv, const BinAxis &ax, const BinAxis &ay, const BinBounds &bb,
                              double *sum, uint32_t *count, bool accumulate, void *ws, size_t ws_bytes,
                              cudaStream_t st);

// mean(v): bases[0] = SUM(v), bases[1] = COUNT(v), nothing else.
static bool cached_mean_eligible(const PointsParams &p, uint32_t flags) {
    return p.nbases == 2 && p.bases[0].op == DSGB_BASE_SUM && p.bases[1].op == DSGB_BASE_COUNT &&
           p.bases[0].col >= 0 && p.bases[0].col == p.bases[1].col && p.bases[0].cat_col < 0 &&
           p.bases[1].cat_col < 0 && !(flags & (DSGB_FLAG_EXACT_BIN | DSGB_FLAG_WARP_AGG | DSGB_FLAG_DETERMINISTIC)) &&
           !p.x_log && !p.y_log && fast_path_ok(p.ax, p.ay);
}

// The hot-tile paths serve a plain count() of every row on a canvas that the
// float32 fast path may bin: the per-CTA kernel of points_hot.cu first, the
// global-selection kernels of points_cached.cu when it declines.
static bool cached_eligible(const PointsParams &p, uint32_t flags) {
    return p.nbases == 1 && p.bases[0].op == DSGB_BASE_COUNT && p.bases[0].col < 0 &&
           p.bases[0].cat_col < 0 && !(flags & (DSGB_FLAG_EXACT_BIN | DSGB_FLAG_WARP_AGG)) &&
           !p.x_log && !p.y_log && fast_path_ok(p.ax, p.ay);
}

size_t det_workspace_size(int64_t n);
int det_sums(const PointsParams &p, bool fast, void *ws, size_t ws_bytes, cudaStream_t st);
size_t part_workspace_size(int64_t n, const dsgb_canvas *cv, const dsgb_base *bases, int32_t nbases);
int launch_points_part(const PointsParams &p, const dsgb_base *bases, void *ws, size_t ws_bytes, cudaStream_t st);

static bool has_sum_base(const PointsParams &p) {
    for (int b = 0; b < p.nbases; ++b)
        if (p.bases[b].op == DSGB_BASE_SUM) return true;
    return false;
}

int finalize_outputs(const dsgb_column *cols, int32_t ncols, int64_t row_offset,
                     const dsgb_base *bases, int32_t nbases, const dsgb_output *outs, int32_t nouts,
                     int64_t ncells, cudaStream_t st);
// The same with the gather bound: a selected row outside [row_offset,
// row_offset + ncol_rows) (one that an earlier call accumulated) gathers NaN.
int finalize_outputs(const dsgb_column *cols, int32_t ncols, int64_t row_offset,
                     const dsgb_base *bases, int32_t nbases, const dsgb_output *outs, int32_t nouts,
                     int64_t ncells, cudaStream_t st, int64_t ncol_rows);

}  // namespace dsgb

namespace dsgb {
DSGB_STATUS_READER(status_points)
}

using namespace dsgb;

static int points_impl(const dsgb_column *cols, int32_t ncols, int64_t n, int64_t row_offset,
                       int32_t x_col, int32_t y_col, const dsgb_canvas *canvas,
                       const dsgb_base *bases, int32_t nbases,
                       const dsgb_output *outs, int32_t nouts,
                       void *workspace, size_t ws_bytes, uint32_t flags, void *stream) {
    NvtxRange range("dsgb_points");
    PointsParams p;
    int rc = build_params(p, cols, ncols, n, row_offset, x_col, y_col, canvas, bases, nbases);
    if (rc) return rc;
    p.debug = (flags & DSGB_FLAG_DEBUG_CHECKS) != 0;
    if (p.debug) workspace = nullptr;       // the checked appends live in the generic kernels
    cudaStream_t st = as_stream(stream);
    const int64_t ncells = (int64_t)canvas->width * canvas->height;
    if ((flags & DSGB_FLAG_DETERMINISTIC) && has_sum_base(p)) {
        // float64 sums in row order (points_det.cu); the other bases as usual
        if (!(flags & DSGB_FLAG_NO_INIT)) {
            rc = bases_init(bases, nbases, ncells, st);
            if (rc) return rc;
        }
        const bool fast = !(flags & DSGB_FLAG_EXACT_BIN) && !p.x_log && !p.y_log && fast_path_ok(p.ax, p.ay);
        PointsParams rest = p;
        bool any_rest = false;
        for (int b = 0; b < rest.nbases; ++b) {
            if (rest.bases[b].op == DSGB_BASE_SUM) rest.bases[b].op = 0;     // skipped by the append
            else any_rest = true;
        }
        if (any_rest) {
            rc = launch_points(rest, flags & ~DSGB_FLAG_WARP_AGG, st);
            if (rc) return rc;
        }
        rc = det_sums(p, fast, workspace, ws_bytes, st);
        if (rc) return rc;
        if (!(flags & DSGB_FLAG_NO_FINALIZE) && nouts > 0)
            rc = finalize_outputs(cols, ncols, row_offset, bases, nbases, outs, nouts, ncells, st, n);
        return rc;
    }
    if (cached_eligible(p, flags)) {
        // float32 coordinates, count(): the per-SM hot-tile kernel (points_hot.cu)
        rc = launch_points_hot(p.cols[x_col], p.cols[y_col], n, canvas, p.ax, p.ay, p.bb,
                               (uint32_t *)p.bases[0].agg, (flags & DSGB_FLAG_NO_INIT) != 0, st);
        if (rc != DSGB_E_UNSUPPORTED) return rc;
    }
    if (workspace && cached_eligible(p, flags)) {
        rc = launch_points_cached(p.cols[x_col], p.cols[y_col], n, canvas, p.ax, p.ay, p.bb,
                                  (uint32_t *)p.bases[0].agg, (flags & DSGB_FLAG_NO_INIT) != 0,
                                  workspace, ws_bytes, st);
        if (rc != DSGB_E_UNSUPPORTED) return rc;
    }
    if (cached_mean_eligible(p, flags)) {
        // float32 coordinates, mean(v) with a float64 v: the per-SM hot-tile kernel (points_hot.cu)
        rc = launch_points_hot_mean(p.cols[x_col], p.cols[y_col], p.cols[p.bases[0].col], n, canvas, p.ax, p.ay,
                                    p.bb, (double *)p.bases[0].agg, (uint32_t *)p.bases[1].agg,
                                    (flags & DSGB_FLAG_NO_INIT) != 0, st);
        if (rc == DSGB_OK && !(flags & DSGB_FLAG_NO_FINALIZE) && nouts > 0)
            rc = finalize_outputs(cols, ncols, row_offset, bases, nbases, outs, nouts, ncells, st, n);
        if (rc != DSGB_E_UNSUPPORTED) return rc;
    }
    if (workspace && cached_mean_eligible(p, flags)) {
        rc = launch_points_cached_mean(p.cols[x_col], p.cols[y_col], p.cols[p.bases[0].col], n, canvas, p.ax, p.ay,
                                       p.bb, (double *)p.bases[0].agg, (uint32_t *)p.bases[1].agg,
                                       (flags & DSGB_FLAG_NO_INIT) != 0, workspace, ws_bytes, st);
        if (rc == DSGB_OK && !(flags & DSGB_FLAG_NO_FINALIZE) && nouts > 0)
            rc = finalize_outputs(cols, ncols, row_offset, bases, nbases, outs, nouts, ncells, st, n);
        if (rc != DSGB_E_UNSUPPORTED) return rc;
    }
    if (!(flags & DSGB_FLAG_NO_INIT)) {
        rc = bases_init(bases, nbases, ncells, st);
        if (rc) return rc;
    }
    rc = DSGB_E_UNSUPPORTED;
    if (workspace && !(flags & (DSGB_FLAG_EXACT_BIN | DSGB_FLAG_WARP_AGG))) {
        // plans of several bases: rows partitioned by canvas block, bases in shared memory (points_part.cu)
        rc = launch_points_part(p, bases, workspace, ws_bytes, st);
        if (rc != DSGB_OK && rc != DSGB_E_UNSUPPORTED) return rc;
    }
    if (rc == DSGB_E_UNSUPPORTED) {
        rc = launch_points(p, flags, st);
        if (rc) return rc;
    }
    if (!(flags & DSGB_FLAG_NO_FINALIZE) && nouts > 0)
        rc = finalize_outputs(cols, ncols, row_offset, bases, nbases, outs, nouts, ncells, st, n);
    return rc;
}

extern "C" int dsgb_points(const dsgb_column *cols, int32_t ncols, int64_t n, int64_t row_offset,
                           int32_t x_col, int32_t y_col, const dsgb_canvas *canvas,
                           const dsgb_base *bases, int32_t nbases,
                           const dsgb_output *outs, int32_t nouts,
                           uint32_t flags, void *stream) {
    return points_impl(cols, ncols, n, row_offset, x_col, y_col, canvas, bases, nbases, outs, nouts,
                       nullptr, 0, flags, stream);
}

extern "C" size_t dsgb_points_workspace_size(int64_t n, const dsgb_canvas *canvas,
                                             const dsgb_base *bases, int32_t nbases) {
    if (!canvas || n < 0 || !bases) return 0;
    const bool count = nbases == 1 && bases[0].op == DSGB_BASE_COUNT && bases[0].col < 0 && bases[0].cat_col < 0;
    const bool mean = nbases == 2 && bases[0].op == DSGB_BASE_SUM && bases[1].op == DSGB_BASE_COUNT &&
                      bases[0].col >= 0 && bases[0].col == bases[1].col && bases[0].cat_col < 0 &&
                      bases[1].cat_col < 0;
    if (!count && !mean) return part_workspace_size(n, canvas, bases, nbases);
    return cached_workspace_size(n, canvas->width, canvas->height);
}

extern "C" size_t dsgb_points_workspace_size_flags(int64_t n, const dsgb_canvas *canvas, const dsgb_base *bases,
                                                   int32_t nbases, uint32_t flags) {
    if (!canvas || n < 0 || nbases < 0 || (nbases > 0 && !bases)) return 0;
    size_t need = dsgb_points_workspace_size(n, canvas, bases, nbases);
    if (flags & DSGB_FLAG_DETERMINISTIC) {
        for (int b = 0; b < nbases; ++b)
            if (bases[b].op == DSGB_BASE_SUM) {
                const size_t d = det_workspace_size(n);
                if (d > need) need = d;
                break;
            }
    }
    return need;
}

extern "C" int dsgb_points_ws(const dsgb_column *cols, int32_t ncols, int64_t n, int64_t row_offset,
                              int32_t x_col, int32_t y_col, const dsgb_canvas *canvas,
                              const dsgb_base *bases, int32_t nbases,
                              const dsgb_output *outs, int32_t nouts,
                              void *workspace, size_t workspace_bytes, uint32_t flags, void *stream) {
    return points_impl(cols, ncols, n, row_offset, x_col, y_col, canvas, bases, nbases, outs, nouts,
                       workspace, workspace_bytes, flags, stream);
}

extern "C" int dsgb_points_segments(const dsgb_column *cols, int32_t ncols, int64_t n, int32_t x_col,
                                    int32_t y_col, const dsgb_canvas *canvas, const dsgb_base *bases,
                                    int32_t nbases, const dsgb_output *outs, int32_t nouts,
                                    const int64_t *seg_begin, const int64_t *seg_end, int32_t nseg,
                                    uint32_t flags, void *stream) {
    if (nseg < 0 || nseg > MAX_SEGMENTS || (nseg > 0 && (!seg_begin || !seg_end))) {
        set_error("dsgb_points_segments: nseg=%d outside 0..%d or null segment arrays", nseg, MAX_SEGMENTS);
        return DSGB_E_INVALID;
    }
    PointsParams p;
    int rc = build_params(p, cols, ncols, n, 0, x_col, y_col, canvas, bases, nbases);
    if (rc) return rc;
    p.debug = (flags & DSGB_FLAG_DEBUG_CHECKS) != 0;
    SegList s;
    memset(&s, 0, sizeof(s));
    int64_t maxlen = 0;
    int k = 0;
    for (int i = 0; i < nseg; ++i) {
        if (seg_begin[i] < 0 || seg_end[i] < seg_begin[i] || seg_end[i] > n) {
            set_error("dsgb_points_segments: segment %d [%lld, %lld) outside [0, %lld)", i,
                      (long long)seg_begin[i], (long long)seg_end[i], (long long)n);
            return DSGB_E_INVALID;
        }
        if (seg_end[i] == seg_begin[i]) continue;
        s.begin[k] = seg_begin[i];
        s.end[k] = seg_end[i];
        if (seg_end[i] - seg_begin[i] > maxlen) maxlen = seg_end[i] - seg_begin[i];
        ++k;
    }
    cudaStream_t st = as_stream(stream);
    const int64_t ncells = (int64_t)canvas->width * canvas->height;
    if (!(flags & DSGB_FLAG_NO_INIT)) {
        rc = bases_init(bases, nbases, ncells, st);
        if (rc) return rc;
    }
    rc = launch_points_segments(p, s, k, maxlen, flags, st);
    if (rc) return rc;
    if (!(flags & DSGB_FLAG_NO_FINALIZE) && nouts > 0)
        rc = finalize_outputs(cols, ncols, 0, bases, nbases, outs, nouts, ncells, st);
    return rc;
}
