/*
 * dsgb_oracle.c -- CPU oracle (test infrastructure only).
 *
 * This file is the checker for the GPU aggregation path.  It restates, in
 * plain C and row by row, the algorithm of datashader's numba CPU path
 * (datashader 0.19.1).  It is never linked into the product library: only
 * the test suite, the smoke check and the CPU-baseline leg of the benchmark
 * load it.
 *
 * Every function cites the reference file:line whose behaviour it follows.
 * It is compiled with -ffp-contract=off because numba (no fastmath,
 * datashader/utils.py:51) emits no fused multiply-adds: every product and
 * sum below is rounded separately, exactly as in the reference.
 *
 * Columns are passed as float64 arrays.  That is the same promotion numba
 * performs when an int32 / int64 / float32 column meets a float64 scale or
 * a float64 aggregate (e.g. glyphs/points.py:199 `x * sx + tx`,
 * reductions.py:1058 `agg[y, x] += field`).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* Reduction kinds (user-level reductions of datashader/reductions.py). */
enum {
    ORK_COUNT = 1,     /* count(col?)            reductions.py:532-664 */
    ORK_ANY = 2,       /* any(col?)              reductions.py:824-889 */
    ORK_SUM = 3,       /* sum(col), NaN-init     reductions.py:1030-1098 */
    ORK_SUM_ZERO = 4,  /* _sum_zero(col)         reductions.py:938-996 */
    ORK_MEAN = 5,      /* mean = _sum_zero + _count_ignore_antialiasing, reductions.py:1280-1297 */
    ORK_MIN = 6,       /* min(col)               reductions.py:1160-1213 */
    ORK_MAX = 7,       /* max(col)               reductions.py:1216-1260 */
    ORK_FIRST = 8,     /* first(col)             reductions.py:1375-1412 */
    ORK_LAST = 9,      /* last(col)              reductions.py:1415-1454 */
    ORK_MIN_ROW = 10,  /* _min_row_index()       reductions.py:2310-2372 */
    ORK_MAX_ROW = 11,  /* _max_row_index()       reductions.py:2251-2307 */
    ORK_WHERE = 12,    /* where(selector, lookup) reductions.py:1842-2166 */
    ORK_COUNT_IGNORE_AA = 13 /* _count_ignore_antialiasing(col) reductions.py:667-693 */
};

typedef struct {
    int32_t kind;
    int32_t col;         /* value column index, -1 = none */
    int32_t sel_kind;    /* WHERE: selector kind (ORK_MIN/MAX/FIRST/LAST/MIN_ROW/MAX_ROW) */
    int32_t sel_col;     /* WHERE: selector column */
    int32_t lookup_col;  /* WHERE: lookup column, -1 = row index */
    int32_t cat_col;     /* by(cat, ...): category code column, -1 = not categorical */
    int32_t ncat;        /* number of categories (1 when not categorical) */
    int32_t self_intersect; /* antialiased lines: 1 = self-intersecting variant */
    void *agg;           /* main aggregate [H][W][ncat] */
    void *agg2;          /* MEAN: uint32 counts; WHERE: selector aggregate */
} oracle_red;

/* utils.py:598-603 -- isnull(v) = not (v <= 0 or v > 0). */
static int isnull_d(double v) { return !(v <= 0.0 || v > 0.0); }

/* The aggregate dtypes follow out_dshape: count -> uint32 (float32 when
 * antialiased, reductions.py:542-543), any -> bool (float32 when
 * antialiased, :838-839), floating reductions -> float64 (:930-931),
 * row indexes and where(..., None) -> int64 (:1887-1891, :2245-2246). */

static int64_t red_cells(int64_t ncells, const oracle_red *r) {
    return ncells * (r->ncat > 0 ? r->ncat : 1);
}

static int where_lookup_is_row(const oracle_red *r) { return r->lookup_col < 0; }

static int sel_is_row(int k) { return k == ORK_MIN_ROW || k == ORK_MAX_ROW; }

/* reductions.py:397-472 -- Reduction._create_* initial values. */
void oracle_init(oracle_red *reds, int nreds, int64_t ncells, int antialias) {
    for (int r = 0; r < nreds; ++r) {
        oracle_red *rd = &reds[r];
        int64_t n = red_cells(ncells, rd);
        switch (rd->kind) {
        case ORK_COUNT:
            if (antialias) { float *a = (float *)rd->agg; for (int64_t i = 0; i < n; ++i) a[i] = NAN; }
            else memset(rd->agg, 0, (size_t)n * 4);
            break;
        case ORK_COUNT_IGNORE_AA:
            memset(rd->agg, 0, (size_t)n * 4);
            break;
        case ORK_ANY:
            if (antialias) { float *a = (float *)rd->agg; for (int64_t i = 0; i < n; ++i) a[i] = NAN; }
            else memset(rd->agg, 0, (size_t)n);
            break;
        case ORK_SUM: case ORK_MIN: case ORK_MAX: case ORK_FIRST: case ORK_LAST: {
            double *a = (double *)rd->agg; for (int64_t i = 0; i < n; ++i) a[i] = NAN; break; }
        case ORK_SUM_ZERO: memset(rd->agg, 0, (size_t)n * 8); break;
        case ORK_MEAN: memset(rd->agg, 0, (size_t)n * 8); memset(rd->agg2, 0, (size_t)n * 4); break;
        case ORK_MIN_ROW: case ORK_MAX_ROW: {
            int64_t *a = (int64_t *)rd->agg; for (int64_t i = 0; i < n; ++i) a[i] = -1; break; }
        case ORK_WHERE: {
            if (where_lookup_is_row(rd)) { int64_t *a = (int64_t *)rd->agg; for (int64_t i = 0; i < n; ++i) a[i] = -1; }
            else { double *a = (double *)rd->agg; for (int64_t i = 0; i < n; ++i) a[i] = NAN; }
            if (sel_is_row(rd->sel_kind)) { int64_t *s = (int64_t *)rd->agg2; for (int64_t i = 0; i < n; ++i) s[i] = -1; }
            else { double *s = (double *)rd->agg2; for (int64_t i = 0; i < n; ++i) s[i] = NAN; }
            break; }
        default: break;
        }
    }
}

/* ---------------------------------------------------------------------- */
/* Non-antialiased append functions (CPU forms).                           */
/* Each returns 0 when the aggregate was updated and -1 otherwise, the     */
/* return convention that where() relies on (compiler.py:400-437).         */
/* ---------------------------------------------------------------------- */

/* reductions.py:1175-1182 (min._append): strict '>' so the first row wins ties. */
static int app_min(double *agg, int64_t p, double field) {
    if (!isnull_d(field) && (isnull_d(agg[p]) || agg[p] > field)) { agg[p] = field; return 0; }
    return -1;
}
/* reductions.py:1220-1227 (max._append). */
static int app_max(double *agg, int64_t p, double field) {
    if (!isnull_d(field) && (isnull_d(agg[p]) || agg[p] < field)) { agg[p] = field; return 0; }
    return -1;
}
/* reductions.py:1398-1404 (first._append). */
static int app_first(double *agg, int64_t p, double field) {
    if (!isnull_d(field) && isnull_d(agg[p])) { agg[p] = field; return 0; }
    return -1;
}
/* reductions.py:1436-1442 (last._append). */
static int app_last(double *agg, int64_t p, double field) {
    if (!isnull_d(field)) { agg[p] = field; return 0; }
    return -1;
}
/* reductions.py:2332-2338 (_min_row_index._append). */
static int app_min_row(int64_t *agg, int64_t p, int64_t row) {
    if (row != -1 && (agg[p] == -1 || row < agg[p])) { agg[p] = row; return 0; }
    return -1;
}
/* reductions.py:2266-2272 (_max_row_index._append). */
static int app_max_row(int64_t *agg, int64_t p, int64_t row) {
    if (row > agg[p]) { agg[p] = row; return 0; }
    return -1;
}

static int app_selector(int kind, void *agg, int64_t p, double field, int64_t row) {
    switch (kind) {
    case ORK_MIN: return app_min((double *)agg, p, field);
    case ORK_MAX: return app_max((double *)agg, p, field);
    case ORK_FIRST: return app_first((double *)agg, p, field);
    case ORK_LAST: return app_last((double *)agg, p, field);
    case ORK_MIN_ROW: return app_min_row((int64_t *)agg, p, row);
    case ORK_MAX_ROW: return app_max_row((int64_t *)agg, p, row);
    default: return -1;
    }
}

static inline double colval(const double *const *cols, int c, int64_t i) { return cols[c][i]; }

/* The fused append that compiler.py:make_append (321-475) generates, for
 * one row i landing on pixel (x, y), executed for each reduction in order. */
static void append_row(oracle_red *reds, int nreds, const double *const *cols,
                       int64_t i, int64_t row, int64_t pix) {
    for (int r = 0; r < nreds; ++r) {
        oracle_red *rd = &reds[r];
        int64_t p = pix;
        if (rd->cat_col >= 0) {
            /* compiler.py:379-390: agg[:, :, int(codes[i])]; a negative code
             * indexes from the end, as numba does. */
            int64_t c = (int64_t)cols[rd->cat_col][i];
            if (c < 0) c += rd->ncat;
            if (c < 0 || c >= rd->ncat) continue;
            p = pix * rd->ncat + c;
        }
        double field = rd->col >= 0 ? colval(cols, rd->col, i) : 0.0;
        switch (rd->kind) {
        case ORK_COUNT: /* reductions.py:552-558, 580-584 */
            if (rd->col < 0 || !isnull_d(field)) ((uint32_t *)rd->agg)[p] += 1u;
            break;
        case ORK_COUNT_IGNORE_AA:
            if (!isnull_d(field)) ((uint32_t *)rd->agg)[p] += 1u;
            break;
        case ORK_ANY: /* reductions.py:842-854 */
            if (rd->col < 0 || !isnull_d(field)) ((uint8_t *)rd->agg)[p] = 1;
            break;
        case ORK_SUM: { /* reductions.py:1054-1063 */
            double *a = (double *)rd->agg;
            if (!isnull_d(field)) { if (isnull_d(a[p])) a[p] = field; else a[p] += field; }
            break; }
        case ORK_SUM_ZERO: /* reductions.py:958-963 */
            if (!isnull_d(field)) ((double *)rd->agg)[p] += field;
            break;
        case ORK_MEAN: /* bases (_sum_zero, _count_ignore_antialiasing) */
            if (!isnull_d(field)) { ((double *)rd->agg)[p] += field; ((uint32_t *)rd->agg2)[p] += 1u; }
            break;
        case ORK_MIN: app_min((double *)rd->agg, p, field); break;
        case ORK_MAX: app_max((double *)rd->agg, p, field); break;
        case ORK_FIRST: app_first((double *)rd->agg, p, field); break;
        case ORK_LAST: app_last((double *)rd->agg, p, field); break;
        case ORK_MIN_ROW: app_min_row((int64_t *)rd->agg, p, row); break;
        case ORK_MAX_ROW: app_max_row((int64_t *)rd->agg, p, row); break;
        case ORK_WHERE: {
            /* compiler.py:400-437: the selector runs first and its return
             * value gates the where append (reductions.py:1935-1941). */
            double sfield = rd->sel_col >= 0 ? colval(cols, rd->sel_col, i) : 0.0;
            int upd = app_selector(rd->sel_kind, rd->agg2, p, sfield, row);
            if (upd >= 0) {
                if (where_lookup_is_row(rd)) ((int64_t *)rd->agg)[p] = row;
                else ((double *)rd->agg)[p] = colval(cols, rd->lookup_col, i);
            }
            break; }
        default: break;
        }
    }
}

/* glyphs/points.py:190-212 -- Point._build_extend, CPU loop.
 * Bounds test, `int(x * sx + tx)` (truncation toward zero), upper-edge clamp.
 * Returns the pixel index, or -1 when the row is outside the bounds. */
static inline int64_t point_pixel(double x, double y, int32_t width, int32_t height,
                                  double sx, double tx, double sy, double ty,
                                  double xmin, double xmax, double ymin, double ymax,
                                  int32_t x_log, int32_t y_log) {
    if (!((xmin <= x && x <= xmax) && (ymin <= y && y <= ymax))) return -1;
    /* core.py:131-134 LogAxis.mapper = log10(float(val)) */
    double mx = x_log ? log10(x) : x;
    double my = y_log ? log10(y) : y;
    double fx = mx * sx;
    fx = fx + tx;
    double fy = my * sy;
    fy = fy + ty;
    int64_t xx = (int64_t)fx;  /* Python int(): truncation toward zero */
    int64_t yy = (int64_t)fy;
    int64_t xi = xx >= width ? width - 1 : xx;
    int64_t yi = yy >= height ? height - 1 : yy;
    /* numba indexes negative positions from the end. */
    if (xi < 0) xi += width;
    if (yi < 0) yi += height;
    if (xi < 0 || yi < 0) return -1;
    return yi * (int64_t)width + xi;
}

int oracle_points(int64_t n, const double *xs, const double *ys,
                  const double *const *cols, int64_t row_offset,
                  int32_t width, int32_t height,
                  double sx, double tx, double sy, double ty,
                  double xmin, double xmax, double ymin, double ymax,
                  int32_t x_log, int32_t y_log,
                  oracle_red *reds, int nreds) {
    for (int64_t i = 0; i < n; ++i) {
        const int64_t pix = point_pixel(xs[i], ys[i], width, height, sx, tx, sy, ty, xmin, xmax, ymin, ymax,
                                        x_log, y_log);
        if (pix >= 0) append_row(reds, nreds, cols, i, i + row_offset, pix);
    }
    return 0;
}

/* The same loop over float32 coordinate columns: each value is widened to
 * float64 inside the loop, where numba widens a float32 column element that
 * meets the float64 bounds and scale (glyphs/points.py:193-204). */
int oracle_points_xy32(int64_t n, const float *xs, const float *ys,
                       const double *const *cols, int64_t row_offset,
                       int32_t width, int32_t height,
                       double sx, double tx, double sy, double ty,
                       double xmin, double xmax, double ymin, double ymax,
                       int32_t x_log, int32_t y_log,
                       oracle_red *reds, int nreds) {
    for (int64_t i = 0; i < n; ++i) {
        const int64_t pix = point_pixel((double)xs[i], (double)ys[i], width, height, sx, tx, sy, ty,
                                        xmin, xmax, ymin, ymax, x_log, y_log);
        if (pix >= 0) append_row(reds, nreds, cols, i, i + row_offset, pix);
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* LineAxis0: glyphs/line.py                                               */
/* ---------------------------------------------------------------------- */

/* Antialiased append functions (CPU forms).  aa = aa_factor, pa = prev_aa_factor. */
static void append_row_aa(oracle_red *reds, int nreds, const double *const *cols,
                          int64_t i, int64_t row, int64_t pix, double aa, double pa) {
    for (int r = 0; r < nreds; ++r) {
        oracle_red *rd = &reds[r];
        int64_t p = pix;
        if (rd->cat_col >= 0) {
            int64_t c = (int64_t)cols[rd->cat_col][i];
            if (c < 0) c += rd->ncat;
            if (c < 0 || c >= rd->ncat) continue;
            p = pix * rd->ncat + c;
        }
        double field = rd->col >= 0 ? colval(cols, rd->col, i) : 0.0;
        int has = (rd->col < 0) || !isnull_d(field);
        switch (rd->kind) {
        case ORK_COUNT: {
            float *a = (float *)rd->agg;
            if (!has) break;
            if (rd->self_intersect) {
                /* reductions.py:560-569, 586-592: float32 aggregate, the
                 * increment is computed in float64 then stored as float32. */
                double d = aa - pa;
                if (isnull_d((double)a[p])) a[p] = (float)d;
                else a[p] = (float)((double)a[p] + d);
            } else {
                /* reductions.py:571-577, 594-599 */
                if (isnull_d((double)a[p]) || aa > (double)a[p]) a[p] = (float)aa;
            }
            break; }
        case ORK_COUNT_IGNORE_AA: /* reductions.py:680-693 */
            if (!isnull_d(field) && pa == 0.0) ((uint32_t *)rd->agg)[p] += 1u;
            break;
        case ORK_ANY: { /* reductions.py:848-852, 860-864 */
            float *a = (float *)rd->agg;
            if (has && (isnull_d((double)a[p]) || aa > (double)a[p])) a[p] = (float)aa;
            break; }
        case ORK_SUM: {
            double *a = (double *)rd->agg;
            if (rd->self_intersect) { /* reductions.py:1065-1075 */
                double value = field * (aa - pa);
                if (!isnull_d(value)) { if (isnull_d(a[p])) a[p] = value; else a[p] += value; }
            } else { /* reductions.py:1077-1084 */
                double value = field * aa;
                if (!isnull_d(value) && (isnull_d(a[p]) || value > a[p])) a[p] = value;
            }
            break; }
        case ORK_SUM_ZERO: { /* reductions.py:966-973 */
            double value = field * (aa - pa);
            if (!isnull_d(value)) ((double *)rd->agg)[p] += value;
            break; }
        case ORK_MEAN: {
            double value = field * (aa - pa);
            if (!isnull_d(value)) ((double *)rd->agg)[p] += value;
            if (!isnull_d(field) && pa == 0.0) ((uint32_t *)rd->agg2)[p] += 1u;
            break; }
        case ORK_MIN: case ORK_MAX: case ORK_FIRST: case ORK_LAST: {
            /* reductions.py:1186-1192, 1231-1237, 1406-1412, 1444-1450:
             * every antialiased form keeps the largest field*aa_factor. */
            double *a = (double *)rd->agg;
            double value = field * aa;
            if (!isnull_d(value) && (isnull_d(a[p]) || value > a[p])) a[p] = value;
            break; }
        case ORK_MIN_ROW: app_min_row((int64_t *)rd->agg, p, row); break; /* :2340-2346 */
        case ORK_MAX_ROW: app_max_row((int64_t *)rd->agg, p, row); break; /* :2274-2281 */
        case ORK_WHERE: {
            /* reductions.py:1943-1950: where ignores aa_factor; its selector
             * uses its antialiased append and gates the write. */
            int upd = -1;
            if (sel_is_row(rd->sel_kind)) {
                upd = app_selector(rd->sel_kind, rd->agg2, p, 0.0, row);
            } else {
                double sfield = colval(cols, rd->sel_col, i);
                double value = sfield * aa;
                double *s = (double *)rd->agg2;
                if (!isnull_d(value) && (isnull_d(s[p]) || value > s[p])) { s[p] = value; upd = 0; }
            }
            if (upd >= 0) {
                if (where_lookup_is_row(rd)) ((int64_t *)rd->agg)[p] = row;
                else ((double *)rd->agg)[p] = colval(cols, rd->lookup_col, i);
            }
            break; }
        default: break;
        }
    }
}

static void append_any(oracle_red *reds, int nreds, const double *const *cols, int64_t i,
                       int64_t row, int64_t x, int64_t y, int32_t width, int antialias,
                       double aa, double pa) {
    int64_t pix = y * (int64_t)width + x;
    if (antialias) append_row_aa(reds, nreds, cols, i, row, pix, aa, pa);
    else append_row(reds, nreds, cols, i, row, pix);
}

/* line.py:783-800 */
static int clipt(double p, double q, double *t0, double *t1) {
    int accept = 1;
    if (p < 0 && q < 0) {
        double r = q / p;
        if (r > *t1) accept = 0;
        else if (r > *t0) *t0 = r;
    } else if (p > 0 && q < p) {
        double r = q / p;
        if (r < *t0) accept = 0;
        else if (r < *t1) *t1 = r;
    } else if (q < 0) {
        accept = 0;
    }
    return accept;
}

/* line.py:734-780 -- Liang-Barsky clipping. */
static void liang_barsky(double xmin, double xmax, double ymin, double ymax,
                         double *x0, double *x1, double *y0, double *y1, int *skip,
                         int *clipped_start, int *clipped_end) {
    if (*x0 < xmin && *x1 < xmin) *skip = 1;
    else if (*x0 > xmax && *x1 > xmax) *skip = 1;
    else if (*y0 < ymin && *y1 < ymin) *skip = 1;
    else if (*y0 > ymax && *y1 > ymax) *skip = 1;
    double t0 = 0, t1 = 1;
    double dx1 = *x1 - *x0;
    if (!clipt(-dx1, *x0 - xmin, &t0, &t1)) *skip = 1;
    if (!clipt(dx1, xmax - *x0, &t0, &t1)) *skip = 1;
    double dy1 = *y1 - *y0;
    if (!clipt(-dy1, *y0 - ymin, &t0, &t1)) *skip = 1;
    if (!clipt(dy1, ymax - *y0, &t0, &t1)) *skip = 1;
    if (t1 < 1) {
        *clipped_end = 1;
        *x1 = *x0 + t1 * dx1;
        *y1 = *y0 + t1 * dy1;
    } else *clipped_end = 0;
    if (t0 > 0) {
        *clipped_start = 1;
        *x0 = *x0 + t0 * dx1;
        *y0 = *y0 + t0 * dy1;
    } else *clipped_start = 0;
}

static double pyround(double v) { return nearbyint(v); } /* round-half-even, like Python round() */

static double clampd(double x, double lo, double hi) { double m = x < hi ? x : hi; return lo > m ? lo : m; }
static int64_t clampi(int64_t x, int64_t lo, int64_t hi) { int64_t m = x < hi ? x : hi; return lo > m ? lo : m; }

/* line.py:808-811 */
static double linearstep(double e0, double e1, double x) { return clampd((x - e0) / (e1 - e0), 0.0, 1.0); }

/* line.py:814-821 */
static double x_intercept(double y, double cx0, double cy0, double cx1, double cy1) {
    if (cy0 == cy1) return cx1;
    double frac = (y - cy0) / (cy1 - cy0);
    return cx0 + frac * (cx1 - cx0);
}

static double sq(double v) { return v * v; }

/* line.py:826-981 -- _full_antialias, the antialiased wide-line scan conversion. */
static void full_antialias(double line_width, int overwrite, int64_t i, int64_t row,
                           double x0, double x1, double y0, double y1,
                           int segment_start, int segment_end, double xm, double ym,
                           int64_t nx, int64_t ny, int32_t width,
                           oracle_red *reds, int nreds, const double *const *cols) {
    if (x0 == x1 && y0 == y1) return;
    int flip_xy = fabs(x0 - x1) < fabs(y0 - y1);
    if (flip_xy) {
        double t;
        t = x0; x0 = y0; y0 = t;
        t = x1; x1 = y1; y1 = t;
        t = xm; xm = ym; ym = t;
    }
    double scale = 1.0;
    if (line_width < 1.0) { scale *= line_width; line_width = 1.0; }
    double aa = 1.0;
    double halfwidth = 0.5 * (line_width + aa);
    int flip_order = y1 < y0 || (y1 == y0 && x1 < x0);
    double alongx = x1 - x0;
    double alongy = y1 - y0;
    double length = sqrt(sq(alongx) + sq(alongy));
    alongx /= length;
    alongy /= length;
    double rightx = alongy;
    double righty = -alongx;
    double b[8];
    if (flip_order) {
        b[0] = x1 - halfwidth * (rightx - alongx);
        b[1] = x1 - halfwidth * (-rightx - alongx);
        b[2] = x0 - halfwidth * (-rightx + alongx);
        b[3] = x0 - halfwidth * (rightx + alongx);
        b[4] = y1 - halfwidth * (righty - alongy);
        b[5] = y1 - halfwidth * (-righty - alongy);
        b[6] = y0 - halfwidth * (-righty + alongy);
        b[7] = y0 - halfwidth * (righty + alongy);
    } else {
        b[0] = x0 + halfwidth * (rightx - alongx);
        b[1] = x0 + halfwidth * (-rightx - alongx);
        b[2] = x1 + halfwidth * (-rightx + alongx);
        b[3] = x1 + halfwidth * (rightx + alongx);
        b[4] = y0 + halfwidth * (righty - alongy);
        b[5] = y0 + halfwidth * (-righty - alongy);
        b[6] = y1 + halfwidth * (-righty + alongy);
        b[7] = y1 + halfwidth * (righty + alongy);
    }
    int64_t xmaxi = nx - 1, ymaxi = ny - 1;
    if (flip_xy) { int64_t t = xmaxi; xmaxi = ymaxi; ymaxi = t; }
    int lowindex = flip_order ? (x0 > x1 ? 0 : 1) : (x1 > x0 ? 0 : 1);
    double prev_alongx = 0, prev_alongy = 0, prev_length = 0, prev_rightx = 0, prev_righty = 0;
    if (!overwrite && !segment_start) {
        prev_alongx = x0 - xm;
        prev_alongy = y0 - ym;
        prev_length = sqrt(sq(prev_alongx) + sq(prev_alongy));
        if (prev_length > 0.0) {
            prev_alongx /= prev_length;
            prev_alongy /= prev_length;
            prev_rightx = prev_alongy;
            prev_righty = -prev_alongx;
        } else {
            overwrite = 1;
        }
    }
    int64_t ystart = clampi((int64_t)ceil(b[4 + lowindex]), 0, ymaxi);
    int64_t yend = clampi((int64_t)floor(b[4 + (lowindex + 2) % 4]), 0, ymaxi);
    int ll = lowindex, lu = (ll + 1) % 4, rl = lowindex, ru = (rl + 3) % 4;
    double lw_lo = 0.5 * (line_width - aa);
    for (int64_t y = ystart; y <= yend; ++y) {
        double yd = (double)y;
        if (ll == lowindex && yd > b[4 + lu]) { ll = lu; lu = (ll + 1) % 4; }
        if (rl == lowindex && yd > b[4 + ru]) { rl = ru; ru = (rl + 3) % 4; }
        int64_t xleft = clampi((int64_t)ceil(x_intercept(yd, b[ll], b[4 + ll], b[lu], b[4 + lu])), 0, xmaxi);
        int64_t xright = clampi((int64_t)floor(x_intercept(yd, b[rl], b[4 + rl], b[ru], b[4 + ru])), 0, xmaxi);
        for (int64_t x = xleft; x <= xright; ++x) {
            double xd = (double)x;
            double along = (xd - x0) * alongx + (yd - y0) * alongy;
            int prev_correction = 0;
            double distance;
            if (along < 0.0) {
                if (overwrite || segment_start || (xd - x0) * prev_alongx + (yd - y0) * prev_alongy > 0.0)
                    distance = sqrt(sq(xd - x0) + sq(yd - y0));
                else continue;
            } else if (along > length) {
                if (overwrite || segment_end) distance = sqrt(sq(xd - x1) + sq(yd - y1));
                else continue;
            } else {
                distance = fabs((xd - x0) * rightx + (yd - y0) * righty);
                if (!overwrite && !segment_start) {
                    double pd = (xd - x0) * prev_alongx + (yd - y0) * prev_alongy;
                    if (-prev_length <= pd && pd <= 0.0 &&
                        fabs((xd - x0) * prev_rightx + (yd - y0) * prev_righty) <= halfwidth)
                        prev_correction = 1;
                }
            }
            double value = 1.0 - linearstep(lw_lo, halfwidth, distance);
            value *= scale;
            double prev_value = 0.0;
            if (prev_correction) {
                double prev_distance = fabs((xd - x0) * prev_rightx + (yd - y0) * prev_righty);
                prev_value = 1.0 - linearstep(lw_lo, halfwidth, prev_distance);
                prev_value *= scale;
                if (value <= prev_value) value = 0.0;
            }
            if (value > 0.0) {
                int64_t xx = flip_xy ? y : x;
                int64_t yy = flip_xy ? x : y;
                append_any(reds, nreds, cols, i, row, xx, yy, width, 1, value, prev_value);
            }
        }
    }
}

/* line.py:986-1031 -- integer Bresenham. */
static void bresenham(int64_t i, int64_t row, int segment_start, int64_t x0, int64_t x1,
                      int64_t y0, int64_t y1, int clipped, int32_t width,
                      oracle_red *reds, int nreds, const double *const *cols) {
    int64_t dx = x1 - x0;
    int64_t ix = (dx > 0) - (dx < 0);
    dx = (dx < 0 ? -dx : dx) * 2;
    int64_t dy = y1 - y0;
    int64_t iy = (dy > 0) - (dy < 0);
    dy = (dy < 0 ? -dy : dy) * 2;
    if (!clipped && !(dx | dy)) {
        append_any(reds, nreds, cols, i, row, x0, y0, width, 0, 0, 0);
        return;
    }
    if (segment_start) append_any(reds, nreds, cols, i, row, x0, y0, width, 0, 0, 0);
    if (dx >= dy) {
        int64_t error = 2 * dy - dx;
        while (x0 != x1) {
            if (error >= 0 && (error || ix > 0)) { error -= 2 * dx; y0 += iy; }
            error += 2 * dy;
            x0 += ix;
            append_any(reds, nreds, cols, i, row, x0, y0, width, 0, 0, 0);
        }
    } else {
        int64_t error = 2 * dx - dy;
        while (y0 != y1) {
            if (error >= 0 && (error || iy > 0)) { error -= 2 * dy; x0 += ix; }
            error += 2 * dx;
            y0 += iy;
            append_any(reds, nreds, cols, i, row, x0, y0, width, 0, 0, 0);
        }
    }
}

/* line.py:688-721 -- map_onto_pixel_snap. */
static void map_snap(double sx, double tx, double sy, double ty, double xmax, double ymax,
                     double x, double y, int64_t *xo, int64_t *yo) {
    double fx = x * sx; fx = fx + tx;
    double fy = y * sy; fy = fy + ty;
    int64_t xx = (int64_t)fx, yy = (int64_t)fy;
    double gx = xmax * sx; gx = gx + tx;
    double gy = ymax * sy; gy = gy + ty;
    int64_t xxmax = (int64_t)pyround(gx), yymax = (int64_t)pyround(gy);
    *xo = xx == xxmax ? xx - 1 : xx;
    *yo = yy == yymax ? yy - 1 : yy;
}

/* line.py:723-726 -- map_onto_pixel_no_snap. */
static void map_no_snap(double sx, double tx, double sy, double ty, double x, double y,
                        double *xo, double *yo) {
    double fx = x * sx; fx = fx + tx; fx = fx - 0.5;
    double fy = y * sy; fy = fy + ty; fy = fy - 0.5;
    *xo = fx; *yo = fy;
}

/* line.py:1033-1097 (draw_segment) driven by line.py:1099-1136
 * (_build_extend_line_axis0: perform_extend_line + extend_cpu). */
/* line.py:1033-1097 -- _build_draw_segment: clip, map, AA or Bresenham for
 * one segment whose appends use row i. */
static void draw_segment(int64_t i, int64_t row_offset, double x0, double y0, double x1, double y1,
                         int segment_start, int segment_end, double xm, double ym,
                         const double *const *cols, int32_t width,
                         double sx, double tx, double sy, double ty,
                         double xmin, double xmax, double ymin, double ymax,
                         double line_width, int32_t overwrite, oracle_red *reds, int nreds) {
    int antialias = line_width > 0.0;
    int skip = 0;
    if (isnull_d(x0) || isnull_d(y0) || isnull_d(x1) || isnull_d(y1)) skip = 1;
    int clipped_start = 0, clipped_end = 0;
    liang_barsky(xmin, xmax, ymin, ymax, &x0, &x1, &y0, &y1, &skip, &clipped_start, &clipped_end);
    if (skip) return;
    int clipped = clipped_start || clipped_end;
    segment_start = segment_start || clipped_start;
    if (antialias) {
        double px0, py0, px1, py1, pxm, pym;
        map_no_snap(sx, tx, sy, ty, x0, y0, &px0, &py0);
        map_no_snap(sx, tx, sy, ty, x1, y1, &px1, &py1);
        if (segment_start) { pxm = 0.0; pym = 0.0; }
        else map_no_snap(sx, tx, sy, ty, xm, ym, &pxm, &pym);
        double gx = (xmax - xmin) * sx, gy = (ymax - ymin) * sy;
        int64_t nx = (int64_t)pyround(gx), ny = (int64_t)pyround(gy);
        full_antialias(line_width, overwrite, i, i + row_offset, px0, px1, py0, py1,
                       segment_start, segment_end, pxm, pym, nx, ny, width,
                       reds, nreds, cols);
    } else {
        int64_t ix0, iy0, ix1, iy1;
        map_snap(sx, tx, sy, ty, xmax, ymax, x0, y0, &ix0, &iy0);
        map_snap(sx, tx, sy, ty, xmax, ymax, x1, y1, &ix1, &iy1);
        bresenham(i, i + row_offset, segment_start, ix0, ix1, iy0, iy1, clipped, width,
                  reds, nreds, cols);
    }
}

int oracle_line_axis0(int64_t n, const double *xs, const double *ys,
                      const double *const *cols, int64_t row_offset,
                      int32_t width, int32_t height,
                      double sx, double tx, double sy, double ty,
                      double xmin, double xmax, double ymin, double ymax,
                      double line_width, int32_t plot_start,
                      int32_t overwrite, int32_t use_2_stage_agg,
                      oracle_red *reds, int nreds) {
    for (int64_t i = 0; i + 1 < n; ++i) {
        /* xs[i - 1] with numba's wrap of index -1 onto the last row */
        const int64_t im = i > 0 ? i - 1 : n - 1;
        int segment_start = (i == 0) ? plot_start : (isnull_d(xs[im]) || isnull_d(ys[im]));
        int segment_end = (i == n - 2) || isnull_d(xs[i + 2]) || isnull_d(ys[i + 2]);
        double xm, ym;
        if (segment_start || use_2_stage_agg) { xm = 0.0; ym = 0.0; }
        else { xm = xs[im]; ym = ys[im]; }
        draw_segment(i, row_offset, xs[i], ys[i], xs[i + 1], ys[i + 1], segment_start, segment_end, xm, ym,
                     cols, width, sx, tx, sy, ty, xmin, xmax, ymin, ymax, line_width, overwrite, reds, nreds);
    }
    (void)height;
    return 0;
}

/* Multi-line layouts, in the reference's iteration order:
 *   layout 1, LineAxis0Multi (line.py:1152-1200): xs, ys [nrows][nv], column
 *       j outer, row i inner;
 *   layout 2, LinesAxis1 / XConstant / YConstant (line.py:1244-1437): row i
 *       outer, column j inner, vertex (xs[i*xrow + j], ys[i*yrow + j]). */
int oracle_lines(int32_t layout, int64_t nrows, int64_t nv, const double *xs, const double *ys,
                 int64_t xrow, int64_t yrow, const double *const *cols, int64_t row_offset,
                 int32_t width, int32_t height, double sx, double tx, double sy, double ty,
                 double xmin, double xmax, double ymin, double ymax,
                 double line_width, int32_t plot_start, int32_t overwrite, oracle_red *reds, int nreds) {
    if (layout == 1) {
        for (int64_t j = 0; j < nv; ++j) {
            for (int64_t i = 0; i + 1 < nrows; ++i) {
                const int64_t im = i > 0 ? i - 1 : nrows - 1;
#define XA(r) xs[(r) * nv + j]
#define YA(r) ys[(r) * nv + j]
                int segment_start = (i == 0) ? plot_start : (isnull_d(XA(im)) || isnull_d(YA(im)));
                int segment_end = (i == nrows - 2) || isnull_d(XA(i + 2)) || isnull_d(YA(i + 2));
                double xm = 0.0, ym = 0.0;
                if (!segment_start) { xm = XA(im); ym = YA(im); }
                draw_segment(i, row_offset, XA(i), YA(i), XA(i + 1), YA(i + 1), segment_start, segment_end,
                             xm, ym, cols, width, sx, tx, sy, ty, xmin, xmax, ymin, ymax, line_width, overwrite,
                             reds, nreds);
#undef XA
#undef YA
            }
        }
    } else {
        for (int64_t i = 0; i < nrows; ++i) {
            const double *X = xs + i * xrow, *Y = ys + i * yrow;
            for (int64_t j = 0; j + 1 < nv; ++j) {
                int segment_start = (j == 0) || isnull_d(X[j - 1]) || isnull_d(Y[j - 1]);
                int segment_end = (j == nv - 2) || isnull_d(X[j + 2]) || isnull_d(Y[j + 2]);
                double xm = 0.0, ym = 0.0;
                if (!segment_start) { xm = X[j - 1]; ym = Y[j - 1]; }
                draw_segment(i, row_offset, X[j], Y[j], X[j + 1], Y[j + 1], segment_start, segment_end, xm, ym,
                             cols, width, sx, tx, sy, ty, xmin, xmax, ymin, ymax, line_width, overwrite,
                             reds, nreds);
            }
        }
    }
    (void)height;
    return 0;
}

/* ---------------------------------------------------------------------- */
/* Two-stage antialiased plans over several lines (cpu_antialias_2agg_impl,  */
/* line.py:1203-1226 for LineAxis0Multi, :1300-1318 and siblings for the     */
/* LinesAxis1 family): each line is drawn alone into freshly initialised     */
/* aggregates (every stage-2 zero equals the create() value), then folded   */
/* into the accumulators with the reduction's stage-2 combination           */
/* (compiler.py:198-268); a plan over one line keeps the drawn aggregates.  */
/* ---------------------------------------------------------------------- */

static void draw_one_line(int32_t layout, int64_t L, int64_t nrows, int64_t nv, const double *xs, const double *ys,
                          int64_t xrow, int64_t yrow, const double *const *cols, int64_t row_offset, int32_t width,
                          double sx, double tx, double sy, double ty, double xmin, double xmax, double ymin,
                          double ymax, double line_width, int32_t plot_start, int32_t overwrite,
                          oracle_red *reds, int nreds) {
    if (layout == 1) {
        const int64_t j = L;
        for (int64_t i = 0; i + 1 < nrows; ++i) {
            const int64_t im = i > 0 ? i - 1 : nrows - 1;
#define XA(r) xs[(r) * nv + j]
#define YA(r) ys[(r) * nv + j]
            int segment_start = (i == 0) ? plot_start : (isnull_d(XA(im)) || isnull_d(YA(im)));
            int segment_end = (i == nrows - 2) || isnull_d(XA(i + 2)) || isnull_d(YA(i + 2));
            draw_segment(i, row_offset, XA(i), YA(i), XA(i + 1), YA(i + 1), segment_start, segment_end,
                         0.0, 0.0, cols, width, sx, tx, sy, ty, xmin, xmax, ymin, ymax, line_width, overwrite,
                         reds, nreds);
#undef XA
#undef YA
        }
    } else {
        const int64_t i = L;
        const double *X = xs + i * xrow, *Y = ys + i * yrow;
        for (int64_t j = 0; j + 1 < nv; ++j) {
            int segment_start = (j == 0) || isnull_d(X[j - 1]) || isnull_d(Y[j - 1]);
            int segment_end = (j == nv - 2) || isnull_d(X[j + 2]) || isnull_d(Y[j + 2]);
            draw_segment(i, row_offset, X[j], Y[j], X[j + 1], Y[j + 1], segment_start, segment_end, 0.0, 0.0,
                         cols, width, sx, tx, sy, ty, xmin, xmax, ymin, ymax, line_width, overwrite, reds, nreds);
        }
    }
}

static size_t stage2_elem(int kind) {
    switch (kind) {
    case ORK_COUNT: case ORK_ANY: case ORK_COUNT_IGNORE_AA: return 4;   /* float32 / uint32 */
    case ORK_SUM: case ORK_MIN: case ORK_MAX: case ORK_FIRST: case ORK_LAST:
    case ORK_MIN_ROW: case ORK_MAX_ROW: case ORK_SUM_ZERO: case ORK_MEAN: case ORK_WHERE: return 8;
    default: return 0;                                      /* no stage-2 fold restated here */
    }
}
/* The second aggregate: MEAN's uint32 counts, WHERE's selector (float64 or int64) */
static size_t stage2_elem2(int kind) { return kind == ORK_MEAN ? 4 : kind == ORK_WHERE ? 8 : 0; }

/* where's stage-2 combine (reductions.py:1992-2018, combine_cpu_2d): the other
 * line's selector value, when valid, is offered to the accumulated selector
 * through the selector's own (non-antialiased) append, and where that append
 * updates, the other line's where value is taken. */
static void stage2_fold_where(const oracle_red *rd, void *ret, void *ret_sel, const void *other,
                              const void *other_sel, int64_t n) {
    const int k = rd->sel_kind;
    const int row_sel = sel_is_row(k);
    for (int64_t c = 0; c < n; ++c) {
        int take = 0;
        if (row_sel) {
            int64_t *a = (int64_t *)ret_sel;
            const int64_t v = ((const int64_t *)other_sel)[c];
            if (v == -1) continue;
            take = app_selector(k, a, c, 0.0, v) >= 0;
        } else {
            double *a = (double *)ret_sel;
            const double v = ((const double *)other_sel)[c];
            if (isnull_d(v)) continue;
            take = app_selector(k, a, c, v, 0) >= 0;
        }
        if (take) ((int64_t *)ret)[c] = ((const int64_t *)other)[c];   /* 8-byte where value, row or float64 */
    }
}

/* ret <- combine(ret, other): nansum_in_place (utils.py:885-897, float32 for the
 * float32 count), nanmax_in_place / nanmin_in_place (:639-668),
 * nanfirst_in_place / nanlast_in_place (:615-636), row_max_in_place /
 * row_min_in_place (:901-923).  count and sum fold with SUM_2AGG, any and max
 * with MAX, min with MIN, first / last with FIRST / LAST, the row indexes with
 * MIN / MAX over -1 (reductions.py:545-549, 1040-1045, 837, 1173, 1218, 1396,
 * 1434, 2257, 2311). */
static void stage2_fold(int kind, void *ret, const void *other, int64_t n) {
    if (kind == ORK_COUNT_IGNORE_AA) {
        /* SUM_2AGG over zero-initialised uint32 counts (reductions.py:673-677) */
        uint32_t *r = (uint32_t *)ret;
        const uint32_t *o = (const uint32_t *)other;
        for (int64_t k = 0; k < n; ++k) r[k] += o[k];
        return;
    }
    if (kind == ORK_SUM_ZERO || kind == ORK_MEAN) {
        /* SUM_2AGG over zero-initialised float64 sums (reductions.py:944-948); no NaN
         * reaches them, so nansum_in_place is the plain sum */
        double *r = (double *)ret;
        const double *o = (const double *)other;
        for (int64_t k = 0; k < n; ++k) r[k] = r[k] + o[k];
        return;
    }
    if (kind == ORK_COUNT || kind == ORK_ANY) {
        float *r = (float *)ret;
        const float *o = (const float *)other;
        for (int64_t k = 0; k < n; ++k) {
            const float a = r[k], b = o[k];
            const int an = !(a <= 0.0f || a > 0.0f), bn = !(b <= 0.0f || b > 0.0f);
            if (kind == ORK_COUNT) {
                if (an) { if (!bn) r[k] = b; }
                else if (!bn) r[k] = a + b;
            } else {
                if (an) { if (!bn) r[k] = b; }
                else if (!bn && b > a) r[k] = b;
            }
        }
    } else if (kind == ORK_MIN_ROW || kind == ORK_MAX_ROW) {
        int64_t *r = (int64_t *)ret;
        const int64_t *o = (const int64_t *)other;
        for (int64_t k = 0; k < n; ++k)
            if (o[k] > -1 && (r[k] == -1 || (kind == ORK_MIN_ROW ? o[k] < r[k] : o[k] > r[k]))) r[k] = o[k];
    } else {
        double *r = (double *)ret;
        const double *o = (const double *)other;
        for (int64_t k = 0; k < n; ++k) {
            const double a = r[k], b = o[k];
            const int an = isnull_d(a), bn = isnull_d(b);
            switch (kind) {
            case ORK_SUM: if (an) { if (!bn) r[k] = b; } else if (!bn) r[k] = a + b; break;
            case ORK_MAX: if (an) { if (!bn) r[k] = b; } else if (!bn && b > a) r[k] = b; break;
            case ORK_MIN: if (an) { if (!bn) r[k] = b; } else if (!bn && b < a) r[k] = b; break;
            case ORK_FIRST: if (an && !bn) r[k] = b; break;
            case ORK_LAST: if (!bn) r[k] = b; break;
            default: break;
            }
        }
    }
}

/* The stage-2 driver shared by every two-stage loop: draw line L into the
 * aggregates (initialised by the caller for L = 0, re-initialised here after),
 * copy them on the first pass and fold them afterwards, then copy back.
 * Returns 0, or -2 when a reduction has no stage-2 fold restated here. */
typedef void (*draw_line_fn)(const void *ctx, int64_t L, oracle_red *reds, int nreds);

static int run_two_stage(int64_t nlines, int64_t ncells, draw_line_fn draw, const void *ctx,
                         oracle_red *reds, int nreds) {
    for (int r = 0; r < nreds; ++r)
        if (stage2_elem(reds[r].kind) == 0) return -2;
    void *acc[64], *acc2[64];
    if (nreds > 64) return -2;
    for (int r = 0; r < nreds; ++r) { acc[r] = NULL; acc2[r] = NULL; }
    for (int64_t L = 0; L < nlines; ++L) {
        if (L > 0) oracle_init(reds, nreds, ncells, 1);
        draw(ctx, L, reds, nreds);
        if (nlines == 1) return 0;
        for (int r = 0; r < nreds; ++r) {
            const int64_t n = red_cells(ncells, &reds[r]);
            const size_t bytes = (size_t)n * stage2_elem(reds[r].kind);
            const size_t bytes2 = (size_t)n * stage2_elem2(reds[r].kind);
            if (L == 0) {
                acc[r] = malloc(bytes ? bytes : 1);
                memcpy(acc[r], reds[r].agg, bytes);
                if (bytes2) { acc2[r] = malloc(bytes2); memcpy(acc2[r], reds[r].agg2, bytes2); }
            } else if (reds[r].kind == ORK_WHERE) {
                stage2_fold_where(&reds[r], acc[r], acc2[r], reds[r].agg, reds[r].agg2, n);
            } else {
                stage2_fold(reds[r].kind, acc[r], reds[r].agg, n);
                if (bytes2) stage2_fold(ORK_COUNT_IGNORE_AA, acc2[r], reds[r].agg2, n);
            }
        }
    }
    for (int r = 0; r < nreds && nlines > 1; ++r) {
        const int64_t n = red_cells(ncells, &reds[r]);
        memcpy(reds[r].agg, acc[r], (size_t)n * stage2_elem(reds[r].kind));
        free(acc[r]);
        if (acc2[r]) { memcpy(reds[r].agg2, acc2[r], (size_t)n * stage2_elem2(reds[r].kind)); free(acc2[r]); }
    }
    return 0;
}

typedef struct {
    int32_t layout; int64_t nrows, nv; const double *xs, *ys; int64_t xrow, yrow;
    const double *const *cols; int64_t row_offset; int32_t width;
    double sx, tx, sy, ty, xmin, xmax, ymin, ymax, line_width; int32_t plot_start, overwrite;
} multi_ctx;

static void draw_multi(const void *c, int64_t L, oracle_red *reds, int nreds) {
    const multi_ctx *m = (const multi_ctx *)c;
    draw_one_line(m->layout, L, m->nrows, m->nv, m->xs, m->ys, m->xrow, m->yrow, m->cols, m->row_offset, m->width,
                  m->sx, m->tx, m->sy, m->ty, m->xmin, m->xmax, m->ymin, m->ymax, m->line_width, m->plot_start,
                  m->overwrite, reds, nreds);
}

int oracle_lines_2stage(int32_t layout, int64_t nrows, int64_t nv, const double *xs, const double *ys,
                        int64_t xrow, int64_t yrow, const double *const *cols, int64_t row_offset,
                        int32_t width, int32_t height, double sx, double tx, double sy, double ty,
                        double xmin, double xmax, double ymin, double ymax,
                        double line_width, int32_t plot_start, int32_t overwrite, oracle_red *reds, int nreds) {
    const multi_ctx m = {layout, nrows, nv, xs, ys, xrow, yrow, cols, row_offset, width,
                         sx, tx, sy, ty, xmin, xmax, ymin, ymax, line_width, plot_start, overwrite};
    return run_two_stage(layout == 1 ? nv : nrows, (int64_t)width * height, draw_multi, &m, reds, nreds);
}

/* line.py:1538-1612 -- LinesAxis1Ragged (_build_extend_line_axis1_ragged,
 * single-stage form): row i runs over its own slices of the flat x and y
 * arrays (start indices; the last row ends at the flat length), through
 * the shorter of the two; segment j appends row i. */
typedef struct {
    int64_t nrows; const double *xf; int64_t nx; const int64_t *xstart; const double *yf; int64_t ny;
    const int64_t *ystart; const double *const *cols; int64_t row_offset; int32_t width;
    double sx, tx, sy, ty, xmin, xmax, ymin, ymax, line_width; int32_t overwrite, two_stage;
} ragged_ctx;

/* one ragged row: its slices of the flat arrays, through the shorter of the two;
 * the two-stage form never reads the previous vertex (line.py:1662-1684) */
static void draw_ragged_row(const void *c, int64_t i, oracle_red *reds, int nreds) {
    const ragged_ctx *g = (const ragged_ctx *)c;
    const int64_t x0i = g->xstart[i], x1i = i < g->nrows - 1 ? g->xstart[i + 1] : g->nx;
    const int64_t y0i = g->ystart[i], y1i = i < g->nrows - 1 ? g->ystart[i + 1] : g->ny;
    const int64_t len = (x1i - x0i) < (y1i - y0i) ? (x1i - x0i) : (y1i - y0i);
    const double *X = g->xf + x0i, *Y = g->yf + y0i;
    for (int64_t j = 0; j + 1 < len; ++j) {
        int segment_start = (j == 0) || isnull_d(X[j - 1]) || isnull_d(Y[j - 1]);
        int segment_end = (j == len - 2) || isnull_d(X[j + 2]) || isnull_d(Y[j + 2]);
        double xm = 0.0, ym = 0.0;
        if (!segment_start && !g->two_stage) { xm = X[j - 1]; ym = Y[j - 1]; }
        draw_segment(i, g->row_offset, X[j], Y[j], X[j + 1], Y[j + 1], segment_start, segment_end, xm, ym,
                     g->cols, g->width, g->sx, g->tx, g->sy, g->ty, g->xmin, g->xmax, g->ymin, g->ymax,
                     g->line_width, g->overwrite, reds, nreds);
    }
}

int oracle_lines_ragged(int64_t nrows, const double *xf, int64_t nx, const int64_t *xstart,
                        const double *yf, int64_t ny, const int64_t *ystart,
                        const double *const *cols, int64_t row_offset,
                        int32_t width, int32_t height, double sx, double tx, double sy, double ty,
                        double xmin, double xmax, double ymin, double ymax,
                        double line_width, int32_t overwrite, oracle_red *reds, int nreds) {
    const ragged_ctx g = {nrows, xf, nx, xstart, yf, ny, ystart, cols, row_offset, width,
                          sx, tx, sy, ty, xmin, xmax, ymin, ymax, line_width, overwrite, 0};
    for (int64_t i = 0; i < nrows; ++i) draw_ragged_row(&g, i, reds, nreds);
    (void)height;
    return 0;
}

/* line.py:1616-1693 -- the two-stage ragged loop: one row at a time, folded. */
int oracle_lines_ragged_2stage(int64_t nrows, const double *xf, int64_t nx, const int64_t *xstart,
                               const double *yf, int64_t ny, const int64_t *ystart,
                               const double *const *cols, int64_t row_offset,
                               int32_t width, int32_t height, double sx, double tx, double sy, double ty,
                               double xmin, double xmax, double ymin, double ymax,
                               double line_width, int32_t overwrite, oracle_red *reds, int nreds) {
    const ragged_ctx g = {nrows, xf, nx, xstart, yf, ny, ystart, cols, row_offset, width,
                          sx, tx, sy, ty, xmin, xmax, ymin, ymax, line_width, overwrite, 1};
    return run_two_stage(nrows, (int64_t)width * height, draw_ragged_row, &g, reds, nreds);
}

/* glyph.py:66-78 -- _compute_bounds_numba: NaN-skipping min/max. */
void oracle_bounds(int64_t n, const double *v, double *out_min, double *out_max) {
    double mn = INFINITY, mx = -INFINITY;
    for (int64_t i = 0; i < n; ++i) {
        double x = v[i];
        if (!isnan(x)) { if (x < mn) mn = x; if (x > mx) mx = x; }
    }
    *out_min = mn; *out_max = mx;
}
