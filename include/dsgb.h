/*
 * dsgb.h -- C ABI of libdsgb, the GB300 (sm_103a) projection + aggregation
 * library behind datashader's Canvas.points / Canvas.line / tf.shade(eq_hist).
 *
 * Plain C: pointers, sizes and PODs only, no C++ or torch types.  Every
 * entry point returns DSGB_OK (0) or a negative DSGB_E_* code and never
 * aborts; dsgb_last_error() gives a thread-local message.  All device memory
 * (columns, base accumulators, outputs, workspaces) is owned by the caller;
 * calls are asynchronous on the caller's stream (a cudaStream_t passed as
 * void*, NULL = legacy default stream).
 *
 * Mapping onto the reference (datashader 0.19.1):
 *   - dsgb_points      replaces Point._build_extend's extend()
 *                      (datashader/glyphs/points.py:182-242) together with
 *                      the create/append/finalize functions that
 *                      compiler.compile_components builds
 *                      (datashader/compiler.py:36-150, 294-536).
 *   - dsgb_line_axis0  replaces LineAxis0._internal_build_extend's extend()
 *                      (datashader/glyphs/line.py:59-103, 1033-1149).
 *   - dsgb_eq_hist_u32 / dsgb_eq_hist_f64 replace tf.eq_hist
 *                      (datashader/transfer_functions/__init__.py:148-223)
 *                      plus the mask/offset prologue of _interpolate
 *                      (:251-297) and, optionally, the list-colormap RGBA
 *                      step (:317-351).
 *   - dsgb_bounds      replaces Glyph._compute_bounds_numba
 *                      (datashader/glyphs/glyph.py:66-78).
 *   - dsgb_pyramid     renders a quadtree of tiles in one persistent launch
 *                      (each tile equal to a Canvas.points call, see
 *                      datashader/tiles.py:70-130 for the reference's
 *                      per-tile driver).
 *   - dsgb_line_axis0_backward is the adjoint of dsgb_line_axis0 for the
 *                      antialiased sum reduction (no reference counterpart;
 *                      it differentiates line.py:826-981).
 */
#ifndef DSGB_H
#define DSGB_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DSGB_ABI_VERSION 2   /* 2: list colormaps as float64 channels, up to 256 colours */

/* Status codes. */
#define DSGB_OK             0
#define DSGB_E_INVALID     -1  /* bad argument (null pointer, size, index) */
#define DSGB_E_UNSUPPORTED -2  /* dtype / op combination not implemented */
#define DSGB_E_CUDA        -3  /* CUDA runtime error (message in dsgb_last_error) */
#define DSGB_E_TIMEOUT     -4  /* a bounded device wait gave up */
#define DSGB_E_NOSPACE     -5  /* workspace too small */

/* Column element types. */
typedef enum {
    DSGB_F32 = 1, DSGB_F64 = 2, DSGB_I8 = 3, DSGB_U8 = 4, DSGB_I16 = 5,
    DSGB_I32 = 6, DSGB_I64 = 7, DSGB_U32 = 8, DSGB_BOOL = 9
} dsgb_dtype;

typedef struct {
    const void *data;   /* device pointer, n elements, contiguous */
    int32_t dtype;      /* dsgb_dtype */
    int32_t reserved;
} dsgb_column;

/* The canvas of one aggregation.  s/t are computed by the caller exactly as
 * Axis.compute_scale_and_translate (datashader/core.py:62-81):
 * s = n/(end-start), t = -start*s on the mapped range; x_log / y_log select
 * LogAxis.mapper (core.py:127-145) on the device. */
typedef struct {
    int32_t width, height;
    int32_t x_log, y_log;
    double sx, tx, sy, ty;
    double xmin, xmax, ymin, ymax;   /* inclusive bounds (points.py:198) */
} dsgb_canvas;

/* Base accumulator operations (the GPU form of Reduction._build_bases,
 * reductions.py).  Each base owns one caller-allocated device array of
 * height*width*ncat elements, laid out [y][x][cat] (row 0 = y_min). */
typedef enum {
    DSGB_BASE_COUNT     = 1,  /* uint32: rows (col<0) or non-NaN col values      */
    DSGB_BASE_ANY       = 2,  /* uint8 : 1 where some row (non-NaN col) landed  */
    DSGB_BASE_SUM       = 3,  /* double: sum of non-NaN col values, zero-init   */
    DSGB_BASE_MAX       = 4,  /* int64 : order-preserving key of the max value  */
    DSGB_BASE_MIN       = 5,  /* int64 : order-preserving key of the min value  */
    DSGB_BASE_MIN_ROW   = 6,  /* int64 : smallest row index with non-NaN col    */
    DSGB_BASE_MAX_ROW   = 7,  /* int64 : largest row index with non-NaN col     */
    DSGB_BASE_ARGMAX    = 8,  /* 2 x int64 {key,row}: max value, first row on ties */
    DSGB_BASE_ARGMIN    = 9,  /* 2 x int64 {key,row}: min value, first row on ties */
    /* antialiased-line forms (value = col * coverage) */
    DSGB_BASE_AA_SUM    = 10, /* double: sum of w*(aa - prev_aa), w = col or 1    */
    DSGB_BASE_AA_CNT0   = 11, /* uint32: rows whose prev_aa == 0 (mean count)   */
    DSGB_BASE_AA_MAX    = 12, /* int64 key: max of w*aa, w = col or 1            */
    DSGB_BASE_AA_ARGMAX = 13  /* {key,row}: max of w*aa, first row on ties       */
} dsgb_base_op;

#define DSGB_BASEF_UNWEIGHTED 0x1  /* antialiased forms: the column only gates NaN rows,
                                       the value is the coverage itself */

typedef struct {
    int32_t op;        /* dsgb_base_op */
    int32_t col;       /* value column index, -1 = none (count/any of every row) */
    int32_t cat_col;   /* category-code column index, -1 = not categorical */
    int32_t ncat;      /* categories (>= 1) */
    int32_t flags;     /* DSGB_BASEF_* */
    int32_t reserved;
    void *agg;         /* device accumulator */
} dsgb_base;

/* Finalize operations (Reduction._finalize / make_finalize, compiler.py:510-536). */
typedef enum {
    DSGB_FIN_SUM_NAN    = 1,  /* f64 out = any ? sum : NaN          (b0 SUM/AA_SUM, b1 COUNT/ANY) */
    DSGB_FIN_MEAN       = 2,  /* f64 out = cnt>0 ? sum/cnt : NaN    (b0 SUM/AA_SUM, b1 COUNT/AA_CNT0) */
    DSGB_FIN_KEY_F64    = 3,  /* f64 out = decode(key) or NaN       (b0 MAX/MIN/ARGMAX/ARGMIN/AA_MAX) */
    DSGB_FIN_ROW        = 4,  /* i64 out = row or -1                (b0 MIN_ROW/MAX_ROW/ARGMAX/ARGMIN) */
    DSGB_FIN_GATHER     = 5,  /* f64 out = col[row-row_offset] or NaN (b0 row-valued base, col) */
    DSGB_FIN_KEY_F32    = 6,  /* f32 out = (float)decode(key) or NaN (b0 AA_MAX) */
    DSGB_FIN_SUM_F32    = 7,  /* f32 out = any ? (float)sum : NaN   (b0 AA_SUM, b1 ANY) */
    DSGB_FIN_COPY       = 8   /* out = base bytes (count, any)       (b0) */
} dsgb_fin_op;

typedef struct {
    int32_t op;        /* dsgb_fin_op */
    int32_t base0, base1;
    int32_t col;       /* DSGB_FIN_GATHER: lookup column */
    void *out;         /* device output, height*width*ncat elements of the op's type */
} dsgb_output;

/* Flags. */
#define DSGB_FLAG_NO_INIT      0x1u  /* accumulate into the bases as they are */
#define DSGB_FLAG_NO_FINALIZE  0x2u  /* skip the finalize step */
#define DSGB_FLAG_EXACT_BIN    0x4u  /* always bin in float64 (disable the float32 fast path);
                                       * dsgb_line_axis0_ws: antialiased pixels scanned per
                                       * segment, without the float32 classification */
#define DSGB_FLAG_WARP_AGG     0x8u  /* warp-level pre-aggregation of identical pixels */
#define DSGB_FLAG_DETERMINISTIC 0x10u /* float64 sums in row order (bit-identical to the
                                         reference's CPU loop and run to run); needs the
                                         workspace of dsgb_points_workspace_size_flags */
#define DSGB_FLAG_ROW_ORDER    0x20u /* dsgb_lines, layout 1: row-index bases (first / last / where) keep
                                       global rows, the semantics of a partitioned source (dask.py:86-219,
                                       row-index reductions), instead of the line-major visit order */
#define DSGB_FLAG_DEBUG_CHECKS 0x40u /* dsgb_points / dsgb_line_axis0 / dsgb_lines: every append checks its
                                       aggregate index against the base (pixel inside the canvas, category
                                       code inside 0..ncat-1); an append that fails is skipped and raises
                                       DSGB_STATUS_INDEX.  Takes the generic kernels (no hot-tile path).
                                       The reference's numba appends do no such check. */

/* Device status bits, read by dsgb_device_status.  Kernels never trap: a
 * condition that no valid input produces sets a bit instead. */
#define DSGB_STATUS_CAS_GUARD  0x1u  /* a where(max|min) {key,row} CAS loop reached its iteration guard and
                                       left one row's update undone */
#define DSGB_STATUS_INDEX      0x2u  /* DSGB_FLAG_DEBUG_CHECKS: an append's index fell outside its base */

/* ---- informational ---------------------------------------------------- */
int dsgb_abi_version(void);
const char *dsgb_last_error(void);
/* Waits for the current device (cudaDeviceSynchronize), then ORs into *bits
 * the DSGB_STATUS_* bits that any kernel of this library raised on it since
 * the last clear, and clears them when `clear` is non-zero.  No counterpart
 * in the reference, whose appends run unchecked. */
int dsgb_device_status(uint32_t *bits, int32_t clear);
/* Launches a float64 FMA throughput probe (8 independent chains a thread,
 * iters FMAs each, blocks_per_sm blocks of 256 threads an SM) and returns
 * the FLOPs it performs in *flops; the caller times the launch with CUDA
 * events.  A measurement aid for the roofline of the float64-bound kernels;
 * no counterpart in the reference. */
int dsgb_fp64_probe(double *sink, int32_t iters, int32_t blocks_per_sm, int64_t *flops, void *stream);
/* Number of SMs of the current device (grid sizing), or a negative code. */
int dsgb_device_sm_count(void);

/* ---- bases ------------------------------------------------------------ */
/* Fill each base with its initial value (reductions.py:397-472). */
int dsgb_bases_init(const dsgb_base *bases, int32_t nbases, int64_t ncells, void *stream);
/* Run the finalize step for bases that were filled by earlier calls. */
int dsgb_finalize(const dsgb_column *cols, int32_t ncols, int64_t row_offset,
                  const dsgb_base *bases, int32_t nbases,
                  const dsgb_output *outs, int32_t nouts, int64_t ncells, void *stream);
/* dsgb_finalize for bases combined (dsgb_combine) from row partitions
 * (dask.py:86-219, each partition numbering its rows from its own offset,
 * :102-117): part_cols[p * ncols + c] is column c of partition p, whose
 * rows are the global rows [part_first[p], part_first[p] + part_rows[p])
 * (host arrays, nparts <= 64).  A gather output (first / last / where with
 * a lookup column) reads the selected row from the partition that holds it;
 * every other output is finalized as by dsgb_finalize. */
int dsgb_finalize_partitioned(const dsgb_column *part_cols, int32_t ncols, int32_t nparts,
                              const int64_t *part_first, const int64_t *part_rows,
                              const dsgb_base *bases, int32_t nbases, const dsgb_output *outs,
                              int32_t nouts, int64_t ncells, void *stream);
/* The gather outputs of partitions held by different processes: partition p
 * (global rows [part_first[p], part_first[p] + part_rows[p])) finalized its
 * own gather output (part_vals[p], device float64, one value per cell);
 * out[i] takes the value of the partition holding the row that the combined
 * row_base (MIN_ROW / MAX_ROW or a {key,row} pair base) selected at cell i,
 * so no process needs another's columns.  Replaces the paired selector /
 * lookup combine of where, first and last across partitions
 * (reductions.py:1992-2018, dask.py:168-217).  nparts <= 64. */
int dsgb_select_by_owner(const dsgb_base *row_base, int32_t nparts, const int64_t *part_first,
                         const int64_t *part_rows, const double *const *part_vals, double *out,
                         int64_t ncells, void *stream);

/* ---- Canvas.points ------------------------------------------------------
 * Replaces points.py:182-242 (+ compiler.py create/append/finalize).
 * n rows of columns cols[0..ncols); x_col / y_col index the coordinates;
 * row_offset is added to row indexes (first/last/where). */
int dsgb_points(const dsgb_column *cols, int32_t ncols, int64_t n, int64_t row_offset,
                int32_t x_col, int32_t y_col, const dsgb_canvas *canvas,
                const dsgb_base *bases, int32_t nbases,
                const dsgb_output *outs, int32_t nouts,
                uint32_t flags, void *stream);

/* Canvas.points with a caller-provided workspace.  A plain count() of every
 * row of float32 coordinates (at least 2^20 rows) takes a path that keeps
 * the densest canvas tiles in shared memory: a 1% sample picks the tiles,
 * one CTA per SM counts rows of cached tiles with shared-memory atomics and
 * the others with L2 reductions, and each CTA adds its tiles into the output
 * at the end.  Every other plan, or a workspace smaller than
 * dsgb_points_workspace_size(), runs exactly as dsgb_points.  The workspace
 * must be 256-byte aligned and not used by another call in flight. */
size_t dsgb_points_workspace_size(int64_t n, const dsgb_canvas *canvas,
                                  const dsgb_base *bases, int32_t nbases);
/* Workspace for dsgb_points_ws under `flags` (the deterministic mode needs
 * about 16 bytes per row). */
size_t dsgb_points_workspace_size_flags(int64_t n, const dsgb_canvas *canvas,
                                        const dsgb_base *bases, int32_t nbases, uint32_t flags);
int dsgb_points_ws(const dsgb_column *cols, int32_t ncols, int64_t n, int64_t row_offset,
                   int32_t x_col, int32_t y_col, const dsgb_canvas *canvas,
                   const dsgb_base *bases, int32_t nbases,
                   const dsgb_output *outs, int32_t nouts,
                   void *workspace, size_t workspace_bytes, uint32_t flags, void *stream);

/* Canvas.points over the rows in segments [seg_begin[i], seg_end[i]) of the
 * columns (host arrays, nseg <= 256): the same reductions and flags as
 * dsgb_points (row index = position in the columns; row_offset 0).  The
 * serving path uses it on a bucketed store (dsgb_bucket_sort) so that a
 * viewport reads only the bucket rows it overlaps.  No reference
 * counterpart (the reference scans every row, glyphs/points.py:210-242). */
int dsgb_points_segments(const dsgb_column *cols, int32_t ncols, int64_t n,
                         int32_t x_col, int32_t y_col, const dsgb_canvas *canvas,
                         const dsgb_base *bases, int32_t nbases,
                         const dsgb_output *outs, int32_t nouts,
                         const int64_t *seg_begin, const int64_t *seg_end, int32_t nseg,
                         uint32_t flags, void *stream);

/* Regroup every column by a grid x grid bucketing of the domain square
 * (domain = {x0, x1, y0, y1}, host; grid <= 128): bucket (bx, by) is
 * number by * grid + bx, and bucket grid*grid holds the points outside the
 * domain or with NaN coordinates.  out_data: one device pointer per column
 * (same dtype, n rows); bucket_start (device, grid*grid + 2 int64): row
 * offset of each bucket.  Bucket ids are float64 estimates: a viewport
 * reading buckets must widen its bucket range by one on each side.  No
 * reference counterpart. */
size_t dsgb_bucket_sort_workspace_size(int32_t grid);
int dsgb_bucket_sort(const dsgb_column *cols, int32_t ncols, int64_t n, int32_t x_col, int32_t y_col,
                     const double *domain, int32_t grid, void *const *out_data, int64_t *bucket_start,
                     void *workspace, size_t workspace_bytes, void *stream);

/* Combine the partial bases `src` of one row partition into `dst` (same
 * plan, same canvas): counts and sums add, any ORs, min/max keys and row
 * indexes take the min/max, {key,row} pairs keep the better pair (ties: the
 * smaller global row).  Replaces the per-reduction _combine of datashader's
 * partitioned (dask) path, dask.py:86-219 / compiler.py:478-507.
 * Antialiased line bases of single-stage plans (dsgb_line_axis0 with
 * use_2_stage_agg = 0) combine like their plain forms: coverage sums and
 * counts add, maxima and {key,row} maxima keep the larger. */
int dsgb_combine(const dsgb_base *dst, const dsgb_base *src, int32_t nbases, int64_t ncells, void *stream);

/* ---- Canvas.line, LineAxis0 glyph ----------------------------------------
 * Replaces line.py:59-103 + 1033-1149.  line_width == 0 draws Bresenham
 * lines, > 0 antialiased lines; overwrite / use_2_stage_agg follow
 * antialias.py:30-58 (two_stage_agg) for the reductions in `bases`.
 * Antialiased pixels are classified in float32 and worked off by case
 * (segments in row order here, in work order with dsgb_line_axis0_ws). */
int dsgb_line_axis0(const dsgb_column *cols, int32_t ncols, int64_t n, int64_t row_offset,
                    int32_t x_col, int32_t y_col, const dsgb_canvas *canvas,
                    double line_width, int32_t plot_start, int32_t overwrite,
                    int32_t use_2_stage_agg,
                    const dsgb_base *bases, int32_t nbases,
                    const dsgb_output *outs, int32_t nouts,
                    uint32_t flags, void *stream);

/* dsgb_line_axis0 with a workspace of dsgb_line_workspace_size(n) bytes
 * (256-byte aligned): antialiased segments are then drawn in order of
 * their estimated pixel work, so that the lanes of a warp do similar work.
 * Same results. */
size_t dsgb_line_workspace_size(int64_t n);
int dsgb_line_axis0_ws(const dsgb_column *cols, int32_t ncols, int64_t n, int64_t row_offset,
                       int32_t x_col, int32_t y_col, const dsgb_canvas *canvas,
                       double line_width, int32_t plot_start, int32_t overwrite,
                       int32_t use_2_stage_agg,
                       const dsgb_base *bases, int32_t nbases,
                       const dsgb_output *outs, int32_t nouts,
                       void *workspace, size_t workspace_bytes, uint32_t flags, void *stream);

/* Canvas.line with the multi-line glyphs (line.py:106-430, 1152-1437):
 * layout 1 = LineAxis0Multi (xs, ys float64 [nrows][nv], nv lines running
 * down the rows); layout 2 = LinesAxis1 family (one line per row through nv
 * vertices: vertex (i, j) = (xs[i*x_row_stride + j], ys[i*y_row_stride + j]),
 * a stride of 0 shares one array across the rows: XConstant / YConstant).
 * Segment (i, j) appends row i's fields (cols).  Reductions as
 * dsgb_line_axis0; two-stage antialiased plans are not supported.  With
 * layout 1 and nv > 1, first / last / where follow the reference's visit
 * order (line j outer, row i inner: line.py:1190-1194), so their row-index
 * bases cannot accumulate across calls (DSGB_FLAG_NO_INIT is rejected). */
int dsgb_lines(const dsgb_column *cols, int32_t ncols, int64_t nrows, int64_t row_offset,
               int32_t layout, const double *xs, const double *ys, int64_t nv,
               int64_t x_row_stride, int64_t y_row_stride, const dsgb_canvas *canvas,
               double line_width, int32_t plot_start, int32_t overwrite,
               const dsgb_base *bases, int32_t nbases,
               const dsgb_output *outs, int32_t nouts, uint32_t flags, void *stream);

/* Two-stage antialiased plans over several lines (the reference's
 * cpu_antialias_2agg_impl, line.py:1203-1226 for LineAxis0Multi and
 * :1300-1318 with its siblings for the LinesAxis1 family; compiler.py:198-268
 * for the folds).  Each line is drawn alone: line 0 into the bases, every
 * later line into `line_aggs[b]` (caller-owned device buffers of the same
 * size as bases[b].agg, initialised here), which is then folded into
 * bases[b].agg with folds[b], in line order.  Arguments otherwise as
 * dsgb_lines; line_width > 0.  The previous vertex is never read (two-stage
 * plans draw every segment as if it started a line, line.py:1170, 1266).
 * Supported bases and folds: DSGB_BASE_AA_MAX with any value fold,
 * DSGB_BASE_MIN_ROW with DSGB_FOLD_ROW_MIN, DSGB_BASE_MAX_ROW with
 * DSGB_FOLD_MAX, DSGB_BASE_AA_SUM / DSGB_BASE_AA_CNT0 / DSGB_BASE_COUNT with DSGB_FOLD_ADD,
 * DSGB_BASE_AA_ARGMAX with DSGB_FOLD_WHERE_*.  Cost: one launch per line plus one initialisation and one
 * fold of each base over the canvas per line after the first. */
enum {
    DSGB_FOLD_SUM      = 1,  /* nansum_in_place, float64 (count / sum, self_intersect=False) */
    DSGB_FOLD_SUM_F32  = 2,  /* nansum_in_place on a float32 aggregate (antialiased count)   */
    DSGB_FOLD_MAX      = 3,  /* nanmax_in_place (any, max) / row_max_in_place (MAX_ROW)      */
    DSGB_FOLD_MIN      = 4,  /* nanmin_in_place (min)                                       */
    DSGB_FOLD_FIRST    = 5,  /* nanfirst_in_place (first)                                   */
    DSGB_FOLD_LAST     = 6,  /* nanlast_in_place (last)                                     */
    DSGB_FOLD_ROW_MIN  = 7,  /* row_min_in_place (MIN_ROW)                                  */
    DSGB_FOLD_ADD      = 8,  /* nansum_in_place of additive bases (AA_SUM, AA_CNT0 and the COUNT
                                row mask: mean / _sum_zero / _count_ignore_antialiasing, and
                                count / sum in a plan that keeps self_intersect): every line
                                draws straight into the accumulator; line_aggs[b] unused */
    DSGB_FOLD_WHERE_MAX   = 9,   /* where(max | min | first | last) on AA_ARGMAX pairs: the   */
    DSGB_FOLD_WHERE_MIN   = 10,  /* selector's own append decides, the row follows           */
    DSGB_FOLD_WHERE_FIRST = 11,  /* (reductions.py:1992-2018)                                 */
    DSGB_FOLD_WHERE_LAST  = 12
};
int dsgb_lines_2stage(const dsgb_column *cols, int32_t ncols, int64_t nrows, int64_t row_offset,
                      int32_t layout, const double *xs, const double *ys, int64_t nv,
                      int64_t x_row_stride, int64_t y_row_stride, const dsgb_canvas *canvas,
                      double line_width, int32_t overwrite, const dsgb_base *bases, int32_t nbases,
                      const int32_t *folds, void *const *line_aggs, const dsgb_output *outs,
                      int32_t nouts, uint32_t flags, void *stream);

/* dsgb_lines_ragged's two-stage antialiased form (the reference's
 * extend_cpu_antialias_2agg of LinesAxis1Ragged, line.py:1616-1693): one row
 * at a time, folds and per-line aggregates as dsgb_lines_2stage. */
int dsgb_lines_ragged_2stage(const dsgb_column *cols, int32_t ncols, int64_t nrows, int64_t row_offset,
                             const double *x_flat, int64_t nx, const int64_t *x_start,
                             const double *y_flat, int64_t ny, const int64_t *y_start,
                             const dsgb_canvas *canvas, double line_width, int32_t overwrite,
                             const dsgb_base *bases, int32_t nbases, const int32_t *folds,
                             void *const *line_aggs, const dsgb_output *outs, int32_t nouts,
                             uint32_t flags, void *stream);

/* Canvas.line(axis=1) over ragged x / y columns (LinesAxis1Ragged,
 * line.py:457-523 and 1538-1612): row i's vertices are x_flat[x_start[i] ..
 * x_start[i+1]) and y_flat[y_start[i] .. y_start[i+1]) (the last row to nx /
 * ny; starts are device int64, non-decreasing), drawn through the shorter of
 * the two; segment j appends row i's fields (cols).  Reductions as
 * dsgb_lines; two-stage antialiased plans are not supported. */
int dsgb_lines_ragged(const dsgb_column *cols, int32_t ncols, int64_t nrows, int64_t row_offset,
                      const double *x_flat, int64_t nx, const int64_t *x_start,
                      const double *y_flat, int64_t ny, const int64_t *y_start,
                      const dsgb_canvas *canvas, double line_width, int32_t overwrite,
                      const dsgb_base *bases, int32_t nbases, const dsgb_output *outs, int32_t nouts,
                      uint32_t flags, void *stream);

/* Adjoint of the antialiased LineAxis0 sum('v') aggregate (self-intersecting
 * form): given dL/dagg (f64, height*width), accumulate dL/dv (f64, n) and
 * dL/dy (f64, n, y in data units) with coverage recomputed, not stored.
 * `agg_any` (uint8, may be NULL) masks pixels that the forward left NaN. */
int dsgb_line_axis0_backward(const dsgb_column *cols, int32_t ncols, int64_t n,
                             int32_t x_col, int32_t y_col, int32_t v_col,
                             const dsgb_canvas *canvas, double line_width,
                             int32_t plot_start, const double *grad_agg,
                             const uint8_t *agg_any, double *grad_v, double *grad_y,
                             void *stream);

/* dsgb_line_axis0_backward with a workspace of dsgb_line_workspace_size(n)
 * bytes (256-byte aligned): the segments are recomputed in the forward's
 * work order (bucketed by estimated pixel count), so the lanes of a warp do
 * similar work.  Same results up to the order of the float64 atomics that
 * accumulate dL/dy; a missing or short workspace runs in row order. */
int dsgb_line_axis0_backward_ws(const dsgb_column *cols, int32_t ncols, int64_t n,
                                int32_t x_col, int32_t y_col, int32_t v_col,
                                const dsgb_canvas *canvas, double line_width,
                                int32_t plot_start, const double *grad_agg,
                                const uint8_t *agg_any, double *grad_v, double *grad_y,
                                void *workspace, size_t workspace_bytes, void *stream);

/* Adjoint of points sum / mean w.r.t. the value column (gather):
 * grad_v[i] = grad_agg[p(i)] (sum) or grad_agg[p(i)]/count[p(i)] (mean when
 * counts != NULL); rows that are NaN or out of bounds get 0. */
int dsgb_points_backward(const dsgb_column *cols, int32_t ncols, int64_t n,
                         int32_t x_col, int32_t y_col, int32_t v_col,
                         const dsgb_canvas *canvas, const double *grad_agg,
                         const uint32_t *counts, double *grad_v, uint32_t flags, void *stream);

/* ---- autorange ----------------------------------------------------------
 * glyph.py:66-78: NaN-skipping min and max of a column into out_minmax[0..1]
 * (device, double).  Empty / all-NaN gives (+inf, -inf). */
int dsgb_bounds(const dsgb_column *col, int64_t n, double *out_minmax, void *stream);

/* ---- eq_hist (transfer_functions/__init__.py:148-223, 251-297) -----------
 * Input: a uint32 aggregate (count) or a float64 aggregate; masked pixels are
 * 0 (uint32) or NaN (float64).  Output: out (f64, NaN where masked) = the
 * equalised value; *levels (device int64) = discrete_levels; when rgba != NULL
 * the list-colormap RGBA image (uint32) is also written, with `ncolors` colour
 * stops in `cmap_rgb` (host, 3*ncolors float64 channels, 1 <= ncolors <= 256: a
 * colour tuple may hold floats, interpolated before the uint8 truncation as
 * numpy does) and `alpha`, `rescale` as in
 * tf.shade.  `workspace` must hold dsgb_eq_hist_workspace_size() bytes. */
size_t dsgb_eq_hist_workspace_size(int32_t nbins);
int dsgb_eq_hist_u32(const uint32_t *data, int64_t n, int32_t nbins,
                     double *out, int64_t *levels, uint32_t *rgba,
                     const double *cmap_rgb, int32_t ncolors, int32_t alpha,
                     int32_t rescale_discrete_levels,
                     void *workspace, size_t workspace_bytes, void *stream);
int dsgb_eq_hist_f64(const double *data, int64_t n, int32_t nbins,
                     double *out, int64_t *levels, uint32_t *rgba,
                     const double *cmap_rgb, int32_t ncolors, int32_t alpha,
                     int32_t rescale_discrete_levels,
                     void *workspace, size_t workspace_bytes, void *stream);

/* dsgb_eq_hist_u32 for callers that cannot allocate device memory (no
 * counterpart in the reference).  The scratch is a file-scope device array
 * inside libdsgb sized for nbins <= 65536 (about 1.25 MiB, held on every GPU
 * that loads the library until the process exits); larger nbins are
 * rejected with DSGB_E_INVALID.  Nothing is allocated: the first call on a
 * device looks up the array's device address (with that device current)
 * and caches it with the device's current context, so make that first call
 * before any stream capture; after a cudaDeviceReset (a new context) the
 * next call looks the address up again.  Every
 * call shares the one array and resets what must start at zero, so calls
 * whose work overlaps on the GPU (different streams, or host threads racing
 * on one device) corrupt each other: serialise them. */
int dsgb_eq_hist_u32_static(const uint32_t *data, int64_t n, int32_t nbins,
                            double *out, int64_t *levels, uint32_t *rgba,
                            const double *cmap_rgb, int32_t ncolors, int32_t alpha,
                            int32_t rescale_discrete_levels, void *stream);

/* tf.shade(how='linear' | 'log' | 'cbrt') of a 2-D aggregate
 * (transfer_functions/__init__.py:220-356): how 0 = linear, 1 = log,
 * 2 = cbrt; span (host, 2 doubles) or NULL; a list colormap (cmap_rgb: host,
 * 3*ncolors float64 channels, ncolors <= 256) or, when single_rgb != NULL, one colour with an alpha
 * ramp from min_alpha to alpha.  rgba: uint32 per pixel.  The workspace is
 * dsgb_shade_workspace_size() bytes, 256-byte aligned. */
size_t dsgb_shade_workspace_size(void);
int dsgb_shade_u32(const uint32_t *data, int64_t n, int32_t how, const double *span,
                   const double *cmap_rgb, int32_t ncolors, const uint8_t *single_rgb,
                   int32_t alpha, int32_t min_alpha, uint32_t *rgba,
                   void *workspace, size_t workspace_bytes, void *stream);
int dsgb_shade_f64(const double *data, int64_t n, int32_t how, const double *span,
                   const double *cmap_rgb, int32_t ncolors, const uint8_t *single_rgb,
                   int32_t alpha, int32_t min_alpha, uint32_t *rgba,
                   void *workspace, size_t workspace_bytes, void *stream);

/* Image compositing (datashader/composite.py:31-127; tf.stack
 * transfer_functions/__init__.py:115-145 and tf.set_background :748-767):
 * out[i] = op(src[i], dst ? dst[i] : dst_value) on uint32 RGBA pixels, op
 * 0 = source, 1 = over, 2 = add, 3 = saturate, bit-identical to the
 * reference's float64 arithmetic.  out may alias src or dst. */
int dsgb_composite(const uint32_t *src, const uint32_t *dst, uint32_t dst_value, int64_t n, int32_t op,
                   uint32_t *out, void *stream);

/* ---- batched tile pyramid --------------------------------------------------
 * Every tile (z, tx, ty), zmin <= z <= zmax, of the square [x0,x1]x[y0,y1]
 * in one pass: tile (z, tx, ty) equals
 *   Canvas(ts, ts, x_range=(lo(tx), lo(tx+1)), y_range=(lo(ty), lo(ty+1)))
 *       .points(df, 'x', 'y', count() / max('v'))
 * with lo(t) = x0 + (x1 - x0) * (t / 2^z) in float64, i.e. one reference
 * call per tile (glyphs/points.py:182-242 with core.py:62-81); points on a
 * shared edge count in both tiles.  Tiles are stored level by level
 * (dsgb_pyramid_tile_offset), row-major by (ty, tx), each [ts][ts] with
 * row 0 at the tile's lower y.  counts: uint32; max_out (when v_col >= 0):
 * float64, NaN where empty, max of +-0 reported as +0.  x, y, v float32;
 * zmax <= 6.  The knobs (autotuned by the caller): split (the
 * shared-memory footprint of the finest level is ts >> (1 + split) pixels
 * on a side), threads (render CTA size: 256, 512 or 1024) and chunk (points
 * per work item).  No reference counterpart: the reference renders tiles
 * one Canvas call at a time (tiles.py:70-130). */
typedef struct {
    int32_t zmin, zmax, tile_size, split;
    int32_t threads, chunk;
    double x0, x1, y0, y1;
} dsgb_pyramid_config;
int64_t dsgb_pyramid_tile_offset(int32_t zmin, int32_t z, int32_t tile_size);
size_t dsgb_pyramid_workspace_size(int64_t n, int32_t has_v, const dsgb_pyramid_config *config);
/* flags: DSGB_PYRAMID_CAP_SHIFT(k) uses 1/2^k of the workspace's queue and
 * slot capacities (k = 0..31; a smaller workspace footprint for callers
 * that know their data, and the way to test the overflow status bits). */
#define DSGB_PYRAMID_CAP_SHIFT(k) (((uint32_t)(k) & 31u) << 8)
int dsgb_pyramid(const dsgb_column *cols, int32_t ncols, int64_t n,
                 int32_t x_col, int32_t y_col, int32_t v_col,
                 const dsgb_pyramid_config *config,
                 uint32_t *counts, double *max_out,
                 void *workspace, size_t workspace_bytes, uint32_t flags, void *stream);
/* Status bits of the last dsgb_pyramid on this workspace (synchronises the
 * stream): 1 = edge-contribution queue overflowed, 2 = a max update gave up,
 * 4 = partial slots exhausted.  Non-zero means the pyramid is incomplete. */
int dsgb_pyramid_status(const void *workspace, int64_t n, int32_t has_v,
                        const dsgb_pyramid_config *config, uint32_t *flags_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* DSGB_H */
