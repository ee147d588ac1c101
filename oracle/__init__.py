"""CPU oracle for the datashader aggregation hot path -- TEST INFRASTRUCTURE ONLY.

This package restates the reference's CPU algorithm (datashader 0.19.1, the
numba path) so that the GPU kernels can be checked against it:

* ``dsgb_oracle.c`` -- points binning, the reduction append functions, and
  LineAxis0 (clipping, Bresenham, antialiased coverage), row by row, serial,
  compiled with ``-ffp-contract=off``;
* ``eq_hist.py`` -- the eq_hist histogram/CDF step and the list-colormap
  shading of ``tf.shade`` restated with numpy (the reference calls numpy for
  these steps itself).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker / baseline.
The product path (``datashader_gb300``) never imports it.

Parity is pinned by ``tests/test_oracle_golden.py`` against the golden
vectors of the reference's own test-suite (extracted to ``tests/golden/``).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lock = threading.Lock()
_lib = None

KIND = {
    "count": 1, "any": 2, "sum": 3, "sum_zero": 4, "mean": 5, "min": 6, "max": 7,
    "first": 8, "last": 9, "min_row": 10, "max_row": 11, "where": 12,
    "count_ignore_aa": 13,
}


class _Red(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32), ("col", ctypes.c_int32), ("sel_kind", ctypes.c_int32),
        ("sel_col", ctypes.c_int32), ("lookup_col", ctypes.c_int32), ("cat_col", ctypes.c_int32),
        ("ncat", ctypes.c_int32), ("self_intersect", ctypes.c_int32),
        ("agg", ctypes.c_void_p), ("agg2", ctypes.c_void_p),
    ]


def build(force: bool = False) -> str:
    """Compile the C oracle (gcc, -ffp-contract=off) into oracle/_build."""
    src = os.path.join(_HERE, "dsgb_oracle.c")
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src)):
        return _LIB_PATH
    os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call([
        os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
        "-std=c11", "-shared", "-o", tmp, src, "-lm"])
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            L.oracle_init.argtypes = [ctypes.POINTER(_Red), ctypes.c_int, ctypes.c_int64, ctypes.c_int]
            L.oracle_points.argtypes = [
                ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                ctypes.c_int32, ctypes.c_int32] + [ctypes.c_double] * 8 + [
                ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_Red), ctypes.c_int]
            L.oracle_points_xy32.argtypes = L.oracle_points.argtypes
            L.oracle_line_axis0.argtypes = [
                ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                ctypes.c_int32, ctypes.c_int32] + [ctypes.c_double] * 9 + [
                ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_Red), ctypes.c_int]
            L.oracle_lines.argtypes = [
                ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                ctypes.c_int32, ctypes.c_int32] + [ctypes.c_double] * 9 + [
                ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_Red), ctypes.c_int]
            L.oracle_lines_2stage.argtypes = L.oracle_lines.argtypes
            L.oracle_lines_ragged.argtypes = [
                ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                ctypes.c_int32, ctypes.c_int32] + [ctypes.c_double] * 9 + [
                ctypes.c_int32, ctypes.POINTER(_Red), ctypes.c_int]
            L.oracle_lines_ragged_2stage.argtypes = L.oracle_lines_ragged.argtypes
            L.oracle_bounds.argtypes = [ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
            _lib = L
    return _lib


# --------------------------------------------------------------------------
# Reduction specs.  A spec is a dict:
#   {"kind": <KIND key>, "column": name|None, "selector": spec|None,
#    "lookup": name|None, "cat": name|None, "ncat": int, "self_intersect": bool}
# --------------------------------------------------------------------------

def spec(kind, column=None, *, selector=None, lookup=None, cat=None, ncat=1,
         self_intersect=True):
    return dict(kind=kind, column=column, selector=selector, lookup=lookup, cat=cat,
                ncat=ncat, self_intersect=self_intersect)


def scale_translate(rng, n, log=False):
    """core.py:62-81 -- s = n/(end-start), t = -start*s, in Python floats."""
    start, end = rng
    if log:
        start, end = math.log10(float(start)), math.log10(float(end))
    s = n / (end - start)
    t = -start * s
    return s, t


def maybe_expand_bounds(bounds):
    """glyph.py:42-49."""
    mn, mx = bounds
    if not (np.isfinite(mn) and np.isfinite(mx)):
        mn, mx = -1.0, 1.0
    elif mn == mx:
        mn, mx = mn - 1, mn + 1
    return mn, mx


def compute_bounds(v):
    """glyph.py:66-78 via the C restatement."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    mn, mx = ctypes.c_double(), ctypes.c_double()
    lib().oracle_bounds(v.size, v.ctypes.data, ctypes.byref(mn), ctypes.byref(mx))
    return mn.value, mx.value


def _agg_dtype(kind, antialias, lookup_is_row=False):
    if kind == "count":
        return np.float32 if antialias else np.uint32
    if kind == "count_ignore_aa":
        return np.uint32
    if kind == "any":
        return np.float32 if antialias else np.uint8
    if kind in ("min_row", "max_row"):
        return np.int64
    if kind == "where":
        return np.int64 if lookup_is_row else np.float64
    return np.float64


def _prepare(cols, specs, shape, antialias):
    names = []

    def cidx(name):
        if name is None:
            return -1
        if name not in names:
            names.append(name)
        return names.index(name)

    H, W = shape
    reds = (_Red * len(specs))()
    keep = []
    for k, s in enumerate(specs):
        ncat = int(s.get("ncat") or 1) if s.get("cat") is not None else 1
        r = reds[k]
        r.kind = KIND[s["kind"]]
        r.col = cidx(s.get("column"))
        r.cat_col = cidx(s.get("cat"))
        r.ncat = ncat
        r.self_intersect = 1 if s.get("self_intersect", True) else 0
        r.sel_kind = 0
        r.sel_col = -1
        r.lookup_col = -1
        full = (H, W, ncat) if s.get("cat") is not None else (H, W)
        if s["kind"] == "where":
            sel = s["selector"]
            r.sel_kind = KIND[sel["kind"]]
            r.sel_col = cidx(sel.get("column"))
            r.lookup_col = cidx(s.get("lookup"))
            agg = np.empty(full, _agg_dtype("where", antialias, s.get("lookup") is None))
            agg2 = np.empty(full, np.int64 if sel["kind"] in ("min_row", "max_row") else np.float64)
        elif s["kind"] == "mean":
            agg = np.empty(full, np.float64)
            agg2 = np.empty(full, np.uint32)
        else:
            agg = np.empty(full, _agg_dtype(s["kind"], antialias))
            agg2 = None
        r.agg = agg.ctypes.data
        r.agg2 = agg2.ctypes.data if agg2 is not None else None
        keep.append((agg, agg2))
    colarrs = [np.ascontiguousarray(cols[n], dtype=np.float64) for n in names]
    ptrs = (ctypes.c_void_p * max(1, len(colarrs)))(*[a.ctypes.data for a in colarrs])
    return reds, keep, colarrs, ptrs


def _finalize(specs, keep):
    out = []
    for s, (agg, agg2) in zip(specs, keep):
        if s["kind"] == "mean":
            with np.errstate(divide="ignore", invalid="ignore"):
                out.append(np.where(agg2 > 0, agg / agg2, np.nan))     # reductions.py:1290-1296
        elif s["kind"] == "any" and agg.dtype == np.uint8:
            out.append(agg.astype(bool))
        else:
            out.append(agg)
    return out


def points(cols, x, y, width, height, x_range, y_range, specs, row_offset=0,
           x_axis="linear", y_axis="linear", raw=False):
    """Canvas.points via pandas.default + Point.extend_cpu (pandas.py:26-66, points.py:182-212).

    float32 x and y columns are read as float32 and widened row by row inside
    the C loop, as numba does; other coordinate dtypes are converted to
    float64 first."""
    f32 = (np.asarray(cols[x]).dtype == np.float32 and np.asarray(cols[y]).dtype == np.float32)
    cdt = np.float32 if f32 else np.float64
    xs = np.ascontiguousarray(cols[x], dtype=cdt)
    ys = np.ascontiguousarray(cols[y], dtype=cdt)
    if x_range is None:
        x_range = maybe_expand_bounds(compute_bounds(xs))
    if y_range is None:
        y_range = maybe_expand_bounds(compute_bounds(ys))
    sx, tx = scale_translate(x_range, width, x_axis == "log")
    sy, ty = scale_translate(y_range, height, y_axis == "log")
    reds, keep, colarrs, ptrs = _prepare(cols, specs, (height, width), False)
    L = lib()
    L.oracle_init(reds, len(specs), height * width, 0)
    loop = L.oracle_points_xy32 if f32 else L.oracle_points
    loop(xs.size, xs.ctypes.data, ys.ctypes.data, ptrs, row_offset, width, height,
                    sx, tx, sy, ty, float(x_range[0]), float(x_range[1]),
                    float(y_range[0]), float(y_range[1]),
                    1 if x_axis == "log" else 0, 1 if y_axis == "log" else 0,
                    reds, len(specs))
    return keep if raw else _finalize(specs, keep)


def combine_partials(specs, parts):
    """Fold the raw (agg, agg2) bases of row partitions, in row order, the way
    datashader's dask path combines partition aggregates (compiler.py:478-507,
    reductions.py `_combine` of each base; dask.py:168-217), then finalize.
    ``parts``: one list of (agg, agg2) per partition, earlier rows first."""
    acc = [tuple(None if a is None else a.copy() for a in pair) for pair in parts[0]]
    for part in parts[1:]:
        for k, s in enumerate(specs):
            (a, a2), (b, b2) = acc[k], part[k]
            kind = s["kind"]
            if kind in ("count", "count_ignore_aa", "sum_zero"):
                a += b
            elif kind == "any":
                np.maximum(a, b, out=a)
            elif kind == "mean":
                a += b
                a2 += b2
            elif kind == "sum":                 # nansum, NaN where both are empty
                both = np.isnan(a) & np.isnan(b)
                a[...] = np.where(both, np.nan, np.nan_to_num(a, nan=0.0) + np.nan_to_num(b, nan=0.0))
            elif kind == "max":
                np.fmax(a, b, out=a)
            elif kind == "min":
                np.fmin(a, b, out=a)
            elif kind == "first":               # the earlier partition's value wins
                a[...] = np.where(np.isnan(a), b, a)
            elif kind == "last":
                a[...] = np.where(np.isnan(b), a, b)
            elif kind == "min_row":
                a[...] = np.where(a < 0, b, np.where(b < 0, a, np.minimum(a, b)))
            elif kind == "max_row":
                np.maximum(a, b, out=a)
            elif kind == "where":
                sk = s["selector"]["kind"]
                if sk in ("max", "min"):        # strictly better selector value wins; ties keep the earlier rows
                    better = (~np.isnan(b2)) & (np.isnan(a2) | ((b2 > a2) if sk == "max" else (b2 < a2)))
                elif sk == "first":
                    better = np.isnan(a2) & ~np.isnan(b2)
                elif sk == "last":
                    better = ~np.isnan(b2)
                elif sk == "min_row":
                    better = (b2 >= 0) & (a2 < 0)
                else:                            # max_row
                    better = b2 > a2
                a[...] = np.where(better, b, a)
                a2[...] = np.where(better, b2, a2)
            else:
                raise NotImplementedError(kind)
    return _finalize(specs, acc)


def points_parallel(cols, x, y, width, height, x_range, y_range, specs, threads=None):
    """oracle.points over one row partition per host thread (the C loop
    releases the GIL), partial bases folded by :func:`combine_partials`.
    Fixed ranges only."""
    threads = threads or os.cpu_count() or 1
    n = len(cols[x])
    bounds = np.linspace(0, n, threads + 1).astype(np.int64)
    parts = [None] * threads

    def work(k):
        a, b = bounds[k], bounds[k + 1]
        sub = {c: v[a:b] for c, v in cols.items()}
        parts[k] = points(sub, x, y, width, height, x_range, y_range, specs, row_offset=int(a), raw=True)

    ts = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return combine_partials(specs, parts)


# AntialiasCombination values (antialias.py:8-14).
SUM_1AGG, SUM_2AGG, MIN, MAX, FIRST, LAST = range(1, 7)


def _requires_2_stages(s):
    """Reduction._antialias_requires_2_stages overrides (reductions.py)."""
    k = s["kind"]
    if k in ("count", "sum"):
        return not s.get("self_intersect", True)
    return k in ("min", "first", "last", "min_row")


def _combinations(s, self_intersect):
    """Reduction._antialias_stage_2 of each base of a spec."""
    k = s["kind"]
    if k in ("count", "sum", "sum_zero", "count_ignore_aa"):
        return [SUM_1AGG if self_intersect else SUM_2AGG]
    if k == "mean":
        return [SUM_1AGG if self_intersect else SUM_2AGG] * 2
    if k in ("any", "max", "max_row"):
        return [MAX]
    if k in ("min", "min_row"):
        return [MIN]
    if k == "first":
        return [FIRST]
    if k == "last":
        return [LAST]
    if k == "where":
        sel = _combinations(s["selector"], self_intersect)
        return sel + sel
    raise ValueError(k)


def aa_flags(specs):
    """compiler.py:539-554 (make_antialias_stage_2) + antialias.py:30-58 (two_stage_agg).

    Returns (self_intersect, overwrite, use_2_stage_agg)."""
    self_intersect = not any(_requires_2_stages(s) for s in specs)
    combos = [c for s in specs for c in _combinations(s, self_intersect)]
    use_2_stage = any(c in (SUM_2AGG, MIN, FIRST, LAST) for c in combos)
    overwrite = not any(c == SUM_1AGG for c in combos)
    return self_intersect, overwrite, use_2_stage


def line_axis0(cols, x, y, width, height, x_range, y_range, specs, line_width=0.0,
               plot_start=True, row_offset=0):
    """Canvas.line with the LineAxis0 glyph (core.py:234-478, line.py:59-103, 1099-1136)."""
    xs = np.ascontiguousarray(cols[x], dtype=np.float64)
    ys = np.ascontiguousarray(cols[y], dtype=np.float64)
    if x_range is None:
        x_range = maybe_expand_bounds(compute_bounds(xs))
    if y_range is None:
        y_range = maybe_expand_bounds(compute_bounds(ys))
    sx, tx = scale_translate(x_range, width)
    sy, ty = scale_translate(y_range, height)
    antialias = line_width > 0
    if antialias:
        self_intersect, overwrite, use_2_stage = aa_flags(specs)
        specs = [dict(s, self_intersect=self_intersect) for s in specs]
    else:
        overwrite, use_2_stage = False, False
    reds, keep, colarrs, ptrs = _prepare(cols, specs, (height, width), antialias)
    L = lib()
    L.oracle_init(reds, len(specs), height * width, 1 if antialias else 0)
    L.oracle_line_axis0(xs.size, xs.ctypes.data, ys.ctypes.data, ptrs, row_offset, width, height,
                        sx, tx, sy, ty, float(x_range[0]), float(x_range[1]),
                        float(y_range[0]), float(y_range[1]), float(line_width),
                        1 if plot_start else 0, 1 if overwrite else 0, 1 if use_2_stage else 0,
                        reds, len(specs))
    return _finalize(specs, keep)


def lines(cols, layout, xs, ys, width, height, x_range, y_range, specs, line_width=0.0, plot_start=True,
          row_offset=0):
    """Canvas.line with a multi-line glyph (line.py:1152-1437).

    layout 1 (LineAxis0Multi): xs, ys float64 [nrows][nlines].
    layout 2 (LinesAxis1 family): xs [nrows][nv] or [nv] (XConstant), ys [nrows][nv]
    or [nv] (YConstant).  ``cols`` holds the field columns, indexed by row."""
    xs = np.ascontiguousarray(xs, dtype=np.float64)
    ys = np.ascontiguousarray(ys, dtype=np.float64)
    if layout == 1:
        nrows, nv = xs.shape
        xrow = yrow = nv
    else:
        nv = xs.shape[-1] if xs.ndim == 2 else ys.shape[-1]
        nrows = ys.shape[0] if ys.ndim == 2 else xs.shape[0]
        xrow = nv if xs.ndim == 2 else 0
        yrow = nv if ys.ndim == 2 else 0
    if x_range is None:
        x_range = maybe_expand_bounds(compute_bounds(xs.ravel()))
    if y_range is None:
        y_range = maybe_expand_bounds(compute_bounds(ys.ravel()))
    sx, tx = scale_translate(x_range, width)
    sy, ty = scale_translate(y_range, height)
    antialias = line_width > 0
    use_2_stage = False
    if antialias:
        self_intersect, overwrite, use_2_stage = aa_flags(specs)
        specs = [dict(s, self_intersect=self_intersect) for s in specs]
    else:
        overwrite = False
    reds, keep, colarrs, ptrs = _prepare(cols, specs, (height, width), antialias)
    L = lib()
    L.oracle_init(reds, len(specs), height * width, 1 if antialias else 0)
    fn = L.oracle_lines_2stage if use_2_stage else L.oracle_lines
    rc = fn(layout, nrows, nv, xs.ctypes.data, ys.ctypes.data, xrow, yrow, ptrs, row_offset, width, height,
            sx, tx, sy, ty, float(x_range[0]), float(x_range[1]), float(y_range[0]), float(y_range[1]),
            float(line_width), 1 if plot_start else 0, 1 if overwrite else 0, reds, len(specs))
    if rc == -2:
        raise NotImplementedError("a reduction of this two-stage antialiased plan has no stage-2 fold in the oracle")
    return _finalize(specs, keep)


def lines_ragged(cols, x_rows, y_rows, width, height, x_range, y_range, specs, line_width=0.0, row_offset=0):
    """Canvas.line(axis=1) over ragged x / y columns (LinesAxis1Ragged,
    line.py:457-523, 1538-1612): ``x_rows`` / ``y_rows`` are lists of
    per-row vertex lists; ``cols`` holds the field columns, indexed by row."""
    nrows = len(x_rows)
    xf = np.ascontiguousarray(np.concatenate([np.asarray(r, dtype=np.float64) for r in x_rows])
                              if nrows else np.zeros(0), dtype=np.float64)
    yf = np.ascontiguousarray(np.concatenate([np.asarray(r, dtype=np.float64) for r in y_rows])
                              if nrows else np.zeros(0), dtype=np.float64)
    xstart = np.ascontiguousarray(np.concatenate([[0], np.cumsum([len(r) for r in x_rows])[:-1]]), dtype=np.int64)
    ystart = np.ascontiguousarray(np.concatenate([[0], np.cumsum([len(r) for r in y_rows])[:-1]]), dtype=np.int64)
    if x_range is None:
        x_range = maybe_expand_bounds(compute_bounds(xf))
    if y_range is None:
        y_range = maybe_expand_bounds(compute_bounds(yf))
    sx, tx = scale_translate(x_range, width)
    sy, ty = scale_translate(y_range, height)
    antialias = line_width > 0
    overwrite = False
    use_2_stage = False
    if antialias:
        self_intersect, overwrite, use_2_stage = aa_flags(specs)
        specs = [dict(s, self_intersect=self_intersect) for s in specs]
    reds, keep, colarrs, ptrs = _prepare(cols, specs, (height, width), antialias)
    L = lib()
    L.oracle_init(reds, len(specs), height * width, 1 if antialias else 0)
    fn = L.oracle_lines_ragged_2stage if use_2_stage else L.oracle_lines_ragged
    rc = fn(nrows, xf.ctypes.data, xf.size, xstart.ctypes.data, yf.ctypes.data, yf.size,
            ystart.ctypes.data, ptrs, row_offset, width, height, sx, tx, sy, ty,
            float(x_range[0]), float(x_range[1]), float(y_range[0]), float(y_range[1]),
            float(line_width), 1 if overwrite else 0, reds, len(specs))
    if rc == -2:
        raise NotImplementedError("a reduction of this two-stage antialiased plan has no stage-2 fold in the oracle")
    return _finalize(specs, keep)


from .eq_hist import eq_hist, shade_eq_hist, shade_interp, interpolate_prologue  # noqa: E402,F401
