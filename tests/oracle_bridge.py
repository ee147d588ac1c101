"""Translate datashader_gb300 reduction objects into oracle specs and run the oracle."""
from __future__ import annotations

import numpy as np

import oracle
from datashader_gb300 import reductions as rd


def _spec(red, cat=None, ncat=1):
    k = None
    col = red.column if red.column != rd.SpecialColumn.RowIndex else None
    si = getattr(red, "self_intersect", True)
    if isinstance(red, rd._count_ignore_antialiasing):
        k = "count_ignore_aa"
    elif isinstance(red, rd.count):
        k = "count"
    elif isinstance(red, rd.any):
        k = "any"
    elif isinstance(red, rd._sum_zero):
        k = "sum_zero"
    elif isinstance(red, rd.sum):
        k = "sum"
    elif isinstance(red, rd.mean):
        k = "mean"
    elif isinstance(red, rd.min):
        k = "min"
    elif isinstance(red, rd.max):
        k = "max"
    elif isinstance(red, rd.first):
        k = "first"
    elif isinstance(red, rd.last):
        k = "last"
    elif isinstance(red, rd._min_row_index):
        k, col = "min_row", None
    elif isinstance(red, rd._max_row_index):
        k, col = "max_row", None
    elif isinstance(red, rd.where):
        sel = _spec(red.selector)
        return oracle.spec("where", None, selector=sel, lookup=col, cat=cat, ncat=ncat)
    else:
        raise NotImplementedError(type(red))
    return oracle.spec(k, col, cat=cat, ncat=ncat, self_intersect=si)


def specs_of(agg, frame_cols, categories):
    """(keys, specs, extra columns) for a reduction tree."""
    extra = {}
    out = []
    keys = []
    items = zip(agg.keys, agg.values) if isinstance(agg, rd.summary) else [(None, agg)]
    for key, red in items:
        if isinstance(red, rd.by):
            cz = red.categorizer
            if isinstance(cz, rd.category_modulo):
                name = f"__mod_{cz.column}"
                extra[name] = ((np.asarray(frame_cols[cz.column]).astype(np.int64) - cz.offset)
                               % cz.modulo).astype(np.float64)
                ncat = cz.modulo
            else:
                name = cz.column
                ncat = len(categories[cz.column])
            out.append(_spec(red.reduction, cat=name, ncat=ncat))
        else:
            out.append(_spec(red))
        keys.append(key)
    return keys, out, extra


def _canvas_ranges(canvas):
    return canvas.get("x_range"), canvas.get("y_range")


def run_points(frame_cols, categories, agg, canvas, x="x", y="y", row_offset=0):
    keys, specs, extra = specs_of(agg, frame_cols, categories)
    cols = {k: np.asarray(v, dtype=np.float64) for k, v in frame_cols.items()}
    cols.update(extra)
    xr, yr = _canvas_ranges(canvas)
    res = oracle.points(cols, x, y, canvas["plot_width"], canvas["plot_height"], xr, yr, specs,
                        row_offset=row_offset, x_axis=canvas.get("x_axis_type", "linear"),
                        y_axis=canvas.get("y_axis_type", "linear"))
    return res[0] if keys == [None] else dict(zip(keys, res))


def run_line(frame_cols, categories, agg, canvas, line_width, x="x", y="y"):
    keys, specs, extra = specs_of(agg, frame_cols, categories)
    cols = {k: np.asarray(v, dtype=np.float64) for k, v in frame_cols.items()}
    cols.update(extra)
    xr, yr = _canvas_ranges(canvas)
    res = oracle.line_axis0(cols, x, y, canvas["plot_width"], canvas["plot_height"], xr, yr, specs,
                            line_width=line_width)
    return res[0] if keys == [None] else dict(zip(keys, res))
