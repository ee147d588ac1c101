"""numpy restatement of eq_hist and the list-colormap shading (test infrastructure only).

Follows datashader/transfer_functions/__init__.py:
  * eq_hist                 148-223
  * _interpolate prologue   251-297 (copy, mask, offset, ``data -= offset``)
  * span + rescale          299-316, _rescale_discrete_levels 234-248
  * list-cmap RGBA branch   317-351 (interp of each channel, alpha mask)

The reference itself calls numpy (np.unique, np.histogram, cumsum, np.interp)
for these steps, so the oracle calls the same numpy routines.
"""
from __future__ import annotations

import numpy as np

# CSS colour hex codes used by the tests and by shade's default colormap.
_NAMED = {
    "lightblue": "#ADD8E6", "darkblue": "#00008B", "pink": "#FFC0CB", "red": "#FF0000",
    "white": "#FFFFFF", "black": "#000000", "blue": "#0000FF", "green": "#008000",
}


def rgb(c):
    """colors.py:82-128 -- colour name or '#RRGGBB' to an (r, g, b) tuple."""
    if isinstance(c, tuple):
        return c
    h = _NAMED.get(c, c)
    h = h.lstrip("#")
    return int(h[0:2], 16), int(h[2:4], 16), int(h[4:6], 16)


def eq_hist(data, mask=None, nbins=256 * 256):
    """transfer_functions/__init__.py:148-223.  Returns (out, discrete_levels)."""
    if mask is not None and mask.all():
        return np.full_like(data, np.nan, dtype=np.float64), 0
    sample = data if mask is None else data[~mask]
    integral = sample.dtype == bool or np.issubdtype(sample.dtype, np.integer)
    if integral and np.ptp(sample) < nbins:
        # exact per-value counts over [vmin, vmax]            (:183-191)
        values, counts = np.unique(sample, return_counts=True)
        lo, hi = values[0].item(), values[-1].item()
        centers = np.arange(lo, hi + 1)
        hist = np.zeros(hi - lo + 1, dtype=np.uint64)
        hist[values - lo] = counts
        levels = len(values)
    else:
        # binned histogram with empty bins dropped              (:192-199)
        hist, edges = np.histogram(sample, bins=nbins)
        centers = (edges[:-1] + edges[1:]) / 2
        keep = hist > 0
        levels = int(np.count_nonzero(keep))
        if levels != len(hist):
            hist = hist[keep]
            centers = centers[keep]
    cdf = hist.cumsum()
    cdf = cdf / float(cdf[-1])                                    # (:200-201)
    out = np.interp(data, centers, cdf).reshape(data.shape)      # (:202)
    if mask is not None:
        out = np.where(mask, np.nan, out)
    return out, levels


def interpolate_prologue(agg):
    """transfer_functions/__init__.py:263-293: returns (data - offset, mask)."""
    data = agg.copy()
    if data.dtype == bool:
        mask = ~data
        data = data.astype(np.int8)
    elif data.dtype.kind == "u":
        mask = data == 0
    else:
        mask = np.isnan(data)
    if mask.all():
        return None, mask
    offset = np.nanmin(data[~mask])
    data -= offset
    return data, mask


def _rescale_discrete_levels(levels, span):
    """transfer_functions/__init__.py:234-248."""
    m = -0.5 / 98.0
    c = 1.5 - 2 * m
    multiple = m * levels + c
    if multiple > 1:
        lower = max(span[1] - multiple * (span[1] - span[0]), 0)
        span = (lower, 1)
    return span


def shade_eq_hist(agg, cmap=("lightblue", "darkblue"), alpha=255, rescale_discrete_levels=False):
    """tf.shade(agg, cmap=<list>, how='eq_hist') for a 2-D aggregate -> uint32 RGBA."""
    data, mask = interpolate_prologue(agg)
    if data is None:
        return np.zeros(agg.shape, dtype=np.uint32)
    with np.errstate(invalid="ignore", divide="ignore"):
        data, levels = eq_hist(data, mask)
        masked = np.where(~mask, data, np.nan)
        span = np.nanmin(masked), np.nanmax(masked)
        if rescale_discrete_levels:
            span = _rescale_discrete_levels(levels, span)
    chans = np.array([rgb(c) for c in cmap], dtype=np.float64).T
    span = np.linspace(span[0], span[1], len(cmap))
    r = np.nan_to_num(np.interp(data, span, chans[0], left=255), copy=False).astype(np.uint8)
    g = np.nan_to_num(np.interp(data, span, chans[1], left=255), copy=False).astype(np.uint8)
    b = np.nan_to_num(np.interp(data, span, chans[2], left=255), copy=False).astype(np.uint8)
    a = np.where(np.isnan(data), 0, alpha).astype(np.uint8)
    return np.dstack([r, g, b, a]).view(np.uint32).reshape(data.shape)


_HOW = {"log": lambda d, m: np.log1p(np.where(m, np.nan, d)),          # transfer_functions/__init__.py:220-223
        "cbrt": lambda d, m: np.where(m, np.nan, d) ** (1 / 3.),
        "linear": lambda d, m: np.where(m, np.nan, d)}


def shade_interp(agg, how="linear", cmap=("lightblue", "darkblue"), alpha=255, min_alpha=40, span=None):
    """tf.shade(agg, cmap, how in {linear, log, cbrt}, span) for a 2-D uint32 or float64
    aggregate -> uint32 RGBA (transfer_functions/__init__.py:251-356).  ``cmap`` is a list
    of colours, or one colour (str or RGB tuple) for the alpha-ramp branch."""
    f = _HOW[how]
    data = agg.copy()
    mask = data == 0 if data.dtype.kind == "u" else np.isnan(data)
    if mask.all():
        return np.zeros(agg.shape, dtype=np.uint32)
    if span is None:
        offset = np.nanmin(data[~mask])
    else:
        offset = np.array(span, dtype=data.dtype)[0]
        lo, hi = np.array(span, dtype=data.dtype)
        data = np.where(mask, data, np.clip(data, lo, hi))              # masked_clip_2d
    data -= offset
    with np.errstate(invalid="ignore", divide="ignore"):
        data = f(data, mask)
        if span is None:
            masked = np.where(~mask, data, np.nan)
            span = np.nanmin(masked), np.nanmax(masked)
        else:
            span = f(np.array([0, span[1] - span[0]], dtype=np.float64), 0)
    single = isinstance(cmap, str) or (isinstance(cmap, tuple) and not isinstance(cmap[0], str))
    if not single:
        chans = np.array([rgb(c) for c in cmap], dtype=np.float64).T
        sp = np.linspace(span[0], span[1], len(cmap))
        r = np.nan_to_num(np.interp(data, sp, chans[0], left=255), copy=False).astype(np.uint8)
        g = np.nan_to_num(np.interp(data, sp, chans[1], left=255), copy=False).astype(np.uint8)
        b = np.nan_to_num(np.interp(data, sp, chans[2], left=255), copy=False).astype(np.uint8)
        a = np.where(np.isnan(data), 0, alpha).astype(np.uint8)
    else:
        color = rgb(cmap)
        aspan = np.arange(min_alpha, alpha + 1)
        sp = np.linspace(span[0], span[1], len(aspan))
        r = np.full(data.shape, color[0], dtype=np.uint8)
        g = np.full(data.shape, color[1], dtype=np.uint8)
        b = np.full(data.shape, color[2], dtype=np.uint8)
        a = np.nan_to_num(np.interp(data, sp, aspan, left=0, right=255), copy=False).astype(np.uint8)
    return np.dstack([r, g, b, a]).view(np.uint32).reshape(data.shape)
