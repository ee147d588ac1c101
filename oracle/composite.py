"""Image compositing operators, restated with numpy -- TEST INFRASTRUCTURE.

The oracle for the GPU compositing kernel (tf.stack / tf.set_background);
only tests may import it.  Follows datashader/composite.py:

* components of a uint32 RGBA pixel as float64 in [0, 1], each byte / 255
  (extract_scaled, :31-38);
* back to uint32: each component * 255 truncated to an integer and capped
  at 255 (combine_scaled, :41-49);
* source (:77-82), over (:85-97), add (:100-111), saturate (:114-127), with
  a result alpha of 0 giving the pixel 0.

numba compiles these without FMA contraction, and numpy performs each
float64 operation separately in the same order, so the results are the
reference's bit for bit (pinned by the reference's own test_composite.py
vectors in tests/golden/composite.json).
"""
from __future__ import annotations

import numpy as np


def _components(x):
    x = np.asarray(x, dtype=np.uint32)
    return [((x >> np.uint32(s)) & np.uint32(255)).astype(np.float64) / 255 for s in (0, 8, 16, 24)]


def _pack(r, g, b, a):
    out = np.zeros(np.shape(a), dtype=np.uint32)
    for shift, c in ((0, r), (8, g), (16, b), (24, a)):
        out |= np.minimum(np.uint32(255), (c * 255).astype(np.uint32)) << np.uint32(shift)
    return out


def _finish(r, g, b, a):
    with np.errstate(divide="ignore", invalid="ignore"):
        out = _pack(np.nan_to_num(r), np.nan_to_num(g), np.nan_to_num(b), a)
    return np.where(a == 0, np.uint32(0), out).astype(np.uint32)


def source(src, dst):
    src = np.asarray(src, dtype=np.uint32)
    dst = np.broadcast_to(np.asarray(dst, dtype=np.uint32), src.shape)
    return np.where(src & np.uint32(0xFF000000), src, dst).astype(np.uint32)


def over(src, dst):
    sr, sg, sb, sa = _components(src)
    dr, dg, db, da = (np.broadcast_to(c, sa.shape) for c in _components(dst))
    factor = 1 - sa
    a = sa + da * factor
    with np.errstate(divide="ignore", invalid="ignore"):
        r = (sr * sa + dr * da * factor) / a
        g = (sg * sa + dg * da * factor) / a
        b = (sb * sa + db * da * factor) / a
    return _finish(r, g, b, a)


def add(src, dst):
    sr, sg, sb, sa = _components(src)
    dr, dg, db, da = (np.broadcast_to(c, sa.shape) for c in _components(dst))
    a = np.minimum(1.0, sa + da)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = (sr * sa + dr * da) / a
        g = (sg * sa + dg * da) / a
        b = (sb * sa + db * da) / a
    return _finish(r, g, b, a)


def saturate(src, dst):
    sr, sg, sb, sa = _components(src)
    dr, dg, db, da = (np.broadcast_to(c, sa.shape) for c in _components(dst))
    a = np.minimum(1.0, sa + da)
    factor = np.minimum(sa, 1 - da)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = (factor * sr + dr * da) / a
        g = (factor * sg + dg * da) / a
        b = (factor * sb + db * da) / a
    return _finish(r, g, b, a)


OPS = {"source": source, "over": over, "add": add, "saturate": saturate}
