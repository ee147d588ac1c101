"""Deterministic mode: sum / mean added in row order.

Bit-identical to the oracle (the reference's CPU loop adds a pixel's values
in row order) and from run to run: compared as raw float64 bit patterns.
The one documented difference: a pixel whose only values are -0.0 sums to
+0.0 (the sum starts from 0.0, as the reference's _sum_zero base does), so
the inputs here hold no negative zeros.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
import oracle
from datashader_gb300 import synthetic
from gpu_helpers import to_numpy

pytestmark = pytest.mark.gpu


def _bits(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return np.where(np.isnan(a), 0x7ff8000000000000, a.view(np.int64))


def _cols(n, seed, xdtype=np.float32):
    rng = np.random.default_rng(seed)
    x, y = synthetic.gaussian_mixture_np(n, seed=seed, dtype=xdtype)
    v = rng.lognormal(0.0, 1.0, n) * rng.choice([-1.0, 1.0], n)
    v[rng.random(n) < 0.02] = np.nan
    cat = rng.integers(0, 8, n).astype(np.int8)
    return {"x": x, "y": y, "v": v, "cat": cat}


def _frame(cols):
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in cols.items()}
    return ds.TensorFrame(t, categories={"cat": list(range(8))})


def _oracle(cols, w, h, xr, yr, specs):
    c = {k: np.asarray(v, dtype=np.float64) for k, v in cols.items()}
    return oracle.points(c, "x", "y", w, h, xr, yr, specs)


@pytest.mark.parametrize("xdtype,w,h", [(np.float32, 512, 512), (np.float64, 300, 200), (np.float32, 4096, 2160)])
def test_sum_and_mean_bit_identical_to_row_order(xdtype, w, h):
    cols = _cols(400_000, seed=11, xdtype=xdtype)
    frame = _frame(cols)
    xr, yr = (-4.0, 4.0), (-3.0, 3.5)
    cvs = ds.Canvas(plot_width=w, plot_height=h, x_range=xr, y_range=yr)
    agg = ds.summary(s=ds.sum("v"), m=ds.mean("v"), c=ds.count(), mx=ds.max("v"))
    a = to_numpy(cvs.points(frame, "x", "y", agg, deterministic=True))
    b = to_numpy(cvs.points(frame, "x", "y", agg, deterministic=True))
    rs, rm, rc, rmx = _oracle(cols, w, h, xr, yr, [oracle.spec("sum", "v"), oracle.spec("mean", "v"),
                                                   oracle.spec("count"), oracle.spec("max", "v")])
    for k in ("s", "m", "mx"):
        assert np.array_equal(_bits(a[k]), _bits(b[k])), f"run to run: {k}"
    assert np.array_equal(_bits(a["s"]), _bits(rs))
    assert np.array_equal(_bits(a["m"]), _bits(rm))
    assert np.array_equal(_bits(a["mx"]), _bits(rmx))
    np.testing.assert_array_equal(a["c"], rc)


def test_categorical_sum_and_edge_cases():
    cols = _cols(250_000, seed=12)
    frame = _frame(cols)
    xr, yr = (-3.0, 3.0), (-3.0, 3.0)
    cvs = ds.Canvas(plot_width=97, plot_height=131, x_range=xr, y_range=yr)
    got = to_numpy(cvs.points(frame, "x", "y", ds.by("cat", ds.sum("v")), deterministic=True))
    ref = _oracle(cols, 97, 131, xr, yr, [oracle.spec("sum", "v", cat="cat", ncat=8)])[0]
    assert np.array_equal(_bits(got), _bits(ref))
    # every row outside the canvas, and an empty frame
    far = ds.Canvas(plot_width=64, plot_height=64, x_range=(100.0, 101.0), y_range=(100.0, 101.0))
    out = to_numpy(far.points(frame, "x", "y", ds.sum("v"), deterministic=True))
    assert np.isnan(out).all()
    empty = _frame({k: v[:0] for k, v in cols.items()})
    out = to_numpy(cvs.points(empty, "x", "y", ds.mean("v"), deterministic=True))
    assert np.isnan(out).all()


def test_deterministic_matches_atomic_within_tolerance():
    cols = _cols(300_000, seed=13)
    cols["v"] = np.abs(cols["v"])            # positive values: the 1e-12 relative contract of sum
    frame = _frame(cols)
    cvs = ds.Canvas(plot_width=256, plot_height=256, x_range=(-4, 4), y_range=(-4, 4))
    det = to_numpy(cvs.points(frame, "x", "y", ds.sum("v"), deterministic=True))
    fast = to_numpy(cvs.points(frame, "x", "y", ds.sum("v")))
    np.testing.assert_allclose(fast, det, rtol=1e-12, atol=1e-12, equal_nan=True)
