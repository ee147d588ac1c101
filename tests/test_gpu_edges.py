"""Degenerate inputs on every GPU path, each against the oracle: no rows, one row,
rows that are all NaN, zero-length and axis-parallel segments, segments along the
canvas border or far outside it, ragged rows of zero and one vertex, and
aggregates that shade to nothing or to a single level.

Tolerances as the parity tests: integer / index / min / max / first / last /
where bit-exact; float64 sums 1e-12 relative; float32 antialiased counts 3e-7."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
import oracle
from gpu_helpers import assert_same, frame_from_numpy, to_numpy
from oracle_bridge import run_line, run_points

pytestmark = pytest.mark.gpu

RTOL_SUM = 1e-12

NAN = np.nan
LINE_CASES = {
    "empty": ([], []),
    "one_row": ([0.3], [0.4]),
    "two_rows": ([0.1, 0.9], [0.2, 0.8]),
    "all_nan": ([NAN, NAN, NAN], [NAN, NAN, NAN]),
    "nan_ends": ([NAN, 0.1, 0.5, 0.9, NAN], [0.5, 0.2, 0.7, 0.3, 0.1]),
    "nan_every_other": ([0.1, NAN, 0.3, NAN, 0.5, 0.6], [0.1, 0.9, NAN, 0.2, 0.5, 0.9]),
    "zero_length": ([0.5, 0.5, 0.5, 0.7], [0.5, 0.5, 0.5, 0.7]),
    "axis_parallel": ([0.1, 0.9, 0.9, 0.1, 0.1], [0.1, 0.1, 0.9, 0.9, 0.1]),
    "on_border": ([0.0, 1.0, 1.0, 0.0, 0.0], [0.0, 0.0, 1.0, 1.0, 0.0]),
    "outside": ([-3.0, -2.0, 5.0, 6.0], [-3.0, 4.0, -2.0, 7.0]),
    "crossing_far": ([-1e12, 1e12, 0.5, 0.5], [0.5, 0.5, -1e12, 1e12]),
    "steep_shallow": ([0.0, 0.01, 1.0, 0.99], [0.0, 1.0, 0.0, 1.0]),
}


def _line_cols(name):
    x, y = (np.asarray(v, dtype=np.float64) for v in LINE_CASES[name])
    v = np.linspace(0.25, 2.0, x.size)
    if x.size > 2:
        v[1] = NAN
    return {"x": x, "y": y, "v": v}


@pytest.mark.parametrize("name", sorted(LINE_CASES))
def test_line_axis0_degenerate_bresenham(name):
    cols = _line_cols(name)
    canvas = dict(plot_width=23, plot_height=17, x_range=(0.0, 1.0), y_range=(0.0, 1.0))
    agg = ds.summary(c=ds.count(), s=ds.sum("v"), mx=ds.max("v"), mn=ds.min("v"), f=ds.first("v"),
                     l=ds.last("v"), w=ds.where(ds.max("v")), a=ds.any())
    got = to_numpy(ds.Canvas(**canvas).line(frame_from_numpy(cols), "x", "y", agg=agg))
    ref = run_line(cols, {}, agg, canvas, 0)
    for k in ref:
        assert_same(got[k], ref[k], rtol=RTOL_SUM if k == "s" else 0.0, what=f"{name} {k}")


@pytest.mark.parametrize("name", sorted(LINE_CASES))
@pytest.mark.parametrize("aggname", ["sum", "count", "max", "first_2stage"])
def test_line_axis0_degenerate_antialiased(name, aggname):
    cols = _line_cols(name)
    canvas = dict(plot_width=23, plot_height=17, x_range=(0.0, 1.0), y_range=(0.0, 1.0))
    agg = {"sum": ds.sum("v"), "count": ds.count(), "max": ds.max("v"), "first_2stage": ds.first("v")}[aggname]
    got = to_numpy(ds.Canvas(**canvas).line(frame_from_numpy(cols), "x", "y", agg=agg, line_width=1.5))
    ref = run_line(cols, {}, agg, canvas, 1.5)
    if ref.dtype == np.float32:
        assert_same(got, ref, rtol=3e-7, atol=1e-7, what=name)
    else:
        assert_same(got, ref, rtol=RTOL_SUM, atol=1e-13, what=name)


@pytest.mark.parametrize("name", ["empty", "one_row", "all_nan"])
def test_line_axis0_degenerate_autorange(name):
    """Bounds of no finite value expand to (-1, 1) (glyph.py:42-49)."""
    cols = _line_cols(name)
    got = ds.Canvas(plot_width=11, plot_height=7).line(frame_from_numpy(cols), "x", "y", agg=ds.count())
    ref = run_line(cols, {}, ds.count(), dict(plot_width=11, plot_height=7), 0)
    assert_same(to_numpy(got), ref, what=name)


@pytest.mark.parametrize("nrows", [0, 1, 2])
def test_multi_lines_few_rows(nrows):
    rng = np.random.default_rng(nrows)
    cols = {f"x{j}": rng.uniform(0, 1, nrows) for j in range(3)}
    cols.update({f"y{j}": rng.uniform(0, 1, nrows) for j in range(3)})
    cols["v"] = rng.uniform(0, 1, nrows)
    frame = ds.TensorFrame({k: torch.from_numpy(v).cuda() for k, v in cols.items()})
    cvs = ds.Canvas(plot_width=13, plot_height=9, x_range=(0.0, 1.0), y_range=(0.0, 1.0))
    xs = np.stack([cols[f"x{j}"] for j in range(3)], axis=1).reshape(nrows, 3)
    ys = np.stack([cols[f"y{j}"] for j in range(3)], axis=1).reshape(nrows, 3)
    for axis, layout, kx, ky in ((0, 1, xs, ys), (1, 2, xs, ys)):
        agg = ds.summary(c=ds.count(), f=ds.first("v"), s=ds.sum("v"))
        got = to_numpy(cvs.line(frame, x=[f"x{j}" for j in range(3)], y=[f"y{j}" for j in range(3)], axis=axis,
                                agg=agg))
        ref = oracle.lines({"v": cols["v"]}, layout, kx, ky, 13, 9, (0.0, 1.0), (0.0, 1.0),
                           [oracle.spec("count"), oracle.spec("first", "v"), oracle.spec("sum", "v")])
        for k, r in zip(("c", "f", "s"), ref):
            assert_same(got[k], r, rtol=RTOL_SUM if k == "s" else 0.0, what=f"axis={axis} {k}")


def test_lines_axis1_single_vertex_rows():
    """One vertex a row: no segment, an empty canvas."""
    ys = np.array([[0.2], [0.7]])
    xs = np.array([[0.3], [0.6]])
    frame = ds.TensorFrame({"x0": torch.from_numpy(xs[:, 0]).cuda(), "y0": torch.from_numpy(ys[:, 0]).cuda()})
    cvs = ds.Canvas(plot_width=5, plot_height=5, x_range=(0.0, 1.0), y_range=(0.0, 1.0))
    got = to_numpy(cvs.line(frame, x=["x0"], y=["y0"], axis=1, agg=ds.count()))
    ref = oracle.lines({}, 2, xs, ys, 5, 5, (0.0, 1.0), (0.0, 1.0), [oracle.spec("count")])[0]
    assert_same(got, ref)
    assert not got.any()


@pytest.mark.parametrize("lw", [0.0, 1.5])
def test_ragged_degenerate_rows(lw):
    xr = [[], [0.5], [0.1, 0.9], [NAN, 0.2, 0.4, NAN], [], [0.3, 0.3], [0.0, 1.0, 1.0]]
    yr = [[], [0.5], [0.9, 0.1], [0.5, NAN, 0.4, 0.6], [], [0.3, 0.3], [0.0, 0.0, 1.0]]
    v = np.array([1.0, 2.0, 3.0, NAN, 5.0, 6.0, 7.0])
    frame = ds.TensorFrame({"x": ds.RaggedColumn(xr), "y": ds.RaggedColumn(yr),
                            "v": torch.from_numpy(v).cuda()})
    cvs = ds.Canvas(plot_width=12, plot_height=10, x_range=(0.0, 1.0), y_range=(0.0, 1.0))
    for red, spec in ((ds.count(), oracle.spec("count")), (ds.sum("v"), oracle.spec("sum", "v"))):
        got = to_numpy(cvs.line(frame, x="x", y="y", axis=1, agg=red, line_width=lw))
        ref = oracle.lines_ragged({"v": v}, xr, yr, 12, 10, (0.0, 1.0), (0.0, 1.0), [spec], line_width=lw)[0]
        if ref.dtype == np.float32:
            assert_same(got, ref, rtol=3e-7, atol=1e-7)
        else:
            assert_same(got, ref, rtol=RTOL_SUM)


def test_ragged_all_rows_empty():
    frame = ds.TensorFrame({"x": ds.RaggedColumn([[], []]), "y": ds.RaggedColumn([[], []])})
    cvs = ds.Canvas(plot_width=6, plot_height=4, x_range=(0.0, 1.0), y_range=(0.0, 1.0))
    got = to_numpy(cvs.line(frame, x="x", y="y", axis=1, agg=ds.count()))
    assert got.shape == (4, 6) and not got.any()


@pytest.mark.parametrize("n", [1, 2, 3, 5])
def test_points_fewer_rows_than_a_vector(n):
    """Row counts below and around one float4: the scalar tail of every kernel."""
    rng = np.random.default_rng(n)
    cols = {"x": rng.uniform(-1, 1, n).astype(np.float32), "y": rng.uniform(-1, 1, n).astype(np.float32),
            "v": rng.uniform(0, 1, n)}
    canvas = dict(plot_width=7, plot_height=5, x_range=(-1.0, 1.0), y_range=(-1.0, 1.0))
    agg = ds.summary(c=ds.count(), s=ds.sum("v"), m=ds.mean("v"), l=ds.last("v"), w=ds.where(ds.min("v")))
    got = to_numpy(ds.Canvas(**canvas).points(frame_from_numpy(cols), "x", "y", agg))
    ref = run_points(cols, {}, agg, canvas)
    for k in ref:
        assert_same(got[k], ref[k], rtol=RTOL_SUM if k in ("s", "m") else 0.0, what=k)


def test_points_all_nan_coordinates():
    n = 4099
    cols = {"x": np.full(n, np.nan, np.float32), "y": np.zeros(n, np.float32), "v": np.ones(n)}
    canvas = dict(plot_width=8, plot_height=8, x_range=(-1.0, 1.0), y_range=(-1.0, 1.0))
    got = to_numpy(ds.Canvas(**canvas).points(frame_from_numpy(cols), "x", "y", ds.summary(c=ds.count(),
                                                                                          m=ds.mean("v"))))
    assert not got["c"].any() and np.isnan(got["m"]).all()


@pytest.mark.parametrize("kind", ["all_zero", "one_pixel", "two_levels", "float_constant", "float_all_nan"])
def test_eq_hist_degenerate_aggregates(kind):
    a = {"all_zero": np.zeros((9, 11), np.uint32),
         "one_pixel": np.zeros((9, 11), np.uint32),
         "two_levels": np.where(np.arange(99).reshape(9, 11) % 3 == 0, 5, 2).astype(np.uint32),
         "float_constant": np.where(np.arange(99).reshape(9, 11) % 2 == 0, 1.5, np.nan),
         "float_all_nan": np.full((9, 11), np.nan)}[kind]
    if kind == "one_pixel":
        a[4, 5] = 7
    if a.dtype == np.uint32:
        t = torch.from_numpy(a.view(np.int32)).cuda().view(torch.uint32)
    else:
        t = torch.from_numpy(a).cuda()
    agg = ds.Aggregate(t, ["y", "x"], {}, dict(x_range=(0.0, 1.0), y_range=(0.0, 1.0)))
    img = ds.tf.shade(agg, cmap=["lightblue", "darkblue"], how="eq_hist")
    got = img.data.view(torch.int32).cpu().numpy().view(np.uint32)
    assert_same(got, oracle.shade_eq_hist(a, ["lightblue", "darkblue"]), what=kind)
