"""Parity at the benchmark configurations' full sizes, against the oracle.

* 1e7 float64 points on 512x512, count (the CPU-runnable configuration);
* 1e8 float32 points on 1024x1024 (the headline configuration): count and
  mean through the hot-tile kernels, the whole reduction set of the
  configuration (count, sum, mean, max, min, first, where(max('v')) as a row
  index and with an 'index' lookup column, by('cat', count())), and
  tf.shade(how='eq_hist') of the count;
* the differentiation workload: Canvas.line of 1000 series x 10,000 float64
  vertices on 1024x512, sum('v'), line_width 1.5 -- the forward against the
  oracle, and the adjoint against central differences of the GPU forward at
  64 random coordinates.

The oracle runs on one row partition per host thread and folds the
partitions' bases as datashader's dask path does (oracle.points_parallel).
Tolerances as everywhere: integer, index, min / max / first / where /
by-count results and eq_hist exact; float64 sums and means 1e-12 relative.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
import oracle
from datashader_gb300 import autograd as ag
from datashader_gb300 import synthetic
from gpu_helpers import assert_same, to_numpy
from oracle_bridge import specs_of

pytestmark = pytest.mark.gpu

RTOL_SUM = 1e-12
N2 = 100_000_000


def _oracle(cols, cats, agg, width, height, x_range, y_range):
    keys, specs, extra = specs_of(agg, cols, cats)
    c = dict(cols)
    for k, v in c.items():
        if k not in ("x", "y"):
            c[k] = np.asarray(v, dtype=np.float64)
    c.update(extra)
    res = oracle.points_parallel(c, "x", "y", width, height, x_range, y_range, specs)
    return res[0] if keys == [None] else dict(zip(keys, res))


@pytest.fixture(scope="module")
def cfg2():
    """1e8 rows: x, y float32 (5-Gaussian mixture), v float64 lognormal with 1 %
    NaN, cat int8 over 8 categories, index int64 = row number."""
    x, y = synthetic.gaussian_mixture_np(N2, seed=0, dtype=np.float32)
    rng = np.random.default_rng(1)
    v = rng.lognormal(0.0, 1.0, N2)
    v[rng.integers(0, N2, N2 // 100)] = np.nan
    cat = rng.integers(0, 8, N2).astype(np.int8)
    index = np.arange(N2, dtype=np.int64)
    cols = {"x": x, "y": y, "v": v, "cat": cat, "index": index}
    cats = {"cat": list(range(8))}
    frame = ds.TensorFrame({k: torch.from_numpy(a).cuda() for k, a in cols.items()}, categories=cats)
    yield cols, cats, frame
    del frame
    torch.cuda.empty_cache()


CANVAS2 = dict(plot_width=1024, plot_height=1024, x_range=(-4, 4), y_range=(-4, 4))


def test_cfg1_count_full_size():
    x, y = synthetic.gaussian_mixture_np(10_000_000, seed=0, dtype=np.float64)
    frame = ds.TensorFrame({"x": torch.from_numpy(x).cuda(), "y": torch.from_numpy(y).cuda()})
    got = to_numpy(ds.Canvas(plot_width=512, plot_height=512, x_range=(-4, 4), y_range=(-4, 4)).points(
        frame, "x", "y", ds.count()))
    ref = _oracle({"x": x, "y": y}, {}, ds.count(), 512, 512, (-4, 4), (-4, 4))
    assert got.sum() == ref.sum() > 9_000_000
    assert_same(got, ref)


def test_cfg2_count_full_size(cfg2):
    cols, cats, frame = cfg2
    got = to_numpy(ds.Canvas(**CANVAS2).points(frame, "x", "y", ds.count()))
    ref = _oracle({"x": cols["x"], "y": cols["y"]}, {}, ds.count(), 1024, 1024, (-4, 4), (-4, 4))
    assert ref.sum() > 0.95 * N2
    assert_same(got, ref)


def test_cfg2_mean_full_size(cfg2):
    cols, cats, frame = cfg2
    got = to_numpy(ds.Canvas(**CANVAS2).points(frame, "x", "y", ds.mean("v")))
    ref = _oracle({"x": cols["x"], "y": cols["y"], "v": cols["v"]}, {}, ds.mean("v"), 1024, 1024, (-4, 4), (-4, 4))
    assert_same(got, ref, rtol=RTOL_SUM)


def test_cfg2_reduction_set_full_size(cfg2):
    cols, cats, frame = cfg2
    agg = ds.summary(count=ds.count(), sum=ds.sum("v"), mean=ds.mean("v"), max=ds.max("v"), min=ds.min("v"),
                     first=ds.first("v"), where_row=ds.where(ds.max("v")),
                     where_index=ds.where(ds.max("v"), "index"), by_cat=ds.by("cat", ds.count()))
    got = to_numpy(ds.Canvas(**CANVAS2).points(frame, "x", "y", agg))
    ref = _oracle(cols, cats, agg, 1024, 1024, (-4, 4), (-4, 4))
    for k in ("count", "max", "min", "first", "where_row", "where_index", "by_cat"):
        assert_same(got[k], ref[k], what=k)
    for k in ("sum", "mean"):
        assert_same(got[k], ref[k], rtol=RTOL_SUM, what=k)
    assert (got["where_row"] >= 0).sum() > 0.5 * (got["count"] > 0).sum()


def test_gpu_eq_hist_rescale_discrete_levels_golden():
    """test_transfer_functions.py:113-120, 199-201: shade(how='eq_hist',
    rescale_discrete_levels=True) on the reference's u4 and f8 aggregates,
    within 1 per channel of its solution (the reference's own tolerance) and
    equal to the oracle."""
    import refcases
    a, c = refcases.eq_hist_agg_a()
    g = refcases.load_golden("eq_hist.json", "eq_hist_sol_rescale_discrete_levels")
    for data, key in ((a, "a"), (c, "c")):
        t = torch.from_numpy(data.view(np.int32) if data.dtype == np.uint32 else data).cuda()
        if data.dtype == np.uint32:
            t = t.view(torch.uint32)
        img = ds.tf.shade(ds.Aggregate(t, ["y_axis", "x_axis"], {}, {}), cmap=["pink", "red"], how="eq_hist",
                          rescale_discrete_levels=True)
        got = img.data.view(torch.int32).cpu().numpy().view(np.uint32)
        sol = refcases.golden_array(g[key])
        assert np.abs(got.view(np.uint8).astype(int) - sol.view(np.uint8).astype(int)).max() <= 1
        assert_same(got, oracle.shade_eq_hist(data, ["pink", "red"], rescale_discrete_levels=True))


def test_cfg2_eq_hist_full_size(cfg2):
    cols, cats, frame = cfg2
    agg = ds.Canvas(**CANVAS2).points(frame, "x", "y", ds.count())
    data = to_numpy(agg)
    out, levels = ds.tf.eq_hist_agg(agg)
    pro, mask = oracle.interpolate_prologue(data)
    ref, ref_levels = oracle.eq_hist(pro, mask)
    assert levels == ref_levels
    assert_same(out.cpu().numpy(), ref)
    img = ds.tf.shade(agg, cmap=["lightblue", "darkblue"], how="eq_hist")
    got = img.data.view(torch.int32).cpu().numpy().view(np.uint32)
    assert_same(got, oracle.shade_eq_hist(data, ["lightblue", "darkblue"]))


@pytest.fixture(scope="module")
def cfg3():
    x, y, v, _ = synthetic.time_series_np(1000, 10_000, seed=0)
    X, Y, V = (torch.from_numpy(a).cuda() for a in (x, y, v))
    agg = ds.Canvas(plot_width=1024, plot_height=512, x_range=(0.0, 1.0)).line(
        ds.TensorFrame({"x": X, "y": Y, "v": V}), "x", "y", agg=ds.sum("v"), line_width=1.5)
    cvs = ds.Canvas(plot_width=1024, plot_height=512, x_range=(0.0, 1.0), y_range=tuple(agg.attrs["y_range"]))
    yield x, y, v, X, Y, V, agg, cvs


def test_cfg3_line_forward_full_size(cfg3):
    x, y, v, X, Y, V, agg, cvs = cfg3
    ref = oracle.line_axis0({"x": x, "y": y, "v": v}, "x", "y", 1024, 512, cvs.x_range, cvs.y_range,
                            [oracle.spec("sum", "v")], line_width=1.5)[0]
    assert_same(to_numpy(agg), ref, rtol=RTOL_SUM)


def test_cfg3_adjoint_full_size(cfg3):
    """dL/dy and dL/dv of L = mean((nan_to_num(agg) - target)^2) at 64 random
    coordinates (32 y, 32 v) against central differences of the GPU forward.

    The differences are taken over the pixel columns a vertex can reach
    (its segments span under a pixel in x): the float64 atomics of the other
    512k pixels add in a different order on each forward, and that rounding,
    summed over the whole canvas, would swamp a one-vertex difference."""
    x, y, v, X, Y, V, agg, cvs = cfg3
    rng = np.random.default_rng(7)
    YT = torch.from_numpy(y + rng.normal(0.0, 0.005, y.shape)).cuda()
    target = torch.nan_to_num(ag.line_sum(X, YT, V, cvs)).detach()
    Yg, Vg = Y.clone().requires_grad_(True), V.clone().requires_grad_(True)
    npx = 1024 * 512
    loss = torch.mean((torch.nan_to_num(ag.line_sum(X, Yg, Vg, cvs)) - target) ** 2)
    loss.backward()
    gy, gv = Yg.grad.cpu().numpy(), Vg.grad.cpu().numpy()
    valid = np.flatnonzero(~np.isnan(y))
    picks = rng.choice(valid, 64, replace=False)
    sx = 1024.0 / (cvs.x_range[1] - cvs.x_range[0])

    def window_loss(which, k, d):
        arr = (Y if which == "y" else V).clone()
        arr[k] += d
        yy, vv = (arr, V) if which == "y" else (Y, arr)
        a = torch.nan_to_num(ag.line_sum(X, yy, vv, cvs))
        c = int(x[k] * sx)
        lo, hi = max(0, c - 4), min(1024, c + 5)
        return float(((a[:, lo:hi] - target[:, lo:hi]) ** 2).sum()) / npx

    kinks, checked = [], 0
    for which, grad in (("y", gy), ("v", gv)):
        for k in (picks[:32] if which == "y" else picks[32:]):
            h = 1e-6 if which == "y" else 1e-3
            f0 = window_loss(which, k, 0.0)
            fp, fm = window_loss(which, k, h), window_loss(which, k, -h)
            central = (fp - fm) / (2 * h)
            scale = max(abs(central), abs(grad[k]), 1e-14)
            if which == "y":
                a1 = (fp + fm - 2 * f0) / h
                q = h / 8
                a2 = (window_loss(which, k, q) + window_loss(which, k, -q) - 2 * f0) / q
                if abs(a2) > 0.5 * abs(a1) and abs(a1) > 1e-6 * scale:
                    kinks.append(int(k))
                    continue
            checked += 1
            assert abs(grad[k] - central) <= 1e-4 * scale + 1e-13, (which, int(k), grad[k], central)
    assert checked >= 56, f"too many kink coordinates: {kinks}"
