"""GPU parity on the reference test-suite's golden cases.

Every case runs through the public API (Canvas.points / Canvas.line ->
libdsgb kernels) and is compared both with the reference's expected output
and with the CPU oracle.  Integer, index and order-independent float
results are bit-exact; antialiased float sums allow 1e-12 relative for the
float64 accumulation order and float32 aggregates 2 ulp (the reference
accumulates them in float32, the GPU in float64).
"""
from __future__ import annotations

import numpy as np
import torch
import pytest

import datashader_gb300 as ds
import oracle
import refcases
from datashader_gb300 import synthetic
from gpu_helpers import assert_same, frame_from_numpy, to_numpy
from oracle_bridge import run_line, run_points

pytestmark = pytest.mark.gpu

POINT_CASES = refcases.point_cases()
LINE_CASES = refcases.line_cases()


def _tol(exp):
    if isinstance(exp, dict):
        return 0.0, 0.0
    return 0.0, 0.0


@pytest.mark.parametrize("case", POINT_CASES, ids=[c["id"] for c in POINT_CASES])
def test_gpu_points_golden(case):
    if case["frame"] is None:
        cols, cats = refcases.pandas_frame()
    else:
        cols, cats = case["frame"], {}
    frame = frame_from_numpy(cols, cats)
    cvs = ds.Canvas(**case["canvas"])
    got = to_numpy(cvs.points(frame, case["x"], case["y"], agg=case["agg"]))
    ref = run_points(cols, cats, case["agg"], case["canvas"], case["x"], case["y"])
    exp = case["expected"]
    if isinstance(exp, dict):
        for k in exp:
            assert_same(got[k], np.asarray(exp[k]).astype(got[k].dtype), what=case["id"] + k)
    else:
        assert_same(got, np.asarray(exp).astype(got.dtype), what=case["id"])
    # sums of at most 5 small integers are exact in any order: bit-exact vs the oracle
    assert_same(got, ref, what=case["id"] + " vs oracle")


def _line_tol(got):
    if isinstance(got, np.ndarray) and got.dtype == np.float32:
        return 3e-7, 1e-7
    return 1e-12, 1e-15


@pytest.mark.parametrize("case", LINE_CASES, ids=[c["id"] for c in LINE_CASES])
def test_gpu_line_golden(case):
    cats = case.get("categories", {})
    frame = frame_from_numpy(case["frame"], cats)
    cvs = ds.Canvas(**case["canvas"])
    agg = cvs.line(frame, "x", "y", agg=case["agg"], line_width=case["line_width"])
    got = to_numpy(agg)
    ref = run_line(case["frame"], cats, case["agg"], case["canvas"], case["line_width"])
    if case["close"]:
        np.testing.assert_array_almost_equal(got, case["expected"], decimal=5)
        rtol, atol = _line_tol(got)
        assert_same(got, ref, rtol=rtol, atol=atol, what=case["id"] + " vs oracle")
    else:
        assert_same(got, np.asarray(case["expected"]).astype(got.dtype), what=case["id"])
        assert_same(got, ref, what=case["id"] + " vs oracle")


def test_gpu_eq_hist_rgba_golden():
    """test_transfer_functions.py:194-201 on the GPU: exact RGBA."""
    import torch
    a, c = refcases.eq_hist_agg_a()
    sol = refcases.golden_array(refcases.load_golden("eq_hist.json", "eq_hist_sol"))
    for data in (a, c):
        t = torch.from_numpy(data.view(np.int32) if data.dtype == np.uint32 else data).cuda()
        if data.dtype == np.uint32:
            t = t.view(torch.uint32)
        agg = ds.Aggregate(t, ["y_axis", "x_axis"], {}, {})
        img = ds.tf.shade(agg, cmap=["pink", "red"], how="eq_hist")
        got = img.data.view(torch.int32).cpu().numpy().view(np.uint32)
        np.testing.assert_array_equal(got, sol)
        np.testing.assert_array_equal(got, oracle.shade_eq_hist(data, ["pink", "red"]))


# ---- tf.shade(how='linear' | 'log' | 'cbrt') on the GPU ------------------

def _shade_gpu(data, how, cmap, span=None):
    if data.dtype == np.uint32:
        t = torch.from_numpy(data.view(np.int32)).cuda().view(torch.uint32)
    else:
        t = torch.from_numpy(data).cuda()
    agg = ds.Aggregate(t, ["y", "x"], {}, {})
    img = ds.tf.shade(agg, cmap=cmap, how=how, span=span)
    return img.data.view(torch.int32).cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("how", ["linear", "log", "cbrt"])
@pytest.mark.parametrize("span", [None, [11, 17], [11.0, 17.0]])
def test_gpu_shade_interp_golden(how, span):
    """test_transfer_functions.py:175-193 for the u4 and f8 aggregates, and the
    check_span variants (:130-149)."""
    a, c = refcases.eq_hist_agg_a()
    sol = refcases.shade_golden("solution_lists", how)
    for agg in (a, c):
        np.testing.assert_array_equal(_shade_gpu(agg, how, ["pink", "red"], span), sol)
        if span is not None:
            for x, s in refcases.span_variants(agg, sol):
                np.testing.assert_array_equal(_shade_gpu(x, how, ("#FFC0CB", "#FF0000"), span), s)


@pytest.mark.parametrize("cmap", ["black", (0, 0, 0), "#000000"])
def test_gpu_shade_single_colour_and_three_colours(cmap):
    a, _ = refcases.eq_hist_agg_a()
    sol = refcases.shade_golden("test_span_cmap_single")
    np.testing.assert_array_equal(_shade_gpu(a, "log", cmap), sol)
    for x, s in refcases.span_variants(a, sol):
        np.testing.assert_array_equal(_shade_gpu(x, "log", cmap, [11.0, 17.0]), s)
    np.testing.assert_array_equal(_shade_gpu(a, "log", ["red", (0, 255, 0), "#0000FF"]),
                                  refcases.shade_golden("test_shade_cmap"))


@pytest.mark.parametrize("how", ["linear", "log", "cbrt"])
def test_gpu_shade_large_vs_oracle(how):
    """Count and float64 aggregates of real size against the numpy restatement:
    linear bit-identical; log / cbrt call CUDA's log1p / pow and numpy the C
    library's, so a channel may differ by one step on a colour boundary."""
    rng = np.random.default_rng(3)
    cnt = rng.poisson(rng.gamma(0.5, 30.0, (700, 900))).astype(np.uint32)
    val = rng.lognormal(0.0, 2.0, (700, 900))
    val[rng.random(val.shape) < 0.3] = np.nan
    for data in (cnt, val):
        for cmap in (["lightblue", "darkblue"], ["red", (0, 255, 0), "#0000FF", "white"], "black"):
            got = _shade_gpu(data, how, cmap)
            ref = oracle.shade_interp(data, how, cmap)
            g = got.view(np.uint8).astype(int)
            r = ref.view(np.uint8).astype(int)
            if how == "linear":
                np.testing.assert_array_equal(got, ref)
            else:
                assert np.abs(g - r).max() <= 1
                assert (g != r).mean() < 1e-3
            span = (float(np.nanpercentile(data[data > 0] if data.dtype.kind == "u" else data, 20)),
                    float(np.nanpercentile(data[data > 0] if data.dtype.kind == "u" else data, 80)))
            if data.dtype.kind == "u":
                span = (int(span[0]), int(span[1]))
            got = _shade_gpu(data, how, cmap, span)
            ref = oracle.shade_interp(data, how, cmap, span=span)
            if how == "linear":
                np.testing.assert_array_equal(got, ref)
            else:
                assert np.abs(got.view(np.uint8).astype(int) - ref.view(np.uint8).astype(int)).max() <= 1


AA_IMAGE_CASES = refcases.antialias_image_cases()


@pytest.mark.parametrize("case", AA_IMAGE_CASES, ids=[c["id"] for c in AA_IMAGE_CASES])
def test_gpu_antialias_images(case):
    """test_antialias.py::test_antialiasing through the GPU path: each line's
    Canvas.line(max('val')) aggregate, their NaN-skipping sum (the test's own
    xr.concat(...).sum('stack'), host glue), tf.shade with the 50-colour binary
    colormap (eq_hist) and set_background white; exactly the reference's PNG."""
    cvs = ds.Canvas(**case["canvas"])
    aggs = [to_numpy(cvs.line(frame_from_numpy(f), "x", "y", agg=ds.max("val"), line_width=case["line_width"]))
            for f in case["frames"]]
    total = torch.from_numpy(refcases.stack_sum(aggs)).cuda()
    agg = ds.Aggregate(total, ["y", "x"], {}, dict(x_range=case["canvas"]["x_range"], y_range=case["canvas"]["y_range"]))
    img = ds.tf.set_background(ds.tf.shade(agg, cmap=refcases.binary_cmap50()), "#ffffff")
    got = img.data.view(torch.int32).cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(got, case["expected"], err_msg=case["id"])


def test_gpu_shade_bool_golden():
    """test_shade_bool (test_transfer_functions.py:260-272): a bool aggregate, every
    `how`, cmap ['pink', 'red'] -> opaque red where True, transparent elsewhere."""
    data = ~np.eye(3, dtype=bool)
    agg = ds.Aggregate(torch.from_numpy(data).cuda(), ["y", "x"], {}, {})
    sol = np.where(data, 4278190335, 0).astype(np.uint32)
    for how in ("log", "cbrt", "linear", "eq_hist"):
        img = ds.tf.shade(agg, cmap=["pink", "red"], how=how)
        np.testing.assert_array_equal(img.data.view(torch.int32).cpu().numpy().view(np.uint32), sol, err_msg=how)


@pytest.mark.parametrize("how", ["linear", "log", "cbrt", "eq_hist"])
def test_gpu_shade_float32_line_aggregate(how):
    """Shading the float32 aggregate of an antialiased line count: against the
    oracle's numpy restatement run on the float32 array itself, within one colour
    step per channel (the reference's float32 offset / log1p / cbrt steps)."""
    x, y, v, _ = synthetic.time_series_np(20, 300, seed=5)
    agg = ds.Canvas(plot_width=160, plot_height=90).line(frame_from_numpy({"x": x, "y": y}), "x", "y",
                                                         agg=ds.count(), line_width=1.5)
    assert agg.data.dtype == torch.float32
    img = ds.tf.shade(agg, cmap=["lightblue", "darkblue"], how=how)
    got = img.data.view(torch.int32).cpu().numpy().view(np.uint32)
    a = agg.data.cpu().numpy()
    ref = (oracle.shade_eq_hist(a, ["lightblue", "darkblue"]) if how == "eq_hist"
           else oracle.shade_interp(a, how=how, cmap=["lightblue", "darkblue"]))
    g8, r8 = got.view(np.uint8).astype(int), ref.view(np.uint8).astype(int)
    assert np.abs(g8 - r8).max() <= 1
    assert (got != ref).mean() < 0.01
