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
import pytest

import datashader_gb300 as ds
import oracle
import refcases
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
