"""Pin the CPU oracle against the reference test-suite's golden vectors (no GPU)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import refcases
from oracle_bridge import run_line, run_points

POINT_CASES = refcases.point_cases()
LINE_CASES = refcases.line_cases()


def _check(got, exp, close):
    if isinstance(exp, dict):
        assert sorted(got) == sorted(exp)
        for k in exp:
            _check(got[k], exp[k], close)
        return
    got = np.asarray(got)
    assert got.shape == np.shape(exp)
    if close:
        # the reference's assert_eq_ndarray(close=True): 5 decimals
        np.testing.assert_array_almost_equal(got, exp, decimal=5)
    else:
        np.testing.assert_array_equal(got, exp)


@pytest.mark.parametrize("case", POINT_CASES, ids=[c["id"] for c in POINT_CASES])
def test_oracle_points_golden(case):
    if case["frame"] is None:
        cols, cats = refcases.pandas_frame()
    else:
        cols, cats = case["frame"], {}
    got = run_points(cols, cats, case["agg"], case["canvas"], case["x"], case["y"])
    _check(got, case["expected"], case["close"])


@pytest.mark.parametrize("case", LINE_CASES, ids=[c["id"] for c in LINE_CASES])
def test_oracle_line_golden(case):
    got = run_line(case["frame"], case.get("categories", {}), case["agg"], case["canvas"], case["line_width"])
    _check(got, case["expected"], case["close"])


@pytest.mark.parametrize("high", [9, 10, 99, 100])
def test_oracle_uniform_diagonal_points(high):
    """test_pandas.py:1147-1168."""
    import datashader_gb300 as ds
    low = 0
    width = height = high - low
    n = width * height
    cols = {"time": np.ones(n, dtype="i4"),
            "x": np.array([np.arange(low, high, dtype="f8")] * width).flatten(),
            "y": np.array([np.arange(low, high, dtype="f8")] * height).flatten()}
    agg = run_points(cols, {}, ds.count("time"),
                     dict(plot_width=2, plot_height=2, x_range=(low, high), y_range=(low, high)))
    diagonal = agg.diagonal(0)
    assert diagonal.sum() == n
    assert abs(high - low) % 2 == abs(diagonal[1] / high - diagonal[0] / high)


def _eq_sol(name):
    return refcases.golden_array(refcases.load_golden("eq_hist.json", name))


def test_oracle_eq_hist_rgba_golden():
    """test_transfer_functions.py:194-201: shade(how='eq_hist') exact RGBA for u4 and f8 aggs."""
    a, c = refcases.eq_hist_agg_a()
    sol = _eq_sol("eq_hist_sol")
    cmap = ["pink", "red"]
    np.testing.assert_array_equal(oracle.shade_eq_hist(a, cmap), sol)
    np.testing.assert_array_equal(oracle.shade_eq_hist(c, cmap), sol)


def test_oracle_eq_hist_rescale_golden():
    """test_transfer_functions.py:113-120, 199-201 (tolerance 1 per channel)."""
    a, c = refcases.eq_hist_agg_a()
    g = refcases.load_golden("eq_hist.json", "eq_hist_sol_rescale_discrete_levels")
    for data, key in ((a, "a"), (c, "c")):
        sol = refcases.golden_array(g[key]).view(np.uint8).astype(int)
        got = oracle.shade_eq_hist(data, ["pink", "red"], rescale_discrete_levels=True).view(np.uint8).astype(int)
        assert np.abs(got - sol).max() <= 1


def _check_cdf_slope(eq):
    """test_transfer_functions.py:1131-1137."""
    cdf = np.histogram(eq[~np.isnan(eq)], bins=256)[0].cumsum()
    cdf = cdf / cdf[-1]
    slope = np.polyfit(np.linspace(0, 1, cdf.size), cdf, 1)[0]
    assert 0.9 < slope < 1.1


def test_oracle_eq_hist_slope(rng):
    """test_transfer_functions.py:1140-1153."""
    data = rng.normal(size=300 ** 2)
    data[rng.integers(300 ** 2, size=100)] = np.nan
    data = (data - np.nanmin(data)).reshape((300, 300))
    mask = np.isnan(data)
    eq, _ = oracle.eq_hist(data, mask)
    _check_cdf_slope(eq)
    assert (np.isnan(eq) == mask).all()
    data = rng.normal(scale=100, size=(300, 300)).astype("i8")
    data = data - data.min()
    eq, _ = oracle.eq_hist(data)
    _check_cdf_slope(eq)


def test_oracle_mutation_is_caught():
    """A mistake planted in the oracle's inputs must change the golden comparison."""
    import datashader_gb300 as ds
    cols, cats = refcases.pandas_frame()
    cols = dict(cols)
    cols["x"] = cols["x"].copy()
    cols["x"][0] = 1.0           # move one row to the other column of pixels
    got = run_points(cols, cats, ds.count(), refcases.C2)
    assert not np.array_equal(got, np.array([[5, 5], [5, 5]]))


# ---- tf.shade(how='linear' | 'log' | 'cbrt') -----------------------------

@pytest.mark.parametrize("how", ["linear", "log", "cbrt"])
@pytest.mark.parametrize("span", [None, [11, 17], [11.0, 17.0]])
def test_oracle_shade_interp_golden(how, span):
    """test_transfer_functions.py:175-193 (test_shade) for the u4 and f8 aggregates."""
    a, c = refcases.eq_hist_agg_a()
    sol = refcases.shade_golden("solution_lists", how)
    for agg in (a, c):
        np.testing.assert_array_equal(oracle.shade_interp(agg, how, ["pink", "red"], span=span), sol)


@pytest.mark.parametrize("how", ["linear", "log", "cbrt"])
@pytest.mark.parametrize("cmap", [["pink", "red"], ("#FFC0CB", "#FF0000")])
def test_oracle_shade_span_cmap_list(how, cmap):
    """test_span_cmap_list / check_span (test_transfer_functions.py:130-149, 214-222)."""
    a, c = refcases.eq_hist_agg_a()
    for agg in (a, c):
        for x, sol in refcases.span_variants(agg, refcases.shade_golden("solution_lists", how)):
            np.testing.assert_array_equal(oracle.shade_interp(x, how, cmap, span=[11.0, 17.0]), sol)


@pytest.mark.parametrize("cmap", ["black", (0, 0, 0), "#000000"])
def test_oracle_shade_single_colour(cmap):
    """test_span_cmap_single and test_shade_cmap_non_categorical_alpha (:225-239, 282-290)."""
    a, _ = refcases.eq_hist_agg_a()
    sol = refcases.shade_golden("test_span_cmap_single")
    np.testing.assert_array_equal(oracle.shade_interp(a, "log", cmap), sol)
    for x, s in refcases.span_variants(a, sol):
        np.testing.assert_array_equal(oracle.shade_interp(x, "log", cmap, span=[11.0, 17.0]), s)


def test_oracle_shade_three_colours():
    """test_shade_cmap (:272-279)."""
    a, _ = refcases.eq_hist_agg_a()
    np.testing.assert_array_equal(oracle.shade_interp(a, "log", ["red", (0, 255, 0), "#0000FF"]),
                                  refcases.shade_golden("test_shade_cmap"))


# ---- multi-line glyphs (LineAxis0Multi, LinesAxis1 / XConstant / YConstant) ----

def test_oracle_multi_line_manual_range_golden():
    """test_pandas.py:1654-1749 (test_line_manual_range), every case incl. ragged arrays: count on 7x7."""
    sol = refcases.golden_array(refcases.lines_golden("test_line_manual_range")[0])
    for case in refcases.lines_golden("line_manual_range_params")["cases"]:
        if case.get("ragged"):
            c = case["columns"]
            got = oracle.lines_ragged({}, c["x"], c["y"], 7, 7, (-3, 3), (-3, 3), [oracle.spec("count")])[0]
            np.testing.assert_array_equal(got, sol, err_msg="ragged")
            continue
        layout, xs, ys = refcases.multi_line_arrays(case["columns"], case["kwargs"])
        got = oracle.lines({}, layout, xs, ys, 7, 7, (-3, 3), (-3, 3), [oracle.spec("count")])[0]
        np.testing.assert_array_equal(got, sol, err_msg=str(case["kwargs"]))


@pytest.mark.parametrize("line_width", [0, 1])
def test_oracle_multi_line_autorange_golden(line_width):
    """test_pandas.py:1752-1860 (test_line_autorange): count, autoranged 9x9, lw 0 and 1."""
    sols = refcases.lines_golden("test_line_autorange")
    sol = refcases.golden_array(sols[0] if line_width else sols[1])
    for case in refcases.lines_golden("line_autorange_params")["cases"]:
        if case.get("ragged"):
            c = case["columns"]
            got = oracle.lines_ragged({}, c["x"], c["y"], 9, 9, None, None, [oracle.spec("count")],
                                      line_width=line_width)[0]
        else:
            layout, xs, ys = refcases.multi_line_arrays(case["columns"], case["kwargs"])
            got = oracle.lines({}, layout, xs, ys, 9, 9, None, None, [oracle.spec("count")],
                               line_width=line_width)[0]
        if line_width:
            np.testing.assert_allclose(got, sol, rtol=1e-6, atol=1e-6, equal_nan=True)
        else:
            np.testing.assert_array_equal(got, sol)


def test_oracle_axis1_x_constant_and_sum_golden():
    """test_pandas.py:1863-1932: LinesAxis1XConstant autorange count; LinesAxis1 sum('v')
    (the frame of test_line_agg_sum_axis1_none_constant is the axis1 manual-range case plus
    v = [7, 9])."""
    sol = refcases.golden_array(refcases.lines_golden("test_line_autorange_axis1_x_constant")[0])
    cols = {"y0": [0.0, 0.0], "y1": [-4.0, 4.0], "y2": [0.0, 0.0]}
    layout, xs, ys = refcases.multi_line_arrays(cols, {"x": {"array": [-4, 0, 4]}, "y": ["y0", "y1", "y2"],
                                                       "axis": 1})
    got = oracle.lines({}, layout, xs, ys, 9, 9, None, None, [oracle.spec("count")])[0]
    np.testing.assert_array_equal(got, sol)
    case = refcases.lines_golden("line_manual_range_params")["cases"][0]
    cols = dict(case["columns"], v=[7.0, 9.0])
    layout, xs, ys = refcases.multi_line_arrays(cols, case["kwargs"])
    got = oracle.lines({"v": np.array([7.0, 9.0])}, layout, xs, ys, 7, 7, (-3, 3), (-3, 3),
                       [oracle.spec("sum", "v")])[0]
    sol = refcases.golden_array(refcases.lines_golden("test_line_agg_sum_axis1_none_constant")[0])
    np.testing.assert_array_equal(got, sol)


BOTH_SRC, BOTH_CANVAS, BOTH_CASES = refcases.both_lines_cases()


@pytest.mark.parametrize("case", BOTH_CASES, ids=[c["id"] for c in BOTH_CASES])
def test_oracle_both_lines_golden(case):
    """Two lines as LineAxis0Multi at line_width 1, including the two-stage plans
    (count / sum with self_intersect=False, min, first, last, min row index)."""
    from oracle_bridge import specs_of
    _, specs, _ = specs_of(case["agg"], BOTH_SRC, {})
    xs = np.stack([BOTH_SRC["x0"], BOTH_SRC["x1"]], axis=1)
    ys = np.stack([BOTH_SRC["y0"], BOTH_SRC["y1"]], axis=1)
    cv = BOTH_CANVAS
    got = oracle.lines({"value": BOTH_SRC["value"]}, 1, xs, ys, cv["plot_width"], cv["plot_height"],
                       cv["x_range"], cv["y_range"], specs, line_width=1)[0]
    assert oracle.aa_flags(specs)[2] == case["two_stage"]
    _check(got, case["expected"], got.dtype.kind == "f")


AA_IMAGE_CASES = refcases.antialias_image_cases()


@pytest.mark.parametrize("case", AA_IMAGE_CASES, ids=[c["id"] for c in AA_IMAGE_CASES])
def test_oracle_antialias_images(case):
    """test_antialias.py::test_antialiasing: every image of the 28, exactly."""
    from oracle import composite
    cv = case["canvas"]
    aggs = [oracle.line_axis0(f, "x", "y", cv["plot_width"], cv["plot_height"], cv["x_range"], cv["y_range"],
                              [oracle.spec("max", "val")], line_width=case["line_width"])[0] for f in case["frames"]]
    img = oracle.shade_eq_hist(refcases.stack_sum(aggs), refcases.binary_cmap50())
    white = np.array([0xFFFFFFFF], dtype=np.uint32)[0]
    got = composite.over(img, white)
    np.testing.assert_array_equal(got, case["expected"])


SUMMARY_SRC, SUMMARY_CANVAS, SUMMARY_CASES = refcases.both_lines_summary_cases()


@pytest.mark.parametrize("case", SUMMARY_CASES, ids=[c["id"] for c in SUMMARY_CASES])
def test_oracle_both_lines_summary_golden(case):
    from oracle_bridge import specs_of
    keys, specs, _ = specs_of(case["agg"], SUMMARY_SRC, {})
    xs = np.stack([SUMMARY_SRC["x0"], SUMMARY_SRC["x1"]], axis=1)
    ys = np.stack([SUMMARY_SRC["y0"], SUMMARY_SRC["y1"]], axis=1)
    cv = SUMMARY_CANVAS
    res = oracle.lines({"value": SUMMARY_SRC["value"]}, 1, xs, ys, cv["plot_width"], cv["plot_height"],
                       cv["x_range"], cv["y_range"], specs, line_width=1)
    for k, r in zip(keys, res):
        np.testing.assert_array_almost_equal(r, case["expected"][k], decimal=5, err_msg=f"{case['id']} {k}")


NAN_CASES = refcases.antialias_nan_multi_cases()


@pytest.mark.parametrize("si", [False, True])
@pytest.mark.parametrize("case", NAN_CASES, ids=[c["id"] for c in NAN_CASES])
def test_oracle_antialias_nan_multi_golden(case, si):
    spec = oracle.spec("count", self_intersect=si)
    cols, kw = case["columns"], case["kwargs"]
    if case["id"] == "ragged":
        got = oracle.lines_ragged({}, cols["x"], cols["y"], 12, 12, (-1, 11), (-1, 11), [spec], line_width=2)[0]
    else:
        layout, xs, ys = refcases.multi_line_arrays(cols, kw)
        got = oracle.lines({}, layout, xs, ys, 12, 12, (-1, 11), (-1, 11), [spec], line_width=2)[0]
    np.testing.assert_array_almost_equal(got, case["expected"], decimal=5)


def test_oracle_ragged_autorange_golden():
    """test_line_autorange_axis1_ragged (test_pandas.py:1935-1966)."""
    x = [[4.0, 0.0], [0.0, -4.0, 0.0, 4.0]]
    y = [[0.0, -4.0], [-4.0, 0.0, 4.0, 0.0]]
    got = oracle.lines_ragged({}, x, y, 9, 9, None, None, [oracle.spec("count")])[0]
    np.testing.assert_array_equal(got, refcases.golden_array(refcases.lines_golden("test_line_autorange_axis1_ragged")[0]))


@pytest.mark.parametrize("si", [False, True])
def test_oracle_antialias_duplicate_points(si):
    """test_line_antialias_duplicate_points (test_pandas.py:3050-3064)."""
    spec = [oracle.spec("count", self_intersect=si)]
    a = oracle.line_axis0({"x": np.array([0.0, 1.0]), "y": np.array([1.0, 2.0])}, "x", "y", 10, 10, (-0.1, 1.1),
                          (0.9, 2.1), spec, line_width=1)[0]
    b = oracle.line_axis0({"x": np.array([0.0, 0.0, 1.0]), "y": np.array([1.0, 1.0, 2.0])}, "x", "y", 10, 10,
                          (-0.1, 1.1), (0.9, 2.1), spec, line_width=1)[0]
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("kind", ["first", "count", "min", "where_last", "mean", "sum"])
def test_oracle_two_stage_ragged_equals_axis1(kind):
    """Property of the two restated loops: ragged rows that all have the same
    length are a LinesAxis1 frame, so their two-stage results agree exactly
    (line.py:1300-1318 against :1616-1693)."""
    rng = np.random.default_rng(5)
    xs = np.linspace(0, 1, 40)[None, :] + rng.normal(0, 0.002, (25, 40))
    ys = np.cumsum(rng.normal(0, 0.05, (25, 40)), axis=1)
    ys[rng.random(ys.shape) < 0.03] = np.nan
    v = rng.uniform(0, 1, 25)
    xr, yr = (0.0, 1.0), (float(np.nanmin(ys)), float(np.nanmax(ys)))
    spec = {"first": oracle.spec("first", "v"), "count": oracle.spec("count", self_intersect=False),
            "min": oracle.spec("min", "v"), "where_last": oracle.spec("where", selector=oracle.spec("last", "v")),
            "mean": oracle.spec("mean", "v"), "sum": oracle.spec("sum", "v", self_intersect=False)}[kind]
    specs = [spec, oracle.spec("first", "v")]                # first makes every plan two-stage
    a = oracle.lines({"v": v}, 2, xs, ys, 50, 40, xr, yr, specs, line_width=1.5)[0]
    b = oracle.lines_ragged({"v": v}, list(xs), list(ys), 50, 40, xr, yr, specs, line_width=1.5)[0]
    np.testing.assert_array_equal(a, b)
