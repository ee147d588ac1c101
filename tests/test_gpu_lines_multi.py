"""Multi-line glyphs on the GPU (LineAxis0Multi, LinesAxis1, LinesAxis1XConstant,
LinesAxis1YConstant): the reference's golden images, then larger random
cases against the oracle.  Integer reductions bit-exact; float64 sums 1e-12
relative; antialiased float32 aggregates 3e-7 relative (the reference
accumulates them in float32)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
import oracle
import refcases
from gpu_helpers import assert_same, to_numpy

pytestmark = pytest.mark.gpu


def _frame(cols, ragged=False):
    if ragged:
        return ds.TensorFrame({k: ds.RaggedColumn(v) for k, v in cols.items()})
    return ds.TensorFrame({k: torch.from_numpy(np.asarray(v, dtype=np.float64)).cuda() for k, v in cols.items()})


def test_manual_range_golden():
    sol = refcases.golden_array(refcases.lines_golden("test_line_manual_range")[0])
    for case in refcases.lines_golden("line_manual_range_params")["cases"]:
        cvs = ds.Canvas(plot_width=7, plot_height=7, x_range=(-3, 3), y_range=(-3, 3))
        agg = cvs.line(_frame(case["columns"], case.get("ragged", False)), agg=ds.count(),
                       **refcases.line_kwargs(case["kwargs"]))
        np.testing.assert_array_equal(to_numpy(agg), sol, err_msg=str(case["kwargs"]))


@pytest.mark.parametrize("line_width", [0, 1])
def test_autorange_golden(line_width):
    sols = refcases.lines_golden("test_line_autorange")
    sol = refcases.golden_array(sols[0] if line_width else sols[1])
    for case in refcases.lines_golden("line_autorange_params")["cases"]:
        cvs = ds.Canvas(plot_width=9, plot_height=9)
        agg = cvs.line(_frame(case["columns"], case.get("ragged", False)), agg=ds.count(), line_width=line_width,
                       **refcases.line_kwargs(case["kwargs"]))
        assert agg.attrs["x_range"] == (-4.0, 4.0) and agg.attrs["y_range"] == (-4.0, 4.0)
        if line_width:
            np.testing.assert_allclose(to_numpy(agg), sol, rtol=1e-6, atol=1e-6, equal_nan=True)
        else:
            np.testing.assert_array_equal(to_numpy(agg), sol)


def test_axis1_x_constant_and_sum_golden():
    sol = refcases.golden_array(refcases.lines_golden("test_line_autorange_axis1_x_constant")[0])
    frame = _frame({"y0": [0.0, 0.0], "y1": [-4.0, 4.0], "y2": [0.0, 0.0]})
    agg = ds.Canvas(plot_width=9, plot_height=9).line(frame, np.array([-4, 0, 4]), ["y0", "y1", "y2"], ds.count(),
                                                      axis=1)
    np.testing.assert_array_equal(to_numpy(agg), sol)
    case = refcases.lines_golden("line_manual_range_params")["cases"][0]
    frame = _frame(dict(case["columns"], v=[7.0, 9.0]))
    agg = ds.Canvas(plot_width=7, plot_height=7, x_range=(-3, 3), y_range=(-3, 3)).line(
        frame, ["x0", "x1", "x2"], ["y0", "y1", "y2"], ds.sum("v"), axis=1)
    sol = refcases.golden_array(refcases.lines_golden("test_line_agg_sum_axis1_none_constant")[0])
    np.testing.assert_array_equal(to_numpy(agg), sol)


def _random_case(kind, nrows, nv, seed):
    rng = np.random.default_rng(seed)
    cols = {}
    if kind == "axis0multi":
        for j in range(nv):
            cols[f"x{j}"] = np.linspace(0, 1, nrows) + 0.01 * j
            cols[f"y{j}"] = np.cumsum(rng.normal(0, 0.05, nrows))
            cols[f"y{j}"][rng.random(nrows) < 0.02] = np.nan
        kw = dict(x=[f"x{j}" for j in range(nv)], y=[f"y{j}" for j in range(nv)], axis=0)
    else:
        ys = np.cumsum(rng.normal(0, 0.05, (nrows, nv)), axis=1)
        ys[rng.random(ys.shape) < 0.02] = np.nan
        for j in range(nv):
            cols[f"y{j}"] = ys[:, j]
        if kind == "xconst":
            kw = dict(x=np.linspace(0, 1, nv), y=[f"y{j}" for j in range(nv)], axis=1)
        else:
            xs = np.linspace(0, 1, nv)[None, :] + rng.normal(0, 0.002, (nrows, nv))
            for j in range(nv):
                cols[f"x{j}"] = xs[:, j]
            kw = dict(x=[f"x{j}" for j in range(nv)], y=[f"y{j}" for j in range(nv)], axis=1)
    cols["v"] = rng.uniform(0, 1, nrows)
    cols["v"][rng.random(nrows) < 0.05] = np.nan
    return cols, kw


REDS = [("count", ds.count(), oracle.spec("count"), 0.0),
        ("sum", ds.sum("v"), oracle.spec("sum", "v"), 1e-12),
        ("max", ds.max("v"), oracle.spec("max", "v"), 0.0),
        ("first", ds.first("v"), oracle.spec("first", "v"), 0.0),
        ("any", ds.any(), oracle.spec("any"), 0.0)]


@pytest.mark.parametrize("kind", ["axis0multi", "xconst", "axis1"])
@pytest.mark.parametrize("line_width", [0, 1.5])
def test_random_multi_lines_vs_oracle(kind, line_width):
    cols, kw = _random_case(kind, 600 if kind == "axis0multi" else 120, 6 if kind == "axis0multi" else 250, 7)
    frame = _frame(cols)
    layout, xs, ys = refcases.multi_line_arrays(cols, kw)
    xr, yr = (0.0, 1.0), (float(np.nanmin(ys)), float(np.nanmax(ys)))
    for name, red, spec, rtol in REDS:
        cvs = ds.Canvas(plot_width=300, plot_height=200, x_range=xr, y_range=yr)
        got = to_numpy(cvs.line(frame, agg=red, line_width=line_width, **kw))
        ref = oracle.lines({"v": cols["v"]}, layout, xs, ys, 300, 200, xr, yr, [spec], line_width=line_width)[0]
        if line_width and name in ("count", "any"):
            assert_same(got, ref, rtol=3e-7, atol=1e-7, what=f"{kind} {name}")
        else:
            assert_same(got, ref, rtol=rtol, what=f"{kind} {name}")


BOTH_SRC, BOTH_CANVAS, BOTH_CASES = refcases.both_lines_cases()


@pytest.mark.parametrize("case", BOTH_CASES, ids=[c["id"] for c in BOTH_CASES])
def test_both_lines_golden(case):
    """TestLineAntialias both_lines (test_pandas.py:2698-2785): two lines of
    line_antialias_df as LineAxis0Multi at line_width 1, the two-stage plans
    (count / sum with self_intersect=False, min, first, last, min row index)
    folded line by line."""
    frame = _frame(BOTH_SRC)
    cvs = ds.Canvas(**BOTH_CANVAS)
    got = to_numpy(cvs.line(frame, x=["x0", "x1"], y=["y0", "y1"], agg=case["agg"], line_width=1))
    exp = case["expected"]
    if got.dtype.kind == "f":
        np.testing.assert_array_almost_equal(got, exp, decimal=5)      # the reference's close=True
    else:
        np.testing.assert_array_equal(got, exp)
    from oracle_bridge import specs_of
    _, specs, _ = specs_of(case["agg"], BOTH_SRC, {})
    xs = np.stack([BOTH_SRC["x0"], BOTH_SRC["x1"]], axis=1)
    ys = np.stack([BOTH_SRC["y0"], BOTH_SRC["y1"]], axis=1)
    ref = oracle.lines({"value": BOTH_SRC["value"]}, 1, xs, ys, 11, 11, BOTH_CANVAS["x_range"],
                       BOTH_CANVAS["y_range"], specs, line_width=1)[0]
    if ref.dtype == np.float32:
        assert_same(got, ref, rtol=3e-7, atol=1e-7)
    else:
        assert_same(got, ref, rtol=1e-12, atol=1e-15)


TWO_STAGE = [("count", ds.count(self_intersect=False), oracle.spec("count", self_intersect=False)),
             ("sum", ds.sum("v", self_intersect=False), oracle.spec("sum", "v", self_intersect=False)),
             ("min", ds.min("v"), oracle.spec("min", "v")),
             ("first", ds.first("v"), oracle.spec("first", "v")),
             ("last", ds.last("v"), oracle.spec("last", "v")),
             ("min_row", ds._min_row_index(), oracle.spec("min_row"))]


@pytest.mark.parametrize("kind", ["axis0multi", "xconst", "axis1"])
@pytest.mark.parametrize("name", [t[0] for t in TWO_STAGE])
def test_two_stage_multi_lines_vs_oracle(kind, name):
    """Two-stage antialiased plans over several lines, each line drawn alone and
    folded in line order (line.py:1203-1226, 1300-1318 and siblings): float32 count
    3e-7 relative, float64 sum in the reference's line order 1e-12, the rest exact."""
    _, red, spec = next(t for t in TWO_STAGE if t[0] == name)
    cols, kw = _random_case(kind, 400 if kind == "axis0multi" else 60, 5 if kind == "axis0multi" else 120, 19)
    frame = _frame(cols)
    layout, xs, ys = refcases.multi_line_arrays(cols, kw)
    xr, yr = (0.0, 1.0), (float(np.nanmin(ys)), float(np.nanmax(ys)))
    got = to_numpy(ds.Canvas(plot_width=160, plot_height=90, x_range=xr, y_range=yr).line(
        frame, agg=red, line_width=1.5, **kw))
    ref = oracle.lines({"v": cols["v"]}, layout, xs, ys, 160, 90, xr, yr, [spec], line_width=1.5)[0]
    if ref.dtype == np.float32:
        assert_same(got, ref, rtol=3e-7, atol=1e-7, what=f"{kind} {name}")
    elif ref.dtype.kind == "f":
        assert_same(got, ref, rtol=1e-12, what=f"{kind} {name}")
    else:
        assert_same(got, ref, what=f"{kind} {name}")


def test_two_stage_summary_and_unserved_plans():
    cols, kw = _random_case("axis0multi", 300, 4, 23)
    frame = _frame(cols)
    layout, xs, ys = refcases.multi_line_arrays(cols, kw)
    xr, yr = (0.0, 1.0), (float(np.nanmin(ys)), float(np.nanmax(ys)))
    cvs = ds.Canvas(plot_width=70, plot_height=50, x_range=xr, y_range=yr)
    agg = ds.summary(c=ds.count(), mn=ds.min("v"), mx=ds.max("v"), f=ds.first("v"), a=ds.any())
    got = cvs.line(frame, agg=agg, line_width=1.5, **kw)
    specs = [oracle.spec("count"), oracle.spec("min", "v"), oracle.spec("max", "v"), oracle.spec("first", "v"),
             oracle.spec("any")]
    ref = oracle.lines({"v": cols["v"]}, layout, xs, ys, 70, 50, xr, yr, specs, line_width=1.5)
    for k, r in zip(("c", "mn", "mx", "f", "a"), ref):
        if r.dtype == np.float32:
            assert_same(to_numpy(got[k]), r, rtol=3e-7, atol=1e-7, what=k)
        else:
            assert_same(to_numpy(got[k]), r, what=k)
    # mean and _count_ignore_antialiasing inside a two-stage plan: additive within and across lines
    agg = ds.summary(m=ds.mean("v"), f=ds.first("v"), k=ds._count_ignore_antialiasing("v"))
    got = cvs.line(frame, agg=agg, line_width=1.5, **kw)
    ref = oracle.lines({"v": cols["v"]}, layout, xs, ys, 70, 50, xr, yr,
                       [oracle.spec("mean", "v"), oracle.spec("first", "v"), oracle.spec("count_ignore_aa", "v")],
                       line_width=1.5)
    assert_same(to_numpy(got["m"]), ref[0], rtol=1e-12, atol=1e-15, what="mean")
    assert_same(to_numpy(got["f"]), ref[1], what="first")
    assert_same(to_numpy(got["k"]), ref[2], what="count_ignore_aa")
    # where(min | first | last) are two-stage; where(max) folds inside a two-stage summary
    w = np.arange(300.0) * 0.5
    frame_w = _frame(dict(cols, w=w))
    for sel, cls in (("min", ds.min), ("first", ds.first), ("last", ds.last), ("max", ds.max)):
        agg = ds.summary(r=ds.where(cls("v")), l=ds.where(cls("v"), "w"), f=ds.first("v"))
        got = cvs.line(frame_w, agg=agg, line_width=1.5, **kw)
        ref = oracle.lines({"v": cols["v"], "w": w}, layout, xs, ys, 70, 50, xr, yr,
                           [oracle.spec("where", selector=oracle.spec(sel, "v")),
                            oracle.spec("where", selector=oracle.spec(sel, "v"), lookup="w"),
                            oracle.spec("first", "v")], line_width=1.5)
        assert_same(to_numpy(got["r"]), ref[0], what=f"where({sel}) row")
        assert_same(to_numpy(got["l"]), ref[1], what=f"where({sel}, w)")


@pytest.mark.parametrize("name", [t[0] for t in TWO_STAGE] + ["where_last", "mean", "si_count_where"])
def test_two_stage_ragged_vs_oracle(name):
    """Two-stage plans over ragged rows (line.py:1616-1693): one row at a time, folded."""
    rng = np.random.default_rng(29)
    lens = rng.integers(0, 40, 30)
    xr_rows = [list(np.sort(rng.uniform(0, 1, k))) for k in lens]
    yr_rows = [list(np.cumsum(rng.normal(0, 0.08, k))) for k in lens]
    for r in yr_rows[::7]:
        if len(r) > 3:
            r[2] = np.nan
    v = rng.uniform(0, 1, 30)
    frame = ds.TensorFrame({"x": ds.RaggedColumn(xr_rows), "y": ds.RaggedColumn(yr_rows),
                            "v": torch.from_numpy(v).cuda()})
    if name == "where_last":
        red, spec = ds.where(ds.last("v")), oracle.spec("where", selector=oracle.spec("last", "v"))
    elif name == "mean":
        red, spec = ds.summary(m=ds.mean("v"), f=ds.first("v")), None
    elif name == "si_count_where":
        # where alone keeps self_intersect: a two-stage plan whose count and sum stay additive
        red, spec = ds.summary(c=ds.count(), s=ds.sum("v"), w=ds.where(ds.first("v"))), None
    else:
        _, red, spec = next(t for t in TWO_STAGE if t[0] == name)
    yall = np.concatenate([np.asarray(r) for r in yr_rows if len(r)])
    xrng, yrng = (0.0, 1.0), (float(np.nanmin(yall)), float(np.nanmax(yall)))
    cvs = ds.Canvas(plot_width=80, plot_height=60, x_range=xrng, y_range=yrng)
    got = cvs.line(frame, x="x", y="y", axis=1, agg=red, line_width=1.5)
    if name == "si_count_where":
        ref = oracle.lines_ragged({"v": v}, xr_rows, yr_rows, 80, 60, xrng, yrng,
                                  [oracle.spec("count"), oracle.spec("sum", "v"),
                                   oracle.spec("where", selector=oracle.spec("first", "v"))], line_width=1.5)
        assert_same(to_numpy(got["c"]), ref[0], rtol=3e-7, atol=1e-7)
        assert_same(to_numpy(got["s"]), ref[1], rtol=1e-12, atol=1e-15)
        assert_same(to_numpy(got["w"]), ref[2])
        return
    if spec is None:
        ref = oracle.lines_ragged({"v": v}, xr_rows, yr_rows, 80, 60, xrng, yrng,
                                  [oracle.spec("mean", "v"), oracle.spec("first", "v")], line_width=1.5)
        assert_same(to_numpy(got["m"]), ref[0], rtol=1e-12, atol=1e-15)
        assert_same(to_numpy(got["f"]), ref[1])
        return
    ref = oracle.lines_ragged({"v": v}, xr_rows, yr_rows, 80, 60, xrng, yrng, [spec], line_width=1.5)[0]
    got = to_numpy(got)
    if ref.dtype == np.float32:
        assert_same(got, ref, rtol=3e-7, atol=1e-7, what=name)
    elif ref.dtype.kind == "f":
        assert_same(got, ref, rtol=1e-12, what=name)
    else:
        assert_same(got, ref, what=name)


@pytest.mark.parametrize("nv", [2, 6])
def test_axis0multi_row_index_reductions_follow_line_order(nv):
    """first / last / where over several axis=0 lines: the reference visits line j
    outer, row i inner (line.py:1190-1194), so on pixels that several lines cross the
    first row of line 0 wins over an earlier row of line 1.  The lines overlap on
    most pixels of a 40 x 30 canvas, so row order and (line, row) order disagree."""
    cols, kw = _random_case("axis0multi", 900, nv, 11)
    rng = np.random.default_rng(12)
    cols["w"] = rng.normal(0, 1, 900)
    frame = _frame(cols)
    layout, xs, ys = refcases.multi_line_arrays(cols, kw)
    xr, yr = (0.0, 1.0), (float(np.nanmin(ys)), float(np.nanmax(ys)))
    cvs = ds.Canvas(plot_width=40, plot_height=30, x_range=xr, y_range=yr)
    agg = ds.summary(f=ds.first("v"), l=ds.last("v"), wr=ds.where(ds.max("v")),
                     wl=ds.where(ds.min("v"), "w"), c=ds.count())
    got = cvs.line(frame, agg=agg, **kw)
    specs = [oracle.spec("first", "v"), oracle.spec("last", "v"),
             oracle.spec("where", selector=oracle.spec("max", "v")),
             oracle.spec("where", selector=oracle.spec("min", "v"), lookup="w"), oracle.spec("count")]
    ref = oracle.lines({"v": cols["v"], "w": cols["w"]}, layout, xs, ys, 40, 30, xr, yr, specs)
    for k, r in zip(("f", "l", "wr", "wl", "c"), ref):
        assert_same(to_numpy(got[k]), r, what=f"nv={nv} {k}")


@pytest.mark.parametrize("lw", [0.0, 1.5])
@pytest.mark.parametrize("red", ["count", "sum", "max", "mean"])
def test_ragged_random_vs_oracle(lw, red):
    """LinesAxis1Ragged on rows of every length (0, 1, 2, many; x and y of
    different lengths, NaN breaks) against the oracle's restatement of
    line.py:1538-1612."""
    rng = np.random.default_rng(31)
    nrows = 400
    xr, yr = [], []
    for i in range(nrows):
        lx = int(rng.integers(0, 40)) if i % 7 else int(rng.integers(0, 3))
        ly = lx if i % 5 else max(0, lx + int(rng.integers(-3, 4)))
        x = np.cumsum(rng.uniform(0.0, 0.05, lx)) + rng.uniform(-1, 1)
        y = np.cumsum(rng.normal(0.0, 0.08, ly)) + rng.uniform(-1, 1)
        if lx > 4 and i % 3 == 0:
            x[lx // 2] = np.nan
        xr.append(x)
        yr.append(y)
    v = rng.uniform(0.5, 2.0, nrows)
    frame = ds.TensorFrame({"x": ds.RaggedColumn(xr), "y": ds.RaggedColumn(yr),
                            "v": torch.from_numpy(v).cuda()})
    agg = {"count": ds.count(), "sum": ds.sum("v"), "max": ds.max("v"), "mean": ds.mean("v")}[red]
    cvs = ds.Canvas(plot_width=200, plot_height=150, x_range=(-1.5, 2.5), y_range=(-2.5, 2.5))
    got = to_numpy(cvs.line(frame, "x", "y", agg=agg, axis=1, line_width=lw))
    spec = oracle.spec(red, None if red == "count" else "v")
    ref = oracle.lines_ragged({"v": v}, xr, yr, 200, 150, (-1.5, 2.5), (-2.5, 2.5), [spec], line_width=lw)[0]
    rtol = 0.0 if red in ("count", "max") and lw == 0 else (3e-7 if ref.dtype == np.float32 else 1e-12)
    assert_same(got, ref, rtol=rtol, what=f"{red} lw={lw}")
    auto = ds.Canvas(plot_width=64, plot_height=48).line(frame, "x", "y", agg=ds.count(), axis=1)
    ref_auto = oracle.lines_ragged({}, xr, yr, 64, 48, None, None, [oracle.spec("count")])[0]
    assert_same(to_numpy(auto), ref_auto)


def test_two_stage_categorical_and_y_constant():
    """Two-stage folds over categorical aggregates (by(cat, ...): the fold runs
    over every category cell) on LineAxis0Multi, and a LinesAxis1YConstant
    frame (one y array shared by every row)."""
    cols, kw = _random_case("axis0multi", 350, 3, 31)
    rng = np.random.default_rng(32)
    cols["cat"] = rng.integers(0, 3, 350).astype(np.float64)
    layout, xs, ys = refcases.multi_line_arrays(cols, kw)
    xr, yr = (0.0, 1.0), (float(np.nanmin(ys)), float(np.nanmax(ys)))
    t = {k: torch.from_numpy(np.asarray(v, dtype=np.float64)).cuda() for k, v in cols.items() if k != "cat"}
    t["cat"] = torch.from_numpy(cols["cat"].astype(np.int8)).cuda()
    frame = ds.TensorFrame(t, categories={"cat": [0, 1, 2]})
    cvs = ds.Canvas(plot_width=60, plot_height=40, x_range=xr, y_range=yr)
    for red, spec in ((ds.by("cat", ds.count(self_intersect=False)), oracle.spec("count", cat="cat", ncat=3,
                                                                                  self_intersect=False)),
                      (ds.by("cat", ds.first("v")), oracle.spec("first", "v", cat="cat", ncat=3))):
        got = to_numpy(cvs.line(frame, agg=red, line_width=1.5, **kw))
        ref = oracle.lines({"v": cols["v"], "cat": cols["cat"]}, layout, xs, ys, 60, 40, xr, yr, [spec],
                           line_width=1.5)[0]
        if ref.dtype == np.float32:
            assert_same(got, ref, rtol=3e-7, atol=1e-7)
        else:
            assert_same(got, ref)
    # LinesAxis1YConstant: x per row, one shared y
    rng = np.random.default_rng(33)
    nv = 50
    xcols = {f"x{j}": np.linspace(0, 1, 40) * 0.02 + j / nv + rng.normal(0, 0.003, 40) for j in range(nv)}
    xcols["v"] = rng.uniform(0, 1, 40)
    yconst = np.sin(np.linspace(0, 3, nv))
    kw = dict(x=[f"x{j}" for j in range(nv)], y=yconst, axis=1)
    frame = _frame(xcols)
    xs = np.stack([xcols[f"x{j}"] for j in range(nv)], axis=1)
    yr = (float(yconst.min()), float(yconst.max()))
    cvs = ds.Canvas(plot_width=70, plot_height=30, x_range=(0.0, 1.05), y_range=yr)
    for red, spec in ((ds.min("v"), oracle.spec("min", "v")), (ds.last("v"), oracle.spec("last", "v"))):
        got = to_numpy(cvs.line(frame, agg=red, line_width=1.5, **kw))
        ref = oracle.lines({"v": xcols["v"]}, 2, xs, yconst, 70, 30, (0.0, 1.05), yr, [spec], line_width=1.5)[0]
        assert_same(got, ref)


SUMMARY_SRC, SUMMARY_CANVAS, SUMMARY_CASES = refcases.both_lines_summary_cases()


@pytest.mark.parametrize("case", SUMMARY_CASES, ids=[c["id"] for c in SUMMARY_CASES])
def test_both_lines_summary_golden(case):
    """TestLineAntialiasSummary (test_pandas.py:2802-2890) through the GPU path."""
    got = ds.Canvas(**SUMMARY_CANVAS).line(_frame(SUMMARY_SRC), x=["x0", "x1"], y=["y0", "y1"], agg=case["agg"],
                                           line_width=1)
    for k, exp in case["expected"].items():
        np.testing.assert_array_almost_equal(to_numpy(got[k]), exp, decimal=5, err_msg=f"{case['id']} {k}")


NAN_CASES = refcases.antialias_nan_multi_cases()


@pytest.mark.parametrize("si", [False, True])
@pytest.mark.parametrize("case", NAN_CASES, ids=[c["id"] for c in NAN_CASES])
def test_antialias_nan_multi_golden(case, si):
    """test_line_antialias_nan's multi-line entries (test_pandas.py:2931-3024):
    end caps at NaN vertices; self_intersect=False is a two-stage plan."""
    cols = case["columns"]
    if case["id"] == "ragged":
        frame = ds.TensorFrame({k: ds.RaggedColumn(v) for k, v in cols.items()})
    else:
        frame = ds.TensorFrame({k: torch.from_numpy(v).cuda() for k, v in cols.items()})
    cvs = ds.Canvas(plot_width=12, plot_height=12, x_range=(-1, 11), y_range=(-1, 11))
    got = to_numpy(cvs.line(frame, line_width=2, agg=ds.count(self_intersect=si), **case["kwargs"]))
    np.testing.assert_array_almost_equal(got, case["expected"], decimal=5)


def _ragged_autorange_frame():
    """test_line_autorange_axis1_ragged (test_pandas.py:1935-1966): two float32 ragged rows."""
    x = [[4.0, 0.0], [0.0, -4.0, 0.0, 4.0]]
    y = [[0.0, -4.0], [-4.0, 0.0, 4.0, 0.0]]
    return x, y


def test_ragged_autorange_golden():
    x, y = _ragged_autorange_frame()
    frame = ds.TensorFrame({"x": ds.RaggedColumn(x), "y": ds.RaggedColumn(y)})
    agg = ds.Canvas(plot_width=9, plot_height=9).line(frame, "x", "y", ds.count(), axis=1)
    sol = refcases.golden_array(refcases.lines_golden("test_line_autorange_axis1_ragged")[0])
    np.testing.assert_array_equal(to_numpy(agg), sol)
    assert agg.x_range == (-4.0, 4.0) and agg.y_range == (-4.0, 4.0)


@pytest.mark.parametrize("si", [False, True])
def test_antialias_duplicate_points(si):
    """test_line_antialias_duplicate_points (test_pandas.py:3050-3064): a repeated
    vertex draws the same image as the line without it (no division by zero)."""
    cvs = ds.Canvas(plot_width=10, plot_height=10, x_range=(-0.1, 1.1), y_range=(0.9, 2.1))
    a = cvs.line(_frame({"x": [0.0, 1.0], "y": [1.0, 2.0]}), "x", "y", line_width=1, agg=ds.count(self_intersect=si))
    b = cvs.line(_frame({"x": [0.0, 0.0, 1.0], "y": [1.0, 1.0, 2.0]}), "x", "y", line_width=1,
                 agg=ds.count(self_intersect=si))
    np.testing.assert_array_equal(to_numpy(a), to_numpy(b))


def test_line_coordinate_lengths():
    """test_line_coordinate_lengths (test_pandas.py:3310-3334): mismatched x / y
    lists or constant arrays raise ValueError('x and y coordinate lengths do not match')."""
    cvs = ds.Canvas(plot_width=10, plot_height=6)
    msg = r"^x and y coordinate lengths do not match"
    df = _frame(dict(x0=[0, 0.2, 1], y0=[0, 0.4, 1], x1=[0, 0.6, 1], y1=[1, 0.8, 1]))
    for axis in (0, 1):
        with pytest.raises(ValueError, match=msg):
            cvs.line(source=df, x=["x0"], y=["y0", "y1"], axis=axis)
        with pytest.raises(ValueError, match=msg):
            cvs.line(source=df, x=["x0", "x1"], y=["y0"], axis=axis)
    df = _frame(dict(y0=[0, 1, 0, 1], y1=[0, 1, 1, 0]))
    for nx in (1, 3):
        with pytest.raises(ValueError, match=msg):
            cvs.line(source=df, x=np.arange(nx), y=["y0", "y1"], axis=1)
    df = _frame(dict(x0=[0, 1, 0, 1], x1=[0, 1, 1, 0]))
    for ny in (1, 3):
        with pytest.raises(ValueError, match=msg):
            cvs.line(source=df, x=["x0", "x1"], y=np.arange(ny), axis=1)
