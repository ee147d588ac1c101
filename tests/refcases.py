"""Golden cases of the reference's own test-suite, restated as data.

Each case cites the test in datashader/tests/test_pandas.py whose inputs and
expected outputs it restates.  Small inputs are rebuilt here from the same
definitions; the larger solution arrays come from tests/golden/*.json
(extracted by tests/golden/make_golden.py).  The same cases drive the CPU
oracle tests (test_oracle_golden.py) and the GPU parity tests
(test_gpu_golden.py).
"""
from __future__ import annotations

import json
import os

import numpy as np

import datashader_gb300 as ds

HERE = os.path.dirname(os.path.abspath(__file__))
nan = np.nan


def load_golden(fname, key=None):
    with open(os.path.join(HERE, "golden", fname)) as f:
        g = json.load(f)
    return g if key is None else g[key]


def golden_array(entry):
    data = [np.nan if v is None else v for v in entry["data"]]
    return np.array(data, dtype=entry["dtype"]).reshape(entry["shape"])


def pandas_frame():
    """test_pandas.py:27-57 (_pandas): 20 rows on a 2x2 canvas.

    Returns (columns, categories); categorical columns hold int8 codes."""
    cols = {
        "x": np.array([0.] * 10 + [1] * 10),
        "y": np.array([0.] * 5 + [1] * 5 + [0] * 5 + [1] * 5),
        "log_x": np.array([1.] * 10 + [10] * 10),
        "log_y": np.array([1.] * 5 + [10] * 5 + [1] * 5 + [10] * 5),
        "i32": np.arange(20, dtype="i4"),
        "i64": np.arange(20, dtype="i8"),
        "f32": np.arange(20, dtype="f4"),
        "f64": np.arange(20, dtype="f8"),
        "reverse": np.arange(20, 0, -1).astype("f8"),
        "plusminus": np.arange(20, dtype="f8") * ([1, -1] * 10),
        "empty_bin": np.array([0.] * 15 + [np.nan] * 5),
        "cat": np.repeat(np.arange(4, dtype="i1"), 5),
        "cat2": np.tile(np.arange(4, dtype="i1"), 5),
        "onecat": np.zeros(20, dtype="i1"),
        "cat_int": np.array([10] * 5 + [11] * 5 + [12] * 5 + [13] * 5, dtype="i8"),
    }
    cols["f32"][2] = np.nan
    cols["f64"][2] = np.nan
    cols["reverse"][6] = np.nan
    cols["plusminus"][2] = np.nan
    cats = {"cat": ["a", "b", "c", "d"], "cat2": ["a", "b", "c", "d"], "onecat": ["one"]}
    return cols, cats


C2 = dict(plot_width=2, plot_height=2, x_range=(0, 1), y_range=(0, 1))


def _pf():
    return pandas_frame()[0]


def _r(a):
    return a.reshape((2, 2, 5))


def point_cases():
    """(id, agg, canvas kwargs, expected, x, y, frame builder) for Canvas.points."""
    df = _pf()
    cases = []

    def add(cid, agg, expected, canvas=C2, x="x", y="y", frame=None, close=False):
        cases.append(dict(id=cid, agg=agg, canvas=canvas, expected=expected, x=x, y=y,
                          frame=frame, close=close))

    # test_count (:194-203)
    for c in ("i32", "i64", None):
        add(f"count_{c}", ds.count(c) if c else ds.count(), np.array([[5, 5], [5, 5]]))
    for c in ("f32", "f64"):
        add(f"count_{c}", ds.count(c), np.array([[4, 5], [5, 5]]))
    # test_any (:206-214)
    for c in ("i64", "f64", None):
        add(f"any_{c}", ds.any(c) if c else ds.any(), np.array([[True, True], [True, True]]))
    add("any_empty_bin", ds.any("empty_bin"), np.array([[True, True], [True, False]]))
    # test_sum (:217-225)
    for c in ("i32", "i64"):
        add(f"sum_{c}", ds.sum(c), _r(df["i32"]).sum(axis=2, dtype="f8").T)
    for c in ("f32", "f64"):
        add(f"sum_{c}", ds.sum(c), np.nansum(_r(df["f64"]), axis=2).T)
    # test_min / test_max (:228-243)
    for c in ("i32", "i64", "f32", "f64"):
        add(f"min_{c}", ds.min(c), _r(df["i64"]).min(axis=2).astype("f8").T)
        add(f"max_{c}", ds.max(c), _r(df["i64"]).max(axis=2).astype("f8").T)
    # test_mean (:698-705)
    for c in ("i32", "i64"):
        add(f"mean_{c}", ds.mean(c), _r(df["i32"]).mean(axis=2, dtype="f8").T)
    for c in ("f32", "f64"):
        add(f"mean_{c}", ds.mean(c), np.nanmean(_r(df["f64"]), axis=2).T)
    # test_first / test_last (:991-1005)
    for c in ("i32", "i64", "f32", "f64"):
        add(f"first_{c}", ds.first(c), np.array([[0, 10], [5, 15]], "f8"))
        add(f"last_{c}", ds.last(c), np.array([[4, 14], [9, 19]], "f8"))
    # test_where_min_row_index / max_row_index (:421-428)
    add("where_min_row_index", ds.where(ds._min_row_index(), "plusminus"), np.array([[0, 10], [-5, -15]], "f8"))
    add("where_max_row_index", ds.where(ds._max_row_index(), "plusminus"), np.array([[4, 14], [-9, -19]], "f8"))
    # test_where_first / last / max / min (:448-510)
    for c in ("i32", "i64", "f32", "f64"):
        add(f"where_first_{c}", ds.where(ds.first(c), "reverse"), np.array([[20, 10], [15, 5]], "f8"))
        add(f"where_first_row_{c}", ds.where(ds.first(c)), np.array([[0, 10], [5, 15]]))
        add(f"where_last_{c}", ds.where(ds.last(c), "reverse"), np.array([[16, 6], [11, 1]], "f8"))
        add(f"where_last_row_{c}", ds.where(ds.last(c)), np.array([[4, 14], [9, 19]]))
        add(f"where_max_{c}", ds.where(ds.max(c), "reverse"), np.array([[16, 6], [11, 1]], "f8"))
        add(f"where_max_row_{c}", ds.where(ds.max(c)), np.array([[4, 14], [9, 19]]))
        add(f"where_min_{c}", ds.where(ds.min(c), "reverse"), np.array([[20, 10], [15, 5]], "f8"))
        add(f"where_min_row_{c}", ds.where(ds.min(c)), np.array([[0, 10], [5, 15]]))
    # test_count_cat / test_categorical_count (:731-760)
    sol = np.array([[[5, 0, 0, 0], [0, 0, 5, 0]], [[0, 5, 0, 0], [0, 0, 0, 5]]])
    add("count_cat", ds.count_cat("cat"), sol)
    add("by_cat_count_i32", ds.by("cat", ds.count("i32")), sol)
    add("by_modulo_count", ds.by(ds.category_modulo("cat_int", modulo=4, offset=10), ds.count()), sol)
    # test_one_category (:763-775)
    add("by_onecat", ds.by("onecat", ds.count("i32")), np.array([[[5], [5]], [[5], [5]]]))
    # test_categorical_min / max (:268-287)
    sol_int = np.array([[[0, 1, 2, 3], [12, 13, 10, 11]], [[8, 5, 6, 7], [16, 17, 18, 15]]], "f8")
    sol_float = np.array([[[0, 1, nan, 3], [12, 13, 10, 11]], [[8, 5, 6, 7], [16, 17, 18, 15]]])
    for c in ("i32", "i64"):
        add(f"by_cat2_min_{c}", ds.by("cat2", ds.min(c)), sol_int)
    for c in ("f32", "f64"):
        add(f"by_cat2_min_{c}", ds.by("cat2", ds.min(c)), sol_float)
    sol_int = np.array([[[4, 1, 2, 3], [12, 13, 14, 11]], [[8, 9, 6, 7], [16, 17, 18, 19]]], "f8")
    sol_float = np.array([[[4, 1, nan, 3], [12, 13, 14, 11]], [[8, 9, 6, 7], [16, 17, 18, 19]]])
    for c in ("i32", "i64"):
        add(f"by_cat2_max_{c}", ds.by("cat2", ds.max(c)), sol_int)
    for c in ("f32", "f64"):
        add(f"by_cat2_max_{c}", ds.by("cat2", ds.max(c)), sol_float)
    # test_categorical_min_row_index / max_row_index (:318-327)
    add("by_cat2_min_row", ds.by("cat2", ds._min_row_index()),
        np.array([[[0, 1, 2, 3], [12, 13, 10, 11]], [[8, 5, 6, 7], [16, 17, 18, 15]]]))
    add("by_cat2_max_row", ds.by("cat2", ds._max_row_index()),
        np.array([[[4, 1, 2, 3], [12, 13, 14, 11]], [[8, 9, 6, 7], [16, 17, 18, 19]]]))
    # test_categorical_first / last (:360-379)
    add("by_cat2_first", ds.by("cat2", ds.first("plusminus")),
        np.array([[[0, -1, nan, -3], [12, -13, 10, -11]], [[8, -5, 6, -7], [16, -17, 18, -15]]]))
    add("by_cat2_last", ds.by("cat2", ds.last("plusminus")),
        np.array([[[4, -1, nan, -3], [12, -13, 14, -11]], [[8, -9, 6, -7], [16, -17, 18, -19]]]))
    # test_multiple_aggregates (:1067-1077)
    add("summary", ds.summary(f64_mean=ds.mean("f64"), i32_sum=ds.sum("i32"), i32_count=ds.count("i32")),
        {"f64_mean": np.nanmean(_r(df["f64"]), axis=2).T,
         "i32_sum": _r(df["i32"]).sum(axis=2, dtype="f8").T,
         "i32_count": np.array([[5, 5], [5, 5]])})
    # test_log_axis_points (:1171-1188)
    for xa, ya, xr, yr, cx, cy in (("log", "linear", (1, 10), (0, 1), "log_x", "y"),
                                   ("linear", "log", (0, 1), (1, 10), "x", "log_y"),
                                   ("log", "log", (1, 10), (1, 10), "log_x", "log_y")):
        add(f"log_axis_{cx}_{cy}", ds.count("i32"), np.array([[5, 5], [5, 5]]),
            canvas=dict(plot_width=2, plot_height=2, x_range=xr, y_range=yr,
                        x_axis_type=xa, y_axis_type=ya), x=cx, y=cy)
    # test_points_on_edge (:1279-1296)
    edge = {"x": np.array([0, 0.5, 1.1, 1.5, 2.2, 3, 3, 0]), "y": np.array([0, 0, 0, 0, 0, 0, 3, 3.])}
    add("points_on_edge", ds.count(), np.array([[2, 2, 2], [0, 0, 0], [1, 0, 1]]),
        canvas=dict(plot_width=3, plot_height=3, x_range=(0, 3), y_range=(0, 3)), frame=edge)
    # test_uniform_points (:1132-1144)
    n = 101
    uni = {"time": np.ones(2 * n, dtype="i4"),
           "x": np.concatenate((np.arange(n, dtype="f8"), np.arange(n, dtype="f8"))),
           "y": np.concatenate(([0.] * n, [1.] * n))}
    add("uniform_points", ds.count("time"), np.array([[10] * 9 + [11], [10] * 9 + [11]]),
        canvas=dict(plot_width=10, plot_height=2, y_range=(0, 1)), frame=uni)
    # test_auto_range_points (:1080-1129)
    for nn, w, sol_fn in ((10, 10, "diag"), (10, 11, "diag11"), (4, 8, "d8"), (4, 9, "d9")):
        data = np.arange(nn, dtype="i4")
        fr = {"time": np.arange(nn), "x": data, "y": data}
        sol = np.zeros((w, w), int)
        if sol_fn == "diag":
            np.fill_diagonal(sol, 1)
        elif sol_fn == "diag11":
            np.fill_diagonal(sol, 1)
            sol[5, 5] = 0
        elif sol_fn == "d8":
            np.fill_diagonal(sol, 1)
            sol[np.array([tuple(range(1, 4, 2))])] = 0
            sol[np.array([tuple(range(4, 8, 2))])] = 0
        else:
            for k in (0, 3, 6, 8):
                sol[k, k] = 1
        add(f"auto_range_{nn}_{w}", ds.count("time"), sol,
            canvas=dict(plot_width=w, plot_height=w), frame=fr)
    # test_uniform_diagonal_points (:1147-1168): checked by property in the tests
    return cases


def line_cases():
    """Canvas.line cases (LineAxis0)."""
    cases = []
    # test_line (:1256-1276)
    df = {"x": np.array([4, 0, -4, -3, -2, -1.9, 0, 10, 10, 0, 4.]),
          "y": np.array([0, -4, 0, 1, 2, 2.1, 4, 20, 30, 4, 0.])}
    sol = np.array([[0, 0, 1, 0, 1, 0, 0], [0, 1, 0, 0, 0, 1, 0], [1, 0, 0, 0, 0, 0, 1],
                    [0, 0, 0, 0, 0, 0, 0], [1, 0, 0, 0, 0, 0, 1], [0, 2, 0, 0, 0, 1, 0],
                    [0, 0, 1, 0, 1, 0, 0]])
    cases.append(dict(id="line_bresenham", frame=df, agg=ds.count(), expected=sol, line_width=0,
                      canvas=dict(plot_width=7, plot_height=7, x_range=(-3, 3), y_range=(-3, 3)),
                      close=False))
    # test_lines_on_edge (:1299-1316)
    df = {"x": np.array([0, 3, 3, 0.]), "y": np.array([0, 0, 3, 3.])}
    cases.append(dict(id="lines_on_edge", frame=df, agg=ds.count(),
                      expected=np.array([[1, 1, 1], [0, 0, 1], [1, 1, 1]]), line_width=0,
                      canvas=dict(plot_width=3, plot_height=3, x_range=(0, 3), y_range=(0, 3)),
                      close=False))
    # TestLineAntialias (:2460-2800): first (self-intersecting) and second line
    g = load_golden("line_antialias.json")
    src = {k: golden_array(v) for k, v in g["line_antialias_df"]["columns"].items()}
    A = {k: golden_array(v) for k, v in g.items() if k.startswith("line_antialias_sol")}
    cv = dict(plot_width=11, plot_height=11, x_range=(-0.1875, 1.1875), y_range=(-0.1875, 1.1875))
    for which, x, y in (("0", "x0", "y0"), ("1", "x1", "y1")):
        s = A[f"line_antialias_sol_{which}"]
        s_int = A.get(f"line_antialias_sol_{which}_intersect", s)
        cnt = A[f"line_antialias_sol_count_ignore_aa_{which}"]
        for cid, agg, exp, close in (
                ("any", ds.any(), s, True),
                ("count_no_intersect", ds.count(self_intersect=False), s, True),
                ("count_intersect", ds.count(self_intersect=True), s_int, True),
                ("sum_no_intersect", ds.sum("value", self_intersect=False), 3 * s, True),
                ("sum_intersect", ds.sum("value", self_intersect=True), 3 * s_int, True),
                ("max", ds.max("value"), 3 * s, True),
                ("min", ds.min("value"), 3 * s, True),
                ("first", ds.first("value"), 3 * s, True),
                ("last", ds.last("value"), 3 * s, True),
                ("count_ignore_aa", ds._count_ignore_antialiasing("value"), cnt, True),
                ("mean", ds.mean("value"), 3 * s_int / cnt, True),
                ("min_row_index", ds._min_row_index(), A[f"line_antialias_sol_min_index_{which}"], False),
                ("max_row_index", ds._max_row_index(), A[f"line_antialias_sol_max_index_{which}"], False)):
            with np.errstate(divide="ignore", invalid="ignore"):
                exp = np.array(exp)
            cases.append(dict(id=f"aa_line{which}_{cid}", frame={"x": src[x], "y": src[y], "value": src["value"]},
                              agg=agg, expected=exp, line_width=1, canvas=cv, close=close))
    # test_line_antialias_nan (:2901-3024), LineAxis0 entry
    e = g["line_antialias_nan_axis0"]
    fr = {k: golden_array(v) for k, v in e["columns"].items()}
    for si, key in ((False, "sol_self_intersect_false"), (True, "sol_self_intersect_true")):
        cases.append(dict(id=f"aa_nan_si{int(si)}", frame=fr, agg=ds.count(self_intersect=si),
                          expected=golden_array(e[key]), line_width=2,
                          canvas=dict(plot_width=12, plot_height=12, x_range=(-1, 11), y_range=(-1, 11)),
                          close=True))
    # test_line_antialias_categorical (:3027-3046)
    fr = {"x": np.asarray([0, 1, 1, 0, np.nan, 0, 1 / 3.0, 2 / 3.0, 1]),
          "y": np.asarray([0, 1, 0, 1, np.nan, 0.125, 0.15, 0.175, 0.2]),
          "cat": np.array([0, 0, 0, 0, 0, 1, 1, 1, 1], dtype="i1")}
    for si, s0 in ((False, A["line_antialias_sol_0"]), (True, A["line_antialias_sol_0_intersect"])):
        exp = np.stack([s0, A["line_antialias_sol_1"]], axis=-1)
        cases.append(dict(id=f"aa_categorical_si{int(si)}", frame=fr, categories={"cat": [1, 2]},
                          agg=ds.by("cat", ds.count(self_intersect=si)), expected=exp, line_width=1,
                          canvas=cv, close=True))
    return cases


def both_lines_cases():
    """TestLineAntialias both_lines (test_pandas.py:2698-2785): the two lines of
    line_antialias_df drawn together as LineAxis0Multi (x=["x0", "x1"],
    y=["y0", "y1"], line_width=1), each expected image built from the single-line
    solutions as the reference test builds it (nansum / nanmax / nanmin / rowmin /
    rowmax, :2304-2331).  Returns (columns, canvas, cases); `two_stage` marks the
    plans the reference runs line by line with a stage-2 fold."""
    g = load_golden("line_antialias.json")
    src = {k: golden_array(v) for k, v in g["line_antialias_df"]["columns"].items()}
    A = {k: golden_array(v) for k, v in g.items() if k.startswith("line_antialias_sol")}
    s0, s1, s0i = A["line_antialias_sol_0"], A["line_antialias_sol_1"], A["line_antialias_sol_0_intersect"]
    c0, c1 = A["line_antialias_sol_count_ignore_aa_0"], A["line_antialias_sol_count_ignore_aa_1"]

    def both_nan(a, b):
        return np.isnan(a) & np.isnan(b)

    def nansum(a, b):
        r = np.nan_to_num(a) + np.nan_to_num(b)
        r[both_nan(a, b)] = np.nan
        return r

    def nanmax(a, b):
        r = np.maximum(np.nan_to_num(a), np.nan_to_num(b))
        r[both_nan(a, b)] = np.nan
        return r

    def nanmin(a, b):
        r = np.minimum(np.nan_to_num(a, nan=1e10), np.nan_to_num(b, nan=1e10))
        r[both_nan(a, b)] = np.nan
        return r

    def rowmin(a, b):
        big = max(a.max(), b.max()) + 1
        r = np.minimum(np.where(a < 0, big, a), np.where(b < 0, big, b))
        return np.where(r == big, -1, r)

    with np.errstate(divide="ignore", invalid="ignore"):
        mean = 3 * (np.nan_to_num(s0i) + np.nan_to_num(s1)) / (np.nan_to_num(c0) + np.nan_to_num(c1))
    cases = [
        ("any", ds.any(), nanmax(s0, s1), False),
        ("count_no_intersect", ds.count(self_intersect=False), nansum(s0, s1), True),
        ("count_intersect", ds.count(self_intersect=True), nansum(s0i, s1), False),
        ("sum_no_intersect", ds.sum("value", self_intersect=False), 3 * nansum(s0, s1), True),
        ("sum_intersect", ds.sum("value", self_intersect=True), 3 * nansum(s0i, s1), False),
        ("max", ds.max("value"), 3 * nanmax(s0, s1), False),
        ("min", ds.min("value"), 3 * nanmin(s0, s1), True),
        ("first", ds.first("value"), 3 * np.where(np.isnan(s0), s1, s0), True),
        ("last", ds.last("value"), 3 * np.where(np.isnan(s1), s0, s1), True),
        ("count_ignore_aa", ds._count_ignore_antialiasing("value"), c0 + c1, False),
        ("mean", ds.mean("value"), mean, False),
        ("min_row_index", ds._min_row_index(),
         rowmin(A["line_antialias_sol_min_index_0"], A["line_antialias_sol_min_index_1"]), True),
        ("max_row_index", ds._max_row_index(),
         np.maximum(A["line_antialias_sol_max_index_0"], A["line_antialias_sol_max_index_1"]), False),
    ]
    canvas = dict(plot_width=11, plot_height=11, x_range=(-0.1875, 1.1875), y_range=(-0.1875, 1.1875))
    out = [dict(id=f"both_lines_{cid}", agg=agg, expected=exp, two_stage=two) for cid, agg, exp, two in cases]
    return src, canvas, out


def both_lines_summary_cases():
    """TestLineAntialiasSummary (test_pandas.py:2802-2890): summaries over the
    same two lines, mixing self_intersect settings (a plan turns two-stage, and
    every count / sum in it non-self-intersecting, as soon as one reduction asks
    for it).  Returns (columns, canvas, cases) with a dict of expected arrays."""
    src, canvas, _ = both_lines_cases()
    g = load_golden("line_antialias.json")
    A = {k: golden_array(v) for k, v in g.items() if k.startswith("line_antialias_sol")}
    s0, s1, s0i = A["line_antialias_sol_0"], A["line_antialias_sol_1"], A["line_antialias_sol_0_intersect"]

    def nansum(a, b):
        r = np.nan_to_num(a) + np.nan_to_num(b)
        r[np.isnan(a) & np.isnan(b)] = np.nan
        return r

    def nanmin(a, b):
        r = np.minimum(np.nan_to_num(a, nan=1e10), np.nan_to_num(b, nan=1e10))
        r[np.isnan(a) & np.isnan(b)] = np.nan
        return r

    cnt, cnt_i = nansum(s0, s1), nansum(s0i, s1)
    first = 3 * np.where(np.isnan(s0), s1, s0)
    last = 3 * np.where(np.isnan(s1), s0, s1)
    cases = [
        ("count_sum_intersect_true", ds.summary(count=ds.count("value", self_intersect=True),
                                                sum=ds.sum("value", self_intersect=True)),
         {"count": cnt_i, "sum": 3 * cnt_i}),
        ("count_sum_intersect_false", ds.summary(count=ds.count("value", self_intersect=False),
                                                 sum=ds.sum("value", self_intersect=False)),
         {"count": cnt, "sum": 3 * cnt}),
        ("count_sum_intersect_mixed", ds.summary(count=ds.count("value", self_intersect=True),
                                                 sum=ds.sum("value", self_intersect=False)),
         {"count": cnt, "sum": 3 * cnt}),
        ("count_min", ds.summary(count=ds.count("value", self_intersect=True), min=ds.min("value")),
         {"count": cnt, "min": 3 * nanmin(s0, s1)}),
        ("count_first", ds.summary(count=ds.count("value", self_intersect=True), first=ds.first("value")),
         {"count": cnt, "first": first}),
        ("count_last", ds.summary(count=ds.count("value", self_intersect=True), last=ds.last("value")),
         {"count": cnt, "last": last}),
    ]
    return src, canvas, [dict(id=f"both_lines_summary_{c}", agg=a, expected=e) for c, a, e in cases]


def antialias_nan_multi_cases():
    """test_line_antialias_nan (test_pandas.py:2931-3024), the multi-line entries:
    two lines with a NaN vertex each, float32 columns, on a 12 x 12 canvas over
    [-1, 11]^2, line_width 2, count(self_intersect=False | True); every layout
    expects line_antialias_nan_sol_intersect (transposed for YConstant, whose
    lines run along y).  Each case: (id, kind, columns, kwargs, expected)."""
    g = load_golden("line_antialias.json")
    sol = golden_array(g["line_antialias_nan_sol_intersect"])
    f32 = lambda v: np.asarray(v, dtype=np.float32)    # noqa: E731
    nan = np.nan
    a, b = [0.5, 1.5, nan, 4.5, 9.5], [9.5, 8.5, nan, 5.5, 0.5]
    cases = [
        ("multi_axis0", dict(x0=f32(a), x1=f32(a), y0=f32(a), y1=f32(b)),
         dict(x=["x0", "x1"], y=["y0", "y1"], axis=0), sol),
        ("lines_axis1", {**{f"x{j}": f32([a[j], a[j]]) for j in range(5)},
                         **{f"y{j}": f32([a[j], b[j]]) for j in range(5)}},
         dict(x=[f"x{j}" for j in range(5)], y=[f"y{j}" for j in range(5)], axis=1), sol),
        ("x_constant", {f"y{j}": f32([a[j], b[j]]) for j in range(5)},
         dict(x=np.array(a), y=[f"y{j}" for j in range(5)], axis=1), sol),
        ("y_constant", {f"x{j}": f32([a[j], b[j]]) for j in range(5)},
         dict(y=np.array(a), x=[f"x{j}" for j in range(5)], axis=1), sol.T),
        ("ragged", dict(x=[list(map(float, f32(a))), list(map(float, f32(a)))],
                        y=[list(map(float, f32(a))), list(map(float, f32(b)))]),
         dict(x="x", y="y", axis=1), sol),
    ]
    return [dict(id=c, columns=cols, kwargs=kw, expected=e) for c, cols, kw, e in cases]


def binary_cmap50():
    """test_antialias.py:40-42 ``cmap01``: matplotlib's ``cm.binary`` sampled at
    np.linspace(0, 1) (50 points), each channel times 255.  matplotlib is not a
    dependency here, so its published colormap steps are restated: the 'binary'
    segment data ((0, 1, 1), (1, 0, 0)) per channel expanded into a 256-entry
    lookup table as LinearSegmentedColormap builds it (x scaled by N - 1, the
    sample points (N - 1) * linspace(0, 1, N), linear pieces between the
    anchors, clipped to [0, 1]), then Colormap.__call__'s float lookup (x * N
    truncated, x == 1 taking the last entry)."""
    n = 256
    x = np.array([0.0, 1.0]) * (n - 1)
    y0 = np.array([1.0, 0.0])
    y1 = np.array([1.0, 0.0])
    xind = (n - 1) * np.linspace(0, 1, n) ** 1.0
    ind = np.searchsorted(x, xind)[1:-1]
    distance = (xind[1:-1] - x[ind - 1]) / (x[ind] - x[ind - 1])
    lut = np.clip(np.concatenate([[y1[0]], distance * (y0[ind] - y1[ind - 1]) + y1[ind - 1], [y0[-1]]]), 0.0, 1.0)
    xa = np.linspace(0, 1) * n
    xa[xa == n] = n - 1
    return [tuple(float(lut[i]) * 255. for _ in range(3)) for i in xa.astype(int)]


def antialias_image_cases():
    """test_antialias.py:141-408: the 7 line sets x {antialiased, not} x {the
    50 x 50 canvas over [0, 49]^2, the clipped 20 x 20 canvas over [14, 34]^2}.
    Sets 001-005 and 007 are separate two-vertex lines, each its own
    Canvas.line(max('val')) aggregate, summed as xr.concat(...).sum('stack')
    sums them (NaN counts as 0, so an empty pixel is 0); set 006 is one line
    through its vertices.  The image is tf.shade(agg, cmap=cmap01) (eq_hist)
    over a white background.  Expected: the PNG the module wrote, decoded
    (tests/golden/antialias_images.json)."""
    g = load_golden("antialias_images.json")
    sets = {
        "test_001": [((1, 1), (49, a)) for a in range(1, 55, 6)],
        "test_002": [((1, 1), (a, 49)) for a in range(1, 55, 6)],
        "test_003": [((49, 49), (1, a)) for a in range(1, 55, 6)],
        "test_004": [((49, 49), (a, 1)) for a in range(1, 55, 6)],
        "test_005": [((1, 1), (1, 49)), ((1, 49), (2, 1)), ((2, 1), (2, 49)), ((2, 49), (4, 1)),
                     ((4, 1), (4, 49)), ((4, 49), (8, 1)), ((8, 1), (8, 49)), ((8, 49), (16, 1)),
                     ((16, 1), (16, 49)), ((16, 49), (32, 1)), ((32, 1), (32, 49)), ((32, 49), (49, 1)),
                     ((49, 1), (49, 49))],
        "test_006": [(1, 1), (1, 49), (2, 1), (2, 49), (4, 1), (4, 49), (8, 1), (8, 49), (16, 1), (16, 49),
                     (32, 1), (32, 49), (49, 1), (49, 49)],
        "test_007": [((0.5, 0.5), (1.5, 48.5)), ((0.5, 0.5), (48.5, 1.5)), ((48.5, 48.5), (47.5, 0.5)),
                     ((48.5, 48.5), (0.5, 47.5))],
    }
    canvases = {"normal": dict(plot_width=50, plot_height=50, x_range=(0, 49), y_range=(0, 49)),
                "clipped": dict(plot_width=20, plot_height=20, x_range=(14, 34), y_range=(14, 34))}
    cases = []
    for name, pts in sets.items():
        if name == "test_006":
            frames = [{"x": np.array([p[0] for p in pts], dtype=np.float64),
                       "y": np.array([p[1] for p in pts], dtype=np.float64)}]
        else:
            frames = [{"x": np.array([a[0], b[0]], dtype=np.float64), "y": np.array([a[1], b[1]], dtype=np.float64)}
                      for a, b in pts]
        for f in frames:
            f["val"] = np.full(f["x"].size, 5.0)
        for aa in ("antialias", "noaa"):
            for cv in ("normal", "clipped"):
                key = f"{name}_{aa}_{cv}"
                cases.append(dict(id=key, frames=frames, canvas=canvases[cv], line_width=1.0 if aa == "antialias" else 0.0,
                                  expected=golden_array(g[key])))
    return cases


def stack_sum(aggs):
    """xr.concat(aggs, 'stack').sum(dim='stack'): NaN skipped, the float64 sum
    taken along the stack in order (an all-NaN pixel sums to 0)."""
    acc = None
    for a in aggs:
        a = np.where(np.isnan(a), 0.0, a)
        acc = a if acc is None else acc + a
    return acc


def eq_hist_agg_a():
    """test_transfer_functions.py:23-37 build_agg 'a' (uint32, zero diagonal)."""
    a = np.arange(10, 19, dtype="u4").reshape((3, 3))
    a[[0, 1, 2], [0, 1, 2]] = 0
    c = np.arange(10, 19, dtype="f8").reshape((3, 3))
    c[[0, 1, 2], [0, 1, 2]] = np.nan
    return a, c


def shade_golden(key, how=None):
    """test_transfer_functions.py solution images (uint32 RGBA) from tests/golden/shade.json."""
    g = load_golden("shade.json", key)
    return golden_array(g[how] if how is not None else g)


def span_variants(x, sol):
    """check_span (test_transfer_functions.py:130-149): mask one pixel, then also
    the largest value; the masked pixels become transparent."""
    x = x.copy()
    sol = sol.copy()
    x[0, 1] = 0 if x.dtype.kind in "iu" else np.nan
    sol[0, 1] = sol[0, 0]
    yield x.copy(), sol.copy()
    x[2, 1] = 0 if x.dtype.kind in "iu" else np.nan
    sol[2, 1] = sol[0, 0]
    yield x.copy(), sol.copy()


def lines_golden(key):
    return load_golden("lines_multi.json", key)


def line_kwargs(kw):
    """The Canvas.line keyword arguments of a golden case (constant arrays as numpy)."""
    out = {}
    for k, v in kw.items():
        out[k] = np.array(v["array"]) if isinstance(v, dict) else v
    return out


def multi_line_arrays(columns, kw):
    """(layout, xs, ys) float64 arrays of a multi-line case, as the glyphs see them
    (core.py:412-456 dispatch with the column broadcast of :1433-1443)."""
    x, y, axis = kw["x"], kw["y"], kw.get("axis", 0)
    if isinstance(x, str) and isinstance(y, (list, tuple)):
        x = [x] * len(y)
    if isinstance(y, str) and isinstance(x, (list, tuple)):
        y = [y] * len(x)

    def arr(spec):
        if isinstance(spec, dict):
            return np.array(spec["array"], dtype=np.float64)
        if isinstance(spec, np.ndarray):
            return spec.astype(np.float64)
        return np.stack([np.asarray(columns[c], dtype=np.float64) for c in spec], axis=1)

    return (1 if axis == 0 else 2), arr(x), arr(y)
