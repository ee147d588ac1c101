"""Partitioned sources: every row partition aggregated into its own partial
bases, combined elementwise (dsgb_combine), finalized once, must equal the
same rows as one frame (datashader's dask path, dask.py:86-219).  Bit-exact
except float64 sums (1e-12 relative: another addition order)."""
from __future__ import annotations

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
from datashader_gb300 import synthetic
from gpu_helpers import assert_same, to_numpy

pytestmark = pytest.mark.gpu


def _cols(n, seed):
    rng = np.random.default_rng(seed)
    x, y = synthetic.gaussian_mixture_np(n, seed=seed, dtype=np.float32)
    v = rng.lognormal(0.0, 1.0, n)
    v[rng.random(n) < 0.05] = np.nan
    cat = rng.integers(0, 6, n).astype(np.int8)
    return {"x": x, "y": y, "v": v, "cat": cat}


def _frame(cols, lo=0, hi=None, offset=0):
    t = {k: torch.from_numpy(np.ascontiguousarray(v[lo:hi])).cuda() for k, v in cols.items()}
    return ds.TensorFrame(t, categories={"cat": list(range(6))}, row_offset=offset)


AGG = ds.summary(count=ds.count(), s=ds.sum("v"), m=ds.mean("v"), mx=ds.max("v"), mn=ds.min("v"),
                 w=ds.where(ds.max("v")), wmin=ds.where(ds.min("v")), by=ds.by("cat", ds.count()),
                 any=ds.any("v"))


@pytest.mark.parametrize("cuts", [(0, 1_200_000), (0, 37, 400_001, 1_999_999, 2_000_000)])
def test_partitions_equal_one_frame(cuts):
    n = 2_000_000
    cols = _cols(n, seed=21)
    whole = to_numpy(ds.Canvas(600, 400, (-4, 4), (-3, 3)).points(_frame(cols), "x", "y", AGG))
    bounds = list(cuts) + [n] if cuts[-1] != n else list(cuts)
    parts = [_frame(cols, a, b) for a, b in zip(bounds[:-1], bounds[1:])]
    got = to_numpy(ds.Canvas(600, 400, (-4, 4), (-3, 3)).points(ds.PartitionedFrame(parts), "x", "y", AGG))
    for k in whole:
        if k in ("s", "m"):
            assert_same(got[k], whole[k], rtol=1e-12, what=k)
        else:
            assert_same(got[k], whole[k], what=k)


def test_partitions_autorange_and_count_path():
    cols = _cols(3_000_000, seed=22)
    cvs = ds.Canvas(1024, 1024)
    whole = cvs.points(_frame(cols), "x", "y", ds.count())
    parts = ds.PartitionedFrame([_frame(cols, 0, 1_500_000), _frame(cols, 1_500_000)])
    got = cvs.points(parts, "x", "y", ds.count())
    assert got.attrs["x_range"] == whole.attrs["x_range"] and got.attrs["y_range"] == whole.attrs["y_range"]
    assert_same(to_numpy(got), to_numpy(whole))


GATHER = ds.summary(f=ds.first("v"), l=ds.last("v"), wy=ds.where(ds.max("v"), "y"),
                    wx=ds.where(ds.min("v"), "x"), byf=ds.by("cat", ds.first("v")))


@pytest.mark.parametrize("cuts", [(0, 1_000_000), (0, 1, 250_000, 250_001, 1_500_000)])
def test_partitions_gather_lookups_from_the_holding_partition(cuts):
    """first / last / where with a lookup column: the combined row-index base
    picks a global row, the finalize reads it from the partition holding it."""
    n = 1_800_000
    cols = _cols(n, seed=23)
    cvs = ds.Canvas(500, 300, (-4, 4), (-3, 3))
    whole = to_numpy(cvs.points(_frame(cols), "x", "y", GATHER))
    bounds = list(cuts) + [n]
    parts = [_frame(cols, a, b, offset=a) for a, b in zip(bounds[:-1], bounds[1:])]
    got = to_numpy(cvs.points(ds.PartitionedFrame(parts), "x", "y", GATHER))
    for k in whole:
        assert_same(got[k], whole[k], what=k)


def test_partitions_reject_gathered_lookups_beyond_64():
    cols = _cols(6500, seed=24)
    parts = ds.PartitionedFrame([_frame(cols, a, a + 100, offset=a) for a in range(0, 6500, 100)])
    with pytest.raises(NotImplementedError):
        ds.Canvas(16, 16, (-4, 4), (-4, 4)).points(parts, "x", "y", ds.first("v"))


def _line_frame(cols, lo, hi):
    return ds.TensorFrame({k: torch.from_numpy(np.ascontiguousarray(v[lo:hi])).cuda() for k, v in cols.items()})


@pytest.mark.parametrize("lw", [0.0, 1.5])
@pytest.mark.parametrize("red", ["count", "sum", "max"])
def test_partitioned_lines_follow_the_reference_dask_path(lw, red):
    """LineAxis0 over row partitions (dask.py:222-266): partition 0 drawn with
    plot_start, every later one behind the previous partition's last row with
    plot_start False; partials combined, finalized once.  Against the oracle
    run on the same chunks and combined the reference's way (sum / nansum /
    nanmax)."""
    from datashader_gb300 import synthetic as S
    import oracle
    x, y, v, _ = S.time_series_np(8, 500, seed=4)
    cols = {"x": x, "y": y, "v": v}
    n = len(x)
    cuts = [0, 700, 701, 2004, 3006, n]               # inside a series, next to it, on NaN separators
    parts = [_line_frame(cols, a, b) for a, b in zip(cuts[:-1], cuts[1:])]
    yr = (float(np.nanmin(y)) - 0.01, float(np.nanmax(y)) + 0.01)
    cvs = ds.Canvas(plot_width=300, plot_height=200, x_range=(0.0, 1.0), y_range=yr)
    agg = {"count": ds.count(), "sum": ds.sum("v"), "max": ds.max("v")}[red]
    got = to_numpy(cvs.line(ds.PartitionedFrame(parts), "x", "y", agg=agg, line_width=lw))
    spec = oracle.spec(red, None if red == "count" else "v")
    partials = []
    for i, (a, b) in enumerate(zip(cuts[:-1], cuts[1:])):
        lo = a if i == 0 else a - 1
        chunk = {k: val[lo:b] for k, val in cols.items()}
        partials.append(oracle.line_axis0(chunk, "x", "y", 300, 200, (0.0, 1.0), yr, [spec], line_width=lw,
                                          plot_start=(i == 0), row_offset=lo)[0])
    stack = np.stack([np.asarray(p, dtype=np.float64) for p in partials])
    if red == "max":
        want = np.fmax.reduce(stack, axis=0)
    elif np.issubdtype(partials[0].dtype, np.integer):
        want = stack.sum(axis=0)
    else:
        with np.errstate(invalid="ignore"):
            want = np.where(np.isnan(stack).all(axis=0), np.nan, np.nansum(stack, axis=0))
    want = want.astype(partials[0].dtype)
    rtol = 0.0 if red == "max" or (red == "count" and lw == 0) else (3e-7 if partials[0].dtype == np.float32 else 1e-12)
    assert_same(got, want, rtol=rtol, what=f"{red} lw={lw}")


def _multi_cols(nrows, nv, seed):
    rng = np.random.default_rng(seed)
    cols = {}
    for j in range(nv):
        cols[f"x{j}"] = np.linspace(0, 1, nrows) + 0.01 * j
        cols[f"y{j}"] = np.cumsum(rng.normal(0, 0.05, nrows))
    cols["v"] = rng.uniform(0, 1, nrows)
    return cols


@pytest.mark.parametrize("lw", [0.0, 1.5])
def test_partitioned_lines_axis1_equal_one_frame(lw):
    """The LinesAxis1 family over row partitions (the generic dask path,
    dask.py:86-219): a line is one row, so partitions lose nothing and the
    combined result equals the single-frame one (first / last by global row,
    which for one line per row is the visit order too)."""
    cols = _multi_cols(300, 40, 41)
    xs = [f"x{j}" for j in range(40)]
    ys = [f"y{j}" for j in range(40)]
    whole = _line_frame(cols, 0, None)
    cuts = [0, 1, 77, 150, 299, 300]
    parts = ds.PartitionedFrame([_line_frame(cols, a, b) for a, b in zip(cuts[:-1], cuts[1:])])
    aggs = {"count": ds.count(), "sum": ds.sum("v"), "max": ds.max("v"), "any": ds.any()}
    if lw == 0:
        aggs.update(first=ds.first("v"), last=ds.last("v"), where=ds.where(ds.min("v")))
    cvs = ds.Canvas(plot_width=120, plot_height=80)
    for axis, kx in ((1, xs), (1, np.linspace(0, 1, 40))):
        for name, agg in aggs.items():
            got = to_numpy(cvs.line(parts, x=kx, y=ys, axis=axis, agg=agg, line_width=lw))
            ref = to_numpy(cvs.line(whole, x=kx, y=ys, axis=axis, agg=agg, line_width=lw))
            rtol = 1e-12 if name == "sum" else (3e-7 if ref.dtype == np.float32 else 0.0)
            assert_same(got, ref, rtol=rtol, atol=1e-7 if ref.dtype == np.float32 else 0.0, what=name)


def test_partitioned_line_axis0_multi_by_partition():
    """LineAxis0Multi over row partitions: each partition's segments drawn
    alone (the generic dask path has no overlap for these glyphs), partials
    combined; first by the smallest global row (a row-index reduction), against
    the oracle run per partition and combined the reference's way."""
    import oracle
    import refcases
    cols = _multi_cols(500, 3, 43)
    kw = dict(x=[f"x{j}" for j in range(3)], y=[f"y{j}" for j in range(3)])
    cuts = [0, 120, 121, 333, 500]
    parts = ds.PartitionedFrame([_line_frame(cols, a, b) for a, b in zip(cuts[:-1], cuts[1:])])
    layout, xs, ys = refcases.multi_line_arrays(cols, kw)
    xr, yr = (0.0, 1.1), (float(ys.min()), float(ys.max()))
    cvs = ds.Canvas(plot_width=150, plot_height=90, x_range=xr, y_range=yr)
    specs = [oracle.spec("count"), oracle.spec("max", "v"), oracle.spec("min_row")]
    partials = [oracle.lines({"v": cols["v"][a:b]}, 1, xs[a:b], ys[a:b], 150, 90, xr, yr, specs, row_offset=a)
                for a, b in zip(cuts[:-1], cuts[1:])]
    got = cvs.line(parts, agg=ds.summary(c=ds.count(), m=ds.max("v"), f=ds.first("v")), **kw)
    assert_same(to_numpy(got["c"]), np.sum([p[0] for p in partials], axis=0).astype(np.uint32))
    assert_same(to_numpy(got["m"]), np.fmax.reduce(np.stack([p[1] for p in partials]), axis=0))
    rows = np.stack([np.where(p[2] < 0, np.iinfo(np.int64).max, p[2]) for p in partials]).min(axis=0)
    want_first = np.where(rows == np.iinfo(np.int64).max, np.nan, cols["v"][np.minimum(rows, 499)])
    assert_same(to_numpy(got["f"]), want_first)
