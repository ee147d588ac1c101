"""Plans of several bases over at least 2^20 float32 rows: the partitioned
path (rows grouped by canvas block, every base of a block in shared memory).

Against the oracle: integer, index, min / max / first / last / where / by
results exact, float64 sums and means 1e-12 relative.  The cases cover
NaN values, negative and out-of-range category codes, pixel-edge and
out-of-bounds coordinates, canvases whose sides are not multiples of the
block, global row numbers past 2^32, accumulation over chunks (HostFrame),
value and category columns of other dtypes, and (against the generic
kernels, themselves pinned to the oracle) more rows than one pass takes.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
from datashader_gb300 import synthetic
from gpu_helpers import assert_same, frame_from_numpy, to_numpy
from oracle_bridge import run_points

pytestmark = pytest.mark.gpu

RTOL_SUM = 1e-12
N = (1 << 21) + 3
EXACT = ("count", "any", "max", "min", "first", "last", "where_row", "where_index", "where_min", "by_cat",
         "by_max", "count_v")


def _cols(n, seed, w_range=(-4.0, 4.0), h_range=(-4.0, 4.0), w=1024, h=1024):
    x, y = synthetic.gaussian_mixture_np(n, seed=seed, dtype=np.float32)
    rng = np.random.default_rng(seed + 1)
    sx = (w_range[1] - w_range[0]) / 8.0
    sy = (h_range[1] - h_range[0]) / 8.0
    x = (w_range[0] + (x + 4.0) * sx).astype(np.float32)
    y = (h_range[0] + (y + 4.0) * sy).astype(np.float32)
    # pixel edges, their float neighbours, the bounds and beyond, NaN
    m = 4096
    ex = (w_range[0] + np.arange(w + 1) * (w_range[1] - w_range[0]) / w).astype(np.float32)
    ey = (h_range[0] + np.arange(h + 1) * (h_range[1] - h_range[0]) / h).astype(np.float32)
    probe_x = np.concatenate([ex, np.nextafter(ex, np.float32(np.inf)), np.nextafter(ex, np.float32(-np.inf)),
                              np.float32([np.nan, np.inf, -np.inf, 1e30])])
    probe_y = np.concatenate([ey, np.nextafter(ey, np.float32(np.inf)), np.nextafter(ey, np.float32(-np.inf)),
                              np.float32([np.nan, np.inf, -np.inf, -1e30])])
    idx = rng.choice(n, size=m, replace=False)
    x[idx] = probe_x[rng.integers(0, probe_x.size, m)]
    y[idx] = probe_y[rng.integers(0, probe_y.size, m)]
    v = rng.lognormal(0.0, 1.0, n)
    v[rng.random(n) < 0.02] = np.nan
    v[rng.integers(0, n, 2000)] = 7.5                # ties of values across rows
    cat = rng.integers(-9, 9, n).astype(np.int8)     # -8..-1 wrap, 8 and -9 are skipped
    index = (np.arange(n, dtype=np.int64) * 7) % 1_000_003
    return {"x": x, "y": y, "v": v, "cat": cat, "index": index}


def _summary():
    return ds.summary(
        count=ds.count(), count_v=ds.count("v"), any=ds.any("v"), sum=ds.sum("v"), mean=ds.mean("v"),
        max=ds.max("v"), min=ds.min("v"), first=ds.first("v"), last=ds.last("v"),
        where_row=ds.where(ds.max("v")), where_index=ds.where(ds.max("v"), "index"),
        where_min=ds.where(ds.min("v"), "index"), by_cat=ds.by("cat", ds.count()))


def _check(got, ref):
    for k in ref:
        if k in EXACT:
            assert_same(got[k], ref[k], what=k)
        else:
            assert_same(got[k], ref[k], rtol=RTOL_SUM, what=k)


CATS = {"cat": list(range(8))}


@pytest.mark.parametrize("w,h,xr,yr", [(1024, 1024, (-4.0, 4.0), (-4.0, 4.0)),
                                       (1000, 999, (-3.3, 2.7), (0.1, 0.7)),
                                       (4096, 2160, (-4.0, 4.0), (-4.0, 4.0)),
                                       (70, 33, (-2.0, 2.0), (-1.0, 3.0))])
def test_part_summary_vs_oracle(w, h, xr, yr):
    cols = _cols(N, seed=w + h, w_range=xr, h_range=yr, w=w, h=h)
    canvas = dict(plot_width=w, plot_height=h, x_range=xr, y_range=yr)
    agg = _summary()
    got = to_numpy(ds.Canvas(**canvas).points(frame_from_numpy(cols, CATS), "x", "y", agg))
    ref = run_points(cols, CATS, agg, canvas)
    _check(got, ref)
    assert got["count"].sum() > 0.9 * N


def test_part_value_and_category_dtypes():
    """float32 and int32 value columns, uint8 and int64 category codes; by()
    over value reductions (a category dimension on sum / max)."""
    cols = _cols(N, seed=5)
    rng = np.random.default_rng(6)
    cols["vf"] = rng.normal(size=N).astype(np.float32)
    cols["vf"][rng.random(N) < 0.01] = np.nan
    cols["vi"] = rng.integers(-1000, 1000, N).astype(np.int32)
    cols["cu"] = rng.integers(0, 5, N).astype(np.uint8)
    cols["cl"] = rng.integers(-3, 5, N).astype(np.int64)
    cats = {"cu": list(range(5)), "cl": list(range(4))}
    canvas = dict(plot_width=640, plot_height=480, x_range=(-4.0, 4.0), y_range=(-4.0, 4.0))
    for agg in (ds.summary(count=ds.count(), sum=ds.sum("vf"), max=ds.max("vf"), by_max=ds.by("cu", ds.max("vf"))),
                ds.summary(sum=ds.sum("vi"), min=ds.min("vi"), last=ds.last("vi"), by_cat=ds.by("cl", ds.sum("vi")))):
        got = to_numpy(ds.Canvas(**canvas).points(frame_from_numpy(cols, cats), "x", "y", agg))
        _check(got, run_points(cols, cats, agg, canvas))


def test_part_global_rows_past_2_32():
    """first / last / where with a frame whose rows start at 2^33 + 5."""
    cols = _cols(N, seed=9)
    off = (1 << 33) + 5
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in cols.items()}
    frame = ds.TensorFrame(t, categories=CATS, row_offset=off)
    canvas = dict(plot_width=800, plot_height=600, x_range=(-4.0, 4.0), y_range=(-4.0, 4.0))
    agg = ds.summary(first=ds.first("v"), last=ds.last("v"), where_row=ds.where(ds.max("v")),
                     where_min=ds.where(ds.min("v"), "index"), count=ds.count())
    got = to_numpy(ds.Canvas(**canvas).points(frame, "x", "y", agg))
    ref = run_points(cols, CATS, agg, canvas, row_offset=off)
    _check(got, ref)
    assert got["where_row"].max() > (1 << 32)


def test_part_hostframe_chunks_accumulate():
    """A host frame streamed in chunks of 2^20 + 7 rows: three chunks take the
    partitioned path and accumulate into the same bases, the short last one
    the generic kernels; equal to the oracle over all rows."""
    n = 3 * ((1 << 20) + 7) + 54_321
    cols = _cols(n, seed=21)
    host = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in cols.items()}
    frame = ds.HostFrame(host, categories=CATS, chunk_rows=(1 << 20) + 7)
    canvas = dict(plot_width=1024, plot_height=768, x_range=(-4.0, 4.0), y_range=(-3.0, 3.0))
    agg = _summary()
    got = to_numpy(ds.Canvas(**canvas).points(frame, "x", "y", agg))
    _check(got, run_points(cols, CATS, agg, canvas))


def test_part_matches_generic_kernels_past_one_pass():
    """1.4e8 rows (more than the 2^27 rows of one pass): equal to the generic
    kernels (selected by the exact-binning flag), exact but for the float64
    sums."""
    from datashader_gb300 import _native as N_
    from datashader_gb300.core import gpu_pipeline
    from datashader_gb300.glyphs import Point
    n = 140_000_001
    dev = torch.device("cuda", 0)
    x, y = synthetic.gaussian_mixture_torch(n, seed=4, device=dev)
    g = torch.Generator(device=dev).manual_seed(4)
    v = torch.empty(n, dtype=torch.float64, device=dev).log_normal_(0.0, 1.0, generator=g)
    cat = torch.randint(0, 8, (n,), dtype=torch.int8, device=dev, generator=g)
    frame = ds.TensorFrame({"x": x, "y": y, "v": v, "cat": cat}, categories=CATS)
    cv = ds.Canvas(plot_width=1024, plot_height=1024, x_range=(-4, 4), y_range=(-4, 4))
    agg = ds.summary(count=ds.count(), sum=ds.sum("v"), max=ds.max("v"), first=ds.first("v"),
                     last=ds.last("v"), where_row=ds.where(ds.min("v")), by_cat=ds.by("cat", ds.count()))
    a = to_numpy(gpu_pipeline(frame, cv, Point("x", "y"), agg))
    b = to_numpy(gpu_pipeline(frame, cv, Point("x", "y"), agg, flags=N_.FLAG_EXACT_BIN))
    for k in a:
        if k == "sum":
            assert_same(a[k], b[k], rtol=RTOL_SUM, what=k)
        else:
            assert_same(a[k], b[k], what=k)
    assert int(a["count"].sum()) > 0.95 * n
    assert a["where_row"].max() > (1 << 27)


def test_part_rows_past_a_blocks_room_take_the_direct_path():
    """The block rooms come from a sample of one tile of 1,024 rows in eight.
    Rows laid out so that the sampled tiles fall left of x = 0 and every other
    row right of it: the right half's blocks get the minimum room and most of
    their rows go straight to the bases (L2 atomics).  Equal to the oracle."""
    n = (1 << 21) + 3
    cols = _cols(n, seed=31)
    tile = np.arange(n) // 1024
    x = np.abs(cols["x"]).astype(np.float32)
    cols["x"] = np.where(tile % 8 == 0, -x, x).astype(np.float32)
    canvas = dict(plot_width=1024, plot_height=1024, x_range=(-4.0, 4.0), y_range=(-4.0, 4.0))
    agg = _summary()
    got = to_numpy(ds.Canvas(**canvas).points(frame_from_numpy(cols, CATS), "x", "y", agg))
    _check(got, run_points(cols, CATS, agg, canvas))
    assert got["count"][:, 600:].sum() > 0.8 * n * 7 / 8 / 2
