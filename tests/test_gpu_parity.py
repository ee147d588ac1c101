"""GPU vs CPU oracle on seeded synthetic inputs shaped like the benchmark configs.

Tolerances: integer / index / min / max / first / last / where / by-count
results and the eq_hist histogram are bit-exact.  float64 sums and means are
accumulated by atomics in a different order than the oracle's row-order
fold: 1e-12 relative.  Antialiased line sums: 1e-12 relative (the coverage
values themselves are bit-identical; only the summation order differs).
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
import oracle
from datashader_gb300 import synthetic
from gpu_helpers import assert_same, frame_from_numpy, to_numpy
from oracle_bridge import run_line, run_points

pytestmark = pytest.mark.gpu

CANVAS2 = dict(plot_width=1024, plot_height=1024, x_range=(-4, 4), y_range=(-4, 4))
RTOL_SUM = 1e-12


def _cfg2_frame(n, seed=0, xy_dtype=np.float32):
    x, y = synthetic.gaussian_mixture_np(n, seed, dtype=xy_dtype)
    rng = np.random.default_rng(seed + 1)
    v = rng.lognormal(0.0, 1.0, n)
    v[rng.integers(0, n, n // 100)] = np.nan          # NaN values are skipped by every reduction
    cat = rng.integers(0, 8, n).astype(np.int8)
    idx = np.arange(n, dtype=np.int64)
    # rows exactly on the bounds, on pixel edges, just inside/outside, NaN coordinates
    k = np.arange(64)
    edge = (-4 + k / 128.0).astype(xy_dtype)
    x[:64] = edge
    y[:64] = edge[::-1]
    x[64:70] = np.array([-4, 4, 4, -4, np.nan, 4.0000001], dtype=xy_dtype)
    y[64:70] = np.array([-4, 4, -4, 4, 0, 0], dtype=xy_dtype)
    nxt = np.nextafter(edge, np.array(np.inf, dtype=xy_dtype))
    x[70:134] = nxt
    y[70:134] = np.nextafter(edge, np.array(-np.inf, dtype=xy_dtype))
    cols = {"x": x, "y": y, "v": v, "cat": cat, "index": idx}
    return cols, {"cat": list(range(8))}


def _cfg2_summary():
    return ds.summary(
        count=ds.count(), sum=ds.sum("v"), mean=ds.mean("v"), max=ds.max("v"), min=ds.min("v"),
        first=ds.first("v"), last=ds.last("v"), where_row=ds.where(ds.max("v")),
        where_index=ds.where(ds.max("v"), "index"), by_cat=ds.by("cat", ds.count()))


@pytest.mark.parametrize("xy_dtype", [np.float32, np.float64])
def test_points_cfg2_summary_vs_oracle(xy_dtype):
    cols, cats = _cfg2_frame(300_000, seed=3, xy_dtype=xy_dtype)
    agg = _cfg2_summary()
    got = to_numpy(ds.Canvas(**CANVAS2).points(frame_from_numpy(cols, cats), "x", "y", agg))
    ref = run_points(cols, cats, agg, CANVAS2)
    for k in ("count", "max", "min", "first", "last", "where_row", "where_index", "by_cat"):
        assert_same(got[k], ref[k], what=k)
    for k in ("sum", "mean"):
        assert_same(got[k], ref[k], rtol=RTOL_SUM, what=k)


@pytest.mark.parametrize("warp_agg", [False, True])
def test_points_cfg1_count_f64(warp_agg):
    x, y = synthetic.gaussian_mixture_np(500_000, seed=7)
    cols = {"x": x, "y": y}
    canvas = dict(plot_width=512, plot_height=512, x_range=(-4, 4), y_range=(-4, 4))
    frame = frame_from_numpy(cols)
    from datashader_gb300.core import gpu_pipeline
    from datashader_gb300 import _native as N
    from datashader_gb300.glyphs import Point
    flags = N.FLAG_WARP_AGG if warp_agg else 0
    got = to_numpy(gpu_pipeline(frame, ds.Canvas(**canvas), Point("x", "y"), ds.count(), flags=flags))
    ref = run_points(cols, {}, ds.count(), canvas)
    assert_same(got, ref)


def test_points_exact_flag_matches_fast_path():
    cols, cats = _cfg2_frame(200_000, seed=11)
    frame = frame_from_numpy(cols, cats)
    from datashader_gb300.core import gpu_pipeline
    from datashader_gb300 import _native as N
    from datashader_gb300.glyphs import Point
    cv = ds.Canvas(**CANVAS2)
    a = to_numpy(gpu_pipeline(frame, cv, Point("x", "y"), ds.count()))
    b = to_numpy(gpu_pipeline(frame, cv, Point("x", "y"), ds.count(), flags=N.FLAG_EXACT_BIN))
    assert_same(a, b)


def test_points_pixel_edges_dense():
    """Every float32 value within a few ulp of every pixel edge of a 1024 px axis."""
    edges = (-4 + np.arange(1025) / 128.0).astype(np.float32)
    vals = [edges]
    up, dn = edges.copy(), edges.copy()
    for _ in range(3):
        up = np.nextafter(up, np.float32(np.inf))
        dn = np.nextafter(dn, np.float32(-np.inf))
        vals += [up.copy(), dn.copy()]
    xs = np.concatenate(vals)
    rng = np.random.default_rng(5)
    ys = rng.permutation(xs)
    cols = {"x": xs, "y": ys}
    got = to_numpy(ds.Canvas(**CANVAS2).points(frame_from_numpy(cols), "x", "y", ds.count()))
    ref = run_points(cols, {}, ds.count(), CANVAS2)
    assert_same(got, ref)


def test_points_offset_range_uses_exact_path():
    """A range far from zero (float32 binning error bound too large): exact path."""
    rng = np.random.default_rng(9)
    x = 1e6 + rng.uniform(0, 1, 100_000)
    y = rng.uniform(0, 1, 100_000)
    cols = {"x": x, "y": y, "v": rng.normal(size=100_000)}
    canvas = dict(plot_width=300, plot_height=200, x_range=(1e6, 1e6 + 1), y_range=(0, 1))
    agg = ds.summary(c=ds.count(), m=ds.max("v"))
    got = to_numpy(ds.Canvas(**canvas).points(frame_from_numpy(cols), "x", "y", agg))
    ref = run_points(cols, {}, agg, canvas)
    assert_same(got, ref)


def test_points_row_offset_and_unaligned_columns():
    cols, cats = _cfg2_frame(50_001, seed=13)
    # a frame of column views starting one element in (not 16-byte aligned)
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in cols.items()}
    sl = {k: v[1:] for k, v in t.items()}
    frame = ds.TensorFrame(sl, categories=cats, row_offset=1000)
    agg = ds.summary(first=ds.first("v"), where_row=ds.where(ds.max("v")), c=ds.count())
    got = to_numpy(ds.Canvas(**CANVAS2).points(frame, "x", "y", agg))
    sub = {k: v[1:] for k, v in cols.items()}
    ref = run_points(sub, cats, agg, CANVAS2, row_offset=1000)
    assert_same(got, ref)


def test_points_empty_and_all_outside():
    for n in (0, 17):
        cols = {"x": np.full(n, 100.0), "y": np.full(n, 100.0), "v": np.ones(n)}
        agg = ds.summary(c=ds.count(), s=ds.sum("v"), m=ds.max("v"), w=ds.where(ds.min("v")))
        got = to_numpy(ds.Canvas(**CANVAS2).points(frame_from_numpy(cols), "x", "y", agg))
        ref = run_points(cols, {}, agg, CANVAS2)
        assert_same(got, ref)


def test_points_autorange():
    x, y = synthetic.gaussian_mixture_np(10_000, seed=21)
    x[5] = np.nan
    cols = {"x": x, "y": y}
    canvas = dict(plot_width=200, plot_height=100)
    got = ds.Canvas(**canvas).points(frame_from_numpy(cols), "x", "y", ds.count())
    ref = run_points(cols, {}, ds.count(), canvas)
    assert_same(to_numpy(got), ref)
    assert got.x_range == oracle.maybe_expand_bounds(oracle.compute_bounds(x))


def test_points_deterministic_repeat():
    cols, cats = _cfg2_frame(100_000, seed=17)
    frame = frame_from_numpy(cols, cats)
    cvs = ds.Canvas(**CANVAS2)
    agg = ds.summary(c=ds.count(), w=ds.where(ds.max("v")), f=ds.first("v"), b=ds.by("cat", ds.count()))
    a = to_numpy(cvs.points(frame, "x", "y", agg))
    b = to_numpy(cvs.points(frame, "x", "y", agg))
    assert_same(a, b)


# ------------------------------------------------------------------ lines

def _series(nseries, length, seed=0):
    x, y, v, _ = synthetic.time_series_np(nseries, length, seed)
    return {"x": x, "y": y, "v": v}


@pytest.mark.parametrize("line_width", [1.5, 1.0, 0.5, 2.0])
def test_line_aa_sum_vs_oracle(line_width):
    cols = _series(40, 400, seed=1)
    canvas = dict(plot_width=256, plot_height=128)
    got = ds.Canvas(**canvas).line(frame_from_numpy(cols), "x", "y", agg=ds.sum("v"), line_width=line_width)
    ref = run_line(cols, {}, ds.sum("v"), canvas, line_width)
    assert_same(to_numpy(got), ref, rtol=RTOL_SUM, atol=1e-13)


@pytest.mark.parametrize("agg_name", ["count", "any", "max", "mean", "min_row", "summary2stage"])
def test_line_aa_reductions_vs_oracle(agg_name):
    cols = _series(10, 300, seed=2)
    canvas = dict(plot_width=200, plot_height=100)
    agg = {"count": ds.count(), "any": ds.any(), "max": ds.max("v"), "mean": ds.mean("v"),
           "min_row": ds._min_row_index(),
           "summary2stage": ds.summary(c=ds.count(), mn=ds.min("v"), w=ds.where(ds.max("v")))}[agg_name]
    got = to_numpy(ds.Canvas(**canvas).line(frame_from_numpy(cols), "x", "y", agg=agg, line_width=1.5))
    ref = run_line(cols, {}, agg, canvas, 1.5)
    pairs = ref.items() if isinstance(ref, dict) else [(None, ref)]
    for k, r in pairs:
        g = got[k] if k is not None else got
        if r.dtype == np.float32:      # the reference sums float32 aggregates in float32
            assert_same(g, r, rtol=3e-7, atol=1e-7, what=str(k))
        elif r.dtype.kind == "f":
            assert_same(g, r, rtol=RTOL_SUM, atol=1e-13, what=str(k))
        else:
            assert_same(g, r, what=str(k))


@pytest.mark.parametrize("line_width", [1.5, 0.5, 3.0])
def test_line_aa_queued_matches_per_segment_kernel(line_width):
    """The antialiased forward with pixels classified in float32 and worked off
    by case against the per-segment scan (DSGB_FLAG_EXACT_BIN): the same pixels
    and coverage, float64 sums in another atomic order.  Time series, plus a
    staircase of axis-aligned steps between pixel centres, where the along /
    length and previous-direction tests meet their thresholds exactly."""
    from datashader_gb300 import _native as N_
    from datashader_gb300.core import gpu_pipeline
    from datashader_gb300.glyphs import LineAxis0
    cols = _series(30, 500, seed=7)
    ylo, yhi = float(np.nanmin(cols["y"])), float(np.nanmax(cols["y"]))
    k = np.arange(500)
    px, py = 50 + (k + 1) // 2, 20 + k // 2          # unit steps right / up between pixel centres
    stair = {"x": (px + 0.5) / 400.0, "y": ylo + (py + 0.5) * (yhi - ylo) / 300.0, "v": np.linspace(0.0, 1.0, k.size)}
    cols = {c: np.concatenate([cols[c], [np.nan], stair[c]]) for c in cols}
    frame = frame_from_numpy(cols)
    cv = ds.Canvas(plot_width=400, plot_height=300, x_range=(0.0, 1.0), y_range=(ylo, yhi))
    glyph = LineAxis0("x", "y")
    glyph.set_line_width(line_width)
    agg = ds.summary(c=ds.count(), s=ds.sum("v"), m=ds.max("v"))
    a = to_numpy(gpu_pipeline(frame, cv, glyph, agg, antialias=True))
    b = to_numpy(gpu_pipeline(frame, cv, glyph, agg, antialias=True, flags=N_.FLAG_EXACT_BIN))
    assert_same(a["m"], b["m"], what="max")
    for key in ("c", "s"):
        if a[key].dtype == np.float32:     # float32 coverage sums: atomic order at float32 rounding
            assert_same(a[key], b[key], rtol=3e-7, atol=1e-7, what=key)
        else:
            assert_same(a[key], b[key], rtol=RTOL_SUM, atol=1e-13, what=key)
    assert np.nansum(a["c"]) > 1000


def test_line_aa_without_workspace_matches_workspace():
    """dsgb_line_axis0 without a workspace draws the segments in row order
    (the queued scan without the work order); with one, in work order: the
    same pixels and coverage, float sums in another atomic order."""
    import ctypes
    from datashader_gb300 import _native as N_
    from datashader_gb300.autograd import _canvas_desc
    from datashader_gb300.compiler import compile_plan
    from datashader_gb300.core import Executor
    from datashader_gb300.glyphs import LineAxis0
    cols = _series(25, 400, seed=13)
    frame = frame_from_numpy(cols)
    ylo, yhi = float(np.nanmin(cols["y"])), float(np.nanmax(cols["y"]))
    cv = ds.Canvas(plot_width=300, plot_height=200, x_range=(0.0, 1.0), y_range=(ylo, yhi))
    cd = _canvas_desc(cv, cv.x_range, cv.y_range)
    glyph = LineAxis0("x", "y")
    glyph.set_line_width(1.5)
    agg = ds.summary(c=ds.count(), s=ds.sum("v"), m=ds.max("v"))
    L = N_.lib()
    st = torch.cuda.current_stream().cuda_stream
    n = len(frame)
    got = []
    for with_ws in (False, True):
        plan = compile_plan(agg, frame, antialias=True)
        ex = Executor(frame, plan, glyph)
        ex.allocate(200, 300, torch.device("cuda"))
        args = (ex.cols, len(ex.names), n, 0, 0, 1, ctypes.byref(cd), 1.5, 1, int(plan.overwrite),
                int(plan.use_2_stage), ex.bases, len(plan.bases), ex.outs, ex.nouts)
        if with_ws:
            wsz = int(L.dsgb_line_workspace_size(n))
            ws = torch.empty(wsz, dtype=torch.uint8, device="cuda")
            N_.check(L.dsgb_line_axis0_ws(*args, ws.data_ptr(), wsz, 0, st), "dsgb_line_axis0_ws")
        else:
            N_.check(L.dsgb_line_axis0(*args, 0, st), "dsgb_line_axis0")
        torch.cuda.synchronize()
        got.append([t.cpu().numpy().copy() for t in ex.out_tensors])
    for a, b in zip(*got):
        if a.dtype == np.float32:
            assert_same(a, b, rtol=3e-7, atol=1e-7)
        elif a.dtype.kind == "f":
            assert_same(a, b, rtol=RTOL_SUM, atol=1e-13)
        else:
            assert_same(a, b)
    assert sum(float(np.nansum(a)) for a in got[0]) > 0


def test_line_bresenham_vs_oracle():
    cols = _series(30, 500, seed=3)
    canvas = dict(plot_width=300, plot_height=150)
    agg = ds.summary(c=ds.count(), s=ds.sum("v"), l=ds.last("v"))
    got = to_numpy(ds.Canvas(**canvas).line(frame_from_numpy(cols), "x", "y", agg=agg))
    ref = run_line(cols, {}, agg, canvas, 0)
    assert_same(got["c"], ref["c"])
    assert_same(got["l"], ref["l"])
    assert_same(got["s"], ref["s"], rtol=RTOL_SUM)


# ---------------------------------------------------------------- eq_hist

def test_eq_hist_count_agg_vs_oracle():
    cols, cats = _cfg2_frame(400_000, seed=23)
    agg = ds.Canvas(**CANVAS2).points(frame_from_numpy(cols, cats), "x", "y", ds.count())
    out, levels = ds.tf.eq_hist_agg(agg)
    data, mask = oracle.interpolate_prologue(to_numpy(agg))
    ref, ref_levels = oracle.eq_hist(data, mask)
    assert levels == ref_levels
    assert_same(out.cpu().numpy(), ref)
    img = ds.tf.shade(agg, cmap=["lightblue", "darkblue"], how="eq_hist")
    got = img.data.view(torch.int32).cpu().numpy().view(np.uint32)
    assert_same(got, oracle.shade_eq_hist(to_numpy(agg), ["lightblue", "darkblue"]))


def test_eq_hist_binned_paths_vs_oracle():
    """uint32 data with ptp >= 65536 and float64 data take numpy.histogram's binned path."""
    rng = np.random.default_rng(31)
    u = rng.integers(0, 3_000_000, size=(300, 400)).astype(np.uint32)
    u[rng.random(u.shape) < 0.1] = 0
    f = rng.lognormal(0, 2, size=(300, 400))
    f[rng.random(f.shape) < 0.1] = np.nan
    for data in (u, f):
        t = torch.from_numpy(data.view(np.int32) if data.dtype == np.uint32 else data).cuda()
        if data.dtype == np.uint32:
            t = t.view(torch.uint32)
        out, levels = ds.tf.eq_hist_agg(t)
        d, mask = oracle.interpolate_prologue(data)
        ref, ref_levels = oracle.eq_hist(d, mask)
        assert levels == ref_levels
        # np.interp between bin centres: FMA contraction differs between numpy builds
        assert_same(out.cpu().numpy(), ref, rtol=1e-12, atol=1e-15)


# ----------------------------------------- hot-tile count path (workspace path)

@pytest.mark.parametrize("shape", [(1024, 1024), (512, 256), (1920, 1080), (4096, 2160), (1000, 999),
                                   (3, 5)])
@pytest.mark.parametrize("n", [8191, (1 << 20) + 3, 1_500_000])
def test_cached_count_shapes_vs_oracle(shape, n):
    w, h = shape
    x, y = synthetic.gaussian_mixture_np(n, seed=n + w, dtype=np.float32)
    cols = {"x": x, "y": y}
    canvas = dict(plot_width=w, plot_height=h, x_range=(-4, 4), y_range=(-3, 3))
    got = to_numpy(ds.Canvas(**canvas).points(frame_from_numpy(cols), "x", "y", ds.count()))
    ref = run_points(cols, {}, ds.count(), canvas)
    assert_same(got, ref)


def _count_ws(frame, width, height, x_range, y_range, flags_seq=(0,)):
    import ctypes
    from datashader_gb300 import _native as N
    from datashader_gb300.compiler import compile_plan
    from datashader_gb300.core import Executor
    from datashader_gb300.glyphs import Point
    plan = compile_plan(ds.count(), frame)
    ex = Executor(frame, plan, Point("x", "y"))
    ex.allocate(height, width, frame.device)
    cvs = ds.Canvas(width, height, x_range, y_range)
    sx, tx = cvs.x_axis.compute_scale_and_translate(x_range, width)
    sy, ty = cvs.y_axis.compute_scale_and_translate(y_range, height)
    cv = N.CanvasDesc(width, height, 0, 0, sx, tx, sy, ty, float(x_range[0]), float(x_range[1]),
                      float(y_range[0]), float(y_range[1]))
    L = N.lib()
    wsz = int(L.dsgb_points_workspace_size(len(frame), ctypes.byref(cv), ex.bases, 1))
    assert wsz > 0
    ws = torch.empty(wsz, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    for flags in flags_seq:
        N.check(L.dsgb_points_ws(ex.cols, len(ex.names), len(frame), 0, 0, 1, ctypes.byref(cv), ex.bases, 1,
                                 ex.outs, 0, ws.data_ptr(), wsz, flags, st), "dsgb_points_ws")
    return to_numpy(type("A", (), {"data": ex.out_tensors[0]})())


def test_cached_count_accumulate():
    from datashader_gb300 import _native as N
    x, y = synthetic.gaussian_mixture_np(1_300_001, seed=4, dtype=np.float32)
    cols = {"x": x, "y": y}
    got = _count_ws(frame_from_numpy(cols), 1024, 1024, (-4, 4), (-4, 4), (0, N.FLAG_NO_INIT))
    ref = run_points(cols, {}, ds.count(), CANVAS2)
    assert_same(got, 2 * ref)


def test_cached_count_single_hot_pixel():
    """Nearly every row on two pixels: the cached counters take every row."""
    n = 12_000_000
    x = np.full(n, 0.1, dtype=np.float32)
    y = np.full(n, -0.2, dtype=np.float32)
    x[::7] = 0.7                      # a second hot pixel
    got = _count_ws(frame_from_numpy({"x": x, "y": y}), 1024, 1024, (-4, 4), (-4, 4))
    ref = run_points({"x": x, "y": y}, {}, ds.count(), CANVAS2)
    assert_same(got, ref)
    assert int(got.astype(np.int64).sum()) == n


# ----------------------------------------- hot-tile mean path (workspace path)

@pytest.mark.parametrize("shape", [(1024, 1024), (1000, 999), (4096, 2160), (6, 4)])
def test_cached_mean_vs_oracle(shape):
    """mean('v') through the shared-memory tile cache: float64 sums in another
    order than the reference's row order, 1e-12 relative; NaN values skipped."""
    w, h = shape
    n = 1_400_003
    rng = np.random.default_rng(w)
    x, y = synthetic.gaussian_mixture_np(n, seed=w + 1, dtype=np.float32)
    v = rng.lognormal(0.0, 1.0, n)
    v[rng.random(n) < 0.03] = np.nan
    cols = {"x": x, "y": y, "v": v}
    canvas = dict(plot_width=w, plot_height=h, x_range=(-4, 4), y_range=(-3, 3))
    agg = ds.summary(m=ds.mean("v"), c=ds.count("v"))
    got = to_numpy(ds.Canvas(**canvas).points(frame_from_numpy(cols), "x", "y", ds.mean("v")))
    ref = run_points(cols, {}, ds.mean("v"), canvas)
    assert_same(got, ref, rtol=1e-12)
    both = to_numpy(ds.Canvas(**canvas).points(frame_from_numpy(cols), "x", "y", agg))
    assert_same(both["m"], ref, rtol=1e-12)


def test_cached_mean_single_hot_pixel():
    n = 6_000_000
    x = np.full(n, 0.1, dtype=np.float32)
    y = np.full(n, -0.2, dtype=np.float32)
    x[::5] = 2.5
    v = np.linspace(0.5, 1.5, n)
    cols = {"x": x, "y": y, "v": v}
    got = to_numpy(ds.Canvas(**CANVAS2).points(frame_from_numpy(cols), "x", "y", ds.mean("v")))
    ref = run_points(cols, {}, ds.mean("v"), CANVAS2)
    assert_same(got, ref, rtol=1e-12)


def _edge_coords(lo, hi, npx, rng, m):
    """float32 coordinates that probe every decision of the binning: each
    pixel edge and its float neighbours, the bounds and the floats just
    beyond them, half-pixel bands inside and outside, non-finite and huge
    values; the rest Gaussian."""
    lo32, hi32 = np.float32(lo), np.float32(hi)
    px = (hi - lo) / npx
    edges = (lo + np.arange(npx + 1) * px).astype(np.float32)
    specials = [lo32, hi32, np.nextafter(lo32, np.float32(-np.inf)), np.nextafter(lo32, np.float32(np.inf)),
                np.nextafter(hi32, np.float32(-np.inf)), np.nextafter(hi32, np.float32(np.inf))]
    for f in (-2.0, -1.5, -1.0, -0.75, -0.5, -0.25, 0.25, 0.5, 0.75):
        specials += [np.float32(lo + f * px), np.float32(hi - f * px)]
    specials += [np.nan, np.inf, -np.inf, 1e30, -1e30, 3e38, -3e38, 1e7, -1e7, 0.0, -0.0, 1e-40]
    probe = np.concatenate([edges, np.nextafter(edges, np.float32(np.inf)),
                            np.nextafter(edges, np.float32(-np.inf)), np.asarray(specials, np.float32)])
    out = rng.normal((lo + hi) / 2, (hi - lo) / 5, m).astype(np.float32)
    idx = rng.choice(m, size=min(m // 3, 40 * probe.size), replace=False)
    out[idx] = probe[rng.integers(0, probe.size, idx.size)]
    return out


@pytest.mark.parametrize("w,h,xr,yr", [(1024, 1024, (-4.0, 4.0), (-4.0, 4.0)),
                                       (1000, 999, (-3.3, 2.7), (0.1, 0.7)),
                                       (333, 4096, (1e3, 1e3 + 17.0), (-1e-3, 2e-3))])
def test_cached_paths_adversarial_coordinates(w, h, xr, yr):
    """The cached count / mean kernels classify rows by the float32 image
    alone (no bounds compares): bit-exact counts and 1e-12 means against the
    oracle on coordinates at every pixel edge, at and beyond the bounds, and
    non-finite or huge."""
    n = 1_300_000
    rng = np.random.default_rng(w + h)
    x = _edge_coords(xr[0], xr[1], w, rng, n)
    y = _edge_coords(yr[0], yr[1], h, rng, n)
    v = rng.lognormal(0.0, 1.0, n)
    v[rng.random(n) < 0.02] = np.nan
    canvas = dict(plot_width=w, plot_height=h, x_range=xr, y_range=yr)
    cols = {"x": x, "y": y, "v": v}
    got = to_numpy(ds.Canvas(**canvas).points(frame_from_numpy(cols), "x", "y", ds.count()))
    assert_same(got, run_points(cols, {}, ds.count(), canvas))
    got = to_numpy(ds.Canvas(**canvas).points(frame_from_numpy(cols), "x", "y", ds.mean("v")))
    assert_same(got, run_points(cols, {}, ds.mean("v"), canvas), rtol=1e-12)


def _edge_coords64(lo, hi, npx, rng, m):
    """float64 coordinates for the same decisions: pixel edges and the
    doubles next to them, the bounds and beyond, values below the float32
    normal range (1e-40, 1e-310) and beyond its top (1e39, 1e300), non-finite."""
    px = (hi - lo) / npx
    edges = lo + np.arange(npx + 1) * px
    specials = [lo, hi, np.nextafter(lo, -np.inf), np.nextafter(lo, np.inf), np.nextafter(hi, -np.inf),
                np.nextafter(hi, np.inf)]
    for f in (-2.0, -1.0, -0.5, -1e-9, 1e-9, 0.5, 0.75):
        specials += [lo + f * px, hi - f * px]
    specials += [np.nan, np.inf, -np.inf, 1e39, -1e39, 1e300, -1e300, 0.0, -0.0, 1e-40, -1e-40, 1e-310, 5e-324]
    probe = np.concatenate([edges, np.nextafter(edges, np.inf), np.nextafter(edges, -np.inf),
                            edges + 1e-8 * px, edges - 1e-8 * px, np.asarray(specials, np.float64)])
    out = rng.normal((lo + hi) / 2, (hi - lo) / 5, m)
    idx = rng.choice(m, size=min(m // 3, 40 * probe.size), replace=False)
    out[idx] = probe[rng.integers(0, probe.size, idx.size)]
    return out


@pytest.mark.parametrize("w,h,xr,yr", [(512, 512, (-4.0, 4.0), (-4.0, 4.0)),
                                       (1024, 768, (-1e-3, 2e-3), (-3.3, 2.7))])
def test_hot_count_float64_adversarial_coordinates(w, h, xr, yr):
    """float64 coordinates through the hot-tile count kernel (float32 images
    by truncation, proven by the error bound): bit-exact against the oracle."""
    n = 1_500_000
    rng = np.random.default_rng(w * 7 + h)
    cols = {"x": _edge_coords64(xr[0], xr[1], w, rng, n), "y": _edge_coords64(yr[0], yr[1], h, rng, n)}
    canvas = dict(plot_width=w, plot_height=h, x_range=xr, y_range=yr)
    got = to_numpy(ds.Canvas(**canvas).points(frame_from_numpy(cols), "x", "y", ds.count()))
    assert_same(got, run_points(cols, {}, ds.count(), canvas))
