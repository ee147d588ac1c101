"""Host-resident frames streamed to the GPU in chunks (HostFrame).

The same Canvas.points over a HostFrame (pinned host columns, several
chunks, a ragged last chunk, copies overlapping the aggregation) and over a
device TensorFrame of the same rows: integer and row-index results
bit-exact, float64 sums and means 1e-12 relative (atomics in another
order), first / last / where gathered from the host column by global row.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
import oracle
from datashader_gb300 import synthetic
from gpu_helpers import assert_same, to_numpy

pytestmark = pytest.mark.gpu


def _cols(n, seed):
    rng = np.random.default_rng(seed)
    x, y = synthetic.gaussian_mixture_np(n, seed=seed, dtype=np.float32)
    v = rng.lognormal(0.0, 1.0, n)
    v[rng.random(n) < 0.03] = np.nan
    cat = rng.integers(0, 6, n).astype(np.int8)
    return {"x": x, "y": y, "v": v, "cat": cat}


AGG = ds.summary(c=ds.count(), s=ds.sum("v"), m=ds.mean("v"), mx=ds.max("v"), mn=ds.min("v"),
                 f=ds.first("v"), l=ds.last("v"), w=ds.where(ds.max("v")), b=ds.by("cat", ds.count()))
TOL = {"s": 1e-12, "m": 1e-12}


@pytest.mark.parametrize("n,chunk,offset", [(1_000_003, 100_000, 0), (1_300_000, 1 << 20, 77), (5000, 1 << 24, 3)])
def test_host_frame_equals_device_frame(n, chunk, offset):
    cols = _cols(n, seed=n % 97)
    cats = {"cat": list(range(6))}
    dev = ds.TensorFrame({k: torch.from_numpy(v).cuda() for k, v in cols.items()}, categories=cats,
                         row_offset=offset)
    host = ds.HostFrame(cols, categories=cats, chunk_rows=chunk, row_offset=offset)
    assert all(host[k].is_pinned() for k in cols)
    for cvs in (ds.Canvas(plot_width=512, plot_height=384, x_range=(-4, 4), y_range=(-3, 3)),
                ds.Canvas(plot_width=300, plot_height=200)):                   # autorange: a bounds pass
        want = to_numpy(cvs.points(dev, "x", "y", AGG))
        got = to_numpy(cvs.points(host, "x", "y", AGG))
        for k in want:
            assert_same(got[k], want[k], rtol=TOL.get(k, 0.0), what=k)
    # count alone takes the hot-tile path in every large chunk: against the oracle
    cvs = ds.Canvas(plot_width=1024, plot_height=1024, x_range=(-4, 4), y_range=(-4, 4))
    ref = oracle.points({k: np.asarray(v, dtype=np.float64) for k, v in cols.items()}, "x", "y", 1024, 1024,
                        (-4, 4), (-4, 4), [oracle.spec("count")])[0]
    assert_same(to_numpy(cvs.points(host, "x", "y", ds.count())), ref)


def test_host_frame_edges():
    empty = ds.HostFrame({"x": np.zeros(0, np.float32), "y": np.zeros(0, np.float32)})
    out = to_numpy(ds.Canvas(plot_width=16, plot_height=8, x_range=(0, 1), y_range=(0, 1)).points(empty, "x", "y"))
    assert out.shape == (8, 16) and not out.any()
    h = ds.HostFrame({"x": np.float32([0.5]), "y": np.float32([0.5])}, chunk_rows=1)
    with pytest.raises(NotImplementedError):
        ds.Canvas(plot_width=8, plot_height=8, x_range=(0, 1), y_range=(0, 1)).points(h, "x", "y", deterministic=True)
    with pytest.raises(ValueError):
        ds.HostFrame({"x": np.float32([0.5])}, chunk_rows=0)


@pytest.mark.parametrize("lw", [0.0, 1.5])
def test_host_frame_lines_equal_device_frame(lw):
    """Canvas.line over a HostFrame: the frame is copied to the GPU once (a line
    reads its neighbours across any chunk edge), then the device path; equal to
    the same columns given as a device frame, for LineAxis0 and a multi-line glyph."""
    from datashader_gb300 import synthetic as S
    x, y, v, _ = S.time_series_np(6, 400, seed=9)
    cols = {"x": x, "y": y, "v": v}
    host = ds.HostFrame(cols, chunk_rows=100)
    dev = ds.TensorFrame({k: torch.from_numpy(a).cuda() for k, a in cols.items()})
    cvs = ds.Canvas(plot_width=90, plot_height=60)
    agg = ds.summary(c=ds.count(), s=ds.sum("v"), m=ds.max("v"))
    got = cvs.line(host, "x", "y", agg=agg, line_width=lw)
    ref = cvs.line(dev, "x", "y", agg=agg, line_width=lw)
    for k in ("c", "s", "m"):
        assert_same(to_numpy(got[k]), to_numpy(ref[k]), rtol=1e-12 if k == "s" else 0.0, what=k)
    rng = np.random.default_rng(3)
    mcols = {f"y{j}": np.cumsum(rng.normal(0, 0.1, 200)) for j in range(4)}
    mcols["x"] = np.linspace(0, 1, 200)
    hm = ds.HostFrame(mcols)
    dm = ds.TensorFrame({k: torch.from_numpy(a).cuda() for k, a in mcols.items()})
    kw = dict(x="x", y=[f"y{j}" for j in range(4)], axis=0, agg=ds.count(), line_width=lw)
    assert_same(to_numpy(cvs.line(hm, **kw)), to_numpy(cvs.line(dm, **kw)))
