"""Batched tile pyramid against one Canvas.points call per tile.

Each tile of the pyramid must equal the plain Canvas.points(count, max('v'))
of that tile's ranges (the plain GPU path, itself pinned to the oracle by the
parity tests; a few tiles are also compared with the oracle directly).  The
data holds the cases that separate a pyramid from a mipmap: points exactly on
tile edges at every level (counted in both tiles), on the outer edges of the
square, corners, NaN coordinates and values, and points outside the square.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
import oracle
from datashader_gb300 import pyramid as P
from datashader_gb300 import synthetic
from gpu_helpers import assert_same, to_numpy

pytestmark = pytest.mark.gpu


def _data(n, seed, x_range=(0.0, 1.0), y_range=(0.0, 1.0), zmax=6):
    rng = np.random.default_rng(seed)
    x, y = synthetic.pyramid_points_np(n, seed=seed)
    (x0, x1), (y0, y1) = x_range, y_range
    x = (x0 + (x1 - x0) * x.astype(np.float64)).astype(np.float32)
    y = (y0 + (y1 - y0) * y.astype(np.float64)).astype(np.float32)
    v = rng.standard_normal(n).astype(np.float32)
    extra_x, extra_y = [], []
    for z in range(zmax + 1):
        for _ in range(40):
            tx, ty = rng.integers(0, (1 << z) + 1, 2)
            ex = np.float32(P.tile_range(z, int(tx), x0, x1)[0])     # on a vertical edge
            ey = np.float32(P.tile_range(z, int(ty), y0, y1)[0])
            extra_x += [ex, ex, np.float32(x0 + (x1 - x0) * rng.random())]
            extra_y += [ey, np.float32(y0 + (y1 - y0) * rng.random()), ey]
    extra_x += [np.float32(x0), np.float32(x1), np.float32(x1), np.nan, np.float32(x1 + 0.25), np.float32(x0 - 1.0)]
    extra_y += [np.float32(y0), np.float32(y1), np.float32(y0), np.float32(y0), np.float32(y0), np.float32(y1)]
    ex = np.array(extra_x, dtype=np.float32)
    ey = np.array(extra_y, dtype=np.float32)
    ev = rng.standard_normal(ex.size).astype(np.float32)
    ev[::7] = np.nan
    # values whose float64 widening takes every branch: subnormals, infinities, extremes
    special = np.array([1e-40, -1e-42, 1.4e-45, -1.4e-45, np.inf, -np.inf, 3.4e38, -3.4e38, 1.17549435e-38,
                        -0.0, 0.0], dtype=np.float32)
    ev[3::11][:special.size] = special[:ev[3::11].size]
    x = np.concatenate([x, ex, ex])      # edge points twice: counts of 2 on edges
    y = np.concatenate([y, ey, ey])
    v = np.concatenate([v, ev, ev[::-1]])
    perm = rng.permutation(x.size)
    return x[perm], y[perm], v[perm]


def _plain_tile(frame, pyr, z, tx, ty):
    xr, yr = pyr.tile_ranges(z, tx, ty)
    agg = ds.Canvas(plot_width=pyr.ts, plot_height=pyr.ts, x_range=xr, y_range=yr).points(
        frame, "x", "y", ds.summary(count=ds.count(), max=ds.max("v")))
    return to_numpy(agg["count"]), to_numpy(agg["max"])


def _check_tiles(pyr, frame, tiles):
    for z, tx, ty in tiles:
        c, m = pyr.tile(z, tx, ty)
        c = c.view(torch.int32).cpu().numpy().view(np.uint32)
        m = m.cpu().numpy()
        rc, rm = _plain_tile(frame, pyr, z, tx, ty)
        assert_same(c, rc, what=f"count tile {(z, tx, ty)}")
        assert_same(m, rm, what=f"max tile {(z, tx, ty)}")


def _all_tiles(zmin, zmax):
    return [(z, tx, ty) for z in range(zmin, zmax + 1) for ty in range(1 << z) for tx in range(1 << z)]


@pytest.mark.parametrize("config", [dict(split=0, threads=1024, chunk=65536),
                                    dict(split=1, threads=512, chunk=4096),
                                    dict(split=0, threads=256, chunk=2048)])
def test_pyramid_matches_per_tile_calls(config):
    x, y, v = _data(120_000, seed=1, zmax=4)
    X, Y, V = (torch.from_numpy(a).cuda() for a in (x, y, v))
    frame = ds.TensorFrame({"x": X, "y": Y, "v": V})
    pyr = P.TilePyramid(X, Y, V, zmin=0, zmax=4, config=config, graph=False).render().check()
    _check_tiles(pyr, frame, _all_tiles(0, 4))


def test_pyramid_deep_levels_and_graph_replay():
    x, y, v = _data(300_000, seed=2, zmax=6)
    X, Y, V = (torch.from_numpy(a).cuda() for a in (x, y, v))
    frame = ds.TensorFrame({"x": X, "y": Y, "v": V})
    pyr = P.TilePyramid(X, Y, V, zmin=0, zmax=6, config=dict(split=1, threads=1024, chunk=8192))
    pyr.render().check()
    first_c, first_m = pyr.counts.clone(), pyr.max.clone()
    pyr.counts.fill_(7)
    pyr.render().check()                                   # graph replay overwrites every cell
    assert torch.equal(pyr.counts.view(torch.int32), first_c.view(torch.int32))
    assert torch.equal(torch.nan_to_num(pyr.max, nan=-1e300), torch.nan_to_num(first_m, nan=-1e300))
    rng = np.random.default_rng(5)
    tiles = _all_tiles(0, 2)
    for z in (3, 4, 5, 6):
        for _ in range(6):
            tx, ty = (int(t) for t in rng.integers(0, 1 << z, 2))
            tiles.append((z, tx, ty))
    _check_tiles(pyr, frame, tiles)
    total = int(pyr.counts[: 256 * 256].view(torch.int32).sum())
    inside = (x >= 0) & (x <= 1) & (y >= 0) & (y <= 1)
    assert total == int(inside.sum())                      # level 0 is the whole square


def test_pyramid_general_square_and_oracle():
    """A square whose tile bounds are not dyadic: every bin goes through the
    float64 formula of each tile, and a few tiles are checked with the oracle."""
    xr, yr = (-0.3, 0.7123), (0.1, 0.9000001)
    x, y, v = _data(60_000, seed=3, x_range=xr, y_range=yr, zmax=3)
    X, Y, V = (torch.from_numpy(a).cuda() for a in (x, y, v))
    frame = ds.TensorFrame({"x": X, "y": Y, "v": V})
    pyr = P.TilePyramid(X, Y, V, zmin=1, zmax=3, x_range=xr, y_range=yr,
                        config=dict(split=0, threads=512, chunk=4096), graph=False).render().check()
    _check_tiles(pyr, frame, _all_tiles(1, 3))
    for z, tx, ty in ((1, 0, 1), (3, 5, 2), (2, 3, 3)):
        c, m = pyr.tile(z, tx, ty)
        txr, tyr = pyr.tile_ranges(z, tx, ty)
        rc, rm = oracle.points({"x": x.astype(np.float64), "y": y.astype(np.float64), "v": v.astype(np.float64)},
                               "x", "y", pyr.ts, pyr.ts, txr, tyr,
                               [oracle.spec("count"), oracle.spec("max", "v")])
        assert_same(c.view(torch.int32).cpu().numpy().view(np.uint32), rc, what="oracle count")
        assert_same(m.cpu().numpy(), rm, what="oracle max")


def test_pyramid_count_only_and_autotune():
    x, y, _ = _data(50_000, seed=4, zmax=3)
    X, Y = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    frame = ds.TensorFrame({"x": X, "y": Y, "v": torch.zeros_like(X)})
    pyr = P.TilePyramid(X, Y, None, zmin=0, zmax=3, graph=False)
    best, results = P.autotune(pyr, candidates=P.CANDIDATES[:4], repeats=1)
    assert pyr.config == best and len(results) >= 1
    pyr.render().check()
    for z, tx, ty in _all_tiles(0, 3):
        c, m = pyr.tile(z, tx, ty)
        assert m is None
        rc, _ = _plain_tile(frame, pyr, z, tx, ty)
        assert_same(c.view(torch.int32).cpu().numpy().view(np.uint32), rc, what=f"count {(z, tx, ty)}")


def test_pyramid_overflow_status_raises():
    """With the edge queue and slot capacities shrunk to nothing, a render
    that needs them reports an incomplete pyramid: check() raises, and the
    full capacity renders the same data completely."""
    x, y, v = _data(300_000, seed=21)
    # a dense cluster so that buckets split into chunks (partial slots)
    x = np.concatenate([x, np.full(200_000, 0.3001, np.float32)])
    y = np.concatenate([y, np.full(200_000, 0.7003, np.float32)])
    v = np.concatenate([v, np.ones(200_000, np.float32)])
    X, Y, V = (torch.from_numpy(a).cuda() for a in (x, y, v))
    cfg = dict(split=0, threads=512, chunk=16384)
    bad = P.TilePyramid(X, Y, V, zmax=4, tile_size=64, config=cfg, graph=False, capacity_shift=31).render()
    with pytest.raises(ds._native.DsgbError, match="incomplete render"):
        bad.check()
    assert bad.status() & 0x5          # queue overflow and / or slots exhausted
    good = P.TilePyramid(X, Y, V, zmax=4, tile_size=64, config=cfg, graph=False).render()
    good.check()
    with pytest.raises(ValueError):
        P.TilePyramid(X, Y, V, zmax=4, tile_size=64, capacity_shift=32)
