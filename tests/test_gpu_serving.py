"""Viewport serving: each request's result in the concurrent mix equals the
same request computed alone with a plain whole-frame Canvas.points call.

Tolerances: count, max(v) and by(cat, count) bit-exact; mean(v) 1e-12
relative (float64 atomic sums in a different order: the bucketed store
reorders the rows).
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
from datashader_gb300 import serving as S
from datashader_gb300 import synthetic
from gpu_helpers import assert_same, to_numpy

pytestmark = pytest.mark.gpu


def _frame(n=1_000_000, seed=0):
    rng = np.random.default_rng(seed)
    x, y = synthetic.pyramid_points_np(n, seed=seed)
    v = rng.standard_normal(n).astype(np.float32)
    v[::97] = np.nan
    cat = rng.integers(0, 16, n).astype(np.uint8)
    # points on bucket and viewport edges, outside the domain, NaN coordinates
    edge = np.float32(np.arange(0, 65) / 64.0)
    ex = np.concatenate([edge, edge, np.full(4, 0.5, np.float32), [np.nan, 1.5, -0.25]]).astype(np.float32)
    ey = np.concatenate([edge[::-1], np.full(65, 0.25, np.float32), np.float32([0.0, 1.0, 0.5, 0.25]),
                         [0.3, 0.3, 0.3]]).astype(np.float32)
    x = np.concatenate([x, ex]).astype(np.float32)
    y = np.concatenate([y, ey]).astype(np.float32)
    v = np.concatenate([v, rng.standard_normal(ex.size).astype(np.float32)])
    cat = np.concatenate([cat, rng.integers(0, 16, ex.size).astype(np.uint8)])
    t = {"x": torch.from_numpy(x).cuda(), "y": torch.from_numpy(y).cuda(), "v": torch.from_numpy(v).cuda(),
         "cat": torch.from_numpy(cat).cuda()}
    return ds.TensorFrame(t, categories={"cat": list(range(16))})


def _requests():
    reqs = S.generate_requests(40, rate=1e7, seed=7)
    extra = [((0.0, 1.0), (0.0, 1.0)), ((0.25, 0.5), (0.25, 0.5)), ((-0.5, 2.0), (0.2, 0.4)),
             ((0.5, 0.515625), (0.234375, 0.25))]
    for i, (xr, yr) in enumerate(extra):
        for k, kind in enumerate(S.REDUCTIONS):
            reqs.append(S.Request(1000 + 4 * i + k, 0.0, xr, yr, (333, 512)[k % 2], (200, 512)[k % 2], kind))
    return reqs


def _alone(frame, req):
    agg = S.make_agg(req.kind)
    return ds.Canvas(req.width, req.height, req.x_range, req.y_range).points(frame, "x", "y", agg)


def _compare(got, ref, kind, what):
    g, r = to_numpy(got), to_numpy(ref)
    if kind == "mean":
        assert_same(g, r, rtol=1e-12, what=what)
    else:
        assert_same(g, r, what=what)


def test_results_in_the_mix_equal_alone():
    frame = _frame()
    store = S.BucketedStore(frame, grid=64, domain=(0.0, 1.0, 0.0, 1.0))
    ex = S.SegmentExecutor(store)
    reqs = _requests()
    server = S.ViewportServer(ex, slots=4, mem_budget=64 << 20)
    server.run(reqs, keep_results=True)
    torch.cuda.synchronize()
    assert server.peak_inflight > 1                      # the requests did overlap
    assert server.peak_mem_shared <= 64 << 20           # only a request larger than the budget runs alone
    for r in reqs:
        _compare(r.result, _alone(frame, r), r.kind, f"request {r.rid} ({r.kind})")
    # and run one at a time through the same store: identical to the mix
    seq = [S.Request(r.rid, 0.0, r.x_range, r.y_range, r.width, r.height, r.kind) for r in reqs[:12]]
    S.ViewportServer(ex, slots=4).run(seq, mode="sequential", keep_results=True)
    for a, b in zip(seq, reqs[:12]):
        _compare(a.result, b.result, a.kind, f"sequential {a.rid}")


def test_store_keeps_every_row_and_bucket_order():
    frame = _frame(200_000, seed=1)
    store = S.BucketedStore(frame, grid=32, domain=(0.0, 1.0, 0.0, 1.0))
    st = store.starts
    assert st[0] == 0 and st[-1] == len(frame) and np.all(np.diff(st) >= 0)
    xs = store.frame["x"].cpu().numpy()
    ys = store.frame["y"].cpu().numpy()
    # the multiset of rows is unchanged
    a = np.sort(np.stack([frame["x"].cpu().numpy(), frame["y"].cpu().numpy()], 1).view(np.complex64).ravel())
    b = np.sort(np.stack([xs, ys], 1).view(np.complex64).ravel())
    assert np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])
    for bk in (0, 5, 17 * 32 + 3, 32 * 32 - 1):
        seg = slice(st[bk], st[bk + 1])
        bx, by = bk % 32, bk // 32
        assert np.all(np.floor(xs[seg].astype(np.float64) * 32).clip(0, 31) == bx)
        assert np.all(np.floor(ys[seg].astype(np.float64) * 32).clip(0, 31) == by)
    out = slice(st[32 * 32], st[32 * 32 + 1])
    assert st[32 * 32 + 1] - st[32 * 32] == 3                     # NaN, 1.5 and -0.25
    assert np.all(~((xs[out] >= 0) & (xs[out] <= 1) & (ys[out] >= 0) & (ys[out] <= 1)))
