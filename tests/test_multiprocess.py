"""Row-sharded aggregation across processes (world size 2, gloo, CPU).

The path shards by rows: each rank aggregates its rows (row_offset = the
rank's first row) and one exchange combines the partials, as datashader's
dask path combines partitions (dask.py:86-219, nansum_missing / nanmax /
nanmin combines).  Here each rank runs the oracle on its shard and the
partials meet in gloo all-reduces; rank 0 checks them against the oracle on
all rows.  The bench's cross-rank helpers (barrier, max over ranks) run on
the same process group.
"""
from __future__ import annotations

import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _data(n=200_000, seed=5):
    rng = np.random.default_rng(seed)
    from datashader_gb300 import synthetic
    x, y = synthetic.gaussian_mixture_np(n, seed=seed)
    v = rng.lognormal(0.0, 1.0, n)
    v[rng.random(n) < 0.05] = np.nan
    return {"x": x, "y": y, "v": v}


SPECS = ("count", "count_v", "sum", "max", "min", "first_row")


def _aggregate(cols, lo, hi):
    import oracle
    part = {k: v[lo:hi] for k, v in cols.items()}
    specs = [oracle.spec("count"), oracle.spec("count", "v"), oracle.spec("sum", "v"),
             oracle.spec("max", "v"), oracle.spec("min", "v"), oracle.spec("min_row", "v")]
    return oracle.points(part, "x", "y", 64, 48, (-4, 4), (-3, 3), specs, row_offset=lo)


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        bench._barrier(world)
        top = bench._max_over_ranks(world, float(10 * (rank + 1)))
        cols = _data()
        n = len(cols["x"])
        lo, hi = rank * n // world, (rank + 1) * n // world
        cnt, cnt_v, s, mx, mn, first = _aggregate(cols, lo, hi)
        # combines: counts add; sums add where present (NaN means no value);
        # max / min ignore NaN; the first row is the smallest (-1 means none)
        t_cnt = torch.from_numpy(cnt.astype(np.int64))
        t_cv = torch.from_numpy(cnt_v.astype(np.int64))
        t_s = torch.from_numpy(np.nan_to_num(s, nan=0.0))
        t_mx = torch.from_numpy(np.where(np.isnan(mx), -np.inf, mx))
        t_mn = torch.from_numpy(np.where(np.isnan(mn), np.inf, mn))
        t_first = torch.from_numpy(np.where(first < 0, np.iinfo(np.int64).max, first).astype(np.int64))
        for t in (t_cnt, t_cv, t_s):
            dist.all_reduce(t, op=dist.ReduceOp.SUM)
        dist.all_reduce(t_mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(t_mn, op=dist.ReduceOp.MIN)
        dist.all_reduce(t_first, op=dist.ReduceOp.MIN)
        if rank == 0:
            cv = t_cv.numpy()
            comb = (t_cnt.numpy(), np.where(cv > 0, t_s.numpy(), np.nan),
                    np.where(np.isinf(t_mx.numpy()), np.nan, t_mx.numpy()),
                    np.where(np.isinf(t_mn.numpy()), np.nan, t_mn.numpy()),
                    np.where(t_first.numpy() == np.iinfo(np.int64).max, -1, t_first.numpy()))
            np.savez(out, top=top, cnt=comb[0], s=comb[1], mx=comb[2], mn=comb[3], first=comb[4])
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_row_shards_combine_over_gloo(tmp_path):
    sys.path.insert(0, ROOT)
    out = str(tmp_path / "comb.npz")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    r = np.load(out)
    assert float(r["top"]) == 20.0
    cols = _data()
    cnt, cnt_v, s, mx, mn, first = _aggregate(cols, 0, len(cols["x"]))
    np.testing.assert_array_equal(r["cnt"], cnt)
    np.testing.assert_allclose(r["s"], s, rtol=1e-12, equal_nan=True)   # another addition order
    np.testing.assert_array_equal(r["mx"], mx)
    np.testing.assert_array_equal(r["mn"], mn)
    np.testing.assert_array_equal(r["first"], first)
