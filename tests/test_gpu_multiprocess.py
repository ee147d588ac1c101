"""Row shards aggregated by two processes and combined by the library.

Each of two gloo ranks (both on cuda:0) runs ``points_partial`` on its row
shard (row_offset = its first global row), ships the partial's host arrays
to rank 0 over gloo, and rank 0 folds them with ``combine_partials``
(dsgb_combine, then dsgb_finalize and dsgb_select_by_owner for the gather
outputs) -- datashader's dask combine (dask.py:168-217, compiler.py:478-507,
where's paired combine reductions.py:1992-2018) across processes.  The
result must equal Canvas.points over all rows in one frame: exact for
count / max / min / first / last / where / by, 1e-12 for sums and means.
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

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N = 1_500_000


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _data():
    from datashader_gb300 import synthetic
    x, y = synthetic.gaussian_mixture_np(N, seed=12, dtype=np.float32)
    rng = np.random.default_rng(12)
    v = rng.lognormal(0.0, 1.0, N)
    v[rng.random(N) < 0.02] = np.nan
    v[: N // 2: 997] = 50.0                   # ties of the maximum across both shards
    v[N // 2 + 13:: 997] = 50.0
    cat = rng.integers(0, 5, N).astype(np.int8)
    return {"x": x, "y": y, "v": v, "cat": cat, "index": np.arange(N, dtype=np.int64) * 3}


def _agg():
    import datashader_gb300 as ds
    return ds.summary(count=ds.count(), sum=ds.sum("v"), mean=ds.mean("v"), max=ds.max("v"), min=ds.min("v"),
                      first=ds.first("v"), last=ds.last("v"), where_row=ds.where(ds.max("v")),
                      where_index=ds.where(ds.max("v"), "index"), where_min=ds.where(ds.min("v"), "index"),
                      by_cat=ds.by("cat", ds.count()))


def _canvas():
    import datashader_gb300 as ds
    return ds.Canvas(plot_width=300, plot_height=200, x_range=(-4, 4), y_range=(-3.5, 3.5))


def _frame(cols, lo, hi):
    import datashader_gb300 as ds
    return ds.TensorFrame({k: torch.from_numpy(v[lo:hi]).cuda() for k, v in cols.items()},
                          categories={"cat": list(range(5))}, row_offset=lo)


def _worker(rank, world, port, out_path):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from datashader_gb300.partials import points_partial, combine_partials
        torch.cuda.set_device(0)
        cols = _data()
        lo, hi = rank * N // world, (rank + 1) * N // world
        part = points_partial(_canvas(), _frame(cols, lo, hi), "x", "y", _agg()).to_host()
        gathered = [None] * world
        dist.all_gather_object(gathered, part)
        if rank == 0:
            from gpu_helpers import to_numpy
            got = to_numpy(combine_partials(gathered, _canvas()))
            ref = to_numpy(_canvas().points(_frame(cols, 0, N), "x", "y", _agg()))
            np.savez(out_path, **{f"got_{k}": v for k, v in got.items()}, **{f"ref_{k}": v for k, v in ref.items()})
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _compare(got, ref):
    assert sorted(got) == sorted(ref)
    for k in ref:
        if k in ("sum", "mean"):
            np.testing.assert_allclose(got[k], ref[k], rtol=1e-12, atol=0, equal_nan=True, err_msg=k)
        else:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


def test_two_process_shards_combine_like_one_frame(tmp_path):
    out = str(tmp_path / "combined.npz")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    res = np.load(out)
    got = {k[4:]: res[k] for k in res.files if k.startswith("got_")}
    ref = {k[4:]: res[k] for k in res.files if k.startswith("ref_")}
    _compare(got, ref)
    w = got["where_row"]
    assert (w >= N // 2).any() and ((w >= 0) & (w < N // 2)).any()      # winners from both shards


def test_partial_host_round_trip_single_process():
    """One process, three shards: the same fold without a transport."""
    from datashader_gb300.partials import points_partial, combine_partials
    from gpu_helpers import to_numpy
    cols = _data()
    cuts = [0, N // 3, 2 * N // 3, N]
    parts = [points_partial(_canvas(), _frame(cols, a, b), "x", "y", _agg()).to_host()
             for a, b in zip(cuts[:-1], cuts[1:])]
    got = to_numpy(combine_partials(parts[::-1], _canvas()))       # any order: folded by first row
    ref = to_numpy(_canvas().points(_frame(cols, 0, N), "x", "y", _agg()))
    _compare(got, ref)
