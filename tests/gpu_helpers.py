"""Helpers shared by the GPU tests."""
from __future__ import annotations

import numpy as np
import torch

import datashader_gb300 as ds


def frame_from_numpy(cols, categories=None, row_offset=0):
    t = {}
    for k, v in cols.items():
        a = np.ascontiguousarray(v)
        if a.dtype == np.uint32:
            t[k] = torch.from_numpy(a.view(np.int32)).cuda().view(torch.uint32)
        else:
            t[k] = torch.from_numpy(a).cuda()
    return ds.TensorFrame(t, categories=categories or {}, row_offset=row_offset)


def to_numpy(agg):
    if isinstance(agg, dict):
        return {k: to_numpy(v) for k, v in agg.items()}
    d = agg.data
    if d.dtype == torch.uint32:
        return d.view(torch.int32).cpu().numpy().view(np.uint32)
    return d.cpu().numpy()


def assert_same(got, ref, rtol=0.0, atol=0.0, what=""):
    """Bit-exact (rtol=atol=0, NaNs in the same places) or within tolerance."""
    if isinstance(ref, dict):
        assert sorted(got) == sorted(ref)
        for k in ref:
            assert_same(got[k], ref[k], rtol, atol, what=f"{what}[{k}]")
        return
    got = np.asarray(got)
    ref = np.asarray(ref)
    assert got.shape == ref.shape, f"{what}: shape {got.shape} != {ref.shape}"
    if rtol == 0 and atol == 0:
        np.testing.assert_array_equal(got, ref, err_msg=what)
    else:
        np.testing.assert_allclose(got, ref, rtol=rtol, atol=atol, equal_nan=True, err_msg=what)
