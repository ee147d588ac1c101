"""The allocation-free eq_hist entry point (dsgb_eq_hist_u32_static).

Callers that may not allocate device memory when they shade (a latency-bound
host thread, a stream callback, a plugin whose host owns every allocation)
use the variant whose scratch is a static device array inside libdsgb.  It
must give the same image as the workspace entry point, call after call.

This file is named so that pytest collects it last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from datashader_gb300 import _native as N

pytestmark = pytest.mark.gpu

CMAP = (ctypes.c_double * 6)(0xAD, 0xD8, 0xE6, 0x00, 0x00, 0x8B)   # lightblue -> darkblue


def _aggregate(seed, shape=(700, 900)):
    rng = np.random.default_rng(seed)
    a = rng.poisson(rng.gamma(0.6, 40.0, size=shape)).astype(np.uint32)   # many zeros (masked), skewed
    return torch.from_numpy(a.view(np.int32)).cuda().view(torch.uint32)


def _run(fn, data, nbins, use_ws):
    dev = data.device
    out = torch.empty(data.shape, dtype=torch.float64, device=dev)
    levels = torch.zeros(1, dtype=torch.int64, device=dev)
    rgba = torch.empty(data.shape, dtype=torch.uint32, device=dev)
    st = torch.cuda.current_stream().cuda_stream
    if use_ws:
        size = int(N.lib().dsgb_eq_hist_workspace_size(nbins))
        ws = torch.empty(size, dtype=torch.uint8, device=dev)
        rc = fn(data.data_ptr(), data.numel(), nbins, out.data_ptr(), levels.data_ptr(), rgba.data_ptr(),
                CMAP, 2, 255, 0, ws.data_ptr(), size, st)
    else:
        rc = fn(data.data_ptr(), data.numel(), nbins, out.data_ptr(), levels.data_ptr(), rgba.data_ptr(),
                CMAP, 2, 255, 0, st)
    N.check(rc, "eq_hist")
    torch.cuda.synchronize()
    return (out.cpu().numpy(), int(levels.item()), rgba.view(torch.int32).cpu().numpy().view(np.uint32))


def test_static_matches_workspace_entry_point_on_consecutive_calls():
    L = N.lib()
    for seed in (1, 2):          # two calls in a row reuse the same static scratch
        data = _aggregate(seed)
        ref = _run(L.dsgb_eq_hist_u32, data, 65536, True)
        got = _run(L.dsgb_eq_hist_u32_static, data, 65536, False)
        np.testing.assert_array_equal(got[0], ref[0])     # bit-exact, NaN where masked
        assert got[1] == ref[1]
        np.testing.assert_array_equal(got[2], ref[2])


def test_static_rejects_more_bins_than_its_scratch():
    L = N.lib()
    data = _aggregate(3, (8, 8))
    out = torch.empty(data.shape, dtype=torch.float64, device="cuda")
    levels = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = L.dsgb_eq_hist_u32_static(data.data_ptr(), data.numel(), 65537, out.data_ptr(), levels.data_ptr(),
                                   None, None, 0, 255, 0, torch.cuda.current_stream().cuda_stream)
    assert rc == -1
    assert b"static scratch" in L.dsgb_last_error()
