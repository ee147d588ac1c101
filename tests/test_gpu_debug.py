"""Debug mode: checked appends and the device status word.

``ds.debug_checks()`` runs Canvas.points / Canvas.line with
DSGB_FLAG_DEBUG_CHECKS (every append's aggregate index checked on the
device) and raises when a kernel reports a status bit.  Results on valid
input equal the unchecked path; an invalid category code is reported
instead of being skipped silently.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
from datashader_gb300 import _native as N
from datashader_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _frame(n=200_000, seed=3, bad_code=None):
    x, y = synthetic.gaussian_mixture_np(n, seed=seed, dtype=np.float32)
    rng = np.random.default_rng(seed)
    v = rng.lognormal(0, 1, n)
    cat = rng.integers(0, 4, n).astype(np.int8)
    if bad_code is not None:
        cat[::1000] = bad_code
    return ds.TensorFrame({"x": x, "y": y, "v": v, "cat": cat}, categories={"cat": list("abcd")})


def test_debug_checks_equal_results_and_clean_status():
    f = _frame()
    cvs = ds.Canvas(plot_width=300, plot_height=200, x_range=(-4, 4), y_range=(-4, 4))
    red = ds.summary(c=ds.count(), s=ds.sum("v"), m=ds.max("v"), w=ds.where(ds.max("v")),
                     b=ds.by("cat", ds.count()))
    plain = cvs.points(f, "x", "y", red)
    assert N.device_status() == 0
    with ds.debug_checks():
        checked = cvs.points(f, "x", "y", red)
        line = cvs.line(f, "x", "y", agg=ds.sum("v"), line_width=1.5)
    for k in ("c", "m", "w", "b"):                  # NaN-aware equality
        np.testing.assert_array_equal(plain[k].data.cpu().numpy(), checked[k].data.cpu().numpy(), err_msg=k)
    torch.testing.assert_close(plain["s"].data, checked["s"].data, rtol=1e-12, atol=0, equal_nan=True)
    assert torch.isfinite(torch.nan_to_num(line.data)).all()
    ds.check_device_status()


def test_debug_checks_report_an_invalid_category_code():
    f = _frame(bad_code=7)            # 4 categories: code 7 has no cell
    cvs = ds.Canvas(plot_width=64, plot_height=64, x_range=(-4, 4), y_range=(-4, 4))
    agg = cvs.points(f, "x", "y", ds.by("cat", ds.count()))     # unchecked: the row is skipped
    assert int(agg.data.sum()) < len(f)
    assert N.device_status() == 0
    with ds.debug_checks():
        with pytest.raises(N.DsgbError, match="outside its aggregate"):
            cvs.points(f, "x", "y", ds.by("cat", ds.count()))
    assert N.device_status() == 0     # the check cleared the word
