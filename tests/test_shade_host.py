"""Host-side validation of tf.shade (no GPU): colour errors are raised before any
device work, as the reference raises them (test_transfer_functions.py:295-300)."""
from __future__ import annotations

import pytest
import torch

import datashader_gb300 as ds


def _agg():
    return ds.Aggregate(torch.zeros((3, 3), dtype=torch.float64), ["y", "x"], {}, {})


@pytest.mark.parametrize("how", ["eq_hist", "linear", "log", "cbrt"])
def test_shade_cmap_errors(how):
    with pytest.raises(ValueError):
        ds.tf.shade(_agg(), cmap="foo", how=how)
    with pytest.raises(ValueError):
        ds.tf.shade(_agg(), cmap=[], how=how)
    with pytest.raises(ValueError):
        ds.tf.shade(_agg(), cmap=["red", "nosuchcolour"], how=how)
    with pytest.raises(ValueError):
        ds.tf.shade(_agg(), cmap=["red", (0, 300, 0)], how=how)


def test_shade_argument_errors():
    with pytest.raises(ValueError):
        ds.tf.shade(_agg(), how="linear", alpha=300)
    with pytest.raises(ValueError):
        ds.tf.shade(_agg(), how="nosuchhow")
    with pytest.raises(TypeError):
        ds.tf.shade(torch.zeros((3, 3)))
