"""datashader_gb300 -- datashader's projection + aggregation hot path on GB300.

Drop-in for ``Canvas.points`` / ``Canvas.line`` (LineAxis0) with the
reductions count, any, sum, mean, min, max, first, last, where, by /
count_cat and summary, and for ``tf.shade(how='eq_hist')``.  Every
aggregation runs in hand-written sm_103a CUDA kernels (libdsgb, C ABI in
include/dsgb.h) on torch CUDA tensors; there is no CPU fallback.

Usage mirrors ``import datashader as ds``::

    import datashader_gb300 as ds
    frame = ds.TensorFrame({"x": x, "y": y, "v": v})
    agg = ds.Canvas(1024, 1024, (-4, 4), (-4, 4)).points(frame, "x", "y", ds.mean("v"))
"""
from __future__ import annotations

from .core import Canvas, TensorFrame, PartitionedFrame, HostFrame, RaggedColumn, Aggregate, AggregateSet, bypixel, LinearAxis, LogAxis  # noqa: F401
from .core import debug_checks, check_device_status  # noqa: F401
from .reductions import (  # noqa: F401
    count, any, sum, mean, min, max, first, last, where, by, count_cat, summary,
    _sum_zero, _count_ignore_antialiasing, _min_row_index, _max_row_index,
    category_codes, category_modulo, SpecialColumn,
)
from . import transfer_functions  # noqa: F401
from . import transfer_functions as tf  # noqa: F401

__version__ = "0.1.0"
