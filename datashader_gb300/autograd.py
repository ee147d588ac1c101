"""Differentiable aggregation: torch.autograd.Functions over libdsgb.

* :func:`points_sum` / :func:`points_mean` -- Canvas.points sum('v') / mean('v')
  as a function of the value column; the adjoint is the gather
  dL/dv_i = g[pixel(i)] (divided by the pixel's count for mean).
* :func:`line_sum` -- Canvas.line (LineAxis0, antialiased, sum('v'),
  self-intersecting) as a function of the value column and the vertex y
  coordinates; the adjoint recomputes the coverage in forward-mode dual
  arithmetic (dsgb_line_axis0_backward), it is not stored.

The canvas (ranges, size) is fixed: autoranged bounds are not differentiated.
The aggregate keeps the reference's NaN for pixels nothing reached; losses
usually wrap it in ``torch.nan_to_num``, whose backward zeroes those pixels.
"""
from __future__ import annotations

import ctypes

import torch

from . import _native as N
from . import reductions as rd
from .core import Canvas, TensorFrame, dsgb_dtype


def _canvas_desc(canvas, x_range, y_range):
    w, h = canvas.plot_width, canvas.plot_height
    sx, tx = canvas.x_axis.compute_scale_and_translate(x_range, w)
    sy, ty = canvas.y_axis.compute_scale_and_translate(y_range, h)
    return N.CanvasDesc(w, h, int(canvas.x_axis.is_log), int(canvas.y_axis.is_log), sx, tx, sy, ty,
                        float(x_range[0]), float(x_range[1]), float(y_range[0]), float(y_range[1]))


def _ranges(canvas, x, y):
    if canvas.x_range is None or canvas.y_range is None:
        raise ValueError("differentiable aggregation needs a canvas with fixed x_range and y_range")
    return canvas.x_range, canvas.y_range


class _PointsAgg(torch.autograd.Function):
    @staticmethod
    def forward(ctx, v, x, y, canvas, mean):
        x_range, y_range = _ranges(canvas, x, y)
        frame = TensorFrame({"x": x, "y": y, "v": v.detach()})
        red = rd.mean("v") if mean else rd.sum("v")
        out = Canvas(canvas.plot_width, canvas.plot_height, x_range, y_range).points(
            frame, "x", "y", rd.summary(agg=red, cnt=rd.count("v")))
        # The frame's columns are contiguous and on the aggregation device: the
        # backward kernel reads these, never the caller's (possibly strided,
        # expanded or host) tensors.
        ctx.save_for_backward(frame["x"], frame["y"], frame["v"])
        ctx.v_like = (v.dtype, v.device)
        ctx.canvas = canvas
        ctx.counts = out["cnt"].data if mean else None
        return out["agg"].data

    @staticmethod
    def backward(ctx, grad):
        x, y, v = ctx.saved_tensors
        canvas = ctx.canvas
        cv = _canvas_desc(canvas, canvas.x_range, canvas.y_range)
        grad = grad.contiguous().to(torch.float64)
        gv = torch.empty(v.shape, dtype=torch.float64, device=v.device)
        cols = (N.Column * 3)(N.Column(x.data_ptr(), dsgb_dtype(x), 0), N.Column(y.data_ptr(), dsgb_dtype(y), 0),
                              N.Column(v.data_ptr(), dsgb_dtype(v), 0))
        counts = ctx.counts.data_ptr() if ctx.counts is not None else None
        N.check(N.lib().dsgb_points_backward(cols, 3, v.numel(), 0, 1, 2, ctypes.byref(cv), grad.data_ptr(),
                                             counts, gv.data_ptr(), 0,
                                             torch.cuda.current_stream(v.device).cuda_stream),
                "dsgb_points_backward")
        dtype, device = ctx.v_like
        return gv.to(device=device, dtype=dtype), None, None, None, None


def points_sum(x, y, v, canvas):
    """Canvas.points(..., sum('v')) differentiable in ``v``."""
    return _PointsAgg.apply(v, x, y, canvas, False)


def points_mean(x, y, v, canvas):
    """Canvas.points(..., mean('v')) differentiable in ``v``."""
    return _PointsAgg.apply(v, x, y, canvas, True)


class _LineSum(torch.autograd.Function):
    @staticmethod
    def forward(ctx, v, y, x, canvas, line_width):
        x_range, y_range = _ranges(canvas, x, y)
        if not line_width > 0:
            raise ValueError("line_sum differentiates antialiased lines: line_width must be > 0")
        frame = TensorFrame({"x": x, "y": y.detach(), "v": v.detach()})
        out = Canvas(canvas.plot_width, canvas.plot_height, x_range, y_range).line(
            frame, "x", "y", agg=rd.sum("v"), line_width=line_width)
        # contiguous device copies (the frame's columns), as in _PointsAgg
        ctx.save_for_backward(frame["x"], frame["y"], frame["v"])
        ctx.like = ((v.dtype, v.device), (y.dtype, y.device))
        ctx.canvas = canvas
        ctx.line_width = line_width
        return out.data

    @staticmethod
    def backward(ctx, grad):
        x, y, v = ctx.saved_tensors
        canvas = ctx.canvas
        cv = _canvas_desc(canvas, canvas.x_range, canvas.y_range)
        grad = grad.contiguous().to(torch.float64)
        n = v.numel()
        gv = torch.empty(n, dtype=torch.float64, device=v.device)
        gy = torch.empty(n, dtype=torch.float64, device=v.device)
        cols = (N.Column * 3)(N.Column(x.data_ptr(), dsgb_dtype(x), 0), N.Column(y.data_ptr(), dsgb_dtype(y), 0),
                              N.Column(v.data_ptr(), dsgb_dtype(v), 0))
        L = N.lib()
        wsz = int(L.dsgb_line_workspace_size(n))
        ws = torch.empty(max(wsz, 1), dtype=torch.uint8, device=v.device)
        N.check(L.dsgb_line_axis0_backward_ws(cols, 3, n, 0, 1, 2, ctypes.byref(cv), float(ctx.line_width), 1,
                                              grad.data_ptr(), None, gv.data_ptr(), gy.data_ptr(),
                                              ws.data_ptr(), wsz, torch.cuda.current_stream(v.device).cuda_stream),
                "dsgb_line_axis0_backward_ws")
        (vd, vdev), (yd, ydev) = ctx.like
        return gv.to(device=vdev, dtype=vd), gy.to(device=ydev, dtype=yd), None, None, None


def line_sum(x, y, v, canvas, line_width=1.5):
    """Canvas.line(..., sum('v'), line_width) (LineAxis0), differentiable in ``v`` and ``y``."""
    return _LineSum.apply(v, y, x, canvas, line_width)
