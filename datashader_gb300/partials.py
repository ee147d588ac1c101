"""Partial aggregates of row shards, combined across processes.

datashader's dask path aggregates each partition into its own partial bases
and folds them elementwise with each base's combine (dask.py:168-217,
compiler.py:478-507); first / last / where fold their selector and lookup
together (reductions.py:1992-2018).  Here one process aggregates its row
shard with :func:`points_partial` (global row numbers from the frame's
``row_offset``), ships :meth:`PartialAggregate.to_host` (host byte arrays
with their dtypes and shapes, picklable: any transport, e.g.
``torch.distributed``) to one process, and :func:`combine_partials` folds
the shards on its device with ``dsgb_combine`` and finalizes.  A gather
output (first / last / where with a lookup column) takes the value that the
shard holding the selected row looked up itself (``dsgb_select_by_owner``):
no process needs another's columns.
"""
from __future__ import annotations

import ctypes

import torch

from . import _native as N
from .compiler import compile_plan
from .core import Executor, _results, as_frame, workspace
from .glyphs import Point


class _HostArray:
    """A tensor on the host as raw bytes (numpy) with its dtype and shape:
    picklable across torch versions for every dtype, uint32 included."""

    def __init__(self, t):
        t = t.detach().contiguous().cpu()
        self.dtype, self.shape = t.dtype, tuple(t.shape)
        self.data = t.view(-1).view(torch.uint8).numpy().copy()

    def to(self, device):
        return torch.from_numpy(self.data).to(device).view(self.dtype).view(self.shape)


def _to_device(t, device):
    return t.to(device) if isinstance(t, (torch.Tensor, _HostArray)) else t


class PartialAggregate:
    """The partial bases of one row shard, plus its own lookups of the
    gather outputs."""

    def __init__(self, plan, bases, lookups, first_row, nrows, width, height, x_range, y_range, labels):
        self.plan = plan
        self.bases = bases                  # one array per plan base
        self.lookups = lookups              # {output index: float64 array}
        self.first_row, self.nrows = int(first_row), int(nrows)
        self.width, self.height = int(width), int(height)
        self.x_range, self.y_range = tuple(x_range), tuple(y_range)
        self.labels = labels                # (x label, y label)

    def to_host(self):
        """A picklable copy on the host."""
        return PartialAggregate(self.plan, [_HostArray(t) for t in self.bases],
                                {k: _HostArray(t) for k, t in self.lookups.items()}, self.first_row, self.nrows,
                                self.width, self.height, self.x_range, self.y_range, self.labels)

    def to(self, device):
        return PartialAggregate(self.plan, [_to_device(t, device) for t in self.bases],
                                {k: _to_device(t, device) for k, t in self.lookups.items()}, self.first_row,
                                self.nrows, self.width, self.height, self.x_range, self.y_range, self.labels)


def _canvas_desc(canvas, x_range, y_range):
    w, h = canvas.plot_width, canvas.plot_height
    x_st = canvas.x_axis.compute_scale_and_translate(x_range, w)
    y_st = canvas.y_axis.compute_scale_and_translate(y_range, h)
    return N.CanvasDesc(w, h, int(canvas.x_axis.is_log), int(canvas.y_axis.is_log), x_st[0], x_st[1],
                        y_st[0], y_st[1], float(x_range[0]), float(x_range[1]), float(y_range[0]),
                        float(y_range[1]))


def _base_structs(plan, tensors):
    arr = (N.Base * max(1, len(plan.bases)))()
    for i, (b, t) in enumerate(zip(plan.bases, tensors)):
        arr[i] = N.Base(b.op, -1, -1, b.ncat, b.flags, 0, t.data_ptr())
    return arr


def points_partial(canvas, source, x, y, agg=None):
    """Canvas.points over one row shard, without the finalize: the shard's
    partial bases (dask.py:168-173).  The canvas needs fixed ranges (every
    shard must bin alike); ``source.row_offset`` numbers the shard's rows
    globally (reductions.py:85-113)."""
    from . import reductions as rd
    if canvas.x_range is None or canvas.y_range is None:
        raise ValueError("points_partial needs a canvas with fixed x_range and y_range")
    frame = as_frame(source)
    glyph = Point(x, y)
    agg = agg if agg is not None else rd.count()
    glyph.validate(frame)
    agg.validate(frame)
    canvas.validate()
    dev = frame.device
    stream = torch.cuda.current_stream(dev).cuda_stream
    plan = compile_plan(agg, frame)
    width, height = canvas.plot_width, canvas.plot_height
    cv = _canvas_desc(canvas, canvas.x_range, canvas.y_range)
    ex = Executor(frame, plan, glyph)
    ex.allocate(height, width, dev)
    L = N.lib()
    wsz = int(L.dsgb_points_workspace_size_flags(len(frame), ctypes.byref(cv), ex.bases, len(plan.bases), 0))
    ws = workspace(dev, stream, wsz) if wsz else None
    N.check(L.dsgb_points_ws(ex.cols, len(ex.names), len(frame), frame.row_offset, 0, 1, ctypes.byref(cv),
                             ex.bases, len(plan.bases), ex.outs, ex.nouts, ws.data_ptr() if ws is not None else None,
                             wsz, N.FLAG_NO_FINALIZE, stream), "dsgb_points_ws (partial)")
    gathers = [(i, o) for i, (_, o) in enumerate(plan.outputs) if o.fin == N.FIN_GATHER]
    lookups = {}
    if gathers:
        outs = (N.Output * len(gathers))(*[N.Output(o.fin, o.b0, o.b1, ex.col_index[o.col],
                                                    ex.out_tensors[i].data_ptr()) for i, o in gathers])
        N.check(L.dsgb_finalize(ex.cols, len(ex.names), frame.row_offset, ex.bases, len(plan.bases), outs,
                                len(gathers), width * height, stream), "dsgb_finalize (partial lookups)")
        lookups = {i: ex.out_tensors[i] for i, _ in gathers}
    return PartialAggregate(plan, ex.base_tensors, lookups, frame.row_offset, len(frame), width, height,
                            canvas.x_range, canvas.y_range, (glyph.x_label, glyph.y_label))


class _Outputs:
    """The finalized output tensors in the shape _results reads."""

    def __init__(self, out_tensors, keep):
        self.out_tensors = out_tensors
        self.keep = keep


def combine_partials(parts, canvas, device=None):
    """Fold the shards' partial bases in global row order and finalize on
    ``device``: the Aggregate / AggregateSet of Canvas.points over all the
    shards' rows."""
    if not parts:
        raise ValueError("combine_partials needs at least one partial")
    if len(parts) > 64:
        raise NotImplementedError("combine_partials folds at most 64 shards")
    device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    parts = sorted(parts, key=lambda p: p.first_row)
    p0 = parts[0]
    for p in parts[1:]:
        if (p.width, p.height, p.x_range, p.y_range) != (p0.width, p0.height, p0.x_range, p0.y_range) or \
                len(p.bases) != len(p0.bases):
            raise ValueError("partials of different canvases or plans cannot be combined")
    plan = p0.plan
    stream = torch.cuda.current_stream(device).cuda_stream
    L = N.lib()
    ncells = p0.width * p0.height
    head = [_to_device(t, device).clone() for t in p0.bases]
    head_structs = _base_structs(plan, head)
    keep = []
    for p in parts[1:]:
        other = [_to_device(t, device) for t in p.bases]
        keep.append(other)
        N.check(L.dsgb_combine(head_structs, _base_structs(plan, other), len(plan.bases), ncells, stream),
                "dsgb_combine")
    out_tensors, outs = [], []
    for i, (_, o) in enumerate(plan.outputs):
        nc = plan.bases[o.b0].ncat
        shape = (p0.height, p0.width, nc) if o.categories is not None else (p0.height, p0.width)
        if o.fin == 0:
            t = head[o.b0].view(shape)
        else:
            t = torch.empty(shape, dtype=o.dtype, device=device)
            if o.fin == N.FIN_GATHER:
                vals = [_to_device(p.lookups[i], device).contiguous() for p in parts]
                keep.append(vals)
                first = (ctypes.c_int64 * len(parts))(*[p.first_row for p in parts])
                rows = (ctypes.c_int64 * len(parts))(*[p.nrows for p in parts])
                ptrs = (ctypes.c_void_p * len(parts))(*[v.data_ptr() for v in vals])
                N.check(L.dsgb_select_by_owner(ctypes.byref(head_structs[o.b0]), len(parts), first, rows, ptrs,
                                               t.data_ptr(), ncells, stream), "dsgb_select_by_owner")
            else:
                outs.append(N.Output(o.fin, o.b0, o.b1, -1, t.data_ptr()))
        if o.as_bool:
            t = t.view(torch.bool)
        out_tensors.append(t)
    if outs:
        arr = (N.Output * len(outs))(*outs)
        N.check(L.dsgb_finalize(None, 0, 0, head_structs, len(plan.bases), arr, len(outs), ncells, stream),
                "dsgb_finalize (combined)")
    x_st = canvas.x_axis.compute_scale_and_translate(p0.x_range, p0.width)
    y_st = canvas.y_axis.compute_scale_and_translate(p0.y_range, p0.height)
    coords = {p0.labels[0]: canvas.x_axis.compute_index(x_st, p0.width),
              p0.labels[1]: canvas.y_axis.compute_index(y_st, p0.height)}
    return _results(plan, _Outputs(out_tensors, (head, keep)), coords, [p0.labels[1], p0.labels[0]],
                    dict(x_range=p0.x_range, y_range=p0.y_range))
