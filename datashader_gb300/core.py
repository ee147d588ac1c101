"""Canvas, axes and the bypixel pipeline on the GPU.

Mirrors datashader/core.py (Canvas 163-478, Axis 45-145, bypixel
1334-1446) and datashader/data_libraries/pandas.py:26-66 (the
create / extend / finalize orchestration).  Sources are
:class:`TensorFrame` objects -- named 1-D torch tensors on a CUDA device,
with category labels for categorical columns -- in place of pandas / cuDF
frames.  Host (numpy) columns are accepted too and copied to the device
first.  All aggregation runs in libdsgb's sm_103a kernels; there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes
import math
from numbers import Number

import numpy as np
import torch

from . import _native as N
from . import reductions as rd
from .compiler import compile_plan
from .glyphs import (Point, LineAxis0, LineAxis0Multi, LinesAxis1, LinesAxis1XConstant,
                     LinesAxis1YConstant, LinesAxis1Ragged, _MultiLine)


# ----------------------------------------------------------------- sources

_TORCH_TO_DSGB = {
    torch.float32: N.F32, torch.float64: N.F64, torch.int8: N.I8, torch.uint8: N.U8,
    torch.int16: N.I16, torch.int32: N.I32, torch.int64: N.I64, torch.uint32: N.U32,
    torch.bool: N.BOOL,
}
_KIND = {torch.float32: "f", torch.float64: "f", torch.float16: "f", torch.bfloat16: "f",
         torch.int8: "i", torch.int16: "i", torch.int32: "i", torch.int64: "i",
         torch.uint8: "u", torch.uint32: "u", torch.bool: "b"}


def dsgb_dtype(t: torch.Tensor) -> int:
    try:
        return _TORCH_TO_DSGB[t.dtype]
    except KeyError:
        raise TypeError(f"unsupported column dtype {t.dtype}") from None


class RaggedColumn:
    """A ragged-array column (the reference's RaggedArray, datashader/
    datatypes.py): row i holds ``flat[starts[i]:starts[i + 1]]``, the last
    row running to the end of ``flat``.  Build it from a list of per-row
    sequences, or from ``flat`` (float64) and ``starts`` (int64,
    non-decreasing, within ``flat``)."""

    def __init__(self, rows=None, *, flat=None, starts=None):
        if rows is not None:
            lens = [len(r) for r in rows]
            flat = np.concatenate([np.asarray(r, dtype=np.float64) for r in rows]) if lens else np.zeros(0)
            starts = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64) if lens else np.zeros(0, np.int64)
        flat = flat if isinstance(flat, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(flat))
        starts = starts if isinstance(starts, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(starts))
        self.flat = flat.to(torch.float64).contiguous()
        self.starts = starts.to(torch.int64).contiguous()
        if self.flat.dim() != 1 or self.starts.dim() != 1:
            raise ValueError("a ragged column needs a 1-D flat array and 1-D start indices")
        if self.starts.numel():
            st = self.starts
            if bool((st[0] < 0) | (st[-1] > self.flat.numel())) or bool((st[1:] < st[:-1]).any()):
                raise ValueError("ragged start indices must be non-decreasing and within the flat array")

    def __len__(self):
        return self.starts.numel()

    @property
    def device(self):
        return self.flat.device

    def to(self, device, non_blocking=False):
        return RaggedColumn(flat=self.flat.to(device, non_blocking=non_blocking),
                            starts=self.starts.to(device, non_blocking=non_blocking))


class TensorFrame:
    """Named, equal-length 1-D columns on one CUDA device.

    ``categories`` maps a column name to its category labels; the column
    itself then holds integer codes (the pandas Categorical ``.cat.codes``).
    Numpy columns are copied to ``device`` (pinned staging) on construction.
    ``row_offset`` is added to row indexes (first/last/where), like the
    ``_datashader_row_offset`` attribute of a partition (reductions.py:85-113).
    """

    def __init__(self, columns, categories=None, device=None, row_offset=0):
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = torch.device(device)
        self._cols = {}
        n = None
        for k, v in dict(columns).items():
            if isinstance(v, RaggedColumn):
                t = v if v.device == self.device else v.to(self.device)
                rows = len(t)
            else:
                t = self._to_device(v)
                if t.dim() != 1:
                    raise ValueError(f"column {k!r} must be 1-D")
                rows = t.shape[0]
            if n is None:
                n = rows
            elif rows != n:
                raise ValueError("columns must have equal length")
            self._cols[k] = t
        self._n = n or 0
        self._cats = {k: list(v) for k, v in (categories or {}).items()}
        for k in self._cats:
            if k not in self._cols:
                raise ValueError(f"categories given for unknown column {k!r}")
        self.row_offset = int(row_offset)

    def _to_device(self, v):
        if isinstance(v, torch.Tensor):
            t = v
        else:
            a = np.ascontiguousarray(v)
            t = torch.from_numpy(a)
            if self.device.type == "cuda":
                t = t.pin_memory()
        if t.device != self.device:
            t = t.to(self.device, non_blocking=True)
        return t.contiguous()

    # schema interface used by reductions / compiler
    def __contains__(self, name):
        return name in self._cols

    def __getitem__(self, name):
        return self._cols[name]

    def __len__(self):
        return self._n

    @property
    def columns(self):
        return list(self._cols)

    def dtype_kind(self, name):
        if name in self._cats:
            return "c"
        if isinstance(self._cols[name], RaggedColumn):
            return "R"
        return _KIND.get(self._cols[name].dtype, "?")

    def is_categorical(self, name):
        return name in self._cats

    def categories(self, name):
        return self._cats[name]

    def signature(self):
        return tuple((k, "ragged" if isinstance(v, RaggedColumn) else str(v.dtype), tuple(self._cats.get(k, ())))
                     for k, v in self._cols.items())


class PartitionedFrame:
    """Row partitions of one frame (the reference's dask DataFrame, dask.py:53-219):
    each partition is aggregated into its own partial bases (rows numbered
    from the partition's ``row_offset``), the partials are combined
    elementwise (``dsgb_combine``) and finalized once.  Partitions may live in
    separate tensors (out-of-core chunks, or shards gathered from elsewhere)."""

    def __init__(self, partitions):
        parts = [as_frame(p) for p in partitions]
        if not parts:
            raise ValueError("PartitionedFrame needs at least one partition")
        sig = parts[0].signature()
        offset = 0
        fixed = []
        for p in parts:
            if p.signature() != sig:
                raise ValueError("partitions must have the same columns, dtypes and categories")
            cats = {c: p.categories(c) for c in p.columns if p.is_categorical(c)}
            fixed.append(TensorFrame({c: p[c] for c in p.columns}, categories=cats, device=p.device,
                                     row_offset=offset))
            offset += len(p)
        self.partitions = fixed
        self.device = fixed[0].device

    def __len__(self):
        return sum(len(p) for p in self.partitions)

    # schema interface (the partitions share it)
    def __contains__(self, name):
        return name in self.partitions[0]

    def __getitem__(self, name):
        return self.partitions[0][name]

    @property
    def columns(self):
        return self.partitions[0].columns

    def dtype_kind(self, name):
        return self.partitions[0].dtype_kind(name)

    def is_categorical(self, name):
        return self.partitions[0].is_categorical(name)

    def categories(self, name):
        return self.partitions[0].categories(name)

    def signature(self):
        return self.partitions[0].signature()


class HostFrame(TensorFrame):
    """Named columns held in pinned host memory (numpy arrays or CPU tensors
    are pinned once, on construction).  Canvas.points streams them to the
    GPU in chunks of ``chunk_rows`` rows through two device buffers: the copy
    of one chunk (its own CUDA stream) overlaps the aggregation of the
    previous one, every chunk accumulates into the same bases with its row
    offset, and one finalize at the end reads the lookup column of first /
    last / where straight from the pinned host memory.  The data never has
    to fit in device memory.  ``device`` is the GPU that aggregates."""

    def __init__(self, columns, categories=None, device=None, row_offset=0, chunk_rows=1 << 24):
        self.gpu = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if int(chunk_rows) < 1:
            raise ValueError("chunk_rows must be positive")
        self.chunk_rows = int(chunk_rows)
        super().__init__(columns, categories=categories, device="cpu", row_offset=row_offset)

    def _to_device(self, v):
        t = v if isinstance(v, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(v))
        t = t.cpu().contiguous()
        return t if t.is_pinned() else t.pin_memory()

    def on_device(self):
        """The same columns as a TensorFrame on the aggregating GPU (one copy
        each, from the pinned host memory)."""
        return TensorFrame(self._cols, categories=self._cats, device=self.gpu, row_offset=self.row_offset)


def as_frame(source):
    if isinstance(source, (TensorFrame, PartitionedFrame)):
        return source
    if isinstance(source, dict):
        return TensorFrame(source)
    raise ValueError("source must be a TensorFrame or a dict of columns")


# -------------------------------------------------------------------- axes

_INDEX_CACHE = {}


class Axis:
    """core.py:45-111."""

    def compute_scale_and_translate(self, range, n):
        """core.py:62-81: s = n/(end-start), t = -start*s (Python floats)."""
        start, end = map(self.mapper, range)
        s = n / (end - start)
        t = -start * s
        return s, t

    def compute_index(self, st, n):
        """core.py:83-99: pixel-centre coordinates (read-only arrays, built
        once per axis type, scale / translate and size)."""
        key = (type(self), float(st[0]), float(st[1]), int(n))
        c = _INDEX_CACHE.get(key)
        if c is None:
            px = np.arange(n) + 0.5
            s, t = st
            c = self.inverse_mapper((px - t) / s)
            c.flags.writeable = False
            if len(_INDEX_CACHE) > 256:
                _INDEX_CACHE.clear()
            _INDEX_CACHE[key] = c
        return c

    def validate(self, range):
        pass


class LinearAxis(Axis):
    is_log = False

    @staticmethod
    def mapper(val):
        return val

    @staticmethod
    def inverse_mapper(val):
        return val


class LogAxis(Axis):
    is_log = True

    @staticmethod
    def mapper(val):
        return math.log10(float(val))

    @staticmethod
    def inverse_mapper(val):
        return 10 ** val

    def validate(self, range):
        if range is None:
            return
        if range[0] <= 0 or range[1] <= 0:
            raise ValueError("Range values must be >0 for logarithmic axes")


_axis_lookup = {"linear": LinearAxis(), "log": LogAxis()}


# ------------------------------------------------------------ instrumentation

class _NvtxRange:
    """An NVTX range (visible in Nsight Systems / ncu --nvtx) around one
    pipeline stage; a no-op when torch has no NVTX support."""

    def __init__(self, name):
        self.name = name

    def __enter__(self):
        try:
            torch.cuda.nvtx.range_push(self.name)
            self.pushed = True
        except Exception:
            self.pushed = False
        return self

    def __exit__(self, *exc):
        if self.pushed:
            torch.cuda.nvtx.range_pop()


_DEBUG = [False]


class debug_checks:
    """Within this context (or after ``debug_checks(True)`` without ``with``),
    every Canvas.points / Canvas.line call checks each append's aggregate
    index on the device (``DSGB_FLAG_DEBUG_CHECKS``: the generic kernels,
    no hot-tile path), then waits for the device and raises ``DsgbError`` if
    any kernel raised a status bit (an index outside its base, a CAS loop at
    its iteration guard).  The reference's numba appends are unchecked."""

    def __init__(self, enabled=True):
        self.prev = _DEBUG[0]
        _DEBUG[0] = bool(enabled)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        _DEBUG[0] = self.prev


def _raise_on_status(bits):
    if bits:
        names = [n for b, n in ((N.STATUS_CAS_GUARD, "a where() CAS loop reached its iteration guard"),
                                (N.STATUS_INDEX, "an append index fell outside its aggregate")) if bits & b]
        raise N.DsgbError(f"device status {bits:#x}: " + "; ".join(names))


def check_device_status(clear=True):
    """Wait for the device and raise ``DsgbError`` if a kernel of the
    library raised a status bit since the last check."""
    _raise_on_status(N.device_status(clear))


# ----------------------------------------------------------------- results

class Aggregate:
    """A 2-D (or 3-D categorical) aggregate: the xr.DataArray of the reference
    (pandas.py:61-66: dims [y, x(, cat)], coords = pixel centres, attrs
    x_range / y_range), with ``data`` a CUDA tensor."""

    def __init__(self, data, dims, coords, attrs, name=None):
        self.data = data
        self.dims = list(dims)
        self.coords = dict(coords)
        self.attrs = dict(attrs)
        self.name = name

    @property
    def values(self):
        return self.data.cpu().numpy()

    def to_numpy(self):
        return self.values

    @property
    def shape(self):
        return tuple(self.data.shape)

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def ndim(self):
        return self.data.dim()

    @property
    def x_range(self):
        return self.attrs.get("x_range")

    @property
    def y_range(self):
        return self.attrs.get("y_range")

    def __repr__(self):
        return f"<Aggregate {self.name or ''} dims={self.dims} shape={self.shape} dtype={self.dtype}>"


class AggregateSet(dict):
    """The xr.Dataset returned for a summary() reduction."""

    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError:
            raise AttributeError(k) from None


# ------------------------------------------------------------------ canvas

def _validate_xy(glyph, x, y, geometry):
    if geometry is not None:
        raise NotImplementedError("geometry columns are not supported on the GPU path")
    if x is None or y is None:
        raise ValueError(f"{glyph} coordinates may be specified by providing both the x and y arguments")


class Canvas:
    """An abstract canvas representing the space in which to bin (core.py:163-185)."""

    def __init__(self, plot_width=600, plot_height=600, x_range=None, y_range=None,
                 x_axis_type="linear", y_axis_type="linear"):
        self.plot_width = plot_width
        self.plot_height = plot_height
        self.x_range = None if x_range is None else tuple(x_range)
        self.y_range = None if y_range is None else tuple(y_range)
        self.x_axis = _axis_lookup[x_axis_type]
        self.y_axis = _axis_lookup[y_axis_type]

    def points(self, source, x=None, y=None, agg=None, geometry=None, *, deterministic=False):
        """Compute a reduction by pixel, mapping data to pixels as points (core.py:187-232).

        ``deterministic=True`` (an addition to the reference's signature) adds
        the float64 sums of sum / mean in row order, bit-identical to the
        reference's CPU loop and from run to run; the other reductions are
        order-independent already."""
        _validate_xy("Point", x, y, geometry)
        if agg is None:
            agg = rd.count()
        return bypixel(source, self, Point(x, y), agg,
                       flags=N.FLAG_DETERMINISTIC if deterministic else 0)

    def line(self, source, x=None, y=None, agg=None, axis=0, geometry=None,
             line_width=0, antialias=False):
        """Compute a reduction by pixel, mapping data to pixels as one line
        (LineAxis0 glyph, core.py:234-478)."""
        _validate_xy("Line", x, y, geometry)
        if agg is None:
            agg = rd.any()
        if line_width is None:
            line_width = 0
        if antialias and line_width != 0:
            raise ValueError("Do not specify values for both the line_width and \n"
                             "antialias keyword arguments; use line_width instead.")
        if antialias:
            line_width = 1.0
        glyph = _line_glyph(x, y, axis)
        glyph.set_line_width(line_width)
        if glyph.antialiased:
            non_cat = agg.reduction if isinstance(agg, rd.by) else agg
            if not isinstance(non_cat, (rd.any, rd.count, rd.max, rd.min, rd.sum, rd.summary,
                                        rd._sum_zero, rd._first_or_last, rd.mean,
                                        rd._max_or_min_row_index, rd.where)):
                raise NotImplementedError(
                    f"{type(non_cat)} reduction not implemented for antialiased lines")
        if glyph.antialiased and isinstance(glyph, _MultiLine):
            from .compiler import compile_plan as _cp
            plan = _cp(agg, as_frame(source), antialias=True)
            if plan.use_2_stage and any(b.fold == 0 for b in plan.bases):
                raise NotImplementedError("a reduction of this two-stage antialiased plan has no stage-2 fold")
        return bypixel(source, self, glyph, agg, antialias=glyph.antialiased)

    def validate_ranges(self, x_range, y_range):
        self.x_axis.validate(x_range)
        self.y_axis.validate(y_range)

    def validate_size(self, width, height):
        if width <= 0 or height <= 0:
            raise ValueError("Invalid size: plot_width and plot_height must be bigger than 0")

    def validate(self):
        self.validate_ranges(self.x_range, self.y_range)
        self.validate_size(self.plot_width, self.plot_height)


def _broadcast_columns(x, y):
    """core.py:1433-1443: a single column name against a list becomes a list."""
    lengths = {len(a) for a in (x, y) if isinstance(a, (list, tuple))}
    if len(lengths) != 1:
        return x, y
    n = lengths.pop()
    return tuple((a,) * n if isinstance(a, (Number, str)) else a for a in (x, y))


def _line_glyph(x, y, axis):
    """core.py:412-456: the glyph for the x / y / axis combination."""
    ox, oy = x, y
    x, y = _broadcast_columns(x, y)
    if axis == 0:
        if isinstance(x, (Number, str)) and isinstance(y, (Number, str)):
            return LineAxis0(x, y)
        if isinstance(x, (list, tuple)) and isinstance(y, (list, tuple)):
            return LineAxis0Multi(tuple(x), tuple(y))
        raise ValueError(f"Invalid combination of x and y arguments to Canvas.line when axis=0.\n"
                         f"    Received:\n        x: {ox!r}\n        y: {oy!r}")
    if axis == 1:
        if isinstance(x, (list, tuple)) and isinstance(y, (list, tuple)):
            return LinesAxis1(tuple(x), tuple(y))
        if isinstance(x, np.ndarray) and isinstance(y, (list, tuple)):
            return LinesAxis1XConstant(x, tuple(y))
        if isinstance(x, (list, tuple)) and isinstance(y, np.ndarray):
            return LinesAxis1YConstant(tuple(x), y)
        if isinstance(x, (Number, str)) and isinstance(y, (Number, str)):
            return LinesAxis1Ragged(x, y)
        raise ValueError(f"Invalid combination of x and y arguments to Canvas.line when axis=1.\n"
                         f"    Received:\n        x: {ox!r}\n        y: {oy!r}")
    raise ValueError(f"The axis argument to Canvas.line must be 0 or 1\n    Received: {axis}")


def _vertex_array(frame, spec, nrows):
    """float64 vertex array of a multi-line glyph: [nrows][len(spec)] from the
    columns, or the constant numpy array itself (1-D)."""
    if isinstance(spec, np.ndarray):
        return torch.as_tensor(np.ascontiguousarray(spec, dtype=np.float64), device=frame.device)
    cols = [frame[c].to(torch.float64) for c in spec]
    return torch.stack(cols, dim=1).contiguous() if cols else torch.empty((nrows, 0), dtype=torch.float64,
                                                                         device=frame.device)


def _array_bounds(t, stream):
    col = N.Column(t.data_ptr(), N.F64, 0)
    out = torch.empty(2, dtype=torch.float64, device=t.device)
    N.check(N.lib().dsgb_bounds(ctypes.byref(col), t.numel(), out.data_ptr(), stream), "dsgb_bounds")
    return _expand_bounds(*out.cpu().tolist())


def bypixel(source, canvas, glyph, agg, *, antialias=False, flags=0):
    """core.py:1334-1359: validate, then run the GPU pipeline."""
    if _DEBUG[0]:
        N.device_status(clear=True)            # start from a clean status word
        out = _bypixel(source, canvas, glyph, agg, antialias=antialias, flags=flags | N.FLAG_DEBUG_CHECKS)
        check_device_status()
        return out
    return _bypixel(source, canvas, glyph, agg, antialias=antialias, flags=flags)


def _bypixel(source, canvas, glyph, agg, *, antialias=False, flags=0):
    with _NvtxRange("dsgb validate"):
        frame = as_frame(source)
        glyph.validate(frame)
        agg.validate(frame)
        canvas.validate()
    if isinstance(frame, PartitionedFrame):
        return partitioned_pipeline(frame, canvas, glyph, agg, flags=flags)
    if isinstance(frame, HostFrame):
        if not isinstance(glyph, Point):
            # a line reads its neighbouring vertices and crosses any chunk edge: copy the frame once
            return gpu_pipeline(frame.on_device(), canvas, glyph, agg, antialias=antialias, flags=flags)
        return streamed_pipeline(frame, canvas, glyph, agg, flags=flags)
    return gpu_pipeline(frame, canvas, glyph, agg, antialias=antialias, flags=flags)


def _raw_array_bounds(t, stream):
    """NaN-skipping (min, max) of a float64 vertex array, unexpanded."""
    t = t.contiguous()
    col = N.Column(t.data_ptr(), N.F64, 0)
    out = torch.empty(2, dtype=torch.float64, device=t.device)
    N.check(N.lib().dsgb_bounds(ctypes.byref(col), t.numel(), out.data_ptr(), stream), "dsgb_bounds")
    return tuple(out.cpu().tolist())


def _column_raw_bounds(frame, name, stream):
    """Glyph._compute_bounds (glyph.py:51-78) on the device: NaN-skipping (min, max)."""
    t = frame[name]
    col = N.Column(t.data_ptr(), dsgb_dtype(t), 0)
    out = torch.empty(2, dtype=torch.float64, device=t.device)
    N.check(N.lib().dsgb_bounds(ctypes.byref(col), t.numel(), out.data_ptr(), stream), "dsgb_bounds")
    return tuple(out.cpu().tolist())


def _expand_bounds(mn, mx):
    """maybe_expand_bounds (glyph.py:42-49)."""
    if not (np.isfinite(mn) and np.isfinite(mx)):
        mn, mx = -1.0, 1.0
    elif mn == mx:
        mn, mx = mn - 1, mn + 1
    return mn, mx


def _column_bounds(frame, name, stream):
    return _expand_bounds(*_column_raw_bounds(frame, name, stream))


def _derived_columns(frame, plan):
    cols = {}
    for name, (col, modulo, offset) in plan.derived.items():
        cols[name] = torch.remainder(frame[col].to(torch.int64) - offset, modulo).to(torch.int32)
    return cols


class Executor:
    """Allocates the bases and outputs of a plan and calls the C ABI."""

    def __init__(self, frame, plan, glyph):
        self.frame = frame
        self.plan = plan
        self.glyph = glyph
        derived = _derived_columns(frame, plan)
        if isinstance(glyph, _MultiLine):
            # vertices travel separately (dsgb_lines); the columns are the appends' fields
            names = list(plan.columns)
        else:
            names = [glyph.x, glyph.y] + [c for c in plan.columns if c not in (glyph.x, glyph.y)]
        self.names = names
        self.tensors = [derived[n] if n in derived else frame[n] for n in names]
        self.col_index = {n: i for i, n in enumerate(names)}
        self.cols = (N.Column * len(names))(*[N.Column(t.data_ptr(), dsgb_dtype(t), 0) for t in self.tensors])

    def allocate(self, height, width, device):
        plan = self.plan
        self.base_tensors = []
        for b in plan.bases:
            n = height * width * b.ncat * b.words
            self.base_tensors.append(torch.empty(n, dtype=b.torch_dtype, device=device))
        self.bases = (N.Base * max(1, len(plan.bases)))()
        for i, (b, t) in enumerate(zip(plan.bases, self.base_tensors)):
            self.bases[i] = N.Base(b.op, self.col_index[b.col] if b.col is not None else -1,
                                   self.col_index[b.cat] if b.cat is not None else -1,
                                   b.ncat, b.flags, 0, t.data_ptr())
        outs = []
        self.out_tensors = []
        for key, o in plan.outputs:
            nc = plan.bases[o.b0].ncat
            shape = (height, width, nc) if o.categories is not None else (height, width)
            if o.fin == 0:
                t = self.base_tensors[o.b0].view(shape)
            else:
                t = torch.empty(shape, dtype=o.dtype, device=device)
                outs.append(N.Output(o.fin, o.b0, o.b1,
                                     self.col_index[o.col] if o.col is not None else -1, t.data_ptr()))
            if o.as_bool:
                t = t.view(torch.bool)
            self.out_tensors.append(t)
        self.outs = (N.Output * max(1, len(outs)))(*outs)
        self.nouts = len(outs)


def _results(plan, ex, coords, dims, attrs):
    items = []
    for (key, o), t in zip(plan.outputs, ex.out_tensors):
        d = list(dims)
        c = dict(coords)
        if o.categories is not None:
            d.append(o.cat_dim)
            c[o.cat_dim] = list(o.categories)
        items.append((key, Aggregate(t, d, c, attrs, name=key)))
    if plan.outputs[0][0] is None:
        return items[0][1]
    return AggregateSet(items)


_WORKSPACES = {}


def workspace(device, stream, nbytes):
    """A device scratch buffer of at least ``nbytes`` owned by (device, stream).

    Calls on one stream run in order, so they may share it; another stream
    gets its own buffer."""
    key = (str(device), int(stream))
    t = _WORKSPACES.get(key)
    if t is None or t.numel() < nbytes:
        t = torch.empty(max(nbytes, 1 << 20), dtype=torch.uint8, device=device)
        _WORKSPACES[key] = t
    return t


def gpu_pipeline(frame, canvas, glyph, agg, *, antialias=False, flags=0, stream=None):
    """pandas.py:26-66 on the GPU: ranges, scale/translate, create+extend+finalize."""
    if stream is None:
        stream = torch.cuda.current_stream(frame.device).cuda_stream
    with _NvtxRange("dsgb plan"):
        plan = compile_plan(agg, frame, antialias=antialias)
    if isinstance(glyph, LinesAxis1Ragged):
        xr, yr = frame[glyph.x], frame[glyph.y]
        x_range = canvas.x_range or _array_bounds(xr.flat, stream)
        y_range = canvas.y_range or _array_bounds(yr.flat, stream)
    elif isinstance(glyph, _MultiLine):
        xs = _vertex_array(frame, glyph.x, len(frame))
        ys = _vertex_array(frame, glyph.y, len(frame))
        x_range = canvas.x_range or _array_bounds(xs, stream)
        y_range = canvas.y_range or _array_bounds(ys, stream)
    else:
        x_range = canvas.x_range or _column_bounds(frame, glyph.x, stream)
        y_range = canvas.y_range or _column_bounds(frame, glyph.y, stream)
    canvas.validate_ranges(x_range, y_range)
    width, height = canvas.plot_width, canvas.plot_height
    x_st = canvas.x_axis.compute_scale_and_translate(x_range, width)
    y_st = canvas.y_axis.compute_scale_and_translate(y_range, height)
    ex = Executor(frame, plan, glyph)
    ex.allocate(height, width, frame.device)
    cv = N.CanvasDesc(width, height, int(canvas.x_axis.is_log), int(canvas.y_axis.is_log),
                      x_st[0], x_st[1], y_st[0], y_st[1],
                      float(x_range[0]), float(x_range[1]), float(y_range[0]), float(y_range[1]))
    L = N.lib()
    if isinstance(glyph, LineAxis0):
        wsz = int(L.dsgb_line_workspace_size(len(frame))) if glyph.line_width > 0 else 0
        ws = workspace(frame.device, stream, wsz) if wsz else None
        rc = L.dsgb_line_axis0_ws(ex.cols, len(ex.names), len(frame), frame.row_offset, 0, 1, ctypes.byref(cv),
                                  float(glyph.line_width), 1, int(plan.overwrite), int(plan.use_2_stage),
                                  ex.bases, len(plan.bases), ex.outs, ex.nouts,
                                  ws.data_ptr() if ws is not None else None, wsz, flags, stream)
        N.check(rc, "dsgb_line_axis0_ws")
    elif isinstance(glyph, LinesAxis1Ragged):
        cols, ncols = ex.cols, len(ex.names)
        if ncols == 0:                       # count() / any(): no field column, any valid pointer
            cols = (N.Column * 1)(N.Column(xr.starts.data_ptr(), N.I64, 0))   # one entry a row
            ncols = 1
        if antialias and plan.use_2_stage:
            # one row at a time, folded row by row (line.py:1616-1693)
            line_aggs = [torch.empty_like(t) for t in ex.base_tensors]
            folds = (ctypes.c_int32 * max(1, len(plan.bases)))(*[b.fold for b in plan.bases])
            ptrs = (ctypes.c_void_p * max(1, len(plan.bases)))(*[t.data_ptr() for t in line_aggs])
            rc = L.dsgb_lines_ragged_2stage(cols, ncols, len(frame), frame.row_offset, xr.flat.data_ptr(),
                                            xr.flat.numel(), xr.starts.data_ptr(), yr.flat.data_ptr(),
                                            yr.flat.numel(), yr.starts.data_ptr(), ctypes.byref(cv),
                                            float(glyph.line_width), int(plan.overwrite), ex.bases,
                                            len(plan.bases), folds, ptrs, ex.outs, ex.nouts, flags, stream)
            N.check(rc, "dsgb_lines_ragged_2stage")
        else:
            rc = L.dsgb_lines_ragged(cols, ncols, len(frame), frame.row_offset, xr.flat.data_ptr(),
                                     xr.flat.numel(), xr.starts.data_ptr(), yr.flat.data_ptr(), yr.flat.numel(),
                                     yr.starts.data_ptr(), ctypes.byref(cv), float(glyph.line_width),
                                     int(plan.overwrite), ex.bases, len(plan.bases), ex.outs, ex.nouts, flags,
                                     stream)
            N.check(rc, "dsgb_lines_ragged")
    elif isinstance(glyph, _MultiLine):
        if glyph.layout == 1:
            nv, xrow, yrow = xs.shape[1], xs.shape[1], ys.shape[1]
        else:
            nv = xs.shape[-1] if xs.dim() == 2 else ys.shape[-1]
            xrow = nv if xs.dim() == 2 else 0
            yrow = nv if ys.dim() == 2 else 0
        cols, ncols = ex.cols, len(ex.names)
        if ncols == 0:                       # count() / any(): no field column, any valid pointer
            cols = (N.Column * 1)(N.Column(ys.data_ptr(), N.F64, 0))
            ncols = 1
        if antialias and plan.use_2_stage:
            # each line alone, folded line by line (line.py:1203-1226 and siblings)
            line_aggs = [torch.empty_like(t) for t in ex.base_tensors]
            folds = (ctypes.c_int32 * max(1, len(plan.bases)))(*[b.fold for b in plan.bases])
            ptrs = (ctypes.c_void_p * max(1, len(plan.bases)))(*[t.data_ptr() for t in line_aggs])
            rc = L.dsgb_lines_2stage(cols, ncols, len(frame), frame.row_offset, glyph.layout, xs.data_ptr(),
                                     ys.data_ptr(), nv, xrow, yrow, ctypes.byref(cv), float(glyph.line_width),
                                     int(plan.overwrite), ex.bases, len(plan.bases), folds, ptrs, ex.outs,
                                     ex.nouts, flags, stream)
            N.check(rc, "dsgb_lines_2stage")
        else:
            rc = L.dsgb_lines(cols, ncols, len(frame), frame.row_offset, glyph.layout, xs.data_ptr(),
                              ys.data_ptr(), nv, xrow, yrow, ctypes.byref(cv), float(glyph.line_width), 1,
                              int(plan.overwrite), ex.bases, len(plan.bases), ex.outs, ex.nouts, flags, stream)
            N.check(rc, "dsgb_lines")
    else:
        wsz = int(L.dsgb_points_workspace_size_flags(len(frame), ctypes.byref(cv), ex.bases, len(plan.bases),
                                                     flags))
        ws = workspace(frame.device, stream, wsz) if wsz else None
        rc = L.dsgb_points_ws(ex.cols, len(ex.names), len(frame), frame.row_offset, 0, 1, ctypes.byref(cv),
                              ex.bases, len(plan.bases), ex.outs, ex.nouts,
                              ws.data_ptr() if ws is not None else None, wsz, flags, stream)
        N.check(rc, "dsgb_points_ws")
    # the coordinates are built while the kernels run
    coords = {glyph.x_label: canvas.x_axis.compute_index(x_st, width),
              glyph.y_label: canvas.y_axis.compute_index(y_st, height)}
    dims = [glyph.y_label, glyph.x_label]
    with _NvtxRange("dsgb results"):
        return _results(plan, ex, coords, dims, dict(x_range=x_range, y_range=y_range))


def _line_chunks(parts):
    """dask.py:222-266: partition 0 alone with plot_start; every later
    partition behind the last row of the previous one, with plot_start False
    (the segment across the boundary is drawn with the later partition)."""
    out = []
    for i, part in enumerate(parts):
        if i == 0 or len(parts[i - 1]) == 0:
            out.append((part, 1))
            continue
        prev = parts[i - 1]
        cols = {c: torch.cat([prev[c][-1:], part[c]]) for c in part.columns}
        cats = {c: part.categories(c) for c in part.columns if part.is_categorical(c)}
        out.append((TensorFrame(cols, categories=cats, device=part.device, row_offset=part.row_offset - 1), 0))
    return out


def partitioned_pipeline(pframe, canvas, glyph, agg, *, flags=0, stream=None):
    """dask.py:86-219 on one GPU: every partition into its own partial bases,
    an elementwise combine, one finalize.  LineAxis0 partitions are drawn as
    the reference's dask line path draws them (dask.py:222-266); the
    multi-line glyphs take the generic path (dask.py:86-219): each partition's
    rows drawn alone, first / last / where by global row (row-index
    reductions), not by the line-major visit order of one frame."""
    is_line = isinstance(glyph, LineAxis0)
    multi = isinstance(glyph, _MultiLine)
    if isinstance(glyph, LinesAxis1Ragged):
        raise NotImplementedError("partitioned sources of ragged lines are not supported")
    if flags & N.FLAG_DETERMINISTIC:
        raise NotImplementedError("the deterministic mode sums one frame in row order; concatenate the partitions")
    parts = pframe.partitions
    dev = pframe.device
    if stream is None:
        stream = torch.cuda.current_stream(dev).cuda_stream
    plan = compile_plan(agg, parts[0], antialias=(is_line or multi) and glyph.antialiased)
    if (is_line or multi) and plan.use_2_stage:
        raise NotImplementedError("two-stage antialiased plans are not supported on partitioned sources")
    if any(o.fin == N.FIN_GATHER for _, o in plan.outputs) and len(parts) > 64:
        raise NotImplementedError("first/last/where with a lookup column gather from at most 64 partitions")
    if canvas.x_range is not None and canvas.y_range is not None:
        x_range, y_range = canvas.x_range, canvas.y_range
    elif multi:
        bx = [_raw_array_bounds(_vertex_array(p, glyph.x, len(p)), stream) for p in parts] or [(np.inf, -np.inf)]
        by = [_raw_array_bounds(_vertex_array(p, glyph.y, len(p)), stream) for p in parts] or [(np.inf, -np.inf)]
        x_range = canvas.x_range or _expand_bounds(min(b[0] for b in bx), max(b[1] for b in bx))
        y_range = canvas.y_range or _expand_bounds(min(b[0] for b in by), max(b[1] for b in by))
    else:
        bx = [_column_raw_bounds(p, glyph.x, stream) for p in parts] or [(np.inf, -np.inf)]
        by = [_column_raw_bounds(p, glyph.y, stream) for p in parts] or [(np.inf, -np.inf)]
        x_range = canvas.x_range or _expand_bounds(min(b[0] for b in bx), max(b[1] for b in bx))
        y_range = canvas.y_range or _expand_bounds(min(b[0] for b in by), max(b[1] for b in by))
    canvas.validate_ranges(x_range, y_range)
    width, height = canvas.plot_width, canvas.plot_height
    x_st = canvas.x_axis.compute_scale_and_translate(x_range, width)
    y_st = canvas.y_axis.compute_scale_and_translate(y_range, height)
    cv = N.CanvasDesc(width, height, int(canvas.x_axis.is_log), int(canvas.y_axis.is_log),
                      x_st[0], x_st[1], y_st[0], y_st[1],
                      float(x_range[0]), float(x_range[1]), float(y_range[0]), float(y_range[1]))
    L = N.lib()
    execs = []
    chunks = _line_chunks(parts) if is_line else [(p, 1) for p in parts]
    for part, plot_start in chunks:
        ex = Executor(part, plan, glyph)
        ex.allocate(height, width, dev)
        if multi:
            xs = _vertex_array(part, glyph.x, len(part))
            ys = _vertex_array(part, glyph.y, len(part))
            if glyph.layout == 1:
                nv, xrow, yrow = xs.shape[1], xs.shape[1], ys.shape[1]
            else:
                nv = xs.shape[-1] if xs.dim() == 2 else ys.shape[-1]
                xrow = nv if xs.dim() == 2 else 0
                yrow = nv if ys.dim() == 2 else 0
            cols, ncols = ex.cols, len(ex.names)
            if ncols == 0:                   # count() / any(): no field column, any valid pointer
                cols = (N.Column * 1)(N.Column(ys.data_ptr(), N.F64, 0))
                ncols = 1
            N.check(L.dsgb_lines(cols, ncols, len(part), part.row_offset, glyph.layout, xs.data_ptr(), ys.data_ptr(),
                                 nv, xrow, yrow, ctypes.byref(cv), float(glyph.line_width), 1, int(plan.overwrite),
                                 ex.bases, len(plan.bases), ex.outs, ex.nouts,
                                 flags | N.FLAG_NO_FINALIZE | N.FLAG_ROW_ORDER, stream), "dsgb_lines (partition)")
            ex.keep = (xs, ys)           # the vertex arrays live until the stream has used them
        elif is_line:
            wsz = int(L.dsgb_line_workspace_size(len(part))) if glyph.line_width > 0 else 0
            ws = workspace(dev, stream, wsz) if wsz else None
            N.check(L.dsgb_line_axis0_ws(ex.cols, len(ex.names), len(part), part.row_offset, 0, 1, ctypes.byref(cv),
                                         float(glyph.line_width), plot_start, int(plan.overwrite), 0,
                                         ex.bases, len(plan.bases), ex.outs, ex.nouts,
                                         ws.data_ptr() if ws is not None else None, wsz,
                                         flags | N.FLAG_NO_FINALIZE, stream), "dsgb_line_axis0_ws (partition)")
        else:
            wsz = int(L.dsgb_points_workspace_size_flags(len(part), ctypes.byref(cv), ex.bases, len(plan.bases),
                                                         flags))
            ws = workspace(dev, stream, wsz) if wsz else None
            N.check(L.dsgb_points_ws(ex.cols, len(ex.names), len(part), part.row_offset, 0, 1, ctypes.byref(cv),
                                     ex.bases, len(plan.bases), ex.outs, ex.nouts,
                                     ws.data_ptr() if ws is not None else None, wsz, flags | N.FLAG_NO_FINALIZE,
                                     stream), "dsgb_points_ws (partition)")
        execs.append(ex)
    head = execs[0]
    for ex in execs[1:]:
        N.check(L.dsgb_combine(head.bases, ex.bases, len(plan.bases), width * height, stream), "dsgb_combine")
    if head.nouts:
        # gathers (first / last / where with a lookup column) read the selected global row
        # from the partition that holds it
        ncols = len(head.names)
        pcols = (N.Column * max(1, ncols * len(execs)))(*[c for ex in execs for c in ex.cols])
        first = (ctypes.c_int64 * len(chunks))(*[c.row_offset for c, _ in chunks])
        rows = (ctypes.c_int64 * len(chunks))(*[len(c) for c, _ in chunks])
        N.check(L.dsgb_finalize_partitioned(pcols, ncols, len(chunks), first, rows, head.bases, len(plan.bases),
                                            head.outs, head.nouts, width * height, stream),
                "dsgb_finalize_partitioned")
    coords = {glyph.x_label: canvas.x_axis.compute_index(x_st, width),
              glyph.y_label: canvas.y_axis.compute_index(y_st, height)}
    dims = [glyph.y_label, glyph.x_label]
    return _results(plan, head, coords, dims, dict(x_range=x_range, y_range=y_range))


_COPY_STREAMS = {}


def _chunks(n, size):
    return [(c0, min(n, c0 + size)) for c0 in range(0, n, size)] or [(0, 0)]


class _Staging:
    """Two device buffers per column and the events that order a chunk's
    copy (on a copy stream) against the kernels that read it."""

    def __init__(self, hframe, names, dev):
        self.hf, self.names, self.dev = hframe, names, dev
        self.rows = min(hframe.chunk_rows, max(len(hframe), 1))
        self.bufs = {k: [torch.empty(self.rows, dtype=hframe[k].dtype, device=dev) for _ in range(2)]
                     for k in names}
        key = str(dev)
        if key not in _COPY_STREAMS:
            _COPY_STREAMS[key] = torch.cuda.Stream(dev)
        self.copy = _COPY_STREAMS[key]
        self.ready = [torch.cuda.Event() for _ in range(2)]
        self.free = [torch.cuda.Event() for _ in range(2)]

    def stage(self, i, c0, c1, compute):
        """Copy rows [c0, c1) into slot i % 2 and make ``compute`` wait for them."""
        s = i % 2
        with torch.cuda.stream(self.copy):
            if i >= 2:
                self.copy.wait_event(self.free[s])       # the kernels of chunk i - 2 are done with the slot
            for k in self.names:
                self.bufs[k][s][:c1 - c0].copy_(self.hf[k][c0:c1], non_blocking=True)
            self.ready[s].record(self.copy)
        compute.wait_event(self.ready[s])
        return {k: self.bufs[k][s][:c1 - c0] for k in self.names}

    def release(self, i, compute):
        self.free[i % 2].record(compute)


def _streamed_bounds(hf, staging, names, compute):
    lo = {k: np.inf for k in names}
    hi = {k: -np.inf for k in names}
    stream = compute.cuda_stream
    for i, (c0, c1) in enumerate(_chunks(len(hf), staging.rows)):
        if c1 == c0:
            continue
        cols = staging.stage(i, c0, c1, compute)
        for k in names:
            t = cols[k]
            out = torch.empty(2, dtype=torch.float64, device=staging.dev)
            N.check(N.lib().dsgb_bounds(ctypes.byref(N.Column(t.data_ptr(), dsgb_dtype(t), 0)), t.numel(),
                                        out.data_ptr(), stream), "dsgb_bounds")
            mn, mx = out.cpu().tolist()
            lo[k], hi[k] = min(lo[k], mn), max(hi[k], mx)
        staging.release(i, compute)
    return {k: _expand_bounds(lo[k], hi[k]) for k in names}


def streamed_pipeline(hf, canvas, glyph, agg, *, flags=0):
    """Canvas.points over a HostFrame: chunks copied on a copy stream while
    the previous chunk aggregates; bases initialised by the first chunk,
    accumulated by the rest (each with its global row offset), finalized
    once (first / last / where gather from the pinned host column)."""
    if not isinstance(glyph, Point):
        raise NotImplementedError("host-resident frames are streamed for Canvas.points")
    if flags & N.FLAG_DETERMINISTIC:
        raise NotImplementedError("the deterministic mode sums one device frame in row order")
    dev = hf.gpu
    compute = torch.cuda.current_stream(dev)
    stream = compute.cuda_stream
    plan = compile_plan(agg, hf)
    needed = [glyph.x, glyph.y]
    for c in list(plan.columns) + [src for src, _, _ in plan.derived.values()]:
        if c in hf and c not in needed:
            needed.append(c)
    staging = _Staging(hf, needed, dev)
    if canvas.x_range is None or canvas.y_range is None:
        b = _streamed_bounds(hf, staging, [k for k, r in ((glyph.x, canvas.x_range), (glyph.y, canvas.y_range))
                                           if r is None], compute)
        x_range = canvas.x_range or b[glyph.x]
        y_range = canvas.y_range or b[glyph.y]
    else:
        x_range, y_range = canvas.x_range, canvas.y_range
    canvas.validate_ranges(x_range, y_range)
    width, height = canvas.plot_width, canvas.plot_height
    x_st = canvas.x_axis.compute_scale_and_translate(x_range, width)
    y_st = canvas.y_axis.compute_scale_and_translate(y_range, height)
    cv = N.CanvasDesc(width, height, int(canvas.x_axis.is_log), int(canvas.y_axis.is_log),
                      x_st[0], x_st[1], y_st[0], y_st[1],
                      float(x_range[0]), float(x_range[1]), float(y_range[0]), float(y_range[1]))
    L = N.lib()
    head = ex = None
    cats = {k: v for k, v in hf._cats.items() if k in needed}
    # without derived columns a chunk's columns are the staging slot's buffers
    # from their first element: each slot's column array is built once
    slot_ex = [None, None] if not plan.derived else None
    wsz = ws = None
    for i, (c0, c1) in enumerate(_chunks(len(hf), staging.rows)):
        cols = staging.stage(i, c0, c1, compute)
        if slot_ex is not None and slot_ex[i % 2] is not None:
            ex = slot_ex[i % 2]
        else:
            chunk = TensorFrame(cols, categories=cats, device=dev, row_offset=hf.row_offset + c0)
            ex = Executor(chunk, plan, glyph)
            if slot_ex is not None:
                slot_ex[i % 2] = ex
        if head is None:
            ex.allocate(height, width, dev)
            head = ex
        m = c1 - c0
        if wsz is None:
            # the first chunk is the longest: its workspace serves every chunk
            wsz = int(L.dsgb_points_workspace_size_flags(m, ctypes.byref(cv), head.bases, len(plan.bases), flags))
            ws = workspace(dev, stream, wsz) if wsz else None
        f = flags | N.FLAG_NO_FINALIZE | (N.FLAG_NO_INIT if i > 0 else 0)
        N.check(L.dsgb_points_ws(ex.cols, len(ex.names), m, hf.row_offset + c0, 0, 1, ctypes.byref(cv),
                                 head.bases, len(plan.bases), head.outs, head.nouts,
                                 ws.data_ptr() if ws is not None else None, wsz, f, stream),
                "dsgb_points_ws (chunk)")
        staging.release(i, compute)
    if head.nouts:
        # the finalize's gathers index global rows: give it the whole pinned host columns
        # (mapped into the device's address space); derived columns are not gathered
        fin = (N.Column * len(ex.names))(*[
            N.Column(hf[k].data_ptr() if k in hf else t.data_ptr(), dsgb_dtype(hf[k] if k in hf else t), 0)
            for k, t in zip(ex.names, ex.tensors)])
        N.check(L.dsgb_finalize(fin, len(ex.names), hf.row_offset, head.bases, len(plan.bases), head.outs,
                                head.nouts, width * height, stream), "dsgb_finalize")
    coords = {glyph.x_label: canvas.x_axis.compute_index(x_st, width),
              glyph.y_label: canvas.y_axis.compute_index(y_st, height)}
    dims = [glyph.y_label, glyph.x_label]
    return _results(plan, head, coords, dims, dict(x_range=x_range, y_range=y_range))
