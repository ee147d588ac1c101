"""Batched tile pyramid: every tile of zoom levels zmin..zmax in one pass.

A tile (z, tx, ty) of the square ``x_range`` x ``y_range`` is what the
reference's tile renderer obtains with one Canvas call per tile
(datashader/tiles.py:70-130 drives ``Canvas.points`` per tile):

    Canvas(ts, ts, x_range=tile_range(z, tx, *x_range),
           y_range=tile_range(z, ty, *y_range)).points(df, 'x', 'y', count() / max('v'))

``TilePyramid`` computes all of them with ``dsgb_pyramid`` (one persistent
render launch behind a bucketing pass), replayed from a CUDA graph, with
the shared-memory tile size, CTA size and chunk length picked by
:func:`autotune`.
"""
from __future__ import annotations

import ctypes
import itertools

import torch

from . import _native as N
from .core import dsgb_dtype


def tile_range(z, t, a0, a1):
    """The float64 data range of tile t at zoom z: the formula both sides use."""
    span = a1 - a0
    return (a0 + span * (t / 2 ** z), a0 + span * ((t + 1) / 2 ** z))


def level_offset(zmin, z, ts):
    return sum((1 << (2 * k)) * ts * ts for k in range(zmin, z))


DEFAULT_CONFIG = {"split": 0, "threads": 1024, "chunk": 65536}
CANDIDATES = [dict(split=s, threads=t, chunk=c)
              for s, t, c in itertools.product((0, 1), (512, 1024), (16384, 65536, 262144))]

_tuned = {}


class TilePyramid:
    """count (uint32) and, with ``v``, max(v) (float64) for every tile."""

    def __init__(self, x, y, v=None, *, zmin=0, zmax=6, tile_size=256, x_range=(0.0, 1.0),
                 y_range=(0.0, 1.0), config=None, graph=True, capacity_shift=0):
        """``capacity_shift`` k renders with 1/2^k of the workspace's edge
        queue and partial-slot capacities (DSGB_PYRAMID_CAP_SHIFT); a render
        that overflows them is incomplete and :meth:`check` raises."""
        if not 0 <= int(capacity_shift) <= 31:
            raise ValueError("capacity_shift must be in 0..31")
        self._flags = int(capacity_shift) << 8
        for t in (x, y) + ((v,) if v is not None else ()):
            if not (t.is_cuda and t.dtype == torch.float32 and t.dim() == 1 and t.is_contiguous()):
                raise TypeError("x, y and v must be contiguous 1-D float32 CUDA tensors")
        self.x, self.y, self.v = x, y, v
        self.n = x.numel()
        self.zmin, self.zmax, self.ts = zmin, zmax, tile_size
        self.x_range, self.y_range = tuple(map(float, x_range)), tuple(map(float, y_range))
        self.device = x.device
        ncells = level_offset(zmin, zmax + 1, tile_size)
        self.counts = torch.empty(ncells, dtype=torch.int32, device=self.device).view(torch.uint32)
        self.max = torch.empty(ncells, dtype=torch.float64, device=self.device) if v is not None else None
        self._cols = (N.Column * 3)(N.Column(x.data_ptr(), dsgb_dtype(x), 0),
                                    N.Column(y.data_ptr(), dsgb_dtype(y), 0),
                                    N.Column(v.data_ptr() if v is not None else 0, N.F32, 0))
        self._graph = None
        self._use_graph = graph
        self.set_config(config or DEFAULT_CONFIG)

    # ---- configuration and launch
    def _cfg(self, c):
        return N.PyramidConfig(self.zmin, self.zmax, self.ts, int(c["split"]), int(c["threads"]), int(c["chunk"]),
                               self.x_range[0], self.x_range[1], self.y_range[0], self.y_range[1])

    def set_config(self, config):
        self.config = dict(config)
        self._c = self._cfg(self.config)
        L = N.lib()
        size = int(L.dsgb_pyramid_workspace_size(self.n, int(self.v is not None), ctypes.byref(self._c)))
        if size == 0:
            raise ValueError(f"unsupported pyramid configuration {self.config} for zmax={self.zmax}, "
                             f"tile_size={self.ts}")
        self.workspace = torch.empty(size, dtype=torch.uint8, device=self.device)
        self._graph = None

    def _launch(self, stream):
        L = N.lib()
        N.check(L.dsgb_pyramid(self._cols, 3, self.n, 0, 1, 2 if self.v is not None else -1, ctypes.byref(self._c),
                               self.counts.data_ptr(), self.max.data_ptr() if self.max is not None else None,
                               self.workspace.data_ptr(), self.workspace.numel(), self._flags, stream.cuda_stream),
                "dsgb_pyramid")

    def _capture(self):
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self._launch(s)                    # eager warm-up: one-time device setup happens here
        torch.cuda.current_stream(self.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
            self._launch(s)
        self._graph = g

    def render(self):
        """Render every tile (asynchronous on the current stream)."""
        if self._use_graph:
            if self._graph is None:
                self._capture()
            self._graph.replay()
        else:
            self._launch(torch.cuda.current_stream(self.device))
        return self

    def status(self):
        """0 when the last render is complete (synchronises)."""
        flags = ctypes.c_uint32(0)
        N.check(N.lib().dsgb_pyramid_status(self.workspace.data_ptr(), self.n, int(self.v is not None),
                                            ctypes.byref(self._c), ctypes.byref(flags),
                                            torch.cuda.current_stream(self.device).cuda_stream),
                "dsgb_pyramid_status")
        return flags.value

    def check(self):
        f = self.status()
        if f:
            raise N.DsgbError(f"dsgb_pyramid: incomplete render (status flags {f:#x})")
        return self

    # ---- results
    def tile(self, z, tx, ty):
        """(count [ts, ts] uint32, max [ts, ts] float64 or None) of tile (z, tx, ty)."""
        if not (self.zmin <= z <= self.zmax and 0 <= tx < (1 << z) and 0 <= ty < (1 << z)):
            raise IndexError((z, tx, ty))
        ts = self.ts
        o = level_offset(self.zmin, z, ts) + ((ty << z) + tx) * ts * ts
        c = self.counts[o:o + ts * ts].view(ts, ts)
        m = self.max[o:o + ts * ts].view(ts, ts) if self.max is not None else None
        return c, m

    def tile_ranges(self, z, tx, ty):
        return tile_range(z, tx, *self.x_range), tile_range(z, ty, *self.y_range)


def autotune(pyr, candidates=None, repeats=3):
    """Pick the fastest configuration for this pyramid's data (CUDA-event
    timing of eager launches); cached by the pyramid's shape and data size."""
    key = (pyr.n, pyr.zmin, pyr.zmax, pyr.ts, pyr.v is not None, pyr.x_range, pyr.y_range)
    if key in _tuned:
        pyr.set_config(_tuned[key][0])
        return _tuned[key]
    stream = torch.cuda.current_stream(pyr.device)
    results = []
    for c in candidates or CANDIDATES:
        try:
            pyr.set_config(c)
        except ValueError:
            continue
        pyr._launch(stream)                    # warm-up
        times = []
        for _ in range(repeats):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            pyr._launch(stream)
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        results.append((min(times), c))
    results.sort(key=lambda r: r[0])
    best = results[0][1]
    pyr.set_config(best)
    _tuned[key] = (best, results)
    return _tuned[key]
