"""Viewport request loop over a resident, spatially bucketed point store.

Serving model: the points stay in HBM, regrouped by a grid of buckets
(:class:`BucketedStore`, ``dsgb_bucket_sort``).  A request is a viewport
(x/y ranges), a canvas size and a reduction; it aggregates only the bucket
rows its viewport overlaps (``dsgb_points_segments``), with the same
binning and reductions as ``Canvas.points`` on the whole frame.

:class:`ViewportServer` runs requests with continuous batching: arrivals
join a FIFO queue; the head is admitted as soon as a stream slot is free
and its aggregate buffers fit in the memory budget; admitted requests run
concurrently on their own CUDA streams; completions are polled without
blocking, so slots and memory are reused at once.  Latency is measured
from a request's arrival to the host observing its completion event.
"""
from __future__ import annotations

import collections
import ctypes
import math
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from . import reductions as rd
from .compiler import compile_plan
from .core import Canvas, Executor, TensorFrame, _results, dsgb_dtype
from .glyphs import Point


# --------------------------------------------------------------- segments

def viewport_segments(starts, grid, domain, x_range, y_range):
    """Row segments [begin, end) of a bucketed store that hold every point of
    the viewport: the overlapped bucket rows, widened by one bucket on each
    side (bucket ids are estimates), merged where contiguous, plus the
    bucket of points outside the domain."""
    x0, x1, y0, y1 = domain
    segs = []
    lo_x, hi_x = max(x_range[0], x0), min(x_range[1], x1)
    lo_y, hi_y = max(y_range[0], y0), min(y_range[1], y1)
    if lo_x <= hi_x and lo_y <= hi_y:
        def cell(v, a0, a1):
            c = (v - a0) / (a1 - a0) * grid
            return int(math.floor(c)) if math.isfinite(c) else 0
        bx0 = max(0, cell(lo_x, x0, x1) - 1)
        bx1 = min(grid - 1, cell(hi_x, x0, x1) + 1)
        by0 = max(0, cell(lo_y, y0, y1) - 1)
        by1 = min(grid - 1, cell(hi_y, y0, y1) + 1)
        for by in range(by0, by1 + 1):
            b, e = int(starts[by * grid + bx0]), int(starts[by * grid + bx1 + 1])
            if e <= b:
                continue
            if segs and segs[-1][1] == b:
                segs[-1] = (segs[-1][0], e)
            else:
                segs.append((b, e))
    ob, oe = int(starts[grid * grid]), int(starts[grid * grid + 1])
    if oe > ob:
        if segs and segs[-1][1] == ob:
            segs[-1] = (segs[-1][0], oe)
        else:
            segs.append((ob, oe))
    return segs


class BucketedStore:
    """Every column of ``frame`` regrouped by a ``grid`` x ``grid`` bucketing
    of ``domain`` = (x0, x1, y0, y1), resident on the frame's device."""

    def __init__(self, frame, x="x", y="y", grid=128, domain=None, stream=None):
        names = [x, y] + [c for c in frame.columns if c not in (x, y)]
        tensors = [frame[c] for c in names]
        dev = frame.device
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        if domain is None:
            xs, ys = frame[x], frame[y]
            domain = (float(torch.nan_to_num(xs, nan=math.inf).min()), float(torch.nan_to_num(xs, nan=-math.inf).max()),
                      float(torch.nan_to_num(ys, nan=math.inf).min()), float(torch.nan_to_num(ys, nan=-math.inf).max()))
            if not (domain[1] > domain[0]):
                domain = (domain[0], domain[0] + 1.0, domain[2], domain[3])
            if not (domain[3] > domain[2]):
                domain = (domain[0], domain[1], domain[2], domain[2] + 1.0)
        self.domain = tuple(float(d) for d in domain)
        self.grid = grid
        self.x, self.y = x, y
        # the sort runs on `stream`: it waits for the work that produced the
        # columns and the buffers (allocated on the current stream), and the
        # buffers are marked as used on `stream` for the caching allocator
        cur = torch.cuda.current_stream(dev)
        out = [torch.empty_like(t) for t in tensors]
        starts = torch.empty(grid * grid + 2, dtype=torch.int64, device=dev)
        L = N.lib()
        ws_size = int(L.dsgb_bucket_sort_workspace_size(grid))
        ws = torch.empty(ws_size, dtype=torch.uint8, device=dev)
        if stream != cur:
            stream.wait_stream(cur)
            for t in out + [starts, ws] + tensors:
                t.record_stream(stream)
        cols = (N.Column * len(tensors))(*[N.Column(t.data_ptr(), dsgb_dtype(t), 0) for t in tensors])
        outs = (ctypes.c_void_p * len(out))(*[t.data_ptr() for t in out])
        dom = (ctypes.c_double * 4)(*self.domain)
        N.check(L.dsgb_bucket_sort(cols, len(tensors), len(frame), 0, 1, dom, grid, outs, starts.data_ptr(),
                                   ws.data_ptr(), ws_size, stream.cuda_stream), "dsgb_bucket_sort")
        cats = {c: frame.categories(c) for c in names if frame.is_categorical(c)}
        self.frame = TensorFrame(dict(zip(names, out)), categories=cats, device=dev)
        stream.synchronize()                   # the bucket offsets are read on the host
        self.starts = starts.cpu().numpy()
        self.n = len(frame)

    def segments(self, x_range, y_range):
        return viewport_segments(self.starts, self.grid, self.domain, x_range, y_range)


# --------------------------------------------------------------- requests

REDUCTIONS = ("count", "mean", "max", "by")


def make_agg(kind, value="v", cat="cat"):
    if kind == "count":
        return rd.count()
    if kind == "mean":
        return rd.mean(value)
    if kind == "max":
        return rd.max(value)
    if kind == "by":
        return rd.by(cat, rd.count())
    raise ValueError(kind)


@dataclass
class Request:
    rid: int
    arrival: float                    # seconds after the start of the run
    x_range: tuple
    y_range: tuple
    width: int
    height: int
    kind: str
    # filled in by the server
    admitted: float = math.nan
    done: float = math.nan
    rows: int = 0
    result: object = None
    segments: object = None

    @property
    def latency(self):
        return self.done - self.arrival


CANVAS_SIZES = ((256, 256), (512, 512), (1024, 1024), (1920, 1080), (4096, 2160))


def generate_requests(n, rate, seed=0, domain=(0.0, 1.0, 0.0, 1.0), zoom=(1.0, 1000.0)):
    """Poisson arrivals at ``rate`` req/s; zoom log-uniform; random pan inside
    the domain; canvas size and reduction drawn uniformly."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=n)
    arrivals = np.cumsum(gaps) - gaps[0]
    x0, x1, y0, y1 = domain
    reqs = []
    for i in range(n):
        z = math.exp(rng.uniform(math.log(zoom[0]), math.log(zoom[1])))
        w, h = CANVAS_SIZES[rng.integers(len(CANVAS_SIZES))]
        ex = (x1 - x0) / z
        ey = min((y1 - y0), ex * h / w * (y1 - y0) / (x1 - x0))
        cx = rng.uniform(x0 + ex / 2, x1 - ex / 2) if ex < (x1 - x0) else (x0 + x1) / 2
        cy = rng.uniform(y0 + ey / 2, y1 - ey / 2) if ey < (y1 - y0) else (y0 + y1) / 2
        reqs.append(Request(i, float(arrivals[i]), (cx - ex / 2, cx + ex / 2), (cy - ey / 2, cy + ey / 2),
                            int(w), int(h), REDUCTIONS[rng.integers(len(REDUCTIONS))]))
    return reqs


# --------------------------------------------------------------- execution

def _itemsize(dtype):
    return torch.empty((), dtype=dtype).element_size()


class SegmentExecutor:
    """Runs one request on a stream: plan (cached per reduction), buffers,
    one dsgb_points_segments call (init + aggregate + finalize)."""

    def __init__(self, store, value="v", cat="cat"):
        self.store = store
        self.value, self.cat = value, cat
        self._plans = {}
        self._glyph = Point(store.x, store.y)
        self._cell_bytes = {}                  # reduction -> aggregate bytes a pixel
        self._row_bytes = None

    def plan(self, kind):
        p = self._plans.get(kind)
        if p is None:
            agg = make_agg(kind, self.value, self.cat)
            p = (agg, compile_plan(agg, self.store.frame))
            self._plans[kind] = p
        return p

    def work_bytes(self, req):
        """Device bytes a request touches: its rows (13 B each on the store) and
        its aggregate buffers.  Caches the request's segments."""
        wb = getattr(req, "_work_bytes", None)
        if wb is None:
            if getattr(req, "segments", None) is None:
                req.segments = self.store.segments(req.x_range, req.y_range)
                req.rows = sum(e - b for b, e in req.segments)
            if self._row_bytes is None:
                self._row_bytes = sum(self.store.frame[c].element_size() for c in self.store.frame.columns)
            wb = req._work_bytes = req.rows * self._row_bytes + self.agg_bytes(req)
        return wb

    def agg_bytes(self, req):
        """Device bytes of the request's aggregate buffers (bases + outputs)."""
        per_cell = self._cell_bytes.get(req.kind)
        if per_cell is None:
            _, plan = self.plan(req.kind)
            per_cell = 0
            for b in plan.bases:
                per_cell += b.ncat * b.words * _itemsize(b.torch_dtype)
            for _, o in plan.outputs:
                if o.fin != 0:
                    nc = plan.bases[o.b0].ncat if o.categories is not None else 1
                    per_cell += nc * _itemsize(o.dtype)
            self._cell_bytes[req.kind] = per_cell
        return req.width * req.height * per_cell

    def launch(self, req, stream, segments=None):
        agg, plan = self.plan(req.kind)
        frame = self.store.frame
        if segments is None:
            segments = getattr(req, "segments", None)
        if segments is None:
            segments = self.store.segments(req.x_range, req.y_range)
        req.rows = sum(e - b for b, e in segments)
        canvas = Canvas(req.width, req.height, req.x_range, req.y_range)
        with torch.cuda.stream(stream):
            ex = Executor(frame, plan, self._glyph)
            ex.allocate(req.height, req.width, frame.device)
            x_st = canvas.x_axis.compute_scale_and_translate(req.x_range, req.width)
            y_st = canvas.y_axis.compute_scale_and_translate(req.y_range, req.height)
            cv = N.CanvasDesc(req.width, req.height, 0, 0, x_st[0], x_st[1], y_st[0], y_st[1],
                              float(req.x_range[0]), float(req.x_range[1]),
                              float(req.y_range[0]), float(req.y_range[1]))
            nseg = len(segments)
            sb = (ctypes.c_int64 * max(1, nseg))(*[b for b, _ in segments])
            se = (ctypes.c_int64 * max(1, nseg))(*[e for _, e in segments])
            N.check(N.lib().dsgb_points_segments(ex.cols, len(ex.names), len(frame), 0, 1, ctypes.byref(cv),
                                                 ex.bases, len(plan.bases), ex.outs, ex.nouts, sb, se, nseg, 0,
                                                 stream.cuda_stream), "dsgb_points_segments")
            x_axis = canvas.x_axis.compute_index(x_st, req.width)
            y_axis = canvas.y_axis.compute_index(y_st, req.height)
            result = _results(plan, ex, {"x": x_axis, "y": y_axis}, ["y", "x"],
                              dict(x_range=req.x_range, y_range=req.y_range))
            ev = torch.cuda.Event()
            ev.record(stream)
        return ev, result

    def launch_plain(self, req, stream):
        """The reference's way: one Canvas.points call over every row."""
        agg, _ = self.plan(req.kind)
        req.rows = sum(e - b for b, e in self.store.segments(req.x_range, req.y_range))
        with torch.cuda.stream(stream):
            result = Canvas(req.width, req.height, req.x_range, req.y_range).points(
                self.store.frame, self.store.x, self.store.y, agg)
            ev = torch.cuda.Event()
            ev.record(stream)
        return ev, result


class ViewportServer:
    """Continuous batching of viewport requests over ``slots`` CUDA streams
    under a ``mem_budget`` of aggregate-buffer bytes.

    Admission: arrived requests are taken in arrival order while a slot is
    free and their aggregate buffers fit in the budget (the first request
    that does not fit waits, and so does everything behind it).  A heavy
    request (more than ``heavy_bytes`` of rows and buffers) runs only while
    fewer than ``max_heavy`` other heavy ones do (``max_heavy_backlogged``
    once more requests wait than there are slots); lighter requests behind
    it may go first, so a large viewport does not hold up small ones, and at
    light load large ones do not slow each other down by sharing the GPU.
    At light load (no more arrived requests than slots) a request of more
    than ``solo_bytes`` runs alone: it starts once the requests in flight are
    done, and only requests of at most ``tiny_bytes`` start beside it, so the
    small viewports that arrive meanwhile do not wait for it."""

    def __init__(self, executor, slots=8, mem_budget=8 << 30, device=None, streams=None,
                 heavy_bytes=256 << 20, max_heavy=1, max_heavy_backlogged=None, solo_bytes=256 << 20,
                 tiny_bytes=4 << 20):
        self.ex = executor
        self.slots = slots
        self.mem_budget = mem_budget
        self.heavy_bytes = heavy_bytes
        self.max_heavy = max_heavy
        self.solo_bytes = solo_bytes
        self.tiny_bytes = tiny_bytes
        # with more arrived requests waiting than there are slots, throughput
        # matters more than one request's latency: let heavy ones overlap
        self.max_heavy_backlogged = slots if max_heavy_backlogged is None else max_heavy_backlogged
        if streams is None:
            dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
            streams = [torch.cuda.Stream(dev) for _ in range(slots)]
        self.streams = list(streams)
        self.peak_mem = 0
        self.peak_mem_shared = 0          # peak bytes while more than one request was in flight
        self.peak_inflight = 0
        self.peak_heavy = 0

    def run(self, requests, mode="batched", keep_results=False, clock=time.perf_counter, idle=None):
        """Serve ``requests`` (sorted by arrival) in real time.

        mode: "batched" (continuous batching over all slots), "sequential"
        (the same segment kernels, one request at a time), or "plain" (one
        whole-frame Canvas.points call per request, one at a time)."""
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        nslots = self.slots if mode == "batched" else 1
        free = list(range(nslots))
        inflight = {}
        mem = 0
        t0 = clock()
        while pending or inflight:
            now = clock() - t0
            progressed = False
            for slot in list(inflight):
                req, ev, nbytes, _, _ = inflight[slot]
                if ev.query():
                    req.done = clock() - t0
                    if not keep_results:
                        req.result = None
                    del inflight[slot]
                    free.append(slot)
                    mem -= nbytes
                    progressed = True
            heavy_now = sum(1 for _, _, _, h, _ in inflight.values() if h)
            solo_now = any(so for _, _, _, _, so in inflight.values())
            backlog = 0
            while backlog < len(pending) and pending[backlog].arrival <= now:
                backlog += 1
            heavy_cap = self.max_heavy if backlog <= self.slots else self.max_heavy_backlogged
            light_load = backlog <= self.slots
            k = 0
            while k < len(pending) and free and pending[k].arrival <= now:
                req = pending[k]
                if light_load and solo_now and self.ex.work_bytes(req) > self.tiny_bytes:
                    break                      # a large request runs alone at light load, but for tiny ones
                nbytes = self.ex.agg_bytes(req)
                if inflight and mem + nbytes > self.mem_budget:
                    break                      # waits for memory to free up, and so does the rest
                heavy = mode == "batched" and self.ex.work_bytes(req) > self.heavy_bytes
                if heavy and heavy_now >= heavy_cap:
                    k += 1                     # lighter requests behind it may go first
                    continue
                solo = mode == "batched" and light_load and self.ex.work_bytes(req) > self.solo_bytes
                if solo and inflight:
                    break                      # starts once those in flight are done; later arrivals wait
                del pending[k]
                slot = free.pop()
                req.admitted = clock() - t0
                if mode == "plain":
                    ev, result = self.ex.launch_plain(req, self.streams[slot])
                else:
                    ev, result = self.ex.launch(req, self.streams[slot])
                req.result = result
                inflight[slot] = (req, ev, nbytes, heavy, solo)
                solo_now = solo_now or solo
                heavy_now += heavy
                mem += nbytes
                self.peak_mem = max(self.peak_mem, mem)
                if len(inflight) > 1:
                    self.peak_mem_shared = max(self.peak_mem_shared, mem)
                self.peak_inflight = max(self.peak_inflight, len(inflight))
                self.peak_heavy = max(self.peak_heavy, heavy_now)
                progressed = True
            if not progressed:
                if idle is not None:
                    idle()
                elif pending and not inflight:
                    wait = pending[0].arrival - (clock() - t0)
                    if wait > 2e-4:
                        time.sleep(wait - 1e-4)
        return requests


def summarize(requests, wall=None):
    lat = np.array([r.latency for r in requests]) * 1e3
    first = min(r.arrival for r in requests)
    last = max(r.done for r in requests)
    span = wall if wall is not None else (last - first)
    rows = sum(r.rows for r in requests)
    return {"requests": len(requests), "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
            "req_per_s": len(requests) / span, "gpoints_per_s": rows / span / 1e9, "makespan_s": span}
