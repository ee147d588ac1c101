"""Host logic of the viewport request loop (no GPU): bucket-row segments and
the continuous-batching scheduler, driven by a fake executor and clock."""
from __future__ import annotations

import numpy as np

from datashader_gb300 import serving as S


def _starts(counts):
    return np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)


def test_segments_cover_widened_bucket_rows_and_merge():
    grid = 4
    counts = np.arange(1, grid * grid + 2)            # 16 buckets + outside
    st = _starts(counts)
    dom = (0.0, 1.0, 0.0, 1.0)
    segs = S.viewport_segments(st, grid, dom, (0.30, 0.40), (0.55, 0.60))
    # x cells 1..1 widened to 0..2, y cells 2..2 widened to 1..3; plus the outside bucket
    want = [(int(st[by * 4 + 0]), int(st[by * 4 + 3])) for by in (1, 2, 3)]
    want.append((int(st[16]), int(st[17])))
    assert segs == want
    full = S.viewport_segments(st, grid, dom, (0.0, 1.0), (0.0, 1.0))
    assert full == [(0, int(st[17]))]                  # every row: one merged segment
    outside_only = S.viewport_segments(st, grid, dom, (2.0, 3.0), (0.0, 1.0))
    assert outside_only == [(int(st[16]), int(st[17]))]
    assert sum(e - b for b, e in S.viewport_segments(_starts(np.zeros(17, int)), grid, dom,
                                                     (0, 1), (0, 1))) == 0


class _Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def idle(self):
        self.t += 1e-4


class _Event:
    def __init__(self, clock, done_at):
        self.clock, self.done_at = clock, done_at

    def query(self):
        return self.clock.t >= self.done_at


class _FakeExecutor:
    def __init__(self, clock):
        self.clock = clock
        self.running = 0
        self.max_running = 0

    def agg_bytes(self, req):
        return req.width * req.height * 4

    def work_bytes(self, req):
        return self.agg_bytes(req) * 10

    def _ev(self, req):
        dur = 1e-3 + req.width * req.height * 1e-9
        self.running_heavy = getattr(self, "running_heavy", [])
        return _Event(self.clock, self.clock.t + dur), ("result", req.rid)

    def launch(self, req, stream, segments=None):
        req.rows = 10
        return self._ev(req)

    def launch_plain(self, req, stream):
        req.rows = 10
        return self._ev(req)


def test_scheduler_admits_by_memory_and_slots_fifo():
    clock = _Clock()
    ex = _FakeExecutor(clock)
    reqs = S.generate_requests(300, rate=5000, seed=3)
    budget = 3 * 4096 * 2160 * 4
    server = S.ViewportServer(ex, slots=6, mem_budget=budget, streams=[None] * 6)
    server.run(reqs, clock=clock, idle=clock.idle, keep_results=True)
    assert all(np.isfinite(r.done) and r.done >= r.admitted >= r.arrival for r in reqs)
    assert server.peak_inflight <= 6
    assert server.peak_mem <= budget and server.peak_mem_shared <= budget
    order = sorted(reqs, key=lambda r: r.arrival)
    for heavy in (False, True):                        # FIFO within each class (lights may overtake heavies)
        adm = [r.admitted for r in order if (ex.work_bytes(r) > server.heavy_bytes) == heavy]
        assert adm == sorted(adm)
    assert all(r.result == ("result", r.rid) for r in reqs)
    stats = S.summarize(reqs)
    assert stats["requests"] == 300 and stats["p99_ms"] >= stats["p50_ms"] > 0


def test_scheduler_sequential_mode_runs_one_at_a_time():
    clock = _Clock()
    ex = _FakeExecutor(clock)
    reqs = S.generate_requests(50, rate=2000, seed=4)
    server = S.ViewportServer(ex, slots=6, mem_budget=1 << 40, streams=[None] * 6)
    server.run(reqs, mode="sequential", clock=clock, idle=clock.idle)
    assert server.peak_inflight == 1
    spans = sorted((r.admitted, r.done) for r in reqs)
    assert all(spans[i][1] <= spans[i + 1][0] for i in range(len(spans) - 1))


def test_oversized_request_runs_alone():
    clock = _Clock()
    ex = _FakeExecutor(clock)
    reqs = [S.Request(i, 0.0, (0, 1), (0, 1), 4096, 2160, "count") for i in range(3)]
    server = S.ViewportServer(ex, slots=4, mem_budget=1000, streams=[None] * 4)
    server.run(reqs, clock=clock, idle=clock.idle)
    assert server.peak_inflight == 1 and all(np.isfinite(r.done) for r in reqs)


def test_heavy_requests_run_one_at_a_time_and_lights_overtake():
    clock = _Clock()
    ex = _FakeExecutor(clock)
    big = [S.Request(i, 0.0, (0, 1), (0, 1), 4096, 2160, "by") for i in range(4)]
    small = [S.Request(100 + i, 0.0, (0, 0.01), (0, 0.01), 256, 256, "count") for i in range(20)]
    reqs = big + small                       # all arrive together, the heavy ones first
    server = S.ViewportServer(ex, slots=4, mem_budget=1 << 40, streams=[None] * 4,
                              heavy_bytes=4096 * 2160 * 4 * 5, max_heavy=1, max_heavy_backlogged=1)
    server.run(reqs, clock=clock, idle=clock.idle)
    assert server.peak_heavy == 1
    assert all(np.isfinite(r.done) for r in reqs)
    spans = sorted((r.admitted, r.done) for r in big)
    assert all(spans[i][1] <= spans[i + 1][0] for i in range(len(spans) - 1))   # heavy ones in turn
    assert max(r.done for r in small) < max(r.done for r in big)                # small ones did not wait


def test_heavy_requests_overlap_when_backlogged():
    clock = _Clock()
    ex = _FakeExecutor(clock)
    reqs = [S.Request(i, 0.0, (0, 1), (0, 1), 4096, 2160, "by") for i in range(12)]
    server = S.ViewportServer(ex, slots=4, mem_budget=1 << 40, streams=[None] * 4,
                              heavy_bytes=1, max_heavy=1)
    server.run(reqs, clock=clock, idle=clock.idle)
    assert server.peak_heavy > 1 and all(np.isfinite(r.done) for r in reqs)


def test_solo_request_at_light_load_lets_only_tiny_requests_beside_it():
    """At light load a large request runs alone, except that requests of at
    most tiny_bytes start beside it; a medium one waits for it."""
    clock = _Clock()
    ex = _FakeExecutor(clock)
    solo = S.Request(0, 0.0, (0, 1), (0, 1), 4096, 2160, "count")          # 354 MB of work: solo
    tiny = S.Request(1, 5e-4, (0, 0.01), (0, 0.01), 256, 256, "count")    # 2.6 MB: tiny
    medium = S.Request(2, 6e-4, (0, 0.1), (0, 0.1), 512, 512, "count")   # 10.5 MB: neither
    server = S.ViewportServer(ex, slots=4, mem_budget=1 << 40, streams=[None] * 4)
    server.run([solo, tiny, medium], clock=clock, idle=clock.idle)
    assert tiny.admitted < solo.done                  # did not wait for the large request
    assert medium.admitted >= solo.done               # waited
    assert all(np.isfinite(r.done) for r in (solo, tiny, medium))
