"""Benchmark: Canvas.points count (and mean) over 1e8 points at 1024x1024 on GB300.

Workload (the full-reduction-set config, 1e8 rows): x, y float32 from a
seeded 5-Gaussian mixture, v float64 ~ lognormal(0, 1), cat int8 over 8
categories; Canvas 1024x1024 over [-4, 4]^2.  One step = one
``Canvas.points(frame, 'x', 'y', ds.count())`` call through the public API
with the columns resident in HBM.  The inputs (800 MB of x/y) are larger
than L2, so no flush is needed between steps.

The JSON line also carries:
  roofline      -- the count kernel alone: algorithmic bytes (8 B/point read
                   + 4 B/pixel written) / CUDA-event kernel time vs the
                   measured HBM copy bandwidth;
  mean          -- the same for Canvas.points(..., ds.mean('v'));
  full_set      -- the whole reduction set of the config plus eq_hist;
  e2e           -- count with host (pinned) inputs: H2D of x/y, the call, D2H
                   of the aggregate, all inside the timed region;
  cpu_baseline  -- the CPU oracle (a restatement of the reference's numba
                   loop) on one host core, on a bounded sample;
  clocks        -- nvidia-smi samples taken during the timed region.

``--impl reference`` times the reference's CPU algorithm (the oracle port,
the reference itself cannot be imported on this machine) over the same
workload with all host threads: rows split into one partition per thread,
partial aggregates summed, as datashader's dask path does.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gpoints/s, Canvas.points count/mean 1e8 pts @1024²; viewport p50/p99 ms"
def workload(n):
    return (f"Canvas.points count, {n:,} float32 points (5-Gaussian mixture), "
            "1024x1024 canvas over [-4,4]^2")


# DRAM bytes (read + write) of one hot-tile count launch, measured by ncu on a
# 2e7-row launch of the same kernel (167.70 MB read, 3.51 MB written): reads
# scale with rows, writes with the touched pixels of the 1024x1024 canvas.
def count_traffic(n):
    return 167.70e6 / 2e7 * n + 3.51e6


# The same for the hot-tile mean('v') launch (x/y float32 + v float64): ncu on
# a 2e7-row launch (372.78 MB read, 3.58 MB written).
def mean_traffic(n):
    return 372.78e6 / 2e7 * n + 3.58e6


# float64 operations of the antialiased line forward per segment (adds + muls +
# 2 x fmas, lanes with the predicate on), counted by ncu on 200 series x
# 10,000 vertices of the same workload: 873.1 M operations for 1,999,800
# segments.  The work per segment does not depend on the series count.
LINE_FP64_FLOPS_PER_SEGMENT = 436.6


def fp64_peak(dev):
    """float64 FMA throughput of this GPU (TFLOP/s): the dsgb_fp64_probe
    kernel timed with CUDA events, best of 5."""
    import torch
    from datashader_gb300 import _native as N
    L = N.lib()
    stream = torch.cuda.current_stream(dev)
    sink = torch.zeros(1, dtype=torch.float64, device=dev)
    fl = ctypes.c_int64(0)

    def probe():
        N.check(L.dsgb_fp64_probe(sink.data_ptr(), 4096, 8, ctypes.byref(fl), stream.cuda_stream), "fp64 probe")

    probe()
    times = _events_time(probe, 5, stream)
    return fl.value / (min(times) / 1e3) / 1e12


def bench_config(n, world):
    """The config dict both arms print (the driver compares them)."""
    return {"workload": workload(n), "n_points": n, "canvas": [1024, 1024], "x_range": [-4, 4],
            "coords": "float32", "reduction": "count",
            "l2": "inputs (800 MB) larger than L2, no flush",
            "parallelism": "replicas" if world > 1 else "one device"}


CFG1 = {"workload": "Canvas.points count, 10,000,000 float64 points (5-Gaussian mixture), 512x512 canvas over "
                    "[-4,4]^2", "n_points": 10_000_000, "canvas": [512, 512], "coords": "float64"}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.gpu), "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def _dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(world, value):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ CPU side

def _oracle_count_threads(xs, ys, threads, width, height, x_range, y_range):
    """The reference's CPU algorithm (oracle port) over row partitions, one per thread."""
    import oracle
    n = xs.size
    bounds = np.linspace(0, n, threads + 1).astype(np.int64)
    parts = [None] * threads

    def work(k):
        a, b = bounds[k], bounds[k + 1]
        parts[k] = oracle.points({"x": xs[a:b], "y": ys[a:b]}, "x", "y", width, height,
                                 x_range, y_range, [oracle.spec("count")])[0]

    ts = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return np.sum(parts, axis=0, dtype=np.uint32)


def cpu_baseline(sample_n=20_000_000, threads=1):
    from datashader_gb300 import synthetic
    xs, ys = synthetic.gaussian_mixture_np(sample_n, seed=0, dtype=np.float32)
    _oracle_count_threads(xs[:100_000], ys[:100_000], 1, 1024, 1024, (-4, 4), (-4, 4))   # warm
    t0 = time.perf_counter()
    _oracle_count_threads(xs, ys, threads, 1024, 1024, (-4, 4), (-4, 4))
    dt = time.perf_counter() - t0
    return sample_n / dt / 1e9, dt


def _oracle_mean_threads(xs, ys, vs, threads):
    import oracle
    return oracle.points_parallel({"x": xs, "y": ys, "v": vs}, "x", "y", 1024, 1024, (-4, 4), (-4, 4),
                                  [oracle.spec("mean", "v")], threads=threads)[0]


def run_reference(args):
    """The reference's CPU algorithm (the oracle port of datashader's numba
    loop) over the same workload: float32 x/y read as float32 and widened in
    the loop as numba does, one row partition per host thread, partials
    summed as datashader's dask path does."""
    world, rank, _ = _dist_init(args)
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    from datashader_gb300 import synthetic
    n = min(args.n, args.reference_sample)
    xs, ys = synthetic.gaussian_mixture_np(n, seed=0, dtype=np.float32)

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        t0 = time.perf_counter()
        for _ in range(steps):
            fn()
        return (time.perf_counter() - t0) / steps

    dt = timed(lambda: _oracle_count_threads(xs, ys, threads, 1024, 1024, (-4, 4), (-4, 4)),
               args.steps, args.warmup)
    v = n / dt / 1e9
    extras = {}
    if args.ref_extras:
        vs = np.random.default_rng(1).lognormal(0.0, 1.0, n)
        mdt = timed(lambda: _oracle_mean_threads(xs, ys, vs, threads), max(1, args.steps // 4), 1)
        extras["mean"] = {"value": n / mdt / 1e9, "unit": "Gpoints/s", "ms_per_step": mdt * 1e3}
        del vs
        x1, y1 = synthetic.gaussian_mixture_np(CFG1["n_points"], seed=0, dtype=np.float64)
        cdt = timed(lambda: _oracle_count_threads(x1, y1, threads, 512, 512, (-4, 4), (-4, 4)),
                    max(1, args.steps // 4), 1)
        extras["cfg1"] = dict(CFG1, value=CFG1["n_points"] / cdt / 1e9, unit="Gpoints/s", ms_per_step=cdt * 1e3)
    sample = (f"all {n:,} rows of the workload per step (float32 x/y), {threads} threads, one row partition "
              "per thread")
    line = {"metric": METRIC, "value": v, "unit": "Gpoints/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": bench_config(n, world),
            "cpu_baseline": {"value": v, "unit": "Gpoints/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "Gpoints/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "datashader cannot be imported here (numba/pandas/xarray absent): the timed CPU "
                    "implementation is the C restatement of its numba CPU loop (oracle/)"}
    line.update(extras)
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ GPU side

def _events_time(fn, k, stream):
    import torch
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
    for i in range(k):
        starts[i].record(stream)
        fn()
        ends[i].record(stream)
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in zip(starts, ends)]


def bench_pyramid(args, dev, peak, peak_kind):
    """The tile-pyramid workload: 2e8 float32 points in [0,1)^2 (half uniform,
    half 20 Gaussians), v float32 ~ N(0,1), zoom 0-6 of 256x256 tiles (5,461
    tiles), count and max(v), one graph replay per pyramid; against one plain
    Canvas.points call per tile (timed on a sample of tiles, scaled to 5,461)."""
    import torch
    import datashader_gb300 as ds
    from datashader_gb300 import pyramid as P
    from datashader_gb300 import synthetic
    n = args.pyramid_n
    stream = torch.cuda.current_stream(dev)
    x, y = synthetic.pyramid_points_torch(n, seed=0, device=dev)
    g = torch.Generator(device=dev)
    g.manual_seed(1)
    v = torch.randn(n, generator=g, device=dev, dtype=torch.float32)
    pyr = P.TilePyramid(x, y, v, zmin=0, zmax=6, tile_size=256)
    if args.pyramid_config:
        sp, th, ch = (int(t) for t in args.pyramid_config.split(","))
        best = dict(split=sp, threads=th, chunk=ch)
        pyr.set_config(best)
        results = []
    else:
        best, results = P.autotune(pyr, repeats=2)
    pyr.render()
    torch.cuda.synchronize()
    status = pyr.status()
    times = _events_time(pyr.render, max(3, args.steps // 2), stream)
    ms = sum(times) / len(times)
    frame = ds.TensorFrame({"x": x, "y": y, "v": v})
    agg = ds.summary(count=ds.count(), max=ds.max("v"))
    rng = np.random.default_rng(0)
    tiles = [(z, int(rng.integers(0, 1 << z)), int(rng.integers(0, 1 << z))) for z in range(7) for _ in range(2)]

    def plain(z, tx, ty):
        xr, yr = pyr.tile_ranges(z, tx, ty)
        return ds.Canvas(plot_width=256, plot_height=256, x_range=xr, y_range=yr).points(frame, "x", "y", agg)

    plain(*tiles[0])
    per_tile = _events_time(lambda: [plain(*t) for t in tiles], 1, stream)[0] / len(tiles)
    same = True
    for t in tiles:
        r = plain(*t)
        c, m = pyr.tile(*t)
        same &= bool(torch.equal(r["count"].data.view(torch.int32), c.view(torch.int32)))
        same &= bool(torch.equal(torch.nan_to_num(r["max"].data, nan=-1e300), torch.nan_to_num(m, nan=-1e300)))
    ntiles = sum(4 ** z for z in range(7))
    out_bytes = pyr.counts.numel() * 4 + pyr.max.numel() * 8
    alg = n * 12 + out_bytes
    achieved = alg / (ms / 1e3) / 1e9
    res = {"workload": f"tile pyramid zoom 0-6, 256x256 tiles ({ntiles}), {n:,} float32 points, count + max(v)",
           "ms_per_pyramid": ms, "gpoints_per_s": n / (ms / 1e3) / 1e9, "status_flags": status,
           "autotuned": best, "candidates": [[round(t, 4), c] for t, c in results],
           "plain_ms_per_tile": per_tile, "plain_ms_per_pyramid_est": per_tile * ntiles,
           "speedup_vs_plain": per_tile * ntiles / ms, "sample_tiles_identical": same,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "peak_kind": peak_kind,
                        "algorithmic_bytes": alg, "note": "12 B/point read + count/max tiles written once"},
           "gpu_launches_per_pyramid": 8}
    del pyr, x, y, v, frame
    torch.cuda.empty_cache()
    return res


def _line_roofline(nseg, f_ms, dev):
    peak = fp64_peak(dev)
    achieved = LINE_FP64_FLOPS_PER_SEGMENT * nseg / (f_ms / 1e3) / 1e12
    return {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_kind": "measured (dsgb_fp64_probe, float64 FMA chains)", "traffic": None,
            "flops_per_segment": LINE_FP64_FLOPS_PER_SEGMENT}


def bench_line(args, dev):
    """The differentiation workload: Canvas.line (LineAxis0, line_width 1.5,
    antialiased) of 1000 series x 10,000 float64 vertices (NaN separators,
    10,010,000 rows) on 1024x512, sum('v'); y autoranged.  Forward alone, and
    forward + backward of the MSE against the same series with y + N(0, 0.005)
    through the hand-written adjoint (gradients w.r.t. v and y)."""
    import torch
    import datashader_gb300 as ds
    from datashader_gb300 import autograd as ag
    from datashader_gb300 import synthetic
    nseries, length = args.line_series, 10_000
    x, y, v, _ = synthetic.time_series_np(nseries, length, seed=0)
    rng = np.random.default_rng(1)
    y_t = y + rng.normal(0.0, 0.005, y.shape)
    X, Y, V = (torch.from_numpy(a).to(dev) for a in (x, y, v))
    YT = torch.from_numpy(y_t).to(dev)
    stream = torch.cuda.current_stream(dev)
    frame = ds.TensorFrame({"x": X, "y": Y, "v": V})
    cvs = ds.Canvas(plot_width=1024, plot_height=512, x_range=(0.0, 1.0))

    def fwd():
        return cvs.line(frame, "x", "y", agg=ds.sum("v"), line_width=1.5)

    agg = fwd()
    y_range = tuple(agg.attrs["y_range"])
    fixed = ds.Canvas(plot_width=1024, plot_height=512, x_range=(0.0, 1.0), y_range=y_range)
    target = torch.nan_to_num(ag.line_sum(X, YT, V, fixed)).detach()
    for _ in range(2):
        fwd()
    f_ms = _events_time(fwd, max(3, args.steps // 2), stream)
    f_ms = sum(f_ms) / len(f_ms)
    Yg = Y.clone().requires_grad_(True)
    Vg = V.clone().requires_grad_(True)

    def step():
        Yg.grad = None
        Vg.grad = None
        loss = torch.mean((torch.nan_to_num(ag.line_sum(X, Yg, Vg, fixed)) - target) ** 2)
        loss.backward()

    for _ in range(2):
        step()
    fb_ms = _events_time(step, max(3, args.steps // 2), stream)
    fb_ms = sum(fb_ms) / len(fb_ms)
    nseg = nseries * (length - 1)
    # the oracle (the reference's CPU line loop) on a bounded sample of the series, one thread
    import oracle
    ns = max(1, min(nseries, args.line_cpu_series))
    rows = ns * (length + 1)
    t0 = time.perf_counter()
    oracle.line_axis0({"x": x[:rows], "y": y[:rows], "v": v[:rows]}, "x", "y", 1024, 512, (0.0, 1.0), y_range,
                      [oracle.spec("sum", "v")], line_width=1.5)
    cpu_s = time.perf_counter() - t0
    res = {"workload": f"Canvas.line LineAxis0 AA lw=1.5, {nseries} series x {length} float64 vertices, "
                       "1024x512, sum('v')",
           "forward_ms": f_ms, "forward_gsegments_per_s": nseg / (f_ms / 1e3) / 1e9,
           "roofline": _line_roofline(nseg, f_ms, dev),
           "forward_backward_ms": fb_ms,
           "cpu_baseline": {"value": ns * (length - 1) / cpu_s / 1e9, "unit": "Gsegments/s", "cores": 1,
                            "kind": "port", "sample": f"{ns} series, one thread, {cpu_s:.2f} s"},
           "gpu_launches_forward": 3, "gpu_launches_forward_backward": 4}
    del X, Y, V, YT, frame, Yg, Vg, target
    torch.cuda.empty_cache()
    return res


def bench_serving(args, dev):
    """The viewport workload: 5e8 points resident (float32 x/y of the pyramid
    distribution, float32 v ~ N(0,1), uint8 cat over 16), Poisson arrivals at
    200 / 1,000 / 5,000 req/s, zoom log-uniform 1x-1000x, random pan, canvas
    from {256^2, 512^2, 1024^2, 1920x1080, 4096x2160}, reduction from {count,
    mean(v), max(v), by(cat, count)}; continuous batching vs the same segment
    kernels one request at a time vs a plain whole-frame Canvas.points call
    per request, one at a time."""
    import torch
    import datashader_gb300 as ds
    from datashader_gb300 import serving as S
    from datashader_gb300 import synthetic
    n = args.serving_n
    x, y = synthetic.pyramid_points_torch(n, seed=3, device=dev)
    g = torch.Generator(device=dev)
    g.manual_seed(4)
    v = torch.randn(n, generator=g, device=dev, dtype=torch.float32)
    cat = torch.randint(0, 16, (n,), generator=g, device=dev, dtype=torch.uint8)
    frame = ds.TensorFrame({"x": x, "y": y, "v": v, "cat": cat}, categories={"cat": list(range(16))})
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    store = S.BucketedStore(frame, grid=128, domain=(0.0, 1.0, 0.0, 1.0))
    torch.cuda.synchronize()
    sort_s = time.perf_counter() - t0
    del frame, x, y, v, cat
    torch.cuda.empty_cache()
    ex = S.SegmentExecutor(store)
    server = S.ViewportServer(ex, slots=args.serving_slots, mem_budget=args.serving_mem_gb << 30)
    warm = S.generate_requests(40, rate=1e6, seed=99)
    server.run(warm)
    server.run([S.Request(r.rid, 0.0, r.x_range, r.y_range, r.width, r.height, r.kind) for r in warm[:8]],
               mode="plain")
    torch.cuda.synchronize()
    out = {"workload": f"{n:,} resident points (13 B/point), {args.serving_requests} requests per rate",
           "store_sort_ms": sort_s * 1e3, "slots": args.serving_slots, "mem_budget_gb": args.serving_mem_gb,
           "rates": {}}
    for rate in (int(r) for r in args.serving_rates.split(",")):
        per = {}
        for mode in args.serving_modes.split(","):
            nreq = args.serving_requests if mode != "plain" else min(args.serving_requests, args.serving_plain_requests)
            reqs = S.generate_requests(nreq, rate=rate, seed=rate)
            server.peak_inflight = 0
            server.run(reqs, mode=mode)
            torch.cuda.synchronize()
            st = S.summarize(reqs)
            st["peak_inflight"] = server.peak_inflight
            per[mode] = {k: (round(v, 4) if isinstance(v, float) else v) for k, v in st.items()}
        out["rates"][str(rate)] = per
    del store, ex, server
    torch.cuda.empty_cache()
    return out


def run_gpu(args):
    import torch
    world, rank, local = _dist_init(args)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import datashader_gb300 as ds
    from datashader_gb300 import _native as N
    from datashader_gb300 import synthetic
    from datashader_gb300.compiler import compile_plan
    from datashader_gb300.core import Executor, dsgb_dtype
    from datashader_gb300.glyphs import Point

    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    n = args.n
    x, y = synthetic.gaussian_mixture_torch(n, seed=rank, device=dev)
    v = synthetic.lognormal_torch(n, seed=100 + rank, device=dev)
    cat = synthetic.categories_torch(n, 8, seed=200 + rank, device=dev)
    frame = ds.TensorFrame({"x": x, "y": y, "v": v, "cat": cat}, categories={"cat": list(range(8))})
    cvs = ds.Canvas(plot_width=1024, plot_height=1024, x_range=(-4, 4), y_range=(-4, 4))
    peak, peak_kind = measured_peak()

    def step_count():
        return cvs.points(frame, "x", "y", ds.count())

    # ---- headline: count through the public API, inputs resident in HBM
    for _ in range(args.warmup):
        step_count()
    torch.cuda.synchronize()
    _barrier(world)
    with ClockSampler(local) as clk:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t_start.record(stream)
        for _ in range(args.steps):
            step_count()
        t_end.record(stream)
        torch.cuda.synchronize()
        elapsed_ms = t_start.elapsed_time(t_end)
    _barrier(world)
    elapsed_ms = _max_over_ranks(world, elapsed_ms)
    value = n * world * args.steps / (elapsed_ms / 1e3) / 1e9

    # ---- kernel-only timing for the roofline (count and mean kernels)
    def kernel_runner(agg):
        plan = compile_plan(agg, frame)
        ex = Executor(frame, plan, Point("x", "y"))
        ex.allocate(1024, 1024, dev)
        x_st = cvs.x_axis.compute_scale_and_translate((-4, 4), 1024)
        y_st = cvs.y_axis.compute_scale_and_translate((-4, 4), 1024)
        cv = N.CanvasDesc(1024, 1024, 0, 0, x_st[0], x_st[1], y_st[0], y_st[1], -4.0, 4.0, -4.0, 4.0)
        L = N.lib()
        N.check(L.dsgb_bases_init(ex.bases, len(plan.bases), 1024 * 1024, stream.cuda_stream), "init")

        wsz = int(L.dsgb_points_workspace_size(n, ctypes.byref(cv), ex.bases, len(plan.bases)))
        ws = torch.empty(max(wsz, 1), dtype=torch.uint8, device=dev)

        def launch():
            N.check(L.dsgb_points_ws(ex.cols, len(ex.names), n, 0, 0, 1, ctypes.byref(cv), ex.bases,
                                     len(plan.bases), ex.outs, 0, ws.data_ptr() if wsz else None, wsz,
                                     N.FLAG_NO_INIT | N.FLAG_NO_FINALIZE, stream.cuda_stream), "dsgb_points_ws")
        return launch

    def roofline(agg, bytes_per_point, bytes_per_pixel, k, traffic=None):
        launch = kernel_runner(agg)
        for _ in range(3):
            launch()
        times = _events_time(launch, k, stream)
        avg_ms = sum(times) / len(times)
        alg = n * bytes_per_point + 1024 * 1024 * bytes_per_pixel
        achieved = alg / (avg_ms / 1e3) / 1e9
        return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": alg, "kernel_ms": avg_ms,
                "kernel_gpts": n / (avg_ms / 1e3) / 1e9}

    rl_count = roofline(ds.count(), 8, 4, args.steps, traffic=count_traffic(n))
    # kernels of one count call: the hot-tile kernel (the output is cleared by
    # cudaMemsetAsync, not a kernel of this library)
    kernels_per_count = 1
    rl_mean = roofline(ds.mean("v"), 16, 12, args.steps, traffic=mean_traffic(n))

    # mean through the public API
    for _ in range(2):
        cvs.points(frame, "x", "y", ds.mean("v"))
    mean_ms = _events_time(lambda: cvs.points(frame, "x", "y", ds.mean("v")), args.steps, stream)
    mean_ms = sum(mean_ms) / len(mean_ms)

    # the whole reduction set of the config + eq_hist on the count
    full = ds.summary(count=ds.count(), sum=ds.sum("v"), mean=ds.mean("v"), max=ds.max("v"),
                      min=ds.min("v"), first=ds.first("v"), where=ds.where(ds.max("v")),
                      by_cat=ds.by("cat", ds.count()))

    def step_full():
        a = cvs.points(frame, "x", "y", full)
        ds.tf.shade(a["count"], how="eq_hist")

    step_full()
    full_ms = _events_time(step_full, max(2, args.steps // 4), stream)
    full_ms = sum(full_ms) / len(full_ms)

    # ---- e2e: host (pinned) inputs -> H2D -> Canvas.points -> D2H, per step.  The
    # public API streams a HostFrame: every step copies all x/y rows to the GPU in
    # chunks (a copy stream) while the previous chunk aggregates, and reads the
    # aggregate back.  The copy-everything-then-aggregate form is timed beside it.
    xh = x.cpu().pin_memory()
    yh = y.cpu().pin_memory()
    hframe = ds.HostFrame({"x": xh, "y": yh})
    xd = torch.empty_like(x)
    yd = torch.empty_like(y)

    def step_e2e():
        return cvs.points(hframe, "x", "y", ds.count()).data.cpu()

    def step_copy_then_compute():
        xd.copy_(xh, non_blocking=True)
        yd.copy_(yh, non_blocking=True)
        return cvs.points(ds.TensorFrame({"x": xd, "y": yd}), "x", "y", ds.count()).data.cpu()

    def _wall(step):
        for _ in range(2):
            step()
        torch.cuda.synchronize()
        _barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        torch.cuda.synchronize()
        return _max_over_ranks(world, time.perf_counter() - t0)

    e2e_s = _wall(step_e2e)
    ctc_s = _wall(step_copy_then_compute)
    e2e = {"value": n * world * args.steps / e2e_s / 1e9, "unit": "Gpoints/s",
           "h2d_bytes_per_step": int(xh.numel() * 4 + yh.numel() * 4),
           "d2h_bytes_per_step": 1024 * 1024 * 4,
           "path": f"HostFrame streamed in chunks of {hframe.chunk_rows} rows",
           "copy_then_compute_gpoints_per_s": n * world * args.steps / ctc_s / 1e9}

    # ---- parity of the timed workload (untimed): the 1e8-row count against the
    # oracle on every host thread, bit for bit
    parity = None
    if rank == 0 and args.parity:
        import oracle
        got = step_count().data.view(torch.int32).cpu().numpy().view(np.uint32)
        t0 = time.perf_counter()
        ref = oracle.points_parallel({"x": xh.numpy(), "y": yh.numpy()}, "x", "y", 1024, 1024, (-4, 4), (-4, 4),
                                     [oracle.spec("count")])[0]
        parity = {"count_bit_exact_vs_oracle": bool(np.array_equal(got, ref)), "rows": n,
                  "oracle_threads": os.cpu_count() or 1, "oracle_s": round(time.perf_counter() - t0, 3)}

    del x, y, v, cat, frame, xh, yh, xd, yd, hframe
    torch.cuda.empty_cache()

    # ---- the 1e7 float64 512^2 count configuration
    cfg1 = None
    if args.cfg1:
        n1 = CFG1["n_points"]
        x1, y1 = synthetic.gaussian_mixture_torch(n1, seed=rank, dtype=torch.float64, device=dev)
        f1 = ds.TensorFrame({"x": x1, "y": y1})
        c1 = ds.Canvas(plot_width=512, plot_height=512, x_range=(-4, 4), y_range=(-4, 4))
        for _ in range(3):
            c1.points(f1, "x", "y", ds.count())
        t1 = _events_time(lambda: c1.points(f1, "x", "y", ds.count()), args.steps, stream)
        ms1 = sum(t1) / len(t1)
        alg1 = n1 * 16 + 512 * 512 * 4
        cfg1 = dict(CFG1, value=n1 / (ms1 / 1e3) / 1e9, unit="Gpoints/s", ms_per_step=ms1,
                    roofline={"bound": "hbm", "achieved": alg1 / (ms1 / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                              "frac": alg1 / (ms1 / 1e3) / 1e9 / peak, "peak_kind": peak_kind,
                              "algorithmic_bytes_per_step": alg1,
                              "note": "16 B/point (x, y float64) + 4 B/pixel, public API call time"})
        if rank == 0 and not args.no_cpu_baseline:
            import oracle
            xn, yn = x1.cpu().numpy(), y1.cpu().numpy()
            t0 = time.perf_counter()
            r1 = oracle.points({"x": xn, "y": yn}, "x", "y", 512, 512, (-4, 4), (-4, 4), [oracle.spec("count")])[0]
            dt1 = time.perf_counter() - t0
            cfg1["cpu_baseline"] = {"value": n1 / dt1 / 1e9, "unit": "Gpoints/s", "cores": 1, "kind": "port",
                                    "sample": f"all {n1:,} rows, one thread, {dt1:.2f} s"}
            g1 = c1.points(f1, "x", "y", ds.count()).data.view(torch.int32).cpu().numpy().view(np.uint32)
            cfg1["count_bit_exact_vs_oracle"] = bool(np.array_equal(g1, r1))
        del x1, y1, f1
        torch.cuda.empty_cache()
    extras = {}
    if world == 1 and args.pyramid_n > 0:
        extras["pyramid"] = bench_pyramid(args, dev, peak, peak_kind)
    if world == 1 and args.line_series > 0:
        extras["line"] = bench_line(args, dev)
    if world == 1 and args.serving_n > 0 and args.serving_requests > 0:
        extras["serving"] = bench_serving(args, dev)

    if rank == 0:
        base = None
        if world == 1 and not args.no_cpu_baseline:
            gpts, dt = cpu_baseline(args.cpu_sample)
            base = {"value": gpts, "unit": "Gpoints/s", "cores": 1, "kind": "port",
                    "sample": f"{args.cpu_sample} rows of the same distribution, count, one thread, "
                              f"{dt:.2f} s"}
            nth = os.cpu_count() or 1
            if nth > 1:      # the same sample over one row partition per host thread
                g_all, dt_all = cpu_baseline(args.cpu_sample, threads=nth)
                base["all_threads"] = {"value": g_all, "unit": "Gpoints/s", "cores": nth,
                                       "sample": f"the same rows, {nth} threads, {dt_all:.2f} s"}
        line = {
            "metric": METRIC, "value": value, "unit": "Gpoints/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": bench_config(n, world),
            "roofline": {k: rl_count[k] for k in ("bound", "achieved", "peak", "unit", "frac", "traffic")},
            "roofline_detail": rl_count,
            "mean": {"value": n / (mean_ms / 1e3) / 1e9, "unit": "Gpoints/s", "ms_per_step": mean_ms,
                     "roofline": rl_mean},
            "full_set": {"ms_per_step": full_ms, "value": n / (full_ms / 1e3) / 1e9, "unit": "Gpoints/s",
                         "reductions": "count,sum,mean,max,min,first,where(max),by(cat,count) + eq_hist"},
            "cpu_baseline": base,
            "e2e": e2e,
            "parity": parity,
            "cfg1": cfg1,
            "gpu_launches": args.steps * kernels_per_count,
            "clocks": clk.summary(),
        }
        line.update(extras)
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=100_000_000)
    ap.add_argument("--cpu-sample", type=int, default=20_000_000)
    ap.add_argument("--reference-sample", type=int, default=100_000_000)
    ap.add_argument("--ref-extras", type=int, default=1, help="reference arm: also time mean and the 512^2 config")
    ap.add_argument("--parity", type=int, default=1, help="compare the timed count with the oracle (untimed)")
    ap.add_argument("--cfg1", type=int, default=1, help="also time the 1e7 float64 512^2 count configuration")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--pyramid-n", type=int, default=200_000_000, help="0 skips the tile-pyramid workload")
    ap.add_argument("--serving-n", type=int, default=500_000_000, help="0 skips the viewport workload")
    ap.add_argument("--serving-requests", type=int, default=10000)
    ap.add_argument("--serving-plain-requests", type=int, default=500,
                    help="plain mode (one whole-frame call per request) runs this prefix of each stream")
    ap.add_argument("--line-series", type=int, default=1000, help="0 skips the line workload")
    ap.add_argument("--line-cpu-series", type=int, default=20)
    ap.add_argument("--serving-slots", type=int, default=8)
    ap.add_argument("--serving-rates", default="200,1000,5000", help="Poisson arrival rates (req/s)")
    ap.add_argument("--serving-modes", default="batched,sequential,plain")
    ap.add_argument("--serving-mem-gb", type=int, default=8)
    ap.add_argument("--only", default="all", choices=["all", "pyramid", "line", "serving"],
                    help="run one secondary workload alone (for profiling); prints its JSON object")
    ap.add_argument("--pyramid-config", default=None,
                    help="split,threads,chunk: skip the autotuner (for profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.only != "all":
        return run_only(args)
    return run_gpu(args)


def run_only(args):
    """One secondary workload alone, e.g. under ncu."""
    import torch
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    peak, peak_kind = measured_peak()
    if args.only == "pyramid":
        out = bench_pyramid(args, dev, peak, peak_kind)
    elif args.only == "line":
        out = bench_line(args, dev)
    else:
        out = bench_serving(args, dev)
    print(json.dumps({args.only: out}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
