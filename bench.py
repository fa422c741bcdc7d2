#!/usr/bin/env python3
"""Escape-time throughput on GB300: Gpixel-iter/s of one frame workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one step = one frame): Mandelbrot, 3840x2160, span 1e-10 (plane
width), centre = a seeded point on the set boundary found by bisection along a
seeded ray from inside the main cardioid to |c| = 2.5, maxIter 20000, 4
jittered samples per pixel (seeded uniform offsets), coloured through a seeded
256-entry RGBA8 palette with linear interpolation.  Unit of work: one
pixel-iteration (one z <- z^2 + c step of one sample; an interior sample
counts maxIter), counted by the kernel itself.

Timed region: K frames, each bracketed by CUDA events on the launching stream,
with a 256 MiB write between frames to flush L2; barrier + synchronize on both
sides; max over ranks.  N > 1 runs independent replicas (one process per GPU,
no collective on the data path).

--impl reference times the reference's own per-sample function
(computeFractal<double>, src/main/cuda/fractals/mandelbrot.cu, host-built by
oracle/build_ref.sh) on the host cores over a bounded sample of the same
frame's sample points; the oracle's C restatement stands in when the
reference build is unavailable.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "chaos-ultra_gb300")
for _p in (PKG_DIR, ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

WORKLOAD_SEED = 2
W, H, SPAN, MAX_ITER, SPP = 3840, 2160, 1e-10, 20000, 4
FULL_W = W  # the plane span is defined on the full 3840-pixel width
METRIC = "Gpixel-iter/s at <=0.1% escape-count mismatch vs FP64 oracle"
MISMATCH_SAMPLE_PIXELS = 4096
E2E_FRAMES = 3  # frames timed through the host-buffer call (each ~4.7 s at C2)
MIN_TIMED_S = 2.5  # shortest timed region of the C1 / C3 lines (clock samples every 200 ms)


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------

def boundary_point(seed, max_iter=MAX_ITER):
    from chaos_gb300.workloads import boundary_point as bp
    return bp(seed, max_iter)


def deep_center(seed, bits=1024):
    from chaos_gb300.workloads import deep_center as dc
    return dc(seed, bits)


def workload(seed=WORKLOAD_SEED):
    from chaos_gb300.palette import seeded_palette
    cx, cy = boundary_point(seed)
    return {"center": (cx, cy), "pixel_size": SPAN / FULL_W, "palette": seeded_palette(256, seed=seed),
            "jitter_seed": 1000 + seed, "interior_rgba": 0xFF000000}


def frame_desc(cg, wl, tier, arith):
    return cg.FrameDesc(width=W, height=H, max_iterations=MAX_ITER, samples_per_pixel=SPP,
                        sample_mode=cg.SAMPLES_JITTER, tier=tier, arith=arith, fractal=cg.MANDELBROT,
                        seed=wl["jitter_seed"], center_x=wl["center"][0], center_y=wl["center"][1],
                        pixel_size=wl["pixel_size"])


def sample_pixels(n, seed=7):
    """Seeded pixel indices spread over the frame."""
    import numpy as np
    return np.sort(np.random.default_rng(seed).choice(W * H, size=n, replace=False))


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = float(parts[2])
                    power.append(float(parts[3]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power) if power else None}


# ---------------------------------------------------------------------------
# CPU leg: the reference's per-sample function (or the oracle port) on the host
# ---------------------------------------------------------------------------

def _cpu_impl(max_iter=MAX_ITER):
    """(kind, threads, runner): runner(xs, ys[, max_iter]) -> (total pixel-iterations, counts)."""
    from oracle import build_oracle
    from oracle.oracle import REF_LIB, Oracle, Reference
    build_oracle.build_oracle()
    try:
        build_oracle.build_reference()
    except RuntimeError:
        pass
    if os.path.exists(REF_LIB):
        try:
            ref = Reference()
            return "reference", ref.max_threads(), lambda xs, ys, mi=max_iter: ref.points_d(xs, ys, mi)
        except OSError:
            pass
    o = Oracle()
    # the oracle's restatement of computeFractal<double> (rounded arithmetic), OpenMP over points
    return "port", o.max_threads(), lambda xs, ys, mi=max_iter: o.mandelbrot_points_d(xs, ys, mi)


def cpu_sample_points(wl, n_pixels, seed=11):
    from oracle.oracle import Oracle
    import numpy as np
    o = Oracle()
    pix = sample_pixels(n_pixels, seed)
    xs, ys = [], []
    for p in pix:
        x, y = o.frame_points(W, H, SPP, 1, wl["jitter_seed"], wl["center"], wl["pixel_size"], int(p), 1)
        xs.append(x)
        ys.append(y)
    return pix, np.concatenate(xs), np.concatenate(ys)


def cpu_baseline(wl, budget_s=12.0):
    """Time the CPU implementation on a bounded sample of the frame's points."""
    kind, threads, run = _cpu_impl()
    n = 256
    while True:
        _, xs, ys = cpu_sample_points(wl, n, seed=11 + n)
        t0 = time.perf_counter()
        total, _ = run(xs, ys)
        dt = time.perf_counter() - t0
        if dt >= budget_s / 4 or n >= min(1 << 17, W * H):
            break
        n = min(1 << 17, W * H, int(n * max(2.0, (budget_s / 4) / max(dt, 1e-3))))
    return {"value": total / dt / 1e9, "unit": "Gpixel-iter/s", "cores": threads, "kind": kind,
            "sample": f"{n} seeded pixels x {SPP} jittered samples of the frame, maxIter {MAX_ITER}, FP64, "
                      f"{total} pixel-iterations in {dt:.2f} s"}


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def aggregate_over_ranks(kernel_ms, pixel_iterations_per_step, steps, world, device=None):
    """Replicas: every rank ran `steps` steps of the same work.  The job's time
    is the slowest rank's; the job's throughput counts every rank's work.
    Returns (max_ms, Gpixel-iter/s of the whole job)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(kernel_ms)], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    max_ms = float(t.item())
    return max_ms, pixel_iterations_per_step * steps * world / (max_ms / 1e3) / 1e9


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    wl = workload()
    kind, threads, run = _cpu_impl()
    # size one step at ~8 s of host work
    n = 512
    _, xs, ys = cpu_sample_points(wl, n, seed=101)
    t0 = time.perf_counter()
    run(xs, ys)
    dt = max(time.perf_counter() - t0, 1e-3)
    n = max(256, min(1 << 18, W * H, int(n * 8.0 / dt)))
    pts = [cpu_sample_points(wl, n, seed=200 + k) for k in range(args.warmup + args.steps)]
    for k in range(args.warmup):
        run(pts[k][1], pts[k][2])
    total, elapsed, lat = 0, 0.0, []
    for k in range(args.steps):
        _, xs, ys = pts[args.warmup + k]
        t0 = time.perf_counter()
        t, _ = run(xs, ys)
        d = time.perf_counter() - t0
        total += t
        elapsed += d
        lat.append(d * 1e3)
    value = total / elapsed / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Gpixel-iter/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded boundary centre, seeded jitter offsets",
            "config": {"workload": f"Mandelbrot {W}x{H} span {SPAN} maxIter {MAX_ITER} {SPP} jittered spp "
                                   f"(each step: {n} seeded pixels of that frame on the host cores)",
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": value, "unit": "Gpixel-iter/s", "cores": threads, "kind": kind,
                             "sample": f"{n} seeded pixels x {SPP} samples per step"},
            "e2e": {"value": value, "unit": "Gpixel-iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    import chaos_gb300 as cg

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    wl = workload()
    # The headline tier is the one that meets the metric's mismatch bar: at this
    # depth (pixel 2.6e-14, maxIter 20000, centre on the boundary) any change of
    # rounding flips ~30% of escape counts, so only binary64 with the
    # reference's rounding (no contraction) is within 0.1% of the FP64 oracle.
    tier, arith = cg.TIER_F64, cg.ARITH_PARITY
    desc = frame_desc(cg, wl, tier, arith)
    dev = torch.device("cuda", local)
    pal = torch.from_numpy(wl["palette"].view(np.int32)).to(dev)
    rgba = torch.zeros(W * H, dtype=torch.int32, device=dev)
    total = torch.zeros(1, dtype=torch.int64, device=dev)
    skipped = torch.zeros(1, dtype=torch.int64, device=dev)
    out = cg.FrameOut(rgba=rgba.data_ptr(), palette=pal.data_ptr(), palette_len=len(wl["palette"]),
                      interior_rgba=wl["interior_rgba"], total_iterations=total.data_ptr(),
                      cycle_skipped=skipped.data_ptr())
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def frame():
        total.zero_()
        skipped.zero_()
        cg.render_frame(desc, out, stream=stream, sync=False)

    for _ in range(args.warmup):
        frame()
    torch.cuda.synchronize()
    iters_per_frame = int(total.item())
    skipped_per_frame = int(skipped.item())

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(k & 255)
        starts[k].record(stream)
        frame()
        ends[k].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    if world > 1:
        dist.barrier()
    lat = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    kernel_ms = sum(lat)
    max_ms, value = aggregate_over_ranks(kernel_ms, iters_per_frame, args.steps, world, dev)

    # end to end: the host-buffer call a caller without device memory makes
    host_rgba = np.zeros(W * H, dtype=np.uint32)
    try:
        host_rgba = torch.empty(W * H, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    except RuntimeError:
        pass
    cg.render_frame_host(desc, wl["palette"], wl["interior_rgba"], host_rgba)  # warm the workspace
    torch.cuda.synchronize()
    e2e_frames = min(args.steps, E2E_FRAMES)
    e0 = time.perf_counter()
    e2e_iters = 0
    for _ in range(e2e_frames):
        e2e_iters += cg.render_frame_host(desc, wl["palette"], wl["interior_rgba"], host_rgba)
    e2e_s = time.perf_counter() - e0
    e2e_value = e2e_iters / e2e_s / 1e9

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    # roofline: FP64 pipe
    peak = cg.measure_fma_peak(cg.TIER_F64)  # FLOP/s with an FMA = 2
    # rounded arithmetic: x*x, y*y, xx-yy, +cx, x*y, fma(2, x*y, cy) = 6
    # operations per step (the reference's literal (2x)*y + cy is 7; both round
    # identically, see step_rounded6).  The kernel forms xx-yy on the integer
    # units (bit-identical), so 5 of the 6 go to the FP64 pipe; `frac` is the
    # algorithmic 6-op figure, `fp64_pipe_frac` the pipe's own occupancy.  The
    # escape test adds 3 per 16-step block.
    ops_per_iter, pipe_ops_per_iter = 6, 5
    rate = iters_per_frame / (kernel_ms / args.steps / 1e3)
    achieved_ops = rate * ops_per_iter
    roof = {"bound": "fp64-pipe", "achieved": achieved_ops / 1e12, "peak": peak / 2 / 1e12, "unit": "Top/s",
            "frac": achieved_ops / (peak / 2), "traffic": None,
            "traffic_note": "FP64-pipe bound, state in registers: the ncu capture of the central 480x270 crop "
                            "read 461 KB and wrote 0 B of DRAM per launch",
            "peak_source": "measured in this run: chaos_measure_fma_peak (full-occupancy DFMA chains)",
            "ops_per_iteration": ops_per_iter, "fp64_pipe_ops_per_iteration": pipe_ops_per_iter,
            "fp64_pipe_frac": rate * pipe_ops_per_iter / (peak / 2),
            "kernel": "k_frame<double,PARITY,mandelbrot>",
            "note": "algorithmic ops = 6 per pixel-iteration (3 products, 2 adds, 1 fused add); one of them (x*x - y*y) runs "
                    "exactly rounded on the integer units, so frac can exceed 1; fp64_pipe_frac counts the 5 "
                    "FP64-pipe instructions per iteration"}

    # CPU leg: reference per-sample function on host cores + FP64-oracle mismatch
    base = cpu_baseline(wl)
    kind, _, run = _cpu_impl()
    pix = sample_pixels(MISMATCH_SAMPLE_PIXELS)
    counts = torch.zeros(W * H * SPP, dtype=torch.int32, device=dev)
    chk = cg.FrameOut(counts=counts.data_ptr())
    cg.render_frame(desc, chk, stream=stream)
    gpu_counts = counts.cpu().numpy().view(np.uint32).reshape(W * H, SPP)[pix].ravel()
    _, xs, ys = cpu_sample_points(wl, MISMATCH_SAMPLE_PIXELS, seed=7)
    _, ref_counts = run(xs, ys)
    mismatch = float((gpu_counts != ref_counts).mean())

    # the other binary64 arithmetic, for reference: throughput and mismatch
    tiers = {}
    for name, t_, a_ in (("f64-fma", cg.TIER_F64, cg.ARITH_FMA),):
        d2 = frame_desc(cg, wl, t_, a_)
        o2 = cg.FrameOut(counts=counts.data_ptr(), total_iterations=total.data_ptr())
        total.zero_()
        cg.render_frame(d2, o2, stream=stream)  # warm
        total.zero_()
        e_s, e_e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e_s.record(stream)
        cg.render_frame(d2, o2, stream=stream, sync=False)
        e_e.record(stream)
        torch.cuda.synchronize()
        ms = e_s.elapsed_time(e_e)
        c2 = counts.cpu().numpy().view(np.uint32).reshape(W * H, SPP)[pix].ravel()
        tiers[name] = {"value": int(total.item()) / (ms / 1e3) / 1e9, "unit": "Gpixel-iter/s", "ms_per_frame": ms,
                       "escape_count_mismatch_rate": float((c2 != ref_counts).mean())}

    line = {
        "metric": METRIC, "value": value, "unit": "Gpixel-iter/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded boundary centre, seeded jitter offsets, seeded palette",
        "config": {"workload": f"Mandelbrot {W}x{H} span {SPAN} maxIter {MAX_ITER} {SPP} jittered spp, "
                               f"256-entry palette with linear interpolation",
                   "center": list(wl["center"]), "tier": "f64", "arith": "rounded (no contraction)",
                   "l2": "flushed between steps (256 MiB write, outside the events)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "pixel_iterations_per_step": iters_per_frame,
        "cycle_skipped_per_step": skipped_per_frame,
        "steps_executed_per_step": iters_per_frame - skipped_per_frame,
        "frame_latency_ms": {"p50": statistics.median(lat), "p99": float(np.percentile(lat, 99)),
                             "max": max(lat)},
        "mismatch": {"vs": f"FP64 oracle ({kind}: computeFractal<double>, rounded arithmetic)",
                     "samples": int(len(ref_counts)), "escape_count_mismatch_rate": mismatch},
        "tiers": tiers,
        "roofline": roof,
        "cpu_baseline": base,
        "e2e": {"value": e2e_value, "unit": "Gpixel-iter/s", "h2d_bytes_per_step": 4 * len(wl["palette"]),
                "d2h_bytes_per_step": 4 * W * H + 8, "call": "chaos_render_frame_host", "frames": e2e_frames},
        "gpu_launches": args.steps,
        "clocks": clk,
        "wall_s_timed": wall,
    }
    if not args.headline_only and W == 3840:
        # after the headline's timed region: the other claims of the path, each
        # with its own clock record (the reference's own GPU kernel on this machine,
        # the C3 deep zoom, the batched C4 forms, the served C5 trace)
        t_sub = time.perf_counter()
        line["vs_reference_kernel"] = measure_vs_reference_kernel()
        line["c3"] = measure_c3(steps=3, warmup=1, compact=True)
        line["c4"] = measure_c4("c4", steps=3, warmup=1, compact=True)
        line["c5"] = measure_c5(seconds=C5_BENCH_SECONDS, compact=True)
        line["wall_s_sub_objects"] = time.perf_counter() - t_sub
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def _l2_flush(torch, dev):
    buf = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    return lambda k: buf.fill_(k & 255)


REF_CUBIN_DIR = os.path.join(ROOT, "oracle", "_ref")
VS_REF_W, VS_REF_H = 1920, 1080


def measure_vs_reference_kernel(launches=3):
    """The reference's own fractalRenderMainDouble against the drop-in modules
    on the same GB300, the way the Java host runs them: module loaded by file
    (cuModuleLoad), 32x32 blocks over ceil(W/32) x ceil(H/32), the legacy
    default stream (CudaFractalRenderer.java:235-269).

    The reference's mandelbrot module is its own source built for sm_103a
    twice: as nvcc builds it by default (contraction on: the build the Java
    application loads) and with --fmad=false (every product and sum rounded,
    the FP64 oracle's arithmetic).  They are set against cudaKernels/ (the
    default build's arithmetic reproduced) and cudaKernels_parity/ (rounded).
    View: the central 1920x1080 of the C2 frame (pixel 1e-10/3840 around the
    seeded boundary centre), maxIter 20000, maxSS 4, adaptive sampling on, in
    the reference's own sampling (sample 0 at the pixel corner, diagonal /
    grid pattern, warp votes).  One untimed launch, then `launches` launches
    between CUDA events with an L2 flush between them; the records of the last
    launch are compared field by field."""
    import torch

    import chaos_gb300 as cg
    from chaos_gb300.dropin import Driver, java_grid, main_params, pitched, read_pixels, same_pixels

    paths = {"reference_nofma": os.path.join(REF_CUBIN_DIR, "ref_mandelbrot_nofma.cubin"),
             "dropin_parity": os.path.join(cg.DROPIN_PARITY_DIR, "mandelbrot.ptx"),
             "reference_default": os.path.join(REF_CUBIN_DIR, "ref_mandelbrot.cubin"),
             "dropin_contracted": os.path.join(cg.DROPIN_DIR, "mandelbrot.ptx")}
    missing = [os.path.relpath(p, ROOT) for p in paths.values() if not os.path.exists(p)]
    if missing:
        return {"unavailable": "not built: " + ", ".join(missing)}
    cx, cy = boundary_point(WORKLOAD_SEED)
    ps = SPAN / FULL_W
    w, h = VS_REF_W, VS_REF_H
    rect = (cx - w / 2 * ps, cy - h / 2 * ps, cx + w / 2 * ps, cy + h / 2 * ps)
    drv = Driver()
    buf, pitch = pitched(torch, w, h)
    grid, block = java_grid(w, h)
    flush = _l2_flush(torch, torch.device("cuda", 0))
    ms, recs = {}, {}
    clocks = ClockSampler(0)
    clocks.start()
    for name, path in paths.items():
        mod = drv.load(path)
        try:
            drv.write_constant(mod, "VISUALIZE_SAMPLE_COUNT", b"\0")
            fn = drv.function(mod, "fractalRenderMainDouble")
            params = main_params(buf.data_ptr(), pitch, w, h, rect, MAX_ITER, 4.0, cg.FLAG_ADAPTIVE_SS, True)
            drv.launch(fn, grid, block, params)
            times = []
            for k in range(launches):
                flush(k)
                buf.zero_()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                drv.launch(fn, grid, block, params, sync=False)
                e1.record()
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1))
            ms[name] = times
            recs[name] = read_pixels(buf, w)
        finally:
            drv.unload(mod)
    clk = clocks.stop()
    med = {k: statistics.median(v) for k, v in ms.items()}
    return {
        "view": f"C2 central {w}x{h}: pixel {SPAN}/{FULL_W}, maxIter {MAX_ITER}, maxSS 4, adaptive sampling, "
                "fractalRenderMainDouble in the Java launch shape",
        "launches": launches, "ms": ms, "ms_median": med,
        "speedup": {"dropin_parity_vs_reference_nofma": med["reference_nofma"] / med["dropin_parity"],
                    "dropin_contracted_vs_reference_default": med["reference_default"] / med["dropin_contracted"]},
        "records_differing": {
            "dropin_parity_vs_reference_nofma": float(same_pixels(recs["dropin_parity"],
                                                                  recs["reference_nofma"]).mean()),
            "dropin_contracted_vs_reference_default": float(same_pixels(recs["dropin_contracted"],
                                                                        recs["reference_default"]).mean())},
        "reference_build": "the reference's src/main/cuda mandelbrot module built from source for sm_103a "
                           "(oracle/build_ref.sh): default nvcc contraction and --fmad=false",
        "clocks": clk}


def _timed_launches(torch, stream, flush, launch, n):
    """One untimed launch, then n launches between CUDA events on `stream`
    with an L2 flush before each; returns the list of ms."""
    launch()
    torch.cuda.synchronize()
    ms = []
    for k in range(n):
        flush(k)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        launch()
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    return ms


def measure_c4(workload="c4", steps=3, warmup=3, compact=False):
    """C4: 64 viewports (side 256..2048, span 1e-12..1e-3, maxIter 500..50000,
    seeded boundary centres) in one CUDA-graph launch, tier per viewport.

    Beside the tiered value: the same batch in binary64 rounded as the
    reference's computeFractal<double> (tier F64_ROUNDED, the FP64 oracle's
    counts bit for bit), whose counts give every other form's mismatch against
    the FP64 oracle over all pixels; the plain FP64 drop-in viewport by
    viewport (the library's fractalRenderMainDouble, and the drop-in module
    and the reference's own module, both built --fmad=false, in the Java launch
    shape); and a CPU leg that runs the reference's own host-built
    computeFractal<double> at seeded pixels of every viewport (the CPU
    baseline, and the oracle those counts are checked on).  `compact` leaves
    out the untuned shape and the per-tier breakdown."""
    import numpy as np
    import torch

    import chaos_gb300 as cg
    from chaos_gb300.workloads import c4_palette, c4_viewports

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    specs = c4_viewports()
    if workload == "c4-crop":
        # the central 256 x 256 window of each viewport at the same pixel size (profiler captures)
        for sp in specs:
            side = min(sp["width"], 256)
            sp["span"] = sp["span"] * side / sp["width"]
            sp["width"] = sp["height"] = side
    pal = c4_palette()
    dpal = torch.from_numpy(pal.view(np.int32)).to(dev)

    def make(force_tier, config=None):
        bufs, vps = [], []
        for k, sp in enumerate(specs):
            n = sp["width"] * sp["height"]
            counts = torch.zeros(n, dtype=torch.int32, device=dev)
            rgba = torch.zeros(n, dtype=torch.int32, device=dev)
            bufs.append((counts, rgba))
            vps.append(cg.Viewport(width=sp["width"], height=sp["height"], max_iterations=sp["max_iter"],
                                   samples_per_pixel=1, sample_mode=cg.SAMPLES_CENTER,
                                   tier=force_tier, seed=sp["seed"], center_x=sp["center"][0],
                                   center_y=sp["center"][1], pixel_size=sp["span"] / sp["width"],
                                   counts=counts.data_ptr(), rgba=rgba.data_ptr()))
        return cg.Batch(vps, dpal.data_ptr(), len(pal), 0xFF000000, config), bufs

    # launch shapes per tier from the autotuner (outside the timed region)
    t_tune = time.perf_counter()
    tune_vps = [cg.Viewport(width=sp["width"], height=sp["height"], max_iterations=sp["max_iter"],
                            samples_per_pixel=1, sample_mode=cg.SAMPLES_CENTER, tier=cg.TIER_AUTO, seed=sp["seed"],
                            center_x=sp["center"][0], center_y=sp["center"][1],
                            pixel_size=sp["span"] / sp["width"]) for sp in specs]
    tuned, _ = cg.autotune_batch(tune_vps)
    t_tune = time.perf_counter() - t_tune

    batch, bufs = make(cg.TIER_AUTO, tuned)
    stream = torch.cuda.current_stream()
    flush = _l2_flush(torch, dev)
    for _ in range(warmup):
        batch.launch(stream)
    torch.cuda.synchronize()
    per_launch = batch.read_total()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    clocks = ClockSampler(0)
    clocks.start()
    # an NVTX range around the timed launches only (the autotuner's and the
    # warm-up launches stay outside it): ncu --nvtx --nvtx-include "c4 tiered launches/"
    torch.cuda.nvtx.range_push("c4 tiered launches")
    for k in range(steps):
        flush(k)
        ev[k][0].record(stream)
        batch.launch(stream)
        ev[k][1].record(stream)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = [a.elapsed_time(b) for a, b in ev]
    value = per_launch * steps / (sum(ms) / 1e3) / 1e9
    tiers = batch.tiers()
    tiered_counts = [c.cpu().numpy() for c, _ in bufs]
    batch.close()
    del batch, bufs

    # binary64 rounded as the reference's computeFractal<double> (tier
    # F64_ROUNDED): the FP64 oracle's escape counts, bit for bit, for every pixel
    rounded, rbufs = make(cg.TIER_F64_ROUNDED, tuned)
    rclocks = ClockSampler(0)
    rclocks.start()
    r_ms = _timed_launches(torch, stream, flush, lambda: rounded.launch(stream), steps)
    rclk = rclocks.stop()
    rounded_iters = rounded.read_total()
    rounded_skipped = rounded.read_cycle_skipped()
    rounded_value = rounded_iters * len(r_ms) / (sum(r_ms) / 1e3) / 1e9
    rounded_counts = [c.cpu().numpy() for c, _ in rbufs]
    rounded.close()
    del rounded, rbufs
    total = sum(len(a) for a in rounded_counts)

    def vs_oracle(counts):
        return sum(int((c != r).sum()) for c, r in zip(counts, rounded_counts)) / total

    untuned_ms = None
    if not compact:
        # the same batch with the default launch shape (256 threads, 16-step blocks, chunk 1)
        untuned, ubufs = make(cg.TIER_AUTO)
        untuned_ms = min(_timed_launches(torch, stream, flush, lambda: untuned.launch(stream), 2))
        untuned.close()
        del untuned, ubufs

    plain, pbufs = make(cg.TIER_F64)
    plain_ms = _timed_launches(torch, stream, flush, lambda: plain.launch(stream), 1)[0]
    plain_value = plain.read_total() / (plain_ms / 1e3) / 1e9
    plain_counts = [c.cpu().numpy() for c, _ in pbufs]
    plain.close()
    del plain, pbufs

    # binary32 / float-float / perturbation (the deep viewports on reference orbits)
    deep, dbufs = make(cg.TIER_AUTO_DEEP)
    deep_ms = _timed_launches(torch, stream, flush, lambda: deep.launch(stream), 2)
    deep_value = deep.read_total() / (min(deep_ms) / 1e3) / 1e9
    deep_tiers = deep.tiers()
    deep_counts = [c.cpu().numpy() for c, _ in dbufs]
    deep.close()
    del deep, dbufs

    per_tier = {}
    if not compact:
        # time per tier: the same batch restricted to one tier's viewports
        for tier_id, name in ((2, "floatfloat"), (1, "f64"), (0, "f32")):
            idx = [k for k, t in enumerate(tiers) if t == tier_id]
            if not idx:
                continue
            sub_bufs, sub_vps = [], []
            for k in idx:
                sp = specs[k]
                n = sp["width"] * sp["height"]
                rgba = torch.zeros(n, dtype=torch.int32, device=dev)
                sub_bufs.append(rgba)
                sub_vps.append(cg.Viewport(width=sp["width"], height=sp["height"], max_iterations=sp["max_iter"],
                                           samples_per_pixel=1, sample_mode=cg.SAMPLES_CENTER, tier=tier_id,
                                           seed=sp["seed"], center_x=sp["center"][0], center_y=sp["center"][1],
                                           pixel_size=sp["span"] / sp["width"], rgba=rgba.data_ptr()))
            sb = cg.Batch(sub_vps, dpal.data_ptr(), len(pal), 0xFF000000, tuned)
            t_ms = _timed_launches(torch, stream, flush, lambda: sb.launch(stream), 1)[0]
            it = sb.read_total()
            per_tier[name] = {"viewports": len(idx), "ms": t_ms, "pixel_iterations": it,
                              "Gpixel_iter_s": it / (t_ms / 1e3) / 1e9}
            sb.close()

    # the plain FP64 drop-in, viewport by viewport: fractalRenderMainDouble
    # semantics (rounded arithmetic, one sample at the pixel corner, no
    # adaptive super-sampling) through (i) the library's C ABI, (ii) the
    # drop-in module and (iii) the reference's own module (both --fmad=false)
    # in the Java launch shape.  Each form's pixel-iterations are counted from
    # its own records (value 0 = interior = maxIter).
    from chaos_gb300.dropin import Driver, java_grid, main_params, pitched, read_pixels, same_pixels
    module = cg.Module("mandelbrot")
    drv = Driver()
    forms = {"library": None, "dropin_module": os.path.join(cg.DROPIN_PARITY_DIR, "mandelbrot.ptx"),
             "reference_module": os.path.join(REF_CUBIN_DIR, "ref_mandelbrot_nofma.cubin")}
    fns, mods = {}, []
    for name, path in list(forms.items()):
        if path is None:
            continue
        if not os.path.exists(path):
            forms.pop(name)
            continue
        m = drv.load(path)
        mods.append(m)
        drv.write_constant(m, "VISUALIZE_SAMPLE_COUNT", b"\0")
        fns[name] = drv.function(m, "fractalRenderMainDouble")
    vp_stats = {name: {"ms": 0.0, "iters": 0} for name in forms}
    records_differ = 0
    vp_clocks = ClockSampler(0)
    vp_clocks.start()
    for sp in specs:
        w_, h_ = sp["width"], sp["height"]
        buf, pitch = pitched(torch, w_, h_)
        cx, cy, span = sp["center"][0], sp["center"][1], sp["span"]
        rect = (cx - span / 2, cy - span / 2 * h_ / w_, cx + span / 2, cy + span / 2 * h_ / w_)
        recs = {}
        for name in forms:
            if name == "library":
                def go():
                    module.render_main(buf.data_ptr(), pitch, w_, h_, rect, sp["max_iter"], 1.0, 0, double=True,
                                       arith=cg.ARITH_PARITY, stream=stream)
            else:
                params = main_params(buf.data_ptr(), pitch, w_, h_, rect, sp["max_iter"], 1.0, 0, True)
                grid, block = java_grid(w_, h_)

                def go(fn=fns[name], params=params, grid=grid, block=block):
                    drv.launch(fn, grid, block, params, sync=False)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            go()
            e1.record(stream)
            torch.cuda.synchronize()
            vp_stats[name]["ms"] += e0.elapsed_time(e1)
            recs[name] = read_pixels(buf, w_)
            vals = recs[name]["value"]
            vp_stats[name]["iters"] += int(np.where(vals == 0, sp["max_iter"], vals).astype(np.int64).sum())
        if "reference_module" in recs:
            records_differ += int(same_pixels(recs["dropin_module"], recs["reference_module"]).sum())
        del buf
    vp_clk = vp_clocks.stop()
    for m in mods:
        drv.unload(m)
    plain_forms = {name: {"value": st["iters"] / (st["ms"] / 1e3) / 1e9, "ms": st["ms"],
                          "pixel_iterations": st["iters"]} for name, st in vp_stats.items()}
    dropin_value = plain_forms["library"]["value"]

    # CPU leg: the reference's own computeFractal<double> (host build, all host
    # threads) at seeded pixels of every viewport, the same binary64 sample
    # points: the CPU baseline, and the FP64 oracle the GPU counts are checked on
    from oracle.oracle import Oracle
    kind, cpu_threads, cpu_run = _cpu_impl()
    orc = Oracle()
    rng = np.random.default_rng(44)
    cpu_iters, cpu_s, cpu_n, cpu_bad = 0, 0.0, 0, {"rounded": 0, "tiered": 0, "tiered_deep": 0, "f64_fma": 0}
    per_vp = 256 if (compact or workload != "c4") else 1024
    for k, sp in enumerate(specs):
        n_pix = sp["width"] * sp["height"]
        pix = np.sort(rng.choice(n_pix, size=min(per_vp, n_pix), replace=False))
        pts = [orc.frame_points(sp["width"], sp["height"], 1, 0, sp["seed"], sp["center"], sp["span"] / sp["width"],
                                int(q), 1) for q in pix]
        xs = np.concatenate([a for a, _ in pts])
        ys = np.concatenate([b for _, b in pts])
        t0 = time.perf_counter()
        it, ref_counts = cpu_run(xs, ys, sp["max_iter"])
        cpu_s += time.perf_counter() - t0
        cpu_iters += it
        cpu_n += len(pix)
        for name, arr in (("rounded", rounded_counts), ("tiered", tiered_counts), ("tiered_deep", deep_counts),
                          ("f64_fma", plain_counts)):
            cpu_bad[name] += int((arr[k].view(np.uint32)[pix] != ref_counts).sum())
    cpu_base = {"value": cpu_iters / cpu_s / 1e9, "unit": "Gpixel-iter/s", "cores": cpu_threads, "kind": kind,
                "sample": f"{cpu_n} seeded pixels ({per_vp} per viewport) at the batch's sample points, "
                          f"FP64 computeFractal, {cpu_iters} pixel-iterations in {cpu_s:.2f} s"}
    oracle_mismatch = {name: bad / cpu_n for name, bad in cpu_bad.items()}
    ref_mod = plain_forms.get("reference_module")
    out = {
        "workload": "C4: 64 Mandelbrot viewports, side log-uniform 256..2048, span log-uniform 1e-12..1e-3, "
                    "maxIter log-uniform 500..50000, one CUDA-graph launch",
        "crop": "central 256x256 of each viewport" if workload == "c4-crop" else None,
        "pixels": total, "steps": steps, "warmup": warmup,
        "tiered": {"value": value, "ms": ms, "pixel_iterations": per_launch,
                   "tiers": {"f32": tiers.count(0), "floatfloat": tiers.count(2), "f64": tiers.count(1)},
                   "escape_count_mismatch_vs_fp64_oracle": vs_oracle(tiered_counts),
                   "speedup_of_plain_f64_dropin": value / dropin_value, "clocks": clk},
        "rounded_f64_batch": {
            "value": rounded_value, "ms": r_ms, "pixel_iterations": rounded_iters,
            "cycle_skipped": rounded_skipped, "steps_executed": rounded_iters - rounded_skipped,
            "escape_count_mismatch_vs_fp64_oracle_cpu_sample": oracle_mismatch["rounded"],
            "speedup_of_plain_f64_dropin": rounded_value / dropin_value,
            "speedup_of_reference_module": rounded_value / ref_mod["value"] if ref_mod else None,
            "what": "all 64 viewports in binary64 rounded as the reference's computeFractal<double> "
                    "(tier F64_ROUNDED, one graph launch): the form within 0.1% of the FP64 oracle",
            "clocks": rclk},
        "tiered_deep": {"value": deep_value, "ms": min(deep_ms),
                        "tiers": {"f32": deep_tiers.count(0), "floatfloat": deep_tiers.count(2),
                                  "perturb_f32": deep_tiers.count(3), "perturb_f64": deep_tiers.count(4)},
                        "escape_count_mismatch_vs_fp64_oracle": vs_oracle(deep_counts),
                        "speedup_of_plain_f64_dropin": deep_value / dropin_value,
                        "what": "binary32 / float-float / perturbation on per-viewport reference orbits "
                                "(orbits computed at batch creation, outside the timed launch)"},
        "f64_fma_batch": {"value": plain_value, "ms": plain_ms,
                          "escape_count_mismatch_vs_fp64_oracle": vs_oracle(plain_counts)},
        "plain_f64_dropin": dict(plain_forms["library"], what=(
            "fractalRenderMainDouble semantics (binary64, rounded arithmetic, 1 sample per pixel) viewport by "
            "viewport through the C ABI (chaos_render_main_f64): the plain FP64 drop-in of the 3x target")),
        "plain_f64_java_shape": {
            "dropin_module": plain_forms.get("dropin_module"), "reference_module": ref_mod,
            "records_differing_dropin_vs_reference": records_differ / total if ref_mod else None,
            "what": "the same viewports through cudaKernels_parity/mandelbrot.ptx and the reference's own module "
                    "built --fmad=false, 32x32 blocks per viewport on the default stream", "clocks": vp_clk},
        "target_3x": {
            "bar": ">= 3x the plain FP64 drop-in at <= 0.1% escape-count mismatch vs the FP64 oracle",
            "within_bar_form": "rounded_f64_batch",
            "within_bar_speedup_of_plain_f64_dropin": rounded_value / dropin_value,
            "within_bar_speedup_of_reference_module": rounded_value / ref_mod["value"] if ref_mod else None,
            "tiered_speedup_and_mismatch": [value / dropin_value, vs_oracle(tiered_counts)],
            "tiered_deep_speedup_and_mismatch": [deep_value / dropin_value, vs_oracle(deep_counts)]},
        "escape_count_mismatch_vs_fp64_oracle_cpu_sample": oracle_mismatch,
        "autotune": {"seconds": t_tune,
                     "shape": {name: {"threads": tuned.block_threads[k], "escape_block": tuned.escape_block[k],
                                      "chunk": tuned.chunk[k]}
                               for k, name in enumerate(("f32", "floatfloat", "f64"))},
                     "fp64_warps_per_sm_when_shared": tuned.fp64_warps_per_sm,
                     "default_shape_ms": untuned_ms, "tuned_ms": min(ms)},
        "cpu_baseline": cpu_base,
        "gpu_launches": steps * sum(1 for t in (0, 1, 2) if t in tiers)}
    if per_tier:
        out["per_tier"] = per_tier
    return out


def run_batch(args):
    """The C4 line: tiered batch value, with every other form beside it."""
    c4 = measure_c4(args.workload, args.steps, args.warmup)
    t = c4["tiered"]
    line = {"metric": "Gpixel-iter/s (batched uneven launch)", "value": t["value"], "unit": "Gpixel-iter/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(t["ms"]) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/ff/f64 per viewport",
            "data": "synthetic: seeded viewports and boundary centres",
            "config": {"workload": c4["workload"], "pixels": c4["pixels"], "l2": "flushed between launches",
                       "crop": c4["crop"]},
            "cpu_baseline": c4["cpu_baseline"], "gpu_launches": c4["gpu_launches"],
            "gpu_launches_note": "one persistent kernel per tier present per graph launch", "clocks": t["clocks"],
            "c4": c4}
    print(json.dumps(line), flush=True)


C1_N, C1_MAX_ITER, C1_TOTAL, C1_INTERIOR = 1024, 1000, 181_032_650, 175_986


def run_c1(args):
    """C1: plain Mandelbrot 1024x1024 in binary32, centre (-0.5, 0), span 3.0,
    maxIter 1000, one sample per pixel centre, escape counts + smooth counts.
    The headline tier is binary32 with the reference's rounding (bit-exact to
    its computeFractal<float>: 181,032,650 pixel-iterations, 175,986 interior
    pixels); the fused tier is reported beside it.  The CPU leg runs the
    reference's own host-built computeFractal<float> over the whole frame."""
    import numpy as np
    import torch

    import chaos_gb300 as cg

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    n = C1_N * C1_N
    counts = torch.zeros(n, dtype=torch.int32, device=dev)
    smooth = torch.zeros(n, dtype=torch.float32, device=dev)
    total = torch.zeros(1, dtype=torch.int64, device=dev)
    skipped = torch.zeros(1, dtype=torch.int64, device=dev)
    out = cg.FrameOut(counts=counts.data_ptr(), smooth=smooth.data_ptr(), total_iterations=total.data_ptr(),
                      cycle_skipped=skipped.data_ptr())
    stream = torch.cuda.current_stream()
    flush = _l2_flush(torch, dev)

    def desc(arith):
        return cg.FrameDesc(width=C1_N, height=C1_N, max_iterations=C1_MAX_ITER, samples_per_pixel=1,
                            sample_mode=cg.SAMPLES_CENTER, tier=cg.TIER_F32, arith=arith, fractal=cg.MANDELBROT,
                            seed=0, center_x=-0.5, center_y=0.0, pixel_size=3.0 / C1_N)

    def timed(arith, steps, warmup):
        d = desc(arith)
        for _ in range(warmup):
            cg.render_frame(d, out, stream=stream, sync=False)
        torch.cuda.synchronize()
        total.zero_()
        skipped.zero_()
        ev = []
        for k in range(steps):
            flush(k)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            cg.render_frame(d, out, stream=stream, sync=False)
            e1.record(stream)
            ev.append((e0, e1))
        torch.cuda.synchronize()
        return int(total.item()), sum(a.elapsed_time(b) for a, b in ev)

    # the timed region lasts at least MIN_TIMED_S, so that the clock sampler
    # (one sample per 200 ms) sees it: more frames than --steps when needed
    _, probe_ms = timed(cg.ARITH_PARITY, 3, args.warmup)
    min_s = MIN_TIMED_S if args.min_seconds is None else args.min_seconds
    args.steps = max(args.steps, math.ceil(min_s * 1e3 / max(probe_ms / 3, 1e-3)))
    clocks = ClockSampler(0)
    clocks.start()
    iters, ms = timed(cg.ARITH_PARITY, args.steps, 1)
    clk = clocks.stop()
    skipped_per_frame = int(skipped.item()) // args.steps
    per_frame = iters // args.steps
    c = counts.cpu().numpy().view(np.uint32)
    known = {"pixel_iterations": per_frame, "interior": int((c == C1_MAX_ITER).sum()),
             "matches_reference_known_answer": per_frame == C1_TOTAL and int((c == C1_MAX_ITER).sum()) == C1_INTERIOR}
    value = iters / (ms / 1e3) / 1e9
    f_iters, f_ms = timed(cg.ARITH_FMA, max(args.steps, 3), 1)

    # end to end through the host-buffer call (palette in, RGBA image out)
    from chaos_gb300.palette import seeded_palette
    pal = seeded_palette(256, seed=1)
    host = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    d = desc(cg.ARITH_PARITY)
    cg.render_frame_host(d, pal, 0xFF000000, host)
    e0 = time.perf_counter()
    e_frames = min(args.steps, 2000)
    e_iters = sum(cg.render_frame_host(d, pal, 0xFF000000, host) for _ in range(e_frames))
    e_s = time.perf_counter() - e0

    # roofline: FP32 pipe against the plain step's 6 instructions (the binary32
    # rounded step itself is the reference's literal 7: x*x, y*y, -, +cx, 2*x, *y, +cy)
    peak = cg.measure_fma_peak(cg.TIER_F32)
    ops = 6
    achieved = per_frame / (ms / args.steps / 1e3) * ops
    executed = per_frame - skipped_per_frame
    roof = {"bound": "fp32-pipe", "achieved": achieved / 1e12, "peak": peak / 2 / 1e12, "unit": "Top/s",
            "frac": achieved / (peak / 2), "traffic": None, "ops_per_iteration": ops,
            "peak_source": "measured in this run: chaos_measure_fma_peak (full-occupancy FFMA chains)",
            "kernel": "k_frame<float,PARITY,mandelbrot,64>",
            "steps_executed_per_frame": executed, "pixel_iterations_per_frame": per_frame,
            "frac_of_steps_executed": executed / (ms / args.steps / 1e3) * ops / (peak / 2),
            "note": "pixel-iterations count an interior sample as maxIter (the metric's unit); the kernel stops a "
                    "sample whose rounded state repeats bit for bit (exact cycle detection), so it executes fewer "
                    "steps: frac uses pixel-iterations, frac_of_steps_executed the steps the FP32 pipe ran"}

    # CPU leg: the reference's computeFractal<float> over the whole frame, all host threads
    cpu = None
    try:
        from oracle import build_oracle
        from oracle.oracle import REF_LIB, Reference
        build_oracle.build_oracle()
        try:
            build_oracle.build_reference()
        except RuntimeError:
            pass
        if os.path.exists(REF_LIB):
            ref = Reference()
            t0 = time.perf_counter()
            tot, _ = ref.grid(False, C1_N, C1_N, -2.0 + 0.5 * 3.0 / C1_N, 1.5 - 0.5 * 3.0 / C1_N, 3.0 / C1_N,
                              3.0 / C1_N, C1_MAX_ITER, counts=False)
            dt = time.perf_counter() - t0
            cpu = {"value": tot / dt / 1e9, "unit": "Gpixel-iter/s", "cores": ref.max_threads(),
                   "kind": "reference",
                   "sample": f"the whole frame ({tot} pixel-iterations, reference computeFractal<float>) "
                             f"in {dt:.3f} s"}
    except (ImportError, OSError):
        cpu = None

    line = {"metric": "Gpixel-iter/s (plain binary32 frame)", "value": value, "unit": "Gpixel-iter/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: the C1 plane rectangle",
            "config": {"workload": f"C1: Mandelbrot {C1_N}x{C1_N} binary32, centre (-0.5, 0), span 3.0, maxIter "
                                   f"{C1_MAX_ITER}, 1 sample per pixel centre", "arith": "rounded (reference)",
                       "l2": "flushed between steps"},
            "known_answer": known,
            "pixel_iterations_per_step": per_frame, "steps_executed_per_step": executed,
            "cycle_skipped_per_step": skipped_per_frame,
            "tiers": {"f32-fma": {"value": f_iters / (f_ms / 1e3) / 1e9, "unit": "Gpixel-iter/s"}},
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e_iters / e_s / 1e9, "unit": "Gpixel-iter/s", "h2d_bytes_per_step": 4 * len(pal),
                    "d2h_bytes_per_step": 4 * n + 8, "call": "chaos_render_frame_host"},
            "gpu_launches": args.steps, "clocks": clk}
    print(json.dumps(line), flush=True)


DEEP_W, DEEP_H, DEEP_MAX_ITER, DEEP_SPANS, DEEP_ORBIT_BITS = 1920, 1080, 100000, (1e-60, 1e-200), 1088


def run_deep(args):
    """`--workload c3`: the C3 line (measure_c3) with its CPU leg."""
    print(json.dumps(measure_c3(args.steps, args.warmup, args.min_seconds)), flush=True)


def measure_c3(steps=3, warmup=3, min_seconds=None, compact=False):
    """C3: perturbation deep zoom, 1920x1080, spans 1e-60 and 1e-200, maxIter
    100000, centre = the committed seeded Misiurewicz point (1024-bit fixed
    point), one sample per pixel at pixel centres.  One step = both spans'
    frames with binary32 differences (rescaled by 2^e at these depths); the
    reference orbit (1088 bits) is computed once, outside the timed region of
    `value`, and inside the e2e loop.  `compact` (the default bench line's C3
    object) leaves out the CPU leg and runs 20 e2e steps."""
    import numpy as np
    import torch

    import chaos_gb300 as cg
    from chaos_gb300.palette import seeded_palette
    from chaos_gb300.workloads import deep_zoom_centre

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    d = deep_zoom_centre()
    n = DEEP_W * DEEP_H
    pal_host = seeded_palette(256, seed=3)
    pal = torch.from_numpy(pal_host.view(np.int32)).to(dev)
    rgba = torch.zeros(n, dtype=torch.int32, device=dev)
    total = torch.zeros(1, dtype=torch.int64, device=dev)
    rebases = torch.zeros(1, dtype=torch.int64, device=dev)
    out = cg.FrameOut(rgba=rgba.data_ptr(), palette=pal.data_ptr(), palette_len=len(pal_host),
                      interior_rgba=0xFF000000, total_iterations=total.data_ptr(), rebases=rebases.data_ptr())
    stream = torch.cuda.current_stream()
    flush = _l2_flush(torch, dev)
    t_orbit = time.perf_counter()
    orbit = cg.Orbit(d["center_x"], d["center_y"], DEEP_ORBIT_BITS, DEEP_MAX_ITER)
    t_orbit = time.perf_counter() - t_orbit

    def desc(span, tier):
        return cg.FrameDesc(width=DEEP_W, height=DEEP_H, max_iterations=DEEP_MAX_ITER, samples_per_pixel=1,
                            sample_mode=cg.SAMPLES_CENTER, tier=tier, fractal=cg.MANDELBROT, seed=0,
                            pixel_size=span / DEEP_W)

    def timed(tier, steps, warm):
        descs = [desc(sp, tier) for sp in DEEP_SPANS]
        for _ in range(warm):
            for dd in descs:
                cg.render_frame_perturb(dd, orbit, out, stream=stream, sync=False)
        torch.cuda.synchronize()
        total.zero_()
        rebases.zero_()
        per_span_ms = [0.0] * len(descs)
        ev = []
        for k in range(steps):
            flush(k)
            row = []
            for dd in descs:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                cg.render_frame_perturb(dd, orbit, out, stream=stream, sync=False)
                e1.record(stream)
                row.append((e0, e1))
            ev.append(row)
        torch.cuda.synchronize()
        for row in ev:
            for j, (e0, e1) in enumerate(row):
                per_span_ms[j] += e0.elapsed_time(e1)
        return int(total.item()), per_span_ms, int(rebases.item())

    # per-span iteration counts (for per-span throughput)
    span_iters = []
    for sp in DEEP_SPANS:
        total.zero_()
        cg.render_frame_perturb(desc(sp, cg.TIER_PERTURB_F32), orbit, out, stream=stream)
        span_iters.append(int(total.item()))

    # the timed region lasts at least MIN_TIMED_S (more steps than --steps when needed)
    _, probe_ms, _ = timed(cg.TIER_PERTURB_F32, 2, warmup)
    min_s = MIN_TIMED_S if min_seconds is None else min_seconds
    steps = max(steps, math.ceil(min_s * 1e3 / max(sum(probe_ms) / 2, 1e-3)))
    clocks = ClockSampler(0)
    clocks.start()
    iters, span_ms, rb = timed(cg.TIER_PERTURB_F32, steps, 1)
    clk = clocks.stop()
    kernel_ms = sum(span_ms)
    value = iters / (kernel_ms / 1e3) / 1e9
    f64_iters, f64_ms, f64_rb = timed(cg.TIER_PERTURB_F64, 1, 1)

    # end to end: orbit from the hex centre, palette upload, both frames, images to host
    host = torch.empty(n, dtype=torch.int32, pin_memory=True)
    e0 = time.perf_counter()
    e2e_iters = 0
    e2e_steps = min(steps, 20 if compact else 100)
    for _ in range(e2e_steps):
        o2 = cg.Orbit(d["center_x"], d["center_y"], DEEP_ORBIT_BITS, DEEP_MAX_ITER)
        pal.copy_(torch.from_numpy(pal_host.view(np.int32)), non_blocking=False)
        for sp in DEEP_SPANS:
            total.zero_()
            cg.render_frame_perturb(desc(sp, cg.TIER_PERTURB_F32), o2, out, stream=stream, sync=False)
            host.copy_(rgba, non_blocking=True)
            torch.cuda.synchronize()
            e2e_iters += int(total.item())
        o2.close()
    e2e_s = time.perf_counter() - e0

    # roofline: FP32 pipe against the plain escape step's 6 FP32-pipe
    # instructions per pixel-iteration (the headline unit of every tier).  The
    # perturbation steps themselves cost: a composed block of 16 or 64 linear
    # steps 8 FP32 operations + one 16-byte load; an event-bounded linear step
    # 4 FFMA + 1 load of 2Z; quadratic rescaled step 12; plain-difference step
    # 16 (6 for the difference, 2 for z, 2 for |z|^2, 2 for |d|^2, compares).
    peak = cg.measure_fma_peak(cg.TIER_F32)
    ops = 6
    achieved = iters / (kernel_ms / 1e3) * ops
    roof = {"bound": "fp32-pipe", "achieved": achieved / 1e12, "peak": peak / 2 / 1e12, "unit": "Top/s",
            "frac": achieved / (peak / 2), "traffic": None,
            "peak_source": "measured in this run: chaos_measure_fma_peak (full-occupancy FFMA chains)",
            "ops_per_iteration": ops,
            "step_costs": {"composed_block_16_or_64": 8, "rescaled_linear": 4, "rescaled_quadratic": 12,
                           "plain_difference": 16},
            "kernel": "k_perturb<float,64,rescaled>"}

    # CPU leg: the oracle's multi-word direct iteration on a bounded sample of pixels
    cpu = None
    if not compact:
        from oracle.oracle import Oracle
        o = Oracle()
        rng = np.random.default_rng(5)
        nsamp = 64
        while True:
            pix = rng.choice(n, nsamp, replace=False)
            parts = [o.frame_offsets(DEEP_W, DEEP_H, 1, cg.SAMPLES_CENTER, 0, DEEP_SPANS[1] / DEEP_W, int(p), 1)
                     for p in pix]
            dcx = np.concatenate([p[0] for p in parts])
            dcy = np.concatenate([p[1] for p in parts])
            t0 = time.perf_counter()
            cc, _ = o.hp_escape_batch(d["center_x"], d["center_y"], dcx, dcy, DEEP_ORBIT_BITS, DEEP_MAX_ITER)
            dt = time.perf_counter() - t0
            if dt > 3.0 or nsamp >= 1 << 16:
                break
            nsamp = min(1 << 16, int(nsamp * max(2.0, 3.0 / max(dt, 1e-3))))
        cpu = {"value": float(cc.astype(np.int64).sum()) / dt / 1e9, "unit": "Gpixel-iter/s",
               "cores": o.max_threads(), "kind": "port",
               "sample": f"{nsamp} seeded pixels of the span-1e-200 frame, direct iteration at {DEEP_ORBIT_BITS} "
                         f"bits (the oracle; the reference has no multi-word path), {int(cc.sum())} "
                         f"pixel-iterations in {dt:.2f} s"}

    line = {"metric": "Gpixel-iter/s (perturbation deep zoom)", "value": value, "unit": "Gpixel-iter/s",
            "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": kernel_ms / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (rescaled differences)",
            "data": "synthetic: seeded Misiurewicz centre (1024-bit), seeded palette",
            "config": {"workload": f"C3: Mandelbrot {DEEP_W}x{DEEP_H}, spans 1e-60 and 1e-200 (one frame each per "
                                   f"step), maxIter {DEEP_MAX_ITER}, 1 sample per pixel centre, perturbation",
                       "centre": {"preperiod": d["preperiod"], "period": d["period"], "approx": d["approx"]},
                       "orbit_bits": DEEP_ORBIT_BITS, "l2": "flushed between steps"},
            "pixel_iterations_per_step": iters // steps,
            "per_span": {f"{sp:g}": {"pixel_iterations": it, "ms": ms / steps,
                                     "Gpixel_iter_s": it / (ms / steps / 1e3) / 1e9}
                         for sp, it, ms in zip(DEEP_SPANS, span_iters, span_ms)},
            "rebases_per_step": rb // steps,
            "f64_differences": {"value": f64_iters / (sum(f64_ms) / 1e3) / 1e9, "ms_per_step": sum(f64_ms),
                                "per_span_ms": f64_ms, "rebases": f64_rb},
            "orbit_seconds": t_orbit,
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_iters / e2e_s / 1e9, "unit": "Gpixel-iter/s", "h2d_bytes_per_step": 4 * len(pal_host),
                    "d2h_bytes_per_step": 2 * 4 * n,
                    "call": "chaos_orbit_create + chaos_render_frame_perturb x2 + image reads",
                    "seconds_per_step": e2e_s / e2e_steps, "steps": e2e_steps},
            "gpu_launches": 2 * steps, "clocks": clk}
    orbit.close()
    return line


def run_compose(args):
    """The compose kernel (gen.cu:455-475) alone: an 8K pixel_info_t frame
    (7680x4320 records of 16 B, pitched) through a 1536-entry palette into
    RGBA8.  Algorithmic traffic 20 B per pixel (16 B read, 4 B written); the
    palette sits in shared memory.  Bound: HBM."""
    import numpy as np
    import torch

    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    w, h = 7680, 4320
    pitch = ((16 * w + 511) // 512) * 512
    out_pitch = ((4 * w + 511) // 512) * 512
    rng = np.random.default_rng(9)
    vals = torch.from_numpy(rng.uniform(0, 5000, size=(h, pitch // 4)).astype(np.float32)).to(dev)
    vals.view(h, pitch // 16, 4)[:, :, 1] = 4.0  # weight
    out = torch.zeros((h, out_pitch // 4), dtype=torch.int32, device=dev)
    pal = default_palette()
    dpal = torch.from_numpy(np.ascontiguousarray(pal, dtype=np.uint32).view(np.int32)).to(dev)
    m = cg.Module("mandelbrot")
    stream = torch.cuda.current_stream()
    flush = _l2_flush(torch, dev)

    def go():
        m.compose(vals.data_ptr(), pitch, out.data_ptr(), out_pitch, w, h, dpal.data_ptr(), len(pal), 4.0,
                  stream=stream)

    for _ in range(args.warmup):
        go()
    torch.cuda.synchronize()
    ms = []
    clocks = ClockSampler(0)
    clocks.start()
    for k in range(args.steps):
        flush(k)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        go()
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    per = statistics.median(ms)
    algo = 20.0 * w * h
    peak = None
    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
        src = "MEASURED_PEAKS.json hbm_gbs (torch copy, read + write)"
    except (OSError, KeyError, ValueError):
        peak, src = 6800.0, "fallback 6.8 TB/s"
    gbs = algo / (per / 1e3) / 1e9
    line = {"metric": "GB/s (compose, algorithmic bytes)", "value": gbs, "unit": "GB/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 in, u8x4 out",
            "data": "synthetic: seeded values, the default 1536-entry palette",
            "config": {"workload": f"compose {w}x{h} pixel_info_t -> RGBA8", "l2": "flushed between steps"},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         # dram__bytes_read.sum + dram__bytes_write.sum of one launch of the same
                         # 7680x4320 compose, from the committed ncu summary (k_compose_8k)
                         "traffic": 646.9e6, "traffic_unit": "bytes per launch (ncu capture)",
                         "peak_source": src, "bytes_per_pixel": 20},
            "gpu_launches": args.steps, "clocks": clk}
    print(json.dumps(line), flush=True)


def run_reuse(args):
    """Sample reuse (fractalRenderAdvanced, gen.cu:307-368) alone: an 8K frame
    whose previous frame covers the same plane rectangle, so every pixel but
    the 2-pixel border takes its value and weight from the previous frame by
    bilinear filtering and computes no new sample.  Algorithmic traffic 32 B
    per pixel (16 B of the previous frame, 16 B written).  Bound: HBM."""
    import numpy as np
    import torch

    import chaos_gb300 as cg

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    w, h = 7680, 4320
    pitch = ((16 * w + 511) // 512) * 512
    rng = np.random.default_rng(10)
    prev = torch.from_numpy(rng.uniform(0, 5000, size=(h, pitch // 4)).astype(np.float32)).to(dev)
    prev.view(h, pitch // 16, 4)[:, :, 1] = 4.0  # weight
    prev.view(h, pitch // 16, 4)[:, :, 2] = 0.0  # isReused + padding
    out = torch.zeros_like(prev)
    m = cg.Module("mandelbrot")
    stream = torch.cuda.current_stream()
    flush = _l2_flush(torch, dev)
    rect = (-2.0, -1.5, 1.0, 1.5)

    def go():
        m.render_advanced(out.data_ptr(), pitch, w, h, rect, 100, 4.0, cg.FLAG_SAMPLE_REUSE, rect, prev.data_ptr(),
                          pitch, (w // 2, h // 2), stream=stream)

    for _ in range(args.warmup):
        go()
    torch.cuda.synchronize()
    ms = []
    clocks = ClockSampler(0)
    clocks.start()
    for k in range(args.steps):
        flush(k)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        go()
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    per = statistics.median(ms)
    reused = float((out.view(h, pitch // 16, 4)[:, :w, 2].view(torch.int32) & 0xFF).ne(0).float().mean().item())
    algo = 32.0 * w * h
    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
        src = "MEASURED_PEAKS.json hbm_gbs (torch copy, read + write)"
    except (OSError, KeyError, ValueError):
        peak, src = 6800.0, "fallback 6.8 TB/s"
    gbs = algo / (per / 1e3) / 1e9
    line = {"metric": "GB/s (sample reuse, algorithmic bytes)", "value": gbs, "unit": "GB/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded previous frame (weight 4)",
            "config": {"workload": f"fractalRenderAdvanced {w}x{h}, previous frame on the same rectangle, "
                                   "reuse only", "l2": "flushed between steps", "reused_fraction": reused},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         # dram__bytes_read.sum + dram__bytes_write.sum of one launch of the same
                         # 7680x4320 reuse frame, from the committed ncu summary (k_advanced_reuse_8k)
                         "traffic": 1022.8e6, "traffic_unit": "bytes per launch (ncu capture)",
                         "peak_source": src, "bytes_per_pixel": 32},
            "gpu_launches": args.steps, "clocks": clk}
    print(json.dumps(line), flush=True)


C5_BENCH_SECONDS = 10.0


def measure_c5(seconds=10.0, compact=False, n_cap=40):
    """C5: 16 zoom sessions (720p..2160p), 1.02x zoom per frame toward seeded
    boundary points, Poisson arrivals at 60 Hz per session for `seconds`,
    HBM-budget admission, sample reuse from the previous frame; p50/p99 frame
    latency, queueing delay and render time apart, and the capacity of a
    saturated server (n_cap frames per session submitted at once)."""
    import numpy as np
    import torch

    import chaos_gb300 as cg
    from chaos_gb300.palette import default_palette
    from chaos_gb300.workloads import boundary_points

    torch.cuda.set_device(0)
    rng = np.random.default_rng(5)
    res = [(1280, 720), (1920, 1080), (2560, 1440), (3840, 2160)]
    n_sessions, hz = 16, 60.0
    targets = boundary_points(list(range(500, 500 + n_sessions)), max_iter=2000)
    srv = cg.Server(48 << 30, default_palette())
    sids, shapes = [], []
    for k in range(n_sessions):
        w, h = res[int(rng.integers(0, 4))]
        d = cg.SessionDesc(width=w, height=h, max_iterations=2000, max_super_sampling=2.0, flags=1 | 4 | 8,
                           fractal=cg.MANDELBROT, arith=cg.ARITH_FMA, center_x=-0.5, center_y=0.0, span=3.0,
                           target_x=targets[k][0], target_y=targets[k][1], zoom_per_frame=1.02)
        sids.append(srv.open(d))
        shapes.append((w, h))
    # warm-up: one frame per session (renderQuality) before the timed trace
    for sid in sids:
        srv.submit(sid)
    srv.drain()
    warm = len(srv.records())
    it0 = sum(srv.read(sid)[1] for sid in sids)
    sess, arr = [], []
    for sid in sids:
        t = 0.0
        while True:
            t += rng.exponential(1.0 / hz)
            if t > seconds:
                break
            sess.append(sid)
            arr.append(t)
    order = np.argsort(arr)
    clocks = ClockSampler(0)
    clocks.start()
    t0 = srv.clock()
    srv.run_trace(np.array(sess)[order], np.array(arr)[order])
    t1 = srv.clock()
    clk = clocks.stop()
    recs = srv.records()[warm:]
    ok = [r for r in recs if r[6] == 0]
    lat = np.array([(r[4] - r[2]) * 1e3 for r in ok])
    queue_ms = np.array([(r[3] - r[2]) * 1e3 for r in ok])
    render_ms = np.array([(r[4] - r[3]) * 1e3 for r in ok])
    lat1080 = np.array([(r[4] - r[2]) * 1e3 for r in ok if shapes[r[0]] == (1920, 1080)])
    iters = sum(srv.read(sid)[1] for sid in sids) - it0
    value = iters / (t1 - t0) / 1e9
    precisions = {name: sum(1 for r in recs if r[5] == p) for name, p in
                  (("binary32", cg.PRECISION_SINGLE), ("floatfloat", cg.PRECISION_FLOATFLOAT),
                   ("binary64", cg.PRECISION_DOUBLE), ("perturbation", cg.PRECISION_TOO_BIG))}

    def pct(a, q):
        return float(np.percentile(a, q)) if len(a) else None

    # the served frames against the FP64 oracle: each session's last frame
    # rendered again from the same previous records in binary64 with the
    # reference's rounding (the library's parity path, identical to the
    # reference's --fmad=false kernel); escape values compared on the pixels
    # both renders sampled afresh (reused pixels hold filtered values)
    mism = served_vs_fp64_oracle(srv, sids, shapes)

    # capacity: every session asks for n_cap more frames at once (a saturated server)
    it1 = sum(srv.read(sid)[1] for sid in sids)
    r0 = len(srv.records())
    cap_clocks = ClockSampler(0)
    cap_clocks.start()
    c0 = srv.clock()
    for _ in range(n_cap):
        for sid in sids:
            srv.submit(sid)
    srv.drain()
    c1 = srv.clock()
    cap_clk = cap_clocks.stop()
    cap_iters = sum(srv.read(sid)[1] for sid in sids) - it1
    cap_lat = np.array([(r[4] - r[2]) * 1e3 for r in srv.records()[r0:]])
    capacity = {"frames": int(len(cap_lat)), "seconds": c1 - c0, "Gpixel_iter_s": cap_iters / (c1 - c0) / 1e9,
                "frames_per_s": len(cap_lat) / (c1 - c0),
                "what": f"{n_cap} frames per session submitted at once; latency includes queueing",
                "latency_ms_p50": pct(cap_lat, 50), "latency_ms_p99": pct(cap_lat, 99), "clocks": cap_clk}
    out = {"workload": f"C5: {n_sessions} sessions, 1280x720..3840x2160, zoom 1.02x/frame, Poisson {hz:g} Hz per "
                       f"session for {seconds:g} s, maxIter 2000, maxSS 2, sample reuse + foveation",
           "resolutions": [f"{w}x{h}" for w, h in shapes], "hbm_budget_gib": 48,
           "hbm_used_gib": srv.usage()[0] / 2 ** 30, "frames": len(recs), "warmup_frames": warm,
           "trace_s": t1 - t0, "value": value, "unit": "Gpixel-iter/s", "pixel_iterations": iters,
           "latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99), "max": float(lat.max()) if len(lat) else None,
                          "p50_1080p": pct(lat1080, 50), "p99_1080p": pct(lat1080, 99)},
           "queueing_delay_ms": {"p50": pct(queue_ms, 50), "p99": pct(queue_ms, 99),
                                 "what": "admission into a launch - arrival"},
           "render_ms": {"p50": pct(render_ms, 50), "p99": pct(render_ms, 99),
                         "what": "finished - admitted (the launch's GPU queue and run)"},
           "frames_not_ok": len(recs) - len(ok), "precision_of_frames": precisions,
           "served_vs_fp64_oracle": mism,
           "capacity": capacity, "clocks": clk}
    srv.close()
    return out


def served_vs_fp64_oracle(srv, sids, shapes):
    """Escape-value mismatch of each session's latest served frame against the
    same frame in binary64 with the reference's rounding, over the pixels both
    sampled afresh (not reused)."""
    import numpy as np
    import torch

    import chaos_gb300 as cg
    from chaos_gb300.dropin import Driver, pitched, read_pixels
    drv = Driver()
    module = cg.Module("mandelbrot")
    fresh_total, differ, reused_total, pixels = 0, 0, 0, 0
    per_prec = {}
    for sid in sids:
        st = srv.frame_state(sid)
        if st["precision"] == cg.PRECISION_TOO_BIG:
            continue
        w, h = shapes[sid]
        served = drv.read_pixels(st["pixels"], st["pixels_pitch"], w, h)
        buf, pitch = pitched(torch, w, h)
        if st["advanced"]:
            module.render_advanced(buf.data_ptr(), pitch, w, h, st["rect"], st["max_iterations"],
                                   st["max_super_sampling"], st["flags"], st["rect_reused"], st["previous"],
                                   st["previous_pitch"], (st["focus_x"], st["focus_y"]), double=True,
                                   arith=cg.ARITH_PARITY)
        else:
            module.render_main(buf.data_ptr(), pitch, w, h, st["rect"], st["max_iterations"],
                               st["max_super_sampling"], st["flags"], double=True, arith=cg.ARITH_PARITY)
        torch.cuda.synchronize()
        ref = read_pixels(buf, w)
        fresh = (served["is_reused"] == 0) & (ref["is_reused"] == 0)
        d = int((fresh & (served["value"].view(np.uint32) != ref["value"].view(np.uint32))).sum())
        f = int(fresh.sum())
        fresh_total += f
        differ += d
        reused_total += int((served["is_reused"] != 0).sum())
        pixels += w * h
        name = {cg.PRECISION_SINGLE: "binary32", cg.PRECISION_DOUBLE: "binary64",
                cg.PRECISION_FLOATFLOAT: "floatfloat"}[st["precision"]]
        a = per_prec.setdefault(name, [0, 0])
        a[0] += d
        a[1] += f
        del buf
    module.close()
    return {"what": "each session's latest frame vs the same frame in binary64 with the reference's rounding "
                    "(the FP64 oracle's arithmetic), escape values of the pixels both sampled afresh",
            "fresh_pixels": fresh_total, "reused_fraction": reused_total / max(pixels, 1),
            "escape_value_mismatch_rate": differ / max(fresh_total, 1),
            "by_precision": {k: {"mismatch_rate": v[0] / max(v[1], 1), "fresh_pixels": v[1]}
                             for k, v in per_prec.items()}}


def run_serve(args):
    """The C5 line."""
    c5 = measure_c5(seconds=args.seconds or C5_BENCH_SECONDS)
    line = {"metric": "Gpixel-iter/s; p99 frame latency (serving)", "value": c5["value"], "unit": "Gpixel-iter/s",
            "n_gpus": 1, "steps": c5["frames"], "warmup": c5["warmup_frames"],
            "ms_per_step": c5["latency_ms"]["p50"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32/f64 per frame",
            "data": "synthetic: seeded resolutions, boundary targets and Poisson arrivals",
            "config": {"workload": c5["workload"], "resolutions": c5["resolutions"]},
            "latency_ms": c5["latency_ms"], "clocks": c5["clocks"], "c5": c5}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--seconds", type=float, default=None, help="c5: length of the request trace (default 10)")
    ap.add_argument("--min-seconds", type=float, default=None,
                    help="c1 / c3: shortest timed region (default 2.5; 0 times exactly --steps steps, e.g. under a "
                         "profiler)")
    ap.add_argument("--headline-only", action="store_true",
                    help="C2: leave out the reference-kernel, C4 and C5 sub-objects after the headline")
    ap.add_argument("--workload", choices=["c1", "c2", "c2-crop", "c3", "c4", "c4-crop", "c5", "compose", "reuse"],
                    default="c2",
                    help="c2-crop / c4-crop: the central 480x270 pixels of the frame / 256x256 of each viewport "
                         "(for profiler captures)")
    args = ap.parse_args()
    if args.workload == "c2-crop":
        global W, H
        W, H = 480, 270
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "c1":
        run_c1(args)
    elif args.workload == "compose":
        run_compose(args)
    elif args.workload == "reuse":
        run_reuse(args)
    elif args.workload == "c3":
        run_deep(args)
    elif args.workload in ("c4", "c4-crop"):
        run_batch(args)
    elif args.workload == "c5":
        run_serve(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
