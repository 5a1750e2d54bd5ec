#!/usr/bin/env python3
"""Benchmark of the GB300 fill pipeline on the curves-and-gradients workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload curves|polygons|patterns|strokes]
                    [--impl ours|reference] [--cpu-seconds S]

Workload (default): one 1920x1080 PRGB32 canvas cleared to opaque black, 20,000 closed paths of
4-12 cubic segments (bbox side log-uniform 8-256 px), linear/radial/conic gradients with 2-8
stops and pad/repeat/reflect extend, non-zero/even-odd 50/50, SrcOver; seed 2. A step renders one
full frame of it.

Our arm prints one JSON line:
  value  - Mpix/s of canvas rendered, device-resident inputs (the frame's command data already in
           HBM, each step = the whole device pipeline: LUTs, edge building, binning, coverage and
           composite), timed with CUDA events on the pipeline's stream, L2 flushed between steps;
  e2e    - the same metric through the public C ABI (context begin / submit / flush / end) with
           the command stream and the canvas in host memory: host-side recording, the pinned H2D
           upload, the pipeline and the D2H read-back of the canvas are all inside the timed
           region; two recording threads with a context each take the steps in turn and flush
           asynchronously, so recording overlaps rendering (one_at_a_time_ms_per_step: one
           context, one step after the other);
  roofline, cpu_baseline, clocks, gpu_launches as documented in the repository's design notes.

--impl reference times the reference's CPU path for the same workload on this host's cores: the
reference library built from source (when available on this host) with thread_count = cores, or
else the CPU restatement of it, one frame per core in parallel.
"""
from __future__ import annotations

import argparse
import glob
import json
import os
import re
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {   # name -> (config label, seed)
    "curves": ("curves_gradients_1920x1080_20000_cubic_paths", 2),
    "polygons": ("polygons_512x512_2000_solid", 1),
    "patterns": ("patterns_4096x4096_50000_affine_quads", 3),
    "strokes": ("strokes_1920x1080_20000_stroked_cubic_paths", 10),
}
FALLBACK_HBM_GBS = 6800.0
L2_FLUSH_BYTES = 256 << 20


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="curves", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="bounded CPU-baseline sample (seconds)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="frame", choices=["frame", "batch", "serving"],
                    help="frame: one canvas per step (default); batch: many canvases in one pipeline vs one "
                         "pipeline per canvas; serving: Poisson arrivals through the continuous-batching server")
    ap.add_argument("--batch-count", type=int, default=4096, help="canvases of the batched workload")
    ap.add_argument("--batch-scale", type=float, default=1.0, help="path-count scale of the batched workload (1.0: 10-5000 paths per canvas)")
    ap.add_argument("--serve-requests", type=int, default=48, help="requests per arrival-rate point")
    ap.add_argument("--serve-scale", type=float, default=0.05, help="path-count scale of the serving requests")
    ap.add_argument("--serve-rates", default="20,60,200", help="arrival rates (requests/s) to sweep")
    return ap.parse_args(argv)


def make_stream(workload: str) -> tuple[bytes, int, int, int]:
    from blend2d_gb300 import scenes
    sw = scenes.WORKLOADS[workload]()
    return sw.to_bytes(), sw.width, sw.height, sw.fill_count


# --------------------------------------------------------------------------------------------
# distributed plumbing (replicas: every rank renders its own copy of the workload)
# --------------------------------------------------------------------------------------------

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    def __init__(self, world: int, backend: str):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# --------------------------------------------------------------------------------------------
# clocks sampled during the timed region
# --------------------------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv") if os.path.isdir(
            os.path.join(ROOT, "gpurun_out")) else f"/tmp/blgpu_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.25)

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        under_load = [v for v in sm if v > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(under_load), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------------------------
# roofline inputs
# --------------------------------------------------------------------------------------------

def hbm_peak() -> tuple[float, str]:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(workload: str):
    """DRAM bytes per fine-stage launch pair from the committed ncu summary for this workload."""
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", f"fine_stage_{workload}*.md"))):
        m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", open(path).read())
        if m:
            return float(m.group(1)), os.path.relpath(path, ROOT)
    return None, None


# --------------------------------------------------------------------------------------------
# CPU baselines
# --------------------------------------------------------------------------------------------

def _oracle_frames(stream: bytes, seconds: float, max_frames: int = 64):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    oracle_lib.render(stream)      # build + warm up
    n, t0 = 0, time.perf_counter()
    while n < max_frames:
        oracle_lib.render(stream)
        n += 1
        if time.perf_counter() - t0 >= seconds:
            break
    return n, time.perf_counter() - t0


def _oracle_worker(stream: bytes) -> float:
    """Renders one frame with the CPU restatement; returns its wall time."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    t0 = time.perf_counter()
    oracle_lib.render(stream)
    return time.perf_counter() - t0


def cpu_baseline_port(stream: bytes, mpix: float, seconds: float) -> dict:
    n, dt = _oracle_frames(stream, seconds)
    return {"value": round(n * mpix / dt, 3), "unit": "Mpix/s", "cores": 1, "kind": "port",
            "sample": f"{n} full frames of the same workload rendered by the CPU restatement (oracle/), "
                      f"single thread, {dt:.1f} s"}


def reference_binary():
    path = os.path.join(ROOT, "oracle", "_ref", "b2d_replay_default")
    if not os.path.exists(path):
        return None
    try:
        subprocess.run([path], capture_output=True, timeout=10)
    except (OSError, subprocess.TimeoutExpired):
        return None
    return path


# --------------------------------------------------------------------------------------------
# arms
# --------------------------------------------------------------------------------------------

def run_ours(args) -> int:
    import torch

    import blend2d_gb300 as bg

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = Dist(world, "nccl")
    stream, w, h, fills = make_stream(args.workload)
    mpix = w * h / 1e6
    s = torch.cuda.Stream()
    rt = bg.Runtime(0 if world == 1 else local, cuda_stream=s.cuda_stream)
    flush_buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")

    # ---- e2e: public API, host command stream + pinned host canvas, H2D and D2H inside the step.
    # Two recording threads, each with its own context and pinned canvas, take the steps in turn
    # and flush asynchronously: a step is recorded while the steps before it render (the ctypes
    # calls release the GIL, so the two recordings run on two host cores). A context's end()
    # returns when its image holds the result, and the threads end their last frames inside the
    # timed region, so every step's upload, render and read-back is timed.
    import threading
    threads_n = 2
    hosts = [torch.zeros((h, w), dtype=torch.int32).pin_memory() for _ in range(threads_n)]
    ctxs = [bg.Context(rt) for _ in range(threads_n)]

    def e2e_worker(k, count, errors):
        try:
            c = ctxs[k]
            for i in range(count):
                if i:
                    c.end()
                c.begin(hosts[k])
                c.submit_stream(stream)
                c.flush(bg.FLUSH_ASYNC)
            if count:
                c.end()
        except Exception as e:      # re-raised on the main thread
            errors.append(e)

    def e2e_run(steps):
        errors = []
        ths = [threading.Thread(target=e2e_worker, args=(k, len(range(k, steps, threads_n)), errors))
               for k in range(threads_n)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        if errors:
            raise errors[0]

    e2e_run(max(args.warmup, 3))
    dist.barrier()
    t0 = time.perf_counter()
    e2e_run(args.steps)
    e2e_s = dist.max(time.perf_counter() - t0)
    st = rt.stats()
    h2d, d2h = int(st.h2d_bytes), int(st.d2h_bytes)
    pixel_ops, pattern_ops = int(st.pixel_ops), int(st.pattern_ops)
    segments, vertices = int(st.segments), int(st.input_vertices)
    # the same steps one at a time (record, render, read back, then the next), for reference
    seq_t0 = time.perf_counter()
    for _ in range(args.steps):
        ctxs[0].begin(hosts[0])
        ctxs[0].submit_stream(stream)
        ctxs[0].end()
    e2e_seq_s = dist.max(time.perf_counter() - seq_t0)
    for c in ctxs:
        c.close()

    # ---- device-resident: replay the recorded frame (every kernel of the pipeline runs each step)
    with torch.cuda.stream(s):
        for _ in range(max(args.warmup, 3)):
            flush_buf.fill_(1)
            rt.replay(False)
            rt.synchronize()
        dist.barrier()
        torch.cuda.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        fine_ms, comp_ms, launches = [], [], 0
        for i in range(args.steps):
            flush_buf.fill_(i)                      # L2 flush (256 MiB write) outside the timed step
            starts[i].record(s)
            rt.replay(False)
            ends[i].record(s)
            rt.synchronize()
            stt = rt.stats()
            fine_ms.append(stt.last_fine_ms)
            comp_ms.append(stt.last_composite_ms)
            launches += int(stt.kernel_launches)
        torch.cuda.synchronize()
        clock_info = clocks.stop()
        step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
        dist.barrier()
        total_s = dist.max(sum(step_ms) / 1e3)

        # graph replay of the same frame (launch overhead removed), for reference
        graph_ms = []
        for i in range(args.steps):
            flush_buf.fill_(i)
            starts[i].record(s)
            rt.replay(True)
            ends[i].record(s)
        torch.cuda.synchronize()
        graph_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]

        # the reference's pixel-op count (every command composited, no occlusion culling): one
        # untimed replay with culling off, for the algorithmic bytes of the roofline
        cfg0 = rt.launch_config()
        rt.set_launch_config(bg.LaunchConfig(**{**cfg0.as_dict(), "no_occlusion_cull": 1}))
        rt.replay(False)
        rt.synchronize()
        st_all = rt.stats()
        pixel_ops_alg, pattern_ops_alg = int(st_all.pixel_ops), int(st_all.pattern_ops)
        rt.set_launch_config(cfg0)

    value = world * args.steps * mpix / total_s
    e2e_value = world * args.steps * mpix / e2e_s
    fine_s = statistics.mean(fine_ms) / 1e3
    alg_bytes = pixel_ops_alg * 8 + pattern_ops_alg * 4 + segments * 8 + vertices * 16
    peak, peak_kind = hbm_peak()
    achieved = alg_bytes / fine_s / 1e9
    traffic, traffic_src = ncu_traffic(args.workload)

    line = {
        "metric": "Mpix/s", "value": round(value, 3), "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_s * 1e3 / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8x4 (PRGB32); fp64 edges", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload][0], "canvas": [w, h], "fills": fills,
                   "seed": WORKLOADS[args.workload][1], "frames_per_s": round(value / mpix, 3), "paths_per_s": round(value / mpix * fills, 1),
                   "graph_replay_ms_per_step": round(statistics.median(graph_ms), 4),
                   "l2": "flushed between timed steps (256 MiB write, outside the timed region)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": round(e2e_value, 3), "unit": "Mpix/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_s * 1e3 / args.steps, 3),
                "recording_threads": threads_n, "one_at_a_time_ms_per_step": round(e2e_seq_s * 1e3 / args.steps, 3)},
        "gpu_launches": launches,
        "clocks": clock_info,
        "roofline": {"bound": "hbm", "kernel": "fine stage (coverage: coverage_kernel; composite: cull_kernel + fine_kernel)",
                     "achieved": round(achieved, 2), "peak": peak,
                     "peak_kind": f"of {peak_kind}", "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": traffic, "traffic_source": traffic_src,
                     "algorithmic_bytes_per_launch": alg_bytes, "fine_ms": round(fine_s * 1e3, 4),
                     "composite_kernel_ms": round(statistics.mean(comp_ms), 4),
                     "pixel_ops": pixel_ops_alg, "pattern_ops": pattern_ops_alg,
                     "pixel_ops_composited": pixel_ops, "segments": segments,
                     "input_vertices": vertices},
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_port(stream, mpix, args.cpu_seconds)
    rt.close()
    dist.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_reference(args) -> int:
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    stream, w, h, fills = make_stream(args.workload)
    mpix = w * h / 1e6
    cores = os.cpu_count() or 1
    ref = reference_binary()
    times = []
    if ref:
        import tempfile
        with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
            f.write(stream)
            path = f.name
        try:
            for _ in range(args.warmup):
                subprocess.run([ref, path, "-", "--threads", str(cores)], check=True, capture_output=True)
            for _ in range(args.steps):
                out = subprocess.run([ref, path, "-", "--threads", str(cores), "--frames", "1"], check=True,
                                     capture_output=True, text=True).stdout
                times.append(json.loads(out.strip().splitlines()[-1])["median_ms"] / 1e3)
        finally:
            os.unlink(path)
        frames_per_step = 1
        kind, sample = "reference", (f"one full frame per step, reference fixed pipeline built from source "
                                     f"(no JIT), BLContext thread_count={cores}")
    else:
        import multiprocessing as mp
        pool_ctx = mp.get_context("spawn")
        with pool_ctx.Pool(cores) as pool:
            for _ in range(args.warmup):
                pool.map(_oracle_worker, [stream] * cores)
            for _ in range(args.steps):
                t0 = time.perf_counter()
                pool.map(_oracle_worker, [stream] * cores)
                times.append(time.perf_counter() - t0)
        frames_per_step = cores
        kind, sample = "port", (f"per step, {cores} processes each render one full frame of the same workload "
                                f"with the CPU restatement (oracle/); the reference library is not built on this host")
    total = sum(times)
    value = args.steps * frames_per_step * mpix / total
    line = {
        "impl": "reference", "metric": "Mpix/s", "value": round(value, 3), "unit": "Mpix/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8x4 (PRGB32); fp64 edges",
        "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload][0], "canvas": [w, h], "fills": fills,
                   "seed": WORKLOADS[args.workload][1]},
        "cpu_baseline": {"value": round(value, 3), "unit": "Mpix/s", "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_batch(args) -> int:
    """Many independent canvases (width/height log-uniform 32-2048, log-uniform path counts of the
    polygon and cubic-gradient kinds): one device pipeline for all of them (blgpu_render_batch,
    one persistent fine launch over every canvas's tiles) against one pipeline per canvas."""
    import numpy as np
    import torch

    import blend2d_gb300 as bg
    from blend2d_gb300 import scenes

    sws = scenes.batch_canvases(seed=4, count=args.batch_count, scale=args.batch_scale)
    streams = [sw.to_bytes() for sw in sws]
    mpix = sum(sw.width * sw.height for sw in sws) / 1e6
    paths = sum(sw.fill_count for sw in sws)
    s = torch.cuda.Stream()
    rt = bg.Runtime(0, cuda_stream=s.cuda_stream)
    batched = [np.zeros((sw.height, sw.width), dtype=np.uint32) for sw in sws]
    singles = [np.zeros((sw.height, sw.width), dtype=np.uint32) for sw in sws]
    for _ in range(max(1, args.warmup // 2)):
        rt.render_batch(streams, batched)
    steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(steps):
        rt.render_batch(streams, batched)
    batch_s = (time.perf_counter() - t0) / steps
    batch_dev_ms = rt.stats().last_gpu_ms
    batch_launches = int(rt.stats().kernel_launches)
    # device-resident replay of the whole batch as one CUDA graph
    rt.replay(True)
    rt.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(s):
        ev0.record(s)
        for _ in range(steps):
            rt.replay(True)
        ev1.record(s)
    torch.cuda.synchronize()
    graph_ms = ev0.elapsed_time(ev1) / steps
    # one pipeline per canvas, same public API, same host buffers
    for sw_stream, img in zip(streams[:8], singles[:8]):
        bg.render_stream(rt, sw_stream, img)
    dev_ms = 0.0
    t0 = time.perf_counter()
    for sw_stream, img in zip(streams, singles):
        bg.render_stream(rt, sw_stream, img)
        dev_ms += rt.stats().last_gpu_ms
    single_s = time.perf_counter() - t0
    identical = all(np.array_equal(a, b) for a, b in zip(batched, singles))
    line = {
        "metric": "canvases/s", "mode": "batch", "unit": "canvases/s",
        "value": round(len(sws) / batch_s, 2), "higher_is_better": True, "n_gpus": 1, "steps": steps,
        "config": {"workload": f"batch_{len(sws)}_canvases_32-2048px_scale{args.batch_scale}", "canvases": len(sws),
                   "paths": paths, "mpix": round(mpix, 2), "seed": 4},
        "batched": {"e2e_s": round(batch_s, 4), "canvases_per_s": round(len(sws) / batch_s, 2),
                    "mpix_per_s": round(mpix / batch_s, 2), "device_ms": round(batch_dev_ms, 3),
                    "graph_replay_ms": round(graph_ms, 3), "kernel_launches": batch_launches},
        "per_canvas": {"e2e_s": round(single_s, 4), "canvases_per_s": round(len(sws) / single_s, 2),
                       "mpix_per_s": round(mpix / single_s, 2), "device_ms_sum": round(dev_ms, 3)},
        "speedup_e2e": round(single_s / batch_s, 2),
        "speedup_device": round(dev_ms / max(graph_ms, 1e-9), 2),
        "bit_identical": identical,
    }
    rt.close()
    print(json.dumps(line), flush=True)
    return 0 if identical else 1


def run_serving(args) -> int:
    """Poisson arrivals of render requests (square canvases, side log-uniform 64-4096 px, 1-20,000
    log-uniform paths times a scale) through the continuous-batching server; p50/p99 latency and
    Mpix/s per arrival rate."""
    import random

    import blend2d_gb300 as bg  # noqa: F401
    from blend2d_gb300 import scenes
    from blend2d_gb300.serving import RenderServer, percentile

    reqs = [sw.to_bytes() for sw in scenes.serving_requests(seed=5, count=args.serve_requests, scale=args.serve_scale)]
    mpix_req = [int.from_bytes(r[8:12], "little") * int.from_bytes(r[12:16], "little") / 1e6 for r in reqs]
    points = []
    with RenderServer(workers=2, hbm_budget=150 << 30) as srv:
        for f in [srv.submit(r) for r in reqs[:4]]:     # warm-up: device arenas grow once
            f.result()
        for rate in [float(x) for x in args.serve_rates.split(",")]:
            rng = random.Random(int(rate))
            srv.stats.latencies.clear()
            t0 = time.perf_counter()
            futs = []
            t_next = t0
            for r in reqs:
                now = time.perf_counter()
                if t_next > now:
                    time.sleep(t_next - now)
                futs.append(srv.submit(r))
                t_next += rng.expovariate(rate)
            for f in futs:
                f.result()
            wall = time.perf_counter() - t0
            lat = list(srv.stats.latencies)
            points.append({"rate_rps": rate, "requests": len(reqs), "p50_ms": round(1e3 * percentile(lat, 50), 2),
                           "p99_ms": round(1e3 * percentile(lat, 99), 2), "mpix_per_s": round(sum(mpix_req) / wall, 2),
                           "wall_s": round(wall, 3)})
        batches = srv.stats.batches
        max_inflight = srv.stats.max_inflight_bytes
    line = {"metric": "p50/p99 latency and Mpix/s", "mode": "serving", "unit": "ms | Mpix/s", "n_gpus": 1,
            "config": {"workload": f"serving_{len(reqs)}_requests_side64-4096_paths1-20000_scale{args.serve_scale}",
                       "mpix_per_pass": round(sum(mpix_req), 2), "workers": 2, "hbm_budget_gb": 150, "seed": 5},
            "points": points, "batches": batches, "max_inflight_bytes": max_inflight}
    print(json.dumps(line), flush=True)
    return 0


def main(argv=None) -> int:
    args = parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "batch":
        return run_batch(args)
    if args.mode == "serving":
        return run_serving(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
