#!/usr/bin/env python3
"""Benchmark of the GB300 raster backend: batched canvases (headline), one large frame, serving.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--mode headline|batch|frame|serving] [--workload curves|polygons|patterns|strokes]

Headline workload (default): 4,096 independent PRGB32 canvases, width and height each
log-uniform in 32-2,048 px (975 Mpix in all), 10-5,000 paths per canvas (3.33 M in all), each path
a 10-vertex solid polygon or a closed 4-12 cubic path with a linear/radial/conic gradient,
SrcOver/SrcCopy and non-zero/even-odd mixed; seed 4. A step renders every canvas once, all of
them in one device pipeline (one persistent composite launch over every canvas's tiles).

The line of our arm holds:
  value   - Mpix/s of canvas rendered, device-resident: each step replays the whole batch's device
            pipeline (LUTs, edge building, binning, coverage, composite) on inputs already in
            HBM, timed with CUDA events on the pipeline's stream; the inputs (1.5 GB of commands,
            3.9 GB of canvases) are far larger than L2, so nothing is flushed between steps;
  e2e     - the same metric through the public C ABI (blgpu_render_batch) with the command
            streams and the canvases in host memory (pinned): host recording, the upload, the
            pipeline and the read-back of every canvas are inside each step;
  batch   - frames/s (canvases/s) batched and with one pipeline per canvas (the plain per-canvas
            GPU path, same API, same buffers), the speed-ups, the CUDA-graph replay time;
  parity  - "bit-exact" when every batched canvas equals its per-canvas render and a 64-canvas
            sample equals the CPU oracle's render (the sample includes the canvases whose
            reference renders are recorded in tests/golden/golden.json, checked by hash too);
  roofline- the fine stage (coverage + composite) of the batched frame: bytes the timed kernels
            must move (8 B per composited pixel-op, 4 B more per pattern pixel-op, 8 B per
            segment, 16 B per input vertex) over its CUDA-event time, against the measured HBM
            copy bandwidth; the reference's pixel-op count (no occlusion culling) beside it;
  frame   - the 1920x1080 frame of 20,000 cubic gradient paths (seed 2): device and e2e Mpix/s,
            its own roofline and parity against the oracle and the reference's recorded hash;
  serving - Poisson arrivals of 48 requests (square canvases of side 64-4,096 px, 1-20,000 paths
            of the same kinds, seed 5) through the continuous-batching server at three rates:
            p50/p99 latency and Mpix/s, clocks, parity of the recorded requests;
  cpu_baseline, clocks, gpu_launches.

--impl reference times the reference's CPU path on the same workload: the reference library
(fixed pipeline, no JIT; built from source by oracle/ref.mk where its sources are staged) with
BLContext thread_count = host cores, or else the CPU restatement in oracle/ on every core; each
step renders a fixed sample of 64 canvases (every 64th) of the batch.
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
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FRAMES = {   # frame workloads: name -> (label, seed)
    "curves": ("curves_gradients_1920x1080_20000_cubic_paths", 2),
    "polygons": ("polygons_512x512_2000_solid", 1),
    "patterns": ("patterns_4096x4096_50000_affine_quads", 3),
    "strokes": ("strokes_1920x1080_20000_stroked_cubic_paths", 10),
}
BATCH_SEED = 4
BATCH_LABEL = "batch_{n}_canvases_32-2048px_10-5000_paths"
SERVE_SEED = 5
FALLBACK_HBM_GBS = 6800.0
L2_FLUSH_BYTES = 256 << 20
E2E_RUNTIMES = 3          # runtimes taking the batched e2e steps in turn (device-ordered)
DTYPE = "u8x4 (PRGB32); fp64 edges"


def log(msg: str) -> None:
    """Progress on stderr (the JSON line is the only stdout output)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="headline", choices=["headline", "batch", "frame", "serving", "profile"],
                    help="headline: batch line with frame and serving records; batch / frame / serving alone; "
                         "profile: the first --batch-count canvases rendered twice and replayed once, for profilers")
    ap.add_argument("--workload", default="curves", choices=sorted(FRAMES), help="frame workload (--mode frame)")
    ap.add_argument("--batch-count", type=int, default=4096, help="canvases of the batched workload")
    ap.add_argument("--cpu-seconds", type=float, default=8.0, help="bounded CPU-baseline sample of the frame (seconds)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=48, help="requests per arrival-rate point")
    ap.add_argument("--serve-rates", default="20,60,200", help="arrival rates (requests/s) to sweep")
    ap.add_argument("--serve-workers", type=int, default=4, help="worker runtimes of the server")
    return ap.parse_args(argv)


# --------------------------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------------------------

def _canvas_bytes(i: int) -> bytes:
    from blend2d_gb300 import scenes
    return scenes.batch_canvas(i, seed=BATCH_SEED, count=_canvas_bytes.count).to_bytes()


def _gen_init(count):
    _canvas_bytes.count = count


def batch_streams(count: int, indices=None) -> list[bytes]:
    """Command streams of the batched workload (all canvases, or `indices`), generated on every
    host core (each canvas draws from its own seeded generator)."""
    import multiprocessing as mp
    idx = list(range(count)) if indices is None else list(indices)
    procs = max(1, min(os.cpu_count() or 1, 32))
    if len(idx) < 64 or procs == 1:
        _gen_init(count)
        return [_canvas_bytes(i) for i in idx]
    with mp.get_context("spawn").Pool(procs, initializer=_gen_init, initargs=(count,)) as pool:
        return pool.map(_canvas_bytes, idx, chunksize=max(1, len(idx) // (procs * 8)))


def batch_config(count: int) -> dict:
    from blend2d_gb300 import scenes
    specs = scenes.batch_canvas_specs(seed=BATCH_SEED, count=count)
    return {"workload": BATCH_LABEL.format(n=count), "canvases": count,
            "paths": sum(n for _, _, n in specs), "mpix": round(sum(w * h for w, h, _ in specs) / 1e6, 3),
            "seed": BATCH_SEED,
            "l2": "inputs larger than L2 (1.5 GB of command data and 3.9 GB of canvases per step); no flush"}


def frame_config(workload: str, w: int, h: int, fills: int) -> dict:
    return {"workload": FRAMES[workload][0], "canvas": [w, h], "fills": fills, "seed": FRAMES[workload][1],
            "l2": "flushed between timed steps (256 MiB write, outside the timed region)"}


def batch_sample(count: int) -> list[int]:
    """64 canvases checked against the oracle: the ones tests/golden/golden.json records reference
    renders of, then seeded picks."""
    import numpy as np
    golden = [i for i in golden_batch_hashes() if i < count]
    rest = [int(i) for i in np.random.default_rng(404).permutation(count) if int(i) not in golden]
    return sorted(golden + rest[:max(0, min(count, 64) - len(golden))])


def golden_batch_hashes() -> dict:
    """canvas index -> sha256 of the reference's render (default LUT builder) from the golden file."""
    out = {}
    try:
        with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
            g = json.load(f)
    except OSError:
        return out
    for e in g["scenes"]:
        m = re.fullmatch(r"scenes\.batch_canvas\((\d+)\)", e["expr"])
        if m:
            out[int(m.group(1))] = e["pixels_sha256"]["default"]
    return out


def golden_hash(expr: str):
    try:
        with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
            g = json.load(f)
    except OSError:
        return None
    return next((e["pixels_sha256"]["default"] for e in g["scenes"] if e["expr"] == expr), None)


def sha256(a) -> str:
    import hashlib
    import numpy as np
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# --------------------------------------------------------------------------------------------
# distributed plumbing (replicas: every rank renders its own copy of the workload)
# --------------------------------------------------------------------------------------------

def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


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
# clocks sampled during a timed region
# --------------------------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"blgpu_clocks_{os.getpid()}_{id(self)}.csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.25)
        return self

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
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
        try:
            os.unlink(self.path)
        except OSError:
            pass
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


def ncu_traffic(name: str):
    """DRAM bytes of the fine stage per frame, from the committed ncu summary for this workload."""
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", f"fine_stage_{name}*.md"))):
        with open(path) as f:
            m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", f.read())
        if m:
            return float(m.group(1)), os.path.relpath(path, ROOT)
    return None, None


def roofline(st_culled, st_ref, fine_ms: float, comp_ms: float, traffic_name: str) -> dict:
    """Fine-stage roofline: bytes the timed kernels must move over their CUDA-event time."""
    ops, pat = int(st_culled.pixel_ops), int(st_culled.pattern_ops)
    segs, verts = int(st_culled.segments), int(st_culled.input_vertices)
    alg = ops * 8 + pat * 4 + segs * 8 + verts * 16
    peak, kind = hbm_peak()
    achieved = alg / (fine_ms / 1e3) / 1e9
    traffic, src = ncu_traffic(traffic_name)
    return {"bound": "hbm", "kernel": "fine stage (coverage: coverage_kernel; composite: cull_kernel + fine_kernel)",
            "achieved": round(achieved, 2), "peak": peak, "peak_kind": f"of {kind}", "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic, "traffic_source": src,
            "algorithmic_bytes_per_launch": alg, "fine_ms": round(fine_ms, 4), "composite_kernel_ms": round(comp_ms, 4),
            "pixel_ops_composited": ops, "pattern_ops_composited": pat, "segments": segs, "input_vertices": verts,
            "pixel_ops_reference": int(st_ref.pixel_ops), "pattern_ops_reference": int(st_ref.pattern_ops)}


# --------------------------------------------------------------------------------------------
# CPU renders (reference library or oracle): baselines and the parity checker
# --------------------------------------------------------------------------------------------

def reference_binary():
    """The reference's replay harness built by oracle/ref.mk on this host, if any."""
    for variant in ("native", "default"):
        path = os.path.join(ROOT, "oracle", "_ref", f"b2d_replay_{variant}")
        if not os.path.exists(path):
            continue
        try:
            subprocess.run([path], capture_output=True, timeout=10)
        except (OSError, subprocess.TimeoutExpired):
            continue
        return path, variant
    return None, None


def reference_times(ref: str, streams: list[bytes], threads: int, repeat: int) -> list[float]:
    """Wall seconds of each of `repeat` passes of the reference over `streams`."""
    with tempfile.TemporaryDirectory() as td:
        paths = []
        for i, s in enumerate(streams):
            p = os.path.join(td, f"{i}.bin")
            with open(p, "wb") as f:
                f.write(s)
            paths.append(p)
        lst = os.path.join(td, "list.txt")
        with open(lst, "w") as f:
            f.write("\n".join(paths) + "\n")
        out = subprocess.run([ref, "--batch", lst, "--threads", str(threads), "--repeat", str(repeat)],
                             check=True, capture_output=True, text=True).stdout
    return [t / 1e3 for t in json.loads(out.strip().splitlines()[-1])["times_ms"]]


def oracle_renders(streams: list[bytes], threads: int):
    """CPU-oracle renders of `streams` on `threads` host threads (its ctypes calls release the
    GIL); returns (images, wall seconds)."""
    from concurrent.futures import ThreadPoolExecutor
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    oracle_lib.lib()
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        imgs = list(ex.map(oracle_lib.render, streams))
    return imgs, time.perf_counter() - t0


def cpu_baseline(streams: list[bytes], mpix: float, what: str) -> dict:
    cores = os.cpu_count() or 1
    ref, variant = reference_binary()
    if ref:
        t = reference_times(ref, streams, cores, 2)[-1]
        return {"value": round(mpix / t, 3), "unit": "Mpix/s", "cores": cores, "kind": "reference",
                "sample": f"{what}, rendered by the reference library (fixed pipeline, no JIT, build '{variant}') "
                          f"with BLContext thread_count={cores}, {t:.2f} s"}
    _, t = oracle_renders(streams, cores)
    return {"value": round(mpix / t, 3), "unit": "Mpix/s", "cores": cores, "kind": "port",
            "sample": f"{what}, rendered by the CPU restatement (oracle/) on {cores} threads, one canvas per "
                      f"thread, {t:.2f} s"}


def parity_text(bad_pixels: int, bad_items: list) -> str:
    if not bad_pixels and not bad_items:
        return "bit-exact"
    return f"{bad_pixels} pixels differ" + (f" ({', '.join(bad_items[:8])})" if bad_items else "")


# --------------------------------------------------------------------------------------------
# our arm
# --------------------------------------------------------------------------------------------

def pinned_canvas(h: int, w: int):
    import torch
    return torch.zeros((h, w), dtype=torch.int32).pin_memory()


def time_replays(rt, s, steps: int, warmup: int, flush_buf=None):
    """CUDA-event times (ms) of `steps` eager replays of the runtime's last frame, with the
    fine-stage and composite times and the kernel launches of each."""
    import torch
    with torch.cuda.stream(s):
        for _ in range(warmup):
            if flush_buf is not None:
                flush_buf.fill_(1)
            rt.replay(False)
            rt.synchronize()
        torch.cuda.synchronize()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        fine, comp, launches = [], [], 0
        clocks = ClockSampler(torch.cuda.current_device()).start()
        for i in range(steps):
            if flush_buf is not None:
                flush_buf.fill_(i)                   # L2 flush, outside the timed step
            starts[i].record(s)
            rt.replay(False)
            ends[i].record(s)
            rt.synchronize()
            st = rt.stats()
            fine.append(st.last_fine_ms)
            comp.append(st.last_composite_ms)
            launches += int(st.kernel_launches)
        torch.cuda.synchronize()
        clock_info = clocks.stop()
    return [a.elapsed_time(b) for a, b in zip(starts, ends)], fine, comp, launches, clock_info


def graph_replay_ms(rt, s, steps: int) -> float:
    import torch
    with torch.cuda.stream(s):
        rt.replay(True)
        rt.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(steps):
            rt.replay(True)
        e1.record(s)
        torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def reference_op_counts(rt, bg):
    """The frame's pixel-op counts with occlusion culling off (the reference's work): one
    untimed replay."""
    cfg0 = rt.launch_config()
    rt.set_launch_config(bg.LaunchConfig(**{**cfg0.as_dict(), "no_occlusion_cull": 1}))
    rt.replay(False)
    rt.synchronize()
    st = rt.stats()
    rt.set_launch_config(cfg0)
    rt.replay(False)
    rt.synchronize()
    return st


def batch_record(args, dist, local, cpu: bool) -> dict:
    import numpy as np
    import torch

    import blend2d_gb300 as bg

    n = args.batch_count
    cfg = batch_config(n)
    mpix = cfg["mpix"]
    world = dist.world
    t_gen = time.perf_counter()
    streams = batch_streams(n)
    gen_s = time.perf_counter() - t_gen
    log(f"batch: {n} canvases generated in {gen_s:.1f} s")
    shapes = [tuple(int(v) for v in np.frombuffer(s[8:16], dtype="<u4"))[::-1] for s in streams]   # (h, w)
    s = torch.cuda.Stream()
    rt = bg.Runtime(local, cuda_stream=s.cuda_stream)
    targets = [pinned_canvas(h, w) for h, w in shapes]
    log("batch: pinned canvases allocated")

    # ---- e2e through the public API: host streams, pinned host canvases, one pipeline per step.
    # One eager step first (every array sized from the frame, a host read-back between the
    # halves), for reference. Then three runtimes (each its own stream, arenas and pinned canvases)
    # take the steps in turn from three host threads with graph frames (a step's data is uploaded
    # in place and one captured graph replayed), so a step's host recording and copies overlap the
    # device work of the steps before. Their kernels run one frame after another (device_order):
    # two frames' kernels at once only slow each other down. Every step's upload, render and
    # read-back is inside the timed region.
    import threading
    rt.render_batch(streams, targets)
    # launch shapes and the command-list row height chosen by the autotuner on this batch
    tuned, tuned_ms = rt.autotune(trials=1)
    log(f"batch: autotuned {tuned.as_dict()} ({tuned_ms:.1f} ms)")
    t0 = time.perf_counter()
    rt.render_batch(streams, targets)
    eager_step_s = time.perf_counter() - t0
    cfg0 = rt.launch_config()
    graph_cfg = bg.LaunchConfig(**{**cfg0.as_dict(), "graph_frames": 1, "device_order": 1})
    rts = [rt] + [bg.Runtime(local) for _ in range(E2E_RUNTIMES - 1)]
    tgts = [targets] + [[pinned_canvas(h, w) for h, w in shapes] for _ in range(E2E_RUNTIMES - 1)]
    for r_ in rts:
        r_.set_launch_config(graph_cfg)

    def e2e_steps(count):
        errors = []

        def worker(k):
            try:
                for _ in range(k, count, E2E_RUNTIMES):
                    rts[k].render_batch(streams, tgts[k])
            except Exception as e:      # re-raised on the main thread
                errors.append(e)
        ths = [threading.Thread(target=worker, args=(k,)) for k in range(E2E_RUNTIMES)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        if errors:
            raise errors[0]

    # two warm-up steps per runtime at least: a runtime's first graph-frame call renders eagerly to
    # size its arrays, and its second grows them to capacity and captures the graph (frees and
    # allocations that wait for the whole device); neither belongs in the timed steps
    e2e_steps(max(args.warmup, 2 * E2E_RUNTIMES))
    g0 = sum(int(r_.stats().graph_frames) for r_ in rts)
    dist.barrier()
    clocks = ClockSampler(local).start()
    t0 = time.perf_counter()
    e2e_steps(args.steps)
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e_clocks = clocks.stop()
    graph_steps = sum(int(r_.stats().graph_frames) for r_ in rts) - g0
    stb = rt.stats()
    host_split = {"record_ms": round(stb.last_record_ms, 2), "merge_ms": round(stb.last_merge_ms, 2),
                  "upload_ms": round(stb.last_upload_ms, 2), "run_ms": round(stb.last_run_ms, 2)}
    log(f"batch: last step host split {host_split}")
    log(f"batch: e2e {e2e_s * 1e3 / args.steps:.1f} ms/step ({graph_steps} graph frames), eager step {eager_step_s * 1e3:.1f} ms")
    st = rt.stats()
    h2d, d2h = int(st.h2d_bytes), int(st.d2h_bytes)
    batch_dev_ms = float(st.last_gpu_ms)
    # every runtime's canvases equal the first one's
    mismatched2 = sorted({i for t in tgts[1:] for i, (a, b) in enumerate(zip(tgts[0], t))
                          if not np.array_equal(a.numpy(), b.numpy())})
    for r_ in rts[1:]:
        r_.close()
    for t in tgts[1:]:
        del t[:]
    rt.set_launch_config(cfg0)
    rt.render_batch(streams, targets)       # the eager frame the replays below time

    # ---- device-resident: the batch's device pipeline replayed on its inputs in HBM
    step_ms, fine_ms, comp_ms, launches, dev_clocks = time_replays(rt, s, args.steps, args.warmup)
    dist.barrier()
    total_s = dist.max(sum(step_ms) / 1e3)
    st_culled = rt.stats()
    log(f"batch: device {total_s * 1e3 / args.steps:.1f} ms/step")
    g_ms = graph_replay_ms(rt, s, 3)
    st_ref = reference_op_counts(rt, bg)
    roof = roofline(st_culled, st_ref, statistics.mean(fine_ms), statistics.mean(comp_ms), "batch")

    # ---- the plain per-canvas GPU path: one pipeline per canvas, same API, same buffers
    batched = [t.numpy().view(np.uint32).copy() for t in targets]
    for i in range(min(8, n)):
        bg.render_stream(rt, streams[i], targets[i])
    dev_sum = 0.0
    clocks = ClockSampler(local).start()
    t0 = time.perf_counter()
    for stream, t in zip(streams, targets):
        bg.render_stream(rt, stream, t)
        dev_sum += rt.stats().last_gpu_ms
    single_s = time.perf_counter() - t0
    single_clocks = clocks.stop()
    log(f"batch: per-canvas pass {single_s:.1f} s")
    mismatched = [i for i, (a, t) in enumerate(zip(batched, targets)) if not np.array_equal(a, t.numpy().view(np.uint32))]
    mismatched += [i for i in mismatched2 if i not in mismatched]

    # ---- parity of a 64-canvas sample against the oracle (and the golden reference hashes)
    sample = batch_sample(n)
    bad_px, bad = 0, [f"canvas {i}: batched != per-canvas" for i in mismatched[:4]]
    bad_px += sum(int(np.count_nonzero(batched[i] != targets[i].numpy().view(np.uint32))) for i in mismatched)
    for i, h in golden_batch_hashes().items():
        if i < n and sha256(batched[i]) != h:
            bad.append(f"canvas {i}: reference hash")
    if cpu:
        want, _ = oracle_renders([streams[i] for i in sample], os.cpu_count() or 1)
        for i, w_ in zip(sample, want):
            d = int(np.count_nonzero(batched[i] != w_))
            if d:
                bad_px += d
                bad.append(f"canvas {i}: oracle")
    rt.close()
    log(f"batch: parity checked ({len(bad)} findings)")

    rec = {
        "metric": "Mpix/s", "value": round(world * args.steps * mpix / total_s, 3), "unit": "Mpix/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_s * 1e3 / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE, "data": "synthetic", "config": cfg,
        "e2e": {"value": round(world * args.steps * mpix / e2e_s, 3), "unit": "Mpix/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_s * 1e3 / args.steps, 3), "clocks": e2e_clocks,
                "graph_frames": graph_steps, "eager_ms_per_step": round(eager_step_s * 1e3, 3),
                "pipelining": f"{E2E_RUNTIMES} runtimes take the steps in turn from {E2E_RUNTIMES} host threads; their kernels run one frame after another (device_order), their copies (DMA) overlap",
                "host_split_of_a_step": host_split},
        "gpu_launches": launches,
        "clocks": dev_clocks,
        "roofline": roof,
        "parity": parity_text(bad_px, bad),
        "parity_detail": {"batched_vs_per_canvas": f"{n - len(mismatched)}/{n} identical",
                          "oracle_sample": len(sample) if cpu else 0,
                          "reference_hashes": len([i for i in golden_batch_hashes() if i < n])},
        "batch": {
            "frames_per_s": round(world * args.steps * n / total_s, 2),
            "e2e_frames_per_s": round(world * args.steps * n / e2e_s, 2),
            "graph_replay_ms": round(g_ms, 3), "device_ms_per_batch": round(batch_dev_ms, 3),
            "kernel_launches_per_batch": int(st_culled.kernel_launches),
            "per_canvas": {"e2e_s": round(single_s, 3), "frames_per_s": round(n / single_s, 2),
                           "mpix_per_s": round(mpix / single_s, 3), "device_ms_sum": round(dev_sum, 3),
                           "clocks": single_clocks},
            "speedup_e2e": round(single_s / (e2e_s / args.steps), 2),
            "speedup_device": round(dev_sum / (total_s * 1e3 / args.steps), 2),
            "speedup_device_graph": round(dev_sum / g_ms, 2),
            "stream_generation_s": round(gen_s, 2),
            "autotuned_config": {k: v for k, v in tuned.as_dict().items() if k not in ("graph_frames", "max_segments", "device_order")},
        },
    }
    if cpu:
        ref_sample = [streams[i] for i in range(0, n, 64)]
        smpix = sum(h * w for h, w in shapes[::64]) / 1e6
        rec["cpu_baseline"] = cpu_baseline(ref_sample, smpix, f"every 64th canvas of the batch ({len(ref_sample)} "
                                           f"canvases, {smpix:.1f} Mpix), one pass")
    return rec


def frame_record(args, dist, local, workload: str, cpu: bool) -> dict:
    import threading

    import numpy as np
    import torch

    import blend2d_gb300 as bg
    from blend2d_gb300 import scenes

    sw = scenes.WORKLOADS[workload]()
    stream, w, h, fills = sw.to_bytes(), sw.width, sw.height, sw.fill_count
    mpix = w * h / 1e6
    world = dist.world
    s = torch.cuda.Stream()
    rt = bg.Runtime(local, cuda_stream=s.cuda_stream)
    flush_buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")

    # e2e: two recording threads, each with its own context and pinned canvas, take the steps in
    # turn and flush asynchronously, so a step is recorded while the one before renders; every
    # step's upload, render and read-back is inside the timed region. Graph frames: each step's
    # frame is uploaded in place and runs as one captured graph, with no host round trip inside it.
    cfg0 = rt.launch_config()
    rt.set_launch_config(bg.LaunchConfig(**{**cfg0.as_dict(), "graph_frames": 1}))
    threads_n = 2
    hosts = [pinned_canvas(h, w) for _ in range(threads_n)]
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

    e2e_run(max(args.warmup, 8))        # every context's two recording buffers warmed up
    dist.barrier()
    t0 = time.perf_counter()
    e2e_run(args.steps)
    e2e_s = dist.max(time.perf_counter() - t0)
    st = rt.stats()
    h2d, d2h = int(st.h2d_bytes), int(st.d2h_bytes)
    seq_t0 = time.perf_counter()
    for _ in range(args.steps):
        ctxs[0].begin(hosts[0])
        ctxs[0].submit_stream(stream)
        ctxs[0].end()
    e2e_seq_s = dist.max(time.perf_counter() - seq_t0)
    got = hosts[0].numpy().view(np.uint32).copy()
    for c in ctxs:
        c.close()
    rt.set_launch_config(cfg0)
    ctx = bg.Context(rt, hosts[0])       # the eager frame the replays below time
    ctx.submit_stream(stream)
    ctx.end()
    ctx.close()

    step_ms, fine_ms, comp_ms, launches, clocks = time_replays(rt, s, args.steps, args.warmup, flush_buf)
    dist.barrier()
    total_s = dist.max(sum(step_ms) / 1e3)
    st_culled = rt.stats()
    g_ms = graph_replay_ms(rt, s, args.steps)
    st_ref = reference_op_counts(rt, bg)
    rt.close()

    bad_px, bad = 0, []
    want_hash = golden_hash(f"scenes.{scenes.WORKLOADS[workload].__name__}()")
    if want_hash and sha256(got) != want_hash:
        bad.append("reference hash")
    rec = {
        "metric": "Mpix/s", "value": round(world * args.steps * mpix / total_s, 3), "unit": "Mpix/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_s * 1e3 / args.steps, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE, "data": "synthetic", "config": frame_config(workload, w, h, fills),
        "e2e": {"value": round(world * args.steps * mpix / e2e_s, 3), "unit": "Mpix/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_s * 1e3 / args.steps, 3),
                "recording_threads": threads_n, "one_at_a_time_ms_per_step": round(e2e_seq_s * 1e3 / args.steps, 3)},
        "gpu_launches": launches,
        "clocks": clocks,
        "roofline": roofline(st_culled, st_ref, statistics.mean(fine_ms), statistics.mean(comp_ms), workload),
        "frames_per_s": round(world * args.steps / total_s, 3),
        "paths_per_s": round(world * args.steps * fills / total_s, 1),
        "graph_replay_ms_per_step": round(g_ms, 4),
    }
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_lib
        t0 = time.perf_counter()
        want = oracle_lib.render(stream)
        one = time.perf_counter() - t0
        d = int(np.count_nonzero(got != want))
        if d:
            bad_px += d
            bad.append("oracle")
        reps = max(1, min(64, int(args.cpu_seconds / max(one, 1e-3))))
        rec["cpu_baseline"] = cpu_baseline([stream] * reps, mpix * reps, f"{reps} full frames of the same workload")
    rec["parity"] = parity_text(bad_px, bad)
    log(f"frame {workload}: done")
    return rec


def serving_record(args, local) -> dict:
    import random

    import numpy as np

    from blend2d_gb300 import scenes
    from blend2d_gb300.serving import RenderServer, percentile

    reqs = [sw.to_bytes() for sw in scenes.serving_requests(seed=SERVE_SEED, count=args.serve_requests)]
    mpix_req = [int.from_bytes(r[8:12], "little") * int.from_bytes(r[12:16], "little") / 1e6 for r in reqs]
    points = []
    results = {}
    clocks = ClockSampler(local).start()
    with RenderServer(workers=args.serve_workers, hbm_budget=150 << 30, device=local) as srv:
        for f in [srv.submit(r) for r in reqs[:2 * args.serve_workers]]:     # warm-up: device arenas grow
            f.result()
        log("serving: warmed up")
        for rate in [float(x) for x in args.serve_rates.split(",")]:
            rng = random.Random(int(rate))
            srv.stats.latencies.clear()
            t0 = time.perf_counter()
            futs, t_next = [], t0
            for r in reqs:
                now = time.perf_counter()
                if t_next > now:
                    time.sleep(t_next - now)
                futs.append(srv.submit(r))
                t_next += rng.expovariate(rate)
            imgs = [f.result() for f in futs]
            wall = time.perf_counter() - t0
            lat = list(srv.stats.latencies)
            points.append({"rate_rps": rate, "requests": len(reqs), "p50_ms": round(1e3 * percentile(lat, 50), 2),
                           "p99_ms": round(1e3 * percentile(lat, 99), 2),
                           "mpix_per_s": round(sum(mpix_req) / wall, 2), "wall_s": round(wall, 3)})
            for i in range(len(reqs)):
                results.setdefault(i, []).append(imgs[i])
        st = srv.stats
    clock_info = clocks.stop()
    bad = []
    for i, imgs in results.items():
        if any(not np.array_equal(imgs[0], x) for x in imgs[1:]):
            bad.append(f"request {i}: differs between rates")
        h = golden_hash(f"scenes.serving_request({i})")
        if h and sha256(imgs[0]) != h:
            bad.append(f"request {i}: reference hash")
    return {"metric": "p50/p99 latency (ms) and Mpix/s", "unit": "ms | Mpix/s",
            "config": {"workload": f"serving_{len(reqs)}_requests_side64-4096_paths1-20000",
                       "mpix_per_pass": round(sum(mpix_req), 2), "paths_per_pass": sum(
                           scenes.serving_request_specs(seed=SERVE_SEED, count=args.serve_requests)[i][1]
                           for i in range(len(reqs))),
                       "workers": args.serve_workers, "hbm_budget_gb": 150, "seed": SERVE_SEED},
            "points": points, "batches": st.batches, "max_inflight_bytes": st.max_inflight_bytes,
            "clocks": clock_info, "parity": "bit-exact" if not bad else "; ".join(bad[:6])}


def run_profile(args) -> int:
    """A short, single-process run for profilers: the first --batch-count canvases of the batched
    workload (generated in this process) rendered twice through blgpu_render_batch, then the
    batch's device pipeline replayed once; prints the device times."""
    import numpy as np

    import blend2d_gb300 as bg
    from blend2d_gb300 import scenes

    n = args.batch_count
    streams = [scenes.batch_canvas(i, seed=BATCH_SEED, count=4096).to_bytes() for i in range(n)]
    shapes = [tuple(int(v) for v in np.frombuffer(s[8:16], dtype="<u4"))[::-1] for s in streams]
    targets = [np.zeros(sh, dtype=np.uint32) for sh in shapes]
    out = {"canvases": n}
    with bg.Runtime(0) as rt:
        for k in range(2):
            t0 = time.perf_counter()
            rt.render_batch(streams, targets)
            wall = time.perf_counter() - t0
        st = rt.stats()
        out.update(device_ms=round(st.last_gpu_ms, 3), launches=int(st.kernel_launches), segments=int(st.segments),
                   pixel_ops=int(st.pixel_ops), host_call_ms=round(wall * 1e3, 3), record_ms=round(st.last_record_ms, 3),
                   merge_ms=round(st.last_merge_ms, 3), upload_ms=round(st.last_upload_ms, 3),
                   run_ms=round(st.last_run_ms, 3))
        rt.replay(False)
        rt.synchronize()
        st = rt.stats()
        out.update(replay_ms=round(st.last_gpu_ms, 3), fine_ms=round(st.last_fine_ms, 3),
                   composite_ms=round(st.last_composite_ms, 3))
    print(json.dumps(out), flush=True)
    return 0


def run_ours(args) -> int:
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = Dist(world, "nccl")
    cpu = rank == 0 and world == 1 and not args.no_cpu_baseline
    if args.mode in ("headline", "batch"):
        line = batch_record(args, dist, local, cpu)
        if args.mode == "headline":
            line["frame"] = frame_record(args, dist, local, "curves", cpu)
            if rank == 0:
                line["serving"] = serving_record(args, local)
    elif args.mode == "frame":
        line = frame_record(args, dist, local, args.workload, cpu)
    else:
        line = serving_record(args, local)
    dist.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------------------------
# reference arm
# --------------------------------------------------------------------------------------------

def run_reference(args) -> int:
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    if args.mode == "frame":
        from blend2d_gb300 import scenes
        sw = scenes.WORKLOADS[args.workload]()
        streams = [sw.to_bytes()]
        mpix = sw.width * sw.height / 1e6
        cfg = frame_config(args.workload, sw.width, sw.height, sw.fill_count)
        what = "one full frame of the workload per step"
    else:
        n = args.batch_count
        idx = list(range(0, n, 64))
        streams = batch_streams(n, idx)
        mpix = sum(int.from_bytes(s[8:12], "little") * int.from_bytes(s[12:16], "little") for s in streams) / 1e6
        cfg = batch_config(n)
        what = f"per step, every 64th canvas of the batch ({len(idx)} canvases, {mpix:.1f} Mpix)"
    ref, variant = reference_binary()
    if ref:
        times = reference_times(ref, streams, cores, args.warmup + args.steps)[args.warmup:]
        kind = "reference"
        sample = f"{what}, reference library (fixed pipeline, no JIT; build '{variant}') with BLContext thread_count={cores}"
    else:
        times = []
        for k in range(args.warmup + args.steps):
            _, t = oracle_renders(streams, cores)
            if k >= args.warmup:
                times.append(t)
        kind = "port"
        sample = f"{what}, CPU restatement (oracle/) on {cores} threads, one canvas per thread"
    total = sum(times)
    value = args.steps * mpix / total
    line = {
        "impl": "reference", "metric": "Mpix/s", "value": round(value, 3), "unit": "Mpix/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": DTYPE, "data": "synthetic",
        "config": cfg,
        "cpu_baseline": {"value": round(value, 3), "unit": "Mpix/s", "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main(argv=None) -> int:
    args = parse_args(argv)
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "profile":
        return run_profile(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
