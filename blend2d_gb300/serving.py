"""Continuous-batching render server over the batched C ABI entry point.

Requests (one command stream each, rendered into a new PRGB32 image) are admitted while earlier
batches are still on the GPU: a scheduler thread forms a batch from the waiting requests as soon
as a worker is free and the batch fits the HBM budget. Each worker owns a `Runtime` (its own CUDA
stream and device arenas, kept resident and reused across batches), so batches on different
workers overlap on the device. Every request's pixels are the same as when it is rendered alone:
canvases of one batch share no state (each has its own tiles, commands, styles and LUTs).

Admission is by device bytes. A worker's arenas stay allocated between batches and only grow, so
the server charges every worker what its runtime actually holds (`Runtime.memory()`), and a
batch may start on a worker when the other workers' holdings plus the larger of this worker's
holding and the batch's need fit the budget. A batch's need is estimated per request from its
canvas pixels and stream bytes with coefficients fitted to what the runtimes report each batch
used (inputs, canvases, segments, binning lists), taking the largest ratio seen so the estimate
stays an upper bound of the batches observed.

    server = RenderServer(workers=4, hbm_budget=150 << 30)
    fut = server.submit(stream_bytes)
    image = fut.result()          # (h, w) uint32 PRGB32
    server.close()
"""
from __future__ import annotations

import collections
import struct
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np


def stream_size(stream: bytes) -> tuple[int, int]:
    w, h = struct.unpack_from("<II", stream, 8)
    return w, h


class FootprintModel:
    """Device bytes of a request: per_px * canvas pixels + per_byte * stream bytes + fixed, with the
    two coefficients raised whenever a finished batch used more than the model predicted."""

    def __init__(self, per_px: float = 4.0, per_byte: float = 24.0, fixed: int = 1 << 16):
        self.per_px, self.per_byte, self.fixed = per_px, per_byte, fixed
        self.lock = threading.Lock()

    def estimate(self, stream: bytes) -> int:
        w, h = stream_size(stream)
        with self.lock:
            return int(self.per_px * w * h + self.per_byte * len(stream)) + self.fixed

    def observe(self, streams: list[bytes], used_bytes: int) -> None:
        px = sum(stream_size(s)[0] * stream_size(s)[1] for s in streams)
        nb = sum(len(s) for s in streams)
        with self.lock:
            predicted = self.per_px * px + self.per_byte * nb + self.fixed * len(streams)
            if used_bytes > predicted > 0:
                k = used_bytes / predicted
                self.per_px *= k
                self.per_byte *= k


_DEFAULT_MODEL = FootprintModel()


def footprint_bytes(stream: bytes) -> int:
    """Initial estimate of the device memory one request needs inside a batch (the server's model
    refines it from the bytes its runtimes report)."""
    return _DEFAULT_MODEL.estimate(stream)


@dataclass
class Request:
    stream: bytes
    future: Future
    footprint: int
    t_submit: float
    t_start: float = 0.0
    t_done: float = 0.0
    image: np.ndarray | None = None


@dataclass
class ServerStats:
    completed: int = 0
    batches: int = 0
    pixels: int = 0
    max_inflight_bytes: int = 0      # most device bytes charged at once (holdings and running needs)
    max_held_bytes: int = 0          # most device bytes the runtimes held at once
    releases: int = 0                # idle workers that gave their arenas back to admit a batch
    latencies: list = field(default_factory=list)
    batch_sizes: list = field(default_factory=list)


class RenderServer:
    """Admission by device bytes + continuous batching across `workers` runtimes.

    `runtime_factory` builds one renderer per worker; it must return an object with
    `render_batch(streams, targets)` (blend2d_gb300.Runtime does) and may have `memory()`
    (device bytes it holds and its last frame used); tests inject a fake.
    """

    def __init__(self, workers: int = 4, hbm_budget: int = 150 << 30, max_batch: int = 256,
                 runtime_factory=None, device: int = 0):
        if runtime_factory is None:
            from . import Runtime

            def runtime_factory():
                return Runtime(device)
        self.hbm_budget = int(hbm_budget)
        self.max_batch = int(max_batch)
        self.model = FootprintModel()
        self._runtimes = [runtime_factory() for _ in range(workers)]
        self._free = list(range(workers))
        self._held = [0] * workers            # device bytes each worker's runtime holds
        self._need = [0] * workers            # estimated need of the batch a worker runs (0: idle)
        self._waiting: collections.deque[Request] = collections.deque()
        self._cv = threading.Condition()
        self._closing = False
        self.stats = ServerStats()
        self._scheduler = threading.Thread(target=self._schedule, name="blgpu-scheduler", daemon=True)
        self._scheduler.start()

    # -- client side --------------------------------------------------------------------------
    def submit(self, stream: bytes) -> Future:
        fut: Future = Future()
        req = Request(stream, fut, self.model.estimate(stream), time.perf_counter())
        if req.footprint > self.hbm_budget:
            fut.set_exception(MemoryError(f"request needs ~{req.footprint} B, above the {self.hbm_budget} B budget"))
            return fut
        with self._cv:
            if self._closing:
                raise RuntimeError("server is closed")
            self._waiting.append(req)
            self._cv.notify_all()
        return fut

    def close(self):
        with self._cv:
            self._closing = True
            self._cv.notify_all()
        self._scheduler.join()
        for rt in self._runtimes:
            close = getattr(rt, "close", None)
            if close:
                close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- scheduler ----------------------------------------------------------------------------
    def _committed(self) -> int:
        """Device bytes charged now: what every worker holds, or its running batch's need if
        larger (called under the lock)."""
        return sum(max(h, n) for h, n in zip(self._held, self._need))

    def _take_batch(self, worker: int) -> list[Request]:
        """FIFO batch for `worker` that fits the budget next to the other workers (under the lock)."""
        others = self._committed() - max(self._held[worker], self._need[worker])
        batch, need = [], 0
        while self._waiting and len(batch) < self.max_batch:
            req = self._waiting[0]
            if others + max(self._held[worker], need + req.footprint) > self.hbm_budget:
                break
            batch.append(self._waiting.popleft())
            need += req.footprint
        return batch

    def _schedule(self):
        workers: list[threading.Thread] = []
        while True:
            with self._cv:
                while True:
                    if self._closing and not self._waiting and len(self._free) == len(self._runtimes):
                        for t in workers:
                            t.join()
                        return
                    batch, worker = [], -1
                    if self._free and self._waiting:
                        # the free worker that already holds the most memory goes first: its
                        # arenas absorb the batch without growing the total
                        worker = max(self._free, key=lambda w: self._held[w])
                        batch = self._take_batch(worker)
                        if not batch:
                            idle = [w for w in self._free if self._held[w] > 0]
                            if idle:
                                # the first waiting request does not fit next to what the workers
                                # hold: idle workers give their arenas back, then try again
                                for w in idle:
                                    self._release(w)
                                continue
                            if len(self._free) == len(self._runtimes):
                                # nothing runs and nothing is held: it can never fit
                                req = self._waiting.popleft()
                                req.future.set_exception(MemoryError(
                                    f"request needs ~{req.footprint} B, above the {self.hbm_budget} B budget"))
                                continue
                    if batch:
                        break
                    self._cv.wait(timeout=0.05)
                self._free.remove(worker)
                self._need[worker] = sum(r.footprint for r in batch)
                self.stats.max_inflight_bytes = max(self.stats.max_inflight_bytes, self._committed())
            t = threading.Thread(target=self._run_batch, args=(worker, batch), daemon=True)
            t.start()
            workers = [w for w in workers if w.is_alive()] + [t]

    def _release(self, worker: int):
        """Frees an idle worker's device arenas (under the lock; the worker is not running)."""
        release = getattr(self._runtimes[worker], "release_memory", None)
        if release is not None:
            release()
        self._held[worker] = 0
        self.stats.releases += 1

    def _run_batch(self, worker: int, batch: list[Request]):
        t0 = time.perf_counter()
        for r in batch:
            r.t_start = t0
            w, h = stream_size(r.stream)
            r.image = np.zeros((h, w), dtype=np.uint32)
        error = None
        rt = self._runtimes[worker]
        try:
            rt.render_batch([r.stream for r in batch], [r.image for r in batch])
        except Exception as e:  # noqa: BLE001 - delivered to every request of the batch
            error = e
        held, used = None, None
        mem = getattr(rt, "memory", None)
        if mem is not None:
            try:
                m = mem()
                held, used = int(m.reserved_bytes), int(m.last_frame_bytes)
            except Exception:  # noqa: BLE001 - a failed query keeps the estimate
                pass
        if error is None and used:
            self.model.observe([r.stream for r in batch], used)
        t1 = time.perf_counter()
        with self._cv:
            self._held[worker] = held if held is not None else max(self._held[worker], self._need[worker])
            self._need[worker] = 0
            self._free.append(worker)
            self.stats.batches += 1
            self.stats.batch_sizes.append(len(batch))
            self.stats.max_held_bytes = max(self.stats.max_held_bytes, sum(self._held))
            for r in batch:
                r.t_done = t1
                if error is None:
                    self.stats.completed += 1
                    self.stats.pixels += r.image.size
                    self.stats.latencies.append(t1 - r.t_submit)
            self._cv.notify_all()
        for r in batch:
            if error is None:
                r.future.set_result(r.image)
            else:
                r.future.set_exception(error)


def percentile(values, q: float) -> float:
    if not values:
        return float("nan")
    return float(np.percentile(np.asarray(values, dtype=np.float64), q))
