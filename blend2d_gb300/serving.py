"""Continuous-batching render server over the batched C ABI entry point.

Requests (one command stream each, rendered into a new PRGB32 image) are admitted while earlier
batches are still on the GPU: a scheduler thread forms a batch from the waiting requests as soon
as a worker is free and the batch's estimated device footprint fits in the HBM budget next to
the batches in flight. Each worker owns a `Runtime` (its own CUDA stream and device arena, kept
resident and reused across batches), so batches on different workers overlap on the device.
Every request's pixels are the same as when it is rendered alone: canvases of one batch share
no state (each has its own tiles, commands, styles and LUTs).

    server = RenderServer(workers=2, hbm_budget=150 << 30)
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


def footprint_bytes(stream: bytes) -> int:
    """Upper estimate of the device memory one request needs inside a batch: its canvas plus the
    frame data and the edge/binning work arrays, which scale with the stream's size."""
    w, h = stream_size(stream)
    return 4 * w * h + 24 * len(stream) + (1 << 16)


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
    max_inflight_bytes: int = 0
    latencies: list = field(default_factory=list)
    batch_sizes: list = field(default_factory=list)


class RenderServer:
    """Admission by HBM footprint + continuous batching across `workers` runtimes.

    `runtime_factory` builds one renderer per worker; it must return an object with
    `render_batch(streams, targets)` (blend2d_gb300.Runtime does). Tests inject a fake.
    """

    def __init__(self, workers: int = 2, hbm_budget: int = 150 << 30, max_batch: int = 256,
                 runtime_factory=None, device: int = 0):
        if runtime_factory is None:
            from . import Runtime

            def runtime_factory():
                return Runtime(device)
        self.hbm_budget = int(hbm_budget)
        self.max_batch = int(max_batch)
        self._runtimes = [runtime_factory() for _ in range(workers)]
        self._free = list(range(workers))
        self._waiting: collections.deque[Request] = collections.deque()
        self._inflight_bytes = 0
        self._cv = threading.Condition()
        self._closing = False
        self.stats = ServerStats()
        self._scheduler = threading.Thread(target=self._schedule, name="blgpu-scheduler", daemon=True)
        self._scheduler.start()

    # -- client side --------------------------------------------------------------------------
    def submit(self, stream: bytes) -> Future:
        fut: Future = Future()
        req = Request(stream, fut, footprint_bytes(stream), time.perf_counter())
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
    def _take_batch(self) -> list[Request]:
        """FIFO batch that fits the budget next to the batches in flight (called under the lock)."""
        batch, need = [], 0
        while self._waiting and len(batch) < self.max_batch:
            req = self._waiting[0]
            if self._inflight_bytes + need + req.footprint > self.hbm_budget:
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
                    batch = self._take_batch() if self._free and self._waiting else []
                    if batch:
                        break
                    self._cv.wait(timeout=0.05)
                worker = self._free.pop()
                need = sum(r.footprint for r in batch)
                self._inflight_bytes += need
                self.stats.max_inflight_bytes = max(self.stats.max_inflight_bytes, self._inflight_bytes)
            t = threading.Thread(target=self._run_batch, args=(worker, batch, need), daemon=True)
            t.start()
            workers = [w for w in workers if w.is_alive()] + [t]

    def _run_batch(self, worker: int, batch: list[Request], need: int):
        t0 = time.perf_counter()
        for r in batch:
            r.t_start = t0
            w, h = stream_size(r.stream)
            r.image = np.zeros((h, w), dtype=np.uint32)
        error = None
        try:
            self._runtimes[worker].render_batch([r.stream for r in batch], [r.image for r in batch])
        except Exception as e:  # noqa: BLE001 - delivered to every request of the batch
            error = e
        t1 = time.perf_counter()
        with self._cv:
            self._inflight_bytes -= need
            self._free.append(worker)
            self.stats.batches += 1
            self.stats.batch_sizes.append(len(batch))
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
