"""Host-side logic of the continuous-batching server, with a fake renderer (no GPU): admission
by footprint, FIFO batching, overlap across workers, per-request results and error delivery."""
import threading
import time

import numpy as np
import pytest

from blend2d_gb300 import scenes
from blend2d_gb300.serving import RenderServer, footprint_bytes, percentile


class FakeRuntime:
    """Fills each target with a value derived from its stream; records concurrency."""
    active = 0
    max_active = 0
    lock = threading.Lock()

    def __init__(self, delay=0.02, fail_on=None):
        self.delay = delay
        self.fail_on = fail_on
        self.batches = []

    def render_batch(self, streams, targets):
        with FakeRuntime.lock:
            FakeRuntime.active += 1
            FakeRuntime.max_active = max(FakeRuntime.max_active, FakeRuntime.active)
        try:
            self.batches.append(len(streams))
            time.sleep(self.delay)
            for s, t in zip(streams, targets):
                if self.fail_on is not None and self.fail_on in s:
                    raise RuntimeError("render failed")
                t[...] = np.uint32(len(s) & 0xFFFFFFFF)
        finally:
            with FakeRuntime.lock:
                FakeRuntime.active -= 1


def _streams(n, seed=0):
    return [scenes.random_mix(seed + i, width=16 + i, height=9 + 2 * i, count=3).to_bytes() for i in range(n)]


def test_results_and_batching():
    FakeRuntime.max_active = 0
    rts = []

    def factory():
        rts.append(FakeRuntime())
        return rts[-1]

    streams = _streams(40)
    with RenderServer(workers=2, runtime_factory=factory, max_batch=8) as srv:
        futs = []
        for s in streams:
            futs.append(srv.submit(s))
            time.sleep(0.001)
        outs = [f.result(timeout=10) for f in futs]
    for s, o in zip(streams, outs):
        assert o.shape == (int.from_bytes(s[12:16], "little"), int.from_bytes(s[8:12], "little"))
        assert o.dtype == np.uint32 and np.all(o == (len(s) & 0xFFFFFFFF))
    assert srv.stats.completed == 40
    assert max(srv.stats.batch_sizes) <= 8
    assert srv.stats.batches < 40               # requests were batched
    assert FakeRuntime.max_active == 2          # both workers ran at the same time
    assert len(srv.stats.latencies) == 40 and percentile(srv.stats.latencies, 99) > 0


def test_admission_respects_budget():
    streams = _streams(12)
    budget = max(footprint_bytes(s) for s in streams) * 2
    with RenderServer(workers=3, hbm_budget=budget, runtime_factory=lambda: FakeRuntime(0.01)) as srv:
        futs = [srv.submit(s) for s in streams]
        for f in futs:
            f.result(timeout=10)
    assert srv.stats.max_inflight_bytes <= budget


def test_oversized_request_rejected():
    s = _streams(1)[0]
    with RenderServer(workers=1, hbm_budget=footprint_bytes(s) - 1, runtime_factory=FakeRuntime) as srv:
        with pytest.raises(MemoryError):
            srv.submit(s).result(timeout=5)


def test_errors_reach_every_request_of_the_batch():
    streams = _streams(4)
    marker = streams[2][-40:]
    with RenderServer(workers=1, max_batch=8, runtime_factory=lambda: FakeRuntime(0.05, fail_on=marker)) as srv:
        first = srv.submit(streams[0])          # dispatched alone while the others queue up
        time.sleep(0.01)
        rest = [srv.submit(s) for s in streams[1:]]
        first.result(timeout=5)
        for f in rest:
            with pytest.raises(RuntimeError):
                f.result(timeout=5)


def test_runtime_close_closes_its_contexts_first():
    """A context kept alive past its runtime (a reference cycle, an exception traceback) must not be
    destroyed after the runtime: Runtime.close() closes the contexts still open on it."""
    import blend2d_gb300 as bg

    class FakeLib:
        def __init__(self):
            self.calls = []

        def blgpu_context_destroy(self, h):
            self.calls.append(("ctx", h))

        def blgpu_runtime_destroy(self, h):
            self.calls.append(("rt", h))

    rt = bg.Runtime.__new__(bg.Runtime)
    rt._lib = FakeLib()
    rt.handle = 1
    import weakref
    rt._contexts = weakref.WeakSet()
    ctx = bg.Context.__new__(bg.Context)
    ctx._lib = rt._lib
    ctx.handle = 2
    ctx.rt = rt
    rt._contexts.add(ctx)
    rt.close()
    assert rt._lib.calls == [("ctx", 2), ("rt", 1)]
    assert ctx.handle is None and rt.handle is None


class HoldingRuntime(FakeRuntime):
    """A fake whose arenas keep what its largest batch needed, like a device runtime's."""

    def __init__(self, per_request):
        super().__init__(0.005)
        self.per_request = per_request
        self.held = 0
        self.released = 0

    def render_batch(self, streams, targets):
        super().render_batch(streams, targets)
        self.held = max(self.held, self.per_request * len(streams))

    def memory(self):
        class M:
            pass
        m = M()
        m.reserved_bytes, m.last_frame_bytes = self.held, self.held
        return m

    def release_memory(self):
        self.held = 0
        self.released += 1


def test_admission_charges_what_runtimes_hold_and_releases_idle_arenas():
    """Workers keep their arenas between batches; the server charges what they hold, and when the
    holdings leave no room for the next request, idle workers give their arenas back instead of
    the queue stalling."""
    streams = _streams(30)
    per = max(footprint_bytes(s) for s in streams)
    rts = []

    def factory():
        rts.append(HoldingRuntime(per))
        return rts[-1]

    with RenderServer(workers=3, max_batch=2, hbm_budget=4 * per, runtime_factory=factory) as srv:
        outs = [f.result(timeout=20) for f in [srv.submit(s) for s in streams]]
    assert len(outs) == 30 and srv.stats.completed == 30
    assert srv.stats.max_inflight_bytes <= 4 * per
    assert srv.stats.releases >= 1 and sum(r.released for r in rts) == srv.stats.releases
