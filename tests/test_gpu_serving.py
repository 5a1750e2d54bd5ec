"""Serving on the GPU: every request's pixels are identical when rendered alone and when rendered
inside continuously formed batches that overlap on the device (tolerance: none - bit-exact)."""
import random
import time

import numpy as np
import pytest

import blend2d_gb300 as bg
from blend2d_gb300 import scenes
from blend2d_gb300.serving import RenderServer, percentile
import oracle_lib

pytestmark = pytest.mark.gpu


def _requests():
    reqs = []
    for i in range(18):
        side = [17, 64, 129, 250, 401, 33][i % 6]
        reqs.append(scenes.random_mix(9000 + i, width=side, height=side + (i % 3), count=20 + 15 * (i % 5)).to_bytes())
    for sw in scenes.batch_canvases(seed=41, count=10, max_side=700, max_paths=400):
        reqs.append(sw.to_bytes())
    return reqs


def test_results_alone_equal_results_in_the_mix():
    reqs = _requests()
    with bg.Runtime(0) as rt:
        alone = [bg.render_stream(rt, s) for s in reqs]
    rng = random.Random(5)
    with RenderServer(workers=3, max_batch=6, hbm_budget=2 << 30) as srv:
        futs = []
        # bursts of arrivals: requests that arrive while earlier batches run are batched together
        for k in range(0, len(reqs), 7):
            for s in reqs[k:k + 7]:
                futs.append(srv.submit(s))
            time.sleep(rng.uniform(0.0, 0.004))
        mixed = [f.result(timeout=120) for f in futs]
        stats = srv.stats
    for i, (a, m) in enumerate(zip(alone, mixed)):
        assert np.array_equal(a, m), f"request {i} differs between alone and mixed rendering"
    for i in (0, 7, 20):
        assert np.array_equal(alone[i], oracle_lib.render(reqs[i])), f"request {i} vs oracle"
    assert stats.completed == len(reqs)
    assert stats.batches < len(reqs)
    assert percentile(stats.latencies, 50) > 0
