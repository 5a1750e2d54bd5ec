"""GPU parity: every render goes through the C ABI (libblgpu.so) on cuda:0 and must be bit-exact
to the reference - directly against the golden hashes of the reference's own renders, and against
the oracle (pinned to those hashes) on seeded random scenes."""
import math

import numpy as np
import pytest

import blend2d_gb300 as bg
from blend2d_gb300 import scenes
import oracle_lib

pytestmark = pytest.mark.gpu

GOLDEN = oracle_lib.golden()
LUTS = {"default": bg.LUT_SSE2, "sse2": bg.LUT_SSE2, "avx2": bg.LUT_AVX2, "scalar": bg.LUT_SCALAR}


@pytest.fixture(scope="module")
def runtimes():
    rts = {}
    yield lambda variant="default": rts.setdefault(variant, bg.Runtime(0, LUTS[variant]))
    for rt in rts.values():
        rt.close()


def _diff(got, want):
    bad = np.argwhere(got != want)
    if not len(bad):
        return ""
    y, x = bad[0]
    return f"{len(bad)} pixels differ, first at ({x},{y}): got {got[y, x]:08x} want {want[y, x]:08x}"


GOLDEN_CASES = [(e["name"], v) for e in GOLDEN["scenes"] for v in e["pixels_sha256"]]


@pytest.mark.parametrize("name,variant", GOLDEN_CASES, ids=[f"{n}-{v}" for n, v in GOLDEN_CASES])
def test_golden_scene(runtimes, name, variant):
    entry = next(e for e in GOLDEN["scenes"] if e["name"] == name)
    stream = oracle_lib.golden_stream(entry)
    got = bg.render_stream(runtimes(variant), stream)
    if oracle_lib.sha256(got) != entry["pixels_sha256"][variant]:
        detail = ""
        if got.size <= 2_000_000:
            detail = _diff(got, oracle_lib.render(stream, variant))
        pytest.fail(f"{name}/{variant}: pixels differ from the reference render. {detail}")


RANDOM_CASES = [(seed, w, h, variant)
                for seed, (w, h), variant in zip(range(1000, 1036),
                                                 [(257, 257), (64, 48), (33, 97), (400, 150), (1, 1), (3, 700),
                                                  (129, 129), (640, 31)] * 5,
                                                 ["default", "avx2", "scalar"] * 12)]


@pytest.mark.parametrize("seed,w,h,variant", RANDOM_CASES)
def test_random_mix_vs_oracle(runtimes, seed, w, h, variant):
    stream = scenes.random_mix(seed, width=w, height=h, count=150).to_bytes()
    got = bg.render_stream(runtimes(variant), stream)
    want = oracle_lib.render(stream, variant)
    assert not _diff(got, want), _diff(got, want)


@pytest.mark.parametrize("seed,w,h,variant", [(s, w, h, v) for s, (w, h), v in
                                               zip(range(1100, 1112), [(257, 257), (33, 97), (400, 150), (1, 1),
                                                                       (129, 129), (640, 31)] * 2,
                                                   ["default", "avx2", "scalar"] * 4)])
def test_dithered_gradients_vs_oracle(runtimes, seed, w, h, variant):
    """Gradient quality DITHER (2 gradients in 3; the others NEAREST, whose LUT builder depends on
    the variant): the 64-bit LUT and the ordered-dither threshold of every pixel."""
    stream = scenes.random_mix(seed, width=w, height=h, count=150, dither=True).to_bytes()
    got = bg.render_stream(runtimes(variant), stream)
    want = oracle_lib.render(stream, variant)
    assert not _diff(got, want), _diff(got, want)


@pytest.mark.parametrize("seed", range(6))
def test_edge_cases_vs_oracle(runtimes, seed):
    stream = scenes.edge_cases(seed=seed, width=131 + 17 * seed, height=97 + 5 * seed).to_bytes()
    got = bg.render_stream(runtimes(), stream)
    want = oracle_lib.render(stream)
    assert not _diff(got, want), _diff(got, want)


def test_batch_equals_oracle(runtimes):
    rng = np.random.default_rng(77)
    streams, targets = [], []
    for i in range(24):
        w, h = int(rng.integers(1, 300)), int(rng.integers(1, 300))
        streams.append(scenes.random_mix(5000 + i, width=w, height=h, count=int(rng.integers(0, 120))).to_bytes())
        targets.append(np.zeros((h, w), dtype=np.uint32))
    rt = runtimes()
    rt.render_batch(streams, targets)
    for i, (s, t) in enumerate(zip(streams, targets)):
        want = oracle_lib.render(s)
        assert not _diff(t, want), f"canvas {i}: {_diff(t, want)}"


def test_batch_canvases_workload_matches_individual(runtimes):
    """Batched rendering of the many-canvas workload (reduced scale) equals per-canvas rendering."""
    sws = scenes.batch_canvases(seed=4, count=40, max_side=512, max_paths=300)
    streams = [sw.to_bytes() for sw in sws]
    rt = runtimes()
    batched = [np.zeros((sw.height, sw.width), dtype=np.uint32) for sw in sws]
    rt.render_batch(streams, batched)
    for i, s in enumerate(streams):
        single = bg.render_stream(rt, s)
        assert np.array_equal(single, batched[i]), f"canvas {i}"
        if i % 8 == 0:
            assert np.array_equal(single, oracle_lib.render(s)), f"canvas {i} vs oracle"


def test_batch_of_every_kind_equals_individual(runtimes):
    """Batches are recorded by several threads and merged: canvases with every kind of recorded
    data (dithered and plain gradients, patterns, strokes, A8 masks, blits, shapes) render in a
    batch exactly as they render alone."""
    streams = []
    for k in range(5):
        streams.append(scenes.random_mix(6000 + k, width=90 + 13 * k, height=70 + 7 * k, count=60, dither=k % 2 == 0).to_bytes())
        streams.append(scenes.strokes(seed=6100 + k, width=120, height=90, count=40).to_bytes())
        streams.append(scenes.masks(seed=6200 + k, width=110, height=80, count=30).to_bytes())
        streams.append(scenes.blits(seed=6300 + k, width=100, height=100, count=30).to_bytes())
        streams.append(scenes.shapes(seed=6400 + k, width=130, height=90, count=30).to_bytes())
    rt = runtimes()
    sizes = [oracle_lib.stream_size(s) for s in streams]
    batched = [np.zeros((h, w), dtype=np.uint32) for w, h in sizes]
    rt.render_batch(streams, batched)
    for i, s in enumerate(streams):
        single = bg.render_stream(rt, s)
        assert not _diff(batched[i], single), f"canvas {i}: {_diff(batched[i], single)}"
        if i % 5 == 0 or i < 5:
            want = oracle_lib.render(s)
            assert not _diff(single, want), f"canvas {i} vs oracle: {_diff(single, want)}"


def _oracle_many(streams, variant="default"):
    """Oracle renders of many streams on the host's cores (the oracle's ctypes calls release the
    GIL, so threads render in parallel)."""
    from concurrent.futures import ThreadPoolExecutor
    import os
    with ThreadPoolExecutor(max_workers=max(1, os.cpu_count() or 1)) as ex:
        return list(ex.map(lambda s: oracle_lib.render(s, variant), streams))


# 64 canvases of the full batched workload (4,096 canvases of 32-2,048 px, 10-5,000 paths): the
# canvases whose reference renders are recorded in the golden file (the largest canvas, the most
# paths, the largest area x paths and eight seeded picks) and 53 more seeded picks.
FULL_BATCH_SAMPLE = sorted(set(
    [int(e["expr"].split("(")[1].rstrip(")")) for e in GOLDEN["scenes"] if e["name"].startswith("batch4096_")]
    + np.random.default_rng(404).choice(4096, 53, replace=False).tolist()))


def test_full_batch_sample_vs_oracle(runtimes):
    """A 64-canvas sample of the full-size batched workload, rendered in one batched pipeline:
    every canvas equals the oracle's render, and the ones the golden file holds equal the
    reference's own renders."""
    sws = [scenes.batch_canvas(i) for i in FULL_BATCH_SAMPLE]
    streams = [sw.to_bytes() for sw in sws]
    targets = [np.zeros((sw.height, sw.width), dtype=np.uint32) for sw in sws]
    runtimes().render_batch(streams, targets)
    golden = {e["expr"]: e["pixels_sha256"]["default"] for e in GOLDEN["scenes"] if e["name"].startswith("batch4096_")}
    for i, t in zip(FULL_BATCH_SAMPLE, targets):
        want = golden.get(f"scenes.batch_canvas({i})")
        if want:
            assert oracle_lib.sha256(t) == want, f"canvas {i}: differs from the reference render"
    for i, t, want in zip(FULL_BATCH_SAMPLE, targets, _oracle_many(streams)):
        assert not _diff(t, want), f"canvas {i}: {_diff(t, want)}"


def test_capacity_overflow_is_an_error():
    """A frame whose device work arrays overflow reports BL_ERROR_DATA_TOO_LARGE instead of
    rendering with work dropped: the segment array is capped below what the frame emits (the
    runtime's regrow is disabled for this runtime), and the frame must fail, not draw less."""
    stream = scenes.curves(count=300, width=320, height=200).to_bytes()
    with bg.Runtime(0) as rt:
        rt.set_segment_limit(1000)
        with pytest.raises(bg.BLGpuError) as ei:
            bg.render_stream(rt, stream)
        assert ei.value.code == bg.ERROR_DATA_TOO_LARGE
        rt.set_segment_limit(0)
        got = bg.render_stream(rt, stream)
    assert not _diff(got, oracle_lib.render(stream))


def test_context_calls_match_stream(runtimes):
    """The same scene through individual bl_context_* calls and through a submitted stream."""
    rng = np.random.default_rng(5)
    w, h = 200, 150
    sw = scenes.StreamWriter(w, h)
    img = scenes.premultiplied_noise(rng, 17, 9)
    sw.add_image(img)
    out = np.zeros((h, w), dtype=np.uint32)
    rt = runtimes()
    ctx = bg.Context(rt, out)
    ops = []

    def both(name, *args):
        getattr(sw, {"set_comp_op": "comp_op", "set_fill_rule": "fill_rule", "set_fill_alpha": "fill_alpha",
                     "set_global_alpha": "global_alpha", "set_transform": "transform",
                     "reset_transform": "reset_transform", "set_fill_style_rgba32": "solid",
                     "fill_polygon_d": "fill_polygon", "fill_path_d": "fill_path"}.get(name, name))(*args)
        getattr(ctx, name)(*args)
        ops.append(name)

    both("clear_all")
    both("set_fill_style_rgba32", 0xFF336699)
    both("fill_rect_i", 10, 10, 50, 40)
    both("set_fill_alpha", 0.5)
    both("set_fill_style_rgba32", 0x80FF8000)
    both("fill_rect_d", 20.25, 15.5, 100.75, 60.125)
    both("set_fill_rule", 1)
    both("fill_polygon_d", np.array([[5.0, 5.0], [190.0, 20.0], [40.0, 140.0], [160.0, 130.0]]))
    both("set_comp_op", 1)
    both("set_transform", [math.cos(0.3), math.sin(0.3), -math.sin(0.3), math.cos(0.3), 40.0, -10.0])
    both("fill_box_d", 30.0, 30.0, 120.0, 90.0)
    both("reset_transform")
    both("set_comp_op", 0)
    both("set_fill_alpha", 1.0)
    stops = [(0.0, 0xFF0000FF), (0.5, 0x8000FF00), (1.0, 0xFFFF0000)]
    sw.gradient(scenes.RADIAL, [100, 75, 80, 60, 90, 10], scenes.REFLECT, stops)
    ctx.set_fill_style_gradient(bg.GRADIENT_RADIAL, [100, 75, 80, 60, 90, 10],
                                [(o, scenes.rgba64_from_rgba32(c)) for o, c in stops], bg.EXTEND_REFLECT)
    both("fill_path_d", [0, 4, 4, 4, 5], np.array([[10.0, 140.0], [60.0, -40.0], [140.0, 200.0], [190.0, 10.0],
                                                   [10.0, 140.0]]))
    sw.hint(2, 0)
    ctx.set_hint(2, 0)
    sw.pattern(0, scenes.REPEAT, transform=[1.5, 0.2, -0.2, 1.5, 3.0, 7.0])
    ctx.set_fill_style_pattern(img, extend_mode=bg.EXTEND_REPEAT, transform=[1.5, 0.2, -0.2, 1.5, 3.0, 7.0])
    both("save")
    both("set_global_alpha", 0.7)
    both("fill_rect_d", 100.0, 20.0, 90.0, 120.0)
    both("restore")
    both("fill_rect_i", 0, 100, 60, 50)
    ctx.end()
    ctx.close()
    want = bg.render_stream(rt, sw.to_bytes())
    assert np.array_equal(out, want)
    assert np.array_equal(out, oracle_lib.render(sw.to_bytes()))


def test_rendering_onto_existing_content(runtimes):
    """Without clear_all the pipeline composites onto the image's current pixels."""
    rng = np.random.default_rng(9)
    w, h = 173, 111
    base_sw = scenes.StreamWriter(w, h)
    base_sw.add_image(scenes.premultiplied_noise(rng, w, h))
    base_sw.comp_op(1)
    base_sw.pattern(0, scenes.PAD)
    base_sw.fill_all()
    base = oracle_lib.render(base_sw.to_bytes())
    top = scenes.random_mix(31, width=w, height=h, count=80)
    top.parts = top.parts[1:]             # drop its clear_all
    # the same drawing appended to the base scene, as one stream, for the oracle
    both = scenes.StreamWriter(w, h)
    both.images = base_sw.images + top.images
    both.parts = list(base_sw.parts)
    both.comp_op(0)                        # back to the state a fresh context starts with
    both.reset_transform()
    both.hint(2, 1)
    both.solid(0xFF000000)
    shifted = []
    for rec in top.parts:
        shifted.append(_shift_pattern_index(rec, len(base_sw.images)))
    both.parts += shifted
    want = oracle_lib.render(both.to_bytes())
    img = base.copy()
    bg.render_stream(runtimes(), top.to_bytes(), img)
    assert not _diff(img, want), _diff(img, want)


def _shift_pattern_index(rec: bytes, by: int) -> bytes:
    import struct
    op = struct.unpack_from("<I", rec, 0)[0]
    if op != 10:   # OP_STYLE_PATTERN
        return rec
    idx = struct.unpack_from("<I", rec, 8)[0]
    return rec[:8] + struct.pack("<I", idx + by) + rec[12:]


def test_device_targets(runtimes):
    torch = pytest.importorskip("torch")
    rt = runtimes()
    for (w, h) in [(256, 100), (131, 77)]:     # aligned rows (direct) and unaligned rows (staged)
        stream = scenes.random_mix(77 + w, width=w, height=h, count=100).to_bytes()
        want = oracle_lib.render(stream)
        dev = torch.zeros((h, w), dtype=torch.int32, device="cuda")
        bg.render_stream(rt, stream, dev)
        torch.cuda.synchronize()
        got = dev.cpu().numpy().view(np.uint32)
        assert not _diff(got, want), _diff(got, want)


@pytest.mark.parametrize("use_graph", [False, True])
def test_replay(runtimes, use_graph):
    torch = pytest.importorskip("torch")
    rt = runtimes()
    w, h = 300, 200
    stream = scenes.random_mix(4242, width=w, height=h, count=200).to_bytes()   # starts with clear_all
    want = oracle_lib.render(stream)
    dev = torch.zeros((h, w), dtype=torch.int32, device="cuda")
    bg.render_stream(rt, stream, dev)
    for _ in range(3):
        dev.fill_(0x12345678)
        torch.cuda.synchronize()
        rt.replay(use_graph)
        rt.synchronize()
        got = dev.cpu().numpy().view(np.uint32)
        assert not _diff(got, want), _diff(got, want)
    st = rt.stats()
    assert st.last_gpu_ms > 0 and st.kernel_launches > 0


def test_stats_and_errors(runtimes):
    rt = runtimes()
    img = np.zeros((10, 10), dtype=np.uint32)
    ctx = bg.Context(rt, img)
    for call, args, code in [("set_comp_op", (29,), bg.ERROR_INVALID_VALUE),
                             ("set_comp_op", (2,), bg.ERROR_NOT_IMPLEMENTED),
                             ("set_fill_rule", (2,), bg.ERROR_INVALID_VALUE),
                             ("set_global_alpha", (float("nan"),), bg.ERROR_INVALID_VALUE),
                             ("set_fill_alpha", (float("nan"),), bg.ERROR_INVALID_VALUE),
                             ("set_hint", (3, 0), bg.ERROR_INVALID_VALUE),
                             ("set_hint", (2, 2), bg.ERROR_INVALID_VALUE),
                             ("restore", (), bg.ERROR_NO_STATES_TO_RESTORE)]:
        with pytest.raises(bg.BLGpuError) as ei:
            getattr(ctx, call)(*args)
        assert ei.value.code == code, (call, args)
    ctx.set_fill_style_rgba32(0xFFFFFFFF)
    ctx.fill_rect_i(2, 2, 3, 3)
    ctx.end()
    assert img[3, 3] == 0xFFFFFFFF and img[0, 0] == 0
    with pytest.raises(bg.BLGpuError) as ei:
        ctx.fill_all()
    assert ei.value.code == bg.ERROR_INVALID_STATE
    ctx.close()
    st = rt.stats()
    assert st.frames >= 1 and st.fill_commands == 1


def test_autotune_keeps_pixels_and_every_config_renders_the_same():
    torch = pytest.importorskip("torch")
    w, h = 320, 200
    stream = scenes.random_mix(777, width=w, height=h, count=250).to_bytes()
    want = oracle_lib.render(stream)
    with bg.Runtime(0) as rt:
        dev = torch.zeros((h, w), dtype=torch.int32, device="cuda")
        bg.render_stream(rt, stream, dev)
        best, ms = rt.autotune(trials=2)
        torch.cuda.synchronize()
        assert ms > 0 and best.cover_slots in (0, 16, 32, 64) and best.edge_block in (64, 128, 256)
        assert not _diff(dev.cpu().numpy().view(np.uint32), want)       # tuning left the pixels alone
        for cfg in [dict(cover_slots=16, edge_block=64, fine_blocks_per_sm=1, cover_blocks_per_sm=1, cubic_blocks_per_sm=1),
                    dict(cover_slots=32, edge_block=256, fine_blocks_per_sm=0, cover_blocks_per_sm=0, cubic_blocks_per_sm=0)]:
            rt.set_launch_config(bg.LaunchConfig(**cfg))
            got = bg.render_stream(rt, stream)
            assert not _diff(got, want), cfg
        with pytest.raises(bg.BLGpuError):
            rt.set_launch_config(bg.LaunchConfig(cover_slots=24, edge_block=128))


def test_list_row_heights_render_the_same():
    """The composite's command lists per 4, 8, 16 or 32 pixel rows (a tuning choice): every height
    gives the oracle's pixels, for a frame run with it and for the kept frame replayed after the
    height changed (its binning arrays are sized again)."""
    torch = pytest.importorskip("torch")
    w, h = 336, 211        # rows of 16-byte multiples: the device image is drawn in place, so a replay redraws it
    stream = scenes.random_mix(778, width=w, height=h, count=300).to_bytes()
    want = oracle_lib.render(stream)
    batch = [scenes.random_mix(779 + i, width=90 + 40 * i, height=61 + 30 * i, count=80).to_bytes() for i in range(4)]
    with bg.Runtime(0) as rt:
        for rows in (4, 8, 16, 32):
            rt.set_launch_config(bg.LaunchConfig(edge_block=128, list_rows=rows))
            got = bg.render_stream(rt, stream)
            assert not _diff(got, want), rows
            targets = [np.zeros(oracle_lib.stream_size(s)[::-1], dtype=np.uint32) for s in batch]
            rt.render_batch(batch, targets)
            for s, t in zip(batch, targets):
                assert not _diff(t, oracle_lib.render(s)), rows
        dev = torch.zeros((h, w), dtype=torch.int32, device="cuda")
        rt.set_launch_config(bg.LaunchConfig(edge_block=128, list_rows=32))
        bg.render_stream(rt, stream, dev)
        for rows in (8, 4, 16):
            rt.set_launch_config(bg.LaunchConfig(edge_block=128, list_rows=rows))
            dev.zero_()
            torch.cuda.synchronize()
            rt.replay(False)                   # the canvas is a device image: the replay redraws it
            rt.synchronize()
            torch.cuda.synchronize()
            assert not _diff(dev.cpu().numpy().view(np.uint32), want), rows


@pytest.mark.parametrize("variant,dither", [("default", False), ("avx2", False), ("scalar", False),
                                            ("default", True)])
def test_gradients_with_many_stops(runtimes, variant, dither):
    """Stop counts around the 32-stop chunks of the LUT builder, with repeated offsets and a first
    stop at 0 (the SIMD builders skip it), each gradient filling a band of the canvas; with
    `dither`, the 64-bit LUT builder of gradient quality DITHER."""
    rng = np.random.Generator(np.random.PCG64(77))
    w, band = 300, 6
    counts = [1, 2, 31, 32, 33, 34, 63, 64, 65, 100, 7]
    sw = scenes.StreamWriter(w, band * len(counts))
    sw.solid(0xFF202020)
    sw.fill_all()
    if dither:
        sw.hint(scenes.HINT_GRADIENT_QUALITY, scenes.GRADIENT_DITHER)
    for i, n in enumerate(counts):
        offs = np.sort(rng.uniform(0.0, 1.0, n))
        if n > 3:
            offs[0] = 0.0
            offs[n // 2] = offs[n // 2 - 1]                 # repeated offset
        cols = rng.integers(0, 2**32, n, dtype=np.uint64)
        if i % 2:
            cols |= np.uint64(0xFF000000)                   # opaque stops (the builders' opaque path)
        stops = [(float(o), int(c)) for o, c in zip(offs, cols)]
        sw.gradient(scenes.LINEAR, [3.0 + i, 0.0, w - 7.0, 1.0], i % 3, stops)
        sw.fill_rect_i(0, band * i, w, band)
    stream = sw.to_bytes()
    got = bg.render_stream(runtimes(variant), stream)
    want = oracle_lib.render(stream, variant)
    assert not _diff(got, want), _diff(got, want)


def test_async_flush_pipelines_frames_with_the_same_pixels(runtimes):
    """Two contexts alternate: each records a frame while the other's renders (FLUSH_ASYNC), with
    mid-frame async flushes too; every image matches the synchronous render of its stream."""
    import torch
    rt = runtimes()
    streams = [scenes.random_mix(seed, width=211, height=157, count=200).to_bytes() for seed in range(3100, 3106)]
    want = [bg.render_stream(rt, s) for s in streams]
    hosts = [torch.zeros((157, 211), dtype=torch.int32).pin_memory() for _ in range(2)]
    ctxs = [bg.Context(rt) for _ in range(2)]
    got = []
    active = [None, None]
    for i, s in enumerate(streams):
        c = ctxs[i % 2]
        if active[i % 2] is not None:
            c.end()
            got.append((active[i % 2], hosts[i % 2].numpy().view(np.uint32).copy()))
        hosts[i % 2].zero_()
        c.begin(hosts[i % 2])
        c.submit_stream(s)
        c.flush(bg.FLUSH_ASYNC)
        c.flush(bg.FLUSH_ASYNC)                             # nothing recorded since: a no-op
        active[i % 2] = i
    for k in range(2):
        ctxs[k].end()
        got.append((active[k], hosts[k].numpy().view(np.uint32).copy()))
    assert sorted(i for i, _ in got) == list(range(len(streams)))
    for i, img in got:
        assert not _diff(img, want[i]), (i, _diff(img, want[i]))
    # a frame split by an async flush renders the same as in one piece
    half = scenes.random_mix(3200, width=211, height=157, count=120)
    host = torch.zeros((157, 211), dtype=torch.int32).pin_memory()
    c = ctxs[0]
    c.begin(host)
    c.submit_stream(half.to_bytes())
    c.flush(bg.FLUSH_ASYNC)
    c.fill_rect_i(5, 7, 50, 40)
    c.end()
    ref = torch.zeros((157, 211), dtype=torch.int32).pin_memory()
    c.begin(ref)
    c.submit_stream(half.to_bytes())
    c.fill_rect_i(5, 7, 50, 40)
    c.end()
    assert np.array_equal(host.numpy(), ref.numpy())
    for c in ctxs:
        c.close()


def test_two_threads_record_and_flush_async(runtimes):
    """Two host threads, a context each on one runtime, record and flush asynchronously at the same
    time (the bench's e2e arm); every frame matches its synchronous render."""
    import threading
    import torch
    rt = runtimes()
    streams = [scenes.random_mix(seed, width=173, height=141, count=250).to_bytes() for seed in range(3300, 3308)]
    want = [bg.render_stream(rt, s) for s in streams]
    results, errors = {}, []

    def worker(k):
        try:
            ctx = bg.Context(rt)
            hosts = [torch.zeros((141, 173), dtype=torch.int32).pin_memory() for _ in range(2)]
            for rep in range(3):
                for j, i in enumerate(range(k, len(streams), 2)):
                    host = hosts[j % 2]
                    ctx.begin(host)
                    ctx.submit_stream(streams[i])
                    ctx.flush(bg.FLUSH_ASYNC)
                    ctx.end()
                    results[(rep, i)] = host.numpy().view(np.uint32).copy()
            ctx.close()
        except Exception as e:
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    assert len(results) == 3 * len(streams)
    for (rep, i), img in results.items():
        assert not _diff(img, want[i]), (rep, i, _diff(img, want[i]))


def test_occlusion_cull_keeps_pixels_and_skips_work():
    """SrcCopy quads over each other: the composite with occlusion culling gives the pixels of the
    composite without it (and of the oracle) while compositing fewer pixel-ops."""
    stream = scenes.patterns(count=300, width=512, height=512).to_bytes()
    with bg.Runtime(0) as rt:
        culled = bg.render_stream(rt, stream)
        ops_culled = rt.stats().pixel_ops
        cfg = rt.launch_config()
        rt.set_launch_config(bg.LaunchConfig(**{**cfg.as_dict(), "no_occlusion_cull": 1}))
        full = bg.render_stream(rt, stream)
        ops_full = rt.stats().pixel_ops
    assert np.array_equal(culled, full)
    assert ops_culled < ops_full
    want = oracle_lib.render(stream)
    assert not _diff(culled, want), _diff(culled, want)


# --- stroking ---------------------------------------------------------------------------------------

@pytest.mark.parametrize("seed,variant", [(s, v) for s, v in zip(range(1200, 1212), ["default", "avx2", "scalar"] * 4)])
def test_strokes_vs_oracle(runtimes, seed, variant):
    """Stroked paths, polylines, polygons, boxes, rects and lines with every join and cap, both
    transform orders, solid / gradient / pattern stroke styles (host stroker, device fill)."""
    sw = scenes.strokes(seed=seed, count=120, width=(257, 64, 400)[seed % 3], height=(193, 301, 90)[seed % 3],
                        max_width=(24.0, 6.0, 60.0, 12.0)[seed % 4], curves=seed % 5 != 4)
    stream = sw.to_bytes()
    got = bg.render_stream(runtimes(variant), stream)
    want = oracle_lib.render(stream, variant)
    assert not _diff(got, want), _diff(got, want)


def test_stroke_context_calls_match_stream(runtimes):
    """The stroke entry points and stroke state of the C ABI against the same operations replayed
    from a stream (and the oracle)."""
    w, h = 220, 160
    sw = scenes.StreamWriter(w, h)
    out = np.zeros((h, w), dtype=np.uint32)
    ctx = bg.Context(runtimes(), out)
    sw.solid(0xFF202020); sw.fill_all()
    ctx.set_fill_style_rgba32(0xFF202020); ctx.fill_all()
    sw.stroke_solid(0xFFFFCC00); ctx.set_stroke_style_rgba32(0xFFFFCC00)
    sw.stroke_width(7.5); ctx.set_stroke_width(7.5)
    sw.stroke_join(scenes.JOIN_ROUND); ctx.set_stroke_join(scenes.JOIN_ROUND)
    sw.stroke_caps(scenes.CAP_ROUND, scenes.CAP_TRIANGLE)
    ctx.set_stroke_cap(0, scenes.CAP_ROUND); ctx.set_stroke_cap(1, scenes.CAP_TRIANGLE)
    pl = np.array([[10.0, 20.0], [80.0, 30.0], [40.0, 90.0], [120.0, 70.0]])
    sw.stroke_polyline(pl); ctx.stroke_polyline_d(pl)
    sw.stroke_join(scenes.JOIN_MITER_CLIP); ctx.set_stroke_join(scenes.JOIN_MITER_CLIP)
    sw.stroke_miter_limit(2.5); ctx.set_stroke_miter_limit(2.5)
    sw.stroke_polygon(pl + 80.0); ctx.stroke_polygon_d(pl + 80.0)
    sw.stroke_alpha(0.6); ctx.set_stroke_alpha(0.6)
    sw.stroke_box_d(150.0, 10.0, 210.0, 60.0); ctx.stroke_box_d(150.0, 10.0, 210.0, 60.0)
    sw.stroke_rect_d(15.0, 110.0, 60.0, 35.0); ctx.stroke_rect_d(15.0, 110.0, 60.0, 35.0)
    sw.stroke_caps(scenes.CAP_SQUARE, scenes.CAP_SQUARE); ctx.set_stroke_caps(scenes.CAP_SQUARE)
    sw.stroke_line_d(100.0, 150.0, 200.0, 100.0); ctx.stroke_line_d(100.0, 150.0, 200.0, 100.0)
    m = [1.2, 0.3, -0.2, 0.9, 10.0, 5.0]
    sw.transform(m); ctx.set_transform(m)
    sw.stroke_transform_order(scenes.TRANSFORM_ORDER_BEFORE); ctx.set_stroke_transform_order(scenes.TRANSFORM_ORDER_BEFORE)
    stops = [(0.0, 0xFF00FFFF), (1.0, 0xFFFF00FF)]
    sw.stroke_gradient(scenes.LINEAR, [0.0, 0.0, 150.0, 100.0], scenes.PAD, stops)
    ctx.set_stroke_style_gradient(bg.GRADIENT_LINEAR, [0.0, 0.0, 150.0, 100.0],
                                  [(o, scenes.rgba64_from_rgba32(c)) for o, c in stops], bg.EXTEND_PAD)
    path_c = [0, 4, 4, 1, 2, 1]
    path_xy = np.array([[20.0, 40.0], [60.0, -10.0], [90.0, 90.0], [130.0, 40.0], [150.0, 0.0], [170.0, 60.0]])
    sw.stroke_path(path_c, path_xy); ctx.stroke_path_d(path_c, path_xy)
    ctx.end()
    stream = sw.to_bytes()
    via_stream = bg.render_stream(runtimes(), stream)
    assert not _diff(out, via_stream), _diff(out, via_stream)
    want = oracle_lib.render(stream)
    assert not _diff(out, want), _diff(out, want)
    with pytest.raises(bg.BLGpuError):
        ctx2 = bg.Context(runtimes(), np.zeros((8, 8), dtype=np.uint32))
        try:
            ctx2.stroke_path_d([1, 1], np.array([[0.0, 0.0], [4.0, 4.0]]))   # no MOVE: invalid geometry
        finally:
            ctx2.end()


# --- image blits ----------------------------------------------------------------------------------

@pytest.mark.parametrize("seed", range(1300, 1306))
def test_blits_vs_oracle(runtimes, seed):
    """Integer / fractional / scaled / transformed blits of image areas, clipped, both qualities."""
    sw = scenes.blits(seed=seed, count=150, width=(320, 61, 500)[seed % 3], height=(240, 203, 90)[seed % 3])
    stream = sw.to_bytes()
    got = bg.render_stream(runtimes(), stream)
    want = oracle_lib.render(stream)
    assert not _diff(got, want), _diff(got, want)


def test_blit_context_calls_match_stream(runtimes):
    rng = np.random.default_rng(9)
    w, h = 160, 120
    img = scenes.premultiplied_noise(rng, 37, 23)
    sw = scenes.StreamWriter(w, h)
    sw.add_image(img)
    out = np.zeros((h, w), dtype=np.uint32)
    ctx = bg.Context(runtimes(), out)
    sw.solid(0xFF102030); sw.fill_all()
    ctx.set_fill_style_rgba32(0xFF102030); ctx.fill_all()
    sw.blit_image_i(10, 12, 0); ctx.blit_image_i(10, 12, img)
    sw.blit_image_i(140, 100, 0, [3, 4, 20, 15]); ctx.blit_image_i(140, 100, img, [3, 4, 20, 15])
    sw.blit_image_d(30.25, 60.5, 0); ctx.blit_image_d(30.25, 60.5, img)
    sw.hint(scenes.HINT_PATTERN_QUALITY, scenes.NEAREST); ctx.set_hint(2, 0)
    sw.blit_image_d(80.75, 5.125, 0, [1, 1, 30, 20]); ctx.blit_image_d(80.75, 5.125, img, [1, 1, 30, 20])
    sw.hint(scenes.HINT_PATTERN_QUALITY, scenes.BILINEAR); ctx.set_hint(2, 1)
    sw.global_alpha(0.6); ctx.set_global_alpha(0.6)
    sw.blit_scaled_image_d(90.0, 50.0, 60.5, 40.25, 0); ctx.blit_scaled_image_d(90.0, 50.0, 60.5, 40.25, img)
    sw.blit_scaled_image_i(5, 80, 50, 30, 0, [0, 0, 10, 10]); ctx.blit_scaled_image_i(5, 80, 50, 30, img, [0, 0, 10, 10])
    m = [0.9, 0.4, -0.4, 0.9, 30.0, -10.0]
    sw.transform(m); ctx.set_transform(m)
    sw.blit_image_i(40, 40, 0); ctx.blit_image_i(40, 40, img)
    ctx.end()
    stream = sw.to_bytes()
    assert not _diff(out, bg.render_stream(runtimes(), stream))
    assert not _diff(out, oracle_lib.render(stream))
    ctx2 = bg.Context(runtimes(), np.zeros((8, 8), dtype=np.uint32))
    try:
        with pytest.raises(bg.BLGpuError):
            ctx2.blit_image_i(0, 0, img, [30, 0, 10, 5])        # area outside the image
    finally:
        ctx2.end()


# --- masked fills -------------------------------------------------------------------------------------

@pytest.mark.parametrize("seed", range(1400, 1405))
def test_masked_fills_vs_oracle(runtimes, seed):
    """A8-masked fills: integer / aligned double origins, areas, clipping, solid / gradient / pattern
    styles, fill and global alpha (unsupported placements draw nothing, as in the reference)."""
    sw = scenes.masks(seed=seed, count=120, width=(300, 61, 500)[seed % 3], height=(220, 203, 90)[seed % 3])
    stream = sw.to_bytes()
    got = bg.render_stream(runtimes(), stream)
    want = oracle_lib.render(stream)
    assert not _diff(got, want), _diff(got, want)


def test_fill_mask_context_calls(runtimes):
    rng = np.random.default_rng(11)
    w, h = 120, 90
    mask = rng.integers(0, 256, (40, 50), dtype=np.uint8)
    sw = scenes.StreamWriter(w, h)
    out = np.zeros((h, w), dtype=np.uint32)
    ctx = bg.Context(runtimes(), out)
    sw.solid(0xFF000000); sw.fill_all()
    ctx.set_fill_style_rgba32(0xFF000000); ctx.fill_all()
    sw.solid(0xFF40C0FF); ctx.set_fill_style_rgba32(0xFF40C0FF)
    sw.fill_mask_i(10, 5, mask); ctx.fill_mask_i(10, 5, mask)
    sw.fill_alpha(0.5); ctx.set_fill_alpha(0.5)
    sw.fill_mask_d(80.0, 60.0, mask, [5, 5, 30, 20]); ctx.fill_mask_d(80.0, 60.0, mask, [5, 5, 30, 20])
    with pytest.raises(bg.BLGpuError) as e:
        ctx.fill_mask_d(3.5, 4.0, mask)                      # not pixel aligned
    assert e.value.code == bg.ERROR_NOT_IMPLEMENTED
    ctx.end()
    stream = sw.to_bytes()
    assert not _diff(out, bg.render_stream(runtimes(), stream))
    assert not _diff(out, oracle_lib.render(stream))


# --- shapes ------------------------------------------------------------------------------------------

@pytest.mark.parametrize("seed", range(1500, 1504))
def test_shapes_vs_oracle(runtimes, seed):
    """Circles, ellipses, round rects and triangles, filled (both rules) and stroked."""
    sw = scenes.shapes(seed=seed, count=150, width=(320, 61, 500)[seed % 3], height=(240, 203, 90)[seed % 3])
    stream = sw.to_bytes()
    got = bg.render_stream(runtimes(), stream)
    want = oracle_lib.render(stream)
    assert not _diff(got, want), _diff(got, want)


def test_shape_context_calls_match_stream(runtimes):
    w, h = 140, 100
    sw = scenes.StreamWriter(w, h)
    out = np.zeros((h, w), dtype=np.uint32)
    ctx = bg.Context(runtimes(), out)
    sw.solid(0xFF000000); sw.fill_all()
    ctx.set_fill_style_rgba32(0xFF000000); ctx.fill_all()
    sw.solid(0xFFFF8040); ctx.set_fill_style_rgba32(0xFFFF8040)
    for gt, v in [(scenes.GEOMETRY_CIRCLE, [40, 40, 25]), (scenes.GEOMETRY_ELLIPSE, [100, 30, 30, 12]),
                  (scenes.GEOMETRY_ROUND_RECT, [60, 55, 70, 40, 12, 8]), (scenes.GEOMETRY_TRIANGLE, [5, 95, 40, 60, 70, 98])]:
        sw.fill_geometry(gt, v); ctx.fill_geometry(gt, v)
    sw.stroke_solid(0xFF20FFA0); ctx.set_stroke_style_rgba32(0xFF20FFA0)
    sw.stroke_width(3.0); ctx.set_stroke_width(3.0)
    sw.stroke_geometry(scenes.GEOMETRY_CIRCLE, [40, 40, 30]); ctx.stroke_geometry(scenes.GEOMETRY_CIRCLE, [40, 40, 30])
    sw.fill_geometry(scenes.GEOMETRY_PIE, [100, 70, 25, 20, 0.5, 4.0]); ctx.fill_geometry(scenes.GEOMETRY_PIE, [100, 70, 25, 20, 0.5, 4.0])
    sw.stroke_geometry(scenes.GEOMETRY_ARC, [70, 50, 40, 30, -1.0, -2.5]); ctx.stroke_geometry(scenes.GEOMETRY_ARC, [70, 50, 40, 30, -1.0, -2.5])
    with pytest.raises(bg.BLGpuError) as e:
        ctx.fill_geometry(21, [0, 0, 0, 0, 0, 0])               # BL_GEOMETRY_TYPE_PATH: its own entry point
    assert e.value.code == bg.ERROR_NOT_IMPLEMENTED
    ctx.end()
    stream = sw.to_bytes()
    assert not _diff(out, bg.render_stream(runtimes(), stream))
    assert not _diff(out, oracle_lib.render(stream))


def test_graph_frames_replay_new_frames_bit_exact():
    """With graph frames on, a frame that fits the captured layout is uploaded in place and the
    captured graph replayed (no host round trip inside the frame): different frames in a row,
    single canvases and batches, each bit-exact to the oracle; a frame larger than the layout
    grows it and still renders exactly."""
    with bg.Runtime(0) as rt:
        cfg = rt.launch_config()
        cfg.graph_frames = 1
        rt.set_launch_config(cfg)
        frames = [scenes.random_mix(7000 + i, width=200, height=150, count=120 - 7 * i).to_bytes() for i in range(6)]
        frames.append(scenes.random_mix(7100, width=320, height=240, count=400).to_bytes())   # larger: grows
        frames += [scenes.random_mix(7200 + i, width=180, height=140, count=60).to_bytes() for i in range(3)]
        for i, s in enumerate(frames):
            got = bg.render_stream(rt, s)
            want = oracle_lib.render(s)
            assert not _diff(got, want), f"frame {i}: {_diff(got, want)}"
        assert rt.stats().graph_frames >= 5       # the frames that fit replayed the graph
        # batches of different canvases through the same graph (the first one twice: once to
        # grow the layout to batch size, once through the graph for certain)
        before = rt.stats().graph_frames
        for k in (0, 0, 1, 2):
            sws = scenes.batch_canvases(seed=500 + k, count=12, max_side=300, max_paths=150)
            streams = [sw.to_bytes() for sw in sws]
            targets = [np.zeros((sw.height, sw.width), dtype=np.uint32) for sw in sws]
            rt.render_batch(streams, targets)
            for i, (s, t) in enumerate(zip(streams, targets)):
                assert not _diff(t, oracle_lib.render(s)), f"batch {k} canvas {i}"
        assert rt.stats().graph_frames > before


def test_page_locked_host_images_match_pageable_ones():
    """Page-locked host images are copied to and from the device by a kernel (the device reaches
    them directly), pageable ones by DMA: the same scenes give the same pixels either way, for
    canvases of every width modulo 4, batched and alone, onto existing content and onto a clear."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(91)
    streams, init = [], []
    for i, (w, h) in enumerate([(61, 37), (64, 40), (97, 3), (130, 77), (1, 1), (255, 129)]):
        sw = scenes.StreamWriter(w, h)
        for k in range(12):                       # SrcOver fills onto whatever the canvas holds
            sw.solid(int(rng.integers(0, 2**32)))
            sw.fill_rect_d(rng.uniform(-5, w), rng.uniform(-5, h), rng.uniform(1, w), rng.uniform(1, h))
        streams.append(sw.to_bytes())
        init.append(rng.integers(0, 2**32, (h, w), dtype=np.uint64).astype(np.uint32))
    streams.append(scenes.random_mix(92, width=203, height=101, count=150).to_bytes())
    init.append(np.zeros((101, 203), dtype=np.uint32))
    with bg.Runtime(0) as rt:
        pageable = [a.copy() for a in init]
        rt.render_batch(streams, pageable)
        pinned = [torch.from_numpy(a.view(np.int32).copy()).pin_memory() for a in init]
        rt.render_batch(streams, pinned)
        for i, (p, q) in enumerate(zip(pageable, pinned)):
            assert not _diff(q.numpy().view(np.uint32), p), f"batched canvas {i}"
        for i, s in enumerate(streams):
            p = init[i].copy()
            bg.render_stream(rt, s, p)
            q = torch.from_numpy(init[i].view(np.int32).copy()).pin_memory()
            bg.render_stream(rt, s, q)
            assert not _diff(q.numpy().view(np.uint32), p), f"canvas {i}"
            assert not _diff(p, pageable[i]), f"canvas {i} alone vs batched"


FORMAT_CASES = [(seed, w, h, fmt, xrgb) for seed, (w, h), fmt, xrgb in
                zip(range(1200, 1224), [(257, 257), (61, 37), (1, 1), (333, 97), (129, 130), (5, 600)] * 4,
                    [scenes.FORMAT_XRGB32, scenes.FORMAT_A8] * 12, [False, False, True, True] * 6)]


@pytest.mark.parametrize("seed,w,h,fmt,xrgb", FORMAT_CASES)
def test_target_formats_vs_oracle(runtimes, seed, w, h, fmt, xrgb):
    """XRGB32 and A8 targets (and XRGB32 pattern sources): the comp-op simplified for the formats,
    pattern texels read with their alpha set, A8 canvases one byte per pixel on the device."""
    stream = scenes.random_mix(seed, width=w, height=h, count=150, format=fmt, xrgb_images=xrgb,
                               dither=seed % 3 == 0).to_bytes()
    got = bg.render_stream(runtimes(), stream)
    want = oracle_lib.render(stream)
    assert got.dtype == want.dtype
    assert not _diff(got, want), _diff(got, want)


@pytest.mark.parametrize("fmt", [scenes.FORMAT_PRGB32, scenes.FORMAT_XRGB32, scenes.FORMAT_A8])
def test_blits_of_xrgb_images_vs_oracle(runtimes, fmt):
    stream = scenes.blits(seed=46, format=fmt, xrgb_images=True).to_bytes()
    got = bg.render_stream(runtimes(), stream)
    want = oracle_lib.render(stream)
    assert not _diff(got, want), _diff(got, want)


def test_target_formats_on_device_pinned_and_batched(runtimes):
    """A8 and XRGB32 canvases as CUDA tensors (aligned rows are rendered in place, others are
    staged), page-locked and pageable host images, and one batch mixing the three formats onto
    existing content."""
    torch = pytest.importorskip("torch")
    rt = runtimes()
    rng = np.random.default_rng(1230)
    streams, init = [], []
    for i, (w, h) in enumerate([(256, 64), (131, 77), (16, 9), (97, 40), (1, 1), (203, 101)]):
        fmt = (scenes.FORMAT_A8, scenes.FORMAT_XRGB32, scenes.FORMAT_PRGB32)[i % 3]
        streams.append(scenes.random_mix(1240 + i, width=w, height=h, count=120, format=fmt,
                                         xrgb_images=i % 2 == 0, alphas=True).to_bytes())
        dt = np.uint8 if fmt == scenes.FORMAT_A8 else np.uint32
        init.append(rng.integers(0, 256 if dt == np.uint8 else 2**32, (h, w), dtype=np.uint64).astype(dt))
    want = []
    for s, a in zip(streams, init):
        # the oracle starts from zeros: compare runs onto zeroed canvases with it, and runs onto
        # existing content with each other
        want.append(oracle_lib.render(s))
    for i, s in enumerate(streams):
        h, w = init[i].shape
        a8 = init[i].dtype == np.uint8
        dev = torch.zeros((h, w), dtype=torch.uint8 if a8 else torch.int32, device="cuda")
        bg.render_stream(rt, s, dev)
        torch.cuda.synchronize()
        got = dev.cpu().numpy()
        got = got if a8 else got.view(np.uint32)
        assert not _diff(got, want[i]), f"device canvas {i}: {_diff(got, want[i])}"
        pinned = torch.zeros((h, w), dtype=torch.uint8 if a8 else torch.int32).pin_memory()
        bg.render_stream(rt, s, pinned)
        got = pinned.numpy() if a8 else pinned.numpy().view(np.uint32)
        assert not _diff(got, want[i]), f"page-locked canvas {i}: {_diff(got, want[i])}"
    batched = [a.copy() for a in init]
    rt.render_batch(streams, batched)
    for i, s in enumerate(streams):
        alone = init[i].copy()
        bg.render_stream(rt, s, alone)
        assert not _diff(batched[i], alone), f"canvas {i} batched vs alone"


def test_target_format_context_calls(runtimes):
    """The context API on XRGB32 and A8 targets gives what the same calls recorded as a stream
    give on the oracle; a stream recorded for another format is refused."""
    rt = runtimes()
    img = scenes.premultiplied_noise(np.random.default_rng(3), 23, 17)
    for fmt in (scenes.FORMAT_XRGB32, scenes.FORMAT_A8):
        sw = scenes.StreamWriter(90, 70, fmt)
        x = sw.add_image(img, scenes.FORMAT_XRGB32)
        p = sw.add_image(img)
        target = np.zeros((70, 90), dtype=np.uint8 if fmt == scenes.FORMAT_A8 else np.uint32)
        ctx = bg.Context(rt, target, fmt)
        try:
            for op in (scenes.SRC_OVER, scenes.SRC_COPY):
                sw.comp_op(op); ctx.set_comp_op(op)
                sw.solid(0x80FF2010); ctx.set_fill_style_rgba32(0x80FF2010)
                sw.fill_rect_d(3.5, 4.25, 40, 20); ctx.fill_rect_d(3.5, 4.25, 40, 20)
                sw.pattern(x, scenes.REPEAT, transform=[1, 0.2, -0.1, 1, 10, 5])
                ctx.set_fill_style_pattern(img, extend_mode=bg.EXTEND_REPEAT, transform=[1, 0.2, -0.1, 1, 10, 5],
                                           format=bg.FORMAT_XRGB32)
                sw.fill_rect_d(20, 30, 50, 30); ctx.fill_rect_d(20, 30, 50, 30)
                sw.blit_image_d(50.5, 2.25, p); ctx.blit_image_d(50.5, 2.25, img)
                sw.blit_image_i(1, 50, x); ctx.blit_image_i(1, 50, img, format=bg.FORMAT_XRGB32)
            ctx.end()
        finally:
            ctx.close()
        want = oracle_lib.render(sw.to_bytes())
        assert not _diff(target, want), f"format {fmt}: {_diff(target, want)}"
    prgb_stream = scenes.random_mix(1250, width=40, height=30, count=10).to_bytes()
    with pytest.raises(bg.BLGpuError):
        bg.render_stream(rt, prgb_stream, np.zeros((30, 40), dtype=np.uint8))


def test_device_ordered_runtimes_take_turns():
    """Two runtimes with graph frames and device_order, taking steps in turn from two threads (their
    kernels chained on the device, their copies not): every step's canvases equal the oracle's."""
    import threading
    torch = pytest.importorskip("torch")
    batches = [[scenes.random_mix(1400 + 10 * k + i, width=60 + 23 * i, height=40 + 17 * i, count=90).to_bytes()
                for i in range(5)] for k in range(6)]
    want = [[oracle_lib.render(s) for s in b] for b in batches]
    cfg = bg.LaunchConfig(graph_frames=1, device_order=1, edge_block=128)
    rts = [bg.Runtime(0), bg.Runtime(0)]
    errors, got = [], {}
    try:
        for r in rts:
            r.set_launch_config(cfg)
            assert r.launch_config().device_order == 1

        def worker(k):
            try:
                for step in range(k, len(batches), 2):
                    tg = [torch.zeros(oracle_lib.stream_size(s)[::-1], dtype=torch.int32).pin_memory() for s in batches[step]]
                    rts[k].render_batch(batches[step], tg)
                    got[step] = [t.numpy().view(np.uint32).copy() for t in tg]
            except Exception as e:          # re-raised below
                errors.append(e)
        ths = [threading.Thread(target=worker, args=(k,)) for k in range(2)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
    finally:
        for r in rts:
            r.close()
    assert not errors, errors
    for step in range(len(batches)):
        for i, (g, w) in enumerate(zip(got[step], want[step])):
            assert not _diff(g, w), f"step {step} canvas {i}: {_diff(g, w)}"
