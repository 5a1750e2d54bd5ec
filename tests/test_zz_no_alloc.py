"""The no-allocation entry point (blgpu_render_stream_noalloc): same pixels as the context path,
two calls in a row, no device memory taken by the calls, oversized frames rejected. Kept in its own
file, collected last, so it runs both alone and after every other test."""
import numpy as np
import pytest

import blend2d_gb300 as bg
from blend2d_gb300 import scenes

pytestmark = pytest.mark.gpu


def _render_context(rt, stream, w, h, torch):
    ref = torch.zeros((h, w), dtype=torch.int32, device="cuda")
    bg.render_stream(rt, stream, ref)
    torch.cuda.synchronize()
    return ref.cpu().numpy().view(np.uint32)


def test_noalloc_matches_context_path_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    cases = [(31, 256, 160), (32, 200, 120), (33, 64, 300)]
    with bg.Runtime(0) as rt:
        streams = [scenes.random_mix(seed, width=w, height=h, count=120).to_bytes() for seed, w, h in cases]
        refs = [_render_context(rt, s, w, h, torch) for s, (_, w, h) in zip(streams, cases)]
        outs = [torch.full((h, w), 0x5A5A5A5A, dtype=torch.int32, device="cuda") for _, w, h in cases]
        torch.cuda.synchronize()
        rt.render_stream_noalloc(streams[0], outs[0])          # first call: looks up the scratch area
        free_before = torch.cuda.mem_get_info()[0]
        for s, o in zip(streams, outs):                         # two (and more) calls in a row
            rt.render_stream_noalloc(s, o)
        rt.render_stream_noalloc(streams[1], outs[1])
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        for i, (o, ref) in enumerate(zip(outs, refs)):
            got = o.cpu().numpy().view(np.uint32)
            assert np.array_equal(got, ref), f"case {i}: no-allocation render differs from the context path"
    assert free_after == free_before


def test_noalloc_rejects_frames_beyond_its_area():
    torch = pytest.importorskip("torch")
    sw = scenes.curves(count=20000)              # ~2.2 M segments: far more than the scratch area holds
    out = torch.zeros((sw.height, sw.width), dtype=torch.int32, device="cuda")
    with bg.Runtime(0) as rt:
        with pytest.raises(bg.BLGpuError) as ei:
            rt.render_stream_noalloc(sw.to_bytes(), out)
        assert ei.value.code == bg.ERROR_DATA_TOO_LARGE
    torch.cuda.synchronize()
    assert int(out.abs().sum().item()) == 0     # the image is left unchanged


def test_noalloc_rejects_host_images():
    with bg.Runtime(0) as rt:
        host = np.zeros((16, 16), dtype=np.uint32)
        stream = scenes.random_mix(1, width=16, height=16, count=5).to_bytes()
        with pytest.raises(bg.BLGpuError) as ei:
            rt.render_stream_noalloc(stream, host)
        assert ei.value.code == bg.ERROR_INVALID_VALUE


def test_noalloc_reports_strokes_as_not_implemented():
    """Stroke outlines are sized by a device pass whose buffers the fixed area does not hold."""
    torch = pytest.importorskip("torch")
    sw = scenes.strokes(seed=3, width=64, height=48, count=5)
    out = torch.zeros((sw.height, sw.width), dtype=torch.int32, device="cuda")
    with bg.Runtime(0) as rt:
        with pytest.raises(bg.BLGpuError) as ei:
            rt.render_stream_noalloc(sw.to_bytes(), out)
        assert ei.value.code == bg.ERROR_NOT_IMPLEMENTED
