"""The drop-in boundary on the GPU: the same BLContext calls made on the reference's own raster
context and on a context begun with blgpu_blcontext_begin (include/blgpu_blcontext.h) give the
same pixels (tolerance: none - bit-exact): recorded scenes replayed call by call, and scenes
written against the BLContext API (paths and strokes at origins, per-call styles, transform
operations, integer geometry, state read-back, text)."""
import os
import tempfile

import pytest

import blcontext_lib
import oracle_lib

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not blcontext_lib.available(), reason="reference sources not staged (oracle/stage_ref.sh)")]

STREAM_SCENES = ["polygons", "curves_2k", "patterns_1k", "edge_cases", "conics", "mix_0", "mix_1", "mix_2", "mix_5",
                 "mix_notf_0", "mix_wide", "mix_tall", "mix_dither_1", "strokes_0", "strokes_wide", "strokes_lines",
                 "stroked_paths_2k", "blits_0", "blits_tall", "masks_0", "shapes_0", "shapes_1", "batch_0", "batch_3",
                 # XRGB32 and A8 targets, XRGB32 pattern and blit sources
                 "mix_xrgb_0", "mix_xrgb_1", "mix_a8_0", "mix_a8_1", "mix_a8_dither", "mix_xrgb_images_0",
                 "blits_xrgb_images_xrgb", "blits_xrgb_images_a8"]


def test_recorded_scenes_through_blcontext():
    golden = {e["name"]: e for e in oracle_lib.golden()["scenes"]}
    with tempfile.TemporaryDirectory() as td:
        paths = []
        for name in STREAM_SCENES:
            p = os.path.join(td, f"{name}.bin")
            with open(p, "wb") as f:
                f.write(oracle_lib.golden_stream(golden[name]))
            paths.append(p)
        lst = os.path.join(td, "list.txt")
        with open(lst, "w") as f:
            f.write("\n".join(paths) + "\n")
        rc, out, err = blcontext_lib.run("--streams", lst, "--lut", str(blcontext_lib.LUT))
    assert rc == 0, (out, err[-2000:])
    assert out["streams"] == len(STREAM_SCENES) and out["failed"] == 0


def test_blcontext_api_scenes_and_text():
    args = ["--scenes", "--lut", str(blcontext_lib.LUT)]
    if os.path.isfile(blcontext_lib.FONT):
        args += ["--font", blcontext_lib.FONT]
    rc, out, err = blcontext_lib.run(*args)
    assert rc == 0, (out, err[-2000:])
    assert out["failed"] == 0
