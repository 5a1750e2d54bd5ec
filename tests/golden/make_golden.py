"""Generates tests/golden/golden.json from the reference Blend2D library.

Run in a checkout that has the reference sources (default /root/reference); it builds the
reference with oracle/ref.mk (no CMake) into oracle/_ref/ and records:

  * scenes  - sha256 of the pixels the reference renders for seeded command streams (4 bytes
              per pixel; 1 for the A8 targets of the mix_a8 scenes)
              (blend2d_gb300.scenes; the mix_dither / curves_dither scenes use gradient quality
              DITHER, whose 64-bit LUT has a single builder; strokes_* / stroked_paths_* stroke
              paths, polylines, polygons, boxes, rects and lines; blits_* image blits; masks_* masked fills; shapes_* circles, ellipses, round rects and triangles), for the stock no-JIT x86-64 build ("default", SSE2 LUT
              builder) and, for a subset, the portable-LUT build ("scalar");
  * luts    - sha256 of the gradient LUTs produced by the reference's three builders
              (interpolate_prgb32 / _sse2 / _avx2) for random stop arrays;
  * lines   - sha256 of the dense cell grid the reference's analytic rasterizer produces for
              random 24.8 lines, rasterized band by band; every line is rasterized with four band
              heights and the script asserts the grids agree (the banding invariance the
              reference's own unit test checks, analyticrasterizer_test.cpp:34-155).

The JSON is committed; tests read only the JSON, never the reference.

    python tests/golden/make_golden.py [--ref /root/reference] [--full]
"""

from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from blend2d_gb300 import scenes  # noqa: E402

REF_OUT = os.path.join(ROOT, "oracle", "_ref")


def scene_catalog(full: bool):
    """(name, callable, lut variants) - the callables are re-evaluated by the tests."""
    cat = [
        ("polygons", "scenes.polygons()", ("default", "scalar")),
        ("curves_2k", "scenes.curves(count=2000)", ("default",)),
        ("patterns_1k", "scenes.patterns(count=500, width=1024, height=1024)", ("default",)),
        ("edge_cases", "scenes.edge_cases()", ("default", "scalar")),
        ("conics", "scenes.conic_paths()", ("default",)),
    ]
    for s in range(24):
        cat.append((f"mix_{s}", f"scenes.random_mix({s})", ("default",) if s % 4 else ("default", "scalar")))
    for s in range(4):
        cat.append((f"mix_notf_{s}", f"scenes.random_mix({100 + s}, count=400, transforms=False, alphas=False)", ("default",)))
    cat.append(("mix_wide", "scenes.random_mix(200, width=1031, height=77, count=300)", ("default",)))
    cat.append(("mix_tall", "scenes.random_mix(201, width=61, height=1500, count=300)", ("default",)))
    for s in range(6):
        cat.append((f"mix_dither_{s}", f"scenes.random_mix({300 + s}, dither=True)", ("default",) if s % 2 else ("default", "scalar")))
    cat.append(("curves_dither", "scenes.curves(count=600, width=640, height=360, dither=True)", ("default",)))
    for s in range(6):
        cat.append((f"strokes_{s}", f"scenes.strokes(seed={20 + s}, count=250)", ("default",)))
    cat.append(("strokes_wide", "scenes.strokes(seed=30, count=300, max_width=90.0)", ("default",)))
    cat.append(("strokes_lines", "scenes.strokes(seed=31, count=300, curves=False)", ("default",)))
    cat.append(("strokes_small", "scenes.strokes(seed=32, width=61, height=97, count=60)", ("default",)))
    cat.append(("stroked_paths_2k", "scenes.stroked_paths(count=2000)", ("default",)))
    for s in range(4):
        cat.append((f"blits_{s}", f"scenes.blits(seed={40 + s}, count=200)", ("default",)))
    cat.append(("blits_tall", "scenes.blits(seed=44, width=97, height=301)", ("default",)))
    for s in range(3):
        cat.append((f"masks_{s}", f"scenes.masks(seed={50 + s}, count=150)", ("default",)))
    for s in range(3):
        cat.append((f"shapes_{s}", f"scenes.shapes(seed={60 + s}, count=200)", ("default",)))
    for i in range(6):
        cat.append((f"batch_{i}", f"scenes.batch_canvases(seed=4, count=6, max_side=640, max_paths=400)[{i}]", ("default",)))
    # XRGB32 and A8 targets, XRGB32 pattern and blit sources
    for s in range(4):
        cat.append((f"mix_xrgb_{s}", f"scenes.random_mix({400 + s}, format=scenes.FORMAT_XRGB32, xrgb_images={s % 2 == 1})",
                    ("default",) if s else ("default", "scalar")))
        cat.append((f"mix_a8_{s}", f"scenes.random_mix({410 + s}, format=scenes.FORMAT_A8, xrgb_images={s % 2 == 1})",
                    ("default",) if s else ("default", "scalar")))
        cat.append((f"mix_xrgb_images_{s}", f"scenes.random_mix({420 + s}, xrgb_images=True)", ("default",)))
    cat.append(("mix_a8_dither", "scenes.random_mix(430, format=scenes.FORMAT_A8, dither=True)", ("default",)))
    cat.append(("mix_xrgb_dither", "scenes.random_mix(431, format=scenes.FORMAT_XRGB32, dither=True)", ("default",)))
    for f, tag in (("scenes.FORMAT_PRGB32", "prgb"), ("scenes.FORMAT_XRGB32", "xrgb"), ("scenes.FORMAT_A8", "a8")):
        cat.append((f"blits_xrgb_images_{tag}", f"scenes.blits(seed=45, format={f}, xrgb_images=True)", ("default",)))
    if full:
        # the benchmarked workloads at full size: the 20,000-path curves frame, the 50,000-quad
        # pattern frame, a sample of the 4,096 batched canvases (the largest, the one with the
        # most paths, the largest area x paths, eight seeded picks) and of the serving requests
        cat.append(("curves", "scenes.curves()", ("default", "scalar")))
        cat.append(("patterns", "scenes.patterns()", ("default",)))
        for i in BATCH_SAMPLE:
            cat.append((f"batch4096_{i}", f"scenes.batch_canvas({i})", ("default", "scalar")))
        for i in SERVE_SAMPLE:
            cat.append((f"serve48_{i}", f"scenes.serving_request({i})", ("default",)))
    return cat


# Canvases of scenes.batch_canvases() (4,096) and requests of scenes.serving_requests(count=48)
# recorded at full size: the largest canvas (798), the most paths (2537), the largest area x
# paths (248) and eight seeded picks; for serving, the largest side (9), the most paths (28) and
# two more with over 10,000 paths on large canvases (1, 27).
BATCH_SAMPLE = (248, 429, 701, 798, 1071, 1555, 2537, 3779, 3994, 4004, 4041)
SERVE_SAMPLE = (1, 9, 27, 28)


def build_reference(ref: str):
    for variant in ("default", "scalar"):
        subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "ref.mk"), f"REF={ref}",
                        f"VARIANT={variant}", f"-j{os.cpu_count() or 4}"], check=True, cwd=ROOT)


def render_ref(stream: bytes, variant: str) -> str:
    with tempfile.TemporaryDirectory() as td:
        sp, op = os.path.join(td, "s.bin"), os.path.join(td, "o.raw")
        with open(sp, "wb") as f:
            f.write(stream)
        subprocess.run([os.path.join(REF_OUT, f"b2d_replay_{variant}"), sp, op], check=True)
        with open(op, "rb") as f:
            return hashlib.sha256(f.read()).hexdigest()


def lut_cases(rng, n_cases=96):
    out = []
    for t in range(n_cases):
        k = int(rng.integers(1, 9))
        stops = scenes._random_stops(rng, k)
        if t % 3 == 0:
            stops[0] = (0.0, stops[0][1])
        if t % 5 == 0:
            stops[-1] = (1.0, stops[-1][1])
        if t % 7 == 0 and k > 2:
            stops[1] = (stops[0][0], stops[1][1])
        if t % 11 == 0 and k > 1:
            stops[-1] = (stops[-2][0] + 1e-4 if stops[-2][0] < 0.999 else 1.0, stops[-1][1])
        size = (256, 512, 1024)[t % 3]
        out.append((size, [(o, scenes.rgba64_from_rgba32(c)) for o, c in stops]))
    return out


def _words_sha256(hexstr: str) -> str:
    """The harnesses print u32 words as %08x; hash them as little-endian uint32 arrays."""
    arr = np.frombuffer(bytes.fromhex(hexstr), dtype=">u4").astype("<u4")
    return hashlib.sha256(arr.tobytes()).hexdigest()


def reference_luts(cases):
    lines = []
    for size, stops in cases:
        parts = [str(size), str(len(stops))]
        for off, rgba in stops:
            parts += [float(off).hex(), "%x" % rgba]
        lines.append(" ".join(parts))
    res = subprocess.run([os.path.join(REF_OUT, "b2d_reflut")], input="\n".join(lines) + "\n",
                         capture_output=True, text=True, check=True)
    out = []
    for line in res.stdout.strip().split("\n"):
        a, b, c = line.split()
        out.append({"scalar": _words_sha256(a), "sse2": _words_sha256(b), "avx2": _words_sha256(c)})
    return out


def line_cases(rng, n=240):
    out = []
    for i in range(n):
        w = int(rng.integers(4, 90))
        rows = int(rng.integers(4, 90))
        x0, x1 = (int(v) for v in rng.integers(0, w * 256 + 1, 2))
        y0, y1 = (int(v) for v in rng.integers(0, rows * 256 + 1, 2))
        if i % 9 == 0:
            x1 = x0                     # vertical
        if i % 13 == 0:
            y1 = y0 + int(rng.integers(1, 40))   # nearly horizontal
        if y0 == y1:
            y1 = min(rows * 256, y0 + 1)
            if y0 == y1:
                y0 -= 1
        if y0 > y1:
            x0, x1, y0, y1 = x1, x0, y1, y0
        out.append((w, rows, x0, y0, x1, y1, int(rng.integers(0, 2))))
    return out


def reference_lines(cases):
    grids = {}
    for bh in (1, 4, 16, 64):
        inp = "\n".join(f"{w} {r} {bh} {x0} {y0} {x1} {y1} {s}" for (w, r, x0, y0, x1, y1, s) in cases) + "\n"
        res = subprocess.run([os.path.join(REF_OUT, "b2d_refras")], input=inp, capture_output=True, text=True, check=True)
        grids[bh] = [_words_sha256(x) for x in res.stdout.strip().split("\n")]
    for bh in (4, 16, 64):
        assert grids[bh] == grids[1], f"reference cells depend on band height {bh}"
    return grids[1]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--full", action="store_true", help="also render the full-size curve and pattern workloads")
    ap.add_argument("--update", action="store_true",
                    help="keep the entries of the existing golden.json whose stream bytes are unchanged; render the rest")
    args = ap.parse_args()
    build_reference(args.ref)

    kept = {}
    if args.update:
        with open(os.path.join(HERE, "golden.json")) as f:
            old = json.load(f)
        kept = {e["name"]: e for e in old["scenes"]}
    golden = {"note": "generated by tests/golden/make_golden.py from the reference library", "scenes": [], "luts": [], "lines": []}
    for name, expr, variants in scene_catalog(args.full):
        sw = eval(expr, {"scenes": scenes})
        stream = sw.to_bytes()
        digest = hashlib.sha256(stream).hexdigest()
        prev = kept.get(name)
        if prev and prev["expr"] == expr and prev["stream_sha256"] == digest and set(prev["pixels_sha256"]) == set(variants):
            golden["scenes"].append(prev)
            continue
        entry = {"name": name, "expr": expr, "width": sw.width, "height": sw.height, "format": sw.format,
                 "stream_sha256": digest, "pixels_sha256": {}}
        for v in variants:
            entry["pixels_sha256"][v] = render_ref(stream, v)
        golden["scenes"].append(entry)
        print(name, entry["pixels_sha256"], flush=True)

    rng = np.random.Generator(np.random.PCG64(2024))
    cases = lut_cases(rng)
    hashes = reference_luts(cases)
    for (size, stops), h in zip(cases, hashes):
        golden["luts"].append({"size": size, "stops": [[float(o).hex(), "%x" % c] for o, c in stops], "sha256": h})

    lines = line_cases(rng)
    for (w, r, x0, y0, x1, y1, s), h in zip(lines, reference_lines(lines)):
        golden["lines"].append({"w": w, "rows": r, "x0": x0, "y0": y0, "x1": x1, "y1": y1, "sign": s, "sha256": h})

    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()
