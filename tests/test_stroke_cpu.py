"""CPU checks of stroking. The oracle's stroker is pinned to the reference by the golden stroke
scenes (test_oracle_golden); here the product's host stroker (libblgpu.so, no device needed) is
checked against it: the outline it records, filled non-zero through the oracle's rasterizer, must
give the pixels of the oracle's own stroke of the same geometry, bit for bit."""

import numpy as np
import pytest

import blend2d_gb300 as bg
from blend2d_gb300 import scenes

import oracle_lib as ol


def _pair(seed, count=80, w=240, h=180, max_width=30.0, curves=True, before=False):
    """Two streams: strokes (oracle stroker) and the product outlines of the same strokes as fills."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ss, sf = scenes.StreamWriter(w, h), scenes.StreamWriter(w, h)
    for sw in (ss, sf):
        sw.solid(0xFF000000)
        sw.fill_all()
    lin = None
    if before:
        # transform order BEFORE: the path is mapped by the linear part, the translation stays
        m = [1.1, 0.35, -0.25, 0.8, 13.0, -6.5]
        ss.transform(m)
        ss.stroke_transform_order(scenes.TRANSFORM_ORDER_BEFORE)
        sf.transform([1.0, 0.0, 0.0, 1.0, m[4], m[5]])
        lin = m
    for _ in range(count):
        side = float(rng.uniform(6, 120))
        x0, y0 = (float(v) for v in rng.uniform(-20, max(w, h) - 40, 2))
        width = float(np.exp(rng.uniform(np.log(0.5), np.log(max_width))))
        join = int(rng.integers(0, 5))
        caps = int(rng.integers(0, 6)), int(rng.integers(0, 6))
        ml = float(rng.uniform(1.0, 10.0))
        cmds, xy = [], []
        for _f in range(int(rng.integers(1, 3))):
            fc, fxy = scenes._stroke_figure(rng, x0, y0, side, closed=bool(rng.random() < 0.4), curves=curves)
            cmds += fc
            xy += fxy
        xy = np.array(xy, dtype=np.float64)
        col = int(rng.integers(0, 2**32, dtype=np.uint64))
        ss.stroke_width(width); ss.stroke_join(join); ss.stroke_caps(*caps); ss.stroke_miter_limit(ml)
        ss.stroke_solid(col)
        ss.stroke_path(cmds, xy)
        src = xy
        if lin is not None:
            src = np.stack([xy[:, 0] * lin[0] + xy[:, 1] * lin[2] + 0.0,
                            xy[:, 0] * lin[1] + xy[:, 1] * lin[3] + 0.0], axis=1)
        oc, ox = bg.stroke_outline(cmds, src, width, ml, join, *caps)
        sf.solid(col)
        if len(oc):
            sf.fill_path(oc, ox)
    return ss.to_bytes(), sf.to_bytes()


@pytest.mark.parametrize("seed", range(8))
def test_product_outline_fills_like_the_oracle_stroke(seed):
    a, b = _pair(seed, curves=seed % 4 != 3, max_width=(30.0, 4.0, 80.0, 12.0)[seed % 4])
    ra, rb = ol.render(a), ol.render(b)
    assert int((ra != rb).sum()) == 0


@pytest.mark.parametrize("seed", range(3))
def test_product_outline_transform_order_before(seed):
    a, b = _pair(100 + seed, before=True)
    assert int((ol.render(a) != ol.render(b)).sum()) == 0


def test_outline_of_closed_and_open_figures():
    """A closed square strokes to two figures (outer, inner reversed); an open line to one loop."""
    sq = np.array([[10, 10], [50, 10], [50, 50], [10, 50], [np.nan, np.nan]], dtype=np.float64)
    oc, ox = bg.stroke_outline([0, 1, 1, 1, 5], sq, width=4.0, join=scenes.JOIN_MITER_CLIP)
    assert list(oc).count(scenes.P_MOVE) == 2 and scenes.P_CLOSE not in oc
    assert np.isfinite(ox).all()
    oc, ox = bg.stroke_outline([0, 1], np.array([[0.0, 0.0], [10.0, 0.0]]), width=2.0)
    assert list(oc) == [0, 1, 1, 1, 1]                       # A, butt end cap, B reversed, butt start cap
    np.testing.assert_array_equal(ox, [[0, 1], [10, 1], [10, -1], [0, -1], [0, 1]])


def test_invalid_geometry_is_rejected_with_nothing_drawn():
    with pytest.raises(bg.BLGpuError) as e:
        bg.stroke_outline([1, 1], np.array([[0.0, 0.0], [5.0, 5.0]]))   # no MOVE first
    assert e.value.code == bg.ERROR_INVALID_GEOMETRY
    with pytest.raises(bg.BLGpuError):
        bg.stroke_outline([0, 2], np.array([[0.0, 0.0], [5.0, 5.0]]))   # quad missing its end point
    # a figure with a single point has no direction and strokes to nothing
    oc, _ = bg.stroke_outline([0], np.array([[3.0, 4.0]]))
    assert len(oc) == 0


@pytest.mark.parametrize("join", range(5))
def test_long_figures_through_the_vertex_window(join):
    """Figures far longer than the stroker's window of patchable vertices: closed polygons whose
    closing join moves the figure's first vertex after it was handed out, open polylines, and
    cubic chains."""
    rng = np.random.Generator(np.random.PCG64(700 + join))
    w, h = 300, 220
    ss, sf = scenes.StreamWriter(w, h), scenes.StreamWriter(w, h)
    for sw in (ss, sf):
        sw.solid(0xFF000000)
        sw.fill_all()
    for k in range(6):
        npts = int(rng.integers(40, 160))
        ang = np.sort(rng.uniform(0, 2 * np.pi, npts))
        rad = rng.uniform(30, 100, npts)
        xy = np.stack([150 + rad * np.cos(ang), 110 + rad * np.sin(ang)], axis=1)
        if k % 3 == 0:
            cmds = [0] + [1] * (npts - 1) + [5]
            xy = np.vstack([xy, [np.nan, np.nan]])
        elif k % 3 == 1:
            cmds = [0] + [1] * (npts - 1)
        else:
            m = (npts - 1) // 3
            cmds = [0] + [4, 4, 1] * m
            xy = xy[: 1 + 3 * m]
        width = float(rng.uniform(1.0, 14.0))
        caps = int(rng.integers(0, 6)), int(rng.integers(0, 6))
        col = int(rng.integers(0, 2**32, dtype=np.uint64))
        ss.stroke_width(width); ss.stroke_join(join); ss.stroke_caps(*caps); ss.stroke_miter_limit(8.0)
        ss.stroke_solid(col)
        ss.stroke_path(cmds, xy)
        oc, ox = bg.stroke_outline(cmds, xy, width, 8.0, join, *caps)
        sf.solid(col)
        sf.fill_path(oc, ox)
    assert int((ol.render(ss.to_bytes()) != ol.render(sf.to_bytes())).sum()) == 0
