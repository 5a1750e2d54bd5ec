"""Seeded synthetic render workloads serialized as blgpu command streams.

The stream format is defined in include/blgpu_stream.h; every record mirrors one call of the
reference's BLContext API (blend2d/core/context.h), so the same bytes can be replayed into the
reference library, into the CPU oracle and into the GPU backend.

The workload shapes restate the benchmark configurations this backend is measured on:
  * ``polygons``  - 512x512 canvas, 2,000 ten-vertex polygons in 64x64 boxes, solid colours;
  * ``curves``    - 1920x1080 canvas, 20,000 closed cubic paths with linear/radial/conic gradients;
  * ``patterns``  - 4096x4096 canvas, 50,000 affine-transformed pattern quads (NN/BI, SrcCopy/SrcOver);
  * ``batch``     - many independent canvases of uneven sizes (see ``batch_canvases``);
plus ``random_mix`` - small scenes in the style of the reference's differential context tester
(blend2d-testing/tests/bl_test_context_utilities.h:508-1223): rects, polygons, quad/cubic paths,
all fill styles, both comp-ops, fill alpha and transforms.

Randomness comes from numpy's PCG64, which is platform independent, so a (kind, seed) pair
always serializes to the same bytes.
"""

from __future__ import annotations

import math
import struct

import numpy as np

MAGIC = 0x53443242
VERSION = 1

OP_END = 0
OP_SET_COMP_OP = 1
OP_SET_FILL_RULE = 2
OP_SET_GLOBAL_ALPHA = 3
OP_SET_FILL_ALPHA = 4
OP_SET_HINT = 5
OP_SET_TRANSFORM = 6
OP_RESET_TRANSFORM = 7
OP_STYLE_RGBA32 = 8
OP_STYLE_GRADIENT = 9
OP_STYLE_PATTERN = 10
OP_CLEAR_ALL = 11
OP_FILL_ALL = 12
OP_FILL_RECT_I = 13
OP_FILL_RECT_D = 14
OP_FILL_BOX_D = 15
OP_FILL_POLYGON_D = 16
OP_FILL_PATH_D = 17
OP_SAVE = 18
OP_RESTORE = 19
OP_SET_STROKE_WIDTH = 20
OP_SET_STROKE_MITER_LIMIT = 21
OP_SET_STROKE_JOIN = 22
OP_SET_STROKE_CAPS = 23
OP_SET_STROKE_TRANSFORM_ORDER = 24
OP_SET_STROKE_ALPHA = 25
OP_STROKE_STYLE_RGBA32 = 26
OP_STROKE_STYLE_GRADIENT = 27
OP_STROKE_STYLE_PATTERN = 28
OP_STROKE_PATH_D = 29
OP_STROKE_POLYLINE_D = 30
OP_STROKE_POLYGON_D = 31
OP_STROKE_BOX_D = 32
OP_STROKE_RECT_D = 33
OP_STROKE_LINE_D = 34
OP_BLIT_IMAGE_I = 35
OP_BLIT_IMAGE_D = 36
OP_BLIT_SCALED_IMAGE_I = 37
OP_BLIT_SCALED_IMAGE_D = 38
OP_FILL_MASK_I = 39
OP_FILL_MASK_D = 40
OP_FILL_GEOMETRY = 41
OP_STROKE_GEOMETRY = 42
GEOMETRY_CIRCLE, GEOMETRY_ELLIPSE, GEOMETRY_ROUND_RECT, GEOMETRY_TRIANGLE = 5, 6, 7, 12   # BLGeometryType
GEOMETRY_ARC, GEOMETRY_CHORD, GEOMETRY_PIE = 8, 9, 10

SRC_OVER, SRC_COPY = 0, 1
FORMAT_PRGB32, FORMAT_XRGB32, FORMAT_A8 = 1, 2, 3                                              # BLFormat
NON_ZERO, EVEN_ODD = 0, 1
LINEAR, RADIAL, CONIC = 0, 1, 2
PAD, REPEAT, REFLECT = 0, 1, 2
HINT_GRADIENT_QUALITY, HINT_PATTERN_QUALITY = 1, 2
GRADIENT_NEAREST, GRADIENT_SMOOTH, GRADIENT_DITHER = 0, 1, 2        # BLGradientQuality
NEAREST, BILINEAR = 0, 1
P_MOVE, P_ON, P_QUAD, P_CONIC, P_CUBIC, P_CLOSE = 0, 1, 2, 3, 4, 5
JOIN_MITER_CLIP, JOIN_MITER_BEVEL, JOIN_MITER_ROUND, JOIN_BEVEL, JOIN_ROUND = 0, 1, 2, 3, 4     # BLStrokeJoin
CAP_BUTT, CAP_SQUARE, CAP_ROUND, CAP_ROUND_REV, CAP_TRIANGLE, CAP_TRIANGLE_REV = 0, 1, 2, 3, 4, 5  # BLStrokeCap
TRANSFORM_ORDER_AFTER, TRANSFORM_ORDER_BEFORE = 0, 1                                          # BLStrokeTransformOrder


def rgba64_from_rgba32(c: int) -> int:
    """BLRgba64 from BLRgba32: every 8-bit channel c becomes c * 0x101 (rgba.h)."""
    a, r, g, b = (c >> 24) & 255, (c >> 16) & 255, (c >> 8) & 255, c & 255
    return ((a * 257) << 48) | ((r * 257) << 32) | ((g * 257) << 16) | (b * 257)


class StreamWriter:
    """Builds one command stream (one canvas, one frame)."""

    def __init__(self, width: int, height: int, format: int = FORMAT_PRGB32):
        self.width = int(width)
        self.height = int(height)
        self.format = int(format)             # the target's BLFormat
        self.images: list[np.ndarray] = []
        self.image_formats: list[int] = []
        self.parts: list[bytes] = []
        self.fill_count = 0

    # -- images ---------------------------------------------------------------------------------
    def add_image(self, pixels: np.ndarray, format: int = FORMAT_PRGB32) -> int:
        """A pattern / blit source: 32-bit pixels, PRGB32 or XRGB32 (whose alpha bytes the
        fetchers read as 0xFF)."""
        assert pixels.dtype == np.uint32 and pixels.ndim == 2 and pixels.shape[0] <= 65535
        assert format in (FORMAT_PRGB32, FORMAT_XRGB32)
        self.images.append(np.ascontiguousarray(pixels))
        self.image_formats.append(int(format))
        return len(self.images) - 1

    # -- records --------------------------------------------------------------------------------
    def _rec(self, op: int, payload: bytes = b"") -> None:
        pad = (-len(payload)) % 8
        self.parts.append(struct.pack("<II", op, len(payload) + pad) + payload + b"\0" * pad)

    def comp_op(self, op: int):
        self._rec(OP_SET_COMP_OP, struct.pack("<II", op, 0))

    def fill_rule(self, rule: int):
        self._rec(OP_SET_FILL_RULE, struct.pack("<II", rule, 0))

    def global_alpha(self, a: float):
        self._rec(OP_SET_GLOBAL_ALPHA, struct.pack("<d", a))

    def fill_alpha(self, a: float):
        self._rec(OP_SET_FILL_ALPHA, struct.pack("<d", a))

    def hint(self, hint: int, value: int):
        self._rec(OP_SET_HINT, struct.pack("<II", hint, value))

    def transform(self, m):
        self._rec(OP_SET_TRANSFORM, struct.pack("<6d", *m))

    def reset_transform(self):
        self._rec(OP_RESET_TRANSFORM)

    def solid(self, argb32: int):
        self._rec(OP_STYLE_RGBA32, struct.pack("<II", int(argb32) & 0xFFFFFFFF, 0))

    @staticmethod
    def _gradient_payload(gtype, values, extend, stops, transform):
        vals = list(values) + [0.0] * (6 - len(values))
        tr = list(transform) if transform is not None else [1.0, 0.0, 0.0, 1.0, 0.0, 0.0]
        payload = struct.pack("<IIII6d6d", gtype, extend, len(stops), 1 if transform is not None else 0, *vals, *tr)
        for off, argb in stops:
            payload += struct.pack("<dQ", float(off), rgba64_from_rgba32(int(argb)))
        return payload

    @staticmethod
    def _pattern_payload(image_index, extend, area, transform):
        ar = list(area) if area is not None else [0, 0, 0, 0]
        tr = list(transform) if transform is not None else [1.0, 0.0, 0.0, 1.0, 0.0, 0.0]
        return struct.pack("<II4iII6d", image_index, extend, *ar, 1 if transform is not None else 0, 0, *tr)

    def gradient(self, gtype: int, values, extend: int, stops, transform=None):
        self._rec(OP_STYLE_GRADIENT, self._gradient_payload(gtype, values, extend, stops, transform))

    def pattern(self, image_index: int, extend: int = PAD, area=None, transform=None):
        self._rec(OP_STYLE_PATTERN, self._pattern_payload(image_index, extend, area, transform))

    # -- stroke state (the stroke style slot and BLStrokeOptions) -------------------------------
    def stroke_solid(self, argb32: int):
        self._rec(OP_STROKE_STYLE_RGBA32, struct.pack("<II", int(argb32) & 0xFFFFFFFF, 0))

    def stroke_gradient(self, gtype: int, values, extend: int, stops, transform=None):
        self._rec(OP_STROKE_STYLE_GRADIENT, self._gradient_payload(gtype, values, extend, stops, transform))

    def stroke_pattern(self, image_index: int, extend: int = PAD, area=None, transform=None):
        self._rec(OP_STROKE_STYLE_PATTERN, self._pattern_payload(image_index, extend, area, transform))

    def stroke_alpha(self, a: float):
        self._rec(OP_SET_STROKE_ALPHA, struct.pack("<d", a))

    def stroke_width(self, w: float):
        self._rec(OP_SET_STROKE_WIDTH, struct.pack("<d", w))

    def stroke_miter_limit(self, m: float):
        self._rec(OP_SET_STROKE_MITER_LIMIT, struct.pack("<d", m))

    def stroke_join(self, join: int):
        self._rec(OP_SET_STROKE_JOIN, struct.pack("<II", join, 0))

    def stroke_caps(self, start: int, end: int):
        self._rec(OP_SET_STROKE_CAPS, struct.pack("<II", start, end))

    def stroke_transform_order(self, order: int):
        self._rec(OP_SET_STROKE_TRANSFORM_ORDER, struct.pack("<II", order, 0))

    def clear_all(self):
        self._rec(OP_CLEAR_ALL)
        self.fill_count += 1

    def fill_all(self):
        self._rec(OP_FILL_ALL)
        self.fill_count += 1

    def fill_rect_i(self, x, y, w, h):
        self._rec(OP_FILL_RECT_I, struct.pack("<4i", int(x), int(y), int(w), int(h)))
        self.fill_count += 1

    def fill_rect_d(self, x, y, w, h):
        self._rec(OP_FILL_RECT_D, struct.pack("<4d", x, y, w, h))
        self.fill_count += 1

    def fill_box_d(self, x0, y0, x1, y1):
        self._rec(OP_FILL_BOX_D, struct.pack("<4d", x0, y0, x1, y1))
        self.fill_count += 1

    def fill_polygon(self, xy: np.ndarray):
        xy = np.ascontiguousarray(xy, dtype="<f8").reshape(-1, 2)
        self._rec(OP_FILL_POLYGON_D, struct.pack("<II", xy.shape[0], 0) + xy.tobytes())
        self.fill_count += 1

    def fill_path(self, cmds, xy: np.ndarray):
        cmds = bytes(bytearray(cmds))
        xy = np.ascontiguousarray(xy, dtype="<f8").reshape(-1, 2)
        assert len(cmds) == xy.shape[0]
        pad = (-len(cmds)) % 8
        self._rec(OP_FILL_PATH_D, struct.pack("<II", len(cmds), 0) + cmds + b"\0" * pad + xy.tobytes())
        self.fill_count += 1

    # -- strokes --------------------------------------------------------------------------------
    def stroke_path(self, cmds, xy: np.ndarray):
        cmds = bytes(bytearray(cmds))
        xy = np.ascontiguousarray(xy, dtype="<f8").reshape(-1, 2)
        assert len(cmds) == xy.shape[0]
        pad = (-len(cmds)) % 8
        self._rec(OP_STROKE_PATH_D, struct.pack("<II", len(cmds), 0) + cmds + b"\0" * pad + xy.tobytes())
        self.fill_count += 1

    def stroke_polyline(self, xy: np.ndarray):
        xy = np.ascontiguousarray(xy, dtype="<f8").reshape(-1, 2)
        self._rec(OP_STROKE_POLYLINE_D, struct.pack("<II", xy.shape[0], 0) + xy.tobytes())
        self.fill_count += 1

    def stroke_polygon(self, xy: np.ndarray):
        xy = np.ascontiguousarray(xy, dtype="<f8").reshape(-1, 2)
        self._rec(OP_STROKE_POLYGON_D, struct.pack("<II", xy.shape[0], 0) + xy.tobytes())
        self.fill_count += 1

    def stroke_box_d(self, x0, y0, x1, y1):
        self._rec(OP_STROKE_BOX_D, struct.pack("<4d", x0, y0, x1, y1))
        self.fill_count += 1

    def stroke_rect_d(self, x, y, w, h):
        self._rec(OP_STROKE_RECT_D, struct.pack("<4d", x, y, w, h))
        self.fill_count += 1

    def stroke_line_d(self, x0, y0, x1, y1):
        self._rec(OP_STROKE_LINE_D, struct.pack("<4d", x0, y0, x1, y1))
        self.fill_count += 1

    # -- image blits ----------------------------------------------------------------------------
    def _blit(self, op, rect, image_index, area):
        r = [float(v) for v in rect] + [0.0] * (4 - len(rect))
        ar = list(area) if area is not None else [0, 0, 0, 0]
        self._rec(op, struct.pack("<4dII4i", *r, image_index, 1 if area is not None else 0, *ar))
        self.fill_count += 1

    def blit_image_i(self, x, y, image_index, area=None):
        self._blit(OP_BLIT_IMAGE_I, [int(x), int(y)], image_index, area)

    def blit_image_d(self, x, y, image_index, area=None):
        self._blit(OP_BLIT_IMAGE_D, [x, y], image_index, area)

    def blit_scaled_image_i(self, x, y, w, h, image_index, area=None):
        self._blit(OP_BLIT_SCALED_IMAGE_I, [int(x), int(y), int(w), int(h)], image_index, area)

    def blit_scaled_image_d(self, x, y, w, h, image_index, area=None):
        self._blit(OP_BLIT_SCALED_IMAGE_D, [x, y, w, h], image_index, area)

    # -- masked fills (A8 masks travel in the record) -----------------------------------------------
    def _mask(self, op, x, y, mask: np.ndarray, area):
        mask = np.ascontiguousarray(mask, dtype=np.uint8)
        h, w = mask.shape
        ar = list(area) if area is not None else [0, 0, 0, 0]
        self._rec(op, struct.pack("<2dIIII4i", float(x), float(y), w, h, 1 if area is not None else 0, 0, *ar)
                  + mask.tobytes())
        self.fill_count += 1

    def fill_mask_i(self, x, y, mask, area=None):
        self._mask(OP_FILL_MASK_I, int(x), int(y), mask, area)

    def fill_mask_d(self, x, y, mask, area=None):
        self._mask(OP_FILL_MASK_D, x, y, mask, area)

    # -- shapes (circle, ellipse, round rect, triangle through their paths) -------------------------
    def fill_geometry(self, gtype: int, values):
        v = [float(x) for x in values] + [0.0] * (6 - len(values))
        self._rec(OP_FILL_GEOMETRY, struct.pack("<II6d", gtype, 0, *v))
        self.fill_count += 1

    def stroke_geometry(self, gtype: int, values):
        v = [float(x) for x in values] + [0.0] * (6 - len(values))
        self._rec(OP_STROKE_GEOMETRY, struct.pack("<II6d", gtype, 0, *v))
        self.fill_count += 1

    def save(self):
        self._rec(OP_SAVE)

    def restore(self):
        self._rec(OP_RESTORE)

    # -- output ---------------------------------------------------------------------------------
    def to_bytes(self) -> bytes:
        fmt = 0 if self.format == FORMAT_PRGB32 else self.format     # PRGB32 streams keep their old bytes
        out = [struct.pack("<6I", MAGIC, VERSION, self.width, self.height, len(self.images), fmt)]
        # images assigned to .images directly (without add_image) are PRGB32
        formats = self.image_formats + [FORMAT_PRGB32] * (len(self.images) - len(self.image_formats))
        for img, ifmt in zip(self.images, formats):
            h, w = img.shape
            raw = img.astype("<u4").tobytes()
            out.append(struct.pack("<IHH", w, h, 0 if ifmt == FORMAT_PRGB32 else ifmt) + raw + b"\0" * ((-len(raw)) % 8))
        out.extend(self.parts)
        out.append(struct.pack("<II", OP_END, 0))
        return b"".join(out)


# ------------------------------------------------------------------------------------------------
# Random helpers
# ------------------------------------------------------------------------------------------------

# Transcendental functions evaluated with IEEE +, -, *, / only (no libm, no SIMD math kernels),
# so a seed serializes to the same stream bytes on every platform (x86-64 and aarch64 libm and
# numpy's vectorized exp/log/sin/cos differ in the last bits). Accuracy is ~1e-15 relative, which
# is all a scene generator needs; determinism is what matters.
_LN2_HI = 6.93147180369123816490e-01
_LN2_LO = 1.90821492927058770002e-10
_TWO_PI = 6.283185307179586


def _exp(x):
    x = np.asarray(x, dtype=np.float64)
    k = np.floor(x / 0.6931471805599453 + 0.5)
    r = (x - k * _LN2_HI) - k * _LN2_LO
    term = np.ones_like(r)
    acc = np.ones_like(r)
    for i in range(1, 18):
        term = term * r / float(i)
        acc = acc + term
    return np.ldexp(acc, k.astype(np.int64))


def _log(x):
    x = np.asarray(x, dtype=np.float64)
    m, e = np.frexp(x)                      # x = m * 2^e, m in [0.5, 1)
    small = m < 0.7071067811865476
    m = np.where(small, m * 2.0, m)
    e = np.where(small, e - 1, e).astype(np.float64)
    z = (m - 1.0) / (m + 1.0)               # log(m) = 2 atanh(z), |z| < 0.172
    z2 = z * z
    acc = np.zeros_like(z)
    for k in range(25, 0, -2):
        acc = acc * z2 + 1.0 / float(k)
    return 2.0 * z * acc + e * _LN2_HI + e * _LN2_LO


def _sincos(x: float) -> tuple[float, float]:
    k = math.floor(x / _TWO_PI + 0.5)
    r = x - k * _TWO_PI                     # |r| <= pi (up to rounding)
    r2 = r * r
    s = 1.0                                 # sin r = r (1 - r^2/(2*3) (1 - r^2/(4*5) (1 - ...)))
    for k in range(15, 0, -1):
        s = 1.0 - s * r2 / float((2 * k) * (2 * k + 1))
    c = 1.0                                 # cos r = 1 - r^2/(1*2) (1 - r^2/(3*4) (1 - ...))
    for k in range(15, 0, -1):
        c = 1.0 - c * r2 / float((2 * k - 1) * (2 * k))
    return r * s, c


def _log_uniform(rng, lo, hi, size=None):
    return _exp(rng.uniform(float(_log(lo)), float(_log(hi)), size))


def _random_stops(rng, n):
    offs = np.sort(rng.uniform(0.0, 1.0, n))
    cols = rng.integers(0, 2**32, n, dtype=np.uint64)
    return [(float(o), int(c)) for o, c in zip(offs, cols)]


def premultiplied_noise(rng, w, h) -> np.ndarray:
    """Uniform random premultiplied PRGB32 pixels: a ~ U8, each colour channel ~ U[0, a]."""
    a = rng.integers(0, 256, (h, w), dtype=np.uint32)
    ch = [(rng.random((h, w)) * (a + 1)).astype(np.uint32).clip(0, 255) for _ in range(3)]
    ch = [np.minimum(c, a) for c in ch]
    return (a << 24) | (ch[0] << 16) | (ch[1] << 8) | ch[2]


def _cubic_path(rng, x0, y0, side, nseg):
    """Closed path of `nseg` cubic segments with control points uniform in the bbox."""
    pts = rng.uniform(0.0, side, (3 * nseg, 2)) + np.array([x0, y0])
    start = pts[-1].copy()
    cmds = [P_MOVE]
    xy = [start]
    for i in range(nseg):
        c = pts[3 * i: 3 * i + 3]
        if i == nseg - 1:
            c = c.copy()
            c[2] = start
        cmds += [P_CUBIC, P_CUBIC, P_CUBIC]
        xy += [c[0], c[1], c[2]]
    cmds.append(P_CLOSE)
    xy.append(start)
    return cmds, np.array(xy)


def _gradient_style(rng, sw: StreamWriter, x0, y0, side, kind=None):
    kind = int(rng.integers(0, 3)) if kind is None else kind
    stops = _random_stops(rng, int(rng.integers(2, 9)))
    extend = int(rng.integers(0, 3))
    if kind == LINEAR:
        p = rng.uniform(0, side, 4) + np.array([x0, y0, x0, y0])
        sw.gradient(LINEAR, p.tolist(), extend, stops)
    elif kind == RADIAL:
        c = rng.uniform(0, side, 2) + np.array([x0, y0])
        f = rng.uniform(0, side, 2) + np.array([x0, y0])
        sw.gradient(RADIAL, [c[0], c[1], f[0], f[1], side * 0.5, 0.0], extend, stops)
    else:
        c = rng.uniform(0, side, 2) + np.array([x0, y0])
        sw.gradient(CONIC, [c[0], c[1], float(rng.uniform(0, 2 * math.pi)), 1.0], extend, stops)


# ------------------------------------------------------------------------------------------------
# Benchmark workloads
# ------------------------------------------------------------------------------------------------

def polygons(seed: int = 1, width: int = 512, height: int = 512, count: int = 2000, box: float = 64.0) -> StreamWriter:
    """Opaque-black canvas, `count` random 10-vertex polygons in box x box squares, solid
    random ARGB32 colours (premultiplied by the context), NonZero, SrcOver, identity transform."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sw = StreamWriter(width, height)
    sw.solid(0xFF000000)
    sw.fill_all()
    sw.fill_rule(NON_ZERO)
    sw.comp_op(SRC_OVER)
    org = rng.uniform(0.0, 1.0, (count, 2)) * np.array([width - box, height - box])
    verts = rng.uniform(0.0, box, (count, 10, 2)) + org[:, None, :]
    cols = rng.integers(0, 2**32, count, dtype=np.uint64)
    for i in range(count):
        sw.solid(int(cols[i]))
        sw.fill_polygon(verts[i])
    return sw


def curves(seed: int = 2, width: int = 1920, height: int = 1080, count: int = 20000,
           dither: bool = False) -> StreamWriter:
    """Closed cubic paths (4-12 segments, bbox side log-uniform 8-256 px, partly outside the
    canvas), NonZero/EvenOdd 50/50, linear/radial/conic gradients with 2-8 stops and
    pad/repeat/reflect extend, SrcOver. `dither`: gradient quality DITHER for every gradient."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sw = StreamWriter(width, height)
    sw.solid(0xFF000000)
    sw.fill_all()
    sw.comp_op(SRC_OVER)
    if dither:
        sw.hint(HINT_GRADIENT_QUALITY, GRADIENT_DITHER)
    for i in range(count):
        side = float(_log_uniform(rng, 8.0, 256.0))
        x0 = float(rng.uniform(-side * 0.5, width - side * 0.5))
        y0 = float(rng.uniform(-side * 0.5, height - side * 0.5))
        nseg = int(rng.integers(4, 13))
        cmds, xy = _cubic_path(rng, x0, y0, side, nseg)
        sw.fill_rule(int(rng.integers(0, 2)))
        _gradient_style(rng, sw, x0, y0, side, kind=i % 3)
        sw.fill_path(cmds, xy)
    return sw


def patterns(seed: int = 3, width: int = 4096, height: int = 4096, count: int = 50000,
             image_size: int = 256, image_count: int = 8) -> StreamWriter:
    """Affine pattern quads: image rect mapped by translate * rotate * scale about the image
    centre, filled as a 4-point polygon with BLPattern(image, PAD, T); NN/BI and SrcCopy/SrcOver
    50/50."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sw = StreamWriter(width, height)
    for _ in range(image_count):
        sw.add_image(premultiplied_noise(rng, image_size, image_size))
    sw.solid(0xFF000000)
    sw.fill_all()
    sw.fill_rule(NON_ZERO)
    half = image_size * 0.5
    corners = np.array([[0, 0], [image_size, 0], [image_size, image_size], [0, image_size]], dtype=np.float64)
    for _ in range(count):
        tx, ty = rng.uniform(0, width), rng.uniform(0, height)
        ang = rng.uniform(0, 2 * math.pi)
        s = float(_log_uniform(rng, 0.25, 4.0))
        sn, c = _sincos(ang)
        c, sn = c * s, sn * s
        # T = translate(tx, ty) * rotate(ang) * scale(s) * translate(-half, -half), row-vector form.
        m = [c, sn, -sn, c, tx - (c * half - sn * half), ty - (sn * half + c * half)]
        quad = np.stack([corners[:, 0] * m[0] + corners[:, 1] * m[2] + m[4],
                         corners[:, 0] * m[1] + corners[:, 1] * m[3] + m[5]], axis=1)
        sw.hint(HINT_PATTERN_QUALITY, int(rng.integers(0, 2)))
        sw.comp_op(int(rng.integers(0, 2)))
        sw.pattern(int(rng.integers(0, image_count)), PAD, transform=m)
        sw.fill_polygon(quad)
    return sw


def _ragged_rows(parts, n: int) -> np.ndarray:
    """Row-wise concatenation of ragged parts: row i of the result is, for each (padded, lengths)
    part in order, the first lengths[i] words of padded[i]; rows follow each other."""
    lens = np.stack([l for _, l in parts], axis=1)
    row_tot = lens.sum(axis=1)
    row_start = np.cumsum(row_tot) - row_tot
    out = np.empty(int(row_tot.sum()), dtype=np.uint64)
    within = np.zeros(n, dtype=np.int64)
    for arr, l in parts:
        mask = np.arange(arr.shape[1])[None, :] < l[:, None]
        vals = arr[mask]
        first = np.cumsum(l) - l
        dest = np.repeat(row_start + within, l) + (np.arange(vals.size) - np.repeat(first, l))
        out[dest] = vals
        within += l
    return out


def _rec_word(op: int, payload_bytes) -> np.ndarray:
    """First word of a record: op code, payload size (little-endian <II)."""
    return np.uint64(op) | (np.asarray(payload_bytes, dtype=np.uint64) << np.uint64(32))


def _rgba64_words(c: np.ndarray) -> np.ndarray:
    """Vectorized rgba64_from_rgba32 on uint64 arrays of ARGB32 values."""
    out = np.zeros_like(c)
    for sh in (0, 8, 16, 24):
        out |= ((c >> np.uint64(sh)) & np.uint64(255)) * np.uint64(257) << np.uint64(2 * sh)
    return out


def _mixed_canvas(rng, w: int, h: int, n: int) -> StreamWriter:
    """Opaque-black canvas with `n` paths of the polygon kind (10-vertex polygon in the path's
    box, solid colour) or the curve kind (closed path of 4-12 cubics with control points in the
    box, linear/radial/conic gradient with 2-8 stops and pad/repeat/reflect extend), each with a
    random comp-op (SrcOver/SrcCopy) and fill rule; box side log-uniform 8-256 px (at most the
    canvas side), placed so that at least a quarter of the box lies on the canvas. The records are
    laid out with whole-array operations (a canvas of 5,000 paths takes milliseconds)."""
    u64 = np.uint64
    side = np.minimum(_log_uniform(rng, 8.0, 256.0, n), float(max(w, h)))
    x0 = rng.uniform(-side * 0.25, np.maximum(w - side * 0.75, 1.0))
    y0 = rng.uniform(-side * 0.25, np.maximum(h - side * 0.75, 1.0))
    comp = rng.integers(0, 2, n).astype(u64)
    rule = rng.integers(0, 2, n).astype(u64)
    curve = rng.integers(0, 2, n).astype(bool)
    org = np.stack([x0, y0], axis=1)
    # per-kind draws: solid colours and polygon vertices for the polygon rows, gradients and
    # cubic control points for the curve rows
    ip, ic = np.flatnonzero(~curve), np.flatnonzero(curve)
    npoly, nc = ip.size, ic.size
    color = np.zeros(n, dtype=u64)
    color[ip] = rng.integers(0, 2**32, npoly, dtype=u64)
    xy = np.zeros((n, 38, 2))
    xy[ip, :10] = rng.uniform(0.0, 1.0, (npoly, 10, 2)) * side[ip, None, None] + org[ip, None, :]
    gkind = np.zeros(n, dtype=np.int64)
    nst = np.zeros(n, dtype=np.int64)
    ext = np.zeros(n, dtype=u64)
    gkind[ic] = rng.integers(0, 3, nc)
    nst[ic] = rng.integers(2, 9, nc)
    ext[ic] = rng.integers(0, 3, nc).astype(u64)
    offs = np.full((n, 8), 2.0)
    offs[ic] = rng.uniform(0.0, 1.0, (nc, 8))
    offs = np.sort(np.where(np.arange(8)[None, :] < nst[:, None], offs, 2.0), axis=1)
    scol = np.zeros((n, 8), dtype=u64)
    scol[ic] = _rgba64_words(rng.integers(0, 2**32, (nc, 8), dtype=u64))
    gp = np.zeros((n, 4))
    gp[ic] = rng.uniform(0.0, 1.0, (nc, 4)) * side[ic, None] + np.stack([x0[ic], y0[ic], x0[ic], y0[ic]], axis=1)
    angle = np.zeros(n)
    angle[ic] = rng.uniform(0.0, 2 * math.pi, nc)
    nseg = np.full(n, 4, dtype=np.int64)
    nseg[ic] = rng.integers(4, 13, nc)
    ctrl = rng.uniform(0.0, 1.0, (nc, 36, 2)) * side[ic, None, None] + org[ic, None, :]

    # comp-op and fill-rule records (4 words)
    pre = np.empty((n, 4), dtype=u64)
    pre[:, 0] = _rec_word(OP_SET_COMP_OP, 8)
    pre[:, 1] = comp
    pre[:, 2] = _rec_word(OP_SET_FILL_RULE, 8)
    pre[:, 3] = rule
    # style: solid colour (2 words) or gradient (15 + 2 * stops words)
    sty = np.zeros((n, 31), dtype=u64)
    sty_len = np.where(curve, 15 + 2 * nst, 2)
    sty[:, 0] = np.where(curve, _rec_word(OP_STYLE_GRADIENT, 112 + 16 * nst), _rec_word(OP_STYLE_RGBA32, 8))
    sty[:, 1] = np.where(curve, gkind.astype(u64) | (ext << u64(32)), color)
    sty[:, 2] = nst.astype(u64)                                   # stop count, no transform
    vals = np.zeros((n, 6))
    vals[:, 0:4] = gp                                             # linear: p0, p1; radial: c, f
    vals[:, 4] = np.where(gkind == RADIAL, side * 0.5, 0.0)       # radial r0 (r1 = 0)
    con = gkind == CONIC
    vals[con, 2] = angle[con]                                     # conic: c, angle, repeat 1
    vals[con, 3] = 1.0
    sty[:, 3:9] = vals.view(u64)
    sty[:, 9:15] = np.array([1.0, 0.0, 0.0, 1.0, 0.0, 0.0]).view(u64)[None, :]
    sty[:, 15:31:2] = offs.view(u64)
    sty[:, 16:31:2] = scol
    # geometry: polygon (2 + 20 words) or path (2 + command words + 2 * vertices)
    ncmd = 3 * nseg + 2
    cw = (ncmd + 7) // 8
    geo = np.empty((n, 2), dtype=u64)
    geo[:, 0] = np.where(curve, _rec_word(OP_FILL_PATH_D, 8 + 8 * cw + 16 * ncmd), _rec_word(OP_FILL_POLYGON_D, 168))
    geo[:, 1] = np.where(curve, ncmd, 10).astype(u64)
    cmd_bytes = np.zeros((n, 40), dtype=np.uint8)
    cmd_bytes[:, 0] = P_MOVE
    cmd_bytes[:, 1:37] = P_CUBIC
    rows = np.arange(n)
    cmd_bytes[rows, 1 + 3 * nseg] = P_CLOSE
    cmd_bytes[np.arange(40)[None, :] > (1 + 3 * nseg)[:, None]] = 0
    cmd_words = cmd_bytes.view(u64)
    start = ctrl[np.arange(nc), 3 * nseg[ic] - 1]
    xy[ic, 0] = start
    xy[ic, 1:37] = ctrl
    xy[ic, 1 + 3 * nseg[ic]] = start
    xy_words = xy.reshape(n, 76).view(u64)
    body = _ragged_rows([(pre, np.full(n, 4)), (sty, sty_len), (geo, np.full(n, 2)),
                         (cmd_words, np.where(curve, cw, 0)), (xy_words, np.where(curve, 2 * ncmd, 20))], n)
    sw = StreamWriter(w, h)
    sw.solid(0xFF000000)
    sw.fill_all()
    sw.parts.append(body.astype("<u8").tobytes())
    sw.fill_count += n
    return sw


def batch_canvas_specs(seed: int = 4, count: int = 4096, min_side: int = 32, max_side: int = 2048,
                       min_paths: int = 10, max_paths: int = 5000, scale: float = 1.0):
    """(width, height, paths) of every canvas of the batched workload: width and height
    log-uniform in [min_side, max_side], path count log-uniform in [min_paths, max_paths] (times
    `scale`, at least 1)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    w = _log_uniform(rng, min_side, max_side, count).astype(np.int64)
    h = _log_uniform(rng, min_side, max_side, count).astype(np.int64)
    n = np.maximum(1, (_log_uniform(rng, min_paths, max_paths, count) * scale).astype(np.int64))
    return [(int(a), int(b), int(c)) for a, b, c in zip(w, h, n)]


def batch_canvas(index: int, seed: int = 4, count: int = 4096, **kw) -> StreamWriter:
    """Canvas `index` of batch_canvases(seed, count, **kw), generated on its own: each canvas
    draws from its own generator, seeded with (seed, index)."""
    w, h, n = batch_canvas_specs(seed, count, **kw)[index]
    return _mixed_canvas(np.random.Generator(np.random.PCG64([seed, index])), w, h, n)


def batch_canvases(seed: int = 4, count: int = 4096, min_side: int = 32, max_side: int = 2048,
                   min_paths: int = 10, max_paths: int = 5000, scale: float = 1.0):
    """Independent canvases for the batched renderer: width and height log-uniform in
    [min_side, max_side], log-uniform path counts, each path of the polygon or cubic kind with a
    mixed style (solid or gradient) and comp-op. `scale` shrinks path counts for quick runs."""
    specs = batch_canvas_specs(seed, count, min_side, max_side, min_paths, max_paths, scale)
    return [_mixed_canvas(np.random.Generator(np.random.PCG64([seed, i])), w, h, n)
            for i, (w, h, n) in enumerate(specs)]


def serving_request_specs(seed: int = 5, count: int = 48, min_side: int = 64, max_side: int = 4096,
                          min_paths: int = 1, max_paths: int = 20000, scale: float = 1.0):
    """(side, paths) of every request of serving_requests(seed, count, ...)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sides = _log_uniform(rng, min_side, max_side, count).astype(np.int64)
    n = np.maximum(1, (_log_uniform(rng, min_paths, max_paths, count) * scale).astype(np.int64))
    return [(int(s), int(k)) for s, k in zip(sides, n)]


def serving_request(index: int, seed: int = 5, count: int = 48, **kw) -> StreamWriter:
    """Request `index` of serving_requests(seed, count, **kw), generated on its own."""
    s, k = serving_request_specs(seed, count, **kw)[index]
    return _mixed_canvas(np.random.Generator(np.random.PCG64([seed, index])), s, s, k)


def serving_requests(seed: int = 5, count: int = 48, min_side: int = 64, max_side: int = 4096,
                     min_paths: int = 1, max_paths: int = 20000, scale: float = 1.0):
    """Render requests for the serving loop: square canvases with side log-uniform in
    [min_side, max_side] and log-uniform path counts in [min_paths, max_paths] (times `scale`),
    paths of the polygon and curve kinds with mixed styles."""
    specs = serving_request_specs(seed, count, min_side, max_side, min_paths, max_paths, scale)
    return [_mixed_canvas(np.random.Generator(np.random.PCG64([seed, i])), s, s, k)
            for i, (s, k) in enumerate(specs)]


# ------------------------------------------------------------------------------------------------
# Differential-test scenes
# ------------------------------------------------------------------------------------------------

def random_mix(seed: int, width: int = 257, height: int = 257, count: int = 200,
               styles=("solid", "linear", "radial", "conic", "pattern_nn", "pattern_bi"),
               commands=("rect_i", "rect_d", "box_d", "polygon", "path_quad", "path_cubic"),
               transforms: bool = True, alphas: bool = True, dither: bool = False,
               format: int = FORMAT_PRGB32, xrgb_images: bool = False) -> StreamWriter:
    """Mixed commands/styles/comp-ops over a canvas slightly larger than the shapes' range
    (coordinates span -30 .. size+30 like the reference tester, so clipping is exercised).
    `dither`: each gradient is set with gradient quality DITHER (2 in 3) or NEAREST.
    `format`: the target's pixel format; `xrgb_images`: the first and third pattern images are
    XRGB32 (the random draws are the same either way)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sw = StreamWriter(width, height, format)
    for k in range(3):
        sw.add_image(premultiplied_noise(rng, int(rng.integers(5, 80)), int(rng.integers(5, 80))),
                     FORMAT_XRGB32 if xrgb_images and k != 1 else FORMAT_PRGB32)
    sw.clear_all()
    lo_x, hi_x, lo_y, hi_y = -30.0, width + 30.0, -30.0, height + 30.0

    def pt(n):
        return np.stack([rng.uniform(lo_x, hi_x, n), rng.uniform(lo_y, hi_y, n)], axis=1)

    for i in range(count):
        sw.comp_op(int(rng.integers(0, 2)))
        sw.fill_rule(int(rng.integers(0, 2)))
        if alphas:
            r = rng.integers(0, 4)
            sw.fill_alpha(1.0 if r < 2 else (0.0 if r == 2 else float(rng.uniform())))
        if transforms and rng.integers(0, 4) == 0:
            a = rng.uniform(-0.5, 0.5)
            s = rng.uniform(0.7, 1.3)
            cx, cy = width * 0.5, height * 0.5
            sn, c = _sincos(a)
            c, sn = c * s, sn * s
            sw.transform([c, sn, -sn, c, cx - (c * cx - sn * cy), cy - (sn * cx + c * cy)])
        elif transforms:
            sw.reset_transform()

        style = styles[int(rng.integers(0, len(styles)))]
        if style == "solid":
            sw.solid(int(rng.integers(0, 2**32, dtype=np.uint64)))
        elif style in ("linear", "radial", "conic"):
            if dither:
                sw.hint(HINT_GRADIENT_QUALITY, GRADIENT_DITHER if rng.integers(0, 3) else GRADIENT_NEAREST)
            side = float(rng.uniform(20, max(20, width, height)))
            x0, y0 = float(rng.uniform(lo_x, max(lo_x, hi_x - side))), float(rng.uniform(lo_y, max(lo_y, hi_y - side)))
            _gradient_style(rng, sw, x0, y0, side, kind={"linear": LINEAR, "radial": RADIAL, "conic": CONIC}[style])
        else:
            sw.hint(HINT_PATTERN_QUALITY, NEAREST if style == "pattern_nn" else BILINEAR)
            idx = int(rng.integers(0, len(sw.images)))
            ang = rng.uniform(0, 2 * math.pi) if rng.integers(0, 2) else 0.0
            s = float(_log_uniform(rng, 0.3, 3.0))
            sn, c = _sincos(ang)
            c, sn = c * s, sn * s
            tx, ty = rng.uniform(lo_x, hi_x), rng.uniform(lo_y, hi_y)
            sw.pattern(idx, int(rng.integers(0, 3)), transform=[c, sn, -sn, c, tx, ty])

        cmd = commands[int(rng.integers(0, len(commands)))]
        if cmd == "rect_i":
            x, y = rng.integers(-30, width + 30), rng.integers(-30, height + 30)
            sw.fill_rect_i(x, y, rng.integers(1, max(2, width // 2)), rng.integers(1, max(2, height // 2)))
        elif cmd == "rect_d":
            x, y = rng.uniform(lo_x, hi_x), rng.uniform(lo_y, hi_y)
            sw.fill_rect_d(x, y, rng.uniform(0.5, width * 0.5), rng.uniform(0.5, height * 0.5))
        elif cmd == "box_d":
            a, b = pt(2)
            sw.fill_box_d(min(a[0], b[0]), min(a[1], b[1]), max(a[0], b[0]), max(a[1], b[1]))
        elif cmd == "polygon":
            sw.fill_polygon(pt(int(rng.integers(3, 11))))
        elif cmd == "path_quad":
            n = int(rng.integers(1, 6))
            p = pt(2 * n + 1)
            sw.fill_path([P_MOVE] + [P_QUAD, P_QUAD] * n, p)
        else:
            n = int(rng.integers(1, 5))
            p = pt(3 * n + 1)
            sw.fill_path([P_MOVE] + [P_CUBIC, P_CUBIC, P_CUBIC] * n + [P_CLOSE], np.vstack([p, p[:1]]))
    return sw


def conic_paths(seed: int = 8, width: int = 300, height: int = 200, count: int = 120) -> StreamWriter:
    """Closed paths of conic segments as BLPath stores them (CONIC p1, WEIGHT (w, NaN), ON p2),
    partly outside the canvas, solid and gradient styles, both fill rules, with transforms."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sw = StreamWriter(width, height)
    sw.solid(0xFF000000)
    sw.fill_all()
    for i in range(count):
        sw.fill_rule(int(rng.integers(0, 2)))
        sw.comp_op(int(rng.integers(0, 2)))
        side = float(_log_uniform(rng, 10.0, 160.0))
        x0 = float(rng.uniform(-side * 0.3, width - side * 0.7))
        y0 = float(rng.uniform(-side * 0.3, height - side * 0.7))
        if i % 3:
            sw.solid(int(rng.integers(0, 2**32, dtype=np.uint64)))
        else:
            _gradient_style(rng, sw, x0, y0, side)
        if i % 5 == 0:
            a = float(rng.uniform(-0.4, 0.4))
            sn, c = _sincos(a)
            sw.transform([c, sn, -sn, c, 20.0, -10.0])
        elif i % 5 == 1:
            sw.reset_transform()
        n = int(rng.integers(2, 6))
        pts = rng.uniform(0, side, (2 * n + 1, 2)) + np.array([x0, y0])
        cmds, xy = [P_MOVE], [pts[0]]
        for k in range(n):
            w = float(_log_uniform(rng, 0.25, 4.0))
            cmds += [P_CONIC, 6, P_ON]
            xy += [pts[2 * k + 1], np.array([w, np.nan]), pts[2 * k + 2]]
        cmds.append(P_CLOSE)
        xy.append(pts[0])
        sw.fill_path(cmds, np.array(xy))
    return sw


def _stroke_figure(rng, x0, y0, side, closed: bool, curves: bool):
    """One figure for stroking: lines, quads and cubics with control points in the bbox, some
    points repeated or collinear (the stroker's degenerate branches)."""
    n = int(rng.integers(1, 7))
    pts = lambda k: rng.uniform(0.0, side, (k, 2)) + np.array([x0, y0])
    p0 = pts(1)[0]
    cmds, xy = [P_MOVE], [p0]
    cur = p0
    for _ in range(n):
        kind = int(rng.integers(0, 3)) if curves else 0
        r = float(rng.random())
        if kind == 0:
            q = pts(1)[0]
            if r < 0.08:
                q = cur.copy()                                     # zero-length line
            elif r < 0.16:
                q = cur + (cur - xy[-2] if len(xy) > 1 else np.array([3.0, 0.0]))   # collinear
            cmds.append(P_ON); xy.append(q); cur = q
        elif kind == 1:
            c, q = pts(2)
            if r < 0.15:
                c = cur + (q - cur) * float(rng.uniform(-0.5, 1.5))       # collinear (cusp when outside)
            cmds += [P_QUAD, P_ON]; xy += [c, q]; cur = q
        else:
            c1, c2, q = pts(3)
            if r < 0.1:
                t = rng.uniform(-0.5, 1.5, 2)
                c1, c2 = cur + (q - cur) * t[0], cur + (q - cur) * t[1]   # flat cubic
            elif r < 0.2:
                c1, c2 = c2.copy(), c1.copy()
                c2 = c1.copy()                                     # cusp-prone: equal controls
            cmds += [P_CUBIC, P_CUBIC, P_ON]; xy += [c1, c2, q]; cur = q
    if closed:
        cmds.append(P_CLOSE); xy.append(np.array([np.nan, np.nan]))
    return cmds, xy


def strokes(seed: int = 9, width: int = 640, height: int = 480, count: int = 400, curves: bool = True,
            max_width: float = 24.0) -> StreamWriter:
    """Stroked geometry: open and closed paths (lines, quads, cubics, degenerate segments),
    polylines, polygons, boxes, rects and lines, with every join, both caps drawn from all six,
    miter limits 1-10, widths log-uniform 0.5..max_width, solid/gradient/pattern stroke styles,
    stroke alpha, SrcOver/SrcCopy, rotated and scaled transforms in both transform orders."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sw = StreamWriter(width, height)
    sw.solid(0xFF101010)
    sw.fill_all()
    sw.add_image(premultiplied_noise(rng, 64, 48))
    for i in range(count):
        side = float(_log_uniform(rng, 8.0, 200.0))
        x0 = float(rng.uniform(-side * 0.3, max(-side * 0.3, width - side * 0.7)))
        y0 = float(rng.uniform(-side * 0.3, max(-side * 0.3, height - side * 0.7)))
        sw.stroke_width(float(_log_uniform(rng, 0.5, max_width)))
        sw.stroke_join(int(rng.integers(0, 5)))
        sw.stroke_caps(int(rng.integers(0, 6)), int(rng.integers(0, 6)))
        sw.stroke_miter_limit(float(rng.uniform(1.0, 10.0)))
        sw.comp_op(SRC_COPY if rng.random() < 0.15 else SRC_OVER)
        r = float(rng.random())
        if r < 0.6:
            sw.stroke_solid(int(rng.integers(0, 2**32, dtype=np.uint64)) | (0xFF000000 if rng.random() < 0.5 else 0))
        elif r < 0.85:
            kind = int(rng.integers(0, 3))
            stops = _random_stops(rng, int(rng.integers(2, 6)))
            if kind == LINEAR:
                p = rng.uniform(0, side, 4) + np.array([x0, y0, x0, y0])
                sw.stroke_gradient(LINEAR, p.tolist(), int(rng.integers(0, 3)), stops)
            elif kind == RADIAL:
                c = rng.uniform(0, side, 2) + np.array([x0, y0])
                sw.stroke_gradient(RADIAL, [c[0], c[1], c[0], c[1], side * 0.5, 0.0], int(rng.integers(0, 3)), stops)
            else:
                c = rng.uniform(0, side, 2) + np.array([x0, y0])
                sw.stroke_gradient(CONIC, [c[0], c[1], float(rng.uniform(0, 2 * math.pi)), 1.0], 0, stops)
        else:
            sw.hint(HINT_PATTERN_QUALITY, int(rng.integers(0, 2)))
            sw.stroke_pattern(0, int(rng.integers(0, 3)), transform=[1.0, 0.0, 0.0, 1.0, x0, y0])
        if rng.random() < 0.1:
            sw.stroke_alpha(float(rng.uniform(0.2, 1.0)))
        elif rng.random() < 0.1:
            sw.stroke_alpha(1.0)
        t = float(rng.random())
        if t < 0.2:
            a = float(rng.uniform(-0.6, 0.6))
            sc = float(_log_uniform(rng, 0.5, 2.0))
            sn, c = _sincos(a)
            sw.transform([c * sc, sn * sc, -sn * sc * 0.8, c * sc * 0.8, 15.0, -7.5])
            sw.stroke_transform_order(int(rng.integers(0, 2)))
        elif t < 0.3:
            sw.transform([1.5, 0.0, 0.0, 0.75, -10.0, 20.0])
        elif t < 0.5:
            sw.reset_transform()
        g = float(rng.random())
        if g < 0.45:
            cmds, xy = [], []
            for f in range(int(rng.integers(1, 3))):
                fc, fxy = _stroke_figure(rng, x0, y0, side, closed=rng.random() < 0.4, curves=curves)
                cmds += fc; xy += fxy
            sw.stroke_path(cmds, np.array(xy))
        elif g < 0.65:
            k = int(rng.integers(2, 10))
            sw.stroke_polyline(rng.uniform(0, side, (k, 2)) + np.array([x0, y0]))
        elif g < 0.8:
            k = int(rng.integers(3, 10))
            sw.stroke_polygon(rng.uniform(0, side, (k, 2)) + np.array([x0, y0]))
        elif g < 0.88:
            sw.stroke_box_d(x0, y0, x0 + side * float(rng.random()), y0 + side * float(rng.random()))
        elif g < 0.94:
            sw.stroke_rect_d(x0, y0, side * float(rng.random()), side * float(rng.random()))
        else:
            p = rng.uniform(0, side, 4) + np.array([x0, y0, x0, y0])
            sw.stroke_line_d(*p.tolist())
    return sw


def blits(seed: int = 40, width: int = 320, height: int = 240, count: int = 150,
          format: int = FORMAT_PRGB32, xrgb_images: bool = False) -> StreamWriter:
    """Image blits: integer and fractional origins, scaled rectangles, image areas (some outside the
    image, which the reference rejects), partly clipped, with translations, rotations and scales,
    nearest and bilinear quality, SrcOver/SrcCopy and global alpha. `format` and `xrgb_images`
    as in random_mix."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sw = StreamWriter(width, height, format)
    sw.solid(0xFF303030)
    sw.fill_all()
    for k in range(3):
        sw.add_image(premultiplied_noise(rng, int(rng.integers(1, 90)), int(rng.integers(1, 70))),
                     FORMAT_XRGB32 if xrgb_images and k != 1 else FORMAT_PRGB32)
    sizes = [im.shape for im in sw.images]
    for i in range(count):
        idx = int(rng.integers(0, len(sizes)))
        ih, iw = sizes[idx]
        area = None
        if rng.random() < 0.4:
            ax, ay = int(rng.integers(0, iw)), int(rng.integers(0, ih))
            # non-empty: the reference divides by the area's size in its pattern set-up
            area = [ax, ay, int(rng.integers(1, iw - ax + 1)), int(rng.integers(1, ih - ay + 1))]
            if rng.random() < 0.1:
                area[2] += 1                                   # outside the image: rejected
        sw.comp_op(SRC_COPY if rng.random() < 0.2 else SRC_OVER)
        sw.hint(HINT_PATTERN_QUALITY, int(rng.integers(0, 2)))
        if rng.random() < 0.15:
            sw.global_alpha(float(rng.uniform(0.1, 1.0)))
        elif rng.random() < 0.15:
            sw.global_alpha(1.0)
        t = float(rng.random())
        if t < 0.15:
            a = float(rng.uniform(-0.7, 0.7))
            sn, c = _sincos(a)
            sc = float(_log_uniform(rng, 0.5, 2.0))
            sw.transform([c * sc, sn * sc, -sn * sc, c * sc, float(rng.uniform(-20, 40)), float(rng.uniform(-20, 40))])
        elif t < 0.3:
            sw.transform([1.0, 0.0, 0.0, 1.0, float(rng.integers(-30, 30)), float(rng.integers(-30, 30))])
        elif t < 0.4:
            sw.transform([1.0, 0.0, 0.0, 1.0, float(rng.uniform(-30, 30)), float(rng.uniform(-30, 30))])
        elif t < 0.5:
            sw.transform([1.5, 0.0, 0.0, 0.75, 5.0, -3.0])
        elif t < 0.7:
            sw.reset_transform()
        x, y = float(rng.uniform(-60, width)), float(rng.uniform(-60, height))
        k = float(rng.random())
        if k < 0.35:
            sw.blit_image_i(int(x), int(y), idx, area)
        elif k < 0.65:
            sw.blit_image_d(x if rng.random() < 0.7 else float(int(x)), y, idx, area)
        elif k < 0.85:
            sw.blit_scaled_image_d(x, y, float(rng.uniform(1, 200)), float(rng.uniform(1, 150)), idx, area)
        else:
            sw.blit_scaled_image_i(int(x), int(y), int(rng.integers(1, 200)), int(rng.integers(1, 150)), idx, area)
    return sw


def masks(seed: int = 50, width: int = 300, height: int = 220, count: int = 120) -> StreamWriter:
    """Masked fills: A8 masks (noise, gradients, binary), integer and pixel-aligned double origins,
    mask areas, clipping, translations (fractional ones and rotations: not supported by the
    reference's masked fill, which draws nothing there), solid / gradient / pattern fill styles,
    fill and global alpha, SrcOver/SrcCopy."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sw = StreamWriter(width, height)
    sw.solid(0xFF202020)
    sw.fill_all()
    sw.add_image(premultiplied_noise(rng, 40, 30))
    for i in range(count):
        mw, mh = int(rng.integers(1, 90)), int(rng.integers(1, 70))
        kind = int(rng.integers(0, 3))
        if kind == 0:
            mask = rng.integers(0, 256, (mh, mw), dtype=np.uint8)
        elif kind == 1:
            mask = (np.add.outer(np.arange(mh) * 3, np.arange(mw) * 2) % 256).astype(np.uint8)
        else:
            mask = (rng.random((mh, mw)) < 0.5).astype(np.uint8) * 255
        area = None
        if rng.random() < 0.3:
            ax, ay = int(rng.integers(0, mw)), int(rng.integers(0, mh))
            area = [ax, ay, int(rng.integers(1, mw - ax + 1)), int(rng.integers(1, mh - ay + 1))]
        r = float(rng.random())
        if r < 0.5:
            sw.solid(int(rng.integers(0, 2**32, dtype=np.uint64)))
        elif r < 0.8:
            _gradient_style(rng, sw, 0.0, 0.0, float(max(width, height)))
        else:
            sw.pattern(0, int(rng.integers(0, 3)), transform=[1.0, 0.0, 0.0, 1.0, float(rng.integers(0, 50)), 3.0])
        sw.comp_op(SRC_COPY if rng.random() < 0.2 else SRC_OVER)
        if rng.random() < 0.2:
            sw.fill_alpha(float(rng.uniform(0.1, 1.0)))
        elif rng.random() < 0.2:
            sw.fill_alpha(1.0)
        if rng.random() < 0.1:
            sw.global_alpha(float(rng.uniform(0.3, 1.0)))
        t = float(rng.random())
        if t < 0.15:
            sw.transform([1.0, 0.0, 0.0, 1.0, float(rng.integers(-20, 20)), float(rng.integers(-20, 20))])
        elif t < 0.2:
            sw.transform([1.0, 0.0, 0.0, 1.0, float(rng.uniform(-20, 20)), 2.5])
        elif t < 0.25:
            sw.transform([0.9, 0.3, -0.3, 0.9, 10.0, 5.0])
        elif t < 0.45:
            sw.reset_transform()
        x, y = int(rng.integers(-40, width)), int(rng.integers(-40, height))
        if rng.random() < 0.5:
            sw.fill_mask_i(x, y, mask, area)
        else:
            sw.fill_mask_d(float(x) + (0.5 if rng.random() < 0.15 else 0.0), float(y), mask, area)
    return sw


def shapes(seed: int = 60, width: int = 320, height: int = 240, count: int = 200) -> StreamWriter:
    """Circles (negative radii too), ellipses, round rectangles (radii clamped, degenerate ones as
    boxes), triangles and arcs / chords / pies (sweeps of either sign, full turns), filled with
    both fill rules and stroked with every join and cap, under identity, scale and rotation
    transforms."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sw = StreamWriter(width, height)
    sw.solid(0xFF000000)
    sw.fill_all()
    for i in range(count):
        cx, cy = float(rng.uniform(-20, width + 20)), float(rng.uniform(-20, height + 20))
        size = float(_log_uniform(rng, 2.0, 120.0))
        t = int(rng.integers(0, 5))
        if t == 4:
            sweep = float(rng.uniform(-7.0, 7.0))
            gt = (GEOMETRY_ARC, GEOMETRY_CHORD, GEOMETRY_PIE)[int(rng.integers(0, 3))]
            v = [cx, cy, size, float(rng.uniform(2.0, 90.0)), float(rng.uniform(-4.0, 4.0)), sweep]
        elif t == 0:
            gt, v = GEOMETRY_CIRCLE, [cx, cy, size * (1 if rng.random() < 0.9 else -1)]
        elif t == 1:
            gt, v = GEOMETRY_ELLIPSE, [cx, cy, size, float(rng.uniform(1.0, 80.0))]
        elif t == 2:
            w, h = size * 2, float(rng.uniform(2.0, 150.0))
            r = [float(rng.uniform(0.0, 40.0)), float(rng.uniform(-40.0, 40.0))]
            if rng.random() < 0.1:
                r = [0.0, 5.0]                                   # degenerate: a box
            gt, v = GEOMETRY_ROUND_RECT, [cx - w / 2, cy - h / 2, w, h] + r
        else:
            gt, v = GEOMETRY_TRIANGLE, list((rng.uniform(-size, size, 6) + np.array([cx, cy] * 3)).astype(float))
        if rng.random() < 0.25:
            a = float(rng.uniform(-0.8, 0.8))
            sn, c = _sincos(a)
            sw.transform([c, sn, -sn, c * 0.7, 10.0, -5.0])
        elif rng.random() < 0.3:
            sw.reset_transform()
        if rng.random() < 0.5:
            sw.fill_rule(int(rng.integers(0, 2)))
            sw.solid(int(rng.integers(0, 2**32, dtype=np.uint64)))
            sw.fill_geometry(gt, v)
        else:
            sw.stroke_width(float(_log_uniform(rng, 0.5, 20.0)))
            sw.stroke_join(int(rng.integers(0, 5)))
            sw.stroke_caps(int(rng.integers(0, 6)), int(rng.integers(0, 6)))
            sw.stroke_solid(int(rng.integers(0, 2**32, dtype=np.uint64)))
            sw.stroke_geometry(gt, v)
    return sw


def stroked_paths(seed: int = 10, width: int = 1920, height: int = 1080, count: int = 20000) -> StreamWriter:
    """Stroking benchmark: `count` open cubic paths (2-6 segments, bbox side log-uniform 8-256 px)
    stroked with widths log-uniform 1-16 px, round/miter/bevel joins and butt/square/round caps,
    solid colours, SrcOver, identity transform."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sw = StreamWriter(width, height)
    sw.solid(0xFF000000)
    sw.fill_all()
    for i in range(count):
        side = float(_log_uniform(rng, 8.0, 256.0))
        x0 = float(rng.uniform(-side * 0.5, width - side * 0.5))
        y0 = float(rng.uniform(-side * 0.5, height - side * 0.5))
        sw.stroke_width(float(_log_uniform(rng, 1.0, 16.0)))
        sw.stroke_join((JOIN_ROUND, JOIN_MITER_CLIP, JOIN_BEVEL)[i % 3])
        cap = (CAP_BUTT, CAP_SQUARE, CAP_ROUND)[(i // 3) % 3]
        sw.stroke_caps(cap, cap)
        sw.stroke_solid(int(rng.integers(0, 2**32, dtype=np.uint64)))
        nseg = int(rng.integers(2, 7))
        pts = rng.uniform(0.0, side, (3 * nseg + 1, 2)) + np.array([x0, y0])
        cmds = [P_MOVE] + [P_CUBIC, P_CUBIC, P_ON] * nseg
        sw.stroke_path(cmds, pts)
    return sw


WORKLOADS = {
    "polygons": polygons,
    "curves": curves,
    "patterns": patterns,
    "strokes": stroked_paths,
}


def edge_cases(seed: int = 7, width: int = 131, height: int = 97) -> StreamWriter:
    """Degenerate and boundary inputs the reference tolerates: empty and zero-area shapes,
    horizontal-only polygons, single points, shapes far outside the canvas, coordinates at the
    canvas border, huge coordinates that need clipping, NaN vertices (rejected as invalid
    geometry), zero alpha, fully transparent colours (DstCopy NOP), opaque colours (SrcOver ->
    SrcCopy), collinear curves, cusps, zero-length gradients and out-of-range stop offsets."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sw = StreamWriter(width, height)
    sw.add_image(premultiplied_noise(rng, 1, 1))
    sw.add_image(premultiplied_noise(rng, 7, 3))
    sw.solid(0xFF204060)
    sw.fill_all()
    W, H = float(width), float(height)
    polys = [
        np.array([[10, 10], [10, 10], [10, 10]]),                      # single point
        np.array([[5, 20], [60, 20], [30, 20]]),                        # horizontal only
        np.array([[0, 0], [W, 0], [W, H], [0, H]]),                     # exactly the canvas
        np.array([[-1e6, -1e6], [1e6, -1e6], [1e6, 1e6]]),              # huge, clipped
        np.array([[-50, 10], [-10, 80], [-30, 40]]),                    # left of the canvas
        np.array([[W + 5, 10], [W + 50, 80], [W + 9, 40]]),             # right of the canvas
        np.array([[10, -80], [60, -5], [30, -40]]),                     # above
        np.array([[10, H + 3], [60, H + 90], [30, H + 40]]),            # below
        np.array([[-20, -20], [W + 20, 30], [40, H + 20]]),             # crosses every edge
        np.array([[0.5, 0.5], [0.75, 0.5], [0.75, 0.75]]),              # sub-pixel
        np.array([[W - 0.25, 3], [W + 0.25, 30], [W - 0.1, 60]]),       # at the right border
        np.array([[1, 1], [40, 40], [80, 80], [120, 120]]),             # collinear
        np.array([[10, 10], [np.nan, 20], [30, 40]]),                   # NaN vertex
        np.array([[30, 5], [31, 90], [32, 5], [33, 90], [34, 5]]),      # thin spikes
    ]
    for i, pts in enumerate(polys):
        sw.fill_rule(i & 1)
        sw.comp_op(SRC_OVER if i % 3 else SRC_COPY)
        sw.solid(int(rng.integers(0, 2**32, dtype=np.uint64)))
        sw.fill_polygon(pts.astype(np.float64))
    # zero-alpha / transparent / opaque colours
    sw.comp_op(SRC_OVER)
    sw.solid(0x00000000); sw.fill_rect_d(5, 5, 50, 50)
    sw.solid(0x00FFFFFF); sw.fill_rect_d(5, 5, 50, 50)
    sw.solid(0xFF00FF00); sw.fill_rect_d(6.3, 7.7, 20.2, 0.4)
    sw.fill_alpha(0.0); sw.fill_rect_i(0, 0, width, height); sw.fill_alpha(1.0)
    sw.global_alpha(0.5); sw.solid(0x80FF0000); sw.fill_box_d(-3.5, -2.25, 40.125, 30.75); sw.global_alpha(1.0)
    # rect edge cases
    sw.comp_op(SRC_COPY)
    sw.solid(0xC0112233)
    sw.fill_rect_i(-10, -10, 5, 5)      # fully outside
    sw.fill_rect_i(10, 10, 0, 8)        # zero width
    sw.fill_rect_i(10, 10, -4, 8)       # negative width
    sw.fill_rect_d(20.5, 30.5, 1e-3, 1e-3)
    sw.fill_rect_d(W - 1.5, H - 1.5, 10, 10)
    sw.fill_box_d(70.1, 10.9, 71.0, 60.2)   # one pixel wide, fractional
    sw.fill_box_d(40.0, 60.0, 90.0, 61.0)   # aligned, one row
    # curves: cusp, collinear, all-equal, huge, crossing
    sw.comp_op(SRC_OVER)
    curves_list = [
        ([P_MOVE, P_CUBIC, P_CUBIC, P_CUBIC], [[10, 50], [90, 10], [10, 10], [90, 50]]),
        ([P_MOVE, P_CUBIC, P_CUBIC, P_CUBIC], [[10, 60], [40, 60], [70, 60], [100, 60]]),
        ([P_MOVE, P_CUBIC, P_CUBIC, P_CUBIC], [[20, 20], [20, 20], [20, 20], [20, 20]]),
        ([P_MOVE, P_CUBIC, P_CUBIC, P_CUBIC], [[-500, -500], [5000, 100], [-3000, 900], [600, -200]]),
        ([P_MOVE, P_QUAD, P_QUAD, P_QUAD, P_QUAD], [[0, 96], [65, -40], [130, 96], [65, 200], [0, 96]]),
        ([P_MOVE, P_ON, P_ON, P_CLOSE, P_MOVE, P_ON, P_ON, P_CLOSE], [[5, 5], [60, 30], [20, 80], [0, 0], [70, 5], [125, 30], [85, 80], [0, 0]]),
    ]
    for i, (cmds, xy) in enumerate(curves_list):
        sw.fill_rule(i & 1)
        _gradient_style(rng, sw, 0.0, 0.0, 120.0, kind=i % 3)
        sw.fill_path(cmds, np.array(xy, dtype=np.float64))
    # degenerate gradients
    sw.gradient(LINEAR, [30, 30, 30, 30], PAD, [(0.0, 0xFF0000FF), (1.0, 0xFFFF0000)])           # zero length
    sw.fill_rect_d(0, 0, 60, 40)
    sw.gradient(RADIAL, [50, 50, 50, 50, 0.0, 0.0], REFLECT, [(0.0, 0xFF00FF00), (1.0, 0x8000FFFF)])  # zero radius
    sw.fill_rect_d(30, 30, 60, 40)
    sw.gradient(LINEAR, [0, 0, 100, 0], REPEAT, [(0.5, 0xFF00FF00)])                              # single stop
    sw.fill_rect_d(10, 60, 100, 20)
    sw.gradient(LINEAR, [0, 0, 100, 0], PAD, [(0.0, 0x00000000), (1.0, 0x00000000)])              # all transparent
    sw.fill_rect_d(10, 60, 100, 20)
    sw.gradient(CONIC, [60, 45, 0.0, 1.0], PAD, [(0.0, 0xFF0000FF), (0.5, 0xFFFFFFFF), (0.5, 0xFF000000), (1.0, 0xFF00FF00)])
    sw.fill_rect_d(20, 10, 90, 80)
    # tiny patterns (1x1 and 7x3) with every extend mode and translation-only transforms
    for ext in (PAD, REPEAT, REFLECT):
        for q in (NEAREST, BILINEAR):
            sw.hint(HINT_PATTERN_QUALITY, q)
            sw.pattern(1, ext, transform=[1, 0, 0, 1, 3.0 * ext + 0.5 * q, 2.25 * q])
            sw.fill_rect_d(4 + 40 * ext, 4 + 40 * q, 37.5, 33.25)
    sw.pattern(0, REPEAT)
    sw.fill_rect_i(100, 70, 20, 20)
    sw.pattern(1, REFLECT, area=[2, 1, 4, 2])
    sw.fill_rect_i(60, 70, 30, 20)
    return sw
