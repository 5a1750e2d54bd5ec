"""ctypes access to the CPU oracle (oracle/, test infrastructure) and the golden fixtures.

Only tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""

from __future__ import annotations

import ctypes
import hashlib
import json
import os
import struct
import subprocess
import threading

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.json")

LUT_SSE2, LUT_AVX2, LUT_SCALAR = 0, 1, 2
LUT_VARIANTS = {"default": LUT_SSE2, "sse2": LUT_SSE2, "avx2": LUT_AVX2, "scalar": LUT_SCALAR}

_lock = threading.Lock()
_lib = None


class OracleOptions(ctypes.Structure):
    _fields_ = [("lut_variant", ctypes.c_uint32), ("band_height", ctypes.c_uint32), ("reserved", ctypes.c_uint32 * 6)]


class OracleStats(ctypes.Structure):
    _fields_ = [("fill_calls", ctypes.c_uint64), ("composited_pixels", ctypes.c_uint64),
                ("edge_points", ctypes.c_uint64), ("input_vertices", ctypes.c_uint64)]


def build():
    subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile")], check=True, cwd=ROOT)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            l = ctypes.CDLL(ORACLE_SO)
            l.b2d_oracle_render.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_void_p,
                                            ctypes.POINTER(OracleOptions), ctypes.POINTER(OracleStats)]
            l.b2d_oracle_render.restype = ctypes.c_int
            l.b2d_oracle_build_lut.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32]
            l.b2d_oracle_rasterize_line.argtypes = [ctypes.c_int] * 4 + [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
            l.b2d_oracle_rasterize_line.restype = ctypes.c_int
            _lib = l
        return _lib


FORMAT_PRGB32, FORMAT_XRGB32, FORMAT_A8 = 1, 2, 3


def stream_size(stream: bytes):
    w, h = struct.unpack_from("<II", stream, 8)
    return w, h


def stream_format(stream: bytes) -> int:
    """The target format of a stream (BLGPU_STREAM_FORMAT_*; 0 in the header reads as PRGB32)."""
    return struct.unpack_from("<I", stream, 20)[0] or FORMAT_PRGB32


def render(stream: bytes, lut: str = "default", band_height: int = 0, stats: bool = False):
    """Renders a command stream on the CPU oracle; returns (h, w) pixels, uint32 (uint8 for an A8
    target) [and stats]."""
    w, h = stream_size(stream)
    out = np.zeros((h, w), dtype=np.uint8 if stream_format(stream) == FORMAT_A8 else np.uint32)
    opt = OracleOptions(LUT_VARIANTS[lut], band_height)
    st = OracleStats()
    rc = lib().b2d_oracle_render(stream, len(stream), out.ctypes.data, ctypes.byref(opt), ctypes.byref(st))
    if rc != 0:
        raise RuntimeError(f"oracle render failed ({rc})")
    return (out, st) if stats else out


def build_lut(size: int, stops, variant: str = "default") -> np.ndarray:
    """stops: [(offset, rgba64)]"""
    raw = b"".join(struct.pack("<dQ", float(o), int(c)) for o, c in stops)
    out = np.zeros(size, dtype=np.uint32)
    lib().b2d_oracle_build_lut(out.ctypes.data, size, raw, len(stops), LUT_VARIANTS[variant])
    return out


def rasterize_line(w, rows, x0, y0, x1, y1, sign, band_height=16) -> np.ndarray:
    cells = np.zeros((rows, w + 2), dtype=np.uint32)
    lib().b2d_oracle_rasterize_line(x0, y0, x1, y1, sign, band_height, w, rows, cells.ctypes.data)
    return cells


def sha256(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def golden_stream(entry) -> bytes:
    """Re-evaluates a golden scene expression and checks the stream bytes are the recorded ones."""
    from blend2d_gb300 import scenes  # noqa: F401
    stream = eval(entry["expr"], {"scenes": scenes}).to_bytes()
    assert hashlib.sha256(stream).hexdigest() == entry["stream_sha256"], entry["name"]
    return stream


def golden_stops(entry):
    return [(float.fromhex(o), int(c, 16)) for o, c in entry["stops"]]
