"""blend2d_gb300 - a GB300 (sm_103a) raster backend for Blend2D's fill pipeline.

The product is `_build/libblgpu.so` (C ABI declared in include/blgpu.h). This module is a thin
ctypes mirror of that ABI with the reference's vocabulary (BLContext-like calls, BLResult codes).
There is no CPU fallback: if the library is missing, importing the bindings raises.
"""
from __future__ import annotations

import ctypes
import os
import struct
import threading
import weakref

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libblgpu.so")

# BLResult codes (blend2d/core/api.h)
SUCCESS = 0
ERROR_OUT_OF_MEMORY = 0x00010000
ERROR_INVALID_VALUE = 0x00010001
ERROR_INVALID_STATE = 0x00010002
ERROR_NOT_IMPLEMENTED = 0x00010007
ERROR_NO_STATES_TO_RESTORE = 0x00010038
ERROR_DATA_TOO_LARGE = 0x00010032
ERROR_INVALID_GEOMETRY = 0x00010034
ERROR_DEVICE = 0x00011000

FORMAT_PRGB32 = 1
FORMAT_XRGB32 = 2
FORMAT_A8 = 3
IMAGE_DEVICE_MEMORY = 1
FLUSH_SYNC = 0x80000000
FLUSH_ASYNC = 0x1            # start rendering what is recorded and return (see include/blgpu.h)
LUT_SSE2, LUT_AVX2, LUT_SCALAR = 0, 1, 2

COMP_OP_SRC_OVER, COMP_OP_SRC_COPY = 0, 1
FILL_RULE_NON_ZERO, FILL_RULE_EVEN_ODD = 0, 1
HINT_RENDERING_QUALITY, HINT_GRADIENT_QUALITY, HINT_PATTERN_QUALITY = 0, 1, 2
GRADIENT_LINEAR, GRADIENT_RADIAL, GRADIENT_CONIC = 0, 1, 2
EXTEND_PAD, EXTEND_REPEAT, EXTEND_REFLECT = 0, 1, 2
PATH_MOVE, PATH_ON, PATH_QUAD, PATH_CONIC, PATH_CUBIC, PATH_CLOSE = 0, 1, 2, 3, 4, 5


class BLGpuError(RuntimeError):
    def __init__(self, code: int, what: str = "", detail: str = ""):
        super().__init__(f"{what} failed with BLResult 0x{code:08x}{detail}")
        self.code = code


class RuntimeCreateInfo(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("lut_variant", ctypes.c_uint32), ("cuda_stream", ctypes.c_void_p),
                ("reserved", ctypes.c_uint32 * 4)]


class Image(ctypes.Structure):
    _fields_ = [("pixel_data", ctypes.c_void_p), ("stride", ctypes.c_ssize_t), ("width", ctypes.c_int32),
                ("height", ctypes.c_int32), ("format", ctypes.c_uint32), ("flags", ctypes.c_uint32)]


class GradientStop(ctypes.Structure):
    _fields_ = [("offset", ctypes.c_double), ("rgba64", ctypes.c_uint64)]


class Gradient(ctypes.Structure):
    _fields_ = [("type", ctypes.c_uint32), ("extend_mode", ctypes.c_uint32), ("values", ctypes.c_double * 6),
                ("stops", ctypes.POINTER(GradientStop)), ("stop_count", ctypes.c_size_t),
                ("transform", ctypes.POINTER(ctypes.c_double))]


class Pattern(ctypes.Structure):
    _fields_ = [("image", ctypes.POINTER(Image)), ("area", ctypes.c_int32 * 4), ("extend_mode", ctypes.c_uint32),
                ("transform", ctypes.POINTER(ctypes.c_double))]


class StrokeOptions(ctypes.Structure):
    _fields_ = [("width", ctypes.c_double), ("miter_limit", ctypes.c_double), ("join", ctypes.c_uint32),
                ("start_cap", ctypes.c_uint32), ("end_cap", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class MemoryInfo(ctypes.Structure):
    _fields_ = [("reserved_bytes", ctypes.c_uint64), ("last_frame_bytes", ctypes.c_uint64),
                ("reserved", ctypes.c_uint64 * 6)]


class LaunchConfig(ctypes.Structure):
    _fields_ = [("cover_slots", ctypes.c_int32), ("cover_blocks_per_sm", ctypes.c_int32),
                ("fine_blocks_per_sm", ctypes.c_int32), ("edge_block", ctypes.c_int32),
                ("cubic_blocks_per_sm", ctypes.c_int32), ("no_occlusion_cull", ctypes.c_int32),
                ("max_segments", ctypes.c_int32), ("graph_frames", ctypes.c_int32),
                ("list_rows", ctypes.c_int32), ("device_order", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class Stats(ctypes.Structure):
    _fields_ = [("frames", ctypes.c_uint64), ("fill_commands", ctypes.c_uint64), ("segments", ctypes.c_uint64),
                ("tiles", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64), ("last_gpu_ms", ctypes.c_double),
                ("last_fine_ms", ctypes.c_double), ("pixel_ops", ctypes.c_uint64), ("pattern_ops", ctypes.c_uint64),
                ("input_vertices", ctypes.c_uint64), ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
                ("last_cuda_error", ctypes.c_int64), ("last_composite_ms", ctypes.c_double),
                ("graph_frames", ctypes.c_uint64), ("last_record_ms", ctypes.c_double),
                ("last_merge_ms", ctypes.c_double), ("last_upload_ms", ctypes.c_double),
                ("last_run_ms", ctypes.c_double)]


_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_D = ctypes.c_double
_SIGNATURES = {
    "blgpu_runtime_create": [ctypes.POINTER(_P), ctypes.POINTER(RuntimeCreateInfo)],
    "blgpu_runtime_destroy": [_P],
    "blgpu_runtime_get_stats": [_P, ctypes.POINTER(Stats)],
    "blgpu_runtime_replay": [_P, ctypes.c_int],
    "blgpu_runtime_get_memory": [_P, ctypes.POINTER(MemoryInfo)],
    "blgpu_runtime_release_memory": [_P],
    "blgpu_runtime_synchronize": [_P],
    "blgpu_runtime_get_launch_config": [_P, ctypes.POINTER(LaunchConfig)],
    "blgpu_runtime_set_launch_config": [_P, ctypes.POINTER(LaunchConfig)],
    "blgpu_runtime_autotune": [_P, _U32, ctypes.POINTER(LaunchConfig), ctypes.POINTER(ctypes.c_double)],
    "blgpu_context_create": [ctypes.POINTER(_P), _P],
    "blgpu_context_destroy": [_P],
    "blgpu_context_begin": [_P, ctypes.POINTER(Image)],
    "blgpu_context_end": [_P],
    "blgpu_context_flush": [_P, _U32],
    "blgpu_context_save": [_P],
    "blgpu_context_restore": [_P],
    "blgpu_context_set_comp_op": [_P, _U32],
    "blgpu_context_set_fill_rule": [_P, _U32],
    "blgpu_context_set_global_alpha": [_P, _D],
    "blgpu_context_set_fill_alpha": [_P, _D],
    "blgpu_context_set_hint": [_P, _U32, _U32],
    "blgpu_context_set_transform": [_P, ctypes.POINTER(ctypes.c_double)],
    "blgpu_context_reset_transform": [_P],
    "blgpu_context_set_fill_style_rgba32": [_P, _U32],
    "blgpu_context_set_fill_style_gradient": [_P, ctypes.POINTER(Gradient)],
    "blgpu_context_set_fill_style_pattern": [_P, ctypes.POINTER(Pattern)],
    "blgpu_context_clear_all": [_P],
    "blgpu_context_fill_all": [_P],
    "blgpu_context_fill_rect_i": [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32],
    "blgpu_context_fill_rect_d": [_P, _D, _D, _D, _D],
    "blgpu_context_fill_box_d": [_P, _D, _D, _D, _D],
    "blgpu_context_fill_polygon_d": [_P, _P, ctypes.c_size_t],
    "blgpu_context_fill_path_d": [_P, _P, _P, ctypes.c_size_t],
    "blgpu_context_fill_path_at_d": [_P, ctypes.POINTER(ctypes.c_double), _P, _P, ctypes.c_size_t],
    "blgpu_context_fill_path_fixed_d": [_P, _P, _P, ctypes.c_size_t],
    "blgpu_context_set_stroke_style_rgba32": [_P, _U32],
    "blgpu_context_set_stroke_style_gradient": [_P, ctypes.POINTER(Gradient)],
    "blgpu_context_set_stroke_style_pattern": [_P, ctypes.POINTER(Pattern)],
    "blgpu_context_set_stroke_alpha": [_P, _D],
    "blgpu_context_set_stroke_width": [_P, _D],
    "blgpu_context_set_stroke_miter_limit": [_P, _D],
    "blgpu_context_set_stroke_join": [_P, _U32],
    "blgpu_context_set_stroke_cap": [_P, _U32, _U32],
    "blgpu_context_set_stroke_caps": [_P, _U32],
    "blgpu_context_set_stroke_transform_order": [_P, _U32],
    "blgpu_context_stroke_path_d": [_P, _P, _P, ctypes.c_size_t],
    "blgpu_context_stroke_path_at_d": [_P, ctypes.POINTER(ctypes.c_double), _P, _P, ctypes.c_size_t],
    "blgpu_context_stroke_polyline_d": [_P, _P, ctypes.c_size_t],
    "blgpu_context_stroke_polygon_d": [_P, _P, ctypes.c_size_t],
    "blgpu_context_stroke_box_d": [_P, _D, _D, _D, _D],
    "blgpu_context_stroke_rect_d": [_P, _D, _D, _D, _D],
    "blgpu_context_stroke_line_d": [_P, _D, _D, _D, _D],
    "blgpu_context_blit_image_i": [_P, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(Image), _P],
    "blgpu_context_blit_image_d": [_P, _D, _D, ctypes.POINTER(Image), _P],
    "blgpu_context_blit_scaled_image_i": [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.POINTER(Image), _P],
    "blgpu_context_blit_scaled_image_d": [_P, _D, _D, _D, _D, ctypes.POINTER(Image), _P],
    "blgpu_context_fill_mask_i": [_P, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(Image), _P],
    "blgpu_context_fill_mask_d": [_P, _D, _D, ctypes.POINTER(Image), _P],
    "blgpu_context_fill_geometry": [_P, _U32, ctypes.POINTER(ctypes.c_double)],
    "blgpu_context_stroke_geometry": [_P, _U32, ctypes.POINTER(ctypes.c_double)],
    "blgpu_stroke_outline_d": [_P, _P, ctypes.c_size_t, ctypes.POINTER(StrokeOptions), _P, _P, ctypes.c_size_t,
                               ctypes.POINTER(ctypes.c_size_t)],
    "blgpu_context_submit_stream": [_P, ctypes.c_char_p, ctypes.c_size_t],
    "blgpu_render_batch": [_P, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(Image),
                           _U32],
    "blgpu_render_stream_noalloc": [_P, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(Image)],
}

_lock = threading.Lock()
_lib = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads libblgpu.so (raises if it has not been built: there is no fallback path)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise RuntimeError(f"{path} is missing: build it with `python -m blend2d_gb300.build`")
            lib = ctypes.CDLL(path)
            for name, args in _SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = args
                fn.restype = ctypes.c_uint32
            _lib = lib
        return _lib


def _check(code: int, what: str, runtime=None):
    if code != SUCCESS:
        detail = ""
        if code == ERROR_DEVICE and runtime is not None:
            st = Stats()
            if _lib.blgpu_runtime_get_stats(runtime, ctypes.byref(st)) == SUCCESS:
                detail = f" (cudaError {st.last_cuda_error})"
        raise BLGpuError(code, what, detail)


def _mat(m):
    if m is None:
        return None
    arr = (ctypes.c_double * 6)(*[float(v) for v in m])
    return arr


def make_image(target, format: int | None = None) -> tuple[Image, object]:
    """BLGpuImage for a (h, w) numpy array (host) or torch tensor (host or CUDA): 32-bit pixels
    are PRGB32 unless `format` is FORMAT_XRGB32; 8-bit pixels are A8."""
    if isinstance(target, np.ndarray):
        if target.dtype not in (np.uint32, np.uint8) or target.ndim != 2 or not target.flags["C_CONTIGUOUS"]:
            raise ValueError("target must be a C-contiguous (h, w) uint32 or uint8 array")
        h, w = target.shape
        bpp, flags, ptr = target.itemsize, 0, target.ctypes.data
    else:
        import torch  # device images come from torch tensors
        if not isinstance(target, torch.Tensor) or target.dim() != 2 or target.element_size() not in (1, 4):
            raise ValueError("target must be a 2-D 8-bit or 32-bit tensor")
        if not target.is_contiguous():
            raise ValueError("target tensor must be contiguous")
        h, w = target.shape
        bpp, flags, ptr = target.element_size(), IMAGE_DEVICE_MEMORY if target.is_cuda else 0, target.data_ptr()
    if bpp == 1:
        fmt = FORMAT_A8
    else:
        fmt = FORMAT_PRGB32 if format in (None, 0, FORMAT_A8) else int(format)
    return Image(ptr, w * bpp, w, h, fmt, flags), target


class Runtime:
    """One device, one stream, the device memory of the pipeline (BLGpuRuntime)."""

    def __init__(self, device: int = 0, lut_variant: int = LUT_SSE2, cuda_stream: int | None = None):
        self._lib = load_library()
        info = RuntimeCreateInfo(device, lut_variant, cuda_stream or None)
        h = _P()
        _check(self._lib.blgpu_runtime_create(ctypes.byref(h), ctypes.byref(info)), "blgpu_runtime_create")
        self.handle = h
        self._contexts = weakref.WeakSet()

    def close(self):
        """Destroys the runtime, after every context still open on it: a context must not outlive
        its runtime (its destruction waits on the runtime's frames)."""
        if self.handle:
            for ctx in list(self._contexts):
                ctx.close()
            self._lib.blgpu_runtime_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stats(self) -> Stats:
        s = Stats()
        _check(self._lib.blgpu_runtime_get_stats(self.handle, ctypes.byref(s)), "blgpu_runtime_get_stats")
        return s

    def memory(self) -> MemoryInfo:
        """Device bytes the runtime's arenas hold, and what its last frame used."""
        m = MemoryInfo()
        _check(self._lib.blgpu_runtime_get_memory(self.handle, ctypes.byref(m)), "blgpu_runtime_get_memory")
        return m

    def release_memory(self):
        """Frees the runtime's device arenas (the next frame allocates again)."""
        _check(self._lib.blgpu_runtime_release_memory(self.handle), "blgpu_runtime_release_memory", self.handle)

    def replay(self, use_graph: bool = True):
        _check(self._lib.blgpu_runtime_replay(self.handle, int(use_graph)), "blgpu_runtime_replay")

    def synchronize(self):
        _check(self._lib.blgpu_runtime_synchronize(self.handle), "blgpu_runtime_synchronize")

    def launch_config(self) -> LaunchConfig:
        c = LaunchConfig()
        _check(self._lib.blgpu_runtime_get_launch_config(self.handle, ctypes.byref(c)), "get_launch_config")
        return c

    def set_launch_config(self, config: LaunchConfig):
        _check(self._lib.blgpu_runtime_set_launch_config(self.handle, ctypes.byref(config)), "set_launch_config")

    def set_segment_limit(self, max_segments: int):
        """Caps the segment array at `max_segments` (0: grow as needed); a frame that emits more
        fails with ERROR_DATA_TOO_LARGE."""
        c = self.launch_config()
        c.max_segments = int(max_segments)
        self.set_launch_config(c)

    def autotune(self, trials: int = 3) -> tuple[LaunchConfig, float]:
        """Tunes the launch shapes on the last flushed frame; returns (best config, its ms)."""
        c, ms = LaunchConfig(), ctypes.c_double()
        _check(self._lib.blgpu_runtime_autotune(self.handle, trials, ctypes.byref(c), ctypes.byref(ms)),
               "blgpu_runtime_autotune", self.handle)
        return c, ms.value

    def render_stream_noalloc(self, stream: bytes, device_target) -> None:
        """Renders `stream` into a CUDA tensor without any allocating call (fixed scratch area)."""
        img, _keep = make_image(device_target, stream_format(stream))
        _check(self._lib.blgpu_render_stream_noalloc(self.handle, stream, len(stream), ctypes.byref(img)),
               "blgpu_render_stream_noalloc", self.handle)

    def render_batch(self, streams: list[bytes], targets: list) -> None:
        """Renders each stream into its target (numpy or torch image) in one device pipeline."""
        n = len(streams)
        imgs = (Image * n)()
        keep = []
        for i, t in enumerate(targets):
            imgs[i], k = make_image(t, stream_format(streams[i]))
            keep.append(k)
        ptrs = (ctypes.c_char_p * n)(*streams)
        sizes = (ctypes.c_size_t * n)(*[len(s) for s in streams])
        _check(self._lib.blgpu_render_batch(self.handle, ptrs, sizes, imgs, n), "blgpu_render_batch", self.handle)


class Context:
    """Rendering context bound to one PRGB32, XRGB32 or A8 image (BLContext)."""

    def __init__(self, runtime: Runtime, target=None, format: int | None = None):
        self.rt = runtime
        self._lib = runtime._lib
        h = _P()
        _check(self._lib.blgpu_context_create(ctypes.byref(h), runtime.handle), "blgpu_context_create")
        self.handle = h
        runtime._contexts.add(self)
        self._keep = []
        self._inflight = []
        if target is not None:
            self.begin(target, format)

    def _call(self, name, *args):
        _check(getattr(self._lib, name)(self.handle, *args), name, self.rt.handle)

    def begin(self, target, format: int | None = None):
        """Binds the image: 32-bit pixels are PRGB32 unless `format` is FORMAT_XRGB32, 8-bit ones A8."""
        img, keep = make_image(target, format)
        self._img = img
        self._keep = [keep]
        self._inflight = []
        self._call("blgpu_context_begin", ctypes.byref(img))

    def end(self):
        self._call("blgpu_context_end")
        self._keep = []
        self._inflight = []

    def flush(self, flags: int = FLUSH_SYNC):
        """FLUSH_SYNC renders and waits; FLUSH_ASYNC starts rendering and returns (the target
        holds the result after the next FLUSH_SYNC or end())."""
        self._call("blgpu_context_flush", flags)
        if flags & FLUSH_SYNC:
            self._inflight = []
        elif flags & FLUSH_ASYNC:
            self._inflight.append(self._keep[1:])     # pattern images of frames still rendering
        self._keep = self._keep[:1]

    def close(self):
        if self.handle:
            self._lib.blgpu_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def save(self): self._call("blgpu_context_save")
    def restore(self): self._call("blgpu_context_restore")
    def set_comp_op(self, op): self._call("blgpu_context_set_comp_op", op)
    def set_fill_rule(self, rule): self._call("blgpu_context_set_fill_rule", rule)
    def set_global_alpha(self, a): self._call("blgpu_context_set_global_alpha", a)
    def set_fill_alpha(self, a): self._call("blgpu_context_set_fill_alpha", a)
    def set_hint(self, hint, value): self._call("blgpu_context_set_hint", hint, value)
    def set_transform(self, m): self._call("blgpu_context_set_transform", _mat(m))
    def reset_transform(self): self._call("blgpu_context_reset_transform")
    def set_fill_style_rgba32(self, argb32): self._call("blgpu_context_set_fill_style_rgba32", argb32 & 0xFFFFFFFF)

    def set_fill_style_gradient(self, type, values, stops, extend_mode=EXTEND_PAD, transform=None, _slot="fill"):
        """stops: iterable of (offset, rgba64)."""
        st = (GradientStop * max(len(stops), 1))(*[GradientStop(float(o), int(c)) for o, c in stops])
        vals = list(values) + [0.0] * (6 - len(values))
        m = _mat(transform)
        g = Gradient(type, extend_mode, (ctypes.c_double * 6)(*vals), st, len(stops),
                     ctypes.cast(m, ctypes.POINTER(ctypes.c_double)) if m is not None else None)
        self._call(f"blgpu_context_set_{_slot}_style_gradient", ctypes.byref(g))

    def set_fill_style_pattern(self, image, area=(0, 0, 0, 0), extend_mode=EXTEND_REPEAT, transform=None, _slot="fill",
                               format: int | None = None):
        img, keep = make_image(image, format)
        self._keep.append((img, keep))
        m = _mat(transform)
        p = Pattern(ctypes.pointer(img), (ctypes.c_int32 * 4)(*area), extend_mode,
                    ctypes.cast(m, ctypes.POINTER(ctypes.c_double)) if m is not None else None)
        self._call(f"blgpu_context_set_{_slot}_style_pattern", ctypes.byref(p))

    # -- stroking (the stroke style slot and BLStrokeOptions) --------------------------------------
    def set_stroke_style_rgba32(self, argb32: int): self._call("blgpu_context_set_stroke_style_rgba32", argb32)

    def set_stroke_style_gradient(self, type, values, stops, extend_mode=EXTEND_PAD, transform=None):
        self.set_fill_style_gradient(type, values, stops, extend_mode, transform, _slot="stroke")

    def set_stroke_style_pattern(self, image, area=(0, 0, 0, 0), extend_mode=EXTEND_REPEAT, transform=None):
        self.set_fill_style_pattern(image, area, extend_mode, transform, _slot="stroke")

    def set_stroke_alpha(self, a: float): self._call("blgpu_context_set_stroke_alpha", a)
    def set_stroke_width(self, w: float): self._call("blgpu_context_set_stroke_width", w)
    def set_stroke_miter_limit(self, m: float): self._call("blgpu_context_set_stroke_miter_limit", m)
    def set_stroke_join(self, join: int): self._call("blgpu_context_set_stroke_join", join)
    def set_stroke_cap(self, position: int, cap: int): self._call("blgpu_context_set_stroke_cap", position, cap)
    def set_stroke_caps(self, cap: int): self._call("blgpu_context_set_stroke_caps", cap)
    def set_stroke_transform_order(self, order: int): self._call("blgpu_context_set_stroke_transform_order", order)

    def stroke_path_d(self, cmds, xy, origin=None):
        c = np.ascontiguousarray(cmds, dtype=np.uint8)
        a = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        if c.shape[0] != a.shape[0]:
            raise ValueError("one command per vertex")
        if origin is None:
            self._call("blgpu_context_stroke_path_d", c.ctypes.data, a.ctypes.data, a.shape[0])
        else:
            self._call("blgpu_context_stroke_path_at_d", _mat(list(origin) + [0.0] * 4), c.ctypes.data,
                       a.ctypes.data, a.shape[0])

    def stroke_polyline_d(self, xy):
        a = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        self._call("blgpu_context_stroke_polyline_d", a.ctypes.data, a.shape[0])

    def stroke_polygon_d(self, xy):
        a = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        self._call("blgpu_context_stroke_polygon_d", a.ctypes.data, a.shape[0])

    # -- image blits -----------------------------------------------------------------------------------
    def _blit(self, name, args, image, area, format=None):
        img, keep = make_image(image, format)
        self._keep.append((img, keep))
        ar = (ctypes.c_int32 * 4)(*area) if area is not None else None
        self._call(name, *args, ctypes.byref(img), ctypes.cast(ar, _P) if ar is not None else None)

    # `format`: FORMAT_XRGB32 for a 32-bit image whose alpha bytes are to be read as 0xFF
    def blit_image_i(self, x, y, image, area=None, format=None):
        self._blit("blgpu_context_blit_image_i", (x, y), image, area, format)

    def blit_image_d(self, x, y, image, area=None, format=None):
        self._blit("blgpu_context_blit_image_d", (x, y), image, area, format)

    def blit_scaled_image_i(self, x, y, w, h, image, area=None, format=None):
        self._blit("blgpu_context_blit_scaled_image_i", (x, y, w, h), image, area, format)

    def blit_scaled_image_d(self, x, y, w, h, image, area=None, format=None):
        self._blit("blgpu_context_blit_scaled_image_d", (x, y, w, h), image, area, format)

    # -- masked fills (A8 masks: (h, w) uint8 arrays) ---------------------------------------------------
    def _fill_mask(self, name, x, y, mask, area):
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        if m.ndim != 2:
            raise ValueError("mask must be a (h, w) uint8 array")
        img = Image(m.ctypes.data, m.shape[1], m.shape[1], m.shape[0], FORMAT_A8, 0)
        self._keep.append((img, m))
        ar = (ctypes.c_int32 * 4)(*area) if area is not None else None
        self._call(name, x, y, ctypes.byref(img), ctypes.cast(ar, _P) if ar is not None else None)

    def fill_mask_i(self, x, y, mask, area=None): self._fill_mask("blgpu_context_fill_mask_i", x, y, mask, area)
    def fill_mask_d(self, x, y, mask, area=None): self._fill_mask("blgpu_context_fill_mask_d", x, y, mask, area)

    # -- shapes: BL_GEOMETRY_TYPE_CIRCLE (5), ELLIPSE (6), ROUND_RECT (7), TRIANGLE (12) -------------------
    def fill_geometry(self, gtype: int, values):
        v = (ctypes.c_double * 6)(*([float(x) for x in values] + [0.0] * (6 - len(values))))
        self._call("blgpu_context_fill_geometry", gtype, v)

    def stroke_geometry(self, gtype: int, values):
        v = (ctypes.c_double * 6)(*([float(x) for x in values] + [0.0] * (6 - len(values))))
        self._call("blgpu_context_stroke_geometry", gtype, v)

    def stroke_box_d(self, x0, y0, x1, y1): self._call("blgpu_context_stroke_box_d", x0, y0, x1, y1)
    def stroke_rect_d(self, x, y, w, h): self._call("blgpu_context_stroke_rect_d", x, y, w, h)
    def stroke_line_d(self, x0, y0, x1, y1): self._call("blgpu_context_stroke_line_d", x0, y0, x1, y1)

    def clear_all(self): self._call("blgpu_context_clear_all")
    def fill_all(self): self._call("blgpu_context_fill_all")
    def fill_rect_i(self, x, y, w, h): self._call("blgpu_context_fill_rect_i", x, y, w, h)
    def fill_rect_d(self, x, y, w, h): self._call("blgpu_context_fill_rect_d", x, y, w, h)
    def fill_box_d(self, x0, y0, x1, y1): self._call("blgpu_context_fill_box_d", x0, y0, x1, y1)

    def fill_polygon_d(self, xy):
        a = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        self._call("blgpu_context_fill_polygon_d", a.ctypes.data, a.shape[0])

    def fill_path_d(self, cmds, xy, origin=None):
        c = np.ascontiguousarray(cmds, dtype=np.uint8)
        a = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        if c.shape[0] != a.shape[0]:
            raise ValueError("one command per vertex")
        if origin is None:
            self._call("blgpu_context_fill_path_d", c.ctypes.data, a.ctypes.data, a.shape[0])
        else:
            self._call("blgpu_context_fill_path_at_d", _mat(list(origin) + [0.0] * 4), c.ctypes.data, a.ctypes.data,
                       a.shape[0])

    def fill_path_fixed_d(self, cmds, xy):
        """Fills a path given in 24.8 pixel space (pixel coordinates x 256), non-zero."""
        c = np.ascontiguousarray(cmds, dtype=np.uint8)
        a = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
        if c.shape[0] != a.shape[0]:
            raise ValueError("one command per vertex")
        self._call("blgpu_context_fill_path_fixed_d", c.ctypes.data, a.ctypes.data, a.shape[0])

    def submit_stream(self, stream: bytes):
        self._call("blgpu_context_submit_stream", stream, len(stream))


def stroke_outline(cmds, xy, width=1.0, miter_limit=4.0, join=0, start_cap=0, end_cap=0):
    """The outline a stroke of the path fills non-zero (host-side, no device): (cmds, xy)."""
    lib = load_library()
    c = np.ascontiguousarray(cmds, dtype=np.uint8)
    a = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2)
    opt = StrokeOptions(width, miter_limit, join, start_cap, end_cap, 0)
    n = ctypes.c_size_t(0)
    cap = max(64, 16 * c.shape[0])
    while True:
        oc = np.zeros(cap, dtype=np.uint8)
        ox = np.zeros((cap, 2), dtype=np.float64)
        r = lib.blgpu_stroke_outline_d(c.ctypes.data, a.ctypes.data, c.shape[0], ctypes.byref(opt),
                                       oc.ctypes.data, ox.ctypes.data, cap, ctypes.byref(n))
        if r == ERROR_DATA_TOO_LARGE:
            cap = n.value
            continue
        _check(r, "blgpu_stroke_outline_d")
        return oc[: n.value].copy(), ox[: n.value].copy()


def stream_size(stream: bytes) -> tuple[int, int]:
    w, h = struct.unpack_from("<II", stream, 8)
    return w, h


def stream_format(stream: bytes) -> int:
    """The target format a stream was recorded for (its header's 0 reads as PRGB32)."""
    return struct.unpack_from("<I", stream, 20)[0] or FORMAT_PRGB32


def render_stream(runtime: Runtime, stream: bytes, target=None):
    """Renders a command stream into `target` (default: a new zeroed host image, uint8 for an A8
    stream); returns it."""
    fmt = stream_format(stream)
    if target is None:
        w, h = stream_size(stream)
        target = np.zeros((h, w), dtype=np.uint8 if fmt == FORMAT_A8 else np.uint32)
    ctx = Context(runtime, target, fmt)
    try:
        ctx.submit_stream(stream)
        ctx.end()
    finally:
        ctx.close()
    return target
