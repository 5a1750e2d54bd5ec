/*
 * blgpu.h - C ABI of the GB300 raster backend (libblgpu.so).
 *
 * The entry points mirror the reference's C rendering-context API (blend2d/core/context.h:631-803,
 * bl_context_*): same call names modulo the prefix, same argument meaning, same enum values, same
 * BLResult error codes. A BLGpuContext records fill calls into a frame; flush(SYNC)/end() runs
 * the frame on the GPU and writes the pixels back into the caller's PRGB32 image. Pixels are
 * bit-exact to the reference's synchronous fixed pipeline.
 *
 * Plain pointers and sizes only; no CUDA or C++ types appear in the signatures.
 */
#ifndef BLGPU_H_INCLUDED
#define BLGPU_H_INCLUDED

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef uint32_t BLGpuResult;

/* BLResult values used by this backend (blend2d/core/api.h, BLResultCode). */
enum {
  BLGPU_SUCCESS = 0,
  BLGPU_ERROR_OUT_OF_MEMORY = 0x00010000u,   /* BL_ERROR_OUT_OF_MEMORY */
  BLGPU_ERROR_INVALID_VALUE = 0x00010001u,   /* BL_ERROR_INVALID_VALUE */
  BLGPU_ERROR_INVALID_STATE = 0x00010002u,   /* BL_ERROR_INVALID_STATE */
  BLGPU_ERROR_NOT_IMPLEMENTED = 0x00010007u, /* BL_ERROR_NOT_IMPLEMENTED */
  BLGPU_ERROR_NO_STATES_TO_RESTORE = 0x00010038u, /* BL_ERROR_NO_STATES_TO_RESTORE */
  BLGPU_ERROR_DATA_TOO_LARGE = 0x00010032u,   /* BL_ERROR_DATA_TOO_LARGE */
  BLGPU_ERROR_INVALID_GEOMETRY = 0x00010034u, /* BL_ERROR_INVALID_GEOMETRY */
  BLGPU_ERROR_DEVICE = 0x00011000u           /* CUDA failure (no reference counterpart) */
};

/* Image formats (BLFormat) and image-placement flags. */
enum {
  BLGPU_FORMAT_PRGB32 = 1,                   /* BL_FORMAT_PRGB32 */
  BLGPU_FORMAT_XRGB32 = 2,                   /* BL_FORMAT_XRGB32 (targets; pattern and blit sources) */
  BLGPU_FORMAT_A8 = 3,                       /* BL_FORMAT_A8 (targets; masks for fill_mask) */
  BLGPU_IMAGE_DEVICE_MEMORY = 0x1u           /* pixel_data is a CUDA device pointer */
};

/* bl_context_flush flags (BLContextFlushFlags). SYNC renders everything recorded so far and waits
   (the image holds the result when it returns). ASYNC is this backend's extension, the explicit
   form of the reference's asynchronous context handing a full command batch to its workers
   (rastercontext.cpp:1480-1492): the recorded frame starts rendering and the call returns at once;
   recording continues into a second buffer, frames render in order, and the image holds the
   result after the next SYNC flush or end(). An error of an asynchronous frame is returned there.
   No flag (BL_CONTEXT_FLUSH_NO_FLAGS) does nothing, as in the reference. */
enum {
  BLGPU_FLUSH_ASYNC = 0x1u,
  BLGPU_FLUSH_SYNC = 0x80000000u             /* BL_CONTEXT_FLUSH_SYNC */
};

/* Gradient LUT builder the backend reproduces (blend2d/pixelops/funcs.cpp:22-34). */
enum {
  BLGPU_LUT_SSE2 = 0,    /* reference no-JIT x86-64 build (default) */
  BLGPU_LUT_AVX2 = 1,    /* reference JIT build on AVX2 machines */
  BLGPU_LUT_SCALAR = 2   /* reference no-JIT build on non-x86 hosts */
};

typedef struct BLGpuRuntime BLGpuRuntime;
typedef struct BLGpuContext BLGpuContext;

typedef struct BLGpuRuntimeCreateInfo {
  int32_t device;          /* CUDA device ordinal */
  uint32_t lut_variant;    /* BLGPU_LUT_* */
  void* cuda_stream;       /* cudaStream_t to run on (NULL = a private stream) */
  uint32_t reserved[4];
} BLGpuRuntimeCreateInfo;

/* An image (BLImageData). A render target is PRGB32, XRGB32 or A8. The reference renders into
   an XRGB32 target with the PRGB32 pipelines, its comp-ops simplified for that format
   (compopsimplifyimpl_p.h), and into an A8 target with the alpha byte of the same arithmetic,
   without dithering. Pattern and blit sources are PRGB32 or XRGB32, whose texels are read with
   the alpha byte set. fill_mask masks are A8. */
typedef struct BLGpuImage {
  void* pixel_data;        /* pixels (host memory unless BLGPU_IMAGE_DEVICE_MEMORY) */
  intptr_t stride;         /* bytes per row */
  int32_t width, height;
  uint32_t format;         /* BLGPU_FORMAT_* */
  uint32_t flags;          /* BLGPU_IMAGE_* */
} BLGpuImage;

typedef struct BLGpuGradientStop {
  double offset;
  uint64_t rgba64;         /* BLRgba64: a<<48 | r<<32 | g<<16 | b */
} BLGpuGradientStop;

typedef struct BLGpuGradient {   /* BLGradientCore contents (blend2d/core/gradient.h) */
  uint32_t type;           /* BL_GRADIENT_TYPE_LINEAR / RADIAL / CONIC */
  uint32_t extend_mode;    /* BL_EXTEND_MODE_PAD / REPEAT / REFLECT */
  double values[6];        /* BLLinear/Radial/ConicGradientValues */
  const BLGpuGradientStop* stops;
  size_t stop_count;
  const double* transform; /* BLMatrix2D m00 m01 m10 m11 m20 m21, or NULL */
} BLGpuGradient;

typedef struct BLGpuPattern {    /* BLPatternCore contents (blend2d/core/pattern.h) */
  const BLGpuImage* image; /* PRGB32 source (host memory) */
  int32_t area[4];         /* x, y, w, h; w == 0 selects the whole image */
  uint32_t extend_mode;    /* simple BL_EXTEND_MODE_* */
  const double* transform; /* BLMatrix2D, or NULL */
} BLGpuPattern;

typedef struct BLGpuStats {
  uint64_t frames;
  uint64_t fill_commands;  /* commands of the last frame */
  uint64_t segments;       /* 24.8 segments the last frame's edge builder produced */
  uint64_t tiles;          /* tiles of the last frame */
  uint64_t kernel_launches;/* kernels launched by the last frame's device pipeline */
  double last_gpu_ms;      /* device time of the last frame's pipeline (CUDA events) */
  double last_fine_ms;     /* device time of its fine stage: coverage + composite kernels */
  uint64_t pixel_ops;      /* composited pixels of the last frame (mask != 0, summed over commands) */
  uint64_t pattern_ops;    /* ... of which fetched from a pattern */
  uint64_t input_vertices; /* vertices of the last frame's polygon/path fills */
  uint64_t h2d_bytes;      /* host->device bytes of the last flush (frame data + canvas uploads) */
  uint64_t d2h_bytes;      /* device->host bytes of the last flush (canvas downloads + sizes) */
  int64_t last_cuda_error; /* cudaError_t behind the last BLGPU_ERROR_DEVICE (0 if none) */
  double last_composite_ms;/* ... of which the composite kernel */
  uint64_t graph_frames;   /* frames that ran as a replay of the captured graph (graph_frames launch config) */
  double last_record_ms;   /* host time of the last blgpu_render_batch's recording (all threads) */
  double last_merge_ms;    /* ... of merging its threads' frame parts */
  double last_upload_ms;   /* host time of the last frame's upload call (staging, copies enqueued) */
  double last_run_ms;      /* host time of the last frame's run: upload, pipeline, read-back */
} BLGpuStats;

/* Launch shapes of the device pipeline (0 in a *_blocks_per_sm field = as many as fit). Tile and
 * band geometry are fixed by the pipeline (32-pixel tile columns matching a warp's lanes, the
 * reference's band heights), so the tunable parameters are how work is grouped and gridded. */
typedef struct BLGpuLaunchConfig {
  int32_t cover_slots;          /* slots (command x 4-row strip x 32-px tile column) per coverage block: 16, 32 or 64; 0 = chosen per frame */
  int32_t cover_blocks_per_sm;  /* coverage pass grid */
  int32_t fine_blocks_per_sm;   /* composite pass grid */
  int32_t edge_block;           /* threads per block of the per-item edge builder: 64, 128 or 256 */
  int32_t cubic_blocks_per_sm;  /* lane-scheduled curve-piece flattener grid */
  int32_t no_occlusion_cull;    /* 1: composite every command of every strip (pixel-op counts of the
                                   reference's work; same pixels) */
  int32_t max_segments;         /* 0: the segment array grows as frames need; N > 0: it never holds more
                                   than N segments, and a frame that emits more fails with
                                   BLGPU_ERROR_DATA_TOO_LARGE (a cap on the runtime's device memory) */
  int32_t graph_frames;         /* 1: frames run as one captured CUDA graph over arrays sized by
                                   capacities (grown as frames need, with headroom): a new frame that
                                   fits is uploaded in place and the graph replayed, with no host
                                   round trip inside the frame; a frame that does not fit grows the
                                   capacities and runs eagerly. Frames with strokes, or whose device
                                   targets are drawn in place onto existing content, run eagerly. */
  int32_t list_rows;            /* pixel rows per command list of the composite (4, 8, 16 or 32; 0 =
                                   32): shorter lists hold fewer commands a strip must test, at the
                                   cost of more list entries */
  int32_t device_order;         /* 1: this runtime's frame pipelines and those of the other runtimes on
                                   the device that set it run their kernels one frame after another, in
                                   the order their frames were submitted (their copies are not ordered,
                                   so one frame's transfers overlap another's kernels). For runtimes
                                   taking turns on large frames, whose kernels each fill the device and
                                   only slow each other down when run at once. Such a runtime moves
                                   page-locked canvases by DMA rather than by a copy kernel, so its
                                   copies take no SM time from the other runtimes' kernels. */
} BLGpuLaunchConfig;

/* --- runtime (device, stream, memory) --------------------------------------------------- */
BLGpuResult blgpu_runtime_create(BLGpuRuntime** out, const BLGpuRuntimeCreateInfo* info);
/* Destroy every context created on the runtime first: a context's destruction waits on the
 * runtime's in-flight frames. */
BLGpuResult blgpu_runtime_destroy(BLGpuRuntime* rt);
BLGpuResult blgpu_runtime_get_stats(const BLGpuRuntime* rt, BLGpuStats* out);

/* Device memory of a runtime (no counterpart in the reference, which renders in host memory). */
typedef struct BLGpuMemoryInfo {
  uint64_t reserved_bytes;   /* device memory the runtime's arenas hold now (kept across frames) */
  uint64_t last_frame_bytes; /* device memory the last frame used: inputs, canvases, work arrays,
                                segments and binning lists */
  uint64_t reserved[6];
} BLGpuMemoryInfo;
BLGpuResult blgpu_runtime_get_memory(const BLGpuRuntime* rt, BLGpuMemoryInfo* out);
/* Frees the runtime's device arenas (the next frame allocates what it needs again; the last frame
 * can no longer be replayed). For servers that share a device-memory budget between runtimes. */
BLGpuResult blgpu_runtime_release_memory(BLGpuRuntime* rt);
/* Re-runs the device pipeline of the last flushed frame on its device-resident inputs (no
 * host<->device traffic); `use_graph` replays it as a captured CUDA graph. */
BLGpuResult blgpu_runtime_replay(BLGpuRuntime* rt, int use_graph);
BLGpuResult blgpu_runtime_synchronize(BLGpuRuntime* rt);
BLGpuResult blgpu_runtime_get_launch_config(const BLGpuRuntime* rt, BLGpuLaunchConfig* out);
BLGpuResult blgpu_runtime_set_launch_config(BLGpuRuntime* rt, const BLGpuLaunchConfig* config);
/* Autotuner: times the last flushed frame's pipeline under candidate launch shapes (coordinate
 * descent, median of `trials` replays each), keeps the fastest and reports it; the frame's pixels
 * are restored afterwards. No counterpart in the reference (its pipelines are JIT-specialized). */
BLGpuResult blgpu_runtime_autotune(BLGpuRuntime* rt, uint32_t trials, BLGpuLaunchConfig* best, double* best_ms);

/* --- rendering context: bl_context_* ---------------------------------------------------- */
/* bl_context_init + bl_context_begin (context.cpp:316-328): bind `image` as the target. */
BLGpuResult blgpu_context_create(BLGpuContext** out, BLGpuRuntime* rt);
BLGpuResult blgpu_context_destroy(BLGpuContext* ctx);
BLGpuResult blgpu_context_begin(BLGpuContext* ctx, const BLGpuImage* image);
BLGpuResult blgpu_context_end(BLGpuContext* ctx);                         /* bl_context_end */
BLGpuResult blgpu_context_flush(BLGpuContext* ctx, uint32_t flags);       /* bl_context_flush */
BLGpuResult blgpu_context_save(BLGpuContext* ctx);                        /* bl_context_save */
BLGpuResult blgpu_context_restore(BLGpuContext* ctx);                     /* bl_context_restore */

BLGpuResult blgpu_context_set_comp_op(BLGpuContext* ctx, uint32_t comp_op);       /* bl_context_set_comp_op */
BLGpuResult blgpu_context_set_fill_rule(BLGpuContext* ctx, uint32_t fill_rule);   /* bl_context_set_fill_rule */
BLGpuResult blgpu_context_set_global_alpha(BLGpuContext* ctx, double alpha);      /* bl_context_set_global_alpha */
BLGpuResult blgpu_context_set_fill_alpha(BLGpuContext* ctx, double alpha);        /* bl_context_set_fill_alpha */
BLGpuResult blgpu_context_set_hint(BLGpuContext* ctx, uint32_t hint, uint32_t value); /* bl_context_set_hint */
BLGpuResult blgpu_context_set_transform(BLGpuContext* ctx, const double m[6]);    /* apply_transform_op(ASSIGN) */
BLGpuResult blgpu_context_reset_transform(BLGpuContext* ctx);                     /* apply_transform_op(RESET) */

BLGpuResult blgpu_context_set_fill_style_rgba32(BLGpuContext* ctx, uint32_t argb32);           /* bl_context_set_fill_style_rgba32 */
BLGpuResult blgpu_context_set_fill_style_gradient(BLGpuContext* ctx, const BLGpuGradient* g);  /* bl_context_set_fill_style(BLGradient) */
BLGpuResult blgpu_context_set_fill_style_pattern(BLGpuContext* ctx, const BLGpuPattern* p);    /* bl_context_set_fill_style(BLPattern) */

BLGpuResult blgpu_context_clear_all(BLGpuContext* ctx);                                       /* bl_context_clear_all */
BLGpuResult blgpu_context_fill_all(BLGpuContext* ctx);                                        /* bl_context_fill_all */
BLGpuResult blgpu_context_fill_rect_i(BLGpuContext* ctx, int32_t x, int32_t y, int32_t w, int32_t h); /* bl_context_fill_rect_i */
BLGpuResult blgpu_context_fill_rect_d(BLGpuContext* ctx, double x, double y, double w, double h);     /* bl_context_fill_rect_d */
BLGpuResult blgpu_context_fill_box_d(BLGpuContext* ctx, double x0, double y0, double x1, double y1);  /* fill_geometry(BOXD) */
BLGpuResult blgpu_context_fill_polygon_d(BLGpuContext* ctx, const double* xy, size_t n);              /* fill_geometry(POLYGOND) */
BLGpuResult blgpu_context_fill_path_d(BLGpuContext* ctx, const uint8_t* cmds, const double* xy, size_t n); /* bl_context_fill_path_d, origin (0, 0) */
/* bl_context_fill_path_d with an origin (BLContextVirt::fill_path_d, context.h:477): the path is
 * drawn with the final transform's linear part and the origin mapped by the final transform as the
 * translation (rastercontext.cpp:2813-2821). */
BLGpuResult blgpu_context_fill_path_at_d(BLGpuContext* ctx, const double origin[2], const uint8_t* cmds,
                                         const double* xy, size_t n);
/* Fills a path whose vertices are already in the target's 24.8 fixed-point pixel space (pixel
 * coordinates x 256), with the fill style and non-zero rule: what a font engine produces for a
 * glyph run under the context's final transform (bl_font_get_glyph_run_outlines with
 * final_transform_fixed(origin), then the edge builder's identity transform -
 * rastercontextops_p.h:68-93, rastercontext.cpp:3082-3110). Text fills go through it. */
BLGpuResult blgpu_context_fill_path_fixed_d(BLGpuContext* ctx, const uint8_t* cmds, const double* xy, size_t n);

/* Stroking (rastercontext.cpp:2059-2165 options, :3794-3870 operations). The stroke has its own
 * style slot and alpha; the outline of the stroked geometry (pathstroke.cpp) is filled non-zero.
 * Joins: BLStrokeJoin 0..4; caps: BLStrokeCap 0..5 at position 0 (start) / 1 (end); transform
 * order: 0 AFTER (stroke in user space), 1 BEFORE. A path the stroker rejects draws nothing and
 * returns BLGPU_ERROR_INVALID_GEOMETRY. */
BLGpuResult blgpu_context_set_stroke_style_rgba32(BLGpuContext* ctx, uint32_t argb32);           /* bl_context_set_stroke_style_rgba32 */
BLGpuResult blgpu_context_set_stroke_style_gradient(BLGpuContext* ctx, const BLGpuGradient* g);  /* bl_context_set_stroke_style(BLGradient) */
BLGpuResult blgpu_context_set_stroke_style_pattern(BLGpuContext* ctx, const BLGpuPattern* p);    /* bl_context_set_stroke_style(BLPattern) */
BLGpuResult blgpu_context_set_stroke_alpha(BLGpuContext* ctx, double alpha);        /* bl_context_set_stroke_alpha */
BLGpuResult blgpu_context_set_stroke_width(BLGpuContext* ctx, double width);        /* bl_context_set_stroke_width */
BLGpuResult blgpu_context_set_stroke_miter_limit(BLGpuContext* ctx, double limit);  /* bl_context_set_stroke_miter_limit */
BLGpuResult blgpu_context_set_stroke_join(BLGpuContext* ctx, uint32_t join);        /* bl_context_set_stroke_join */
BLGpuResult blgpu_context_set_stroke_cap(BLGpuContext* ctx, uint32_t position, uint32_t cap); /* bl_context_set_stroke_cap */
BLGpuResult blgpu_context_set_stroke_caps(BLGpuContext* ctx, uint32_t cap);         /* bl_context_set_stroke_caps */
BLGpuResult blgpu_context_set_stroke_transform_order(BLGpuContext* ctx, uint32_t order); /* bl_context_set_stroke_transform_order */
BLGpuResult blgpu_context_stroke_path_d(BLGpuContext* ctx, const uint8_t* cmds, const double* xy, size_t n); /* bl_context_stroke_path_d, origin (0, 0) */
/* bl_context_stroke_path_d with an origin (BLContextVirt::stroke_path_d, context.h:565; origin
 * handling in add_stroked_path_edges, rastercontextops_p.h:95-121). */
BLGpuResult blgpu_context_stroke_path_at_d(BLGpuContext* ctx, const double origin[2], const uint8_t* cmds,
                                           const double* xy, size_t n);
BLGpuResult blgpu_context_stroke_polyline_d(BLGpuContext* ctx, const double* xy, size_t n);   /* stroke_geometry(POLYLINED) */
BLGpuResult blgpu_context_stroke_polygon_d(BLGpuContext* ctx, const double* xy, size_t n);    /* stroke_geometry(POLYGOND) */
BLGpuResult blgpu_context_stroke_box_d(BLGpuContext* ctx, double x0, double y0, double x1, double y1); /* stroke_geometry(BOXD) */
BLGpuResult blgpu_context_stroke_rect_d(BLGpuContext* ctx, double x, double y, double w, double h);    /* stroke_geometry(RECTD) */
BLGpuResult blgpu_context_stroke_line_d(BLGpuContext* ctx, double x0, double y0, double x1, double y1); /* stroke_geometry(LINE) */

/* Image blits (rastercontext.cpp:3941-4160): the image (PRGB32; `area` = {x, y, w, h} or NULL for
 * all of it) composited with the comp-op and the global alpha (not the fill alpha) at the origin,
 * or scaled into the rectangle, through the current transform; the pattern quality hint picks
 * nearest or bilinear where the image is not pixel aligned. An area outside the image returns
 * BLGPU_ERROR_INVALID_VALUE. */
BLGpuResult blgpu_context_blit_image_i(BLGpuContext* ctx, int32_t x, int32_t y, const BLGpuImage* image, const int32_t* area); /* bl_context_blit_image_i */
BLGpuResult blgpu_context_blit_image_d(BLGpuContext* ctx, double x, double y, const BLGpuImage* image, const int32_t* area);   /* bl_context_blit_image_d */
BLGpuResult blgpu_context_blit_scaled_image_i(BLGpuContext* ctx, int32_t x, int32_t y, int32_t w, int32_t h,
                                              const BLGpuImage* image, const int32_t* area);                                  /* bl_context_blit_scaled_image_i */
BLGpuResult blgpu_context_blit_scaled_image_d(BLGpuContext* ctx, double x, double y, double w, double h,
                                              const BLGpuImage* image, const int32_t* area);                                  /* bl_context_blit_scaled_image_d */

/* Masked fills (rastercontext.cpp:3679-3790): the fill style composited through an A8 mask
 * (BLGPU_FORMAT_A8; `area` = {x, y, w, h} of it or NULL) at the origin, per pixel mask x fill alpha.
 * Like the reference, only a pixel-aligned placement under a translation is supported; any other
 * returns BLGPU_ERROR_NOT_IMPLEMENTED. */
BLGpuResult blgpu_context_fill_mask_i(BLGpuContext* ctx, int32_t x, int32_t y, const BLGpuImage* mask, const int32_t* area); /* bl_context_fill_mask_i */
BLGpuResult blgpu_context_fill_mask_d(BLGpuContext* ctx, double x, double y, const BLGpuImage* mask, const int32_t* area);   /* bl_context_fill_mask_d */

/* Shapes (fill_geometry / stroke_geometry, rastercontext.cpp:2926-2980 and :3208-3234): the path
 * BLPath::add_geometry builds (path.cpp:1408-1600) filled with the fill rule or stroked. `type` is a
 * BLGeometryType: BL_GEOMETRY_TYPE_CIRCLE (5) {cx, cy, r}, ELLIPSE (6) {cx, cy, rx, ry}, ROUND_RECT
 * (7) {x, y, w, h, rx, ry}, ARC (8) / CHORD (9) / PIE (10) {cx, cy, rx, ry, start, sweep}, TRIANGLE
 * (12) {x0, y0, x1, y1, x2, y2}; boxes, rects, lines, polylines, polygons and paths have their own
 * entry points; other types return BLGPU_ERROR_NOT_IMPLEMENTED. */
BLGpuResult blgpu_context_fill_geometry(BLGpuContext* ctx, uint32_t type, const double* values);   /* bl_context_fill_geometry */
BLGpuResult blgpu_context_stroke_geometry(BLGpuContext* ctx, uint32_t type, const double* values); /* bl_context_stroke_geometry */

/* BLStrokeOptions without the dash array (core/path.h:330-352). */
typedef struct BLGpuStrokeOptions {
  double width;
  double miter_limit;
  uint32_t join;
  uint32_t start_cap;
  uint32_t end_cap;
  uint32_t reserved;
} BLGpuStrokeOptions;

/* The outline a stroke fills (non-zero), in user space: per closed figure of the input its two
 * offset figures, per open figure one loop (offset, end cap, reversed inner offset, start cap).
 * Host-only; needs no device. *out_n receives the vertex count; BLGPU_ERROR_DATA_TOO_LARGE when
 * it exceeds `capacity` (nothing written). Counterpart of bl_path_add_stroked_path
 * (core/path.h:1232), whose figures are the same segments in a different arrangement. */
BLGpuResult blgpu_stroke_outline_d(const uint8_t* cmds, const double* xy, size_t n, const BLGpuStrokeOptions* options,
                                   uint8_t* out_cmds, double* out_xy, size_t capacity, size_t* out_n);

/* Replays a serialized command stream (include/blgpu_stream.h) into the context; the stream's
 * canvas size must match the bound image. */
BLGpuResult blgpu_context_submit_stream(BLGpuContext* ctx, const void* stream, size_t size);

/* Batched rendering: renders `count` independent command streams (each with its own canvas)
 * into `images` in one device pipeline (one persistent launch over every canvas's tiles). */
BLGpuResult blgpu_render_batch(BLGpuRuntime* rt, const void* const* streams, const size_t* sizes,
                               const BLGpuImage* images, uint32_t count);

/* --- no-allocation variant --------------------------------------------------------------
 * No counterpart in the reference (its raster context allocates band and cell buffers of its own).
 *
 * Renders one command stream (include/blgpu_stream.h) into `device_image`, a PRGB32 image in
 * device memory (BLGPU_IMAGE_DEVICE_MEMORY, 16-byte aligned rows), on the runtime's stream,
 * without any allocating call: no cudaMalloc/cudaFree, no pinned host allocation, no allocating
 * library call. Every device buffer the pipeline needs is carved out of one fixed scratch area per
 * device, a statically allocated 256-byte aligned array of 32 MiB whose address is looked up once
 * per device (cudaGetSymbolAddress, with that device current) on the first call - make the first
 * call before any stream capture. Pixels are identical to blgpu_context_submit_stream + end.
 *
 * Limit: the frame's data, LUTs, pattern images, segments and binning lists must fit in the 32 MiB
 * area (a few thousand fills on a canvas up to about 2048 x 2048); larger frames return
 * BLGPU_ERROR_DATA_TOO_LARGE and leave the image unchanged. Frames with strokes return
 * BLGPU_ERROR_NOT_IMPLEMENTED (their outline sizes come from a device pass whose buffers the area
 * does not hold). Nothing in the area has to start at zero: the call clears every counter and
 * list it accumulates into before use. The area exists once per device in each process (every
 * process that loads the library holds its own 32 MiB copy on each device it uses); calls of one
 * process on one device share it, and calls that overlapped on the GPU would race on it, so the
 * library serializes them on a per-device lock. A cudaDeviceReset after the first call on a
 * device is not supported (the address looked up then is cached). Blocking: returns when the
 * image is written. For callers that must not allocate device memory while rendering, e.g. a
 * renderer running next to a job that owns the device's memory pool, or a process whose memory
 * budget is fixed up front. */
BLGpuResult blgpu_render_stream_noalloc(BLGpuRuntime* rt, const void* stream, size_t size,
                                        const BLGpuImage* device_image);

#ifdef __cplusplus
}
#endif

#endif /* BLGPU_H_INCLUDED */
