/*
 * blgpu_stream.h - serialized render-command stream ("display list") for the blgpu raster backend.
 *
 * A stream is a flat little-endian byte buffer: a header, the pattern source images it references,
 * then a sequence of records. Each record mirrors one BLContext C-API call of the reference
 * (blend2d/core/context.h:631-803) with the same argument meaning, so a stream can be replayed into
 * the reference `BLContext` or into `blgpu_context_submit_stream()` and must produce the same pixels.
 *
 * Record layout: { uint32 op; uint32 payload_bytes; payload[payload_bytes] } with payload_bytes a
 * multiple of 8 (records stay 8-byte aligned). Enum values are the reference's own values.
 */
#ifndef BLGPU_STREAM_H_INCLUDED
#define BLGPU_STREAM_H_INCLUDED

#include <stdint.h>

#define BLGPU_STREAM_MAGIC   0x53443242u /* "B2DS" */
#define BLGPU_STREAM_VERSION 1u

/* Enum values shared with the reference (blend2d/core headers). */
enum {
  BLGPU_COMP_OP_SRC_OVER = 0,          /* BL_COMP_OP_SRC_OVER (context.h:244) */
  BLGPU_COMP_OP_SRC_COPY = 1,          /* BL_COMP_OP_SRC_COPY (context.h:246) */
  BLGPU_FILL_RULE_NON_ZERO = 0,        /* BL_FILL_RULE_NON_ZERO (geometry.h:101) */
  BLGPU_FILL_RULE_EVEN_ODD = 1,        /* BL_FILL_RULE_EVEN_ODD (geometry.h:103) */
  BLGPU_GRADIENT_LINEAR = 0,           /* BL_GRADIENT_TYPE_* (gradient.h:23-27) */
  BLGPU_GRADIENT_RADIAL = 1,
  BLGPU_GRADIENT_CONIC = 2,
  BLGPU_EXTEND_PAD = 0,                /* BL_EXTEND_MODE_* (api.h:1344-1348) */
  BLGPU_EXTEND_REPEAT = 1,
  BLGPU_EXTEND_REFLECT = 2,
  BLGPU_HINT_GRADIENT_QUALITY = 1,     /* BL_CONTEXT_HINT_* (context.h:53-55) */
  BLGPU_HINT_PATTERN_QUALITY = 2,
  BLGPU_PATTERN_NEAREST = 0,           /* BL_PATTERN_QUALITY_* (pattern.h:23-25) */
  BLGPU_PATTERN_BILINEAR = 1,
  BLGPU_PATH_MOVE = 0,                 /* BL_PATH_CMD_* (path.h:22-32) */
  BLGPU_PATH_ON = 1,
  BLGPU_PATH_QUAD = 2,
  BLGPU_PATH_CONIC = 3,
  BLGPU_PATH_CUBIC = 4,
  BLGPU_PATH_CLOSE = 5
};

/* Record opcodes. */
enum {
  BLGPU_OP_END = 0,
  BLGPU_OP_SET_COMP_OP = 1,        /* u32 comp_op, u32 pad                         bl_context_set_comp_op */
  BLGPU_OP_SET_FILL_RULE = 2,      /* u32 fill_rule, u32 pad                       bl_context_set_fill_rule */
  BLGPU_OP_SET_GLOBAL_ALPHA = 3,   /* f64 alpha                                    bl_context_set_global_alpha */
  BLGPU_OP_SET_FILL_ALPHA = 4,     /* f64 alpha                                    bl_context_set_fill_alpha */
  BLGPU_OP_SET_HINT = 5,           /* u32 hint, u32 value                          bl_context_set_hint */
  BLGPU_OP_SET_TRANSFORM = 6,      /* f64 m[6] (m00 m01 m10 m11 m20 m21)           BL_TRANSFORM_OP_ASSIGN */
  BLGPU_OP_RESET_TRANSFORM = 7,    /* -                                            BL_TRANSFORM_OP_RESET */
  BLGPU_OP_STYLE_RGBA32 = 8,       /* u32 argb32, u32 pad                          bl_context_set_fill_style_rgba32 */
  BLGPU_OP_STYLE_GRADIENT = 9,     /* BLGpuStreamGradient + stops[]                bl_context_set_fill_style(BLGradient) */
  BLGPU_OP_STYLE_PATTERN = 10,     /* BLGpuStreamPattern                           bl_context_set_fill_style(BLPattern) */
  BLGPU_OP_CLEAR_ALL = 11,         /* -                                            bl_context_clear_all */
  BLGPU_OP_FILL_ALL = 12,          /* -                                            bl_context_fill_all */
  BLGPU_OP_FILL_RECT_I = 13,       /* i32 x, y, w, h                               bl_context_fill_rect_i */
  BLGPU_OP_FILL_RECT_D = 14,       /* f64 x, y, w, h                               bl_context_fill_rect_d */
  BLGPU_OP_FILL_BOX_D = 15,        /* f64 x0, y0, x1, y1                           fill_geometry(BOXD) */
  BLGPU_OP_FILL_POLYGON_D = 16,    /* u32 n, u32 pad, f64 xy[2n]                   fill_geometry(POLYGOND) */
  BLGPU_OP_FILL_PATH_D = 17,       /* u32 n, u32 pad, u8 cmd[n] (pad 8), f64 xy[2n] bl_context_fill_path_d */
  BLGPU_OP_SAVE = 18,              /* -                                            bl_context_save */
  BLGPU_OP_RESTORE = 19,           /* -                                            bl_context_restore */
  /* stroking (stroke style slot, stroke options; rastercontext.cpp:2059-2165, :3794-3870) */
  BLGPU_OP_SET_STROKE_WIDTH = 20,  /* f64 width                                    bl_context_set_stroke_width */
  BLGPU_OP_SET_STROKE_MITER_LIMIT = 21, /* f64 miter_limit                         bl_context_set_stroke_miter_limit */
  BLGPU_OP_SET_STROKE_JOIN = 22,   /* u32 join, u32 pad                            bl_context_set_stroke_join */
  BLGPU_OP_SET_STROKE_CAPS = 23,   /* u32 start_cap, u32 end_cap                   bl_context_set_stroke_cap x2 */
  BLGPU_OP_SET_STROKE_TRANSFORM_ORDER = 24, /* u32 order, u32 pad                  bl_context_set_stroke_transform_order */
  BLGPU_OP_SET_STROKE_ALPHA = 25,  /* f64 alpha                                    bl_context_set_stroke_alpha */
  BLGPU_OP_STROKE_STYLE_RGBA32 = 26,   /* u32 argb32, u32 pad                      bl_context_set_stroke_style_rgba32 */
  BLGPU_OP_STROKE_STYLE_GRADIENT = 27, /* BLGpuStreamGradient + stops[]            bl_context_set_stroke_style(BLGradient) */
  BLGPU_OP_STROKE_STYLE_PATTERN = 28,  /* BLGpuStreamPattern                       bl_context_set_stroke_style(BLPattern) */
  BLGPU_OP_STROKE_PATH_D = 29,     /* u32 n, u32 pad, u8 cmd[n] (pad 8), f64 xy[2n] bl_context_stroke_path_d */
  BLGPU_OP_STROKE_POLYLINE_D = 30, /* u32 n, u32 pad, f64 xy[2n]                   stroke_geometry(POLYLINED) */
  BLGPU_OP_STROKE_POLYGON_D = 31,  /* u32 n, u32 pad, f64 xy[2n]                   stroke_geometry(POLYGOND) */
  BLGPU_OP_STROKE_BOX_D = 32,      /* f64 x0, y0, x1, y1                           stroke_geometry(BOXD) */
  BLGPU_OP_STROKE_RECT_D = 33,     /* f64 x, y, w, h                               stroke_geometry(RECTD) */
  BLGPU_OP_STROKE_LINE_D = 34,     /* f64 x0, y0, x1, y1                           stroke_geometry(LINE) */
  /* image blits (rastercontext.cpp:3941-4160); the image is one of the stream's images */
  BLGPU_OP_BLIT_IMAGE_I = 35,      /* BLGpuStreamBlit (x, y as integers)           bl_context_blit_image_i */
  BLGPU_OP_BLIT_IMAGE_D = 36,      /* BLGpuStreamBlit (x, y)                       bl_context_blit_image_d */
  BLGPU_OP_BLIT_SCALED_IMAGE_I = 37, /* BLGpuStreamBlit (x, y, w, h as integers)   bl_context_blit_scaled_image_i */
  BLGPU_OP_BLIT_SCALED_IMAGE_D = 38, /* BLGpuStreamBlit (x, y, w, h)               bl_context_blit_scaled_image_d */
  /* masked fills (rastercontext.cpp:3679-3790): the A8 mask travels in the record */
  BLGPU_OP_FILL_MASK_I = 39,       /* BLGpuStreamMask (x, y integral) + u8 mask[w*h] (pad 8)  bl_context_fill_mask_i */
  BLGPU_OP_FILL_MASK_D = 40,       /* BLGpuStreamMask + u8 mask[w*h] (pad 8)       bl_context_fill_mask_d */
  /* shapes through their paths (BLPath::add_geometry): circle, ellipse, round rect, triangle */
  BLGPU_OP_FILL_GEOMETRY = 41,     /* u32 BLGeometryType, u32 pad, f64 values[6]   bl_context_fill_geometry */
  BLGPU_OP_STROKE_GEOMETRY = 42,   /* u32 BLGeometryType, u32 pad, f64 values[6]   bl_context_stroke_geometry */
  BLGPU_OP_COUNT
};

/* Pixel formats of the target and of the images (BLFormat values, image.h:21-31). 0 reads as
 * PRGB32. */
enum {
  BLGPU_STREAM_FORMAT_PRGB32 = 1,      /* BL_FORMAT_PRGB32 */
  BLGPU_STREAM_FORMAT_XRGB32 = 2,      /* BL_FORMAT_XRGB32 */
  BLGPU_STREAM_FORMAT_A8 = 3           /* BL_FORMAT_A8 (targets only) */
};

typedef struct BLGpuStreamHeader {
  uint32_t magic;        /* BLGPU_STREAM_MAGIC */
  uint32_t version;      /* BLGPU_STREAM_VERSION */
  uint32_t width;        /* canvas width in pixels */
  uint32_t height;       /* canvas height in pixels */
  uint32_t image_count;  /* number of pattern images that follow the header */
  uint32_t format;       /* the target's BLGPU_STREAM_FORMAT_* (0: PRGB32) */
} BLGpuStreamHeader;

/* Each image: BLGpuStreamImage followed by w*h 32-bit pixels (tightly packed rows), padded to
 * 8 bytes. An XRGB32 image's pixels are read with the alpha byte forced to 0xFF, as the
 * reference's fetchers read them (PixelIO<..., XRGB32>, pipeline/reference/pixelgeneric_p.h). */
typedef struct BLGpuStreamImage {
  uint32_t width;
  uint16_t height;       /* images are at most 65,535 px high (BL_RUNTIME_MAX_IMAGE_SIZE) */
  uint16_t format;       /* BLGPU_STREAM_FORMAT_PRGB32 or _XRGB32 (0: PRGB32) */
} BLGpuStreamImage;

typedef struct BLGpuStreamGradient {
  uint32_t type;         /* BLGPU_GRADIENT_* */
  uint32_t extend_mode;  /* BLGPU_EXTEND_PAD/REPEAT/REFLECT */
  uint32_t stop_count;
  uint32_t has_transform;
  double values[6];      /* linear: x0 y0 x1 y1; radial: x0 y0 x1 y1 r0 r1; conic: x0 y0 angle repeat */
  double transform[6];   /* gradient transform (BLGradient::set_transform) when has_transform */
  /* followed by stop_count x { f64 offset; u64 rgba64 } (BLGradientStop, gradient.h) */
} BLGpuStreamGradient;

typedef struct BLGpuStreamGradientStop {
  double offset;
  uint64_t rgba64;       /* BLRgba64 layout: a<<48 | r<<32 | g<<16 | b */
} BLGpuStreamGradientStop;

typedef struct BLGpuStreamPattern {
  uint32_t image_index;  /* index into the stream's image table */
  uint32_t extend_mode;  /* BLGPU_EXTEND_* (simple modes) */
  int32_t area[4];       /* x, y, w, h; w == 0 selects the whole image */
  uint32_t has_transform;
  uint32_t reserved;
  double transform[6];   /* pattern transform (BLPattern::set_transform) when has_transform */
} BLGpuStreamPattern;

/* Payload of the blit records: the destination point (or rectangle) and the source area of one
 * of the stream's images (has_area = 0: the whole image). */
typedef struct BLGpuStreamBlit {
  double rect[4];        /* x, y[, w, h]; integral values for the _I records */
  uint32_t image_index;
  uint32_t has_area;
  int32_t area[4];       /* x, y, w, h */
} BLGpuStreamBlit;

/* Payload of the masked-fill records, followed by the A8 mask's rows (w bytes each). */
typedef struct BLGpuStreamMask {
  double origin[2];
  uint32_t width;
  uint32_t height;
  uint32_t has_area;
  uint32_t reserved;
  int32_t area[4];       /* x, y, w, h of the mask */
} BLGpuStreamMask;

#endif /* BLGPU_STREAM_H_INCLUDED */
