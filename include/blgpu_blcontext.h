/*
 * blgpu_blcontext.h - a BLContext that renders on the GB300 backend.
 *
 * The binding a Blend2D application (or Blend2D itself) compiles in next to Blend2D: it creates a
 * BLContextImpl of its own whose virtual function table (BLContextVirt, blend2d/core/context.h:
 * 454-613) forwards every call on the fill path to libblgpu.so (include/blgpu.h). After
 *
 *     BLImage img(w, h, BL_FORMAT_PRGB32);
 *     BLContext ctx;
 *     blgpu_blcontext_begin(&ctx, &img, nullptr);
 *
 * every ordinary BLContext call (set_fill_style, fill_path, stroke_path, fill_utf8_text,
 * blit_image, ...) records GPU work; ctx.flush(BL_CONTEXT_FLUSH_SYNC) and ctx.end() render it and
 * leave the pixels in `img`, bit-exact to the reference's synchronous fixed pipeline. Calls the
 * backend does not support return BL_ERROR_NOT_IMPLEMENTED and draw nothing.
 *
 * Source: blend2d_gb300/blcontext/blgpu_blcontext.cpp. It is built against Blend2D's public headers
 * and linked into the application together with Blend2D and libblgpu.so; it is not part of
 * libblgpu.so, whose C ABI has no Blend2D types.
 */
#ifndef BLGPU_BLCONTEXT_H_INCLUDED
#define BLGPU_BLCONTEXT_H_INCLUDED

#include <blend2d/blend2d.h>

#include "blgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct BLGpuContextCreateInfo {
  BLGpuRuntime* runtime;   /* runtime to render on; NULL = a process-wide runtime per device and
                              LUT builder, created on first use and kept until exit */
  int32_t device;          /* CUDA device of the process-wide runtime (runtime == NULL) */
  uint32_t lut_variant;    /* BLGPU_LUT_* of the process-wide runtime (runtime == NULL) */
  uint32_t reserved[4];
} BLGpuContextCreateInfo;

/* Mirrors bl_context_begin (blend2d/core/context.cpp:316-328): replaces `self` with a GPU
 * rendering context bound to `image` (PRGB32, XRGB32 or A8). The impl is allocated like the raster context's
 * (bl_object_alloc_impl_aligned with a BL_OBJECT_TYPE_CONTEXT marker, rastercontext.cpp:4626-4627),
 * so BLContext's destructor, reset() and end() release it; its destruction renders what is still
 * recorded into the image. */
BLResult blgpu_blcontext_begin(BLContextCore* self, BLImageCore* image, const BLGpuContextCreateInfo* info);

/* The function table every GPU context impl points to (for inspection and tests). */
const BLContextVirt* blgpu_blcontext_virt(void);

#ifdef __cplusplus
}
#endif

#endif /* BLGPU_BLCONTEXT_H_INCLUDED */
