// blgpu_blcontext.cpp - a BLContextImpl whose BLContextVirt forwards to libblgpu.so.
//
// Blend2D dispatches every BLContext call through the function table of the context's impl
// (BLContextVirt, blend2d/core/context.h:454-613; the C++ wrapper calls it inline, context.h:
// 2155-2174). The reference's raster context fills that table in rastercontext.cpp:4500-4600; this
// file fills a second one whose entries record GPU work through the C ABI of include/blgpu.h and
// keep the BLContextState that BLContext's inline accessors read (context.h:614-626) up to date.
//
// Only Blend2D's public headers are used. Build: compile this file with
// -I<blend2d include dir> -Iinclude and link it with Blend2D and libblgpu.so.
#include "blgpu_blcontext.h"

#include <math.h>
#include <string.h>

#include <memory>
#include <mutex>
#include <new>
#include <vector>

namespace {

constexpr BLResult kNotImplemented = BL_ERROR_NOT_IMPLEMENTED;

// Everything a save() keeps of the context's own bookkeeping (the device context keeps its own
// copy of the rendering state).
struct Mirror {
  BLContextState st;
  BLVar style[2];
};

struct GpuImpl : public BLContextImpl {
  BLGpuContext* gpu = nullptr;
  BLImage image;                      // the target: holds the pixels the device writes back into
  Mirror cur;
  std::vector<std::unique_ptr<Mirror>> saved;
  BLGlyphBuffer glyphs;               // text: shaping
  BLPath outline;                     // text: glyph outlines in 24.8 pixel space
};

GpuImpl* self_of(BLContextImpl* impl) { return static_cast<GpuImpl*>(impl); }
const GpuImpl* self_of(const BLContextImpl* impl) { return static_cast<const GpuImpl*>(impl); }

// BLContextState starts as the raster context initializes it (rastercontext.cpp:4380-4415).
void init_state(BLContextState& st, BLImageCore* image, int w, int h) {
  memset(static_cast<void*>(&st), 0, sizeof(st));
  st.target_image = image;
  st.target_size = BLSize(double(w), double(h));
  st.hints.reset();
  st.hints.pattern_quality = BL_PATTERN_QUALITY_BILINEAR;
  st.comp_op = BL_COMP_OP_SRC_OVER;
  st.fill_rule = BL_FILL_RULE_NON_ZERO;
  st.style_type[0] = st.style_type[1] = uint8_t(BL_OBJECT_TYPE_RGBA32);
  st.global_alpha = 1.0;
  st.style_alpha[0] = st.style_alpha[1] = 1.0;
  new (&st.stroke_options) BLStrokeOptions();
  st.approximation_options = bl_default_approximation_options;
  st.meta_transform.reset();
  st.user_transform.reset();
  st.final_transform.reset();
}

void copy_state(BLContextState& dst, const BLContextState& src) {
  BLStrokeOptions keep(static_cast<const BLStrokeOptions&>(src.stroke_options));
  static_cast<BLStrokeOptions&>(dst.stroke_options).~BLStrokeOptions();
  memcpy(static_cast<void*>(&dst), &src, sizeof(dst));
  new (&dst.stroke_options) BLStrokeOptions(keep);
}

// --- object lifetime -----------------------------------------------------------------------

BLResult BL_CDECL destroy_impl(BLObjectImpl* base) noexcept {
  GpuImpl* self = static_cast<GpuImpl*>(static_cast<BLContextImpl*>(base));
  // what is still recorded is rendered into the image, as the raster context flushes on detach
  if (self->gpu) blgpu_context_destroy(self->gpu);
  static_cast<BLStrokeOptions&>(self->cur.st.stroke_options).~BLStrokeOptions();
  for (auto& m : self->saved) static_cast<BLStrokeOptions&>(m->st.stroke_options).~BLStrokeOptions();
  self->~GpuImpl();
  return bl_object_free_impl(base);
}

BLResult BL_CDECL get_property_impl(const BLObjectImpl*, const char*, size_t, BLVarCore* out) noexcept {
  bl_var_assign_null(out);
  return BL_ERROR_INVALID_KEY;
}

BLResult BL_CDECL set_property_impl(BLObjectImpl*, const char*, size_t, const BLVarCore*) noexcept {
  return BL_ERROR_INVALID_KEY;
}

// --- conversions -----------------------------------------------------------------------------

// The device view of an image whose BLFormat is `format`, or (`format` 0) PRGB32 or XRGB32, the
// formats a pattern or blit source may have (BLGPU_FORMAT_* values are BLFormat's).
bool gpu_image_of(const BLImageCore* img, uint32_t format, BLGpuImage& out, BLImageData& d) {
  if (bl_image_get_data(img, &d) != BL_SUCCESS) return false;
  if (format ? d.format != format : (d.format != BL_FORMAT_PRGB32 && d.format != BL_FORMAT_XRGB32)) return false;
  out.pixel_data = d.pixel_data;
  out.stride = d.stride;
  out.width = d.size.w;
  out.height = d.size.h;
  out.format = d.format;
  out.flags = 0;
  return true;
}

// Sets `slot`'s style on the device context from a style object (BLGradient / BLPattern) or solid
// colour object. Only the user transform mode is supported (the style is mapped by the user
// transform at the time it is set, like BL_CONTEXT_STYLE_TRANSFORM_MODE_USER).
BLResult set_style_object(GpuImpl* self, uint32_t slot, const BLObjectCore* style) {
  if (style->_d.is_gradient()) {
    const BLGradient& g = static_cast<const BLGradient&>(*style);
    BLGpuGradient gg{};
    gg.type = uint32_t(g.type());
    gg.extend_mode = uint32_t(g.extend_mode());
    for (int i = 0; i < 6; i++) gg.values[i] = g.value(size_t(i));
    gg.stops = reinterpret_cast<const BLGpuGradientStop*>(g.stops());   // {double, BLRgba64}: same layout
    gg.stop_count = g.size();
    const BLMatrix2D& t = g.transform();
    gg.transform = g.transform_type() != BL_TRANSFORM_TYPE_IDENTITY ? &t.m00 : nullptr;
    return slot ? blgpu_context_set_stroke_style_gradient(self->gpu, &gg) : blgpu_context_set_fill_style_gradient(self->gpu, &gg);
  }
  if (style->_d.is_pattern()) {
    const BLPattern& p = static_cast<const BLPattern&>(*style);
    BLImage img;
    BL_PROPAGATE(bl_pattern_get_image(&p, &img));
    BLGpuImage gi{};
    BLImageData d;
    if (!gpu_image_of(&img, 0, gi, d)) return kNotImplemented;
    BLRectI area;
    BL_PROPAGATE(bl_pattern_get_area(&p, &area));
    BLMatrix2D t;
    BL_PROPAGATE(bl_pattern_get_transform(&p, &t));
    BLGpuPattern gp{};
    gp.image = &gi;
    gp.area[0] = area.x; gp.area[1] = area.y; gp.area[2] = area.w; gp.area[3] = area.h;
    gp.extend_mode = uint32_t(p.extend_mode());
    gp.transform = p.transform_type() != BL_TRANSFORM_TYPE_IDENTITY ? &t.m00 : nullptr;
    return slot ? blgpu_context_set_stroke_style_pattern(self->gpu, &gp) : blgpu_context_set_fill_style_pattern(self->gpu, &gp);
  }
  if (style->_d.is_rgba32()) {
    const uint32_t c = style->_d.rgba32.value;
    return slot ? blgpu_context_set_stroke_style_rgba32(self->gpu, c) : blgpu_context_set_fill_style_rgba32(self->gpu, c);
  }
  return kNotImplemented;   // BLRgba / BLRgba64 solid colours, null style
}

// *_rgba32 / *_ext variants: the call's style replaces the slot's for this call only.
template<typename Fn>
BLResult with_style_rgba32(GpuImpl* self, uint32_t slot, uint32_t rgba32, Fn&& fn) {
  BL_PROPAGATE(blgpu_context_save(self->gpu));
  BLResult r = slot ? blgpu_context_set_stroke_style_rgba32(self->gpu, rgba32) : blgpu_context_set_fill_style_rgba32(self->gpu, rgba32);
  if (r == BL_SUCCESS) r = fn();
  BLResult r2 = blgpu_context_restore(self->gpu);
  return r ? r : r2;
}

template<typename Fn>
BLResult with_style_object(GpuImpl* self, uint32_t slot, const BLObjectCore* style, Fn&& fn) {
  BL_PROPAGATE(blgpu_context_save(self->gpu));
  BLResult r = set_style_object(self, slot, style);
  if (r == BL_SUCCESS) r = fn();
  BLResult r2 = blgpu_context_restore(self->gpu);
  return r ? r : r2;
}

// --- fills -----------------------------------------------------------------------------------

BLResult fill_rect_i_(GpuImpl* self, const BLRectI* r) { return blgpu_context_fill_rect_i(self->gpu, r->x, r->y, r->w, r->h); }
BLResult fill_rect_d_(GpuImpl* self, const BLRect* r) { return blgpu_context_fill_rect_d(self->gpu, r->x, r->y, r->w, r->h); }

BLResult fill_path_(GpuImpl* self, const BLPoint* origin, const BLPathCore* path) {
  const BLPath& p = static_cast<const BLPath&>(*path);
  const double o[2] = {origin->x, origin->y};
  return blgpu_context_fill_path_at_d(self->gpu, o, p.command_data(), reinterpret_cast<const double*>(p.vertex_data()), p.size());
}

BLResult stroke_path_(GpuImpl* self, const BLPoint* origin, const BLPathCore* path) {
  const BLPath& p = static_cast<const BLPath&>(*path);
  const double o[2] = {origin->x, origin->y};
  return blgpu_context_stroke_path_at_d(self->gpu, o, p.command_data(), reinterpret_cast<const double*>(p.vertex_data()), p.size());
}

// BLContext's geometry dispatch for the types the backend takes directly; the simple shapes
// (circle ... pie) become paths on the device side exactly as BLPath::add_geometry builds them.
BLResult geometry_(GpuImpl* self, bool stroke, BLGeometryType type, const void* data) {
  BLGpuContext* g = self->gpu;
  switch (type) {
    case BL_GEOMETRY_TYPE_BOXI: {
      const BLBoxI* b = static_cast<const BLBoxI*>(data);
      return stroke ? blgpu_context_stroke_box_d(g, b->x0, b->y0, b->x1, b->y1) : blgpu_context_fill_box_d(g, b->x0, b->y0, b->x1, b->y1);
    }
    case BL_GEOMETRY_TYPE_BOXD: {
      const BLBox* b = static_cast<const BLBox*>(data);
      return stroke ? blgpu_context_stroke_box_d(g, b->x0, b->y0, b->x1, b->y1) : blgpu_context_fill_box_d(g, b->x0, b->y0, b->x1, b->y1);
    }
    case BL_GEOMETRY_TYPE_RECTI: {
      const BLRectI* r = static_cast<const BLRectI*>(data);
      return stroke ? blgpu_context_stroke_rect_d(g, r->x, r->y, r->w, r->h) : blgpu_context_fill_rect_i(g, r->x, r->y, r->w, r->h);
    }
    case BL_GEOMETRY_TYPE_RECTD: {
      const BLRect* r = static_cast<const BLRect*>(data);
      return stroke ? blgpu_context_stroke_rect_d(g, r->x, r->y, r->w, r->h) : blgpu_context_fill_rect_d(g, r->x, r->y, r->w, r->h);
    }
    case BL_GEOMETRY_TYPE_LINE: {
      if (!stroke) return BL_SUCCESS;   // a line has no area
      const BLLine* l = static_cast<const BLLine*>(data);
      return blgpu_context_stroke_line_d(g, l->x0, l->y0, l->x1, l->y1);
    }
    case BL_GEOMETRY_TYPE_POLYGONI: case BL_GEOMETRY_TYPE_POLYLINEI: {
      const BLArrayView<BLPointI>* a = static_cast<const BLArrayView<BLPointI>*>(data);
      std::vector<double> xy(2 * a->size);
      for (size_t i = 0; i < a->size; i++) { xy[2 * i] = a->data[i].x; xy[2 * i + 1] = a->data[i].y; }
      if (!stroke) return blgpu_context_fill_polygon_d(g, xy.data(), a->size);
      return type == BL_GEOMETRY_TYPE_POLYGONI ? blgpu_context_stroke_polygon_d(g, xy.data(), a->size)
                                               : blgpu_context_stroke_polyline_d(g, xy.data(), a->size);
    }
    case BL_GEOMETRY_TYPE_POLYGOND: case BL_GEOMETRY_TYPE_POLYLINED: {
      const BLArrayView<BLPoint>* a = static_cast<const BLArrayView<BLPoint>*>(data);
      const double* xy = reinterpret_cast<const double*>(a->data);
      if (!stroke) return blgpu_context_fill_polygon_d(g, xy, a->size);
      return type == BL_GEOMETRY_TYPE_POLYGOND ? blgpu_context_stroke_polygon_d(g, xy, a->size)
                                               : blgpu_context_stroke_polyline_d(g, xy, a->size);
    }
    case BL_GEOMETRY_TYPE_PATH: {
      const BLPoint origin(0.0, 0.0);
      return stroke ? stroke_path_(self, &origin, static_cast<const BLPathCore*>(data))
                    : fill_path_(self, &origin, static_cast<const BLPathCore*>(data));
    }
    case BL_GEOMETRY_TYPE_CIRCLE: case BL_GEOMETRY_TYPE_ELLIPSE: case BL_GEOMETRY_TYPE_ROUND_RECT:
    case BL_GEOMETRY_TYPE_ARC: case BL_GEOMETRY_TYPE_CHORD: case BL_GEOMETRY_TYPE_PIE: case BL_GEOMETRY_TYPE_TRIANGLE: {
      double v[6] = {};
      const size_t n = type == BL_GEOMETRY_TYPE_CIRCLE ? 3 : type == BL_GEOMETRY_TYPE_ELLIPSE ? 4 : 6;
      memcpy(v, data, n * sizeof(double));     // BLCircle, BLEllipse, BLRoundRect, BLArc, BLTriangle: doubles in order
      return stroke ? blgpu_context_stroke_geometry(g, uint32_t(type), v) : blgpu_context_fill_geometry(g, uint32_t(type), v);
    }
    default:
      return kNotImplemented;
  }
}

// Text (fill_unclipped_text<kSync>, rastercontext.cpp:3082-3110): the run is shaped, its glyph
// outlines are decoded by the font engine under the final transform in 24.8 space with the origin
// mapped by it (add_filled_glyph_run_edges, rastercontextops_p.h:68-93), and the outlines are
// filled non-zero on the device.
// The glyph run of a text call: shaped from UTF-8/16/32 or Latin-1 text, or given
// (fill_unclipped_text / stroke_unclipped_text, rastercontext.cpp:3082-3110, 3263-3290).
BLResult glyph_run_of(GpuImpl* self, const BLFontCore* font, BLContextRenderTextOp op, const void* data,
                      const BLGlyphRun*& run) {
  const BLFont& f = static_cast<const BLFont&>(*font);
  if (!f.is_valid()) return BL_ERROR_FONT_NOT_INITIALIZED;
  if (uint32_t(op) <= uint32_t(BL_TEXT_ENCODING_MAX_VALUE)) {
    const BLDataView* view = static_cast<const BLDataView*>(data);
    BL_PROPAGATE(self->glyphs.set_text(view->data, view->size, BLTextEncoding(op)));
    BL_PROPAGATE(f.shape(self->glyphs));
    run = &self->glyphs.glyph_run();
    return BL_SUCCESS;
  }
  if (op == BL_CONTEXT_RENDER_TEXT_OP_GLYPH_RUN) {
    run = static_cast<const BLGlyphRun*>(data);
    return BL_SUCCESS;
  }
  return BL_ERROR_INVALID_VALUE;
}

// final_transform_fixed (the final transform post-scaled by 256) and the origin mapped by it.
void fixed_origin(const GpuImpl* self, const BLPoint* origin, BLMatrix2D& ft, BLPoint& of) {
  ft = self->cur.st.final_transform;
  ft.m00 *= 256.0; ft.m01 *= 256.0; ft.m10 *= 256.0; ft.m11 *= 256.0; ft.m20 *= 256.0; ft.m21 *= 256.0;
  of.reset(origin->x * ft.m00 + origin->y * ft.m10 + ft.m20, origin->x * ft.m01 + origin->y * ft.m11 + ft.m21);
}

BLResult fill_text_(GpuImpl* self, const BLPoint* origin, const BLFontCore* font, BLContextRenderTextOp op, const void* data) {
  const BLGlyphRun* run = nullptr;
  BL_PROPAGATE(glyph_run_of(self, font, op, data, run));
  if (run->is_empty()) return BL_SUCCESS;
  BLMatrix2D ft;
  BLPoint of;
  fixed_origin(self, origin, ft, of);
  const BLMatrix2D t(ft.m00, ft.m01, ft.m10, ft.m11, of.x, of.y);
  self->outline.clear();
  BL_PROPAGATE(bl_font_get_glyph_run_outlines(font, run, &t, &self->outline, nullptr, nullptr));
  const BLPath& p = self->outline;
  return blgpu_context_fill_path_fixed_d(self->gpu, p.command_data(), reinterpret_cast<const double*>(p.vertex_data()), p.size());
}

// Stroked text (add_stroked_glyph_run_edges, rastercontextops_p.h:145-187): the glyph outlines are
// stroked figure by figure into one non-zero fill, which is what the device stroker does with the
// run's outline path.
//   AFTER: the outlines decoded with the identity, stroked in user space, the strokes mapped by
//   final_transform_fixed(origin): a stroke of the path at `origin`.
//   BEFORE: the outlines decoded under the user transform's linear part (the font engine composes
//   it with its own matrices, so they are decoded that way here too), stroked in meta space and
//   mapped by meta_transform_fixed(origin). The meta transform is the identity here, so that is
//   an AFTER stroke under an identity user transform, at the origin whose fixed-point image is
//   the real one (division and multiplication by 256 are exact).
BLResult stroke_text_(GpuImpl* self, const BLPoint* origin, const BLFontCore* font, BLContextRenderTextOp op, const void* data) {
  const BLGlyphRun* run = nullptr;
  BL_PROPAGATE(glyph_run_of(self, font, op, data, run));
  if (run->is_empty()) return BL_SUCCESS;
  const BLContextState& st = self->cur.st;
  self->outline.clear();
  if (st.stroke_options.transform_order == BL_STROKE_TRANSFORM_ORDER_AFTER) {
    const BLMatrix2D id = BLMatrix2D::make_identity();
    BL_PROPAGATE(bl_font_get_glyph_run_outlines(font, run, &id, &self->outline, nullptr, nullptr));
    const BLPath& p = self->outline;
    const double o[2] = {origin->x, origin->y};
    return blgpu_context_stroke_path_at_d(self->gpu, o, p.command_data(), reinterpret_cast<const double*>(p.vertex_data()), p.size());
  }
  const BLMatrix2D& u = st.user_transform;
  const BLMatrix2D ut(u.m00, u.m01, u.m10, u.m11, 0.0, 0.0);
  BL_PROPAGATE(bl_font_get_glyph_run_outlines(font, run, &ut, &self->outline, nullptr, nullptr));
  BLMatrix2D ft;
  BLPoint of;
  fixed_origin(self, origin, ft, of);
  const double o[2] = {of.x / 256.0, of.y / 256.0};
  const BLPath& p = self->outline;
  BL_PROPAGATE(blgpu_context_save(self->gpu));
  BLResult r = blgpu_context_reset_transform(self->gpu);
  if (r == BL_SUCCESS) r = blgpu_context_set_stroke_transform_order(self->gpu, BL_STROKE_TRANSFORM_ORDER_AFTER);
  if (r == BL_SUCCESS)
    r = blgpu_context_stroke_path_at_d(self->gpu, o, p.command_data(), reinterpret_cast<const double*>(p.vertex_data()), p.size());
  const BLResult r2 = blgpu_context_restore(self->gpu);
  return r != BL_SUCCESS ? r : r2;
}

BLResult fill_mask_(GpuImpl* self, double x, double y, bool integral, const BLImageCore* mask, const BLRectI* area) {
  BLGpuImage gm{};
  BLImageData d;
  if (!gpu_image_of(mask, BL_FORMAT_A8, gm, d)) return kNotImplemented;
  const int32_t a[4] = {area ? area->x : 0, area ? area->y : 0, area ? area->w : 0, area ? area->h : 0};
  return integral ? blgpu_context_fill_mask_i(self->gpu, int32_t(x), int32_t(y), &gm, area ? a : nullptr)
                  : blgpu_context_fill_mask_d(self->gpu, x, y, &gm, area ? a : nullptr);
}

BLResult blit_(GpuImpl* self, int kind, const double* r, const BLImageCore* img, const BLRectI* area) {
  BLGpuImage gi{};
  BLImageData d;
  if (!gpu_image_of(img, 0, gi, d)) return kNotImplemented;
  const int32_t a[4] = {area ? area->x : 0, area ? area->y : 0, area ? area->w : 0, area ? area->h : 0};
  const int32_t* ap = area ? a : nullptr;
  switch (kind) {
    case 0: return blgpu_context_blit_image_i(self->gpu, int32_t(r[0]), int32_t(r[1]), &gi, ap);
    case 1: return blgpu_context_blit_image_d(self->gpu, r[0], r[1], &gi, ap);
    case 2: return blgpu_context_blit_scaled_image_i(self->gpu, int32_t(r[0]), int32_t(r[1]), int32_t(r[2]), int32_t(r[3]), &gi, ap);
    default: return blgpu_context_blit_scaled_image_d(self->gpu, r[0], r[1], r[2], r[3], &gi, ap);
  }
}

// --- the function table ------------------------------------------------------------------------

#define SELF GpuImpl* self = self_of(impl)

BLResult BL_CDECL v_apply_transform_op(BLContextImpl* impl, BLTransformOp op, const void* data) noexcept {
  SELF;
  BLMatrix2D m = self->cur.st.user_transform;
  BL_PROPAGATE(bl_matrix2d_apply_op(&m, op, data));
  const double a[6] = {m.m00, m.m01, m.m10, m.m11, m.m20, m.m21};
  BL_PROPAGATE(blgpu_context_set_transform(self->gpu, a));
  self->cur.st.user_transform = m;
  self->cur.st.final_transform = m;        // the meta transform is the identity
  return BL_SUCCESS;
}

BLResult BL_CDECL v_fill_rect_i(BLContextImpl* impl, const BLRectI* r) noexcept { SELF; return fill_rect_i_(self, r); }
BLResult BL_CDECL v_fill_rect_i_rgba32(BLContextImpl* impl, const BLRectI* r, uint32_t c) noexcept {
  SELF; return with_style_rgba32(self, 0, c, [&] { return fill_rect_i_(self, r); });
}
BLResult BL_CDECL v_fill_rect_i_ext(BLContextImpl* impl, const BLRectI* r, const BLObjectCore* s) noexcept {
  SELF; return with_style_object(self, 0, s, [&] { return fill_rect_i_(self, r); });
}
BLResult BL_CDECL v_fill_rect_d(BLContextImpl* impl, const BLRect* r) noexcept { SELF; return fill_rect_d_(self, r); }
BLResult BL_CDECL v_fill_rect_d_rgba32(BLContextImpl* impl, const BLRect* r, uint32_t c) noexcept {
  SELF; return with_style_rgba32(self, 0, c, [&] { return fill_rect_d_(self, r); });
}
BLResult BL_CDECL v_fill_rect_d_ext(BLContextImpl* impl, const BLRect* r, const BLObjectCore* s) noexcept {
  SELF; return with_style_object(self, 0, s, [&] { return fill_rect_d_(self, r); });
}
BLResult BL_CDECL v_fill_path_d(BLContextImpl* impl, const BLPoint* o, const BLPathCore* p) noexcept { SELF; return fill_path_(self, o, p); }
BLResult BL_CDECL v_fill_path_d_rgba32(BLContextImpl* impl, const BLPoint* o, const BLPathCore* p, uint32_t c) noexcept {
  SELF; return with_style_rgba32(self, 0, c, [&] { return fill_path_(self, o, p); });
}
BLResult BL_CDECL v_fill_path_d_ext(BLContextImpl* impl, const BLPoint* o, const BLPathCore* p, const BLObjectCore* s) noexcept {
  SELF; return with_style_object(self, 0, s, [&] { return fill_path_(self, o, p); });
}

BLResult BL_CDECL v_blit_image_i(BLContextImpl* impl, const BLPointI* o, const BLImageCore* img, const BLRectI* area) noexcept {
  SELF; const double r[4] = {double(o->x), double(o->y), 0, 0}; return blit_(self, 0, r, img, area);
}
BLResult BL_CDECL v_blit_image_d(BLContextImpl* impl, const BLPoint* o, const BLImageCore* img, const BLRectI* area) noexcept {
  SELF; const double r[4] = {o->x, o->y, 0, 0}; return blit_(self, 1, r, img, area);
}
BLResult BL_CDECL v_blit_scaled_image_i(BLContextImpl* impl, const BLRectI* rc, const BLImageCore* img, const BLRectI* area) noexcept {
  SELF; const double r[4] = {double(rc->x), double(rc->y), double(rc->w), double(rc->h)}; return blit_(self, 2, r, img, area);
}
BLResult BL_CDECL v_blit_scaled_image_d(BLContextImpl* impl, const BLRect* rc, const BLImageCore* img, const BLRectI* area) noexcept {
  SELF; const double r[4] = {rc->x, rc->y, rc->w, rc->h}; return blit_(self, 3, r, img, area);
}

BLResult BL_CDECL v_flush(BLContextImpl* impl, BLContextFlushFlags flags) noexcept {
  SELF;
  if (flags & BL_CONTEXT_FLUSH_SYNC) return blgpu_context_flush(self->gpu, BLGPU_FLUSH_SYNC);
  return BL_SUCCESS;
}

BLResult BL_CDECL v_save(BLContextImpl* impl, BLContextCookie* cookie) noexcept {
  SELF;
  if (cookie) return kNotImplemented;
  BL_PROPAGATE(blgpu_context_save(self->gpu));
  std::unique_ptr<Mirror> m(new Mirror());
  memset(static_cast<void*>(&m->st), 0, sizeof(m->st));
  new (&m->st.stroke_options) BLStrokeOptions();
  copy_state(m->st, self->cur.st);
  m->style[0] = self->cur.style[0];
  m->style[1] = self->cur.style[1];
  self->saved.push_back(std::move(m));
  self->cur.st.saved_state_count = uint32_t(self->saved.size());
  return BL_SUCCESS;
}

BLResult BL_CDECL v_restore(BLContextImpl* impl, const BLContextCookie* cookie) noexcept {
  SELF;
  if (cookie) return kNotImplemented;
  BL_PROPAGATE(blgpu_context_restore(self->gpu));
  if (self->saved.empty()) return BL_ERROR_NO_STATES_TO_RESTORE;
  std::unique_ptr<Mirror> m = std::move(self->saved.back());
  self->saved.pop_back();
  copy_state(self->cur.st, m->st);
  self->cur.style[0] = m->style[0];
  self->cur.style[1] = m->style[1];
  static_cast<BLStrokeOptions&>(m->st.stroke_options).~BLStrokeOptions();
  self->cur.st.saved_state_count = uint32_t(self->saved.size());
  return BL_SUCCESS;
}

BLResult BL_CDECL v_user_to_meta(BLContextImpl*) noexcept { return kNotImplemented; }

BLResult BL_CDECL v_set_hint(BLContextImpl* impl, BLContextHint hint, uint32_t value) noexcept {
  SELF;
  BL_PROPAGATE(blgpu_context_set_hint(self->gpu, uint32_t(hint), value));
  self->cur.st.hints.hints[hint] = uint8_t(value);
  return BL_SUCCESS;
}

BLResult BL_CDECL v_set_hints(BLContextImpl* impl, const BLContextHints* hints) noexcept {
  for (uint32_t h = 0; h <= BL_CONTEXT_HINT_MAX_VALUE; h++)
    BL_PROPAGATE(v_set_hint(impl, BLContextHint(h), hints->hints[h]));
  return BL_SUCCESS;
}

// The device flattens and offsets with the reference's default approximation options only.
BLResult BL_CDECL v_set_flatten_mode(BLContextImpl*, BLFlattenMode mode) noexcept {
  return mode == BLFlattenMode(bl_default_approximation_options.flatten_mode) ? BL_SUCCESS : kNotImplemented;
}
BLResult BL_CDECL v_set_flatten_tolerance(BLContextImpl*, double t) noexcept {
  return t == bl_default_approximation_options.flatten_tolerance ? BL_SUCCESS : kNotImplemented;
}
BLResult BL_CDECL v_set_approximation_options(BLContextImpl*, const BLApproximationOptions* o) noexcept {
  return memcmp(o, &bl_default_approximation_options, sizeof(*o)) == 0 ? BL_SUCCESS : kNotImplemented;
}

BLResult BL_CDECL v_get_style(const BLContextImpl* impl, BLContextStyleSlot slot, bool transformed, BLVarCore* out) noexcept {
  const GpuImpl* self = self_of(impl);
  if (uint32_t(slot) > BL_CONTEXT_STYLE_SLOT_MAX_VALUE) { bl_var_assign_null(out); return BL_ERROR_INVALID_VALUE; }
  const BLVar& v = self->cur.style[slot];
  if (transformed && (v.is_gradient() || v.is_pattern())) return kNotImplemented;
  return bl_var_assign_weak(out, &v);
}

BLResult BL_CDECL v_set_style(BLContextImpl* impl, BLContextStyleSlot slot, const BLObjectCore* style,
                              BLContextStyleTransformMode mode) noexcept {
  SELF;
  if (uint32_t(slot) > BL_CONTEXT_STYLE_SLOT_MAX_VALUE) return BL_ERROR_INVALID_VALUE;
  if (mode != BL_CONTEXT_STYLE_TRANSFORM_MODE_USER) return kNotImplemented;
  BL_PROPAGATE(set_style_object(self, uint32_t(slot), style));
  bl_var_assign_weak(&self->cur.style[slot], style);
  self->cur.st.style_type[slot] = uint8_t(bl_var_get_type(style));
  return BL_SUCCESS;
}

BLResult BL_CDECL v_set_style_rgba32(BLContextImpl* impl, BLContextStyleSlot slot, uint32_t c) noexcept {
  SELF;
  if (uint32_t(slot) > BL_CONTEXT_STYLE_SLOT_MAX_VALUE) return BL_ERROR_INVALID_VALUE;
  BL_PROPAGATE(slot ? blgpu_context_set_stroke_style_rgba32(self->gpu, c) : blgpu_context_set_fill_style_rgba32(self->gpu, c));
  bl_var_assign_rgba32(&self->cur.style[slot], c);
  self->cur.st.style_type[slot] = uint8_t(BL_OBJECT_TYPE_RGBA32);
  return BL_SUCCESS;
}

BLResult BL_CDECL v_set_style_rgba(BLContextImpl*, BLContextStyleSlot, const BLRgba*) noexcept { return kNotImplemented; }
BLResult BL_CDECL v_set_style_rgba64(BLContextImpl*, BLContextStyleSlot, uint64_t) noexcept { return kNotImplemented; }
BLResult BL_CDECL v_disable_style(BLContextImpl*, BLContextStyleSlot) noexcept { return kNotImplemented; }
BLResult BL_CDECL v_swap_styles(BLContextImpl*, BLContextStyleSwapMode) noexcept { return kNotImplemented; }

BLResult BL_CDECL v_set_style_alpha(BLContextImpl* impl, BLContextStyleSlot slot, double alpha) noexcept {
  SELF;
  if (uint32_t(slot) > BL_CONTEXT_STYLE_SLOT_MAX_VALUE) return BL_ERROR_INVALID_VALUE;
  BL_PROPAGATE(slot ? blgpu_context_set_stroke_alpha(self->gpu, alpha) : blgpu_context_set_fill_alpha(self->gpu, alpha));
  self->cur.st.style_alpha[slot] = alpha;
  return BL_SUCCESS;
}

BLResult BL_CDECL v_set_global_alpha(BLContextImpl* impl, double alpha) noexcept {
  SELF;
  BL_PROPAGATE(blgpu_context_set_global_alpha(self->gpu, alpha));
  self->cur.st.global_alpha = alpha;
  return BL_SUCCESS;
}

BLResult BL_CDECL v_set_comp_op(BLContextImpl* impl, BLCompOp op) noexcept {
  SELF;
  BL_PROPAGATE(blgpu_context_set_comp_op(self->gpu, uint32_t(op)));
  self->cur.st.comp_op = uint8_t(op);
  return BL_SUCCESS;
}

BLResult BL_CDECL v_set_fill_rule(BLContextImpl* impl, BLFillRule rule) noexcept {
  SELF;
  BL_PROPAGATE(blgpu_context_set_fill_rule(self->gpu, uint32_t(rule)));
  self->cur.st.fill_rule = uint8_t(rule);
  return BL_SUCCESS;
}

BLResult BL_CDECL v_set_stroke_width(BLContextImpl* impl, double w) noexcept {
  SELF; BL_PROPAGATE(blgpu_context_set_stroke_width(self->gpu, w)); self->cur.st.stroke_options.width = w; return BL_SUCCESS;
}
BLResult BL_CDECL v_set_stroke_miter_limit(BLContextImpl* impl, double m) noexcept {
  SELF; BL_PROPAGATE(blgpu_context_set_stroke_miter_limit(self->gpu, m)); self->cur.st.stroke_options.miter_limit = m; return BL_SUCCESS;
}
BLResult BL_CDECL v_set_stroke_cap(BLContextImpl* impl, BLStrokeCapPosition pos, BLStrokeCap cap) noexcept {
  SELF;
  BL_PROPAGATE(blgpu_context_set_stroke_cap(self->gpu, uint32_t(pos), uint32_t(cap)));
  self->cur.st.stroke_options.caps[pos] = uint8_t(cap);
  return BL_SUCCESS;
}
BLResult BL_CDECL v_set_stroke_caps(BLContextImpl* impl, BLStrokeCap cap) noexcept {
  SELF;
  BL_PROPAGATE(blgpu_context_set_stroke_caps(self->gpu, uint32_t(cap)));
  self->cur.st.stroke_options.start_cap = self->cur.st.stroke_options.end_cap = uint8_t(cap);
  return BL_SUCCESS;
}
BLResult BL_CDECL v_set_stroke_join(BLContextImpl* impl, BLStrokeJoin join) noexcept {
  SELF; BL_PROPAGATE(blgpu_context_set_stroke_join(self->gpu, uint32_t(join))); self->cur.st.stroke_options.join = uint8_t(join); return BL_SUCCESS;
}
// The reference's stroker does not dash (blend2d/core/pathstroke.cpp); the dash settings are kept
// in the state only, as the raster context keeps them.
BLResult BL_CDECL v_set_stroke_dash_offset(BLContextImpl* impl, double off) noexcept {
  SELF; self->cur.st.stroke_options.dash_offset = off; return BL_SUCCESS;
}
BLResult BL_CDECL v_set_stroke_dash_array(BLContextImpl* impl, const BLArrayCore* a) noexcept {
  SELF; return bl_array_assign_weak(&self->cur.st.stroke_options.dash_array, a);
}
BLResult BL_CDECL v_set_stroke_transform_order(BLContextImpl* impl, BLStrokeTransformOrder order) noexcept {
  SELF;
  BL_PROPAGATE(blgpu_context_set_stroke_transform_order(self->gpu, uint32_t(order)));
  self->cur.st.stroke_options.transform_order = uint8_t(order);
  return BL_SUCCESS;
}
BLResult BL_CDECL v_set_stroke_options(BLContextImpl* impl, const BLStrokeOptionsCore* o) noexcept {
  SELF;
  BL_PROPAGATE(blgpu_context_set_stroke_width(self->gpu, o->width));
  BL_PROPAGATE(blgpu_context_set_stroke_miter_limit(self->gpu, o->miter_limit));
  BL_PROPAGATE(blgpu_context_set_stroke_cap(self->gpu, BL_STROKE_CAP_POSITION_START, o->start_cap));
  BL_PROPAGATE(blgpu_context_set_stroke_cap(self->gpu, BL_STROKE_CAP_POSITION_END, o->end_cap));
  BL_PROPAGATE(blgpu_context_set_stroke_join(self->gpu, o->join));
  BL_PROPAGATE(blgpu_context_set_stroke_transform_order(self->gpu, o->transform_order));
  static_cast<BLStrokeOptions&>(self->cur.st.stroke_options) = static_cast<const BLStrokeOptions&>(*o);
  return BL_SUCCESS;
}

// Clipping is not supported: the canvas is the clip box.
BLResult BL_CDECL v_clip_to_rect_i(BLContextImpl*, const BLRectI*) noexcept { return kNotImplemented; }
BLResult BL_CDECL v_clip_to_rect_d(BLContextImpl*, const BLRect*) noexcept { return kNotImplemented; }
BLResult BL_CDECL v_restore_clipping(BLContextImpl*) noexcept { return kNotImplemented; }

BLResult BL_CDECL v_clear_all(BLContextImpl* impl) noexcept { SELF; return blgpu_context_clear_all(self->gpu); }
BLResult BL_CDECL v_clear_recti(BLContextImpl*, const BLRectI*) noexcept { return kNotImplemented; }
BLResult BL_CDECL v_clear_rectd(BLContextImpl*, const BLRect*) noexcept { return kNotImplemented; }

BLResult BL_CDECL v_fill_all(BLContextImpl* impl) noexcept { SELF; return blgpu_context_fill_all(self->gpu); }
BLResult BL_CDECL v_fill_all_rgba32(BLContextImpl* impl, uint32_t c) noexcept {
  SELF; return with_style_rgba32(self, 0, c, [&] { return blgpu_context_fill_all(self->gpu); });
}
BLResult BL_CDECL v_fill_all_ext(BLContextImpl* impl, const BLObjectCore* s) noexcept {
  SELF; return with_style_object(self, 0, s, [&] { return blgpu_context_fill_all(self->gpu); });
}

BLResult BL_CDECL v_fill_geometry(BLContextImpl* impl, BLGeometryType t, const void* d) noexcept { SELF; return geometry_(self, false, t, d); }
BLResult BL_CDECL v_fill_geometry_rgba32(BLContextImpl* impl, BLGeometryType t, const void* d, uint32_t c) noexcept {
  SELF; return with_style_rgba32(self, 0, c, [&] { return geometry_(self, false, t, d); });
}
BLResult BL_CDECL v_fill_geometry_ext(BLContextImpl* impl, BLGeometryType t, const void* d, const BLObjectCore* s) noexcept {
  SELF; return with_style_object(self, 0, s, [&] { return geometry_(self, false, t, d); });
}

BLResult BL_CDECL v_fill_text_op_d(BLContextImpl* impl, const BLPoint* o, const BLFontCore* f, BLContextRenderTextOp op, const void* d) noexcept {
  SELF; return fill_text_(self, o, f, op, d);
}
BLResult BL_CDECL v_fill_text_op_d_rgba32(BLContextImpl* impl, const BLPoint* o, const BLFontCore* f, BLContextRenderTextOp op, const void* d, uint32_t c) noexcept {
  SELF; return with_style_rgba32(self, 0, c, [&] { return fill_text_(self, o, f, op, d); });
}
BLResult BL_CDECL v_fill_text_op_d_ext(BLContextImpl* impl, const BLPoint* o, const BLFontCore* f, BLContextRenderTextOp op, const void* d, const BLObjectCore* s) noexcept {
  SELF; return with_style_object(self, 0, s, [&] { return fill_text_(self, o, f, op, d); });
}
BLResult BL_CDECL v_fill_text_op_i(BLContextImpl* impl, const BLPointI* o, const BLFontCore* f, BLContextRenderTextOp op, const void* d) noexcept {
  const BLPoint od(*o); return v_fill_text_op_d(impl, &od, f, op, d);
}
BLResult BL_CDECL v_fill_text_op_i_rgba32(BLContextImpl* impl, const BLPointI* o, const BLFontCore* f, BLContextRenderTextOp op, const void* d, uint32_t c) noexcept {
  const BLPoint od(*o); return v_fill_text_op_d_rgba32(impl, &od, f, op, d, c);
}
BLResult BL_CDECL v_fill_text_op_i_ext(BLContextImpl* impl, const BLPointI* o, const BLFontCore* f, BLContextRenderTextOp op, const void* d, const BLObjectCore* s) noexcept {
  const BLPoint od(*o); return v_fill_text_op_d_ext(impl, &od, f, op, d, s);
}

BLResult BL_CDECL v_fill_mask_i(BLContextImpl* impl, const BLPointI* o, const BLImageCore* m, const BLRectI* a) noexcept {
  SELF; return fill_mask_(self, o->x, o->y, true, m, a);
}
BLResult BL_CDECL v_fill_mask_i_rgba32(BLContextImpl* impl, const BLPointI* o, const BLImageCore* m, const BLRectI* a, uint32_t c) noexcept {
  SELF; return with_style_rgba32(self, 0, c, [&] { return fill_mask_(self, o->x, o->y, true, m, a); });
}
BLResult BL_CDECL v_fill_mask_i_ext(BLContextImpl* impl, const BLPointI* o, const BLImageCore* m, const BLRectI* a, const BLObjectCore* s) noexcept {
  SELF; return with_style_object(self, 0, s, [&] { return fill_mask_(self, o->x, o->y, true, m, a); });
}
BLResult BL_CDECL v_fill_mask_d(BLContextImpl* impl, const BLPoint* o, const BLImageCore* m, const BLRectI* a) noexcept {
  SELF; return fill_mask_(self, o->x, o->y, false, m, a);
}
BLResult BL_CDECL v_fill_mask_d_rgba32(BLContextImpl* impl, const BLPoint* o, const BLImageCore* m, const BLRectI* a, uint32_t c) noexcept {
  SELF; return with_style_rgba32(self, 0, c, [&] { return fill_mask_(self, o->x, o->y, false, m, a); });
}
BLResult BL_CDECL v_fill_mask_d_ext(BLContextImpl* impl, const BLPoint* o, const BLImageCore* m, const BLRectI* a, const BLObjectCore* s) noexcept {
  SELF; return with_style_object(self, 0, s, [&] { return fill_mask_(self, o->x, o->y, false, m, a); });
}

BLResult BL_CDECL v_stroke_path_d(BLContextImpl* impl, const BLPoint* o, const BLPathCore* p) noexcept { SELF; return stroke_path_(self, o, p); }
BLResult BL_CDECL v_stroke_path_d_rgba32(BLContextImpl* impl, const BLPoint* o, const BLPathCore* p, uint32_t c) noexcept {
  SELF; return with_style_rgba32(self, 1, c, [&] { return stroke_path_(self, o, p); });
}
BLResult BL_CDECL v_stroke_path_d_ext(BLContextImpl* impl, const BLPoint* o, const BLPathCore* p, const BLObjectCore* s) noexcept {
  SELF; return with_style_object(self, 1, s, [&] { return stroke_path_(self, o, p); });
}

BLResult BL_CDECL v_stroke_geometry(BLContextImpl* impl, BLGeometryType t, const void* d) noexcept { SELF; return geometry_(self, true, t, d); }
BLResult BL_CDECL v_stroke_geometry_rgba32(BLContextImpl* impl, BLGeometryType t, const void* d, uint32_t c) noexcept {
  SELF; return with_style_rgba32(self, 1, c, [&] { return geometry_(self, true, t, d); });
}
BLResult BL_CDECL v_stroke_geometry_ext(BLContextImpl* impl, BLGeometryType t, const void* d, const BLObjectCore* s) noexcept {
  SELF; return with_style_object(self, 1, s, [&] { return geometry_(self, true, t, d); });
}

// Stroked text is not supported.
BLResult BL_CDECL v_stroke_text_op_d(BLContextImpl* impl, const BLPoint* o, const BLFontCore* f, BLContextRenderTextOp op, const void* d) noexcept {
  SELF; return stroke_text_(self, o, f, op, d);
}
BLResult BL_CDECL v_stroke_text_op_d_rgba32(BLContextImpl* impl, const BLPoint* o, const BLFontCore* f, BLContextRenderTextOp op, const void* d, uint32_t c) noexcept {
  SELF; return with_style_rgba32(self, 1, c, [&] { return stroke_text_(self, o, f, op, d); });
}
BLResult BL_CDECL v_stroke_text_op_d_ext(BLContextImpl* impl, const BLPoint* o, const BLFontCore* f, BLContextRenderTextOp op, const void* d, const BLObjectCore* s) noexcept {
  SELF; return with_style_object(self, 1, s, [&] { return stroke_text_(self, o, f, op, d); });
}
BLResult BL_CDECL v_stroke_text_op_i(BLContextImpl* impl, const BLPointI* o, const BLFontCore* f, BLContextRenderTextOp op, const void* d) noexcept {
  const BLPoint od(*o); return v_stroke_text_op_d(impl, &od, f, op, d);
}
BLResult BL_CDECL v_stroke_text_op_i_rgba32(BLContextImpl* impl, const BLPointI* o, const BLFontCore* f, BLContextRenderTextOp op, const void* d, uint32_t c) noexcept {
  const BLPoint od(*o); return v_stroke_text_op_d_rgba32(impl, &od, f, op, d, c);
}
BLResult BL_CDECL v_stroke_text_op_i_ext(BLContextImpl* impl, const BLPointI* o, const BLFontCore* f, BLContextRenderTextOp op, const void* d, const BLObjectCore* s) noexcept {
  const BLPoint od(*o); return v_stroke_text_op_d_ext(impl, &od, f, op, d, s);
}

#undef SELF

BLContextVirt make_virt() {
  BLContextVirt v;
  memset(static_cast<void*>(&v), 0, sizeof(v));
  v.base.destroy = destroy_impl;
  v.base.get_property = get_property_impl;
  v.base.set_property = set_property_impl;
  v.apply_transform_op = v_apply_transform_op;
  v.fill_rect_i = v_fill_rect_i; v.fill_rect_i_rgba32 = v_fill_rect_i_rgba32; v.fill_rect_i_ext = v_fill_rect_i_ext;
  v.fill_rect_d = v_fill_rect_d; v.fill_rect_d_rgba32 = v_fill_rect_d_rgba32; v.fill_rect_d_ext = v_fill_rect_d_ext;
  v.fill_path_d = v_fill_path_d; v.fill_path_d_rgba32 = v_fill_path_d_rgba32; v.fill_path_d_ext = v_fill_path_d_ext;
  v.blit_image_i = v_blit_image_i; v.blit_scaled_image_i = v_blit_scaled_image_i;
  v.flush = v_flush;
  v.save = v_save; v.restore = v_restore;
  v.user_to_meta = v_user_to_meta;
  v.set_hint = v_set_hint; v.set_hints = v_set_hints;
  v.set_flatten_mode = v_set_flatten_mode; v.set_flatten_tolerance = v_set_flatten_tolerance;
  v.set_approximation_options = v_set_approximation_options;
  v.get_style = v_get_style; v.set_style = v_set_style; v.set_style_rgba = v_set_style_rgba;
  v.set_style_rgba32 = v_set_style_rgba32; v.set_style_rgba64 = v_set_style_rgba64;
  v.disable_style = v_disable_style; v.set_style_alpha = v_set_style_alpha; v.swap_styles = v_swap_styles;
  v.set_global_alpha = v_set_global_alpha; v.set_comp_op = v_set_comp_op; v.set_fill_rule = v_set_fill_rule;
  v.set_stroke_width = v_set_stroke_width; v.set_stroke_miter_limit = v_set_stroke_miter_limit;
  v.set_stroke_cap = v_set_stroke_cap; v.set_stroke_caps = v_set_stroke_caps; v.set_stroke_join = v_set_stroke_join;
  v.set_stroke_dash_offset = v_set_stroke_dash_offset; v.set_stroke_dash_array = v_set_stroke_dash_array;
  v.set_stroke_transform_order = v_set_stroke_transform_order; v.set_stroke_options = v_set_stroke_options;
  v.clip_to_rect_i = v_clip_to_rect_i; v.clip_to_rect_d = v_clip_to_rect_d; v.restore_clipping = v_restore_clipping;
  v.clear_all = v_clear_all; v.clear_recti = v_clear_recti; v.clear_rectd = v_clear_rectd;
  v.fill_all = v_fill_all; v.fill_all_rgba32 = v_fill_all_rgba32; v.fill_all_ext = v_fill_all_ext;
  v.fill_geometry = v_fill_geometry; v.fill_geometry_rgba32 = v_fill_geometry_rgba32; v.fill_geometry_ext = v_fill_geometry_ext;
  v.fill_text_op_i = v_fill_text_op_i; v.fill_text_op_i_rgba32 = v_fill_text_op_i_rgba32; v.fill_text_op_i_ext = v_fill_text_op_i_ext;
  v.fill_text_op_d = v_fill_text_op_d; v.fill_text_op_d_rgba32 = v_fill_text_op_d_rgba32; v.fill_text_op_d_ext = v_fill_text_op_d_ext;
  v.fill_mask_i = v_fill_mask_i; v.fill_mask_i_rgba32 = v_fill_mask_i_rgba32; v.fill_mask_i_ext = v_fill_mask_i_ext;
  v.fill_mask_d = v_fill_mask_d; v.fill_mask_d_Rgba32 = v_fill_mask_d_rgba32; v.fill_mask_d_ext = v_fill_mask_d_ext;
  v.stroke_path_d = v_stroke_path_d; v.stroke_path_d_rgba32 = v_stroke_path_d_rgba32; v.stroke_path_d_ext = v_stroke_path_d_ext;
  v.stroke_geometry = v_stroke_geometry; v.stroke_geometry_rgba32 = v_stroke_geometry_rgba32; v.stroke_geometry_ext = v_stroke_geometry_ext;
  v.stroke_text_op_i = v_stroke_text_op_i; v.stroke_text_op_i_rgba32 = v_stroke_text_op_i_rgba32; v.stroke_text_op_i_ext = v_stroke_text_op_i_ext;
  v.stroke_text_op_d = v_stroke_text_op_d; v.stroke_text_op_d_rgba32 = v_stroke_text_op_d_rgba32; v.stroke_text_op_d_ext = v_stroke_text_op_d_ext;
  v.blit_image_d = v_blit_image_d; v.blit_scaled_image_d = v_blit_scaled_image_d;
  return v;
}

const BLContextVirt g_virt = make_virt();

// Process-wide runtimes for contexts begun without one: per device and LUT builder, kept until exit.
BLGpuRuntime* shared_runtime(int32_t device, uint32_t lut_variant, BLResult& err) {
  static std::mutex lock;
  static std::vector<std::pair<uint64_t, BLGpuRuntime*>> runtimes;
  const uint64_t key = (uint64_t(uint32_t(device)) << 32) | lut_variant;
  std::lock_guard<std::mutex> g(lock);
  for (auto& kv : runtimes)
    if (kv.first == key) return kv.second;
  BLGpuRuntimeCreateInfo ci{};
  ci.device = device;
  ci.lut_variant = lut_variant;
  BLGpuRuntime* rt = nullptr;
  err = blgpu_runtime_create(&rt, &ci);
  if (err) return nullptr;
  runtimes.emplace_back(key, rt);
  return rt;
}

}  // namespace

extern "C" const BLContextVirt* blgpu_blcontext_virt(void) { return &g_virt; }

extern "C" BLResult blgpu_blcontext_begin(BLContextCore* self, BLImageCore* image, const BLGpuContextCreateInfo* info) {
  if (!self || !image) return BL_ERROR_INVALID_VALUE;
  BLImageData d;
  BL_PROPAGATE(bl_image_make_mutable(image, &d));
  if (d.size.w <= 0 || d.size.h <= 0) return BL_ERROR_INVALID_VALUE;
  if (d.format != BL_FORMAT_PRGB32 && d.format != BL_FORMAT_XRGB32 && d.format != BL_FORMAT_A8) return kNotImplemented;

  BLResult err = BL_SUCCESS;
  BLGpuRuntime* rt = info && info->runtime ? info->runtime
                                           : shared_runtime(info ? info->device : 0, info ? info->lut_variant : BLGPU_LUT_SSE2, err);
  if (!rt) return err ? err : BL_ERROR_INVALID_STATE;

  BLContextCore fresh;
  BL_PROPAGATE(bl_object_alloc_impl_aligned(&fresh, BLObjectInfo::from_type_with_marker(BL_OBJECT_TYPE_CONTEXT).bits,
                                            sizeof(GpuImpl), 64));
  GpuImpl* impl = new (fresh._d.impl) GpuImpl();
  impl->virt = &g_virt;
  impl->state = &impl->cur.st;
  impl->context_type = BL_CONTEXT_TYPE_RASTER;
  init_state(impl->cur.st, image, d.size.w, d.size.h);
  bl_var_assign_rgba32(&impl->cur.style[0], 0xFF000000u);
  bl_var_assign_rgba32(&impl->cur.style[1], 0xFF000000u);
  impl->image.assign(static_cast<const BLImage&>(*image));

  BLGpuImage gi{d.pixel_data, d.stride, d.size.w, d.size.h, d.format, 0};
  BLResult r = blgpu_context_create(&impl->gpu, rt);
  if (r == BL_SUCCESS) r = blgpu_context_begin(impl->gpu, &gi);
  if (r != BL_SUCCESS) {
    destroy_impl(impl);
    return r;
  }
  return bl_context_assign_move(self, &fresh);
}
