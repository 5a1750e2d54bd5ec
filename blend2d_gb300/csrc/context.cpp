// context.cpp - the rendering-context front end and the C ABI (include/blgpu.h).
//
// BLGpuContext keeps the reference's synchronous context state (comp-op, fill rule, alphas,
// hints, user/final transforms, fill style, save/restore stack) and turns every fill call into a
// device command exactly where the reference would dispatch a fill to its pipeline:
//   state & alpha      blend2d/raster/rastercontext.cpp:1805-1833, :1920-2056, :4380-4415
//   transforms         blend2d/raster/rastercontext.cpp:740-800
//   style resolution   blend2d/raster/rastercontext.cpp:363-494, :572-695, :1231-1453
//   comp-op simplify   blend2d/core/compopsimplifyimpl_p.h:86-162
//   fill dispatch      blend2d/raster/rastercontext.cpp:2633-2990, :3317-3500
// Commands accumulate in a frame; flush(SYNC) / end() runs the frame's device pipeline.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <condition_variable>
#include <memory>
#include <mutex>
#include <thread>
#include <new>
#include <vector>

#include "blgpu.h"
#include "blgpu_stream.h"
#include "frontend.h"
#include "noalloc.h"
#include "runtime.h"
#include "stroke.h"

using namespace blgpu;

// A frame handed to the runtime's submission thread by an asynchronous flush, with the pattern
// pixels its stream records brought along.
struct AsyncSlot {
  Frame frame;
  std::deque<std::vector<uint32_t>> images;
  bool in_flight = false;                    // guarded by BLGpuRuntime::queue_lock
  BLGpuResult result = BLGPU_SUCCESS;
};

struct BLGpuRuntime {
  Runtime rt;
  Frame batch_frame;               // reused by blgpu_render_batch (its page-locked arrays persist)
  std::vector<std::unique_ptr<Frame>> batch_parts;   // per recording thread of blgpu_render_batch
  std::mutex batch_lock;
  // One pipeline run at a time: the submission thread and every synchronous entry point that
  // touches `rt` hold it.
  std::mutex exec;
  // Asynchronous flushes: frames run in submission order by one thread, so a frame's canvas
  // upload always sees what the frames before it wrote back.
  std::mutex queue_lock;
  std::condition_variable queue_cv, done_cv;
  std::deque<AsyncSlot*> queue;
  std::thread worker;
  bool stopping = false;

  void submit(AsyncSlot* s) {
    std::lock_guard<std::mutex> g(queue_lock);
    s->in_flight = true;
    queue.push_back(s);
    if (!worker.joinable()) worker = std::thread([this] { work(); });
    queue_cv.notify_one();
  }
  // Waits until `s` is no longer in flight; returns (and clears) its result.
  BLGpuResult wait(AsyncSlot* s) {
    std::unique_lock<std::mutex> g(queue_lock);
    done_cv.wait(g, [&] { return !s->in_flight; });
    BLGpuResult r = s->result;
    s->result = BLGPU_SUCCESS;
    return r;
  }
  void work() {
    std::unique_lock<std::mutex> g(queue_lock);
    for (;;) {
      queue_cv.wait(g, [&] { return stopping || !queue.empty(); });
      if (queue.empty()) return;             // stopping, nothing left
      AsyncSlot* s = queue.front();
      queue.pop_front();
      g.unlock();
      BLGpuResult r;
      {
        std::lock_guard<std::mutex> e(exec);
        r = rt.run(s->frame);
      }
      g.lock();
      s->result = r;
      s->in_flight = false;
      done_cv.notify_all();
    }
  }
  void stop() {
    {
      std::lock_guard<std::mutex> g(queue_lock);
      stopping = true;
      queue_cv.notify_all();
    }
    if (worker.joinable()) worker.join();
  }
};

namespace {

constexpr uint32_t kCompOpSrcOver = 0;
constexpr uint32_t kCompOpSrcCopy = 1;
constexpr uint32_t kCompOpMaxValue = 28;        // BL_COMP_OP_MAX_VALUE
constexpr uint32_t kFillRuleMaxValue = 1;       // BL_FILL_RULE_MAX_VALUE
constexpr uint32_t kHintRenderingQuality = 0;   // BL_CONTEXT_HINT_*
constexpr uint32_t kHintGradientQuality = 1;
constexpr uint32_t kHintPatternQuality = 2;
constexpr uint32_t kGradientQualityDither = 2;
constexpr uint32_t kPatternQualityMaxValue = 1;

// A fill style as the context holds it: resolved fetch data plus what a frame must provide.
struct CtxStyle {
  HostStyle hs;
  bool has_image = false;
  BLGpuImage image{};
  uint64_t frame_gen = 0;       // frame generation the style was registered in
  uint32_t frame_index = 0;
  uint64_t frame_gen_x = 0;     // the same for its copy whose pattern fetches read XRGB32
  uint32_t frame_index_x = 0;
};

// BLFormat values a render target may have, with their bytes per pixel.
static bool target_format_ok(uint32_t f) {
  return f == BLGPU_FORMAT_PRGB32 || f == BLGPU_FORMAT_XRGB32 || f == BLGPU_FORMAT_A8;
}
static intptr_t format_bpp(uint32_t f) { return f == BLGPU_FORMAT_A8 ? 1 : 4; }

// A host or device render target: PRGB32, XRGB32 or A8, at most 65,535 px a side.
static bool valid_target(const BLGpuImage& im) {
  return target_format_ok(im.format) && im.width > 0 && im.height > 0 && im.width <= 65535 &&
         im.height <= 65535 && im.pixel_data && im.stride >= intptr_t(im.width) * format_bpp(im.format);
}

// SrcOver / SrcCopy simplified by the destination and source formats (CompOpSimplifyInfoImpl::
// src_over / src_copy, compopsimplifyimpl_p.h:86-162). False for DstCopy (nothing drawn); else
// `src_copy` and `xrgb_read`: the simplified source format is XRGB32, so a pattern fetcher reads
// every texel with its alpha byte set (PixelIO<..., XRGB32>, pipeline/reference/pixelgeneric_p.h).
// Solid and gradient fetchers do not look at the source format (fixedpiperuntime.cpp:250-270).
//   SrcOver: ZERO32 -> DstCopy; FRGB32 -> SrcCopy; XRGB32 -> SrcCopy of XRGB32; PRGB32 -> SrcOver.
//   SrcCopy: XRGB32 -> SrcCopy of XRGB32; PRGB32 into an XRGB32 target -> SrcCopy of XRGB32.
// An A8 target's simplifications (opaque alpha, transparent) give the alpha these do.
static bool simplify_comp_op(uint32_t dst_format, uint32_t op, int src_format, bool& src_copy, bool& xrgb_read) {
  xrgb_read = src_format == kFmtXRGB32;
  if (op == kCompOpSrcOver) {
    if (src_format == kFmtZERO32) return false;
    if (src_format == kFmtFRGB32 || xrgb_read) op = kCompOpSrcCopy;
  }
  else if (src_format == kFmtPRGB32 && dst_format == BLGPU_FORMAT_XRGB32) {
    xrgb_read = true;
  }
  src_copy = op == kCompOpSrcCopy;
  return true;
}

struct State {
  uint32_t comp_op = kCompOpSrcOver;
  uint32_t fill_rule = 0;
  double global_alpha = 1.0, fill_alpha = 1.0;
  uint32_t global_alpha_i = 255, fill_alpha_i = 255;
  uint32_t gradient_quality = 0, pattern_quality = 1;
  Mat user{1, 0, 0, 1, 0, 0};
  Mat final_t{1, 0, 0, 1, 0, 0};
  Mat final_fixed{256, 0, 0, 256, 0, 0};
  int final_type = kTTIdentity, final_fixed_type = kTTScale;
  bool integral_translation = true;
  int tx_i = 0, ty_i = 0;
  CtxStyle style;               // BL_CONTEXT_STYLE_SLOT_FILL
  CtxStyle stroke_style;        // BL_CONTEXT_STYLE_SLOT_STROKE
  double stroke_alpha = 1.0;
  uint32_t stroke_alpha_i = 255;
  StrokeParams stroke;
  uint64_t xform_gen = 0;       // frame generation of xform_index
  uint32_t xform_index = 0;
  uint64_t meta_xform_gen = 0;  // frame generation of meta_xform_index
  uint32_t meta_xform_index = 0;
};

}  // namespace

struct BLGpuContext {
  BLGpuRuntime* rt = nullptr;
  // Two recording buffers: while one frame renders asynchronously the next one is recorded.
  AsyncSlot slots[2];
  int cur = 0;
  Frame* frame = &slots[0].frame;
  std::deque<std::vector<uint32_t>>* stream_images = &slots[0].images;   // pattern pixels copied out of submitted streams
  bool bound = false;
  BLGpuImage target{};
  uint32_t canvas = 0;
  int w = 0, h = 0;
  State s;
  std::vector<State> stack;
  uint64_t clear_style_gen = 0;
  uint32_t clear_style_index = 0;

  void reset_state() {
    s = State{};
    stack.clear();
    on_transform_changed();
    style_solid(s.style.hs, 0xFF000000u);
    style_solid(s.stroke_style.hs, 0xFF000000u);
  }

  // rastercontext.cpp:741-800
  void on_transform_changed() {
    Mat id{1, 0, 0, 1, 0, 0};
    mat_multiply(s.final_t, s.user, id);
    s.final_fixed = s.final_t;
    s.final_fixed.m00 *= 256.0; s.final_fixed.m01 *= 256.0;
    s.final_fixed.m10 *= 256.0; s.final_fixed.m11 *= 256.0;
    s.final_fixed.m20 *= 256.0; s.final_fixed.m21 *= 256.0;
    s.final_type = mat_type(s.final_t);
    s.final_fixed_type = s.final_type > kTTScale ? s.final_type : int(kTTScale);
    s.integral_translation = false;
    s.xform_gen = 0;
    s.meta_xform_gen = 0;
    if (s.final_type <= kTTTranslate) {
      double mn = floor(double(INT32_MIN + 1) * 256.0);
      double mx = floor(double(INT32_MAX - 1 - (w > h ? w : h)) * 256.0);
      const Mat& ft = s.final_fixed;
      if (ft.m20 >= mn && ft.m20 <= mx && ft.m21 >= mn && ft.m21 <= mx) {
        int64_t tx64 = floor_to_int64(ft.m20), ty64 = floor_to_int64(ft.m21);
        if (((tx64 | ty64) & 0xFF) == 0) {
          s.tx_i = int(tx64 >> 8);
          s.ty_i = int(ty64 >> 8);
          s.integral_translation = true;
        }
      }
    }
  }

  // --- frame registration ---------------------------------------------------------------

  // The style's index in the frame; `xrgb_read`: the copy whose pattern fetches set the alpha byte.
  // Solid styles take the context's one solid entry: their colour travels in the command
  // (DevCmd::color, from Fill::color).
  uint32_t register_style(CtxStyle& cs, bool xrgb_read = false) {
    if (cs.hs.dev.fetch == kFetchSolid) return register_solid_style();
    xrgb_read = xrgb_read && cs.hs.dev.fetch >= kFetchPatAlignedPad;
    if (!xrgb_read && cs.frame_gen == frame->generation) return cs.frame_index;
    if (xrgb_read && cs.frame_gen_x == frame->generation) return cs.frame_index_x;
    DevStyle d = cs.hs.dev;
    d.src_or = xrgb_read ? 0xFF000000u : 0u;
    if (d.lut_size) {
      if (d.dither) frame->lut_words = (frame->lut_words + 1u) & ~1u;   // 8-byte aligned entries
      DevLutJob job{};
      job.style = uint32_t(frame->styles.size());
      job.stop_first = uint32_t(frame->stops.size());
      job.stop_count = uint32_t(cs.hs.stops.size());
      job.lut_offset = frame->lut_words;
      job.lut_size = d.lut_size;
      job.variant = d.dither ? uint32_t(kLut64) : rt->rt.lut_variant;
      frame->stops.append(cs.hs.stops.data(), cs.hs.stops.size());
      frame->lut_jobs.push_back(job);
      d.lut_offset = frame->lut_words;
      frame->lut_words += d.dither ? 2u * d.lut_size : d.lut_size;
    }
    if (cs.has_image) d.src_offset += frame->add_image(cs.image);
    frame->styles.push_back(d);
    if (xrgb_read) {
      cs.frame_gen_x = frame->generation;
      cs.frame_index_x = uint32_t(frame->styles.size() - 1);
    }
    else {
      cs.frame_gen = frame->generation;
      cs.frame_index = uint32_t(frame->styles.size() - 1);
    }
    return uint32_t(frame->styles.size() - 1);
  }

  // The frame entry of every solid fill of this context (and of clear_all / clear_rect, whose
  // colour is 0).
  uint32_t register_solid_style() {
    if (clear_style_gen == frame->generation) return clear_style_index;
    DevStyle d{};
    d.fetch = kFetchSolid;
    d.solid = 0;
    frame->styles.push_back(d);
    clear_style_gen = frame->generation;
    clear_style_index = uint32_t(frame->styles.size() - 1);
    return clear_style_index;
  }

  uint32_t register_xform() {
    if (s.xform_gen == frame->generation) return s.xform_index;
    DevXform x{};
    x.m[0] = s.final_fixed.m00; x.m[1] = s.final_fixed.m01;
    x.m[2] = s.final_fixed.m10; x.m[3] = s.final_fixed.m11;
    x.m[4] = s.final_fixed.m20; x.m[5] = s.final_fixed.m21;
    x.affine = s.final_fixed_type > kTTScale ? 1u : 0u;
    frame->xforms.push_back(x);
    s.xform_gen = frame->generation;
    s.xform_index = uint32_t(frame->xforms.size() - 1);
    return s.xform_index;
  }

  // The edge transform of a stroke in transform order BEFORE: the meta transform (identity) in
  // 24.8 with the final transform's origin (DirectStateAccessor::meta_transform_fixed,
  // rastercontext.cpp:179-182), a scale-type transform.
  uint32_t register_meta_xform() {
    if (s.meta_xform_gen == frame->generation) return s.meta_xform_index;
    DevXform x{};
    x.m[0] = 256.0; x.m[1] = 0.0; x.m[2] = 0.0; x.m[3] = 256.0;
    x.m[4] = s.final_fixed.m20; x.m[5] = s.final_fixed.m21;
    x.affine = 0u;
    frame->xforms.push_back(x);
    s.meta_xform_gen = frame->generation;
    s.meta_xform_index = uint32_t(frame->xforms.size() - 1);
    return s.meta_xform_index;
  }

  // A path drawn at an origin: the final (or, for strokes in transform order BEFORE, the meta)
  // transform's linear part with the origin mapped by the final transform as its translation
  // (fill_unclipped_path_with_origin, rastercontext.cpp:2813-2821; add_stroked_path_edges,
  // rastercontextops_p.h:95-121). origin == nullptr: the registered transform as is.
  uint32_t register_xform_at(const double* origin, bool meta) {
    if (!origin) return meta ? register_meta_xform() : register_xform();
    const Mat& t = s.final_fixed;
    DevXform x{};
    if (meta) { x.m[0] = 256.0; x.m[1] = 0.0; x.m[2] = 0.0; x.m[3] = 256.0; }
    else { x.m[0] = t.m00; x.m[1] = t.m01; x.m[2] = t.m10; x.m[3] = t.m11; }
    x.m[4] = origin[0] * t.m00 + origin[1] * t.m10 + t.m20;      // BLMatrix2D::map_point
    x.m[5] = origin[0] * t.m01 + origin[1] * t.m11 + t.m21;
    x.affine = (!meta && s.final_fixed_type > kTTScale) ? 1u : 0u;
    frame->xforms.push_back(x);
    return uint32_t(frame->xforms.size() - 1);
  }

  // Outlines already in the target's 24.8 space, as a font engine emits a glyph run under the
  // final transform (add_filled_glyph_run_edges, rastercontextops_p.h:68-93: the edge builder
  // takes them with the identity transform).
  uint32_t register_fixed_identity_xform() {
    DevXform x{};
    x.m[0] = 1.0; x.m[3] = 1.0;
    x.affine = 0u;
    frame->xforms.push_back(x);
    return uint32_t(frame->xforms.size() - 1);
  }

  // A resolved fill: the style's frame index, SrcCopy (else SrcOver), the fill alpha and, for a
  // solid style, its premultiplied colour.
  struct Fill { uint32_t style; bool src_copy; uint32_t alpha; uint32_t color = 0; };

  static uint32_t style_color(const CtxStyle& cs) { return cs.hs.dev.fetch == kFetchSolid ? cs.hs.dev.solid : 0u; }

  DevCmd& push_cmd(uint32_t kind, const Fill& f) {
    DevCmd c{};
    c.kind = kind;
    c.canvas = canvas;
    c.style = f.style;
    c.flags = f.src_copy ? 1u : 0u;
    c.alpha = f.alpha;
    c.color = f.color;
    frame->cmds.push_back(c);
    frame->canvases[canvas].cmd_count++;
    return frame->cmds.back();
  }

  // --- fill resolution --------------------------------------------------------------------

  // Returns false for a NOP fill or stroke (no alpha, no style, or a comp-op that simplifies to
  // DstCopy) of the fill (slot 0) or stroke (slot 1) style.
  bool resolve_fill(Fill& f, uint32_t slot = 0) {
    CtxStyle& cs = slot_style(slot);
    uint32_t alpha = slot ? s.stroke_alpha_i : s.fill_alpha_i;
    if (s.global_alpha_i == 0 || alpha == 0 || cs.hs.nop) return false;
    bool xrgb_read = false;
    if (!simplify_comp_op(target.format, s.comp_op, cs.hs.format, f.src_copy, xrgb_read)) return false;
    f.alpha = alpha;
    f.style = register_style(cs, xrgb_read);
    f.color = style_color(cs);
    return true;
  }

  void fill_box_a(const Fill& f, int x0, int y0, int x1, int y1) {
    DevCmd& c = push_cmd(kFillBoxA, f);
    c.box[0] = x0; c.box[1] = y0; c.box[2] = x1; c.box[3] = y1;
    c.fetch_y0 = y0;
  }

  // FillData::init_box_u_8bpc_24x8 (pipedefs_p.h:644-815): the fetcher starts at the first row
  // whose mask is not zero.
  void fill_clipped_box_f(const Fill& f, int x0, int y0, int x1, int y1) {
    if (((x0 | y0 | x1 | y1) & 0xFF) == 0) { fill_box_a(f, x0 >> 8, y0 >> 8, x1 >> 8, y1 >> 8); return; }
    uint32_t alpha = f.alpha;
    uint32_t ax0 = uint32_t(x0) >> 8, ay0 = uint32_t(y0) >> 8;
    uint32_t ax1 = uint32_t(x1 + 0xFF) >> 8, ay1 = uint32_t(y1 + 0xFF) >> 8;
    uint32_t fx0 = uint32_t(x0) & 0xFFu, fy0 = uint32_t(y0) & 0xFFu;
    uint32_t fx1 = (uint32_t(x1 - 1) & 0xFFu) + 1u, fy1 = (uint32_t(y1 - 1) & 0xFFu) + 1u;
    uint32_t w = ax1 - ax0, h = ay1 - ay0;
    fy0 = (h == 1 ? fy1 : 256u) - fy0;
    uint32_t fy0_a = fy0 * alpha, fy1_a = fy1 * alpha;
    uint32_t m_first, m_mid, m_last;
    if (w == 1) {
      uint32_t fw = fx1 - fx0;
      m_first = (fw * fy0_a) >> 16; m_mid = (fw * alpha) >> 8; m_last = (fw * fy1_a) >> 16;
    }
    else {
      m_first = fy0_a >> 8; m_mid = alpha; m_last = fy1_a >> 8;
    }
    uint32_t row_y0 = ay0, row_y1 = ay1;
    if (h == 1) {
      if (!m_first) return;
    }
    else {
      if (!m_first) row_y0++;
      if (!m_last) row_y1--;
      if (!(row_y0 < row_y1) || (w == 1 && m_mid == 0)) return;
    }
    DevCmd& c = push_cmd(kFillBoxU, f);
    c.box[0] = x0; c.box[1] = y0; c.box[2] = x1; c.box[3] = y1;
    c.fetch_y0 = int32_t(row_y0);
  }

  void fill_analytic(const Fill& f, const double* xy, const uint8_t* cmds, size_t n, uint32_t fill_rule,
                     uint32_t xform) {
    DevCmd& c = push_cmd(kFillAnalytic, f);
    c.flags |= fill_rule == 1 ? 2u : 0u;
    c.geom = cmds ? kGeomPath : kGeomPolygon;
    c.geom_first = uint32_t(frame->verts.size() / 2);
    c.geom_count = uint32_t(n);
    c.xform = xform;
    frame->verts.append(xy, 2 * n);
    if (cmds) frame->path_cmds.append(cmds, n);
    else frame->path_cmds.append_fill(n, uint8_t(0));
  }

  void fill_box_d(const Fill& f, double bx0, double by0, double bx1, double by1) {
    const Mat& t = s.final_fixed;
    if (s.final_fixed_type <= kTTSwap) {
      double x0 = bx0 * t.m00 + by0 * t.m10 + t.m20;
      double y0 = bx0 * t.m01 + by0 * t.m11 + t.m21;
      double x1 = bx1 * t.m00 + by1 * t.m10 + t.m20;
      double y1 = bx1 * t.m01 + by1 * t.m11 + t.m21;
      auto dmin = [](double a, double b) { return b < a ? b : a; };
      auto dmax = [](double a, double b) { return a < b ? b : a; };
      double mx0 = dmin(x0, x1), my0 = dmin(y0, y1), mx1 = dmax(x0, x1), my1 = dmax(y0, y1);
      double cx1 = double(w) * 256.0, cy1 = double(h) * 256.0;
      double ix0 = dmax(mx0, 0.0), iy0 = dmax(my0, 0.0), ix1 = dmin(mx1, cx1), iy1 = dmin(my1, cy1);
      if (!((ix0 < ix1) & (iy0 < iy1))) return;
      int ux0 = trunc_to_int(ix0), uy0 = trunc_to_int(iy0), ux1 = trunc_to_int(ix1), uy1 = trunc_to_int(iy1);
      if (ux0 >= ux1 || uy0 >= uy1) return;
      fill_clipped_box_f(f, ux0, uy0, ux1, uy1);
    }
    else {
      double poly[8] = {bx0, by0, bx1, by0, bx1, by1, bx0, by1};
      fill_analytic(f, poly, nullptr, 4, 1, register_xform());
    }
  }

  // --- API ---------------------------------------------------------------------------------

  BLGpuResult begin(const BLGpuImage* image) {
    if (!image || !valid_target(*image)) return BLGPU_ERROR_INVALID_VALUE;
    if (bound) { BLGpuResult r = end(); if (r) return r; }
    target = *image;
    w = image->width;
    h = image->height;
    bound = true;
    frame->clear();
    stream_images->clear();
    canvas = frame->add_canvas(target, true);
    reset_state();
    return BLGPU_SUCCESS;
  }

  // Waits for the frames this context submitted asynchronously; returns the first error.
  BLGpuResult wait_async() {
    BLGpuResult r0 = rt->wait(&slots[0]), r1 = rt->wait(&slots[1]);
    return r0 ? r0 : r1;
  }

  // Runs the recorded frame (canvas content uploaded unless the first command overwrites it)
  // after the ones submitted before it; returns the first error of any of them.
  BLGpuResult flush_frame() {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    BLGpuResult r = frame == &slots[cur].frame ? wait_async() : BLGPU_SUCCESS;
    if (!frame->cmds.empty()) {
      mark_uploads(*frame);
      BLGpuResult rr;
      {
        std::lock_guard<std::mutex> e(rt->exec);
        rr = rt->rt.run(*frame);
      }
      if (!r) r = rr;
    }
    frame->clear();
    stream_images->clear();
    canvas = frame->add_canvas(target, true);
    return r;
  }

  // Hands the recorded frame to the runtime's submission thread and returns; recording goes on in
  // the other buffer (after the frame that used it last has finished). An error of a frame run
  // this way is returned by a later flush.
  BLGpuResult flush_async() {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    if (frame != &slots[cur].frame) return flush_frame();   // an external frame (batch): run it now
    if (frame->cmds.empty()) return BLGPU_SUCCESS;
    mark_uploads(*frame);
    rt->submit(&slots[cur]);
    cur ^= 1;
    BLGpuResult r = rt->wait(&slots[cur]);
    frame = &slots[cur].frame;
    stream_images = &slots[cur].images;
    frame->clear();
    stream_images->clear();
    canvas = frame->add_canvas(target, true);
    if (r) pending_error = r;
    return BLGPU_SUCCESS;
  }
  BLGpuResult pending_error = BLGPU_SUCCESS;

  static void mark_uploads(Frame& fr) {
    for (size_t i = 0; i < fr.canvases.size(); i++) {
      const DevCanvas& cv = fr.canvases[i];
      if (!cv.cmd_count) continue;
      const DevCmd& c = fr.cmds[cv.cmd_first];
      bool overwrites = c.kind == kFillBoxA && (c.flags & 1u) && c.alpha == 255 && c.box[0] == 0 && c.box[1] == 0 &&
                        c.box[2] == cv.w && c.box[3] == cv.h;
      fr.targets[i].upload = !overwrites;
    }
  }

  BLGpuResult end() {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    BLGpuResult r = flush_frame();
    if (!r) r = pending_error;
    pending_error = BLGPU_SUCCESS;
    frame->clear();
    bound = false;
    return r;
  }

  BLGpuResult set_comp_op(uint32_t op) {
    if (op > kCompOpMaxValue) return BLGPU_ERROR_INVALID_VALUE;
    if (op > kCompOpSrcCopy) return BLGPU_ERROR_NOT_IMPLEMENTED;
    s.comp_op = op;
    return BLGPU_SUCCESS;
  }

  BLGpuResult set_fill_rule(uint32_t rule) {
    if (rule > kFillRuleMaxValue) return BLGPU_ERROR_INVALID_VALUE;
    s.fill_rule = rule;
    return BLGPU_SUCCESS;
  }

  BLGpuResult set_global_alpha(double a) {   // rastercontext.cpp:2000-2028
    if (isnan(a)) return BLGPU_ERROR_INVALID_VALUE;
    a = a < 0.0 ? 0.0 : (a > 1.0 ? 1.0 : a);
    double ia = a * 255.0;
    s.global_alpha = a;
    s.global_alpha_i = uint32_t(round_to_int(ia));
    s.fill_alpha_i = uint32_t(round_to_int(ia * s.fill_alpha));
    s.stroke_alpha_i = uint32_t(round_to_int(ia * s.stroke_alpha));
    return BLGPU_SUCCESS;
  }

  BLGpuResult set_stroke_alpha(double a) {   // set_style_alpha(STROKE) (rastercontext.cpp:1920-1939)
    if (isnan(a)) return BLGPU_ERROR_INVALID_VALUE;
    a = a < 0.0 ? 0.0 : (a > 1.0 ? 1.0 : a);
    s.stroke_alpha = a;
    s.stroke_alpha_i = uint32_t(round_to_int(s.global_alpha * 255.0 * a));
    return BLGPU_SUCCESS;
  }

  // Stroke options (rastercontext.cpp:2059-2165): values outside the enums are rejected.
  BLGpuResult set_stroke_width(double v) { s.stroke.width = v; return BLGPU_SUCCESS; }
  BLGpuResult set_stroke_miter_limit(double v) { s.stroke.miter_limit = v; return BLGPU_SUCCESS; }
  BLGpuResult set_stroke_join(uint32_t v) {
    if (v > 4u) return BLGPU_ERROR_INVALID_VALUE;
    s.stroke.join = v;
    return BLGPU_SUCCESS;
  }
  BLGpuResult set_stroke_cap(uint32_t position, uint32_t cap) {
    if (position > 1u || cap > 5u) return BLGPU_ERROR_INVALID_VALUE;
    (position ? s.stroke.end_cap : s.stroke.start_cap) = cap;
    return BLGPU_SUCCESS;
  }
  BLGpuResult set_stroke_transform_order(uint32_t v) {
    if (v > 1u) return BLGPU_ERROR_INVALID_VALUE;
    s.stroke.transform_order = v;
    return BLGPU_SUCCESS;
  }

  BLGpuResult set_fill_alpha(double a) {     // rastercontext.cpp:1920-1945
    if (isnan(a)) return BLGPU_ERROR_INVALID_VALUE;
    a = a < 0.0 ? 0.0 : (a > 1.0 ? 1.0 : a);
    s.fill_alpha = a;
    s.fill_alpha_i = uint32_t(round_to_int(s.global_alpha * 255.0 * a));
    return BLGPU_SUCCESS;
  }

  BLGpuResult set_hint(uint32_t hint, uint32_t value) {   // rastercontext.cpp:1805-1832
    switch (hint) {
      case kHintRenderingQuality:
        return value > 0 ? BLGPU_ERROR_INVALID_VALUE : BLGPU_SUCCESS;
      case kHintGradientQuality:
        if (value > kGradientQualityDither) return BLGPU_ERROR_INVALID_VALUE;
        s.gradient_quality = value;
        return BLGPU_SUCCESS;
      case kHintPatternQuality:
        if (value > kPatternQualityMaxValue) return BLGPU_ERROR_INVALID_VALUE;
        s.pattern_quality = value;
        return BLGPU_SUCCESS;
      default:
        return BLGPU_ERROR_INVALID_VALUE;
    }
  }

  BLGpuResult set_transform(const double* m) {
    if (!m) return BLGPU_ERROR_INVALID_VALUE;
    s.user = Mat{m[0], m[1], m[2], m[3], m[4], m[5]};
    on_transform_changed();
    return BLGPU_SUCCESS;
  }

  BLGpuResult reset_transform() {
    s.user = Mat{1, 0, 0, 1, 0, 0};
    on_transform_changed();
    return BLGPU_SUCCESS;
  }

  // A new style in a slot: the previous one's registration is dropped, its stop storage reused.
  static void reset_style_slot(CtxStyle& cs) {
    cs.has_image = false;
    cs.image = BLGpuImage{};
    cs.frame_gen = 0;
    cs.frame_index = 0;
    cs.frame_gen_x = 0;
    cs.frame_index_x = 0;
  }
  CtxStyle& slot_style(uint32_t slot) { return slot ? s.stroke_style : s.style; }

  BLGpuResult set_style_rgba32(uint32_t c, uint32_t slot = 0) {
    CtxStyle& cs = slot_style(slot);
    reset_style_slot(cs);
    style_solid(cs.hs, c);
    return BLGPU_SUCCESS;
  }

  BLGpuResult set_style_gradient(const BLGpuGradient* g, uint32_t slot = 0) {
    if (!g || g->type > 2 || g->extend_mode > 2 || (g->stop_count && !g->stops)) return BLGPU_ERROR_INVALID_VALUE;
    GradientDesc d;
    d.type = g->type;
    d.extend = g->extend_mode;
    memcpy(d.values, g->values, sizeof(d.values));
    d.stops = reinterpret_cast<const DevStop*>(g->stops);
    d.stop_count = g->stop_count;
    d.transform = g->transform;
    CtxStyle& cs = slot_style(slot);
    reset_style_slot(cs);
    // gradients are not dithered into A8 targets (rastercontext.cpp:456-458)
    style_gradient(cs.hs, d, s.final_t, target.format == BLGPU_FORMAT_A8 ? 0u : s.gradient_quality);
    return BLGPU_SUCCESS;
  }

  BLGpuResult set_style_pattern(const BLGpuPattern* p, uint32_t slot = 0) {
    if (!p || !p->image) return BLGPU_ERROR_INVALID_VALUE;
    const BLGpuImage& im = *p->image;
    if ((im.format != BLGPU_FORMAT_PRGB32 && im.format != BLGPU_FORMAT_XRGB32) || im.width < 0 || im.height < 0 ||
        (im.width && !im.pixel_data) || im.stride < intptr_t(im.width) * 4)
      return BLGPU_ERROR_INVALID_VALUE;
    if (p->extend_mode > 8) return BLGPU_ERROR_INVALID_VALUE;
    if (p->extend_mode > 2) return BLGPU_ERROR_NOT_IMPLEMENTED;   // complex (per-axis) extend modes
    if (p->area[2] > 0) {
      int64_t x = p->area[0], y = p->area[1], aw = p->area[2], ah = p->area[3];
      if (x < 0 || y < 0 || ah < 0 || x + aw > im.width || y + ah > im.height) return BLGPU_ERROR_INVALID_VALUE;
    }
    PatternDesc d;
    d.image = 0;
    d.img_w = im.width;
    d.img_h = im.height;
    memcpy(d.area, p->area, sizeof(d.area));
    d.extend = p->extend_mode;
    d.transform = p->transform;
    CtxStyle& cs = slot_style(slot);
    reset_style_slot(cs);
    style_pattern(cs.hs, d, s.pattern_quality, s.final_t);
    // fetch_data->extra.format is the image's (rastercontext.cpp:415)
    if (im.format == BLGPU_FORMAT_XRGB32) cs.hs.format = kFmtXRGB32;
    if (!cs.hs.nop) {
      cs.has_image = true;
      cs.image = im;
    }
    return BLGPU_SUCCESS;
  }

  BLGpuResult clear_all() {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    Fill f{register_solid_style(), true, 255};
    fill_box_a(f, 0, 0, w, h);
    return BLGPU_SUCCESS;
  }

  BLGpuResult fill_all() {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    Fill f;
    if (!resolve_fill(f)) return BLGPU_SUCCESS;
    fill_box_a(f, 0, 0, w, h);
    return BLGPU_SUCCESS;
  }

  BLGpuResult fill_rect_i(int32_t x, int32_t y, int32_t rw, int32_t rh) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    Fill f;
    if (!resolve_fill(f)) return BLGPU_SUCCESS;
    if (!s.integral_translation) {
      if ((rw <= 0) | (rh <= 0)) return BLGPU_SUCCESS;
      fill_box_d(f, double(x), double(y), double(x) + double(rw), double(y) + double(rh));
      return BLGPU_SUCCESS;
    }
    int64_t x0 = int64_t(x) + s.tx_i, y0 = int64_t(y) + s.ty_i;
    int64_t x1 = int64_t(rw) + x0, y1 = int64_t(rh) + y0;
    x0 = x0 < 0 ? 0 : x0; y0 = y0 < 0 ? 0 : y0;
    x1 = x1 > w ? w : x1; y1 = y1 > h ? h : y1;
    if ((x0 >= x1) | (y0 >= y1)) return BLGPU_SUCCESS;
    fill_box_a(f, int(x0), int(y0), int(x1), int(y1));
    return BLGPU_SUCCESS;
  }

  BLGpuResult fill_box(double x0, double y0, double x1, double y1) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    Fill f;
    if (!resolve_fill(f)) return BLGPU_SUCCESS;
    fill_box_d(f, x0, y0, x1, y1);
    return BLGPU_SUCCESS;
  }

  BLGpuResult fill_polygon(const double* xy, size_t n) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    if (n && !xy) return BLGPU_ERROR_INVALID_VALUE;
    if (n > 0x3FFFFFFFu) return BLGPU_ERROR_INVALID_VALUE;
    Fill f;
    if (!resolve_fill(f)) return BLGPU_SUCCESS;
    if (n < 3) return BLGPU_SUCCESS;
    fill_analytic(f, xy, nullptr, n, s.fill_rule, register_xform());
    return BLGPU_SUCCESS;
  }

  BLGpuResult fill_path(const uint8_t* cmds, const double* xy, size_t n, const double* origin = nullptr) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    if (n && (!xy || !cmds)) return BLGPU_ERROR_INVALID_VALUE;
    if (n > 0x3FFFFFFFu) return BLGPU_ERROR_INVALID_VALUE;
    Fill f;
    if (!resolve_fill(f)) return BLGPU_SUCCESS;
    if (n == 0) return BLGPU_SUCCESS;
    fill_analytic(f, xy, cmds, n, s.fill_rule, register_xform_at(origin, false));
    return BLGPU_SUCCESS;
  }

  // fill_unclipped_text<kSync> (rastercontext.cpp:3082-3110): glyph outlines in 24.8 space,
  // filled non-zero with the fill style.
  BLGpuResult fill_path_fixed(const uint8_t* cmds, const double* xy, size_t n) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    if (n && (!xy || !cmds)) return BLGPU_ERROR_INVALID_VALUE;
    if (n > 0x3FFFFFFFu) return BLGPU_ERROR_INVALID_VALUE;
    Fill f;
    if (!resolve_fill(f)) return BLGPU_SUCCESS;
    if (n == 0) return BLGPU_SUCCESS;
    fill_analytic(f, xy, cmds, n, 0u, register_fixed_identity_xform());
    return BLGPU_SUCCESS;
  }

  // --- strokes ----------------------------------------------------------------------------
  // stroke_unclipped_geometry / stroke_unclipped_path<kSync> (rastercontext.cpp:3180-3234) with
  // add_stroked_path_edges (rastercontextops_p.h:95-140): the path is recorded with its figures
  // and stroke options; the device strokes every figure into the command's outline, which is then
  // filled non-zero with the stroke style like an analytic fill's path.
  std::vector<uint32_t> stroke_ranges;
  std::vector<uint8_t> stroke_in_cmds;
  std::vector<double> stroke_in_xy, stroke_poly_xy;

  BLGpuResult stroke_path(const uint8_t* cmds, const double* xy, size_t n, const double* origin = nullptr) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    if (n && (!xy || !cmds)) return BLGPU_ERROR_INVALID_VALUE;
    if (n > 0x3FFFFFFFu) return BLGPU_ERROR_INVALID_VALUE;
    Fill f;
    if (n == 0 || !resolve_fill(f, 1)) return BLGPU_SUCCESS;
    stroke_ranges.clear();
    BLGpuResult r = stroke_figures(cmds, n, stroke_ranges);
    if (r) return r;
    if (stroke_ranges.empty()) return BLGPU_SUCCESS;
    uint32_t xform;
    if (s.stroke.transform_order != 0) {
      // BEFORE: the path is mapped by the user transform without its translation first
      // (DirectStateAccessor::user_transform, rastercontext.cpp:168-171).
      const Mat& u = s.user;
      stroke_in_xy.resize(2 * n);
      for (size_t i = 0; i < n; i++) {
        double x = xy[2 * i], y = xy[2 * i + 1];
        stroke_in_xy[2 * i] = x * u.m00 + y * u.m10 + 0.0;
        stroke_in_xy[2 * i + 1] = x * u.m01 + y * u.m11 + 0.0;
      }
      xy = stroke_in_xy.data();
      xform = register_xform_at(origin, true);
    }
    else {
      xform = register_xform_at(origin, false);
    }
    DevCmd& c = push_cmd(kFillAnalytic, f);   // non-zero
    c.geom = kGeomPath;
    c.geom_first = 0;                  // the outline's range is set on the device
    c.geom_count = 0;
    c.xform = xform;
    const uint32_t cmd_index = uint32_t(frame->cmds.size() - 1);
    const uint32_t base = uint32_t(frame->stroke_cmds.size());
    frame->stroke_cmds.append(cmds, n);
    frame->stroke_xy.append(xy, 2 * n);
    DevStrokeParams sp{s.stroke.width, s.stroke.miter_limit, s.stroke.join, s.stroke.start_cap, s.stroke.end_cap, 0u};
    const uint32_t param = uint32_t(frame->stroke_params.size());
    frame->stroke_params.push_back(sp);
    const uint32_t figs = uint32_t(stroke_ranges.size() / 2);
    for (uint32_t k = 0; k < figs; k++)
      frame->stroke_figs.push_back(DevStrokeFig{base + stroke_ranges[2 * k], base + stroke_ranges[2 * k + 1], cmd_index,
                                                k == 0 ? figs : 0u, param});
    return BLGPU_SUCCESS;
  }

  // BLPath::add_geometry (path.cpp:1335-1660, direction CW) for the simple geometry types.
  BLGpuResult stroke_poly(const double* xy, size_t n, bool closed) {
    if (n && !xy) return BLGPU_ERROR_INVALID_VALUE;
    if (n > 0x3FFFFFFEu) return BLGPU_ERROR_INVALID_VALUE;
    if (n == 0) return bound ? BLGPU_SUCCESS : BLGPU_ERROR_INVALID_STATE;
    stroke_in_cmds.assign(n, uint8_t(1));
    stroke_in_cmds[0] = 0;
    stroke_poly_xy.assign(xy, xy + 2 * n);
    if (closed) {
      stroke_in_cmds.push_back(5);
      stroke_poly_xy.push_back(NAN);
      stroke_poly_xy.push_back(NAN);
    }
    return stroke_path(stroke_in_cmds.data(), stroke_poly_xy.data(), stroke_in_cmds.size());
  }

  BLGpuResult stroke_box(double x0, double y0, double x1, double y1) {
    const uint8_t c[5] = {0, 1, 1, 1, 5};
    const double v[10] = {x0, y0, x1, y0, x1, y1, x0, y1, NAN, NAN};
    return stroke_path(c, v, 5);
  }

  BLGpuResult stroke_line(double x0, double y0, double x1, double y1) {
    const uint8_t c[2] = {0, 1};
    const double v[4] = {x0, y0, x1, y1};
    return stroke_path(c, v, 2);
  }

  // --- image blits (rastercontext.cpp:3941-4160) -----------------------------------------------
  // A blit composites the image (or its area) with the global alpha only, through the blit
  // fetchers: aligned, fractional (bilinear or nearest by the pattern quality) or affine with
  // REFLECT extend, over a box fill.
  CtxStyle blit_style;

  static bool valid_image(const BLGpuImage* im) {
    return im && (im->format == BLGPU_FORMAT_PRGB32 || im->format == BLGPU_FORMAT_XRGB32) && im->width >= 0 && im->height >= 0 &&
           (im->width == 0 || im->pixel_data) && im->stride >= intptr_t(im->width) * 4;
  }

  // check_image_area (rastercontext.cpp:2305-2319): false for an area outside the image.
  static bool image_area(const BLGpuImage& im, const int32_t* area, int out[4]) {
    out[0] = 0; out[1] = 0; out[2] = im.width; out[3] = im.height;
    if (area) {
      unsigned max_w = unsigned(im.width) - unsigned(area[0]);
      unsigned max_h = unsigned(im.height) - unsigned(area[1]);
      if ((max_w > unsigned(im.width)) | (unsigned(area[2]) > max_w) | (max_h > unsigned(im.height)) |
          (unsigned(area[3]) > max_h))
        return false;
      out[0] = area[0]; out[1] = area[1]; out[2] = area[2]; out[3] = area[3];
    }
    return true;
  }

  // resolve_blit_op (rastercontext.cpp:1331-1342): the comp-op simplified for the image's format,
  // the global alpha; false when the global alpha is zero.
  bool resolve_blit(Fill& f, const BLGpuImage& im) {
    if (s.global_alpha_i == 0 || blit_style.hs.nop) return false;
    bool xrgb_read = false;
    simplify_comp_op(target.format, s.comp_op, im.format == BLGPU_FORMAT_XRGB32 ? kFmtXRGB32 : kFmtPRGB32,
                     f.src_copy, xrgb_read);
    f.alpha = s.global_alpha_i;
    blit_style.has_image = true;
    blit_style.image = im;
    blit_style.frame_gen = 0;
    blit_style.frame_gen_x = 0;
    f.style = register_style(blit_style, xrgb_read);
    f.color = style_color(blit_style);
    return true;
  }

  BLGpuResult blit_image_d(double x, double y, const BLGpuImage* img, const int32_t* area) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    if (!valid_image(img)) return BLGPU_ERROR_INVALID_VALUE;
    int src[4];
    if (!image_area(*img, area, src)) return BLGPU_ERROR_INVALID_VALUE;
    if (s.global_alpha_i == 0) return BLGPU_SUCCESS;
    Fill f;
    if (s.final_type <= kTTTranslate) {
      const Mat& t = s.final_fixed;
      double sx = x * t.m00 + t.m20;
      double sy = y * t.m11 + t.m21;
      double cx1 = double(w) * 256.0, cy1 = double(h) * 256.0;
      double dx0 = sx < 0.0 ? 0.0 : sx;
      double dy0 = sy < 0.0 ? 0.0 : sy;
      double ex = sx + double(src[2]) * t.m00, ey = sy + double(src[3]) * t.m11;
      double dx1 = cx1 < ex ? cx1 : ex;
      double dy1 = cy1 < ey ? cy1 : ey;
      if (!((dx0 < dx1) & (dy0 < dy1))) return BLGPU_SUCCESS;
      int ix0 = trunc_to_int(dx0), iy0 = trunc_to_int(dy0), ix1 = trunc_to_int(dx1), iy1 = trunc_to_int(dy1);
      if (!((ix0 < ix1) & (iy0 < iy1))) return BLGPU_SUCCESS;
      int64_t fx = floor_to_int64(sx), fy = floor_to_int64(sy);
      if (!((fx | fy) & 0xFF)) {
        // pixel aligned: the source area follows the clipped destination box
        int x0 = ix0 >> 8, y0 = iy0 >> 8, x1 = (ix1 + 0xFF) >> 8, y1 = (iy1 + 0xFF) >> 8;
        int tx = int(fx >> 8), ty = int(fy >> 8);
        src[0] += x0 - tx; src[1] += y0 - ty;
        src[2] = x1 - x0; src[3] = y1 - y0;
        style_blit_aligned(blit_style.hs, 0, img->width, src, x0, y0);
      }
      else {
        style_blit_fx_fy(blit_style.hs, 0, img->width, src, s.pattern_quality, fx, fy);
      }
      if (!resolve_blit(f, *img)) return BLGPU_SUCCESS;
      fill_clipped_box_f(f, ix0, iy0, ix1, iy1);
      return BLGPU_SUCCESS;
    }
    Mat ft = s.final_t;
    ft.m20 += x * ft.m00 + y * ft.m10;       // BLMatrix2D::translate
    ft.m21 += x * ft.m01 + y * ft.m11;
    style_blit_affine(blit_style.hs, 0, img->width, src, s.pattern_quality, ft);
    if (!resolve_blit(f, *img)) return BLGPU_SUCCESS;
    fill_box_d(f, x, y, x + double(src[2]), y + double(src[3]));
    return BLGPU_SUCCESS;
  }

  BLGpuResult blit_image_i(int32_t x, int32_t y, const BLGpuImage* img, const int32_t* area) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    if (!valid_image(img)) return BLGPU_ERROR_INVALID_VALUE;
    if (!s.integral_translation) return blit_image_d(double(x), double(y), img, area);
    // translate_and_clip_rect_to_blit_i (rastercontext.cpp:922-990)
    int src[4];
    if (!image_area(*img, area, src)) return BLGPU_ERROR_INVALID_VALUE;
    int64_t dx = int64_t(x) + s.tx_i, dy = int64_t(y) + s.ty_i;
    int64_t x0 = dx, y0 = dy, x1 = x0 + src[2], y1 = y0 + src[3];
    x0 = x0 < 0 ? 0 : x0; y0 = y0 < 0 ? 0 : y0;
    x1 = x1 > w ? w : x1; y1 = y1 > h ? h : y1;
    if ((x0 >= x1) | (y0 >= y1)) return BLGPU_SUCCESS;
    src[0] += int(x0 - dx); src[1] += int(y0 - dy);
    src[2] = int(x1 - x0); src[3] = int(y1 - y0);
    if (s.global_alpha_i == 0) return BLGPU_SUCCESS;
    style_blit_aligned(blit_style.hs, 0, img->width, src, int(x0), int(y0));
    Fill f;
    if (!resolve_blit(f, *img)) return BLGPU_SUCCESS;
    fill_box_a(f, int(x0), int(y0), int(x1), int(y1));
    return BLGPU_SUCCESS;
  }

  // blit_scaled_image_d / _i (rastercontext.cpp:4073-4160)
  BLGpuResult blit_scaled_image(double rx, double ry, double rw, double rh, const BLGpuImage* img, const int32_t* area,
                                bool integral) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    if (!valid_image(img)) return BLGPU_ERROR_INVALID_VALUE;
    int src[4];
    if (!image_area(*img, area, src)) return BLGPU_ERROR_INVALID_VALUE;
    if ((rw == double(src[2])) & (rh == double(src[3])))
      return integral ? blit_image_i(int32_t(rx), int32_t(ry), img, area) : blit_image_d(rx, ry, img, area);
    if (s.global_alpha_i == 0) return BLGPU_SUCCESS;
    Mat sc{rw / double(src[2]), 0.0, 0.0, rh / double(src[3]), rx, ry};
    Mat ft;
    mat_multiply(ft, sc, s.final_t);
    style_blit_affine(blit_style.hs, 0, img->width, src, s.pattern_quality, ft);
    Fill f;
    if (!resolve_blit(f, *img)) return BLGPU_SUCCESS;
    fill_box_d(f, rx, ry, rx + rw, ry + rh);
    return BLGPU_SUCCESS;
  }

  // --- masked fills (rastercontext.cpp:3679-3790) -------------------------------------------
  // The fill style composited through an A8 mask over a pixel-aligned box (fill_box_masked_a):
  // per pixel the mask byte, times the fill alpha below 255. As in the reference, only a pixel
  // aligned mask is supported; any other placement returns BLGPU_ERROR_NOT_IMPLEMENTED.
  static bool valid_mask(const BLGpuImage* im) {
    return im && im->format == BLGPU_FORMAT_A8 && im->width >= 0 && im->height >= 0 &&
           (im->width == 0 || im->pixel_data) && im->stride >= intptr_t(im->width);
  }

  void record_mask(const Fill& f, int x0, int y0, int x1, int y1, const BLGpuImage& mask, int mx, int my) {
    const uint64_t words = frame->add_image(mask);
    const uint64_t off = words * 4u + uint64_t(uint32_t(my)) * uint32_t(mask.width) + uint32_t(mx);
    DevCmd& c = push_cmd(kFillMaskA, f);
    c.box[0] = x0; c.box[1] = y0; c.box[2] = x1; c.box[3] = y1;
    c.fetch_y0 = y0;
    c.geom_first = uint32_t(off);
    c.xform = uint32_t(off >> 32);
    c.geom_count = uint32_t(mask.width);
  }

  BLGpuResult fill_mask_d(double x, double y, const BLGpuImage* mask, const int32_t* area) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    if (!valid_mask(mask)) return BLGPU_ERROR_INVALID_VALUE;
    int src[4];
    if (!image_area(*mask, area, src)) return BLGPU_ERROR_INVALID_VALUE;
    Fill f;
    if (!resolve_fill(f)) return BLGPU_SUCCESS;
    if (s.final_type > kTTTranslate) return BLGPU_ERROR_NOT_IMPLEMENTED;
    // fill_unclipped_mask_d (rastercontext.cpp:3594-3676)
    const Mat& t = s.final_fixed;
    double sx = x * t.m00 + t.m20, sy = y * t.m11 + t.m21;
    double bx0 = sx < 0.0 ? 0.0 : sx, by0 = sy < 0.0 ? 0.0 : sy;
    double ex = sx + double(src[2]) * t.m00, ey = sy + double(src[3]) * t.m11;
    double cx1 = double(w) * 256.0, cy1 = double(h) * 256.0;
    double bx1 = cx1 < ex ? cx1 : ex, by1 = cy1 < ey ? cy1 : ey;
    if (!((bx0 < bx1) & (by0 < by1))) return BLGPU_SUCCESS;
    int64_t fx = floor_to_int64(sx), fy = floor_to_int64(sy);
    int ux0 = trunc_to_int(bx0), uy0 = trunc_to_int(by0), ux1 = trunc_to_int(bx1), uy1 = trunc_to_int(by1);
    if ((fx | fy) & 0xFF) return BLGPU_ERROR_NOT_IMPLEMENTED;
    int x0 = ux0 >> 8, y0 = uy0 >> 8, x1 = (ux1 + 0xFF) >> 8, y1 = (uy1 + 0xFF) >> 8;
    int tx = int(fx >> 8), ty = int(fy >> 8);
    if (((ux0 | uy0 | ux1 | uy1) & 0xFF) != 0) return BLGPU_ERROR_NOT_IMPLEMENTED;
    record_mask(f, x0, y0, x1, y1, *mask, src[0] + x0 - tx, src[1] + y0 - ty);
    return BLGPU_SUCCESS;
  }

  BLGpuResult fill_mask_i(int32_t x, int32_t y, const BLGpuImage* mask, const int32_t* area) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    if (!valid_mask(mask)) return BLGPU_ERROR_INVALID_VALUE;
    if (!s.integral_translation) return fill_mask_d(double(x), double(y), mask, area);
    int src[4];
    if (!image_area(*mask, area, src)) return BLGPU_ERROR_INVALID_VALUE;
    int64_t dx = int64_t(x) + s.tx_i, dy = int64_t(y) + s.ty_i;
    int64_t x0 = dx, y0 = dy, x1 = x0 + src[2], y1 = y0 + src[3];
    x0 = x0 < 0 ? 0 : x0; y0 = y0 < 0 ? 0 : y0;
    x1 = x1 > w ? w : x1; y1 = y1 > h ? h : y1;
    if ((x0 >= x1) | (y0 >= y1)) return BLGPU_SUCCESS;
    Fill f;
    if (!resolve_fill(f)) return BLGPU_SUCCESS;
    record_mask(f, int(x0), int(y0), int(x1), int(y1), *mask, src[0] + int(x0 - dx), src[1] + int(y0 - dy));
    return BLGPU_SUCCESS;
  }

  // --- shapes (fill_unclipped_geometry, rastercontext.cpp:2926-2980): the shape's path, filled
  // with the fill rule or stroked -------------------------------------------------------------
  std::vector<uint8_t> shape_cmds;
  std::vector<double> shape_xy;

  BLGpuResult fill_geometry(uint32_t type, const double* v) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    if (!v) return BLGPU_ERROR_INVALID_VALUE;
    if (!shape_path(type, v, shape_cmds, shape_xy)) return BLGPU_ERROR_NOT_IMPLEMENTED;
    return fill_path(shape_cmds.data(), shape_xy.data(), shape_cmds.size());
  }

  BLGpuResult stroke_geometry(uint32_t type, const double* v) {
    if (!bound) return BLGPU_ERROR_INVALID_STATE;
    if (!v) return BLGPU_ERROR_INVALID_VALUE;
    if (!shape_path(type, v, shape_cmds, shape_xy)) return BLGPU_ERROR_NOT_IMPLEMENTED;
    return stroke_path(shape_cmds.data(), shape_xy.data(), shape_cmds.size());
  }

  BLGpuResult save() { stack.push_back(s); return BLGPU_SUCCESS; }
  BLGpuResult restore() {
    if (stack.empty()) return BLGPU_ERROR_NO_STATES_TO_RESTORE;
    s = stack.back();
    stack.pop_back();
    return BLGPU_SUCCESS;
  }

  BLGpuResult submit_stream(const uint8_t* base, size_t size);

  // Stream payloads are read in place when 8-byte aligned (the normal case), else via scratch.
  std::vector<double> scratch_xy;
  std::vector<BLGpuGradientStop> scratch_stops;
  const double* aligned_doubles(const uint8_t* p, size_t count) {
    if (!(reinterpret_cast<uintptr_t>(p) & 7u)) return reinterpret_cast<const double*>(p);
    scratch_xy.resize(count);
    if (count) memcpy(scratch_xy.data(), p, count * sizeof(double));
    return scratch_xy.data();
  }
};

// Stream replay: the same record semantics as the context calls above.
BLGpuResult BLGpuContext::submit_stream(const uint8_t* base, size_t size) {
  if (!bound) return BLGPU_ERROR_INVALID_STATE;
  if (!base || size < sizeof(BLGpuStreamHeader)) return BLGPU_ERROR_INVALID_VALUE;
  BLGpuStreamHeader hdr;
  memcpy(&hdr, base, sizeof(hdr));
  if (hdr.magic != BLGPU_STREAM_MAGIC || hdr.version != BLGPU_STREAM_VERSION) return BLGPU_ERROR_INVALID_VALUE;
  if (int(hdr.width) != w || int(hdr.height) != h) return BLGPU_ERROR_INVALID_VALUE;
  // the stream was recorded for a target of this format (0 reads as PRGB32)
  if ((hdr.format ? hdr.format : uint32_t(BLGPU_FORMAT_PRGB32)) != target.format) return BLGPU_ERROR_INVALID_VALUE;
  size_t off = sizeof(hdr);
  std::vector<BLGpuImage> images(hdr.image_count);
  for (uint32_t i = 0; i < hdr.image_count; i++) {
    BLGpuStreamImage im;
    if (off + sizeof(im) > size) return BLGPU_ERROR_INVALID_VALUE;
    memcpy(&im, base + off, sizeof(im));
    off += sizeof(im);
    size_t n = size_t(im.width) * im.height;
    if (im.width > 65535 || im.height > 65535 || off + n * 4u > size) return BLGPU_ERROR_INVALID_VALUE;
    stream_images->emplace_back(n ? n : 1);
    memcpy(stream_images->back().data(), base + off, n * 4u);
    if (im.format != 0 && im.format != BLGPU_FORMAT_PRGB32 && im.format != BLGPU_FORMAT_XRGB32)
      return BLGPU_ERROR_INVALID_VALUE;
    images[i] = BLGpuImage{stream_images->back().data(), intptr_t(im.width) * 4, int32_t(im.width), int32_t(im.height),
                           im.format == BLGPU_FORMAT_XRGB32 ? uint32_t(BLGPU_FORMAT_XRGB32) : uint32_t(BLGPU_FORMAT_PRGB32), 0};
    off += (n * 4u + 7u) & ~size_t(7);
  }
  while (off + 8 <= size) {
    uint32_t op, len;
    memcpy(&op, base + off, 4);
    memcpy(&len, base + off + 4, 4);
    const uint8_t* p = base + off + 8;
    if (off + 8 + size_t(len) > size) return BLGPU_ERROR_INVALID_VALUE;
    off += 8 + size_t(len);
    if (op == BLGPU_OP_END) break;
    auto need = [&](size_t bytes) { return size_t(len) >= bytes; };
    BLGpuResult r = BLGPU_SUCCESS;
    switch (op) {
      case BLGPU_OP_SET_COMP_OP: { if (!need(4)) return BLGPU_ERROR_INVALID_VALUE; uint32_t v; memcpy(&v, p, 4); r = set_comp_op(v); break; }
      case BLGPU_OP_SET_FILL_RULE: { if (!need(4)) return BLGPU_ERROR_INVALID_VALUE; uint32_t v; memcpy(&v, p, 4); r = set_fill_rule(v); break; }
      case BLGPU_OP_SET_GLOBAL_ALPHA: { if (!need(8)) return BLGPU_ERROR_INVALID_VALUE; double a; memcpy(&a, p, 8); set_global_alpha(a); break; }
      case BLGPU_OP_SET_FILL_ALPHA: { if (!need(8)) return BLGPU_ERROR_INVALID_VALUE; double a; memcpy(&a, p, 8); set_fill_alpha(a); break; }
      case BLGPU_OP_SET_HINT: {
        if (!need(8)) return BLGPU_ERROR_INVALID_VALUE;
        uint32_t hh, v; memcpy(&hh, p, 4); memcpy(&v, p + 4, 4);
        r = set_hint(hh, v);
        break;
      }
      case BLGPU_OP_SET_TRANSFORM: { if (!need(48)) return BLGPU_ERROR_INVALID_VALUE; double m[6]; memcpy(m, p, 48); set_transform(m); break; }
      case BLGPU_OP_RESET_TRANSFORM: reset_transform(); break;
      case BLGPU_OP_STYLE_RGBA32: { if (!need(4)) return BLGPU_ERROR_INVALID_VALUE; uint32_t v; memcpy(&v, p, 4); set_style_rgba32(v); break; }
      case BLGPU_OP_STYLE_GRADIENT: case BLGPU_OP_STROKE_STYLE_GRADIENT: {
        BLGpuStreamGradient g;
        if (!need(sizeof(g))) return BLGPU_ERROR_INVALID_VALUE;
        memcpy(&g, p, sizeof(g));
        if (!need(sizeof(g) + size_t(g.stop_count) * sizeof(BLGpuStreamGradientStop))) return BLGPU_ERROR_INVALID_VALUE;
        const uint8_t* sp = p + sizeof(g);
        if (g.stop_count && (reinterpret_cast<uintptr_t>(sp) & 7u)) {
          scratch_stops.resize(g.stop_count);
          memcpy(scratch_stops.data(), sp, sizeof(BLGpuGradientStop) * g.stop_count);
          sp = reinterpret_cast<const uint8_t*>(scratch_stops.data());
        }
        BLGpuGradient gg;
        gg.type = g.type;
        gg.extend_mode = g.extend_mode;
        memcpy(gg.values, g.values, sizeof(gg.values));
        gg.stops = reinterpret_cast<const BLGpuGradientStop*>(sp);
        gg.stop_count = g.stop_count;
        gg.transform = g.has_transform ? g.transform : nullptr;
        r = set_style_gradient(&gg, op == BLGPU_OP_STROKE_STYLE_GRADIENT ? 1u : 0u);
        break;
      }
      case BLGPU_OP_STYLE_PATTERN: case BLGPU_OP_STROKE_STYLE_PATTERN: {
        BLGpuStreamPattern pt;
        if (!need(sizeof(pt))) return BLGPU_ERROR_INVALID_VALUE;
        memcpy(&pt, p, sizeof(pt));
        if (pt.image_index >= hdr.image_count) return BLGPU_ERROR_INVALID_VALUE;
        BLGpuPattern pp;
        pp.image = &images[pt.image_index];
        memcpy(pp.area, pt.area, sizeof(pp.area));
        pp.extend_mode = pt.extend_mode;
        pp.transform = pt.has_transform ? pt.transform : nullptr;
        r = set_style_pattern(&pp, op == BLGPU_OP_STROKE_STYLE_PATTERN ? 1u : 0u);
        break;
      }
      case BLGPU_OP_CLEAR_ALL: r = clear_all(); break;
      case BLGPU_OP_FILL_ALL: r = fill_all(); break;
      case BLGPU_OP_FILL_RECT_I: {
        if (!need(16)) return BLGPU_ERROR_INVALID_VALUE;
        int32_t q[4]; memcpy(q, p, 16);
        r = fill_rect_i(q[0], q[1], q[2], q[3]);
        break;
      }
      case BLGPU_OP_FILL_RECT_D: {
        if (!need(32)) return BLGPU_ERROR_INVALID_VALUE;
        double q[4]; memcpy(q, p, 32);
        r = fill_box(q[0], q[1], q[0] + q[2], q[1] + q[3]);
        break;
      }
      case BLGPU_OP_FILL_BOX_D: {
        if (!need(32)) return BLGPU_ERROR_INVALID_VALUE;
        double q[4]; memcpy(q, p, 32);
        r = fill_box(q[0], q[1], q[2], q[3]);
        break;
      }
      case BLGPU_OP_FILL_POLYGON_D: {
        if (!need(8)) return BLGPU_ERROR_INVALID_VALUE;
        uint32_t n; memcpy(&n, p, 4);
        if (!need(8 + size_t(n) * 16)) return BLGPU_ERROR_INVALID_VALUE;
        r = fill_polygon(aligned_doubles(p + 8, size_t(n) * 2), n);
        break;
      }
      case BLGPU_OP_FILL_PATH_D: {
        if (!need(8)) return BLGPU_ERROR_INVALID_VALUE;
        uint32_t n; memcpy(&n, p, 4);
        size_t cmd_bytes = (size_t(n) + 7u) & ~size_t(7);
        if (!need(8 + cmd_bytes + size_t(n) * 16)) return BLGPU_ERROR_INVALID_VALUE;
        r = fill_path(p + 8, aligned_doubles(p + 8 + cmd_bytes, size_t(n) * 2), n);
        break;
      }
      case BLGPU_OP_STROKE_STYLE_RGBA32: { if (!need(4)) return BLGPU_ERROR_INVALID_VALUE; uint32_t v; memcpy(&v, p, 4); set_style_rgba32(v, 1); break; }
      case BLGPU_OP_SET_STROKE_ALPHA: { if (!need(8)) return BLGPU_ERROR_INVALID_VALUE; double a; memcpy(&a, p, 8); set_stroke_alpha(a); break; }
      case BLGPU_OP_SET_STROKE_WIDTH: { if (!need(8)) return BLGPU_ERROR_INVALID_VALUE; double v; memcpy(&v, p, 8); set_stroke_width(v); break; }
      case BLGPU_OP_SET_STROKE_MITER_LIMIT: { if (!need(8)) return BLGPU_ERROR_INVALID_VALUE; double v; memcpy(&v, p, 8); set_stroke_miter_limit(v); break; }
      case BLGPU_OP_SET_STROKE_JOIN: { if (!need(4)) return BLGPU_ERROR_INVALID_VALUE; uint32_t v; memcpy(&v, p, 4); set_stroke_join(v); break; }
      case BLGPU_OP_SET_STROKE_CAPS: {
        if (!need(8)) return BLGPU_ERROR_INVALID_VALUE;
        uint32_t v[2]; memcpy(v, p, 8);
        set_stroke_cap(0, v[0]);
        set_stroke_cap(1, v[1]);
        break;
      }
      case BLGPU_OP_SET_STROKE_TRANSFORM_ORDER: { if (!need(4)) return BLGPU_ERROR_INVALID_VALUE; uint32_t v; memcpy(&v, p, 4); set_stroke_transform_order(v); break; }
      case BLGPU_OP_STROKE_PATH_D: {
        if (!need(8)) return BLGPU_ERROR_INVALID_VALUE;
        uint32_t n; memcpy(&n, p, 4);
        size_t cmd_bytes = (size_t(n) + 7u) & ~size_t(7);
        if (!need(8 + cmd_bytes + size_t(n) * 16)) return BLGPU_ERROR_INVALID_VALUE;
        r = stroke_path(p + 8, aligned_doubles(p + 8 + cmd_bytes, size_t(n) * 2), n);
        break;
      }
      case BLGPU_OP_STROKE_POLYLINE_D: case BLGPU_OP_STROKE_POLYGON_D: {
        if (!need(8)) return BLGPU_ERROR_INVALID_VALUE;
        uint32_t n; memcpy(&n, p, 4);
        if (!need(8 + size_t(n) * 16)) return BLGPU_ERROR_INVALID_VALUE;
        r = stroke_poly(aligned_doubles(p + 8, size_t(n) * 2), n, op == BLGPU_OP_STROKE_POLYGON_D);
        break;
      }
      case BLGPU_OP_STROKE_BOX_D: case BLGPU_OP_STROKE_RECT_D: case BLGPU_OP_STROKE_LINE_D: {
        if (!need(32)) return BLGPU_ERROR_INVALID_VALUE;
        double q[4]; memcpy(q, p, 32);
        if (op == BLGPU_OP_STROKE_BOX_D) r = stroke_box(q[0], q[1], q[2], q[3]);
        else if (op == BLGPU_OP_STROKE_RECT_D) r = stroke_box(q[0], q[1], q[2] + q[0], q[3] + q[1]);
        else r = stroke_line(q[0], q[1], q[2], q[3]);
        break;
      }
      case BLGPU_OP_BLIT_IMAGE_I: case BLGPU_OP_BLIT_IMAGE_D:
      case BLGPU_OP_BLIT_SCALED_IMAGE_I: case BLGPU_OP_BLIT_SCALED_IMAGE_D: {
        BLGpuStreamBlit b;
        if (!need(sizeof(b))) return BLGPU_ERROR_INVALID_VALUE;
        memcpy(&b, p, sizeof(b));
        if (b.image_index >= hdr.image_count) return BLGPU_ERROR_INVALID_VALUE;
        const BLGpuImage* im = &images[b.image_index];
        const int32_t* ar = b.has_area ? b.area : nullptr;
        if (op == BLGPU_OP_BLIT_IMAGE_I) r = blit_image_i(int32_t(b.rect[0]), int32_t(b.rect[1]), im, ar);
        else if (op == BLGPU_OP_BLIT_IMAGE_D) r = blit_image_d(b.rect[0], b.rect[1], im, ar);
        else r = blit_scaled_image(b.rect[0], b.rect[1], b.rect[2], b.rect[3], im, ar, op == BLGPU_OP_BLIT_SCALED_IMAGE_I);
        if (r == BLGPU_ERROR_INVALID_VALUE) r = BLGPU_SUCCESS;   // an area outside the image draws nothing
        break;
      }
      case BLGPU_OP_FILL_MASK_I: case BLGPU_OP_FILL_MASK_D: {
        BLGpuStreamMask m;
        if (!need(sizeof(m))) return BLGPU_ERROR_INVALID_VALUE;
        memcpy(&m, p, sizeof(m));
        if (m.width > 65535u || m.height > 65535u) return BLGPU_ERROR_INVALID_VALUE;
        if (!need(sizeof(m) + size_t(m.width) * m.height)) return BLGPU_ERROR_INVALID_VALUE;
        // copied out of the stream like its pattern images: read when the frame runs
        const size_t nb = size_t(m.width) * m.height;
        stream_images->emplace_back((nb + 3u) / 4u + 1u);
        memcpy(stream_images->back().data(), p + sizeof(m), nb);
        BLGpuImage im{};
        im.pixel_data = stream_images->back().data();
        im.stride = intptr_t(m.width);
        im.width = int32_t(m.width);
        im.height = int32_t(m.height);
        im.format = BLGPU_FORMAT_A8;
        const int32_t* ar = m.has_area ? m.area : nullptr;
        if (op == BLGPU_OP_FILL_MASK_I) r = fill_mask_i(int32_t(m.origin[0]), int32_t(m.origin[1]), &im, ar);
        else r = fill_mask_d(m.origin[0], m.origin[1], &im, ar);
        if (r == BLGPU_ERROR_INVALID_VALUE || r == BLGPU_ERROR_NOT_IMPLEMENTED) r = BLGPU_SUCCESS;
        break;
      }
      case BLGPU_OP_FILL_GEOMETRY: case BLGPU_OP_STROKE_GEOMETRY: {
        if (!need(56)) return BLGPU_ERROR_INVALID_VALUE;
        uint32_t type; memcpy(&type, p, 4);
        double v[6]; memcpy(v, p + 8, 48);
        r = op == BLGPU_OP_FILL_GEOMETRY ? fill_geometry(type, v) : stroke_geometry(type, v);
        if (r == BLGPU_ERROR_NOT_IMPLEMENTED || r == BLGPU_ERROR_INVALID_GEOMETRY) r = BLGPU_SUCCESS;
        break;
      }
      case BLGPU_OP_SAVE: save(); break;
      case BLGPU_OP_RESTORE: restore(); break;
      default: return BLGPU_ERROR_INVALID_VALUE;
    }
    if (r == BLGPU_ERROR_INVALID_GEOMETRY) r = BLGPU_SUCCESS;   // a failed stroke draws nothing; replay goes on
    if (r) return r;
  }
  return BLGPU_SUCCESS;
}

// =============================================================================================
// C ABI
// =============================================================================================

#define BLGPU_API extern "C" __attribute__((visibility("default")))

BLGPU_API BLGpuResult blgpu_runtime_create(BLGpuRuntime** out, const BLGpuRuntimeCreateInfo* info) {
  if (!out) return BLGPU_ERROR_INVALID_VALUE;
  *out = nullptr;
  BLGpuRuntime* r = new (std::nothrow) BLGpuRuntime();
  if (!r) return BLGPU_ERROR_OUT_OF_MEMORY;
  BLGpuResult res = r->rt.init(info);
  if (res) { r->rt.destroy(); delete r; return res; }
  *out = r;
  return BLGPU_SUCCESS;
}

BLGPU_API BLGpuResult blgpu_runtime_destroy(BLGpuRuntime* rt) {
  if (!rt) return BLGPU_ERROR_INVALID_VALUE;
  rt->stop();
  rt->rt.destroy();
  delete rt;
  return BLGPU_SUCCESS;
}

BLGPU_API BLGpuResult blgpu_runtime_get_stats(const BLGpuRuntime* rt, BLGpuStats* out) {
  if (!rt || !out) return BLGPU_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> e(const_cast<BLGpuRuntime*>(rt)->exec);
  *out = rt->rt.stats;
  out->last_cuda_error = last_cuda_error();
  out->graph_frames = rt->rt.graph_frames_run;
  return BLGPU_SUCCESS;
}

BLGPU_API BLGpuResult blgpu_runtime_get_memory(const BLGpuRuntime* rt, BLGpuMemoryInfo* out) {
  if (!rt || !out) return BLGPU_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> e(const_cast<BLGpuRuntime*>(rt)->exec);
  *out = BLGpuMemoryInfo{};
  out->reserved_bytes = rt->rt.reserved_bytes();
  out->last_frame_bytes = rt->rt.last_frame_bytes;
  return BLGPU_SUCCESS;
}

BLGPU_API BLGpuResult blgpu_runtime_release_memory(BLGpuRuntime* rt) {
  if (!rt) return BLGPU_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> e(rt->exec);
  return rt->rt.release_memory();
}

BLGPU_API BLGpuResult blgpu_runtime_replay(BLGpuRuntime* rt, int use_graph) {
  if (!rt) return BLGPU_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> e(rt->exec);
  return rt->rt.replay(use_graph != 0);
}

BLGPU_API BLGpuResult blgpu_runtime_synchronize(BLGpuRuntime* rt) {
  if (!rt) return BLGPU_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> e(rt->exec);
  return rt->rt.synchronize();
}

static void to_abi(const LaunchConfig& c, BLGpuLaunchConfig* out) {
  *out = BLGpuLaunchConfig{};
  out->cover_slots = c.cover_slots;
  out->cover_blocks_per_sm = c.cover_blocks_per_sm;
  out->fine_blocks_per_sm = c.fine_blocks_per_sm;
  out->edge_block = c.edge_block;
  out->cubic_blocks_per_sm = c.cubic_blocks_per_sm;
  out->no_occlusion_cull = c.no_occlusion_cull;
  out->max_segments = c.max_segments;
  out->graph_frames = c.graph_frames;
  out->list_rows = c.list_rows;
  out->device_order = c.device_order;
}

BLGPU_API BLGpuResult blgpu_runtime_get_launch_config(const BLGpuRuntime* rt, BLGpuLaunchConfig* out) {
  if (!rt || !out) return BLGPU_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> e(const_cast<BLGpuRuntime*>(rt)->exec);
  to_abi(rt->rt.cfg, out);
  return BLGPU_SUCCESS;
}

BLGPU_API BLGpuResult blgpu_runtime_set_launch_config(BLGpuRuntime* rt, const BLGpuLaunchConfig* c) {
  if (!rt || !c) return BLGPU_ERROR_INVALID_VALUE;
  if ((c->cover_slots != 0 && c->cover_slots != 16 && c->cover_slots != 32 && c->cover_slots != 64) ||
      (c->edge_block != 64 && c->edge_block != 128 && c->edge_block != 256) ||
      c->cover_blocks_per_sm < 0 || c->fine_blocks_per_sm < 0 || c->cubic_blocks_per_sm < 0 ||
      (c->no_occlusion_cull != 0 && c->no_occlusion_cull != 1) || c->max_segments < 0 ||
      (c->graph_frames != 0 && c->graph_frames != 1) ||
      (c->list_rows != 0 && c->list_rows != 4 && c->list_rows != 8 && c->list_rows != 16 && c->list_rows != 32) ||
      (c->device_order != 0 && c->device_order != 1))
    return BLGPU_ERROR_INVALID_VALUE;
  LaunchConfig lc;
  lc.cover_slots = c->cover_slots;
  lc.cover_blocks_per_sm = c->cover_blocks_per_sm;
  lc.fine_blocks_per_sm = c->fine_blocks_per_sm;
  lc.edge_block = c->edge_block;
  lc.cubic_blocks_per_sm = c->cubic_blocks_per_sm;
  lc.no_occlusion_cull = c->no_occlusion_cull;
  lc.max_segments = c->max_segments;
  lc.graph_frames = c->graph_frames;
  lc.list_rows = c->list_rows ? c->list_rows : 32;
  lc.device_order = c->device_order;
  std::lock_guard<std::mutex> e(rt->exec);
  rt->rt.cfg = lc;
  rt->rt.graph_valid = false;
  return BLGPU_SUCCESS;
}

BLGPU_API BLGpuResult blgpu_runtime_autotune(BLGpuRuntime* rt, uint32_t trials, BLGpuLaunchConfig* best, double* best_ms) {
  if (!rt) return BLGPU_ERROR_INVALID_VALUE;
  LaunchConfig c;
  double ms = 0.0;
  BLGpuResult r;
  {
    std::lock_guard<std::mutex> e(rt->exec);
    r = rt->rt.autotune(int(trials), &c, &ms);
  }
  if (best) to_abi(c, best);
  if (best_ms) *best_ms = ms;
  return r;
}

BLGPU_API BLGpuResult blgpu_context_create(BLGpuContext** out, BLGpuRuntime* rt) {
  if (!out || !rt) return BLGPU_ERROR_INVALID_VALUE;
  BLGpuContext* c = new (std::nothrow) BLGpuContext();
  if (!c) return BLGPU_ERROR_OUT_OF_MEMORY;
  c->rt = rt;
  c->reset_state();
  *out = c;
  return BLGPU_SUCCESS;
}

BLGPU_API BLGpuResult blgpu_context_destroy(BLGpuContext* ctx) {
  if (!ctx) return BLGPU_ERROR_INVALID_VALUE;
  BLGpuResult r = ctx->bound ? ctx->end() : ctx->wait_async();
  delete ctx;
  return r;
}

#define CTX_CALL(expr) do { if (!ctx) return BLGPU_ERROR_INVALID_VALUE; return ctx->expr; } while (0)

BLGPU_API BLGpuResult blgpu_context_begin(BLGpuContext* ctx, const BLGpuImage* image) { CTX_CALL(begin(image)); }
BLGPU_API BLGpuResult blgpu_context_end(BLGpuContext* ctx) { CTX_CALL(end()); }
BLGPU_API BLGpuResult blgpu_context_flush(BLGpuContext* ctx, uint32_t flags) {
  if (!ctx) return BLGPU_ERROR_INVALID_VALUE;
  if (!ctx->bound) return BLGPU_ERROR_INVALID_STATE;
  if (flags & BLGPU_FLUSH_SYNC) {
    BLGpuResult r = ctx->flush_frame();
    if (!r) r = ctx->pending_error;
    ctx->pending_error = BLGPU_SUCCESS;
    return r;
  }
  if (flags & BLGPU_FLUSH_ASYNC) return ctx->flush_async();
  return BLGPU_SUCCESS;
}
BLGPU_API BLGpuResult blgpu_context_save(BLGpuContext* ctx) { CTX_CALL(save()); }
BLGPU_API BLGpuResult blgpu_context_restore(BLGpuContext* ctx) { CTX_CALL(restore()); }
BLGPU_API BLGpuResult blgpu_context_set_comp_op(BLGpuContext* ctx, uint32_t v) { CTX_CALL(set_comp_op(v)); }
BLGPU_API BLGpuResult blgpu_context_set_fill_rule(BLGpuContext* ctx, uint32_t v) { CTX_CALL(set_fill_rule(v)); }
BLGPU_API BLGpuResult blgpu_context_set_global_alpha(BLGpuContext* ctx, double a) { CTX_CALL(set_global_alpha(a)); }
BLGPU_API BLGpuResult blgpu_context_set_fill_alpha(BLGpuContext* ctx, double a) { CTX_CALL(set_fill_alpha(a)); }
BLGPU_API BLGpuResult blgpu_context_set_hint(BLGpuContext* ctx, uint32_t hint, uint32_t v) { CTX_CALL(set_hint(hint, v)); }
BLGPU_API BLGpuResult blgpu_context_set_transform(BLGpuContext* ctx, const double m[6]) { CTX_CALL(set_transform(m)); }
BLGPU_API BLGpuResult blgpu_context_reset_transform(BLGpuContext* ctx) { CTX_CALL(reset_transform()); }
BLGPU_API BLGpuResult blgpu_context_set_fill_style_rgba32(BLGpuContext* ctx, uint32_t c) { CTX_CALL(set_style_rgba32(c)); }
BLGPU_API BLGpuResult blgpu_context_set_fill_style_gradient(BLGpuContext* ctx, const BLGpuGradient* g) { CTX_CALL(set_style_gradient(g)); }
BLGPU_API BLGpuResult blgpu_context_set_fill_style_pattern(BLGpuContext* ctx, const BLGpuPattern* p) { CTX_CALL(set_style_pattern(p)); }
BLGPU_API BLGpuResult blgpu_context_clear_all(BLGpuContext* ctx) { CTX_CALL(clear_all()); }
BLGPU_API BLGpuResult blgpu_context_fill_all(BLGpuContext* ctx) { CTX_CALL(fill_all()); }
BLGPU_API BLGpuResult blgpu_context_fill_rect_i(BLGpuContext* ctx, int32_t x, int32_t y, int32_t w, int32_t h) { CTX_CALL(fill_rect_i(x, y, w, h)); }
BLGPU_API BLGpuResult blgpu_context_fill_rect_d(BLGpuContext* ctx, double x, double y, double w, double h) { CTX_CALL(fill_box(x, y, x + w, y + h)); }
BLGPU_API BLGpuResult blgpu_context_fill_box_d(BLGpuContext* ctx, double x0, double y0, double x1, double y1) { CTX_CALL(fill_box(x0, y0, x1, y1)); }
BLGPU_API BLGpuResult blgpu_context_fill_polygon_d(BLGpuContext* ctx, const double* xy, size_t n) { CTX_CALL(fill_polygon(xy, n)); }
BLGPU_API BLGpuResult blgpu_context_fill_path_d(BLGpuContext* ctx, const uint8_t* cmds, const double* xy, size_t n) { CTX_CALL(fill_path(cmds, xy, n)); }
BLGPU_API BLGpuResult blgpu_context_fill_path_at_d(BLGpuContext* ctx, const double origin[2], const uint8_t* cmds, const double* xy, size_t n) {
  if (!origin) return BLGPU_ERROR_INVALID_VALUE;
  CTX_CALL(fill_path(cmds, xy, n, origin));
}
BLGPU_API BLGpuResult blgpu_context_fill_path_fixed_d(BLGpuContext* ctx, const uint8_t* cmds, const double* xy, size_t n) { CTX_CALL(fill_path_fixed(cmds, xy, n)); }
BLGPU_API BLGpuResult blgpu_context_set_stroke_style_rgba32(BLGpuContext* ctx, uint32_t c) { CTX_CALL(set_style_rgba32(c, 1)); }
BLGPU_API BLGpuResult blgpu_context_set_stroke_style_gradient(BLGpuContext* ctx, const BLGpuGradient* g) { CTX_CALL(set_style_gradient(g, 1)); }
BLGPU_API BLGpuResult blgpu_context_set_stroke_style_pattern(BLGpuContext* ctx, const BLGpuPattern* p) { CTX_CALL(set_style_pattern(p, 1)); }
BLGPU_API BLGpuResult blgpu_context_set_stroke_alpha(BLGpuContext* ctx, double a) { CTX_CALL(set_stroke_alpha(a)); }
BLGPU_API BLGpuResult blgpu_context_set_stroke_width(BLGpuContext* ctx, double w) { CTX_CALL(set_stroke_width(w)); }
BLGPU_API BLGpuResult blgpu_context_set_stroke_miter_limit(BLGpuContext* ctx, double m) { CTX_CALL(set_stroke_miter_limit(m)); }
BLGPU_API BLGpuResult blgpu_context_set_stroke_join(BLGpuContext* ctx, uint32_t join) { CTX_CALL(set_stroke_join(join)); }
BLGPU_API BLGpuResult blgpu_context_set_stroke_cap(BLGpuContext* ctx, uint32_t position, uint32_t cap) { CTX_CALL(set_stroke_cap(position, cap)); }
BLGPU_API BLGpuResult blgpu_context_set_stroke_caps(BLGpuContext* ctx, uint32_t cap) {
  if (!ctx) return BLGPU_ERROR_INVALID_VALUE;
  if (cap > 5u) return BLGPU_ERROR_INVALID_VALUE;
  ctx->set_stroke_cap(0, cap);
  return ctx->set_stroke_cap(1, cap);
}
BLGPU_API BLGpuResult blgpu_context_set_stroke_transform_order(BLGpuContext* ctx, uint32_t order) { CTX_CALL(set_stroke_transform_order(order)); }
BLGPU_API BLGpuResult blgpu_context_stroke_path_d(BLGpuContext* ctx, const uint8_t* cmds, const double* xy, size_t n) { CTX_CALL(stroke_path(cmds, xy, n)); }
BLGPU_API BLGpuResult blgpu_context_stroke_path_at_d(BLGpuContext* ctx, const double origin[2], const uint8_t* cmds, const double* xy, size_t n) {
  if (!origin) return BLGPU_ERROR_INVALID_VALUE;
  CTX_CALL(stroke_path(cmds, xy, n, origin));
}
BLGPU_API BLGpuResult blgpu_context_stroke_polyline_d(BLGpuContext* ctx, const double* xy, size_t n) { CTX_CALL(stroke_poly(xy, n, false)); }
BLGPU_API BLGpuResult blgpu_context_stroke_polygon_d(BLGpuContext* ctx, const double* xy, size_t n) { CTX_CALL(stroke_poly(xy, n, true)); }
BLGPU_API BLGpuResult blgpu_context_stroke_box_d(BLGpuContext* ctx, double x0, double y0, double x1, double y1) { CTX_CALL(stroke_box(x0, y0, x1, y1)); }
BLGPU_API BLGpuResult blgpu_context_stroke_rect_d(BLGpuContext* ctx, double x, double y, double w, double h) { CTX_CALL(stroke_box(x, y, w + x, h + y)); }
BLGPU_API BLGpuResult blgpu_context_stroke_line_d(BLGpuContext* ctx, double x0, double y0, double x1, double y1) { CTX_CALL(stroke_line(x0, y0, x1, y1)); }
BLGPU_API BLGpuResult blgpu_stroke_outline_d(const uint8_t* cmds, const double* xy, size_t n, const BLGpuStrokeOptions* options,
                                             uint8_t* out_cmds, double* out_xy, size_t capacity, size_t* out_n) {
  if (!options || !out_n || (n && (!cmds || !xy)) || (capacity && (!out_cmds || !out_xy))) return BLGPU_ERROR_INVALID_VALUE;
  if (options->join > 4u || options->start_cap > 5u || options->end_cap > 5u) return BLGPU_ERROR_INVALID_VALUE;
  StrokeParams p;
  p.width = options->width;
  p.miter_limit = options->miter_limit;
  p.join = options->join;
  p.start_cap = options->start_cap;
  p.end_cap = options->end_cap;
  std::vector<uint8_t> oc;
  std::vector<double> ox;
  *out_n = 0;
  BLGpuResult r = stroke_outline(cmds, xy, n, p, oc, ox);
  if (r) return r;
  *out_n = oc.size();
  if (oc.size() > capacity) return BLGPU_ERROR_DATA_TOO_LARGE;
  if (!oc.empty()) {
    memcpy(out_cmds, oc.data(), oc.size());
    memcpy(out_xy, ox.data(), ox.size() * sizeof(double));
  }
  return BLGPU_SUCCESS;
}
BLGPU_API BLGpuResult blgpu_context_blit_image_i(BLGpuContext* ctx, int32_t x, int32_t y, const BLGpuImage* image, const int32_t* area) {
  CTX_CALL(blit_image_i(x, y, image, area));
}
BLGPU_API BLGpuResult blgpu_context_blit_image_d(BLGpuContext* ctx, double x, double y, const BLGpuImage* image, const int32_t* area) {
  CTX_CALL(blit_image_d(x, y, image, area));
}
BLGPU_API BLGpuResult blgpu_context_blit_scaled_image_i(BLGpuContext* ctx, int32_t x, int32_t y, int32_t w, int32_t h,
                                                        const BLGpuImage* image, const int32_t* area) {
  CTX_CALL(blit_scaled_image(double(x), double(y), double(w), double(h), image, area, true));
}
BLGPU_API BLGpuResult blgpu_context_blit_scaled_image_d(BLGpuContext* ctx, double x, double y, double w, double h,
                                                        const BLGpuImage* image, const int32_t* area) {
  CTX_CALL(blit_scaled_image(x, y, w, h, image, area, false));
}
BLGPU_API BLGpuResult blgpu_context_fill_mask_i(BLGpuContext* ctx, int32_t x, int32_t y, const BLGpuImage* mask, const int32_t* area) {
  CTX_CALL(fill_mask_i(x, y, mask, area));
}
BLGPU_API BLGpuResult blgpu_context_fill_mask_d(BLGpuContext* ctx, double x, double y, const BLGpuImage* mask, const int32_t* area) {
  CTX_CALL(fill_mask_d(x, y, mask, area));
}
BLGPU_API BLGpuResult blgpu_context_fill_geometry(BLGpuContext* ctx, uint32_t type, const double* values) { CTX_CALL(fill_geometry(type, values)); }
BLGPU_API BLGpuResult blgpu_context_stroke_geometry(BLGpuContext* ctx, uint32_t type, const double* values) { CTX_CALL(stroke_geometry(type, values)); }
BLGPU_API BLGpuResult blgpu_context_submit_stream(BLGpuContext* ctx, const void* stream, size_t size) {
  CTX_CALL(submit_stream(static_cast<const uint8_t*>(stream), size));
}

// Batched rendering: every stream gets its own canvas in one shared frame, so one device
// pipeline (one persistent fine launch) renders all of them. Canvases are independent, so the
// streams are recorded by several threads at once, each into a frame of its own over a contiguous
// range of canvases (balanced by stream bytes), and the parts are then merged into the runtime's
// batch frame in canvas order: the merged frame is the one sequential recording gives.
BLGPU_API BLGpuResult blgpu_render_batch(BLGpuRuntime* rt, const void* const* streams, const size_t* sizes,
                                         const BLGpuImage* images, uint32_t count) {
  if (!rt || (count && (!streams || !sizes || !images))) return BLGPU_ERROR_INVALID_VALUE;
  if (!count) return BLGPU_SUCCESS;
  for (uint32_t i = 0; i < count; i++)
    if (!valid_target(images[i])) return BLGPU_ERROR_INVALID_VALUE;
  std::lock_guard<std::mutex> guard(rt->batch_lock);
  Frame& frame = rt->batch_frame;
  std::vector<BLGpuContext> ctxs(count);
  // recording threads: about one per 8 canvases, at most one per host core (and 32)
  size_t total_bytes = 0;
  for (uint32_t i = 0; i < count; i++) total_bytes += sizes[i];
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const unsigned nt = std::max(1u, std::min({hw, 32u, (count + 7u) / 8u}));
  // the parts' vertices in page-locked memory: the merged frame uploads them from there
  while (rt->batch_parts.size() < nt) {
    rt->batch_parts.emplace_back(new Frame(false));
    rt->batch_parts.back()->verts.pinned = rt->batch_parts.back()->path_cmds.pinned = true;
  }
  std::vector<uint32_t> first(nt + 1, count);
  first[0] = 0;
  {
    size_t acc = 0;
    unsigned t = 1;
    for (uint32_t i = 0; i < count && t < nt; i++) {
      acc += sizes[i];
      if (acc * nt >= total_bytes * t) first[t++] = i + 1;
    }
  }
  std::vector<BLGpuResult> errors(nt, BLGPU_SUCCESS);
  const auto t_record = std::chrono::steady_clock::now();
  auto record = [&](unsigned t) {
    Frame& part = nt == 1 ? frame : *rt->batch_parts[t];
    part.clear();
    for (uint32_t i = first[t]; i < first[t + 1]; i++) {
      BLGpuContext& c = ctxs[i];
      const BLGpuImage& im = images[i];
      c.rt = rt;
      c.frame = &part;
      c.target = im;
      c.w = im.width;
      c.h = im.height;
      c.bound = true;
      c.canvas = part.add_canvas(im, true);
      c.reset_state();
      BLGpuResult r = c.submit_stream(static_cast<const uint8_t*>(streams[i]), sizes[i]);
      c.bound = false;
      if (r) { errors[t] = r; return; }
    }
  };
  if (nt == 1) {
    record(0);
  }
  else {
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; t++) pool.emplace_back(record, t);
    record(0);
    for (auto& th : pool) th.join();
  }
  for (BLGpuResult r : errors)      // the first failing canvas's error, as sequential recording gives
    if (r) return r;
  const auto t_merge = std::chrono::steady_clock::now();
  if (nt > 1) {
    std::vector<Frame*> parts(nt);
    for (unsigned t = 0; t < nt; t++) parts[t] = rt->batch_parts[t].get();
    frame.merge(parts.data(), nt, nt);
  }
  const auto t_end = std::chrono::steady_clock::now();
  {
    std::lock_guard<std::mutex> e(rt->exec);
    rt->rt.stats.last_record_ms = std::chrono::duration<double, std::milli>(t_merge - t_record).count();
    rt->rt.stats.last_merge_ms = std::chrono::duration<double, std::milli>(t_end - t_merge).count();
  }
  if (frame.cmds.empty()) return BLGPU_SUCCESS;
  BLGpuContext::mark_uploads(frame);
  std::lock_guard<std::mutex> e(rt->exec);
  return rt->rt.run(frame);
}

// No-allocation variant: the stream is recorded on the host into a one-canvas frame, then run
// entirely inside the device's fixed scratch area (Runtime::run_noalloc).
BLGPU_API BLGpuResult blgpu_render_stream_noalloc(BLGpuRuntime* rt, const void* stream, size_t size,
                                                  const BLGpuImage* device_image) {
  if (!rt || !stream || !device_image) return BLGPU_ERROR_INVALID_VALUE;
  const BLGpuImage& im = *device_image;
  if (!(im.flags & BLGPU_IMAGE_DEVICE_MEMORY) || !valid_target(im) || (im.stride & 15) ||
      (reinterpret_cast<uintptr_t>(im.pixel_data) & 15))
    return BLGPU_ERROR_INVALID_VALUE;
  // one scratch area per device: this process's calls on the device take turns
  std::lock_guard<std::mutex> guard(noalloc_lock(rt->rt.device));
  Frame frame(false);              // plain heap memory: no page-locked allocation either
  BLGpuContext c;
  c.rt = rt;
  c.frame = &frame;
  c.target = im;
  c.w = im.width;
  c.h = im.height;
  c.bound = true;
  c.canvas = frame.add_canvas(im, true);
  c.reset_state();
  BLGpuResult r = c.submit_stream(static_cast<const uint8_t*>(stream), size);
  c.bound = false;
  if (r) return r;
  if (frame.cmds.empty()) return BLGPU_SUCCESS;
  std::lock_guard<std::mutex> e(rt->exec);
  return rt->rt.run_noalloc(frame);
}
