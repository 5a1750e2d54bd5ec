// blcontext_check.cpp - checks the BLContext binding (include/blgpu_blcontext.h) against the
// reference's own BLContext: the same BLContext calls go into a raster context (thread_count 0)
// and into a context begun with blgpu_blcontext_begin, and the two images must be identical.
//
// Test infrastructure, built by oracle/ref.mk (target `blcontext`) against the reference library.
//
//   b2d_blcontext_<variant> --virt
//       the function table: every slot set; the unsupported ones return BL_ERROR_NOT_IMPLEMENTED
//       (no device is used)
//   b2d_blcontext_<variant> --streams <list.txt> [--lut N]
//       every command stream named in list.txt replayed through both contexts
//   b2d_blcontext_<variant> --scenes [--font file.ttf] [--lut N]
//       scenes written against the BLContext API directly: paths and strokes at origins, the
//       *_rgba32 / *_ext style overrides, transform operations, integer geometry, state read-back,
//       and text (when a font file is given)
// Each mode prints one JSON line and exits 0 when everything matched.
#include "../../oracle/ref_stream.h"

#include <blgpu_blcontext.h>

#include <cmath>
#include <functional>
#include <string>

static uint32_t g_lut = BLGPU_LUT_SSE2;

static bool same_pixels(const BLImage& a, const BLImage& b, size_t& differ) {
  BLImageData da, db;
  a.get_data(&da);
  b.get_data(&db);
  differ = 0;
  if (da.size != db.size || da.format != db.format) { differ = size_t(-1); return false; }
  const size_t bpp = da.format == BL_FORMAT_A8 ? 1u : 4u;
  for (int y = 0; y < da.size.h; y++) {
    const uint8_t* pa = static_cast<const uint8_t*>(da.pixel_data) + intptr_t(y) * da.stride;
    const uint8_t* pb = static_cast<const uint8_t*>(db.pixel_data) + intptr_t(y) * db.stride;
    for (int x = 0; x < da.size.w; x++) differ += memcmp(pa + size_t(x) * bpp, pb + size_t(x) * bpp, bpp) != 0;
  }
  return differ == 0;
}

static BLImage blank(int w, int h, BLFormat format = BL_FORMAT_PRGB32) {
  BLImage img(w, h, format);
  BLImageData d;
  img.make_mutable(&d);
  const size_t bpp = format == BL_FORMAT_A8 ? 1u : 4u;
  for (int y = 0; y < h; y++) memset(static_cast<uint8_t*>(d.pixel_data) + intptr_t(y) * d.stride, 0, size_t(w) * bpp);
  return img;
}

// Draws `scene` into a reference context and into a GPU context, both bound to a zeroed image of
// `format`; returns the differing pixels.
static size_t compare(int w, int h, const std::function<void(BLContext&)>& scene, std::string& error,
                      BLFormat format = BL_FORMAT_PRGB32) {
  BLImage ref = blank(w, h, format), gpu = blank(w, h, format);
  {
    BLContextCreateInfo cci{};
    BLContext ctx(ref, cci);
    scene(ctx);
    ctx.end();
  }
  {
    BLContext ctx;
    BLGpuContextCreateInfo info{};
    info.lut_variant = g_lut;
    BLResult r = blgpu_blcontext_begin(&ctx, &gpu, &info);
    if (r != BL_SUCCESS) { error = "blgpu_blcontext_begin failed: " + std::to_string(r); return size_t(-1); }
    scene(ctx);
    r = ctx.end();
    if (r != BL_SUCCESS) { error = "end failed: " + std::to_string(r); return size_t(-1); }
  }
  size_t differ = 0;
  same_pixels(ref, gpu, differ);
  return differ;
}

// --- --virt ------------------------------------------------------------------------------------

static int check_virt() {
  const BLContextVirt* v = blgpu_blcontext_virt();
  const size_t slots = sizeof(BLContextVirt) / sizeof(void*);
  size_t null_slots = 0;
  for (size_t i = 0; i < slots; i++) {
    void* p;
    memcpy(&p, reinterpret_cast<const char*>(v) + i * sizeof(void*), sizeof(p));
    null_slots += p == nullptr;
  }
  // Unsupported slots answer without touching the context; a zeroed impl is enough to call them.
  alignas(64) unsigned char storage[512] = {};
  BLContextImpl* impl = reinterpret_cast<BLContextImpl*>(storage);
  const BLRectI ri(0, 0, 1, 1);
  const BLRect rd(0, 0, 1, 1);
  const BLRgba rgba(1, 1, 1, 1);
  int bad = 0;
  auto expect = [&](BLResult got, BLResult want, const char* what) {
    if (got != want) { fprintf(stderr, "%s: got 0x%x want 0x%x\n", what, got, want); bad++; }
  };
  expect(v->user_to_meta(impl), BL_ERROR_NOT_IMPLEMENTED, "user_to_meta");
  expect(v->set_style_rgba(impl, BL_CONTEXT_STYLE_SLOT_FILL, &rgba), BL_ERROR_NOT_IMPLEMENTED, "set_style_rgba");
  expect(v->set_style_rgba64(impl, BL_CONTEXT_STYLE_SLOT_FILL, 0xFFFF000000000000ull), BL_ERROR_NOT_IMPLEMENTED, "set_style_rgba64");
  expect(v->disable_style(impl, BL_CONTEXT_STYLE_SLOT_FILL), BL_ERROR_NOT_IMPLEMENTED, "disable_style");
  expect(v->swap_styles(impl, BL_CONTEXT_STYLE_SWAP_MODE_STYLES), BL_ERROR_NOT_IMPLEMENTED, "swap_styles");
  expect(v->clip_to_rect_i(impl, &ri), BL_ERROR_NOT_IMPLEMENTED, "clip_to_rect_i");
  expect(v->clip_to_rect_d(impl, &rd), BL_ERROR_NOT_IMPLEMENTED, "clip_to_rect_d");
  expect(v->restore_clipping(impl), BL_ERROR_NOT_IMPLEMENTED, "restore_clipping");
  expect(v->clear_recti(impl, &ri), BL_ERROR_NOT_IMPLEMENTED, "clear_recti");
  expect(v->clear_rectd(impl, &rd), BL_ERROR_NOT_IMPLEMENTED, "clear_rectd");
  expect(v->set_flatten_tolerance(impl, 0.5), BL_ERROR_NOT_IMPLEMENTED, "set_flatten_tolerance(0.5)");
  expect(v->set_flatten_tolerance(impl, bl_default_approximation_options.flatten_tolerance), BL_SUCCESS, "set_flatten_tolerance(default)");
  expect(v->set_flatten_mode(impl, BL_FLATTEN_MODE_RECURSIVE), BL_ERROR_NOT_IMPLEMENTED, "set_flatten_mode(recursive)");
  expect(v->set_approximation_options(impl, &bl_default_approximation_options), BL_SUCCESS, "set_approximation_options(default)");
  printf("{\"slots\": %zu, \"null_slots\": %zu, \"unexpected\": %d}\n", slots, null_slots, bad);
  return (null_slots == 0 && bad == 0) ? 0 : 1;
}

// --- --streams ---------------------------------------------------------------------------------

static int check_streams(const char* list) {
  FILE* f = fopen(list, "r");
  if (!f) { fprintf(stderr, "cannot open %s\n", list); return 2; }
  char line[4096];
  int n = 0, failed = 0;
  std::string detail;
  while (fgets(line, sizeof(line), f)) {
    size_t len = strlen(line);
    while (len && (line[len - 1] == '\n' || line[len - 1] == '\r')) line[--len] = 0;
    if (!len) continue;
    std::vector<uint8_t> buf = read_file(line);
    Stream s;
    s.base = buf.data();
    s.size = buf.size();
    parse_header(s);
    std::string err;
    const size_t d = compare(int(s.hdr.width), int(s.hdr.height), [&](BLContext& ctx) { replay_records(s, ctx); }, err,
                             target_format(s));
    n++;
    if (d) {
      failed++;
      if (detail.size() < 400) detail += std::string(detail.empty() ? "" : "; ") + line + ": " + (err.empty() ? std::to_string(d) + " pixels" : err);
    }
  }
  fclose(f);
  printf("{\"streams\": %d, \"failed\": %d, \"detail\": \"%s\"}\n", n, failed, detail.c_str());
  return failed ? 1 : 0;
}

// --- --scenes ----------------------------------------------------------------------------------

struct Rng {   // xorshift64*: the scenes' own seeded numbers
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 1) {}
  uint64_t next() { s ^= s >> 12; s ^= s << 25; s ^= s >> 27; return s * 0x2545F4914F6CDD1Dull; }
  double uniform(double a, double b) { return a + (b - a) * double(next() >> 11) * (1.0 / 9007199254740992.0); }
  uint32_t u32() { return uint32_t(next() >> 32); }
};

static BLPath random_path(Rng& r, double x, double y, double side) {
  BLPath p;
  p.move_to(x + r.uniform(0, side), y + r.uniform(0, side));
  const int n = 3 + int(r.u32() % 5);
  for (int i = 0; i < n; i++) {
    switch (r.u32() % 3) {
      case 0: p.line_to(x + r.uniform(0, side), y + r.uniform(0, side)); break;
      case 1: p.quad_to(x + r.uniform(0, side), y + r.uniform(0, side), x + r.uniform(0, side), y + r.uniform(0, side)); break;
      default: p.cubic_to(x + r.uniform(0, side), y + r.uniform(0, side), x + r.uniform(0, side), y + r.uniform(0, side),
                          x + r.uniform(0, side), y + r.uniform(0, side)); break;
    }
  }
  p.close();
  return p;
}

static BLGradient random_gradient(Rng& r, double x, double y, double side) {
  BLGradient g;
  const int kind = int(r.u32() % 3);
  if (kind == 0) g.create(BLLinearGradientValues(x, y, x + r.uniform(1, side), y + r.uniform(1, side)), BLExtendMode(r.u32() % 3));
  else if (kind == 1) g.create(BLRadialGradientValues(x + side / 2, y + side / 2, x + r.uniform(0, side), y + r.uniform(0, side), side / 2, 0), BLExtendMode(r.u32() % 3));
  else g.create(BLConicGradientValues(x + side / 2, y + side / 2, r.uniform(0, 6.28), 1.0));
  const int stops = 2 + int(r.u32() % 4);
  for (int i = 0; i < stops; i++) g.add_stop(r.uniform(0, 1), BLRgba32(r.u32()));
  return g;
}

static int check_scenes(const char* font_path) {
  struct Scene { const char* name; int w, h; std::function<void(BLContext&)> draw; };
  std::vector<Scene> scenes;

  scenes.push_back({"paths_at_origins", 320, 240, [](BLContext& ctx) {
    Rng r(11);
    ctx.fill_all(BLRgba32(0xFF102030u));
    for (int i = 0; i < 120; i++) {
      BLPath p = random_path(r, 0, 0, r.uniform(10, 90));
      ctx.set_fill_rule(BLFillRule(r.u32() & 1));
      ctx.set_comp_op(BLCompOp(r.u32() & 1));
      ctx.fill_path(BLPoint(r.uniform(-40, 300), r.uniform(-40, 220)), p, BLRgba32(r.u32()));
    }
  }});
  scenes.push_back({"strokes_at_origins", 300, 200, [](BLContext& ctx) {
    Rng r(12);
    ctx.clear_all();
    for (int i = 0; i < 60; i++) {
      BLPath p = random_path(r, 0, 0, r.uniform(10, 80));
      ctx.set_stroke_width(r.uniform(0.5, 9));
      ctx.set_stroke_join(BLStrokeJoin(r.u32() % 5));
      ctx.set_stroke_caps(BLStrokeCap(r.u32() % 3));
      ctx.set_stroke_transform_order(BLStrokeTransformOrder(r.u32() & 1));
      if (i % 7 == 0) ctx.rotate(0.1, 150, 100);
      ctx.stroke_path(BLPoint(r.uniform(-20, 280), r.uniform(-20, 180)), p, BLRgba32(r.u32()));
    }
  }});
  scenes.push_back({"style_overrides_and_transforms", 256, 256, [](BLContext& ctx) {
    Rng r(13);
    ctx.fill_all(BLRgba32(0xFFFFFFFFu));
    for (int i = 0; i < 80; i++) {
      ctx.save();
      ctx.translate(r.uniform(-20, 200), r.uniform(-20, 200));
      if (i % 3 == 0) ctx.rotate(r.uniform(-1, 1));
      if (i % 4 == 0) ctx.scale(r.uniform(0.5, 1.8), r.uniform(0.5, 1.8));
      ctx.set_global_alpha(i % 5 == 0 ? 0.5 : 1.0);
      ctx.set_fill_alpha(i % 6 == 0 ? 0.75 : 1.0);
      const double side = r.uniform(10, 70);
      BLGradient g = random_gradient(r, 0, 0, side);
      switch (i % 5) {
        case 0: ctx.fill_rect(BLRect(0, 0, side, side * 0.7), g); break;
        case 1: ctx.fill_path(random_path(r, 0, 0, side), g); break;
        case 2: ctx.fill_box(BLBox(0.5, 0.25, side, side * 0.5), BLRgba32(r.u32())); break;
        case 3: ctx.fill_circle(BLCircle(side / 2, side / 2, side / 2), g); break;
        default: ctx.fill_rect(BLRectI(0, 0, int(side), int(side / 2)), BLRgba32(r.u32())); break;
      }
      ctx.restore();
    }
  }});
  scenes.push_back({"integer_geometry_and_state", 200, 160, [](BLContext& ctx) {
    Rng r(14);
    ctx.clear_all();
    ctx.set_fill_style(BLRgba32(0xFF00C0FFu));
    for (int i = 0; i < 40; i++) {
      BLPointI pts[5];
      for (auto& p : pts) p = BLPointI(int(r.u32() % 220) - 10, int(r.u32() % 180) - 10);
      ctx.fill_polygon(pts, 5, BLRgba32(r.u32()));
      ctx.fill_box(BLBoxI(int(r.u32() % 150), int(r.u32() % 120), 150 + int(r.u32() % 40), 120 + int(r.u32() % 30)), BLRgba32(r.u32()));
    }
    // the state the accessors read is kept across save / restore
    ctx.save();
    ctx.set_comp_op(BL_COMP_OP_SRC_COPY);
    ctx.set_fill_alpha(0.5);
    ctx.restore();
    if (ctx.comp_op() != BL_COMP_OP_SRC_OVER || ctx.fill_alpha() != 1.0 || ctx.saved_state_count() != 0) {
      fprintf(stderr, "state read-back differs\n");
      ctx.fill_all(BLRgba32(0xFFFF0000u));   // makes the pixels differ
    }
    ctx.stroke_rect(BLRectI(10, 10, 100, 60), BLRgba32(0xFF000000u));
  }});

  BLFontFace face;
  const bool have_font = font_path && face.create_from_file(font_path) == BL_SUCCESS;
  if (have_font) {
    scenes.push_back({"text", 420, 160, [&face](BLContext& ctx) {
      Rng r(15);
      ctx.fill_all(BLRgba32(0xFFFFFFFFu));
      const char* lines[] = {"Hello, GB300!", "The quick brown fox jumps", "over the lazy dog 0123456789", "AVAVAVA WAWA fi fl"};
      for (int i = 0; i < 12; i++) {
        BLFont font;
        font.create_from_face(face, float(r.uniform(9, 40)));
        ctx.save();
        if (i % 3 == 1) ctx.rotate(r.uniform(-0.3, 0.3), 200, 80);
        if (i % 4 == 2) ctx.set_fill_style(random_gradient(r, 0, 0, 200));
        else ctx.set_fill_style(BLRgba32(r.u32() | 0x80000000u));
        ctx.fill_utf8_text(BLPoint(r.uniform(-10, 300), r.uniform(10, 150)), font, lines[i % 4]);
        ctx.restore();
      }
    }});
    // stroked text: both transform orders, joins and widths, under rotations and scales
    scenes.push_back({"stroked_text", 420, 200, [&face](BLContext& ctx) {
      Rng r(16);
      ctx.fill_all(BLRgba32(0xFF202020u));
      const char* lines[] = {"Stroked GB300", "quick brown fox", "AVAWA 0123", "fi fl ffi"};
      for (int i = 0; i < 12; i++) {
        BLFont font;
        font.create_from_face(face, float(r.uniform(12, 48)));
        ctx.save();
        if (i % 3 == 1) ctx.rotate(r.uniform(-0.4, 0.4), 200, 100);
        if (i % 4 == 3) ctx.scale(r.uniform(0.6, 1.6), r.uniform(0.6, 1.6));
        ctx.set_stroke_transform_order(i % 2 ? BL_STROKE_TRANSFORM_ORDER_BEFORE : BL_STROKE_TRANSFORM_ORDER_AFTER);
        ctx.set_stroke_width(r.uniform(0.5, 4.0));
        ctx.set_stroke_join(BLStrokeJoin(r.u32() % 5));
        if (i % 4 == 2) ctx.set_stroke_style(random_gradient(r, 0, 0, 200));
        else ctx.set_stroke_style(BLRgba32(r.u32() | 0x80000000u));
        const BLPoint at(r.uniform(-10, 300), r.uniform(10, 190));
        if (i % 5 == 4) ctx.stroke_utf8_text(at, font, lines[i % 4], SIZE_MAX, BLRgba32(0xFFFFC000u));
        else ctx.stroke_utf8_text(at, font, lines[i % 4]);
        ctx.restore();
      }
    }});
  }

  int failed = 0;
  std::string detail;
  for (const Scene& s : scenes) {
    std::string err;
    const size_t d = compare(s.w, s.h, s.draw, err);
    if (d) {
      failed++;
      detail += std::string(detail.empty() ? "" : "; ") + s.name + ": " + (err.empty() ? std::to_string(d) + " pixels" : err);
    }
  }
  printf("{\"scenes\": %zu, \"failed\": %d, \"text\": %s, \"detail\": \"%s\"}\n", scenes.size(), failed,
         have_font ? "true" : "false", detail.c_str());
  return failed ? 1 : 0;
}

int main(int argc, char** argv) {
  const char* font = nullptr;
  for (int i = 1; i + 1 < argc; i++) {
    if (!strcmp(argv[i], "--lut")) g_lut = uint32_t(atoi(argv[i + 1]));
    if (!strcmp(argv[i], "--font")) font = argv[i + 1];
  }
  if (argc >= 2 && !strcmp(argv[1], "--virt")) return check_virt();
  if (argc >= 3 && !strcmp(argv[1], "--streams")) return check_streams(argv[2]);
  if (argc >= 2 && !strcmp(argv[1], "--scenes")) return check_scenes(font);
  fprintf(stderr, "usage: %s --virt | --streams list.txt [--lut N] | --scenes [--font f.ttf] [--lut N]\n", argv[0]);
  return 2;
}
