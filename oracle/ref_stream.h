// ref_stream.h - reads a blgpu command stream (include/blgpu_stream.h) and replays its records
// into a BLContext through the reference's public C++ API (blend2d/core/context.h:2155-2700).
//
// Test infrastructure shared by the reference replay harness (ref_replay.cpp) and the BLContext
// binding check (tests/native/blcontext_check.cpp): the same call sequence goes into the
// reference's own context and into a context begun on another backend.
#pragma once

#include <blend2d/blend2d.h>
#include <blgpu_stream.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

static std::vector<uint8_t> read_file(const char* path) {
  std::vector<uint8_t> buf;
  FILE* f = fopen(path, "rb");
  if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  buf.resize(size_t(n));
  if (n && fread(buf.data(), 1, size_t(n), f) != size_t(n)) { fprintf(stderr, "short read\n"); exit(2); }
  fclose(f);
  return buf;
}

struct Stream {
  const uint8_t* base = nullptr;
  size_t size = 0;
  BLGpuStreamHeader hdr {};
  std::vector<BLImage> images;
  size_t records_offset = 0;
};

static void parse_header(Stream& s) {
  memcpy(&s.hdr, s.base, sizeof(s.hdr));
  if (s.hdr.magic != BLGPU_STREAM_MAGIC || s.hdr.version != BLGPU_STREAM_VERSION) {
    fprintf(stderr, "bad stream header\n");
    exit(2);
  }
  size_t off = sizeof(BLGpuStreamHeader);
  for (uint32_t i = 0; i < s.hdr.image_count; i++) {
    BLGpuStreamImage ih;
    memcpy(&ih, s.base + off, sizeof(ih));
    off += sizeof(ih);
    BLImage img(int(ih.width), int(ih.height), ih.format == BLGPU_STREAM_FORMAT_XRGB32 ? BL_FORMAT_XRGB32 : BL_FORMAT_PRGB32);
    BLImageData d;
    img.make_mutable(&d);
    for (uint32_t y = 0; y < ih.height; y++)
      memcpy(static_cast<uint8_t*>(d.pixel_data) + intptr_t(y) * d.stride, s.base + off + size_t(y) * ih.width * 4u, size_t(ih.width) * 4u);
    off += (size_t(ih.width) * ih.height * 4u + 7u) & ~size_t(7);
    s.images.push_back(img);
  }
  s.records_offset = off;
}

// The target's BLFormat (the header's 0 reads as PRGB32) and its bytes per pixel.
static BLFormat target_format(const Stream& s) {
  return s.hdr.format ? BLFormat(s.hdr.format) : BL_FORMAT_PRGB32;
}
static size_t target_bpp(const Stream& s) { return target_format(s) == BL_FORMAT_A8 ? 1u : 4u; }

template<typename T>
static T rd(const uint8_t* p) { T v; memcpy(&v, p, sizeof(T)); return v; }

static BLGradient make_gradient(const uint8_t* p) {
  BLGpuStreamGradient g = rd<BLGpuStreamGradient>(p);
  std::vector<BLGradientStop> stops(g.stop_count);
  for (uint32_t i = 0; i < g.stop_count; i++) {
    BLGpuStreamGradientStop st = rd<BLGpuStreamGradientStop>(p + sizeof(g) + i * sizeof(st));
    stops[i] = BLGradientStop(st.offset, BLRgba64(st.rgba64));
  }
  BLGradient grad;
  if (g.type == BLGPU_GRADIENT_LINEAR)
    grad.create(BLLinearGradientValues(g.values[0], g.values[1], g.values[2], g.values[3]), BLExtendMode(g.extend_mode));
  else if (g.type == BLGPU_GRADIENT_RADIAL)
    grad.create(BLRadialGradientValues(g.values[0], g.values[1], g.values[2], g.values[3], g.values[4], g.values[5]), BLExtendMode(g.extend_mode));
  else
    grad.create(BLConicGradientValues(g.values[0], g.values[1], g.values[2], g.values[3]), BLExtendMode(g.extend_mode));
  grad.assign_stops(stops.data(), stops.size());
  if (g.has_transform)
    grad.set_transform(BLMatrix2D(g.transform[0], g.transform[1], g.transform[2], g.transform[3], g.transform[4], g.transform[5]));
  return grad;
}

static BLPattern make_pattern(const Stream& s, const uint8_t* p) {
  BLGpuStreamPattern pt = rd<BLGpuStreamPattern>(p);
  const BLImage& src = s.images[pt.image_index];
  BLPattern pat;
  if (pt.area[2] > 0)
    pat.create(src, BLRectI(pt.area[0], pt.area[1], pt.area[2], pt.area[3]), BLExtendMode(pt.extend_mode));
  else
    pat.create(src, BLExtendMode(pt.extend_mode));
  if (pt.has_transform)
    pat.set_transform(BLMatrix2D(pt.transform[0], pt.transform[1], pt.transform[2], pt.transform[3], pt.transform[4], pt.transform[5]));
  return pat;
}

// u32 n, u32 pad, u8 cmd[n] (padded to 8), f64 xy[2n]
static BLPath read_path(const uint8_t* p) {
  uint32_t n = rd<uint32_t>(p);
  const uint8_t* cmds = p + 8;
  const uint8_t* xy = cmds + ((n + 7u) & ~7u);
  BLPath path;
  uint8_t* cmd_out;
  BLPoint* vtx_out;
  path.modify_op(BL_MODIFY_OP_ASSIGN_GROW, n, &cmd_out, &vtx_out);
  memcpy(cmd_out, cmds, n);
  memcpy(vtx_out, xy, size_t(n) * sizeof(BLPoint));
  return path;
}

// Replays every record of `s` into `ctx` (which is already begun on the stream's canvas).
static void replay_records(const Stream& s, BLContext& ctx) {
  std::vector<BLPoint> pts;
  size_t off = s.records_offset;
  while (off + 8 <= s.size) {
    uint32_t op = rd<uint32_t>(s.base + off);
    uint32_t len = rd<uint32_t>(s.base + off + 4);
    const uint8_t* p = s.base + off + 8;
    off += 8 + len;
    if (op == BLGPU_OP_END)
      break;

    switch (op) {
      case BLGPU_OP_SET_COMP_OP: ctx.set_comp_op(BLCompOp(rd<uint32_t>(p))); break;
      case BLGPU_OP_SET_FILL_RULE: ctx.set_fill_rule(BLFillRule(rd<uint32_t>(p))); break;
      case BLGPU_OP_SET_GLOBAL_ALPHA: ctx.set_global_alpha(rd<double>(p)); break;
      case BLGPU_OP_SET_FILL_ALPHA: ctx.set_fill_alpha(rd<double>(p)); break;
      case BLGPU_OP_SET_HINT: ctx.set_hint(BLContextHint(rd<uint32_t>(p)), rd<uint32_t>(p + 4)); break;
      case BLGPU_OP_SET_TRANSFORM: {
        double m[6];
        memcpy(m, p, sizeof(m));
        ctx.set_transform(BLMatrix2D(m[0], m[1], m[2], m[3], m[4], m[5]));
        break;
      }
      case BLGPU_OP_RESET_TRANSFORM: ctx.reset_transform(); break;
      case BLGPU_OP_STYLE_RGBA32: ctx.set_fill_style(BLRgba32(rd<uint32_t>(p))); break;
      case BLGPU_OP_STYLE_GRADIENT: ctx.set_fill_style(make_gradient(p)); break;
      case BLGPU_OP_STYLE_PATTERN: ctx.set_fill_style(make_pattern(s, p)); break;
      case BLGPU_OP_STROKE_STYLE_RGBA32: ctx.set_stroke_style(BLRgba32(rd<uint32_t>(p))); break;
      case BLGPU_OP_STROKE_STYLE_GRADIENT: ctx.set_stroke_style(make_gradient(p)); break;
      case BLGPU_OP_STROKE_STYLE_PATTERN: ctx.set_stroke_style(make_pattern(s, p)); break;
      case BLGPU_OP_SET_STROKE_ALPHA: ctx.set_stroke_alpha(rd<double>(p)); break;
      case BLGPU_OP_SET_STROKE_WIDTH: ctx.set_stroke_width(rd<double>(p)); break;
      case BLGPU_OP_SET_STROKE_MITER_LIMIT: ctx.set_stroke_miter_limit(rd<double>(p)); break;
      case BLGPU_OP_SET_STROKE_JOIN: ctx.set_stroke_join(BLStrokeJoin(rd<uint32_t>(p))); break;
      case BLGPU_OP_SET_STROKE_CAPS:
        ctx.set_stroke_cap(BL_STROKE_CAP_POSITION_START, BLStrokeCap(rd<uint32_t>(p)));
        ctx.set_stroke_cap(BL_STROKE_CAP_POSITION_END, BLStrokeCap(rd<uint32_t>(p + 4)));
        break;
      case BLGPU_OP_SET_STROKE_TRANSFORM_ORDER: ctx.set_stroke_transform_order(BLStrokeTransformOrder(rd<uint32_t>(p))); break;
      case BLGPU_OP_STROKE_PATH_D: ctx.stroke_path(read_path(p)); break;
      case BLGPU_OP_STROKE_POLYLINE_D: case BLGPU_OP_STROKE_POLYGON_D: {
        uint32_t n = rd<uint32_t>(p);
        pts.resize(n);
        memcpy(pts.data(), p + 8, size_t(n) * sizeof(BLPoint));
        if (op == BLGPU_OP_STROKE_POLYLINE_D) ctx.stroke_polyline(pts.data(), n);
        else ctx.stroke_polygon(pts.data(), n);
        break;
      }
      case BLGPU_OP_STROKE_BOX_D: { double b[4]; memcpy(b, p, sizeof(b)); ctx.stroke_box(BLBox(b[0], b[1], b[2], b[3])); break; }
      case BLGPU_OP_STROKE_RECT_D: { double r[4]; memcpy(r, p, sizeof(r)); ctx.stroke_rect(BLRect(r[0], r[1], r[2], r[3])); break; }
      case BLGPU_OP_STROKE_LINE_D: { double l[4]; memcpy(l, p, sizeof(l)); ctx.stroke_line(BLLine(l[0], l[1], l[2], l[3])); break; }
      case BLGPU_OP_CLEAR_ALL: ctx.clear_all(); break;
      case BLGPU_OP_FILL_ALL: ctx.fill_all(); break;
      case BLGPU_OP_FILL_RECT_I: {
        int32_t r[4];
        memcpy(r, p, sizeof(r));
        ctx.fill_rect(BLRectI(r[0], r[1], r[2], r[3]));
        break;
      }
      case BLGPU_OP_FILL_RECT_D: {
        double r[4];
        memcpy(r, p, sizeof(r));
        ctx.fill_rect(BLRect(r[0], r[1], r[2], r[3]));
        break;
      }
      case BLGPU_OP_FILL_BOX_D: {
        double b[4];
        memcpy(b, p, sizeof(b));
        ctx.fill_box(BLBox(b[0], b[1], b[2], b[3]));
        break;
      }
      case BLGPU_OP_FILL_POLYGON_D: {
        uint32_t n = rd<uint32_t>(p);
        pts.resize(n);
        memcpy(pts.data(), p + 8, size_t(n) * sizeof(BLPoint));
        ctx.fill_polygon(pts.data(), n);
        break;
      }
      case BLGPU_OP_FILL_PATH_D: ctx.fill_path(read_path(p)); break;
      case BLGPU_OP_BLIT_IMAGE_I: case BLGPU_OP_BLIT_IMAGE_D:
      case BLGPU_OP_BLIT_SCALED_IMAGE_I: case BLGPU_OP_BLIT_SCALED_IMAGE_D: {
        BLGpuStreamBlit b = rd<BLGpuStreamBlit>(p);
        const BLImage& im = s.images[b.image_index];
        BLRectI area(b.area[0], b.area[1], b.area[2], b.area[3]);
        const BLRectI* ap = b.has_area ? &area : nullptr;
        if (op == BLGPU_OP_BLIT_IMAGE_I) {
          BLPointI o(int(b.rect[0]), int(b.rect[1]));
          bl_context_blit_image_i(&ctx, &o, &im, ap);
        }
        else if (op == BLGPU_OP_BLIT_IMAGE_D) {
          BLPoint o(b.rect[0], b.rect[1]);
          bl_context_blit_image_d(&ctx, &o, &im, ap);
        }
        else if (op == BLGPU_OP_BLIT_SCALED_IMAGE_I) {
          BLRectI r(int(b.rect[0]), int(b.rect[1]), int(b.rect[2]), int(b.rect[3]));
          bl_context_blit_scaled_image_i(&ctx, &r, &im, ap);
        }
        else {
          BLRect r(b.rect[0], b.rect[1], b.rect[2], b.rect[3]);
          bl_context_blit_scaled_image_d(&ctx, &r, &im, ap);
        }
        break;
      }
      case BLGPU_OP_FILL_MASK_I: case BLGPU_OP_FILL_MASK_D: {
        BLGpuStreamMask m = rd<BLGpuStreamMask>(p);
        BLImage mask;
        mask.create_from_data(int(m.width), int(m.height), BL_FORMAT_A8, const_cast<uint8_t*>(p + sizeof(m)), intptr_t(m.width));
        BLRectI area(m.area[0], m.area[1], m.area[2], m.area[3]);
        const BLRectI* ap = m.has_area ? &area : nullptr;
        if (op == BLGPU_OP_FILL_MASK_I) {
          BLPointI o(int(m.origin[0]), int(m.origin[1]));
          bl_context_fill_mask_i(&ctx, &o, &mask, ap);
        }
        else {
          BLPoint o(m.origin[0], m.origin[1]);
          bl_context_fill_mask_d(&ctx, &o, &mask, ap);
        }
        break;
      }
      case BLGPU_OP_FILL_GEOMETRY: case BLGPU_OP_STROKE_GEOMETRY: {
        uint32_t type = rd<uint32_t>(p);
        double v[6];
        memcpy(v, p + 8, sizeof(v));
        BLCircle ci(v[0], v[1], v[2]);
        BLEllipse el(v[0], v[1], v[2], v[3]);
        BLRoundRect rr(v[0], v[1], v[2], v[3], v[4], v[5]);
        BLTriangle tr(v[0], v[1], v[2], v[3], v[4], v[5]);
        BLArc ar(v[0], v[1], v[2], v[3], v[4], v[5]);
        const void* data = type == BL_GEOMETRY_TYPE_CIRCLE ? (const void*)&ci : type == BL_GEOMETRY_TYPE_ELLIPSE ? (const void*)&el
                         : type == BL_GEOMETRY_TYPE_ROUND_RECT ? (const void*)&rr : type == BL_GEOMETRY_TYPE_TRIANGLE ? (const void*)&tr
                         : (const void*)&ar;
        if (op == BLGPU_OP_FILL_GEOMETRY) bl_context_fill_geometry(&ctx, BLGeometryType(type), data);
        else bl_context_stroke_geometry(&ctx, BLGeometryType(type), data);
        break;
      }
      case BLGPU_OP_SAVE: ctx.save(); break;
      case BLGPU_OP_RESTORE: ctx.restore(); break;
      default:
        fprintf(stderr, "unknown op %u\n", op);
        exit(2);
    }
  }
}
