// ref_replay.cpp - replays a blgpu command stream (include/blgpu_stream.h) into the reference
// Blend2D BLContext and writes the resulting PRGB32 pixels.
//
// Test infrastructure: built by oracle/ref.mk against the reference sources (never shipped).
// Every record maps 1:1 onto the reference C++ API (blend2d/core/context.h:2155-2700).
//
//   b2d_replay_<variant> <stream.bin> <out.raw|-> [--threads N] [--frames K]
//   b2d_replay_<variant> --batch <list.txt> [--threads N] [--repeat K] [--out-dir D]
//
// With --frames K the stream is rendered K+1 times (one warm-up) and the median wall time of
// `begin -> all calls -> end()` is printed as JSON on stdout.
// With --batch every stream named in list.txt (one path per line) is read and parsed first, then
// all of them are rendered one after the other (one BLContext per canvas, `thread_count` N), K
// times; the wall time of each pass is printed as JSON. --out-dir writes canvas i's pixels to
// D/<i>.raw after the last pass.

#include <blend2d/blend2d.h>
#include <blgpu_stream.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
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
    BLImage img(int(ih.width), int(ih.height), BL_FORMAT_PRGB32);
    BLImageData d;
    img.make_mutable(&d);
    for (uint32_t y = 0; y < ih.height; y++)
      memcpy(static_cast<uint8_t*>(d.pixel_data) + intptr_t(y) * d.stride, s.base + off + size_t(y) * ih.width * 4u, size_t(ih.width) * 4u);
    off += (size_t(ih.width) * ih.height * 4u + 7u) & ~size_t(7);
    s.images.push_back(img);
  }
  s.records_offset = off;
}

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

static void replay(const Stream& s, BLImage& img, uint32_t threads) {
  BLImageData d;
  img.make_mutable(&d);
  for (int y = 0; y < d.size.h; y++)
    memset(static_cast<uint8_t*>(d.pixel_data) + intptr_t(y) * d.stride, 0, size_t(d.size.w) * 4u);

  BLContextCreateInfo cci {};
  cci.thread_count = threads;
  BLContext ctx(img, cci);

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
  ctx.end();
}

static int run_batch(int argc, char** argv) {
  const char* list = argv[2];
  uint32_t threads = 0;
  int repeat = 1;
  const char* out_dir = nullptr;
  for (int i = 3; i + 1 < argc; i += 2) {
    if (!strcmp(argv[i], "--threads")) threads = uint32_t(atoi(argv[i + 1]));
    else if (!strcmp(argv[i], "--repeat")) repeat = atoi(argv[i + 1]);
    else if (!strcmp(argv[i], "--out-dir")) out_dir = argv[i + 1];
  }
  std::vector<std::vector<uint8_t>> bufs;
  {
    FILE* f = fopen(list, "r");
    if (!f) { fprintf(stderr, "cannot open %s\n", list); return 2; }
    char line[4096];
    while (fgets(line, sizeof(line), f)) {
      size_t n = strlen(line);
      while (n && (line[n - 1] == '\n' || line[n - 1] == '\r')) line[--n] = 0;
      if (n) bufs.push_back(read_file(line));
    }
    fclose(f);
  }
  std::vector<Stream> streams(bufs.size());
  std::vector<BLImage> imgs;
  uint64_t pixels = 0;
  for (size_t i = 0; i < bufs.size(); i++) {
    streams[i].base = bufs[i].data();
    streams[i].size = bufs[i].size();
    parse_header(streams[i]);
    imgs.emplace_back(int(streams[i].hdr.width), int(streams[i].hdr.height), BL_FORMAT_PRGB32);
    pixels += uint64_t(streams[i].hdr.width) * streams[i].hdr.height;
  }
  std::vector<double> ms;
  for (int k = 0; k < repeat; k++) {
    auto t0 = std::chrono::steady_clock::now();
    for (size_t i = 0; i < streams.size(); i++) replay(streams[i], imgs[i], threads);
    auto t1 = std::chrono::steady_clock::now();
    ms.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
  }
  printf("{\"canvases\": %zu, \"pixels\": %llu, \"threads\": %u, \"times_ms\": [", streams.size(),
         (unsigned long long)pixels, threads);
  for (size_t k = 0; k < ms.size(); k++) printf("%s%.4f", k ? ", " : "", ms[k]);
  printf("]}\n");
  if (out_dir) {
    for (size_t i = 0; i < imgs.size(); i++) {
      BLImageData d;
      imgs[i].get_data(&d);
      std::string path = std::string(out_dir) + "/" + std::to_string(i) + ".raw";
      FILE* f = fopen(path.c_str(), "wb");
      if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); return 2; }
      for (int y = 0; y < d.size.h; y++)
        fwrite(static_cast<const uint8_t*>(d.pixel_data) + intptr_t(y) * d.stride, 1, size_t(d.size.w) * 4u, f);
      fclose(f);
    }
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 3 && !strcmp(argv[1], "--batch")) return run_batch(argc, argv);
  if (argc < 3) {
    fprintf(stderr, "usage: %s stream.bin out.raw|- [--threads N] [--frames K]\n", argv[0]);
    return 2;
  }
  uint32_t threads = 0;
  int frames = 0;
  for (int i = 3; i + 1 < argc; i += 2) {
    if (!strcmp(argv[i], "--threads")) threads = uint32_t(atoi(argv[i + 1]));
    else if (!strcmp(argv[i], "--frames")) frames = atoi(argv[i + 1]);
  }

  std::vector<uint8_t> buf = read_file(argv[1]);
  Stream s;
  s.base = buf.data();
  s.size = buf.size();
  parse_header(s);

  BLImage img(int(s.hdr.width), int(s.hdr.height), BL_FORMAT_PRGB32);
  replay(s, img, threads);

  if (frames > 0) {
    std::vector<double> ms;
    for (int f = 0; f < frames; f++) {
      auto t0 = std::chrono::steady_clock::now();
      replay(s, img, threads);
      auto t1 = std::chrono::steady_clock::now();
      ms.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
    }
    std::sort(ms.begin(), ms.end());
    printf("{\"frames\": %d, \"threads\": %u, \"median_ms\": %.4f, \"min_ms\": %.4f}\n", frames, threads, ms[ms.size() / 2], ms[0]);
  }

  if (strcmp(argv[2], "-") != 0) {
    BLImageData d;
    img.get_data(&d);
    FILE* f = fopen(argv[2], "wb");
    for (int y = 0; y < d.size.h; y++)
      fwrite(static_cast<const uint8_t*>(d.pixel_data) + intptr_t(y) * d.stride, 1, size_t(d.size.w) * 4u, f);
    fclose(f);
  }
  return 0;
}
