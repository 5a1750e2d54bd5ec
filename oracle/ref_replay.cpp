// ref_replay.cpp - replays a blgpu command stream (include/blgpu_stream.h) into the reference
// Blend2D BLContext and writes the resulting pixels (4 bytes per pixel, 1 for an A8 target).
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

#include "ref_stream.h"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

static void replay(const Stream& s, BLImage& img, uint32_t threads) {
  BLImageData d;
  img.make_mutable(&d);
  for (int y = 0; y < d.size.h; y++)
    memset(static_cast<uint8_t*>(d.pixel_data) + intptr_t(y) * d.stride, 0, size_t(d.size.w) * target_bpp(s));

  BLContextCreateInfo cci {};
  cci.thread_count = threads;
  BLContext ctx(img, cci);
  replay_records(s, ctx);
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
    imgs.emplace_back(int(streams[i].hdr.width), int(streams[i].hdr.height), target_format(streams[i]));
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
        fwrite(static_cast<const uint8_t*>(d.pixel_data) + intptr_t(y) * d.stride, 1, size_t(d.size.w) * target_bpp(streams[i]), f);
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

  BLImage img(int(s.hdr.width), int(s.hdr.height), target_format(s));
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
      fwrite(static_cast<const uint8_t*>(d.pixel_data) + intptr_t(y) * d.stride, 1, size_t(d.size.w) * target_bpp(s), f);
    fclose(f);
  }
  return 0;
}
