// runtime.cpp - device runtime: one upload per frame, the two halves of the device pipeline, one
// download per host canvas, CUDA-graph replay of the last frame.
//
// The pipeline needs four sizes that only the device knows after edge building (segments,
// seglist entries, (command, tile-row) slots, row-list entries). The counting half computes them
// and the host reads them back in one 16-byte copy; the rendering half then runs on buffers
// sized from them. Replays reuse the cached sizes, so a replayed frame has no host round trip and
// can be captured into a single CUDA graph.
#include "runtime.h"

#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <mutex>
#include <thread>

#include "launch.h"
#include "noalloc.h"

namespace blgpu {

std::atomic<int> g_last_cuda_error{0};

BLGpuResult cuda_result(cudaError_t e) {
  if (e == cudaSuccess) return BLGPU_SUCCESS;
  g_last_cuda_error.store(int(e));
  if (e == cudaErrorMemoryAllocation) return BLGPU_ERROR_OUT_OF_MEMORY;
  return BLGPU_ERROR_DEVICE;
}

#define BLGPU_CHECK(expr)                              \
  do {                                                 \
    cudaError_t e_ = (expr);                           \
    if (e_ != cudaSuccess) return cuda_result(e_);     \
  } while (0)

int last_cuda_error() { return g_last_cuda_error.load(); }

static inline size_t align_up(size_t x, size_t a) { return (x + a - 1) & ~(a - 1); }

// Device order (LaunchConfig::device_order): the graph-frame pipelines of the runtimes on a device
// that set it are chained: each waits, on its stream, for the kernels of the one enqueued before it.
// Copies stay outside the chain.
namespace {
struct DeviceOrder {
  std::mutex m;
  cudaEvent_t last = nullptr;         // recorded after the last ordered pipeline's kernels
};
DeviceOrder& device_order_of(int device) {
  static DeviceOrder orders[64];
  return orders[unsigned(device) % 64u];
}
}  // namespace

// Bytes per pixel of a canvas: an A8 target stays one byte per pixel on the device as well.
static inline int32_t canvas_bpp(const BLGpuImage& im) { return im.format == BLGPU_FORMAT_A8 ? 1 : 4; }
// Row pitch, in pixels, of a canvas kept in the runtime's canvas pool: rows start at 16 bytes.
static inline int32_t pooled_stride(const BLGpuImage& im) {
  return int32_t(align_up(size_t(uint32_t(im.width)), canvas_bpp(im) == 1 ? 16 : 4));
}
// 32-bit words of the canvas pool a canvas takes (every canvas starts at a 256-byte boundary).
static inline uint64_t pooled_words(const BLGpuImage& im) {
  const uint64_t bytes = uint64_t(pooled_stride(im)) * uint32_t(im.height) * uint32_t(canvas_bpp(im));
  return align_up((bytes + 3) / 4, 64);
}

// --- Frame ------------------------------------------------------------------------------------

// Generations are unique across all frames of the process: a context records into two frames in
// turn, and a style registered in one must not look registered in the other.
static std::atomic<uint64_t> g_frame_generation{1};

uint64_t Frame::next_generation() { return g_frame_generation.fetch_add(1) + 1; }

void Frame::clear() {
  cmds.clear(); styles.clear(); xforms.clear(); canvases.clear(); targets.clear();
  verts.clear(); path_cmds.clear(); lut_jobs.clear(); stops.clear(); images.clear();
  stroke_figs.clear(); stroke_params.clear(); stroke_xy.clear(); stroke_cmds.clear();
  image_words = 0; lut_words = 0; tiles = 0; rows = 0;
  vert_parts.clear(); ext_verts = 0;
  generation = next_generation();
}

static int band_height_for(int width) {
  int bh = 64;
  size_t pixel_count = size_t(unsigned(width)) * size_t(bh);
  do {
    if (pixel_count * 4u <= 1024u * 256u) break;
    bh >>= 1;
    pixel_count >>= 1;
  } while (bh > 8);
  return bh;
}

uint32_t Frame::add_canvas(const BLGpuImage& image, bool upload) {
  DevCanvas cv{};
  cv.w = image.width;
  cv.h = image.height;
  cv.band_height = band_height_for(image.width);
  cv.tiles_x = (image.width + kTileW - 1) / kTileW;
  cv.tiles_y = (image.height + kTileH - 1) / kTileH;
  cv.tile_base = tiles;
  cv.row_base = rows;
  cv.cmd_first = uint32_t(cmds.size());
  cv.cmd_count = 0;
  cv.a8 = image.format == BLGPU_FORMAT_A8 ? 1u : 0u;
  tiles += uint32_t(cv.tiles_x) * uint32_t(cv.tiles_y);
  rows += uint32_t(cv.tiles_y);
  canvases.push_back(cv);
  targets.push_back(FrameTarget{image, upload});
  return uint32_t(canvases.size() - 1);
}

uint64_t Frame::add_image(const BLGpuImage& image) {
  const int32_t bpp = image.format == BLGPU_FORMAT_A8 ? 1 : 4;
  for (const FrameImage& im : images)
    if (im.pixels == image.pixel_data && im.w == image.width && im.h == image.height && im.stride == image.stride &&
        im.bpp == bpp)
      return im.pool_offset;
  FrameImage im;
  im.pixels = image.pixel_data;
  im.stride = image.stride;
  im.w = image.width;
  im.h = image.height;
  im.bpp = bpp;
  im.device = (image.flags & BLGPU_IMAGE_DEVICE_MEMORY) != 0;
  im.pool_offset = image_words;
  const uint64_t bytes = uint64_t(uint32_t(image.width)) * uint32_t(image.height) * uint32_t(bpp);
  image_words += align_up((bytes + 3u) / 4u, 4);
  images.push_back(im);
  return im.pool_offset;
}

void Frame::merge(Frame* const* parts, size_t count, unsigned threads) {
  // where each part's elements start in the merged frame
  struct Base {
    size_t cmd, style, xform, canvas, vert, stop, lut_job, image, fig, param, stroke_vert;
    uint64_t image_words;
    uint32_t lut_words, tiles, rows;
  };
  std::vector<Base> base(count + 1);
  Base acc{};
  for (size_t p = 0; p < count; p++) {
    acc.lut_words = (acc.lut_words + 1u) & ~1u;   // 64-bit (dithered) LUT entries stay 8-byte aligned
    base[p] = acc;
    const Frame& f = *parts[p];
    acc.cmd += f.cmds.size(); acc.style += f.styles.size(); acc.xform += f.xforms.size();
    acc.canvas += f.canvases.size(); acc.vert += f.path_cmds.size(); acc.stop += f.stops.size();
    acc.lut_job += f.lut_jobs.size(); acc.image += f.images.size(); acc.fig += f.stroke_figs.size();
    acc.param += f.stroke_params.size(); acc.stroke_vert += f.stroke_cmds.size();
    acc.image_words += f.image_words; acc.lut_words += f.lut_words; acc.tiles += f.tiles; acc.rows += f.rows;
  }
  // vertices recorded in page-locked memory stay where they are (uploaded part by part)
  bool refer_verts = true;
  for (size_t p = 0; p < count; p++) {
    const Frame& f = *parts[p];
    if (!f.path_cmds.empty() && !(f.verts.ptr_pinned && f.path_cmds.ptr_pinned)) refer_verts = false;
  }
  clear();
  cmds.resize_uninit(acc.cmd); styles.resize_uninit(acc.style); xforms.resize_uninit(acc.xform);
  if (refer_verts) {
    for (size_t p = 0; p < count; p++)
      if (!parts[p]->path_cmds.empty()) vert_parts.push_back(parts[p]);
    ext_verts = acc.vert;
  }
  else {
    verts.resize_uninit(2 * acc.vert); path_cmds.resize_uninit(acc.vert);
  }
  lut_jobs.resize_uninit(acc.lut_job);
  stops.resize_uninit(acc.stop); stroke_figs.resize_uninit(acc.fig); stroke_params.resize_uninit(acc.param);
  stroke_xy.resize_uninit(2 * acc.stroke_vert); stroke_cmds.resize_uninit(acc.stroke_vert);
  canvases.resize(acc.canvas);
  targets.resize(acc.canvas);
  images.resize(acc.image);
  image_words = acc.image_words; lut_words = acc.lut_words; tiles = acc.tiles; rows = acc.rows;

  auto copy_part = [&](size_t p) {
    const Frame& f = *parts[p];
    const Base& o = base[p];
    for (size_t i = 0; i < f.cmds.size(); i++) {
      DevCmd c = f.cmds[i];
      c.canvas += uint32_t(o.canvas);
      c.style += uint32_t(o.style);
      if (c.kind == kFillMaskA) {   // geom_first / xform: the mask's byte offset in the image pool
        const uint64_t off = ((uint64_t(c.xform) << 32) | c.geom_first) + o.image_words * 4u;
        c.geom_first = uint32_t(off);
        c.xform = uint32_t(off >> 32);
      }
      else {
        c.xform += uint32_t(o.xform);
        if (c.kind == kFillAnalytic) c.geom_first += uint32_t(o.vert);
      }
      cmds[o.cmd + i] = c;
    }
    for (size_t i = 0; i < f.styles.size(); i++) {
      DevStyle d = f.styles[i];
      if (d.lut_size) d.lut_offset += o.lut_words;
      if (d.fetch >= kFetchPatAlignedPad) d.src_offset += o.image_words;
      styles[o.style + i] = d;
    }
    if (f.xforms.size()) memcpy(&xforms[o.xform], f.xforms.data(), sizeof(DevXform) * f.xforms.size());
    for (size_t i = 0; i < f.canvases.size(); i++) {
      DevCanvas cv = f.canvases[i];
      cv.tile_base += o.tiles;
      cv.row_base += o.rows;
      cv.cmd_first += uint32_t(o.cmd);
      canvases[o.canvas + i] = cv;
      targets[o.canvas + i] = f.targets[i];
    }
    if (f.path_cmds.size() && !refer_verts) {
      memcpy(&verts[2 * o.vert], f.verts.data(), sizeof(double) * f.verts.size());
      memcpy(&path_cmds[o.vert], f.path_cmds.data(), f.path_cmds.size());
    }
    for (size_t i = 0; i < f.lut_jobs.size(); i++) {
      DevLutJob j = f.lut_jobs[i];
      j.style += uint32_t(o.style);
      j.stop_first += uint32_t(o.stop);
      j.lut_offset += o.lut_words;
      lut_jobs[o.lut_job + i] = j;
    }
    if (f.stops.size()) memcpy(&stops[o.stop], f.stops.data(), sizeof(DevStop) * f.stops.size());
    for (size_t i = 0; i < f.images.size(); i++) {
      FrameImage im = f.images[i];
      im.pool_offset += o.image_words;
      images[o.image + i] = im;
    }
    for (size_t i = 0; i < f.stroke_figs.size(); i++) {
      DevStrokeFig g = f.stroke_figs[i];
      g.first += uint32_t(o.stroke_vert);
      g.end += uint32_t(o.stroke_vert);
      g.cmd += uint32_t(o.cmd);
      g.param += uint32_t(o.param);
      stroke_figs[o.fig + i] = g;
    }
    if (f.stroke_params.size())
      memcpy(&stroke_params[o.param], f.stroke_params.data(), sizeof(DevStrokeParams) * f.stroke_params.size());
    if (f.stroke_cmds.size()) {
      memcpy(&stroke_xy[2 * o.stroke_vert], f.stroke_xy.data(), sizeof(double) * f.stroke_xy.size());
      memcpy(&stroke_cmds[o.stroke_vert], f.stroke_cmds.data(), f.stroke_cmds.size());
    }
  };
  const size_t nt = std::max<size_t>(1, std::min<size_t>(threads, count));
  if (nt == 1) {
    for (size_t p = 0; p < count; p++) copy_part(p);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  for (size_t t = 0; t < nt; t++)
    pool.emplace_back([&] { for (size_t p; (p = next.fetch_add(1)) < count;) copy_part(p); });
  for (auto& th : pool) th.join();
}

// --- device memory ----------------------------------------------------------------------------

cudaError_t DeviceBuffer::reserve(size_t bytes) {
  if (bytes <= size) return cudaSuccess;
  release();
  size_t want = std::max(bytes, size_t(1) << 20);
  want = align_up(want + want / 4, size_t(1) << 20);
  cudaError_t e = cudaMalloc(&ptr, want);
  if (e != cudaSuccess) {
    ptr = nullptr;
    e = cudaMalloc(&ptr, bytes);
    if (e != cudaSuccess) { ptr = nullptr; size = 0; return e; }
    want = bytes;
  }
  size = want;
  return cudaSuccess;
}

void DeviceBuffer::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  size = 0;
}

// Bump allocator over a planned layout: first pass measures, second pass assigns.
struct Layout {
  size_t off = 0;
  char* base = nullptr;
  template <typename T>
  T* take(size_t count) {
    off = align_up(off, 256);
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += sizeof(T) * count;
    return p;
  }
};

// --- runtime ----------------------------------------------------------------------------------

BLGpuResult Runtime::init(const BLGpuRuntimeCreateInfo* info) {
  device = info ? info->device : 0;
  lut_variant = info ? info->lut_variant : kLutSSE2;
  if (lut_variant > kLutScalar) return BLGPU_ERROR_INVALID_VALUE;
  int count = 0;
  BLGPU_CHECK(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) return BLGPU_ERROR_INVALID_VALUE;
  BLGPU_CHECK(cudaSetDevice(device));
  BLGPU_CHECK(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device));
  if (info && info->cuda_stream) {
    stream = static_cast<cudaStream_t>(info->cuda_stream);
    own_stream = false;
  }
  else {
    BLGPU_CHECK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    own_stream = true;
  }
  for (auto& e : ev) BLGPU_CHECK(cudaEventCreate(&e));
  BLGPU_CHECK(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
  BLGPU_CHECK(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
  BLGPU_CHECK(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming));
  BLGPU_CHECK(cudaEventCreateWithFlags(&order_ev, cudaEventDisableTiming));
  BLGPU_CHECK(cudaMallocHost(reinterpret_cast<void**>(&host_totals), 128));
  BLGPU_CHECK(cudaMallocHost(reinterpret_cast<void**>(&host_counts), sizeof(uint32_t) * kCntWords));
  BLGPU_CHECK(cudaMalloc(reinterpret_cast<void**>(&counts_dev), sizeof(uint32_t) * kCntWords));
  return BLGPU_SUCCESS;
}

void Runtime::destroy() {
  cudaSetDevice(device);
  if (stream) cudaStreamSynchronize(stream);
  if (graph) cudaGraphExecDestroy(graph);
  graph = nullptr;
  for (auto& e : ev) if (e) cudaEventDestroy(e);
  if (side) { cudaStreamSynchronize(side); cudaStreamDestroy(side); }
  if (fork_ev) cudaEventDestroy(fork_ev);
  if (join_ev) cudaEventDestroy(join_ev);
  side = nullptr; fork_ev = join_ev = nullptr;
  if (order_ev) {
    DeviceOrder& d = device_order_of(device);
    std::lock_guard<std::mutex> g(d.m);
    if (d.last == order_ev) d.last = nullptr;
    cudaEventDestroy(order_ev);
    order_ev = nullptr;
  }
  in_buf.release();
  dyn_buf.release();
  seg_buf.release();
  stroke_buf.release();
  xfer_buf.release();
  xfers.release();
  if (host_staging) cudaFreeHost(host_staging);
  if (host_totals) cudaFreeHost(host_totals);
  if (host_counts) cudaFreeHost(host_counts);
  if (counts_dev) cudaFree(counts_dev);
  host_totals = host_counts = counts_dev = nullptr;
  if (own_stream && stream) cudaStreamDestroy(stream);
  stream = nullptr;
}

bool device_target_direct(const BLGpuImage& im) {
  return (im.flags & BLGPU_IMAGE_DEVICE_MEMORY) && (reinterpret_cast<uintptr_t>(im.pixel_data) & 15u) == 0 &&
         (im.stride & 15) == 0 && im.stride >= intptr_t(im.width) * canvas_bpp(im);
}

// Stroke sizing: the stroke inputs go to the device and the count pass runs once, so the frame's
// vertex arrays can be planned with room for the outlines (their size comes back to the host).
// The pipeline writes the outlines (and, on a replay, counts again).
BLGpuResult Runtime::prepare_strokes(const Frame& fr, FrameView& v, uint32_t& outline_verts) {
  outline_verts = 0;
  const uint32_t nf = uint32_t(fr.stroke_figs.size());
  v.num_stroke_figs = nf;
  v.stroke_vert_base = uint32_t(fr.vertex_count());
  if (!nf) return BLGPU_SUCCESS;
  // Thread order: a counting sort by vertex count (larger first), join and caps, so a warp's
  // figures run the same branches and loops of similar length (the stroker is FP64-bound and a
  // warp's FP64 instruction costs the same for one lane as for 32).
  stroke_order.resize(nf);
  {
    constexpr uint32_t kBuckets = 64u * 8u * 64u;
    std::vector<uint32_t> keys(nf), start(kBuckets + 1, 0u);
    for (uint32_t i = 0; i < nf; i++) {
      const DevStrokeFig& fg = fr.stroke_figs[i];
      const DevStrokeParams& sp = fr.stroke_params[fg.param];
      const uint32_t nv = std::min<uint32_t>(fg.end - fg.first, 63u);
      keys[i] = ((63u - nv) << 9) | ((sp.join & 7u) << 6) | ((sp.start_cap * 6u + sp.end_cap) & 63u);
      start[keys[i] + 1]++;
    }
    for (uint32_t k = 0; k < kBuckets; k++) start[k + 1] += start[k];
    for (uint32_t i = 0; i < nf; i++) stroke_order[start[keys[i]]++] = i;
  }
  auto plan = [&](Layout& L) {
    v.stroke_figs = L.take<DevStrokeFig>(nf);
    v.stroke_order = L.take<uint32_t>(nf);
    v.stroke_params = L.take<DevStrokeParams>(fr.stroke_params.size());
    v.stroke_xy = L.take<double>(fr.stroke_xy.size());
    v.stroke_cmds = L.take<uint8_t>(fr.stroke_cmds.size());
    v.stroke_counts = L.take<uint4>(nf);
    v.stroke_totals = L.take<uint32_t>(nf + 1);
    v.stroke_offsets = L.take<uint32_t>(nf + 1);
    v.stroke_scan_tmp = L.take<uint32_t>(scan_temp_words(nf + 1));
  };
  Layout measure;
  plan(measure);
  stroke_bytes = measure.off;
  if (measure.off > stroke_buf.size) {
    graph_valid = false;
    BLGPU_CHECK(cudaStreamSynchronize(stream));
    BLGPU_CHECK(stroke_buf.reserve(measure.off));
  }
  Layout L;
  L.base = static_cast<char*>(stroke_buf.ptr);
  plan(L);
  auto put = [&](const void* dst, const void* src, size_t bytes) -> cudaError_t {
    if (!bytes) return cudaSuccess;
    h2d_bytes += bytes;
    return cudaMemcpyAsync(const_cast<void*>(dst), src, bytes, cudaMemcpyHostToDevice, stream);
  };
  BLGPU_CHECK(put(v.stroke_figs, fr.stroke_figs.data(), sizeof(DevStrokeFig) * nf));
  BLGPU_CHECK(put(v.stroke_order, stroke_order.data(), sizeof(uint32_t) * nf));
  BLGPU_CHECK(put(v.stroke_params, fr.stroke_params.data(), sizeof(DevStrokeParams) * fr.stroke_params.size()));
  BLGPU_CHECK(put(v.stroke_xy, fr.stroke_xy.data(), sizeof(double) * fr.stroke_xy.size()));
  BLGPU_CHECK(put(v.stroke_cmds, fr.stroke_cmds.data(), fr.stroke_cmds.size()));
  launch_stroke_count(v, stream);
  BLGPU_CHECK(cudaGetLastError());
  BLGPU_CHECK(cudaMemcpyAsync(host_totals + 16, v.stroke_offsets + nf, 4, cudaMemcpyDeviceToHost, stream));
  d2h_bytes += 4;
  BLGPU_CHECK(cudaStreamSynchronize(stream));
  if (host_totals[16] > 0x3FFFFFFFu) return BLGPU_ERROR_DATA_TOO_LARGE;
  outline_verts = host_totals[16];
  strokes_counted = true;
  return BLGPU_SUCCESS;
}

cudaError_t Runtime::put_counts(const Frame& fr, uint32_t* dev) {
  uint32_t* c = host_counts;
  memset(c, 0, sizeof(uint32_t) * kCntWords);
  c[kCntCmds] = uint32_t(fr.cmds.size());
  c[kCntCanvases] = uint32_t(fr.canvases.size());
  c[kCntTiles] = fr.tiles;
  c[kCntRows] = fr.rows;
  c[kCntLutJobs] = uint32_t(fr.lut_jobs.size());
  c[kCntStrokeFigs] = uint32_t(fr.stroke_figs.size());
  c[kCntStrokeVertBase] = uint32_t(fr.vertex_count());
  h2d_bytes += sizeof(uint32_t) * kCntWords;
  return cudaMemcpyAsync(dev, c, sizeof(uint32_t) * kCntWords, cudaMemcpyHostToDevice, stream);
}

FrameSizes sizes_of(const Frame& fr, uint32_t outline_verts) {
  FrameSizes z;
  z.cmds = uint32_t(fr.cmds.size());
  z.styles = uint32_t(fr.styles.size());
  z.xforms = uint32_t(fr.xforms.size());
  z.canvases = uint32_t(fr.canvases.size());
  z.lut_jobs = uint32_t(fr.lut_jobs.size());
  z.stops = uint32_t(fr.stops.size());
  z.tiles = fr.tiles;
  z.rows = fr.rows;
  z.vert_words = 2 * fr.vertex_count() + 2 * uint64_t(outline_verts);
  z.cmd_bytes = fr.vertex_count() + uint64_t(outline_verts);
  z.image_words = fr.image_words;
  z.lut_words = fr.lut_words;
  for (const FrameTarget& t : fr.targets)
    if (!device_target_direct(t.image))
      z.canvas_words += pooled_words(t.image);
  return z;
}

BLGpuResult Runtime::upload_frame(const Frame& fr, const FrameSizes* caps) {
  const uint32_t ncv = uint32_t(fr.canvases.size());
  h2d_bytes = 0;
  d2h_bytes = 0;

  FrameView v{};
  v.counts = counts_dev;
  // the previous frame (and its read of host_counts) has completed: run() returns when it has
  BLGPU_CHECK(put_counts(fr, counts_dev));
  uint32_t outline_verts = 0;
  strokes_counted = false;
  stroke_bytes = 0;
  BLGpuResult sr = prepare_strokes(fr, v, outline_verts);
  if (sr) return sr;
  const FrameSizes z = caps ? *caps : sizes_of(fr, outline_verts);
  const uint32_t nc = z.cmds;
  const uint64_t vert_words = z.vert_words;   // doubles

  // Items: at most one per vertex (a line or curve consumes at least one; a closing line takes
  // the place of the figure's move-to).
  const uint32_t item_capacity = uint32_t(std::min<uint64_t>(vert_words + 1, 0xFFFFFFF0u));
  // a cubic (3 vertices) splits into at most 8 monotonic pieces, a quadratic (2) into at most 3
  const uint32_t piece_capacity = uint32_t(std::min<uint64_t>(vert_words / 2 * 3 + 64, 0xFFFFFFF0u));

  // Plan: [staged inputs][luts][canvases][work arrays]
  auto plan = [&](Layout& L, FrameView& v, std::vector<uint32_t*>* cpix) -> size_t {
    v.cmds_rw = L.take<DevCmd>(nc);
    v.cmds = v.cmds_rw;
    v.styles = L.take<DevStyle>(z.styles);
    v.xforms = L.take<DevXform>(z.xforms);
    v.canvases = L.take<DevCanvas>(z.canvases);
    v.verts = L.take<double>(vert_words);
    v.path_cmds = L.take<uint8_t>(z.cmd_bytes);
    v.lut_jobs = L.take<DevLutJob>(z.lut_jobs);
    v.stops = L.take<DevStop>(z.stops);
    v.images = L.take<uint32_t>(z.image_words);
    size_t staged_end = align_up(L.off, 256);
    v.luts = L.take<uint32_t>(z.lut_words);
    // canvas pixels (host-memory targets): one pool, every canvas at a 256-byte boundary
    uint32_t* pool = L.take<uint32_t>(z.canvas_words);
    if (cpix) {
      size_t off = 0;
      for (uint32_t i = 0; i < ncv; i++) {
        const BLGpuImage& im = fr.targets[i].image;
        if (device_target_direct(im)) { (*cpix)[i] = static_cast<uint32_t*>(im.pixel_data); continue; }
        (*cpix)[i] = pool ? pool + off : nullptr;
        off += pooled_words(im);
      }
    }
    v.items = L.take<DevItem>(item_capacity);
    v.curve_items = L.take<DevItem>(item_capacity);
    v.pieces = L.take<DevPiece>(piece_capacity);
    v.piece_list = L.take<uint32_t>(piece_capacity);
    v.cmd_bbox = L.take<int4>(nc);
    v.cmd_tile_x = L.take<uint32_t>(nc);
    v.cmd_tile_y = L.take<uint32_t>(nc);
    v.cmd_xr = L.take<uint32_t>(nc);
    v.cmd_yr = L.take<uint32_t>(nc);
    cmdrow_per_cmd = L.take<uint32_t>(nc + 1);
    v.cmdrow_base = L.take<uint32_t>(nc + 1);
    // command-list rows: room for the smallest list-row height
    const size_t list_rows = (size_t(z.rows) << kMaxListLog2) + 1;
    v.row_counts = L.take<uint32_t>(list_rows);
    v.row_offsets = L.take<uint32_t>(list_rows);
    v.row_copies = L.take<uint32_t>(list_rows);
    v.strip_start = L.take<uint32_t>((size_t(z.tiles) + 1) * (kTileH / kStripRows));
    row_canvas = L.take<uint32_t>(list_rows);
    v.tile_order = L.take<uint32_t>(z.tiles + 1);
    v.tile_canvas = L.take<uint32_t>(z.tiles + 1);
    // [0] work queue, [1] line items, [2] cubic curves, [3] their queue, [4..12) totals,
    // [12..16) error flags, [16..20) pixel ops (2 x u64), [21] quadratic / conic curves, [22] their
    // queue
    v.work_counter = L.take<uint32_t>(kCounterWords);
    v.totals = v.work_counter + 4;
    v.error_flags = v.work_counter + 12;
    v.pixel_ops = reinterpret_cast<unsigned long long*>(v.work_counter + 16);
    v.rs_count = L.take<uint32_t>(nc + 1);
    v.rs_base = L.take<uint32_t>(nc + 1);
    v.rb_count = L.take<uint32_t>(nc + 1);
    v.rb_base = L.take<uint32_t>(nc + 1);
    scan_tmp = L.take<uint32_t>(scan_temp_words(std::max<uint32_t>(nc + 1, (z.rows << kMaxListLog2) + 1)));
    return staged_end;
  };

  Layout measure;
  plan(measure, v, nullptr);
  size_t total = measure.off;
  in_bytes = total;
  if (total > in_buf.size) {
    graph_valid = false;
    BLGPU_CHECK(cudaStreamSynchronize(stream));
    BLGPU_CHECK(in_buf.reserve(total));
  }
  Layout L;
  L.base = static_cast<char*>(in_buf.ptr);
  canvas_dev.assign(ncv, nullptr);
  plan(L, v, &canvas_dev);

  // Frame arrays recorded in page-locked memory go to the device by DMA straight from where they
  // were recorded; anything else (the canvas table, pattern images, arrays that had to fall back
  // to pageable memory) is packed into the page-locked staging buffer first.
  size_t pack_bytes = align_up(sizeof(DevCanvas) * ncv, 256);
  auto needs_pack = [&](bool pinned_array, size_t bytes) { if (!pinned_array) pack_bytes += align_up(bytes, 256); };
  needs_pack(fr.cmds.ptr_pinned, sizeof(DevCmd) * fr.cmds.size());
  needs_pack(fr.styles.ptr_pinned, sizeof(DevStyle) * fr.styles.size());
  needs_pack(fr.xforms.ptr_pinned, sizeof(DevXform) * fr.xforms.size());
  needs_pack(fr.verts.ptr_pinned, sizeof(double) * fr.verts.size());
  needs_pack(fr.path_cmds.ptr_pinned, fr.path_cmds.size());     // (a merged frame's vert_parts are page-locked)
  needs_pack(fr.lut_jobs.ptr_pinned, sizeof(DevLutJob) * fr.lut_jobs.size());
  needs_pack(fr.stops.ptr_pinned, sizeof(DevStop) * fr.stops.size());
  for (const FrameImage& im : fr.images)
    if (!im.device) pack_bytes += align_up(size_t(im.w) * size_t(im.h) * size_t(im.bpp), 256);
  // the previous frame's copies out of the staging buffer must have completed
  BLGPU_CHECK(cudaStreamSynchronize(stream));
  if (pack_bytes > host_staging_size) {
    if (host_staging) cudaFreeHost(host_staging);
    host_staging = nullptr;
    size_t want = align_up(pack_bytes + pack_bytes / 4, size_t(1) << 20);
    BLGPU_CHECK(cudaMallocHost(&host_staging, want));
    host_staging_size = want;
  }
  char* hs = static_cast<char*>(host_staging);
  size_t hs_off = 0;
  auto put = [&](const void* dev_ptr, const void* src, size_t bytes, bool src_pinned) -> cudaError_t {
    if (!bytes) return cudaSuccess;
    h2d_bytes += bytes;
    if (!src_pinned) {
      memcpy(hs + hs_off, src, bytes);
      src = hs + hs_off;
      hs_off += align_up(bytes, 256);
    }
    return cudaMemcpyAsync(const_cast<void*>(dev_ptr), src, bytes, cudaMemcpyHostToDevice, stream);
  };
  BLGPU_CHECK(put(v.cmds, fr.cmds.data(), sizeof(DevCmd) * fr.cmds.size(), fr.cmds.ptr_pinned));
  BLGPU_CHECK(put(v.styles, fr.styles.data(), sizeof(DevStyle) * fr.styles.size(), fr.styles.ptr_pinned));
  BLGPU_CHECK(put(v.xforms, fr.xforms.data(), sizeof(DevXform) * fr.xforms.size(), fr.xforms.ptr_pinned));
  std::vector<DevCanvas> cvs = fr.canvases;
  canvas_stride.assign(ncv, 0);
  for (uint32_t i = 0; i < ncv; i++) {
    const BLGpuImage& im = fr.targets[i].image;
    cvs[i].pixels = canvas_dev[i];
    cvs[i].stride = device_target_direct(im) ? int32_t(im.stride / canvas_bpp(im)) : pooled_stride(im);
    canvas_stride[i] = cvs[i].stride;
  }
  BLGPU_CHECK(put(v.canvases, cvs.data(), sizeof(DevCanvas) * ncv, false));
  BLGPU_CHECK(put(v.verts, fr.verts.data(), sizeof(double) * fr.verts.size(), fr.verts.ptr_pinned));
  BLGPU_CHECK(put(v.path_cmds, fr.path_cmds.data(), fr.path_cmds.size(), fr.path_cmds.ptr_pinned));
  {
    size_t at = fr.verts.size() / 2;
    for (const Frame* p : fr.vert_parts) {
      BLGPU_CHECK(put(v.verts + 2 * at, p->verts.data(), sizeof(double) * p->verts.size(), true));
      BLGPU_CHECK(put(v.path_cmds + at, p->path_cmds.data(), p->path_cmds.size(), true));
      at += p->path_cmds.size();
    }
  }
  BLGPU_CHECK(put(v.lut_jobs, fr.lut_jobs.data(), sizeof(DevLutJob) * fr.lut_jobs.size(), fr.lut_jobs.ptr_pinned));
  BLGPU_CHECK(put(v.stops, fr.stops.data(), sizeof(DevStop) * fr.stops.size(), fr.stops.ptr_pinned));
  for (const FrameImage& im : fr.images) {
    if (im.device) continue;
    const size_t row = size_t(im.w) * size_t(im.bpp), bytes = row * size_t(im.h);
    char* dst = hs + hs_off;
    for (int y = 0; y < im.h; y++)
      memcpy(dst + size_t(y) * row, static_cast<const char*>(im.pixels) + intptr_t(y) * im.stride, row);
    hs_off += align_up(bytes, 256);
    h2d_bytes += bytes;
    BLGPU_CHECK(cudaMemcpyAsync(const_cast<uint32_t*>(v.images) + im.pool_offset, dst, bytes, cudaMemcpyHostToDevice, stream));
  }
  for (const FrameImage& im : fr.images) {
    if (!im.device) continue;
    BLGPU_CHECK(cudaMemcpy2DAsync(const_cast<uint32_t*>(v.images) + im.pool_offset, size_t(im.w) * size_t(im.bpp), im.pixels,
                                  size_t(im.stride), size_t(im.w) * size_t(im.bpp), size_t(im.h), cudaMemcpyDeviceToDevice, stream));
  }
  // Canvas content (the pipeline composites onto it).
  BLGpuResult cr = stage_canvases(fr);
  if (cr) return cr;

  // Segment array: kept across frames, sized from the vertex count at first and from the actual
  // count whenever a frame overflows it (run() then repeats the counting half).
  size_t want_segs = std::max<size_t>(size_t(seg_capacity), caps ? size_t(caps->dyn.segs) : size_t(vert_words * 2 + 65536));
  want_segs = std::min<size_t>(want_segs, cfg.max_segments > 0 ? size_t(cfg.max_segments) : size_t(0xFFFFFFF0u));
  if (want_segs > seg_capacity) {
    graph_valid = false;
    BLGpuResult rr = reserve_segments(uint32_t(want_segs));
    if (rr) return rr;
  }
  v.segs = static_cast<DevSeg*>(seg_buf.ptr);
  v.seg_meta = reinterpret_cast<uint32_t*>(static_cast<char*>(seg_buf.ptr) + sizeof(DevSeg) * size_t(seg_capacity));
  v.seg_capacity = cfg.max_segments > 0 ? std::min<uint32_t>(seg_capacity, uint32_t(cfg.max_segments)) : seg_capacity;
  v.item_capacity = item_capacity;
  v.piece_capacity = piece_capacity;
  v.num_cmds = nc;
  v.num_canvases = z.canvases;
  v.num_tiles = z.tiles;
  v.num_rows = z.rows;
  v.num_lut_jobs = z.lut_jobs;
  v.pixels = nullptr;
  view = v;
  targets = fr.targets;
  return BLGPU_SUCCESS;
}

BLGpuResult Runtime::reserve_segments(uint32_t count) {
  BLGPU_CHECK(cudaStreamSynchronize(stream));
  BLGPU_CHECK(seg_buf.reserve(size_t(count) * (sizeof(DevSeg) + sizeof(uint32_t))));
  seg_capacity = uint32_t(std::min<size_t>(seg_buf.size / (sizeof(DevSeg) + sizeof(uint32_t)), 0xFFFFFFF0u));
  return BLGPU_SUCCESS;
}

// Counting half: LUTs, edge building (segments appended), tile ranges, row-list sizes, totals.
int Runtime::enqueue_count_half(cudaStream_t st) {
  view.list_shift = list_shift_of(cfg);
  const FrameView& f = view;
  const uint32_t list_rows = f.num_rows << (kTileShift - f.list_shift);
  int k = 0;
  cudaMemsetAsync(f.work_counter, 0, sizeof(uint32_t) * kCounterWords, st);
  cudaMemsetAsync(f.row_counts, 0, sizeof(uint32_t) * (list_rows + 1), st);
  if (f.num_lut_jobs) {
    cudaEventRecord(fork_ev, st);
    cudaStreamWaitEvent(side, fork_ev, 0);
    k += launch_lut(f, side);
    cudaEventRecord(join_ev, side);
  }
  if (f.num_stroke_figs) {
    if (!strokes_counted) k += launch_stroke_count(f, st);
    strokes_counted = false;      // a replay of this frame counts again
    k += launch_stroke_emit(f, st);
  }
  k += launch_edges(f, cfg, st);
  k += launch_cmd_tiles(f, cmdrow_per_cmd, st);
  k += exclusive_scan(cmdrow_per_cmd, f.cmdrow_base, f.num_cmds, scan_tmp, st);
  k += launch_total(cmdrow_per_cmd, f.cmdrow_base, f.num_cmds, f.totals + 2, st);
  k += exclusive_scan(f.row_counts, f.row_offsets, list_rows, scan_tmp, st);
  k += launch_total(f.row_counts, f.row_offsets, list_rows, f.totals + 3, st);
  k += exclusive_scan(f.rs_count, f.rs_base, f.num_cmds, scan_tmp, st);
  k += launch_total(f.rs_count, f.rs_base, f.num_cmds, f.totals + 4, st);
  k += exclusive_scan(f.rb_count, f.rb_base, f.num_cmds, scan_tmp, st);
  k += launch_total(f.rb_count, f.rb_base, f.num_cmds, f.totals + 6, st);
  return k;
}

// Rendering half: segments binned into (command, strip, tile) slots, row command lists, the
// coverage pass, the composite pass.
int Runtime::enqueue_render_half(cudaStream_t st, bool timed) {
  const FrameView& f = view;
  int k = launch_frame_gate(f, st);
  cudaMemsetAsync(f.cmdrow_counts, 0, sizeof(uint32_t) * (f.num_cmdrows + 1), st);
  cudaMemsetAsync(f.backdrop, 0, sizeof(uint32_t) * kStripRows * (size_t(f.num_cmdrows) + 1), st);
  k += launch_seg_bin(f, 0, st);
  k += launch_backdrop_prefix(f, st);
  k += launch_rows_and_tiles(f, row_canvas, st);
  k += launch_row_states(f, st);
  // the fine stage: coverage (masks of analytic fills) + composite, timed together
  if (timed) cudaEventRecord(ev[1], st);
  k += launch_coverage(f, cfg, f.cmdrow_offsets + f.num_cmdrows + 1, st);
  if (timed) cudaEventRecord(ev[4], st);
  if (f.num_lut_jobs) cudaStreamWaitEvent(st, join_ev, 0);     // the composite reads the LUTs
  k += launch_fine(f, cfg, st);
  if (timed) cudaEventRecord(ev[2], st);
  return k;
}

// Buffers sized by the counting half's totals. Slots with segments are at most min(slots, raster
// work items), and each has one block of masks.
static void plan_dynamic(Layout& L, FrameView& v, const FrameTotals& t) {
  const uint32_t slots = std::min(t.cmdrows, t.seglist);
  v.cmdrow_counts = L.take<uint32_t>(t.cmdrows + 1);
  v.cmdrow_offsets = L.take<uint32_t>(t.cmdrows + 1 + scan_temp_words(t.cmdrows + 1));
  v.slot_cmd = L.take<uint32_t>(t.cmdrows + 1);
  v.slot_mask = L.take<uint32_t>(t.cmdrows + 1);
  v.slot_first = L.take<uint32_t>(t.cmdrows + 2);
  v.backdrop = L.take<uint32_t>((size_t(t.cmdrows) + 1) * kStripRows);
  v.entries = L.take<uint2>(size_t(t.seglist) + 1);
  v.mask_slot = L.take<uint32_t>(size_t(slots) + 1);
  v.mask_info = L.take<uint4>(size_t(slots) + 1);
  v.masks = L.take<uint8_t>((size_t(slots) + 1) * kStripRows * kTileW);
  v.row_box = L.take<uint2>(size_t(t.row_entries) + 1);
  v.row_recs = L.take<uint4>(2 * (size_t(t.row_entries) + 1));
  v.row_states = L.take<float4>(t.row_states + 1);
  v.mask_capacity = slots + 1;
  v.num_segs = t.segs;
  v.num_cmdrows = t.cmdrows;
  v.num_seglist = t.seglist;
  v.num_row_states = t.row_states;
  v.num_row_runs = t.row_runs;
  v.num_row_entries = t.row_entries;
}

BLGpuResult Runtime::stage_canvases(const Frame& fr) {
  const uint32_t ncv = uint32_t(fr.canvases.size());
  xfers.clear();
  canvas_xfer.assign(ncv, -1);
  // Page-locked canvases move by a copy kernel, which beats one DMA copy per canvas when the frame
  // has the device to itself. Under device order another runtime's kernels are running, and the
  // copy engines then move them without taking any SM time from those kernels.
  for (uint32_t i = 0; i < ncv && !cfg.device_order; i++) {
    const BLGpuImage& im = fr.targets[i].image;
    if (device_target_direct(im) || im.width == 0 || im.height == 0 || (im.flags & BLGPU_IMAGE_DEVICE_MEMORY) ||
        (im.stride % canvas_bpp(im)) != 0)
      continue;
    // page-locked host memory is reachable from the device at the address the driver reports
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, im.pixel_data) != cudaSuccess) { cudaGetLastError(); continue; }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) continue;
    canvas_xfer[i] = int32_t(xfers.size());
    xfers.push_back(DevXfer{canvas_dev[i], static_cast<uint32_t*>(a.devicePointer), im.width, im.height,
                            canvas_stride[i], int32_t(im.stride / canvas_bpp(im)), canvas_bpp(im) == 1 ? 1 : 0, 0});
  }
  if (!xfers.empty()) {
    BLGPU_CHECK(xfer_buf.reserve(sizeof(DevXfer) * xfers.size()));
    BLGPU_CHECK(cudaMemcpyAsync(xfer_buf.ptr, xfers.data(), sizeof(DevXfer) * xfers.size(), cudaMemcpyHostToDevice, stream));
  }
  // canvases the frame composites onto: their content goes up first
  std::vector<DevXfer> up;
  for (uint32_t i = 0; i < ncv; i++) {
    const FrameTarget& t = fr.targets[i];
    const BLGpuImage& im = t.image;
    if (!t.upload || device_target_direct(im) || im.width == 0 || im.height == 0) continue;
    const bool dev = (im.flags & BLGPU_IMAGE_DEVICE_MEMORY) != 0;
    const size_t bpp = size_t(canvas_bpp(im));
    if (!dev) h2d_bytes += uint64_t(uint32_t(im.width)) * uint32_t(im.height) * bpp;
    if (canvas_xfer[i] >= 0) continue;
    BLGPU_CHECK(cudaMemcpy2DAsync(canvas_dev[i], size_t(canvas_stride[i]) * bpp, im.pixel_data, size_t(im.stride),
                                  size_t(im.width) * bpp, size_t(im.height),
                                  dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, stream));
  }
  // the kernel copy of the page-locked ones, when any of them is uploaded: copy all of them up
  // unless none needs it (those that do not are overwritten by their first fill anyway)
  bool any_up = false;
  for (uint32_t i = 0; i < ncv; i++) any_up |= canvas_xfer[i] >= 0 && fr.targets[i].upload;
  if (any_up) {
    up.reserve(xfers.size());
    for (uint32_t i = 0; i < ncv; i++)
      if (canvas_xfer[i] >= 0 && fr.targets[i].upload) up.push_back(xfers[size_t(canvas_xfer[i])]);
    // a separate table after the download table (the stream orders the copy before the kernel)
    const size_t off = align_up(sizeof(DevXfer) * xfers.size(), 256);
    BLGPU_CHECK(xfer_buf.reserve(off + sizeof(DevXfer) * up.size()));
    DevXfer* dev_up = reinterpret_cast<DevXfer*>(static_cast<char*>(xfer_buf.ptr) + off);
    if (!xfers.empty())   // the reserve above may have moved the table
      BLGPU_CHECK(cudaMemcpyAsync(xfer_buf.ptr, xfers.data(), sizeof(DevXfer) * xfers.size(), cudaMemcpyHostToDevice, stream));
    BLGPU_CHECK(cudaMemcpyAsync(dev_up, up.data(), sizeof(DevXfer) * up.size(), cudaMemcpyHostToDevice, stream));
    launch_canvas_copy(dev_up, uint32_t(up.size()), 0, stream);
    BLGPU_CHECK(cudaGetLastError());
    BLGPU_CHECK(cudaStreamSynchronize(stream));      // `up` is pageable: its copy must be done
  }
  return BLGPU_SUCCESS;
}

BLGpuResult Runtime::download() {
  if (!xfers.empty()) {
    launch_canvas_copy(static_cast<const DevXfer*>(xfer_buf.ptr), uint32_t(xfers.size()), 1, stream);
    BLGPU_CHECK(cudaGetLastError());
  }
  for (size_t i = 0; i < targets.size(); i++) {
    const BLGpuImage& im = targets[i].image;
    if (device_target_direct(im) || im.width == 0 || im.height == 0) continue;
    const size_t bpp = size_t(canvas_bpp(im));
    if (i < canvas_xfer.size() && canvas_xfer[i] >= 0) {
      d2h_bytes += uint64_t(uint32_t(im.width)) * uint32_t(im.height) * bpp;
      continue;
    }
    bool dev = (im.flags & BLGPU_IMAGE_DEVICE_MEMORY) != 0;
    if (!dev) d2h_bytes += uint64_t(uint32_t(im.width)) * uint32_t(im.height) * bpp;
    BLGPU_CHECK(cudaMemcpy2DAsync(im.pixel_data, size_t(im.stride), canvas_dev[i], size_t(canvas_stride[i]) * bpp,
                                  size_t(im.width) * bpp, size_t(im.height),
                                  dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, stream));
  }
  return BLGPU_SUCCESS;
}

static double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

BLGpuResult Runtime::run(const Frame& fr) {
  const auto t0 = std::chrono::steady_clock::now();
  BLGpuResult r = run_frame(fr);
  stats.last_run_ms = ms_since(t0);
  return r;
}

BLGpuResult Runtime::upload(const Frame& fr, const FrameSizes* caps) {
  const auto t0 = std::chrono::steady_clock::now();
  BLGpuResult r = upload_frame(fr, caps);
  stats.last_upload_ms = ms_since(t0);
  return r;
}

BLGpuResult Runtime::run_frame(const Frame& fr) {
  if (cfg.graph_frames && fr.stroke_figs.empty()) {
    // a graph frame that does not fit is re-run eagerly, so its device targets must be redrawable:
    // either copied (host targets, unaligned device rows) or overwritten by the frame's first fill
    bool redrawable = true;
    for (const FrameTarget& t : fr.targets) redrawable &= !device_target_direct(t.image) || !t.upload;
    if (redrawable) return run_graph(fr);
  }
  return run_eager(fr);
}

static uint32_t grow_u32(uint64_t v) { return uint32_t(std::min<uint64_t>(v + v / 4 + 64, 0xFFFFFFF0u)); }
static uint64_t grow_u64(uint64_t v) { return v + v / 4 + 256; }

static void raise_caps(FrameSizes& c, const FrameSizes& need) {
  auto up32 = [](uint32_t& cap, uint32_t want) { if (want > cap) cap = grow_u32(want); };
  auto up64 = [](uint64_t& cap, uint64_t want) { if (want > cap) cap = grow_u64(want); };
  up32(c.cmds, need.cmds); up32(c.styles, need.styles); up32(c.xforms, need.xforms);
  up32(c.canvases, need.canvases); up32(c.lut_jobs, need.lut_jobs); up32(c.stops, need.stops);
  up32(c.tiles, need.tiles); up32(c.rows, need.rows);
  up64(c.vert_words, need.vert_words); up64(c.cmd_bytes, need.cmd_bytes); up64(c.image_words, need.image_words);
  up64(c.lut_words, need.lut_words); up64(c.canvas_words, need.canvas_words);
}

static void raise_dyn(FrameTotals& c, const FrameTotals& t) {
  auto up = [](uint32_t& cap, uint32_t want) { if (want > cap) cap = grow_u32(want); };
  up(c.segs, t.segs); up(c.seglist, t.seglist); up(c.cmdrows, t.cmdrows);
  up(c.row_entries, t.row_entries); up(c.row_states, t.row_states); up(c.row_runs, t.row_runs);
}

// A frame as one launch of the captured graph. Every array is laid out by the capacities in
// `caps` (the first frame runs eagerly to learn the sizes the device computes), so the layout and
// with it the graph stay the same for every frame that fits: the frame's data is copied in place,
// the graph replayed, and the host reads back only the totals and flags after it. A frame whose
// inputs exceed the capacities grows them (the graph is captured again); one whose device-computed
// sizes exceed them skips its rendering half on the device (frame_gate_kernel) and runs again
// eagerly after the capacities grow.
BLGpuResult Runtime::run_graph(const Frame& fr) {
  BLGPU_CHECK(cudaSetDevice(device));
  for (const FrameTarget& t : fr.targets)
    if (t.image.width < 0 || t.image.height < 0) return BLGPU_ERROR_INVALID_VALUE;
  const FrameSizes need = sizes_of(fr, 0);
  if (!caps_ready) {
    BLGpuResult r = run_eager(fr);
    if (r) return r;
    caps = FrameSizes{};
    raise_caps(caps, need);
    raise_dyn(caps.dyn, totals);
    caps_ready = true;
    graph_valid = false;
    return BLGPU_SUCCESS;
  }
  if (!need.fits_in(caps)) {
    raise_caps(caps, need);
    graph_valid = false;
  }
  has_frame = false;
  pending_timing = 0;
  const void* in_ptr = in_buf.ptr;
  BLGpuResult r = upload(fr, &caps);
  if (r) return r;
  if (in_buf.ptr != in_ptr) graph_valid = false;
  Layout measure;
  FrameView probe = view;
  plan_dynamic(measure, probe, caps.dyn);
  if (measure.off > dyn_buf.size) {
    BLGPU_CHECK(cudaStreamSynchronize(stream));
    BLGPU_CHECK(dyn_buf.reserve(measure.off));
    graph_valid = false;
  }
  Layout L;
  L.base = static_cast<char*>(dyn_buf.ptr);
  plan_dynamic(L, view, caps.dyn);
  totals = caps.dyn;
  view_by_caps = true;
  planned_list_shift = list_shift_of(cfg);
  if (!graph_valid) {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    cudaGraph_t g = nullptr;
    BLGPU_CHECK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int launches = enqueue_count_half(stream);
    launches += enqueue_render_half(stream, false);
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (e != cudaSuccess) return cuda_result(e);
    e = cudaGraphInstantiate(&graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { graph = nullptr; return cuda_result(e); }
    graph_valid = true;
    stats.kernel_launches = uint64_t(launches);
  }
  {
    std::unique_lock<std::mutex> order;
    if (cfg.device_order) {
      DeviceOrder& d = device_order_of(device);
      order = std::unique_lock<std::mutex>(d.m);
      if (d.last && d.last != order_ev) BLGPU_CHECK(cudaStreamWaitEvent(stream, d.last, 0));
    }
    BLGPU_CHECK(cudaEventRecord(ev[0], stream));
    BLGPU_CHECK(cudaGraphLaunch(graph, stream));
    BLGPU_CHECK(cudaEventRecord(ev[3], stream));
    if (order) {
      BLGPU_CHECK(cudaEventRecord(order_ev, stream));
      device_order_of(device).last = order_ev;
    }
  }
  BLGPU_CHECK(cudaMemcpyAsync(host_totals, view.totals, 32, cudaMemcpyDeviceToHost, stream));
  BLGPU_CHECK(cudaMemcpyAsync(host_totals + 20, view.error_flags, 32, cudaMemcpyDeviceToHost, stream));
  d2h_bytes += 64;
  // The canvases go back in the same round trip. When the frame turns out not to fit, its render
  // half did not run: each canvas that was uploaded comes back unchanged, and the others are
  // overwritten whole by their first command when the frame runs again below.
  r = download();
  if (r) return r;
  BLGPU_CHECK(cudaStreamSynchronize(stream));
  FrameTotals t;
  t.segs = host_totals[0]; t.seglist = host_totals[1]; t.cmdrows = host_totals[2];
  t.row_entries = host_totals[3]; t.row_states = host_totals[4]; t.row_runs = host_totals[6];
  if (host_totals[20]) {
    // the device-computed sizes did not fit: grow to them and render this frame eagerly
    raise_dyn(caps.dyn, t);
    graph_valid = false;
    return run_eager(fr);
  }
  has_frame = true;
  graph_frames_run++;
  read_pixel_ops();
  totals = t;   // the frame's own sizes (the arrays keep their capacities)
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev[0], ev[3]);
  stats.last_gpu_ms = ms;
  stats.frames++;
  stats.fill_commands = fr.cmds.size();
  stats.segments = t.segs;
  stats.tiles = fr.tiles;
  stats.input_vertices = fr.vertex_count();
  stats.h2d_bytes = h2d_bytes;
  stats.d2h_bytes = d2h_bytes;
  last_frame_bytes = in_bytes + measure.off + uint64_t(caps.dyn.segs) * (sizeof(DevSeg) + sizeof(uint32_t));
  return BLGPU_SUCCESS;
}

BLGpuResult Runtime::run_eager(const Frame& fr) {
  BLGPU_CHECK(cudaSetDevice(device));
  for (const FrameTarget& t : fr.targets)
    if (t.image.width < 0 || t.image.height < 0) return BLGPU_ERROR_INVALID_VALUE;
  graph_valid = false;
  has_frame = false;
  pending_timing = 0;
  BLGpuResult r = upload(fr);
  if (r) return r;

  BLGPU_CHECK(cudaEventRecord(ev[0], stream));
  int launches = enqueue_count_half(stream);
  BLGPU_CHECK(cudaGetLastError());
  BLGPU_CHECK(cudaMemcpyAsync(host_totals, view.totals, 32, cudaMemcpyDeviceToHost, stream));
  d2h_bytes += 32;
  BLGPU_CHECK(cudaStreamSynchronize(stream));
  if (host_totals[0] > view.seg_capacity) {
    if (cfg.max_segments > 0 && host_totals[0] > uint32_t(cfg.max_segments)) return BLGPU_ERROR_DATA_TOO_LARGE;
    // more segments than slots: grow and repeat the counting half (it is idempotent)
    r = reserve_segments(uint32_t(std::min<uint64_t>(uint64_t(host_totals[0]) * 5 / 4 + 1024, 0xFFFFFFF0u)));
    if (r) return r;
    view.segs = static_cast<DevSeg*>(seg_buf.ptr);
    view.seg_meta = reinterpret_cast<uint32_t*>(static_cast<char*>(seg_buf.ptr) + sizeof(DevSeg) * size_t(seg_capacity));
    view.seg_capacity = cfg.max_segments > 0 ? std::min<uint32_t>(seg_capacity, uint32_t(cfg.max_segments)) : seg_capacity;
    BLGPU_CHECK(cudaEventRecord(ev[0], stream));
    launches = enqueue_count_half(stream);
    BLGPU_CHECK(cudaGetLastError());
    BLGPU_CHECK(cudaMemcpyAsync(host_totals, view.totals, 32, cudaMemcpyDeviceToHost, stream));
    d2h_bytes += 32;
    BLGPU_CHECK(cudaStreamSynchronize(stream));
    if (host_totals[0] > view.seg_capacity) return BLGPU_ERROR_OUT_OF_MEMORY;
  }
  totals.segs = host_totals[0];
  totals.seglist = host_totals[1];
  totals.cmdrows = host_totals[2];
  totals.row_entries = host_totals[3];
  totals.row_states = host_totals[4];
  totals.row_runs = host_totals[6];

  // Dynamic buffers.
  Layout measure;
  FrameView probe = view;
  plan_dynamic(measure, probe, totals);
  if (measure.off > dyn_buf.size) BLGPU_CHECK(dyn_buf.reserve(measure.off));
  Layout L;
  L.base = static_cast<char*>(dyn_buf.ptr);
  plan_dynamic(L, view, totals);
  view_by_caps = false;
  planned_list_shift = list_shift_of(cfg);
  last_frame_bytes = in_bytes + stroke_bytes + measure.off + uint64_t(totals.segs) * (sizeof(DevSeg) + sizeof(uint32_t));

  launches += enqueue_render_half(stream, true);
  BLGPU_CHECK(cudaGetLastError());
  BLGPU_CHECK(cudaEventRecord(ev[3], stream));
  // error flags and pixel-op counters in one read-back
  BLGPU_CHECK(cudaMemcpyAsync(host_totals + 20, view.error_flags, 32, cudaMemcpyDeviceToHost, stream));
  r = download();
  if (r) return r;
  BLGPU_CHECK(cudaStreamSynchronize(stream));
  if (host_totals[20]) return BLGPU_ERROR_DATA_TOO_LARGE;   // a work array overflowed: pixels invalid
  has_frame = true;
  read_pixel_ops();
  stats.input_vertices = fr.vertex_count() + uint64_t(fr.stroke_xy.size() / 2);
  stats.h2d_bytes = h2d_bytes;
  stats.d2h_bytes = d2h_bytes + 32;

  float ms = 0.f, fine_ms = 0.f;
  cudaEventElapsedTime(&ms, ev[0], ev[3]);
  cudaEventElapsedTime(&fine_ms, ev[1], ev[2]);
  float comp_ms = 0.f;
  cudaEventElapsedTime(&comp_ms, ev[4], ev[2]);
  stats.last_composite_ms = comp_ms;
  stats.frames++;
  stats.fill_commands = view.num_cmds;
  stats.segments = totals.segs;
  stats.tiles = view.num_tiles;
  stats.kernel_launches = uint64_t(launches);
  stats.last_gpu_ms = ms;
  stats.last_fine_ms = fine_ms;
  return BLGPU_SUCCESS;
}

// One frame, one device-memory canvas, every device buffer carved out of the fixed scratch area
// (noalloc.h): no allocating call at all. Inputs are copied straight from the frame's host vectors.
// The runtime's own frame (kept for replay) is left untouched.
BLGpuResult Runtime::run_noalloc(const Frame& fr) {
  // stroke outlines are sized on the device first; that needs buffers this path does not have
  if (!fr.stroke_figs.empty()) return BLGPU_ERROR_NOT_IMPLEMENTED;
  BLGPU_CHECK(cudaSetDevice(device));
  if (fr.canvases.size() != 1 || !device_target_direct(fr.targets[0].image)) return BLGPU_ERROR_INVALID_VALUE;
  void* arena = nullptr;
  BLGPU_CHECK(noalloc_arena(device, &arena));
  const uint32_t nc = uint32_t(fr.cmds.size());
  const uint32_t item_capacity = uint32_t(std::min<size_t>(fr.verts.size() / 2 + 1, 0xFFFFFFF0u));   // <= one per vertex
  const uint32_t piece_capacity = uint32_t(std::min<size_t>(fr.verts.size() / 2 * 3 + 64, 0xFFFFFFF0u));

  FrameView v{};
  uint32_t* a_cmdrow_per_cmd = nullptr;
  uint32_t* a_row_canvas = nullptr;
  uint32_t* a_scan_tmp = nullptr;
  auto plan_fixed = [&](Layout& L) {
    v.cmds_rw = L.take<DevCmd>(nc);
    v.cmds = v.cmds_rw;
    v.styles = L.take<DevStyle>(fr.styles.size());
    v.xforms = L.take<DevXform>(fr.xforms.size());
    v.canvases = L.take<DevCanvas>(1);
    v.verts = L.take<double>(fr.verts.size());
    v.path_cmds = L.take<uint8_t>(fr.path_cmds.size());
    v.lut_jobs = L.take<DevLutJob>(fr.lut_jobs.size());
    v.stops = L.take<DevStop>(fr.stops.size());
    v.images = L.take<uint32_t>(fr.image_words);
    v.luts = L.take<uint32_t>(fr.lut_words);
    v.items = L.take<DevItem>(item_capacity);
    v.curve_items = L.take<DevItem>(item_capacity);
    v.pieces = L.take<DevPiece>(piece_capacity);
    v.piece_list = L.take<uint32_t>(piece_capacity);
    v.cmd_bbox = L.take<int4>(nc);
    v.cmd_tile_x = L.take<uint32_t>(nc);
    v.cmd_tile_y = L.take<uint32_t>(nc);
    v.cmd_xr = L.take<uint32_t>(nc);
    v.cmd_yr = L.take<uint32_t>(nc);
    a_cmdrow_per_cmd = L.take<uint32_t>(nc + 1);
    v.cmdrow_base = L.take<uint32_t>(nc + 1);
    const size_t list_rows = (size_t(fr.rows) << kMaxListLog2) + 1;
    v.row_counts = L.take<uint32_t>(list_rows);
    v.row_offsets = L.take<uint32_t>(list_rows);
    v.row_copies = L.take<uint32_t>(list_rows);
    v.strip_start = L.take<uint32_t>((size_t(fr.tiles) + 1) * (kTileH / kStripRows));
    a_row_canvas = L.take<uint32_t>(list_rows);
    v.tile_order = L.take<uint32_t>(fr.tiles + 1);
    v.tile_canvas = L.take<uint32_t>(fr.tiles + 1);
    v.work_counter = L.take<uint32_t>(kCounterWords);
    v.totals = v.work_counter + 4;
    v.error_flags = v.work_counter + 12;
    v.pixel_ops = reinterpret_cast<unsigned long long*>(v.work_counter + 16);
    v.rs_count = L.take<uint32_t>(nc + 1);
    v.rs_base = L.take<uint32_t>(nc + 1);
    v.rb_count = L.take<uint32_t>(nc + 1);
    v.rb_base = L.take<uint32_t>(nc + 1);
    a_scan_tmp = L.take<uint32_t>(scan_temp_words(std::max<uint32_t>(nc + 1, (fr.rows << kMaxListLog2) + 1)));
    v.counts = L.take<uint32_t>(kCntWords);
  };
  Layout L;
  L.base = static_cast<char*>(arena);
  plan_fixed(L);
  size_t fixed_end = align_up(L.off, 256);
  if (fixed_end >= kNoAllocArenaBytes) return BLGPU_ERROR_DATA_TOO_LARGE;
  // half of what is left holds segments (20 bytes each), the other half the binning lists
  const size_t seg_bytes = ((kNoAllocArenaBytes - fixed_end) / 2) & ~size_t(255);
  v.seg_capacity = uint32_t(seg_bytes / (sizeof(DevSeg) + sizeof(uint32_t)));
  v.segs = reinterpret_cast<DevSeg*>(static_cast<char*>(arena) + fixed_end);
  v.seg_meta = reinterpret_cast<uint32_t*>(static_cast<char*>(arena) + fixed_end + sizeof(DevSeg) * size_t(v.seg_capacity));
  const size_t dyn_begin = fixed_end + seg_bytes;
  v.item_capacity = item_capacity;
  v.piece_capacity = piece_capacity;
  v.num_cmds = nc;
  v.num_canvases = 1;
  v.num_tiles = fr.tiles;
  v.num_rows = fr.rows;
  v.num_lut_jobs = uint32_t(fr.lut_jobs.size());

  auto put = [&](const void* dev, const void* src, size_t bytes) -> cudaError_t {
    if (!bytes) return cudaSuccess;
    return cudaMemcpyAsync(const_cast<void*>(dev), src, bytes, cudaMemcpyHostToDevice, stream);
  };
  DevCanvas cv = fr.canvases[0];
  const BLGpuImage& im = fr.targets[0].image;
  cv.pixels = static_cast<uint32_t*>(im.pixel_data);
  cv.stride = int32_t(im.stride / canvas_bpp(im));
  uint32_t counts[kCntWords] = {};
  counts[kCntCmds] = nc;
  counts[kCntCanvases] = 1;
  counts[kCntTiles] = fr.tiles;
  counts[kCntRows] = fr.rows;
  counts[kCntLutJobs] = uint32_t(fr.lut_jobs.size());
  counts[kCntStrokeVertBase] = uint32_t(fr.verts.size() / 2);
  BLGPU_CHECK(put(v.counts, counts, sizeof(counts)));     // pageable: staged before the call returns
  BLGPU_CHECK(put(v.cmds, fr.cmds.data(), sizeof(DevCmd) * nc));
  BLGPU_CHECK(put(v.styles, fr.styles.data(), sizeof(DevStyle) * fr.styles.size()));
  BLGPU_CHECK(put(v.xforms, fr.xforms.data(), sizeof(DevXform) * fr.xforms.size()));
  BLGPU_CHECK(put(v.canvases, &cv, sizeof(DevCanvas)));
  BLGPU_CHECK(put(v.verts, fr.verts.data(), sizeof(double) * fr.verts.size()));
  BLGPU_CHECK(put(v.path_cmds, fr.path_cmds.data(), fr.path_cmds.size()));
  BLGPU_CHECK(put(v.lut_jobs, fr.lut_jobs.data(), sizeof(DevLutJob) * fr.lut_jobs.size()));
  BLGPU_CHECK(put(v.stops, fr.stops.data(), sizeof(DevStop) * fr.stops.size()));
  for (const FrameImage& fi : fr.images) {
    BLGPU_CHECK(cudaMemcpy2DAsync(const_cast<uint32_t*>(v.images) + fi.pool_offset, size_t(fi.w) * size_t(fi.bpp), fi.pixels,
                                  size_t(fi.stride), size_t(fi.w) * size_t(fi.bpp), size_t(fi.h),
                                  fi.device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, stream));
  }

  // the pipeline halves read the runtime's current view: point it at the arena for this call
  const FrameView saved_view = view;
  uint32_t* const saved[3] = {cmdrow_per_cmd, row_canvas, scan_tmp};
  auto restore = [&]() {
    view = saved_view;
    cmdrow_per_cmd = saved[0]; row_canvas = saved[1]; scan_tmp = saved[2];
  };
  view = v;
  cmdrow_per_cmd = a_cmdrow_per_cmd; row_canvas = a_row_canvas; scan_tmp = a_scan_tmp;

  BLGpuResult r = BLGPU_SUCCESS;
  do {
    int launches = enqueue_count_half(stream);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(host_totals, view.totals, 32, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) { r = cuda_result(e); break; }
    FrameTotals t;
    t.segs = host_totals[0];
    t.seglist = host_totals[1];
    t.cmdrows = host_totals[2];
    t.row_entries = host_totals[3];
    t.row_states = host_totals[4];
    t.row_runs = host_totals[6];
    if (t.segs > view.seg_capacity) { r = BLGPU_ERROR_DATA_TOO_LARGE; break; }
    Layout D;
    D.base = static_cast<char*>(arena);
    D.off = dyn_begin;
    plan_dynamic(D, view, t);
    if (D.off > kNoAllocArenaBytes) { r = BLGPU_ERROR_DATA_TOO_LARGE; break; }
    launches += enqueue_render_half(stream, false);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(host_totals + 20, view.error_flags, 4, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) { r = cuda_result(e); break; }
    if (host_totals[20]) { r = BLGPU_ERROR_DATA_TOO_LARGE; break; }
    (void)launches;               // the runtime's stats describe its own (kept) frame only
  } while (false);
  cudaStreamSynchronize(side);                 // a LUT build forked before an early exit
  restore();
  return r;
}

// Re-runs the last frame's device pipeline on its device-resident inputs and canvases (the
// canvases keep what the previous run left in them). Asynchronous with respect to the host.
BLGpuResult Runtime::resize_dynamic() {
  BLGPU_CHECK(cudaSetDevice(device));
  enqueue_count_half(stream);
  BLGPU_CHECK(cudaGetLastError());
  BLGPU_CHECK(cudaMemcpyAsync(host_totals, view.totals, 32, cudaMemcpyDeviceToHost, stream));
  BLGPU_CHECK(cudaStreamSynchronize(stream));
  BLGPU_CHECK(cudaStreamSynchronize(side));
  FrameTotals t;
  t.segs = host_totals[0]; t.seglist = host_totals[1]; t.cmdrows = host_totals[2];
  t.row_entries = host_totals[3]; t.row_states = host_totals[4]; t.row_runs = host_totals[6];
  FrameTotals plan_t = t;
  if (view_by_caps) { raise_dyn(caps.dyn, t); plan_t = caps.dyn; }
  Layout measure;
  FrameView probe = view;
  plan_dynamic(measure, probe, plan_t);
  if (measure.off > dyn_buf.size) BLGPU_CHECK(dyn_buf.reserve(measure.off));
  Layout L;
  L.base = static_cast<char*>(dyn_buf.ptr);
  plan_dynamic(L, view, plan_t);
  totals = t;
  planned_list_shift = list_shift_of(cfg);
  graph_valid = false;
  return BLGPU_SUCCESS;
}

BLGpuResult Runtime::replay(bool use_graph) {
  if (!has_frame) return BLGPU_ERROR_INVALID_STATE;
  BLGPU_CHECK(cudaSetDevice(device));
  if (planned_list_shift != list_shift_of(cfg)) {
    BLGpuResult r = resize_dynamic();
    if (r) return r;
  }
  if (!use_graph) {
    BLGPU_CHECK(cudaEventRecord(ev[0], stream));
    int launches = enqueue_count_half(stream);
    launches += enqueue_render_half(stream, true);
    BLGPU_CHECK(cudaGetLastError());
    BLGPU_CHECK(cudaEventRecord(ev[3], stream));
    stats.kernel_launches = uint64_t(launches);
    pending_timing = 2;
    return BLGPU_SUCCESS;
  }
  if (!graph_valid) {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    cudaGraph_t g = nullptr;
    BLGPU_CHECK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int launches = enqueue_count_half(stream);
    launches += enqueue_render_half(stream, false);
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (e != cudaSuccess) return cuda_result(e);
    e = cudaGraphInstantiate(&graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { graph = nullptr; return cuda_result(e); }
    graph_valid = true;
    stats.kernel_launches = uint64_t(launches);
  }
  BLGPU_CHECK(cudaEventRecord(ev[0], stream));
  BLGPU_CHECK(cudaGraphLaunch(graph, stream));
  BLGPU_CHECK(cudaEventRecord(ev[3], stream));
  pending_timing = 1;
  return BLGPU_SUCCESS;
}

void Runtime::read_pixel_ops() {
  uint64_t v[2];
  memcpy(v, host_totals + 24, sizeof(v));
  stats.pixel_ops = v[0];
  stats.pattern_ops = v[1];
}

// Launch-shape autotuner: coordinate descent over the LaunchConfig fields, each candidate timed
// by replaying the last frame (median of `trials` eager replays, CUDA events). The canvases are
// saved before and restored after, so the frame's pixels are unchanged.
BLGpuResult Runtime::autotune(int trials, LaunchConfig* best_out, double* best_ms_out) {
  if (!has_frame) return BLGPU_ERROR_INVALID_STATE;
  BLGPU_CHECK(cudaSetDevice(device));
  BLGPU_CHECK(cudaStreamSynchronize(stream));
  if (trials < 1) trials = 3;
  // save every canvas
  size_t bytes = 0;
  for (size_t i = 0; i < targets.size(); i++)
    bytes += size_t(targets[i].image.height) * size_t(canvas_stride[i]) * size_t(canvas_bpp(targets[i].image));
  void* save = nullptr;
  if (bytes) BLGPU_CHECK(cudaMalloc(&save, bytes));
  auto copy_canvases = [&](bool to_save) -> cudaError_t {
    size_t off = 0;
    for (size_t i = 0; i < targets.size(); i++) {
      size_t pitch = size_t(canvas_stride[i]) * size_t(canvas_bpp(targets[i].image)), h = size_t(targets[i].image.height);
      char* a = static_cast<char*>(save) + off;
      cudaError_t e = to_save ? cudaMemcpyAsync(a, canvas_dev[i], pitch * h, cudaMemcpyDeviceToDevice, stream)
                              : cudaMemcpyAsync(canvas_dev[i], a, pitch * h, cudaMemcpyDeviceToDevice, stream);
      if (e != cudaSuccess) return e;
      off += pitch * h;
    }
    return cudaSuccess;
  };
  cudaError_t e = copy_canvases(true);
  auto measure = [&](const LaunchConfig& c, double& ms) -> BLGpuResult {
    cfg = c;
    std::vector<double> t;
    for (int k = 0; k < trials + 1; k++) {
      BLGpuResult r = replay(false);
      if (r) return r;
      r = synchronize();
      if (r) return r;
      if (k) t.push_back(stats.last_gpu_ms);   // the first run warms caches and lazy set-up
    }
    std::sort(t.begin(), t.end());
    ms = t[t.size() / 2];
    return BLGPU_SUCCESS;
  };
  BLGpuResult r = e == cudaSuccess ? BLGPU_SUCCESS : cuda_result(e);
  LaunchConfig best = cfg;
  double best_ms = 0.0;
  if (!r) r = measure(best, best_ms);
  const int cover_slots[] = {0, 16, 32, 64};
  const int blocks[] = {0, 1, 2, 3};
  const int edge_blocks[] = {64, 128, 256};
  const int list_rows[] = {32, 16, 8, 4};
  // fields: list-row height (binning geometry of the composite), coverage slots per block (the
  // band of slots a block rasterizes), coverage / composite / curve grids, edges per block
  const int order[] = {5, 0, 1, 2, 3, 4};
  for (int fi = 0; fi < 6 && !r; fi++) {
    const int field = order[fi];
    const int* vals = field == 0 ? cover_slots : field == 3 ? edge_blocks : field == 5 ? list_rows : blocks;
    const int nvals = field == 3 ? 3 : 4;
    for (int k = 0; k < nvals && !r; k++) {
      LaunchConfig c = best;
      int* slot = field == 0 ? &c.cover_slots : field == 1 ? &c.cover_blocks_per_sm : field == 2 ? &c.fine_blocks_per_sm
                : field == 3 ? &c.edge_block : field == 4 ? &c.cubic_blocks_per_sm : &c.list_rows;
      if (*slot == vals[k]) continue;
      *slot = vals[k];
      double ms = 0.0;
      r = measure(c, ms);
      if (!r && ms < best_ms) { best = c; best_ms = ms; }
    }
  }
  cfg = best;
  graph_valid = false;                         // a captured graph holds the old launch shapes
  e = copy_canvases(false);
  if (!r && e != cudaSuccess) r = cuda_result(e);
  cudaError_t e2 = cudaStreamSynchronize(stream);
  if (!r && e2 != cudaSuccess) r = cuda_result(e2);
  if (save) cudaFree(save);
  if (best_out) *best_out = best;
  if (best_ms_out) *best_ms_out = best_ms;
  return r;
}

BLGpuResult Runtime::release_memory() {
  BLGPU_CHECK(cudaSetDevice(device));
  BLGPU_CHECK(cudaStreamSynchronize(stream));
  BLGPU_CHECK(cudaStreamSynchronize(side));
  if (graph) cudaGraphExecDestroy(graph);
  graph = nullptr;
  graph_valid = false;
  has_frame = false;
  pending_timing = 0;
  in_buf.release();
  dyn_buf.release();
  seg_buf.release();
  stroke_buf.release();
  seg_capacity = 0;
  return BLGPU_SUCCESS;
}

BLGpuResult Runtime::synchronize() {
  BLGPU_CHECK(cudaSetDevice(device));
  BLGPU_CHECK(cudaStreamSynchronize(stream));
  if (pending_timing) {
    BLGPU_CHECK(cudaMemcpy(host_totals + 20, view.error_flags, 32, cudaMemcpyDeviceToHost));
    if (host_totals[20]) { pending_timing = 0; return BLGPU_ERROR_DATA_TOO_LARGE; }
    read_pixel_ops();
    float ms = 0.f, fine_ms = 0.f;
    cudaEventElapsedTime(&ms, ev[0], ev[3]);
    stats.last_gpu_ms = ms;
    if (pending_timing == 2) {
      cudaEventElapsedTime(&fine_ms, ev[1], ev[2]);
      stats.last_fine_ms = fine_ms;
      float comp_ms = 0.f;
      cudaEventElapsedTime(&comp_ms, ev[4], ev[2]);
      stats.last_composite_ms = comp_ms;
    }
    stats.frames++;
    pending_timing = 0;
  }
  return BLGPU_SUCCESS;
}

}  // namespace blgpu
