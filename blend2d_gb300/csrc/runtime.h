// runtime.h - device runtime: frame staging, device memory, pipeline execution, replay.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <stdlib.h>
#include <string.h>

#include <new>
#include <vector>

#include "blgpu.h"
#include "blgpu_internal.h"
#include "launch.h"

namespace blgpu {

// A pattern source registered in a frame (host or device memory).
struct FrameImage {
  const void* pixels;
  intptr_t stride;          // bytes
  int32_t w, h;
  int32_t bpp;              // bytes per pixel: 4 (PRGB32) or 1 (A8 masks, rows packed tightly)
  bool device;
  uint64_t pool_offset;     // first pixel in the frame's image pool (32-bit words)
};

// A canvas's render target.
struct FrameTarget {
  BLGpuImage image;
  bool upload;              // the pipeline reads the canvas's current content
};

// Growable array of trivially copyable elements in page-locked host memory (or plain heap memory
// when `pinned` is false), so that a frame recorded into it can be copied to the device by DMA
// without an intermediate copy. Capacity is kept across clear().
template <typename T>
struct HostArray {
  T* ptr = nullptr;
  size_t n = 0, cap = 0;
  bool pinned = true;          // allocate page-locked memory
  bool ptr_pinned = false;     // the current block is page-locked (allocation may fall back)

  HostArray() = default;
  HostArray(const HostArray&) = delete;
  HostArray& operator=(const HostArray&) = delete;
  ~HostArray() { release(); }

  void release() {
    if (ptr) { if (ptr_pinned) cudaFreeHost(ptr); else free(ptr); }
    ptr = nullptr; n = cap = 0; ptr_pinned = false;
  }
  void reserve(size_t want) {
    if (want <= cap) return;
    size_t nc = cap ? cap : 1024;
    while (nc < want) nc += nc / 2 + 1;
    T* np = nullptr;
    bool np_pinned = false;
    if (pinned) {
      if (cudaMallocHost(reinterpret_cast<void**>(&np), nc * sizeof(T)) == cudaSuccess) np_pinned = true;
      else { np = nullptr; cudaGetLastError(); }
    }
    if (!np) np = static_cast<T*>(malloc(nc * sizeof(T)));   // pageable fallback still works
    if (!np) throw std::bad_alloc();
    if (n) memcpy(np, ptr, n * sizeof(T));
    if (ptr) { if (ptr_pinned) cudaFreeHost(ptr); else free(ptr); }
    ptr = np; cap = nc; ptr_pinned = np_pinned;
  }
  size_t size() const { return n; }
  bool empty() const { return n == 0; }
  T* data() { return ptr; }
  const T* data() const { return ptr; }
  T* begin() { return ptr; }
  T* end() { return ptr + n; }
  const T* begin() const { return ptr; }
  const T* end() const { return ptr + n; }
  T& operator[](size_t i) { return ptr[i]; }
  const T& operator[](size_t i) const { return ptr[i]; }
  T& back() { return ptr[n - 1]; }
  void clear() { n = 0; }
  void push_back(const T& v) { if (n == cap) reserve(n + 1); ptr[n++] = v; }
  void append(const T* first, size_t count) {
    if (!count) return;
    reserve(n + count);
    memcpy(ptr + n, first, count * sizeof(T));
    n += count;
  }
  // Sets the size to `count` elements; the new ones are left uninitialized (to be written).
  void resize_uninit(size_t count) {
    reserve(count);
    n = count;
  }
  void append_fill(size_t count, const T& v) {
    reserve(n + count);
    for (size_t i = 0; i < count; i++) ptr[n + i] = v;
    n += count;
  }
};

// Everything one device pipeline run consumes, recorded on the host in painter's order.
struct Frame {
  explicit Frame(bool pinned_memory = true) {
    cmds.pinned = styles.pinned = xforms.pinned = verts.pinned = path_cmds.pinned = lut_jobs.pinned = stops.pinned =
        pinned_memory;
    stroke_figs.pinned = stroke_params.pinned = stroke_xy.pinned = stroke_cmds.pinned = pinned_memory;
  }
  HostArray<DevCmd> cmds;
  HostArray<DevStyle> styles;
  HostArray<DevXform> xforms;
  std::vector<DevCanvas> canvases;
  std::vector<FrameTarget> targets;
  HostArray<double> verts;
  HostArray<uint8_t> path_cmds;
  HostArray<DevLutJob> lut_jobs;
  HostArray<DevStop> stops;
  // stroke input paths (user space, or mapped by the user transform's linear part for transform
  // order BEFORE), their figures and parameters
  HostArray<DevStrokeFig> stroke_figs;
  HostArray<DevStrokeParams> stroke_params;
  HostArray<double> stroke_xy;
  HostArray<uint8_t> stroke_cmds;
  std::vector<FrameImage> images;
  uint64_t image_words = 0;
  uint32_t lut_words = 0;
  uint32_t tiles = 0, rows = 0;
  uint64_t generation = next_generation();   // renewed by clear(); per-frame registrations compare against it
  // A merged frame's vertices stay in the parts it was made of when those hold them in page-locked
  // memory: `vert_parts` lists them in order (uploaded by DMA from there) and `ext_verts` counts
  // their vertices, which follow the frame's own `verts` (empty then).
  std::vector<const Frame*> vert_parts;
  uint64_t ext_verts = 0;
  uint64_t vertex_count() const { return verts.size() / 2 + ext_verts; }

  static uint64_t next_generation();
  void clear();
  // Adds a canvas (tile/row bases, band height) for `image`; returns its index.
  uint32_t add_canvas(const BLGpuImage& image, bool upload);
  // Registers a pattern image (deduplicated by pixel pointer); returns the pool offset.
  uint64_t add_image(const BLGpuImage& image);
  // Replaces this frame's content with the concatenation of `parts` (frames recorded on their
  // own, e.g. by several threads), shifting every index a part holds by what the parts before it
  // hold. The copies run on up to `threads` threads. Vertices held in page-locked memory by every
  // part are not copied but referenced (`vert_parts`): the parts must then stay unchanged until the
  // frame has been uploaded.
  void merge(Frame* const* parts, size_t count, unsigned threads);
};

// Sizes produced by the counting half of the pipeline, cached for replay.
struct FrameTotals {
  uint32_t segs = 0, seglist = 0, cmdrows = 0, row_entries = 0, row_states = 0, row_runs = 0;
};

// What a frame's device arrays hold: a frame's own sizes (eager runs) or the capacities of a
// layout that any frame up to them fits (graph frames). The work arrays sized on the device
// (segments, slots, coverage items, row lists, gradient rows) have their own capacities.
struct FrameSizes {
  uint32_t cmds = 0, styles = 0, xforms = 0, canvases = 0, lut_jobs = 0, stops = 0, tiles = 0, rows = 0;
  uint64_t vert_words = 0, cmd_bytes = 0, image_words = 0, lut_words = 0, canvas_words = 0;
  FrameTotals dyn;
  bool fits_in(const FrameSizes& c) const {
    return cmds <= c.cmds && styles <= c.styles && xforms <= c.xforms && canvases <= c.canvases &&
           lut_jobs <= c.lut_jobs && stops <= c.stops && tiles <= c.tiles && rows <= c.rows &&
           vert_words <= c.vert_words && cmd_bytes <= c.cmd_bytes && image_words <= c.image_words &&
           lut_words <= c.lut_words && canvas_words <= c.canvas_words;
  }
};

constexpr int kCounterWords = 48;

struct DeviceBuffer {
  void* ptr = nullptr;
  size_t size = 0;
  cudaError_t reserve(size_t bytes);
  void release();
};

struct Runtime {
  int device = 0;
  uint32_t lut_variant = kLutSSE2;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int sm_count = 0;

  DeviceBuffer in_buf;      // uploaded frame data + canvases + fixed-size work arrays
  DeviceBuffer dyn_buf;     // sizes known after the counting pass (segment and command lists)
  DeviceBuffer seg_buf;     // segments + their metadata, appended by the edge builders
  DeviceBuffer stroke_buf;  // stroke inputs, per-figure outline counts and offsets
  bool strokes_counted = false;   // the upload's sizing pass left this frame's counts in place
  std::vector<uint32_t> stroke_order;   // thread -> figure order of the frame being uploaded
  uint32_t seg_capacity = 0;
  void* host_staging = nullptr;
  size_t host_staging_size = 0;
  uint32_t* counts_dev = nullptr;    // the frame's sizes (CountIndex), read by the kernels
  uint32_t* host_counts = nullptr;   // pinned staging of counts_dev
  uint32_t* host_totals = nullptr;   // pinned: [0..8) frame totals, [16] stroke outline size,
                                     // [20..24) error flags (ErrorFlag bits in [20]), [24..28) pixel ops

  cudaEvent_t ev[5] = {};
  // Gradient LUTs are built on a side stream, forked after the upload and joined before the
  // composite pass, so they overlap the FP64-bound edge building.
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  cudaEvent_t order_ev = nullptr;      // end of this runtime's last ordered pipeline (LaunchConfig::device_order)
  cudaGraphExec_t graph = nullptr;
  bool graph_valid = false;

  // last executed frame (kept for replay)
  FrameView view{};
  FrameTotals totals;
  std::vector<FrameTarget> targets;
  std::vector<uint32_t*> canvas_dev;   // device pixels per canvas
  std::vector<int32_t> canvas_stride;  // device stride in pixels
  // canvases copied by canvas_copy_kernel (page-locked host images): the table (device), its
  // staging copy, and each canvas's index in it (-1: copied with cudaMemcpy2DAsync)
  DeviceBuffer xfer_buf;
  HostArray<DevXfer> xfers;
  std::vector<int32_t> canvas_xfer;
  uint32_t* cmdrow_per_cmd = nullptr;
  uint32_t* row_canvas = nullptr;
  uint32_t* scan_tmp = nullptr;
  bool has_frame = false;
  int pending_timing = 0;   // 1: graph replay timed, 2: eager replay timed (incl. fine kernel)
  uint64_t h2d_bytes = 0, d2h_bytes = 0;
  uint64_t in_bytes = 0, stroke_bytes = 0;   // the last frame's planned input / stroke arena bytes
  uint64_t last_frame_bytes = 0;             // ... and everything it used on the device
  uint64_t reserved_bytes() const { return uint64_t(in_buf.size) + dyn_buf.size + seg_buf.size + stroke_buf.size; }

  BLGpuStats stats{};
  LaunchConfig cfg;

  BLGpuResult init(const BLGpuRuntimeCreateInfo* info);
  void destroy();
  // Uploads `fr`, runs the pipeline, downloads the canvases that live in host memory. Blocking.
  // With cfg.graph_frames the frame runs as a captured graph over capacity-sized arrays when it
  // can (run_graph); otherwise eagerly, every array sized from the frame (run_eager).
  BLGpuResult run(const Frame& fr);
  BLGpuResult run_frame(const Frame& fr);
  BLGpuResult run_eager(const Frame& fr);
  BLGpuResult run_graph(const Frame& fr);
  FrameSizes caps{};             // graph frames: capacities of the layout the graph was captured on
  bool view_by_caps = false;     // the kept frame is laid out by `caps`
  uint32_t planned_list_shift = 5;   // list-row height the kept frame's dynamic arrays were sized for
  // Sizes the dynamic arrays of the kept frame again after a launch-config change that alters
  // what the device computes (the list-row height): one counting half and a read-back.
  BLGpuResult resize_dynamic();
  bool caps_ready = false;
  uint64_t graph_frames_run = 0; // frames that ran as a replay of the captured graph
  BLGpuResult replay(bool use_graph);
  BLGpuResult synchronize();
  // Frees the device arenas (the kept frame is dropped).
  BLGpuResult release_memory();
  // Picks the fastest launch shapes for the last frame (its pixels are left unchanged).
  BLGpuResult autotune(int trials, LaunchConfig* best, double* best_ms);
  // Renders a one-canvas frame into its device-memory image using only the fixed device scratch
  // area (noalloc.h). Blocking. Does not touch the frame kept for replay.
  BLGpuResult run_noalloc(const Frame& fr);

 private:
  int enqueue_count_half(cudaStream_t st);
  int enqueue_render_half(cudaStream_t st, bool timed);
  BLGpuResult prepare_strokes(const Frame& fr, FrameView& v, uint32_t& outline_verts);
  // Fills host_counts with the frame's sizes and copies them to `dev` on the stream.
  cudaError_t put_counts(const Frame& fr, uint32_t* dev);
  // Uploads `fr` into a layout sized by the frame itself, or by `caps` (graph frames).
  BLGpuResult upload(const Frame& fr, const FrameSizes* caps = nullptr);
  BLGpuResult upload_frame(const Frame& fr, const FrameSizes* caps);
  BLGpuResult download();
  // Builds the kernel-copy table of the frame's host canvases and uploads the canvases whose
  // content the frame composites onto.
  BLGpuResult stage_canvases(const Frame& fr);
  BLGpuResult reserve_segments(uint32_t count);
  void read_pixel_ops();
};

BLGpuResult cuda_result(cudaError_t e);
bool device_target_direct(const BLGpuImage& im);
FrameSizes sizes_of(const Frame& fr, uint32_t outline_verts);
int last_cuda_error();

}  // namespace blgpu
