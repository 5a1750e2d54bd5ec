// kernels.cu - the sm_103a render pipeline (K0 LUT build, K1 edge build, K2 binning, K3 fine).
//
// Built with -fmad=false: the FP64 edge builder and the FP32 radial/conic fetchers must not be
// contracted into FMAs, because the reference computes every a*b+c unfused.
#include <cuda_runtime.h>
#include <stdint.h>

#include "blgpu_internal.h"
#include "edge_build.cuh"
#include "pipeline.cuh"
#include "raster.cuh"

namespace blgpu {

// ---------------------------------------------------------------------------------------------
// K0 - gradient LUTs (interpolation.cpp:19-156, interpolation_sse2.cpp:18-171,
// interpolation_avx2.cpp:18-177), one thread per entry: the entry's value is whatever the
// reference's sequential span writer leaves there (later spans overwrite earlier ones).
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ uint32_t rgba32_of(uint64_t v) {
  uint32_t b = uint32_t(v >> 8) & 0xFFu, g = uint32_t(v >> 24) & 0xFFu;
  uint32_t r = uint32_t(v >> 40) & 0xFFu, a = uint32_t(v >> 56) & 0xFFu;
  return (a << 24) | (r << 16) | (g << 8) | b;
}
__device__ __forceinline__ uint32_t simd_div255(uint32_t x) { return (((x + 0x80u) & 0xFFFFu) * 0x101u) >> 16; }
__device__ __forceinline__ uint32_t sat8(uint32_t v) { return v > 255u ? 255u : v; }
__device__ __forceinline__ uint32_t premul_simd(uint32_t c) {
  uint32_t a = c >> 24;
  return (sat8(simd_div255(255u * a)) << 24) | (sat8(simd_div255(((c >> 16) & 255u) * a)) << 16) |
         (sat8(simd_div255(((c >> 8) & 255u) * a)) << 8) | sat8(simd_div255((c & 255u) * a));
}
__device__ __forceinline__ uint32_t premul_avx2_short_span(uint32_t c) {
  uint32_t a = c >> 24;
  return (sat8(simd_div255(a | (255u * a))) << 24) | (sat8(simd_div255((c >> 16) & 255u)) << 16) |
         (sat8(simd_div255((c >> 8) & 255u)) << 8) | sat8(simd_div255(c & 255u));
}
__device__ __forceinline__ uint32_t premul_scalar(uint32_t c) {
  uint32_t a = c >> 24;
  uint32_t v = c | 0xFF000000u;
  uint32_t rb = (v & 0x00FF00FFu) * a + 0x00800080u;
  uint32_t ag = ((v >> 8) & 0x00FF00FFu) * a + 0x00800080u;
  rb = (rb + ((rb >> 8) & 0x00FF00FFu)) & 0xFF00FF00u;
  ag = (ag + ((ag >> 8) & 0x00FF00FFu)) & 0xFF00FF00u;
  return ag | (rb >> 8);
}
__device__ __forceinline__ int round_to_int(double x) {
  int y = (x >= -2147483648.5 && x < 2147483647.5) ? __double2int_rn(x) : INT32_MIN;
  return y + (double(y) - x == -0.5);
}

__device__ uint32_t lut_entry_simd(const DevStop* s, uint32_t n, uint32_t size, uint32_t e, bool avx2) {
  uint32_t d_size = size - 1u;
  double fWidth = double(int32_t(d_size) << 8);
  uint32_t c0 = rgba32_of(s[0].rgba64);
  uint32_t u0 = 0, val = 0, span_end = 0;
  for (uint32_t si = (s[0].offset == 0.0 && n > 1) ? 1u : 0u; si < n; si++) {
    uint32_t c1 = rgba32_of(s[si].rgba64);
    uint32_t u1 = uint32_t(round_to_int(s[si].offset * fWidth));
    uint32_t start = u0 >> 8;
    uint32_t i = (u1 >> 8) - (u0 >> 8);
    u0 = u1;
    if (i <= 1) {
      if (e == start) val = avx2 ? premul_avx2_short_span(c0) : premul_simd(c0);
      else if (i == 1 && e == start + 1) val = avx2 ? premul_avx2_short_span(c1) : premul_simd(c1);
    }
    else if (e >= start && e <= start + i) {
      uint32_t j = e - start;
      double scale = double(1 << 23) / double(int(i));
      uint32_t v[4];
      for (int k = 0; k < 4; k++) {
        int32_t cc = int32_t((c0 >> (8 * k)) & 255u);
        int32_t dd = int32_t((c1 >> (8 * k)) & 255u) - cc;
        double p = double(dd) * scale;
        int32_t dx = (p > -2147483649.0 && p < 2147483648.0) ? __double2int_rz(p) : INT32_MIN;
        int32_t cx = int32_t(uint32_t(cc) << 23) + (1 << 22);
        v[k] = uint32_t(cx + int32_t(uint32_t(dx) * j)) >> 23;
      }
      uint32_t a = v[3];
      val = (sat8(simd_div255(255u * a)) << 24) | (sat8(simd_div255(v[2] * a)) << 16) |
            (sat8(simd_div255(v[1] * a)) << 8) | sat8(simd_div255(v[0] * a));
    }
    span_end = start + i + 1u;
    c0 = c1;
  }
  if (e >= span_end) val = premul_simd(c0);
  if (e == 0) val = premul_simd(rgba32_of(s[0].rgba64));
  return val;
}

__device__ uint32_t lut_entry_scalar(const DevStop* s, uint32_t n, uint32_t size, uint32_t e) {
  uint32_t c0 = rgba32_of(s[0].rgba64), c1 = c0;
  if (n == 1) return premul_scalar(c0);
  uint32_t d_size = size - 1u;
  double fWidth = double(int32_t(d_size) << 8);
  uint32_t p0 = 0, val = 0, span_end = 0;
  for (uint32_t si = 0; si < n; si++) {
    c1 = rgba32_of(s[si].rgba64);
    uint32_t p1 = uint32_t(round_to_int(s[si].offset * fWidth));
    uint32_t start = p0 >> 8;
    uint32_t i = (p1 >> 8) - (p0 >> 8);
    if (i == 0) c0 = c1;
    p0 = p1;
    uint32_t cnt = i + 1u;
    if (e >= start && e < start + cnt) {
      if (c0 == c1 || e == start) val = premul_scalar(c0);
      else {
        const uint32_t kMask = 0xFFu << 23;
        uint32_t k = e - start;
        uint32_t div = cnt - 1u;
        uint32_t r_pos = (c0 << 7) & kMask, g_pos = (c0 << 15) & kMask, b_pos = (c0 << 23) & kMask;
        uint32_t r_inc = uint32_t(int32_t(((c1 << 7) & kMask) - r_pos) / int32_t(div));
        uint32_t g_inc = uint32_t(int32_t(((c1 << 15) & kMask) - g_pos) / int32_t(div));
        uint32_t b_inc = uint32_t(int32_t(((c1 << 23) & kMask) - b_pos) / int32_t(div));
        r_pos += (1u << 22) + k * r_inc;
        g_pos += (1u << 22) + k * g_inc;
        b_pos += (1u << 22) + k * b_inc;
        if (((c0 & c1) >> 24) == 0xFFu) {
          val = 0xFF000000u + ((r_pos & kMask) >> 7) + ((g_pos & kMask) >> 15) + ((b_pos & kMask) >> 23);
        }
        else {
          uint32_t a_pos = (c0 >> 1) & kMask;
          uint32_t a_inc = uint32_t(int32_t(((c1 >> 1) & kMask) - a_pos) / int32_t(div));
          a_pos += (1u << 22) + k * a_inc;
          uint32_t cp = ((b_pos & kMask) >> 23) + ((r_pos & kMask) >> 7);
          uint32_t ca = ((a_pos & kMask) >> 23);
          uint32_t cg = ((g_pos & kMask) >> 23);
          cp = (cp * ca) + 0x00800080u;
          cg = (cg * ca) + 0x00000080u;
          ca <<= 24;
          cp = ((cp + ((cp & 0xFF00FF00u) >> 8)) & 0xFF00FF00u) >> 8;
          cg = ((cg + ((cg & 0xFF00FF00u) >> 8)) & 0xFF00FF00u);
          val = cp + cg + ca;
        }
      }
    }
    if (c0 != c1) c0 = c1;
    span_end = start + cnt;
  }
  if (e >= span_end) val = premul_scalar(c1);
  if (e == 0) val = premul_scalar(rgba32_of(s[0].rgba64));
  return val;
}

__global__ void lut_kernel(const DevLutJob* jobs, const DevStop* stops, uint32_t* luts) {
  DevLutJob job = jobs[blockIdx.x];
  const DevStop* s = stops + job.stop_first;
  for (uint32_t e = threadIdx.x; e < job.lut_size; e += blockDim.x) {
    uint32_t v = job.variant == kLutScalar ? lut_entry_scalar(s, job.stop_count, job.lut_size, e)
                                           : lut_entry_simd(s, job.stop_count, job.lut_size, e, job.variant == kLutAVX2);
    luts[job.lut_offset + e] = v;
  }
}

// ---------------------------------------------------------------------------------------------
// K1 - FP64 edge building, one thread per analytic command; pass 0 counts, pass 1 writes.
// ---------------------------------------------------------------------------------------------

__global__ void edge_kernel(FrameView f, int pass) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= f.num_cmds) return;
  DevCmd cmd = f.cmds[c];
  if (cmd.kind != kFillAnalytic) {
    if (pass == 0) { f.seg_counts[c] = 0; f.seg_rows[c] = 0; }
    return;
  }
  const DevCanvas cv = f.canvases[cmd.canvas];
  const DevXform xf = f.xforms[cmd.xform];

  eb::Builder b;
  b.sink.out = pass ? f.segs + cmd.seg_first : nullptr;
  b.sink.meta = pass ? f.seg_meta + cmd.seg_first : nullptr;
  b.sink.cmd = c;
  b.sink.n = 0;
  b.sink.ymin = INT32_MAX; b.sink.ymax = INT32_MIN; b.sink.xmin = INT32_MAX; b.sink.xmax = INT32_MIN;
  b.cx0 = 0.0; b.cy0 = 0.0; b.cx1 = double(cv.w) * 256.0; b.cy1 = double(cv.h) * 256.0;
  b.icx0 = eb::trunc_i(b.cx0); b.icx1 = eb::trunc_i(b.cx1);
  const double tol = 0.20 * 256.0;
  b.tol_sq = tol * tol;
  b.acc_x0_y0 = b.acc_x0_y1 = b.acc_x1_y0 = b.acc_x1_y1 = b.cy0;
  b.px = b.py = 0; b.psign = 0; b.pasc = false;

  eb::Src src;
  src.xy = f.verts + 2ull * cmd.geom_first;
  src.cmd = cmd.geom == kGeomPath ? f.path_cmds + cmd.geom_first : nullptr;
  src.i = 0;
  src.n = int(cmd.geom_count);
  src.affine = xf.affine != 0;
  src.m00 = xf.m[0]; src.m01 = xf.m[1]; src.m10 = xf.m[2]; src.m11 = xf.m[3]; src.m20 = xf.m[4]; src.m21 = xf.m[5];

  b.sink.rows = 0;
  int rc = eb::build(b, src);
  if (pass == 0) {
    // An invalid geometry (NaN) aborts the whole command in the reference (the edge builder is
    // reverted, rastercontextops.cpp:23-28), so nothing of it is rendered.
    bool ok = rc == 0 && b.sink.n != 0;
    f.seg_counts[c] = ok ? b.sink.n : 0u;
    f.seg_rows[c] = ok ? b.sink.rows : 0u;
    f.cmds_rw[c].status = rc ? 1u : (b.sink.n ? 0u : 2u);
    if (ok) {
      // pixel bbox of the coverage: rows [ymin >> 8, (ymax - 1) >> 8], columns [xmin >> 8, xmax >> 8]
      int y0 = b.sink.ymin >> 8, y1 = (b.sink.ymax - 1) >> 8;
      int x0 = b.sink.xmin >> 8, x1 = b.sink.xmax >> 8;
      f.cmds_rw[c].box[0] = max(x0, 0);
      f.cmds_rw[c].box[1] = max(y0, 0);
      f.cmds_rw[c].box[2] = min(x1, cv.w - 1);
      f.cmds_rw[c].box[3] = min(y1, cv.h - 1);
    }
  }
}

// The K1 emit pass re-reads seg_first from the command; copy the scanned offsets in.
__global__ void set_seg_first_kernel(FrameView f, const uint32_t* offsets) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= f.num_cmds) return;
  f.cmds_rw[c].seg_first = offsets[c];
  f.cmds_rw[c].seg_count = f.seg_counts[c];
}

// ---------------------------------------------------------------------------------------------
// Exclusive scan of u32 (three-phase, recursive on block sums).
// ---------------------------------------------------------------------------------------------

constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* smem, uint32_t& total) {
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[warp] = x;
  __syncthreads();
  int nw = blockDim.x >> 5;
  if (warp == 0) {
    uint32_t w = lane < nw ? smem[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) smem[lane] = w;
  }
  __syncthreads();
  uint32_t warp_off = warp ? smem[warp - 1] : 0u;
  total = smem[nw - 1];
  __syncthreads();
  return warp_off + x - v;
}

__global__ void scan_tiles_kernel(const uint32_t* in, uint32_t* out, uint32_t* block_sums, uint32_t n) {
  __shared__ uint32_t smem[32];
  uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) { v[k] = (base + k < n) ? in[base + k] : 0u; sum += v[k]; }
  uint32_t total;
  uint32_t off = block_exclusive_scan(sum, smem, total);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) { if (base + k < n) out[base + k] = off; off += v[k]; }
  if (threadIdx.x == 0 && block_sums) block_sums[blockIdx.x] = total;
}

__global__ void scan_add_kernel(uint32_t* out, const uint32_t* block_offsets, uint32_t n) {
  uint32_t i = blockIdx.x * kScanTile + threadIdx.x;
  uint32_t add = block_offsets[blockIdx.x];
  for (int k = 0; k < kScanItems; k++, i += kScanThreads)
    if (i < n) out[i] += add;
}

// ---------------------------------------------------------------------------------------------
// K2 - binning
// ---------------------------------------------------------------------------------------------

// Tile ranges of every command (empty commands get 0xFFFFFFFF) and its number of tile rows.
__global__ void cmd_tiles_kernel(FrameView f, uint32_t* cmdrow_counts_per_cmd, uint32_t* row_counts) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= f.num_cmds) return;
  const DevCmd cmd = f.cmds[c];
  const DevCanvas cv = f.canvases[cmd.canvas];
  int x0, y0, x1, y1;   // inclusive pixel range
  bool empty = false;
  if (cmd.kind == kFillAnalytic) {
    empty = cmd.status != 0;
    x0 = cmd.box[0]; y0 = cmd.box[1]; x1 = cmd.box[2]; y1 = cmd.box[3];
  }
  else if (cmd.kind == kFillBoxA) {
    x0 = cmd.box[0]; y0 = cmd.box[1]; x1 = cmd.box[2] - 1; y1 = cmd.box[3] - 1;
  }
  else {
    x0 = cmd.box[0] >> 8; y0 = cmd.box[1] >> 8; x1 = ((cmd.box[2] + 255) >> 8) - 1; y1 = ((cmd.box[3] + 255) >> 8) - 1;
  }
  x0 = max(x0, 0); y0 = max(y0, 0); x1 = min(x1, cv.w - 1); y1 = min(y1, cv.h - 1);
  if (x0 > x1 || y0 > y1) empty = true;
  if (empty) {
    f.cmd_tile_x[c] = 0xFFFFFFFFu;
    f.cmd_tile_y[c] = 0xFFFFFFFFu;
    cmdrow_counts_per_cmd[c] = 0;
    return;
  }
  uint32_t tx0 = uint32_t(x0) >> kTileShift, tx1 = uint32_t(x1) >> kTileShift;
  uint32_t ty0 = uint32_t(y0) >> kTileShift, ty1 = uint32_t(y1) >> kTileShift;
  f.cmd_tile_x[c] = tx0 | (tx1 << 16);
  f.cmd_tile_y[c] = ty0 | (ty1 << 16);
  cmdrow_counts_per_cmd[c] = cmd.kind == kFillAnalytic ? (ty1 - ty0 + 1u) : 0u;
  for (uint32_t r = ty0; r <= ty1; r++) atomicAdd(&row_counts[cv.row_base + r], 1u);
}

// Segments per (command, tile row).
__global__ void seg_bin_kernel(FrameView f, int scatter) {
  uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= f.num_segs) return;
  uint32_t c = f.seg_meta[s] >> 1;
  uint32_t ty = f.cmd_tile_y[c];
  if (ty == 0xFFFFFFFFu) return;
  int ty0 = int(ty & 0xFFFFu), ty1 = int(ty >> 16);
  const DevSeg g = f.segs[s];
  int r0 = max(int(uint32_t(g.y0 >> 8) >> kTileShift), ty0);
  int r1 = min(int(uint32_t((g.y1 - 1) >> 8) >> kTileShift), ty1);
  uint32_t base = f.cmdrow_base[c];
  for (int r = r0; r <= r1; r++) {
    uint32_t slot = base + uint32_t(r - ty0);
    if (!scatter) atomicAdd(&f.cmdrow_counts[slot], 1u);
    else {
      uint32_t pos = atomicAdd(&f.cmdrow_cursor[slot], 1u);
      f.seglist[f.cmdrow_offsets[slot] + pos] = s;
    }
  }
}

// Per tile row: commands overlapping the row in painter's order (one block per row).
__global__ void row_fill_kernel(FrameView f, const uint32_t* row_canvas) {
  __shared__ uint32_t smem[32];
  uint32_t row = blockIdx.x;
  const DevCanvas cv = f.canvases[row_canvas[row]];
  uint32_t r = row - cv.row_base;
  uint32_t out = f.row_offsets[row];
  for (uint32_t base = 0; base < cv.cmd_count; base += blockDim.x) {
    uint32_t c = cv.cmd_first + base + threadIdx.x;
    uint32_t flag = 0;
    if (base + threadIdx.x < cv.cmd_count) {
      uint32_t ty = f.cmd_tile_y[c];
      flag = (ty != 0xFFFFFFFFu && (ty & 0xFFFFu) <= r && (ty >> 16) >= r) ? 1u : 0u;
    }
    uint32_t total;
    uint32_t pos = block_exclusive_scan(flag, smem, total);
    if (flag) f.row_cmds[out + pos] = c;
    out += total;
  }
}

// ---------------------------------------------------------------------------------------------
// K3 - persistent fine kernel
// ---------------------------------------------------------------------------------------------

struct FineShared {
  uint32_t cells[kTileH * kTileW];
  uint32_t backdrop[kTileH];
  uint32_t queue[kFineThreads];
  uint32_t warp_counts[kFineThreads / 32];
  uint32_t tile;
  uint32_t qn;
};

__global__ void __launch_bounds__(kFineThreads) fine_kernel(FrameView f) {
  __shared__ FineShared sh;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int prow = tid >> 3;            // pixel row within the tile
  const int pcol = (tid & 7) * 4;       // first of 4 pixel columns

  uint32_t ops = 0, pat_ops = 0;   // composited pixels of this thread (all tiles)

  for (;;) {
    if (tid == 0) sh.tile = atomicAdd(f.work_counter, 1u);
    __syncthreads();
    uint32_t t = sh.tile;
    __syncthreads();
    if (t >= f.num_tiles) break;
    uint32_t tile = f.tile_order[t];
    const DevCanvas cv = f.canvases[f.tile_canvas[tile]];
    uint32_t local = tile - cv.tile_base;
    int tx = int(local % uint32_t(cv.tiles_x)), ty = int(local / uint32_t(cv.tiles_x));
    int x_base = tx * kTileW, y = ty * kTileH + prow;
    int xp = x_base + pcol;
    bool row_ok = y < cv.h;
    uint32_t* dst = cv.pixels + int64_t(y) * cv.stride + xp;

    uint32_t pix[4];
    bool full = row_ok && (xp + 3 < cv.w);
    if (full) {
      uint4 v = *reinterpret_cast<const uint4*>(dst);
      pix[0] = v.x; pix[1] = v.y; pix[2] = v.z; pix[3] = v.w;
    }
    else {
#pragma unroll
      for (int k = 0; k < 4; k++) pix[k] = (row_ok && xp + k < cv.w) ? dst[k] : 0u;
    }

    uint32_t row_id = cv.row_base + uint32_t(ty);
    uint32_t list_first = f.row_offsets[row_id];
    uint32_t list_count = f.row_counts[row_id];
    ras::TileSink sink{sh.cells, sh.backdrop, x_base};
    int row0 = ty * kTileH;

    for (uint32_t base = 0; base < list_count; base += kFineThreads) {
      // ordered compaction of the commands of this chunk that overlap the tile's columns
      uint32_t c = 0xFFFFFFFFu;
      bool hit = false;
      if (base + tid < list_count) {
        c = f.row_cmds[list_first + base + tid];
        uint32_t tr = f.cmd_tile_x[c];
        hit = (tr & 0xFFFFu) <= uint32_t(tx) && (tr >> 16) >= uint32_t(tx);
      }
      uint32_t ballot = __ballot_sync(0xFFFFFFFFu, hit);
      if (lane == 0) sh.warp_counts[warp] = __popc(ballot);
      __syncthreads();
      uint32_t off = 0, total = 0;
      for (int w = 0; w < kFineThreads / 32; w++) { uint32_t n = sh.warp_counts[w]; off += w < warp ? n : 0u; total += n; }
      if (hit) sh.queue[off + __popc(ballot & ((1u << lane) - 1u))] = c;
      __syncthreads();

      for (uint32_t q = 0; q < total; q++) {
        uint32_t ci = sh.queue[q];
        const DevCmd& cmd = f.cmds[ci];
        const uint32_t kind = cmd.kind;
        const DevStyle& st = f.styles[cmd.style];
        const uint32_t alpha = cmd.alpha;
        const bool src_copy = (cmd.flags & 1u) != 0;
        uint32_t m[4] = {0u, 0u, 0u, 0u};
        int fetch_y0 = cmd.fetch_y0;

        if (kind == kFillAnalytic) {
#pragma unroll
          for (int k = 0; k < 4; k++) sh.cells[tid * 4 + k] = 0u;
          if (tid < kTileH) sh.backdrop[tid] = 0u;
          __syncthreads();
          uint32_t ty0 = f.cmd_tile_y[ci] & 0xFFFFu;
          uint32_t slot = f.cmdrow_base[ci] + uint32_t(ty) - ty0;
          uint32_t s_first = f.cmdrow_offsets[slot];
          uint32_t s_count = f.cmdrow_counts[slot];
          for (uint32_t k = tid; k < s_count; k += kFineThreads) {
            uint32_t si = f.seglist[s_first + k];
            ras::segment_to_tile(f.segs[si], f.seg_meta[si] & 1u, row0, cv.h - 1, sink);
          }
          __syncthreads();
          // coverage sweep: prefix over the row (8 threads x 4 cells) + the carried-in backdrop
          uint32_t cl[4];
#pragma unroll
          for (int k = 0; k < 4; k++) cl[k] = sh.cells[prow * kTileW + pcol + k];
          uint32_t s4 = cl[0] + cl[1] + cl[2] + cl[3];
          uint32_t incl = s4;
#pragma unroll
          for (int o = 1; o < 8; o <<= 1) {
            uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o, 8);
            if ((tid & 7) >= o) incl += v;
          }
          uint32_t cov = (256u << 9) + sh.backdrop[prow] + incl - s4;
          uint32_t rule = (cmd.flags & 2u) ? 0x1FFu : 0xFFFFFFFFu;
#pragma unroll
          for (int k = 0; k < 4; k++) { cov += cl[k]; m[k] = px::calc_mask(cov, rule, alpha); }
          // the reference initializes its fetcher at the start of each band of the command
          int y_start = cmd.box[1];
          fetch_y0 = max(y_start, (y / cv.band_height) * cv.band_height);
          __syncthreads();
        }
        else if (kind == kFillBoxA) {
          bool in_y = y >= cmd.box[1] && y < cmd.box[3];
#pragma unroll
          for (int k = 0; k < 4; k++) m[k] = (in_y && xp + k >= cmd.box[0] && xp + k < cmd.box[2]) ? alpha : 0u;
        }
        else {
#pragma unroll
          for (int k = 0; k < 4; k++) m[k] = px::box_u_mask(cmd.box, alpha, xp + k, y);
        }

        if (row_ok && (m[0] | m[1] | m[2] | m[3])) {
          px::RowState rs = px::row_state(st, y, fetch_y0);
          uint32_t n = 0;
#pragma unroll
          for (int k = 0; k < 4; k++) {
            if (m[k] && xp + k < cv.w) {
              uint32_t s = px::fetch(st, rs, xp + k, f.luts, f.images);
              pix[k] = px::composite(pix[k], s, m[k], src_copy);
              n++;
            }
          }
          ops += n;
          pat_ops += st.fetch >= kFetchPatAlignedPad ? n : 0u;
        }
      }
      __syncthreads();
    }

    if (full) {
      *reinterpret_cast<uint4*>(dst) = make_uint4(pix[0], pix[1], pix[2], pix[3]);
    }
    else {
#pragma unroll
      for (int k = 0; k < 4; k++) if (row_ok && xp + k < cv.w) dst[k] = pix[k];
    }
  }

  ops = __reduce_add_sync(0xFFFFFFFFu, ops);
  pat_ops = __reduce_add_sync(0xFFFFFFFFu, pat_ops);
  if (lane == 0 && ops) {
    atomicAdd(&f.pixel_ops[0], (unsigned long long)ops);
    if (pat_ops) atomicAdd(&f.pixel_ops[1], (unsigned long long)pat_ops);
  }
}

// Tile/row bookkeeping: canvas of every global tile and tile row, identity processing order.
__global__ void tile_setup_kernel(FrameView f, uint32_t* row_canvas) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  // binary search the canvas owning tile i / row i
  if (i < f.num_tiles) {
    uint32_t lo = 0, hi = f.num_canvases - 1;
    while (lo < hi) { uint32_t mid = (lo + hi + 1) >> 1; if (f.canvases[mid].tile_base <= i) lo = mid; else hi = mid - 1; }
    f.tile_canvas[i] = lo;
    f.tile_order[i] = i;
  }
  if (i < f.num_rows) {
    uint32_t lo = 0, hi = f.num_canvases - 1;
    while (lo < hi) { uint32_t mid = (lo + hi + 1) >> 1; if (f.canvases[mid].row_base <= i) lo = mid; else hi = mid - 1; }
    row_canvas[i] = lo;
  }
}

}  // namespace blgpu

// =============================================================================================
// Host-side pipeline orchestration
// =============================================================================================

#include "launch.h"

namespace blgpu {

static inline uint32_t cdiv(uint64_t a, uint64_t b) { return uint32_t((a + b - 1) / b); }

// Exclusive scan of `n` u32 (in may equal out). `tmp` must hold scan_temp_words(n) words.
int exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* tmp, cudaStream_t st) {
  if (n == 0) return 0;
  uint32_t blocks = cdiv(n, kScanTile);
  if (blocks == 1) {
    scan_tiles_kernel<<<1, kScanThreads, 0, st>>>(in, out, nullptr, n);
    return 1;
  }
  uint32_t* sums = tmp;
  scan_tiles_kernel<<<blocks, kScanThreads, 0, st>>>(in, out, sums, n);
  int k = exclusive_scan(sums, sums, blocks, tmp + blocks, st);
  scan_add_kernel<<<blocks, kScanThreads, 0, st>>>(out, sums, n);
  return k + 2;
}

uint32_t scan_temp_words(uint32_t n) {
  uint32_t words = 0;
  while (n > uint32_t(kScanTile)) { n = cdiv(n, kScanTile); words += n; }
  return words + 16;
}

__global__ void total_kernel(const uint32_t* counts, const uint32_t* offsets, uint32_t n, uint32_t* total) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *total = n ? offsets[n - 1] + counts[n - 1] : 0u;
}

// totals[k] += sum(in[0..n)) (totals zeroed by the caller).
__global__ void sum_kernel(const uint32_t* in, uint32_t n, uint32_t* total) {
  __shared__ uint32_t smem[32];
  uint32_t v = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v += in[i];
  uint32_t t;
  block_exclusive_scan(v, smem, t);
  if (threadIdx.x == 0) atomicAdd(total, t);
}

int launch_sum(const uint32_t* in, uint32_t n, uint32_t* total, cudaStream_t st) {
  if (!n) return 0;
  uint32_t blocks = cdiv(n, 1024);
  if (blocks > 1024) blocks = 1024;
  sum_kernel<<<blocks, 1024, 0, st>>>(in, n, total);
  return 1;
}

int launch_total(const uint32_t* counts, const uint32_t* offsets, uint32_t n, uint32_t* total, cudaStream_t st) {
  total_kernel<<<1, 32, 0, st>>>(counts, offsets, n, total);
  return 1;
}

int launch_lut(const FrameView& f, cudaStream_t st) {
  if (!f.num_lut_jobs) return 0;
  lut_kernel<<<f.num_lut_jobs, 256, 0, st>>>(f.lut_jobs, f.stops, f.luts);
  return 1;
}

int launch_edge_count(const FrameView& f, cudaStream_t st) {
  if (!f.num_cmds) return 0;
  edge_kernel<<<cdiv(f.num_cmds, 64), 64, 0, st>>>(f, 0);
  return 1;
}

int launch_edge_emit(const FrameView& f, const uint32_t* seg_offsets, cudaStream_t st) {
  if (!f.num_cmds) return 0;
  set_seg_first_kernel<<<cdiv(f.num_cmds, 256), 256, 0, st>>>(f, seg_offsets);
  if (!f.num_segs) return 1;
  edge_kernel<<<cdiv(f.num_cmds, 64), 64, 0, st>>>(f, 1);
  return 2;
}

int launch_cmd_tiles(const FrameView& f, uint32_t* cmdrow_counts_per_cmd, cudaStream_t st) {
  if (!f.num_cmds) return 0;
  cmd_tiles_kernel<<<cdiv(f.num_cmds, 256), 256, 0, st>>>(f, cmdrow_counts_per_cmd, f.row_counts);
  return 1;
}

int launch_seg_bin(const FrameView& f, int scatter, cudaStream_t st) {
  if (!f.num_segs) return 0;
  seg_bin_kernel<<<cdiv(f.num_segs, 256), 256, 0, st>>>(f, scatter);
  return 1;
}

int launch_rows_and_tiles(const FrameView& f, uint32_t* row_canvas, cudaStream_t st) {
  int k = 0;
  uint32_t n = f.num_tiles > f.num_rows ? f.num_tiles : f.num_rows;
  if (n) { tile_setup_kernel<<<cdiv(n, 256), 256, 0, st>>>(f, row_canvas); k++; }
  if (f.num_rows) { row_fill_kernel<<<f.num_rows, 512, 0, st>>>(f, row_canvas); k++; }
  return k;
}

int fine_grid_size() {
  static int grid = 0;
  if (!grid) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fine_kernel, kFineThreads, 0);
    grid = sms * (per_sm > 0 ? per_sm : 1);
  }
  return grid;
}

// work_counter must be zero on entry.
int launch_fine(const FrameView& f, cudaStream_t st) {
  if (!f.num_tiles) return 0;
  int grid = fine_grid_size();
  if (uint32_t(grid) > f.num_tiles) grid = int(f.num_tiles);
  fine_kernel<<<grid, kFineThreads, 0, st>>>(f);
  return 1;
}

}  // namespace blgpu
