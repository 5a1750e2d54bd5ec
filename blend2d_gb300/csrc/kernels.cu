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

// One interpolation span of a LUT builder: the FP64 part of the builder (stop positions and the
// per-channel increments) is evaluated once per span, one lane per stop; entries only do integer work.
struct LutSpan {
  uint32_t start, count;   // simd: first entry and i (entries start .. start + i); scalar: start, cnt
  uint32_t c0, c1;         // colours at both ends (scalar: after its equal-position rule)
  int32_t inc[4];          // simd: dx per channel (b, g, r, a); scalar: r, g, b, a increments
};

__device__ uint32_t lut_eval_simd(const LutSpan* sp, int nspans, uint32_t e, uint32_t val, bool avx2) {
  for (int k = 0; k < nspans; k++) {
    const LutSpan& q = sp[k];
    uint32_t start = q.start, i = q.count;
    if (i <= 1) {
      if (e == start) val = avx2 ? premul_avx2_short_span(q.c0) : premul_simd(q.c0);
      else if (i == 1 && e == start + 1) val = avx2 ? premul_avx2_short_span(q.c1) : premul_simd(q.c1);
    }
    else if (e >= start && e <= start + i) {
      uint32_t j = e - start;
      uint32_t v[4];
#pragma unroll
      for (int ch = 0; ch < 4; ch++) {
        int32_t cc = int32_t((q.c0 >> (8 * ch)) & 255u);
        int32_t cx = int32_t(uint32_t(cc) << 23) + (1 << 22);
        v[ch] = uint32_t(cx + int32_t(uint32_t(q.inc[ch]) * j)) >> 23;
      }
      uint32_t a = v[3];
      val = (sat8(simd_div255(255u * a)) << 24) | (sat8(simd_div255(v[2] * a)) << 16) |
            (sat8(simd_div255(v[1] * a)) << 8) | sat8(simd_div255(v[0] * a));
    }
  }
  return val;
}

__device__ uint32_t lut_eval_scalar(const LutSpan* sp, int nspans, uint32_t e, uint32_t val) {
  for (int k = 0; k < nspans; k++) {
    const LutSpan& q = sp[k];
    uint32_t start = q.start, cnt = q.count, c0 = q.c0, c1 = q.c1;
    if (e >= start && e < start + cnt) {
      if (c0 == c1 || e == start) val = premul_scalar(c0);
      else {
        const uint32_t kMask = 0xFFu << 23;
        uint32_t j = e - start;
        uint32_t r_pos = (c0 << 7) & kMask, g_pos = (c0 << 15) & kMask, b_pos = (c0 << 23) & kMask;
        r_pos += (1u << 22) + j * uint32_t(q.inc[0]);
        g_pos += (1u << 22) + j * uint32_t(q.inc[1]);
        b_pos += (1u << 22) + j * uint32_t(q.inc[2]);
        if (((c0 & c1) >> 24) == 0xFFu) {
          val = 0xFF000000u + ((r_pos & kMask) >> 7) + ((g_pos & kMask) >> 15) + ((b_pos & kMask) >> 23);
        }
        else {
          uint32_t a_pos = (c0 >> 1) & kMask;
          a_pos += (1u << 22) + j * uint32_t(q.inc[3]);
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
  }
  return val;
}

// 64-bit LUT of dithered gradients: interpolate_prgb64 (interpolation.cpp:161-288). Same span walk
// as the scalar 32-bit builder (a span covers (p1 >> 8) - (p0 >> 8) + 1 entries, its first entry is
// premultiplied c0, later ones step 16.15 fixed-point positions), with 16-bit channels and
// premultiplication by udiv65535 (scalar_p.h:37, :179-222).
struct LutSpan64 {
  uint32_t start, count;
  uint64_t c0, c1;
  uint32_t inc[4];         // r, g, b, a
};

__device__ __forceinline__ uint32_t udiv65535(uint32_t x) { return ((x + 0x8000u) + ((x + 0x8000u) >> 16)) >> 16; }

__device__ __forceinline__ uint64_t premul64(uint64_t c) {
  const uint32_t a = uint32_t(c >> 48);
  const uint32_t r = udiv65535((uint32_t(c >> 32) & 0xFFFFu) * a);
  const uint32_t g = udiv65535((uint32_t(c >> 16) & 0xFFFFu) * a);
  const uint32_t b = udiv65535((uint32_t(c) & 0xFFFFu) * a);
  return (uint64_t(a) << 48) | (uint64_t(r) << 32) | (uint64_t(g) << 16) | uint64_t(b);
}

constexpr uint32_t kLut64Shift = 15, kLut64Mask = 0xFFFFu << 15;

__device__ uint64_t lut_eval64(const LutSpan64* sp, int nspans, uint32_t e, uint64_t val) {
  for (int k = 0; k < nspans; k++) {
    const LutSpan64& q = sp[k];
    if (e >= q.start && e < q.start + q.count) {
      if (q.c0 == q.c1 || e == q.start) val = premul64(q.c0);
      else {
        const uint32_t j = e - q.start, half = 1u << (kLut64Shift - 1);
        const uint32_t r_pos = uint32_t((q.c0 >> (32 - kLut64Shift)) & kLut64Mask) + half + j * q.inc[0];
        const uint32_t g_pos = uint32_t((q.c0 >> (16 - kLut64Shift)) & kLut64Mask) + half + j * q.inc[1];
        const uint32_t b_pos = uint32_t((q.c0 << kLut64Shift) & kLut64Mask) + half + j * q.inc[2];
        if (((q.c0 & q.c1) >> 48) == 0xFFFFu) {
          val = (uint64_t(r_pos & kLut64Mask) << (32 - kLut64Shift)) | (uint64_t(g_pos & kLut64Mask) << (16 - kLut64Shift)) |
                (uint64_t(b_pos & kLut64Mask) >> kLut64Shift) | 0xFFFF000000000000ull;
        }
        else {
          const uint32_t a_pos = uint32_t((q.c0 >> (48 - kLut64Shift)) & kLut64Mask) + half + j * q.inc[3];
          const uint32_t ca = a_pos >> kLut64Shift;
          const uint32_t cr = udiv65535((r_pos >> kLut64Shift) * ca);
          const uint32_t cg = udiv65535((g_pos >> kLut64Shift) * ca);
          const uint32_t cb = udiv65535((b_pos >> kLut64Shift) * ca);
          val = (uint64_t(ca) << 48) | (uint64_t(cr) << 32) | (uint64_t(cg) << 16) | uint64_t(cb);
        }
      }
    }
  }
  return val;
}

// Warp-wide build of one 64-bit LUT, 32 stops per chunk like the 32-bit scalar path below.
__device__ void lut_build64(const DevLutJob& job, const DevStop* s, uint64_t* lut, LutSpan64* spans, int lane) {
  const uint32_t n = job.stop_count;
  const uint64_t first_c = s[0].rgba64;
  const double fWidth = double(int32_t(job.lut_size - 1u) << 8);
  uint32_t car_u0 = 0, span_end = 0;
  uint64_t car_c = first_c;
  bool first_chunk = true;
  for (uint32_t si = 0; si < n; si += 32) {
    const uint32_t k = si + uint32_t(lane);
    const int ns = int(min(32u, n - si));
    uint64_t c1 = 0;
    uint32_t u1 = 0;
    if (k < n) {
      c1 = s[k].rgba64;
      u1 = uint32_t(round_to_int(s[k].offset * fWidth));
    }
    uint32_t u0 = __shfl_up_sync(0xFFFFFFFFu, u1, 1);
    uint64_t c0 = __shfl_up_sync(0xFFFFFFFFu, c1, 1);
    if (lane == 0) { u0 = car_u0; c0 = car_c; }
    if (lane < ns) {
      LutSpan64 sp;
      const uint32_t i = (u1 >> 8) - (u0 >> 8);
      if (i == 0) c0 = c1;
      sp.start = u0 >> 8;
      sp.count = i + 1u;
      sp.c0 = c0;
      sp.c1 = c1;
      if (c0 != c1 && sp.count > 1) {
        const int32_t div = int32_t(sp.count - 1u);
        sp.inc[0] = uint32_t(int32_t(uint32_t((c1 >> (32 - kLut64Shift)) & kLut64Mask) -
                                     uint32_t((c0 >> (32 - kLut64Shift)) & kLut64Mask)) / div);
        sp.inc[1] = uint32_t(int32_t(uint32_t((c1 >> (16 - kLut64Shift)) & kLut64Mask) -
                                     uint32_t((c0 >> (16 - kLut64Shift)) & kLut64Mask)) / div);
        sp.inc[2] = uint32_t(int32_t(uint32_t((c1 << kLut64Shift) & kLut64Mask) -
                                     uint32_t((c0 << kLut64Shift) & kLut64Mask)) / div);
        sp.inc[3] = uint32_t(int32_t(uint32_t((c1 >> (48 - kLut64Shift)) & kLut64Mask) -
                                     uint32_t((c0 >> (48 - kLut64Shift)) & kLut64Mask)) / div);
      }
      spans[lane] = sp;
    }
    car_u0 = __shfl_sync(0xFFFFFFFFu, u1, ns - 1);
    car_c = __shfl_sync(0xFFFFFFFFu, c1, ns - 1);
    __syncwarp();
    span_end = spans[ns - 1].start + spans[ns - 1].count;
    for (uint32_t e = uint32_t(lane); e < job.lut_size; e += 32) {
      const uint64_t v = first_chunk ? 0ull : lut[e];
      lut[e] = lut_eval64(spans, ns, e, v);
    }
    first_chunk = false;
    __syncwarp();
  }
  // the trailing fill is the last stop's colour; entry 0 is the first stop's
  for (uint32_t e = uint32_t(lane); e < job.lut_size; e += 32) {
    uint64_t v = first_chunk ? 0ull : lut[e];
    if (n == 1) v = premul64(first_c);
    else {
      if (e >= span_end) v = premul64(car_c);
      if (e == 0) v = premul64(first_c);
    }
    lut[e] = v;
  }
}

// One warp per LUT. The span table is built 32 stops at a time, one stop per lane: a span depends
// only on its stop and the one before it (position and colour, passed up one lane; the previous
// chunk's last stop is carried), so the FP64 stop positions and increments of a chunk are computed
// in parallel. Every lane then applies the chunk's spans, in order, to its entries (the entry's
// value is whatever the reference's sequential span writer leaves there: later spans overwrite
// earlier ones). The trailing fill and entry 0 are applied last.
constexpr int kLutWarps = 8;

__global__ void __launch_bounds__(32 * kLutWarps) lut_kernel(const DevLutJob* jobs, const DevStop* stops, uint32_t* luts,
                                                             const uint32_t* counts) {
  const uint32_t num_jobs = counts[kCntLutJobs];
  __shared__ LutSpan spans_all[kLutWarps][32];
  __shared__ LutSpan64 spans64_all[kLutWarps][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t jid = blockIdx.x * kLutWarps + uint32_t(warp);
  if (jid >= num_jobs) return;                         // whole warps leave together
  LutSpan* spans = spans_all[warp];
  const DevLutJob job = jobs[jid];
  const DevStop* s = stops + job.stop_first;
  if (job.variant == kLut64) {                         // offset is even: 8-byte aligned entries
    lut_build64(job, s, reinterpret_cast<uint64_t*>(luts + job.lut_offset), spans64_all[warp], lane);
    return;
  }
  const uint32_t n = job.stop_count;
  const bool scalar = job.variant == kLutScalar;
  const bool avx2 = job.variant == kLutAVX2;
  uint32_t* lut = luts + job.lut_offset;
  const uint32_t first_c = rgba32_of(s[0].rgba64);
  const double fWidth = double(int32_t(job.lut_size - 1u) << 8);
  uint32_t car_u0 = 0, car_c0 = first_c, car_c1 = first_c, span_end = 0;
  bool first_chunk = true;
  for (uint32_t si = (!scalar && s[0].offset == 0.0 && n > 1) ? 1u : 0u; si < n; si += 32) {
    const uint32_t k = si + uint32_t(lane);
    const int ns = int(min(32u, n - si));
    uint32_t c1 = 0, u1 = 0;
    if (k < n) {
      c1 = rgba32_of(s[k].rgba64);
      u1 = uint32_t(round_to_int(s[k].offset * fWidth));
    }
    uint32_t u0 = __shfl_up_sync(0xFFFFFFFFu, u1, 1), c0 = __shfl_up_sync(0xFFFFFFFFu, c1, 1);
    if (lane == 0) { u0 = car_u0; c0 = car_c0; }
    if (lane < ns) {
      LutSpan sp;
      sp.start = u0 >> 8;
      if (scalar) {                                     // lut_spans_scalar, one stop
        const uint32_t i = (u1 >> 8) - (u0 >> 8);
        if (i == 0) c0 = c1;
        sp.count = i + 1u;
        sp.c0 = c0;
        sp.c1 = c1;
        if (c0 != c1 && sp.count > 1) {
          const uint32_t kMask = 0xFFu << 23;
          const int32_t div = int32_t(sp.count - 1u);
          sp.inc[0] = int32_t(((c1 << 7) & kMask) - ((c0 << 7) & kMask)) / div;
          sp.inc[1] = int32_t(((c1 << 15) & kMask) - ((c0 << 15) & kMask)) / div;
          sp.inc[2] = int32_t(((c1 << 23) & kMask) - ((c0 << 23) & kMask)) / div;
          sp.inc[3] = int32_t(((c1 >> 1) & kMask) - ((c0 >> 1) & kMask)) / div;
        }
      }
      else {                                            // lut_spans_simd, one stop
        sp.count = (u1 >> 8) - (u0 >> 8);
        sp.c0 = c0;
        sp.c1 = c1;
        if (sp.count > 1) {
          const double scale = double(1 << 23) / double(int(sp.count));
          for (int ch = 0; ch < 4; ch++) {
            const int32_t cc = int32_t((c0 >> (8 * ch)) & 255u);
            const int32_t dd = int32_t((c1 >> (8 * ch)) & 255u) - cc;
            const double pv = double(dd) * scale;
            sp.inc[ch] = (pv > -2147483649.0 && pv < 2147483648.0) ? __double2int_rz(pv) : INT32_MIN;
          }
        }
      }
      spans[lane] = sp;
    }
    // carry the chunk's last stop
    car_u0 = __shfl_sync(0xFFFFFFFFu, u1, ns - 1);
    car_c1 = __shfl_sync(0xFFFFFFFFu, c1, ns - 1);
    car_c0 = car_c1;
    __syncwarp();
    span_end = spans[ns - 1].start + spans[ns - 1].count + (scalar ? 0u : 1u);
    for (uint32_t e = uint32_t(lane); e < job.lut_size; e += 32) {
      const uint32_t v = first_chunk ? 0u : lut[e];
      lut[e] = scalar ? lut_eval_scalar(spans, ns, e, v) : lut_eval_simd(spans, ns, e, v, avx2);
    }
    first_chunk = false;
    __syncwarp();
  }
  // the last stop's colour is the builder's trailing colour (c0 for SIMD, c1 for scalar)
  const uint32_t tail = scalar ? car_c1 : car_c0;
  for (uint32_t e = uint32_t(lane); e < job.lut_size; e += 32) {
    uint32_t v = first_chunk ? 0u : lut[e];
    if (scalar && n == 1) v = premul_scalar(first_c);
    else {
      if (e >= span_end) v = scalar ? premul_scalar(tail) : premul_simd(tail);
      if (e == 0) v = scalar ? premul_scalar(first_c) : premul_simd(first_c);
    }
    lut[e] = v;
  }
}

// ---------------------------------------------------------------------------------------------
// K1 - FP64 edge building. The reference's builder walks a command's figures sequentially, but
// the cells it produces depend only on the multiset of segments, and the segments of one line or
// curve depend only on that line's or curve's own points: clipping decisions come from the
// points' clip flags, the previous curve ends exactly on this one's first point, and the
// left/right border runs it accumulates are vertical lines at the clip box's x0/x1, whose cells
// add up the same whether consecutive runs are merged or not. So `classify` splits every
// analytic command into items (lines, curves, closing lines) and `edge_items` builds each item
// on its own thread with the reference's clipping builder, appending segments with batched
// atomics. An invalid point (NaN) makes the reference reject the whole command; here it marks the
// command invalid and binning drops it.
// ---------------------------------------------------------------------------------------------

enum : uint32_t { kCmdHasSegments = 1u, kCmdInvalid = 2u };

__device__ __forceinline__ void init_builder(eb::Builder& b, const DevCanvas& cv) {
  b.cx0 = 0.0; b.cy0 = 0.0; b.cx1 = double(cv.w) * 256.0; b.cy1 = double(cv.h) * 256.0;
  b.icx0 = eb::trunc_i(b.cx0); b.icx1 = eb::trunc_i(b.cx1);
  const double tol = 0.20 * 256.0;
  b.tol_sq = tol * tol;
  b.acc_x0_y0 = b.acc_x0_y1 = b.acc_x1_y0 = b.acc_x1_y1 = b.cy0;
  b.px = b.py = 0; b.psign = 0; b.pasc = false;
}

// Walks the figures of a command the way add_from_source does (edgebuilder_p.h:1032-1070) and
// calls fn(kind, a, b) for every line, curve and closing line.
template<typename Fn>
__device__ void for_each_item(const uint8_t* cmd, int n, Fn&& fn) {
  int i = 0;
  for (;;) {
    if (cmd) { while (i < n && cmd[i] != 0) i++; }
    if (i >= n) return;
    int start = i++, prev = start;
    for (;;) {
      if (cmd ? (i != n && cmd[i] == 1) : (i != n)) { fn(kItemLine, prev, i); prev = i; i += 1; }
      else if (cmd && i <= n - 2 && cmd[i] == 2) { fn(kItemQuad, prev, i); prev = i + 1; i += 2; }
      else if (cmd && i < n - 2 && cmd[i] == 4) { fn(kItemCubic, prev, i); prev = i + 2; i += 3; }
      else if (cmd && i < n - 2 && cmd[i] == 3) { fn(kItemConic, prev, i); prev = i + 2; i += 2; }
      else { fn(kItemLine, prev, start); break; }
    }
    if (!cmd) return;
  }
}

__global__ void classify_kernel(FrameView f) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= f.counts[kCntCmds]) return;
  const DevCmd cmd = f.cmds[c];
  if (cmd.kind != kFillAnalytic) return;
  f.cmd_bbox[c] = make_int4(INT32_MAX, INT32_MAX, INT32_MIN, INT32_MIN);
  f.cmds_rw[c].status = 0u;
  const uint8_t* pc = cmd.geom == kGeomPath ? f.path_cmds + cmd.geom_first : nullptr;
  const int n = int(cmd.geom_count);
  // A command with a non-finite transformed point is built whole, by one thread, exactly as the
  // reference builds it (its clip flags then depend on the order points are visited in).
  {
    const DevXform xf = f.xforms[cmd.xform];
    const double* xy = f.verts + 2ull * cmd.geom_first;
    bool finite = true;
    for (int k = 0; k < n; k++) {
      double x = xy[2 * k], y = xy[2 * k + 1], tx, ty;
      if (xf.affine) { tx = x * xf.m[0] + y * xf.m[2] + xf.m[4]; ty = x * xf.m[1] + y * xf.m[3] + xf.m[5]; }
      else { tx = x * xf.m[0] + xf.m[4]; ty = y * xf.m[3] + xf.m[5]; }
      finite &= isfinite(tx) & isfinite(ty);
    }
    if (!finite) {
      uint32_t base = atomicAdd(f.work_counter + 1, 1u);
      if (base < f.item_capacity) f.items[base] = DevItem{c, kItemWhole, 0u, 0u};
      else atomicOr(f.error_flags, kErrItems);
      return;
    }
  }
  // Lines go to the item list (edge_items_kernel); cubic curves to the front of the curve list
  // and quadratic / conic curves to its back (edge_curves_kernel<3> / <2>).
  uint32_t lines = 0, cubics = 0, quads = 0;
  for_each_item(pc, n, [&](uint32_t kind, int, int) {
    lines += kind == kItemLine ? 1u : 0u;
    cubics += kind == kItemCubic ? 1u : 0u;
    quads += (kind == kItemQuad) | (kind == kItemConic) ? 1u : 0u;
  });
  uint32_t base = lines ? atomicAdd(f.work_counter + 1, lines) : 0u;
  uint32_t cbase = cubics ? atomicAdd(f.work_counter + 2, cubics) : 0u;
  uint32_t qbase = quads ? atomicAdd(f.work_counter + 21, quads) : 0u;
  // cubics fill the curve list from the front and quadratics from the back: together, and each
  // list on its own, they must fit (the bound is one item per vertex)
  if (base + lines > f.item_capacity || cbase + cubics > f.item_capacity || qbase + quads > f.item_capacity)
    atomicOr(f.error_flags, kErrItems);
  for_each_item(pc, n, [&](uint32_t kind, int a, int b) {
    const DevItem it{c, kind, uint32_t(a), uint32_t(b)};
    if (kind == kItemLine) {
      if (base < f.item_capacity) f.items[base] = it;
      base++;
    }
    else if (kind == kItemCubic) {
      if (cbase < f.item_capacity) f.curve_items[cbase] = it;
      cbase++;
    }
    else {
      if (qbase < f.item_capacity) f.curve_items[f.item_capacity - 1u - qbase] = it;
      qbase++;
    }
  });
}

// The end of a curve's or piece's builder: border runs emitted, segments flushed, the command's
// bbox, status and binning bound updated.
__device__ __forceinline__ void finish_curve(FrameView& f, eb::Builder& b, uint32_t cmd, uint32_t& rows) {
  b.done();
  b.sink.flush();
  if (b.sink.n) {
    int4* bb = f.cmd_bbox + cmd;
    atomicMin(&bb->x, b.sink.xmin);
    atomicMin(&bb->y, b.sink.ymin);
    atomicMax(&bb->z, b.sink.xmax);
    atomicMax(&bb->w, b.sink.ymax);
    atomicOr(&f.cmds_rw[cmd].status, kCmdHasSegments);
    rows += b.sink.rows;
  }
}

// The lanes' subdivision stacks live in local memory with the top entry in registers
// (eb::CachedStack). Holding the next eight entries in shared memory instead measured slower on
// the batched workload (piece kernel 10.8 -> 14.2 ms): the shared-memory carve-out shrinks the L1
// that the stacks' and the segment sinks' local memory hits in.
constexpr int kCurveThreads = 128;
// work_counter words: cubic pieces inside the clip box, clipped cubic pieces, and their queues
constexpr uint32_t kSafePieces = 28, kClipPieces = 29;
// Idle lanes a warp waits for before it takes new pieces: each refill's set-up costs the warp its
// FP64 instructions whatever the number of lanes refilled. On the batched workload 24 and 28
// measured 246-248 ms per step, 16 and 20 250 ms, 32 251 ms, 8 257 ms and 4 259 ms.
constexpr int kPieceRefillLanes = 24;

// Curves in two kernels. curve_split_kernel<DEG>: one thread per curve of the curve list does
// curve_to's set-up (transform, clip flags, a curve entirely on one side of the clip box, the split
// into monotonic pieces: the divergent, FP64-heavy part) with every lane converged on it, and
// writes the pieces. edge_pieces_kernel<DEG> flattens the pieces lane-scheduled, so taking a new
// piece is cheap and the lanes' subdivision steps stay together. A piece is built by its own
// builder: the border runs a curve accumulates are vertical lines at the clip box's x0/x1 whose
// cells add up the same whether the runs of consecutive pieces are merged or not.
template<int DEG>
__global__ void __launch_bounds__(128) curve_split_kernel(FrameView f) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const uint32_t n_cubic = min(f.work_counter[2], f.item_capacity);
  const uint32_t n_items = DEG == 3 ? n_cubic : min(f.work_counter[21], f.item_capacity - n_cubic);
  uint32_t rows = 0, npieces = 0, cmd_i = 0;
  eb::Pt spline[DEG == 3 ? 25 : 7];
  uint32_t any = 0;
  if (t < n_items) {
    const DevItem it = f.curve_items[DEG == 3 ? t : f.item_capacity - 1u - t];
    const DevCmd& cmd = f.cmds[it.cmd];
    const DevXform& xf = f.xforms[cmd.xform];
    eb::Builder b;
    init_builder(b, f.canvases[cmd.canvas]);
    b.sink.init(f.segs, f.seg_meta, f.totals + 0, f.seg_capacity, it.cmd);
    eb::Src src;
    src.xy = f.verts + 2ull * cmd.geom_first;
    src.affine = xf.affine != 0;
    src.m00 = xf.m[0]; src.m01 = xf.m[1]; src.m10 = xf.m[2]; src.m11 = xf.m[3]; src.m20 = xf.m[4]; src.m21 = xf.m[5];
    const eb::Pt p0 = src.tf(int(it.a));
    spline[1] = src.tf(int(it.b));
    if (DEG == 3) { spline[2] = src.tf(int(it.b) + 1); spline[DEG] = src.tf(int(it.b) + 2); }
    else spline[DEG] = src.tf(int(it.b) + (it.kind == kItemConic ? 2 : 1));
    cmd_i = it.cmd;
    // curve_to's set-up (LaneCurve::prepare, restated on this thread's own spline)
    const uint32_t p0_flags = b.fxy(p0);
    uint32_t common = p0_flags;
    any = p0_flags;
#pragma unroll
    for (int i = 1; i <= DEG; i++) { const uint32_t fl = b.fxy(spline[i]); common &= fl; any |= fl; }
    if (common) {
      if (!(common & (eb::CF_Y0 | eb::CF_Y1))) {
        const double y0 = eb::dclamp(p0.y, b.cy0, b.cy1), y1 = eb::dclamp(spline[DEG].y, b.cy0, b.cy1);
        if (common & eb::CF_X0) b.acc_left(y0, y1); else b.acc_right(y0, y1);
      }
      finish_curve(f, b, it.cmd, rows);
    }
    else {
      spline[0] = p0;
      int nout = DEG == 3 ? eb::split_cubic(spline) : eb::split_quad(spline);
      if (nout == 0) nout = DEG;
      npieces = uint32_t(nout / DEG);
    }
  }
  // one atomic per warp for the pieces of its curves
  uint32_t incl = npieces;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += v;
  }
  const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
  uint32_t base = 0;
  if (lane == 31 && total) base = atomicAdd(f.work_counter + (DEG == 3 ? 23 : 25), total);
  base = __shfl_sync(0xFFFFFFFFu, base, 31) + incl - npieces;
  for (uint32_t k = 0; k < npieces; k++) {
    const uint32_t idx = base + k;
    if (idx >= f.piece_capacity) { atomicOr(f.error_flags, kErrPieces); break; }
    DevPiece pc;
#pragma unroll
    for (int i = 0; i <= DEG; i++) pc.p[i] = make_double2(spline[k * DEG + i].x, spline[k * DEG + i].y);
    pc.cmd = cmd_i;
    pc.any = any;
    f.pieces[DEG == 3 ? idx : f.piece_capacity - 1u - idx] = pc;
  }
  if (DEG == 3) {
    // cubic pieces the safe loop flattens listed from the front of piece_list, the others from its
    // back (one atomic per warp for each), in the pieces' order
    uint32_t safe_mask = 0;                    // bit k: piece k flattens as by the safe loop
    if (npieces) {
      eb::Builder cb;
      init_builder(cb, f.canvases[f.cmds[cmd_i].canvas]);
      for (uint32_t k = 0; k < npieces; k++)
        if (eb::piece_flattens_safe(spline + k * DEG, DEG, any, cb)) safe_mask |= 1u << k;
    }
    const uint32_t n_safe = uint32_t(__popc(safe_mask)), n_clip = npieces - n_safe;
    uint32_t is = n_safe, ic = n_clip;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t vs = __shfl_up_sync(0xFFFFFFFFu, is, o), vc = __shfl_up_sync(0xFFFFFFFFu, ic, o);
      if (lane >= o) { is += vs; ic += vc; }
    }
    const uint32_t ts = __shfl_sync(0xFFFFFFFFu, is, 31), tc = __shfl_sync(0xFFFFFFFFu, ic, 31);
    uint32_t bs = 0, bc = 0;
    if (lane == 31) {
      if (ts) bs = atomicAdd(f.work_counter + kSafePieces, ts);
      if (tc) bc = atomicAdd(f.work_counter + kClipPieces, tc);
    }
    bs = __shfl_sync(0xFFFFFFFFu, bs, 31) + is - n_safe;
    bc = __shfl_sync(0xFFFFFFFFu, bc, 31) + ic - n_clip;
    uint32_t ks = 0, kc = 0;
    for (uint32_t k = 0; k < npieces; k++) {
      const uint32_t idx = base + k;
      if (idx >= f.piece_capacity) break;
      if ((safe_mask >> k) & 1u) f.piece_list[bs + ks++] = idx;
      else f.piece_list[f.piece_capacity - 1u - (bc + kc++)] = idx;
    }
  }
  rows = __reduce_add_sync(0xFFFFFFFFu, rows);
  if (lane == 0 && rows) atomicAdd(f.totals + 1, rows);
}

// The cubic pieces the safe loop flattens (those of curves inside the clip box, and the inside
// pieces of clipped curves: eb::piece_flattens_safe), flattened as subdivision trees (eb::TreeNode)
// whose nodes the lanes of a warp share. A lane splits its node, goes on with the left half and keeps the
// right half on its own stack, unless a lane of the warp is out of work: then the right half goes
// to that lane through shared memory. So lanes do not sit idle while other lanes' trees still have
// nodes, and the FP64 instructions (whose cost to the pipe does not depend on the active lanes)
// serve more of them. The segments are those of the loop flattener, in another order; they are
// appended for the warp with one atomic per step, and each lane accumulates the command bounds
// finish_curve would for the run of segments it emits for one command.

// Idle lanes a warp of the tree flattener waits for before it takes new pieces, and its blocks per
// SM: refills of 16, 24 and 32 lanes and 3, 4 and 6 blocks measured within 1 % of each other on the
// batched workload (215.6-218.6 ms per step); 16 was the best on the curves frame (2.60 ms).
constexpr int kTreeRefillLanes = 16;
constexpr int kTreeBlocksPerSM = 3;

struct alignas(16) TreeXchg {
  double x[4], y[4];
  uint32_t cmd, level, sign, pad;
};

__global__ void __launch_bounds__(kCurveThreads) edge_tree_kernel(FrameView f) {
  constexpr int kWarps = kCurveThreads / 32;
  __shared__ TreeXchg xchg[kWarps][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t n_cubic = min(f.work_counter[23], f.piece_capacity);
  const uint32_t n_items = min(f.work_counter[kSafePieces], n_cubic);
  uint32_t* queue = f.work_counter + kSafePieces + 2;
  const double tol = 0.20 * 256.0;
  const double tol_sq = tol * tol;                    // init_builder's
  eb::TreeNode<3> cur;
  eb::TreeNode<3> stack[eb::kStackLevels];
  int nst = 0;
  uint32_t cmd = 0, sign = 0;
  bool busy = false, exhausted = false;
  // bounds of the segments emitted for command acc_cmd since the last flush
  uint32_t acc_cmd = 0xFFFFFFFFu, acc_rows = 0, rows = 0;
  int xmin = INT32_MAX, ymin = INT32_MAX, xmax = INT32_MIN, ymax = INT32_MIN;
  auto flush_bounds = [&]() {
    if (acc_cmd == 0xFFFFFFFFu) return;
    int4* bb = f.cmd_bbox + acc_cmd;
    atomicMin(&bb->x, xmin);
    atomicMin(&bb->y, ymin);
    atomicMax(&bb->z, xmax);
    atomicMax(&bb->w, ymax);
    atomicOr(&f.cmds_rw[acc_cmd].status, kCmdHasSegments);
    rows += acc_rows;
    acc_cmd = 0xFFFFFFFFu;
    acc_rows = 0;
    xmin = ymin = INT32_MAX;
    xmax = ymax = INT32_MIN;
  };

  for (;;) {
    // new pieces for the idle lanes, as edge_pieces_kernel takes them
    const uint32_t want = __ballot_sync(0xFFFFFFFFu, !busy && !exhausted);
    if (want && (__popc(want) >= kTreeRefillLanes || !__any_sync(0xFFFFFFFFu, busy))) {
      const int leader = __ffs(want) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(queue, uint32_t(__popc(want)));
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      if (!busy && !exhausted) {
        const uint32_t t = base + uint32_t(__popc(want & lt));
        if (t >= n_items) {
          exhausted = true;
        }
        else {
          const uint32_t pi = f.piece_list[t];
          // an entry of a piece that did not fit in the piece array (the frame fails) is skipped
          if (pi < n_cubic) {
            const DevPiece pc = f.pieces[pi];
            eb::Pt pts[4];
#pragma unroll
            for (int i = 0; i < 4; i++) pts[i] = eb::Pt{pc.p[i].x, pc.p[i].y};
            cur = eb::tree_root<3>(pts, sign);
            cmd = pc.cmd;
            nst = 0;
            busy = true;
          }
        }
      }
    }
    if (__all_sync(0xFFFFFFFFu, !busy && exhausted)) break;

    eb::TreeNode<3> left, right;
    const bool leaf = busy && eb::tree_step<3>(cur, tol_sq, left, right);
    const bool split = busy && !leaf;

    // a leaf's segment (Builder::add after desc_open, Sink::emit), one atomic for the warp
    int x0 = 0, y0 = 0, x1 = 0, y1 = 0;
    if (leaf) {
      x0 = eb::trunc_i(cur.p[0].x); y0 = eb::trunc_i(cur.p[0].y);
      x1 = eb::trunc_i(cur.p[3].x); y1 = eb::trunc_i(cur.p[3].y);
    }
    const bool emit = leaf && y0 != y1;
    const uint32_t em = __ballot_sync(0xFFFFFFFFu, emit);
    if (em) {
      const int leader = __ffs(em) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(f.totals + 0, uint32_t(__popc(em)));
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      if (emit) {
        const uint32_t idx = base + uint32_t(__popc(em & lt));
        if (idx < f.seg_capacity) {
          f.segs[idx] = DevSeg{x0, y0, x1, y1};
          f.seg_meta[idx] = (cmd << 1) | sign;
        }
        if (cmd != acc_cmd) { flush_bounds(); acc_cmd = cmd; }
        // Sink::emit's bounds and seglist-entry bound
        const uint32_t strips = (uint32_t((y1 - 1) >> 8) >> kStripShift) - (uint32_t(y0 >> 8) >> kStripShift) + 1u;
        const int lo = min(x0, x1) - 256, hi = max(x0, x1) + 256;
        const uint32_t tiles = uint32_t((((hi >> 8) + 1) >> kTileShift) - ((lo >> 8) >> kTileShift) + 1);
        acc_rows += tiles + 3u * strips;
        ymin = min(ymin, y0);
        ymax = max(ymax, y1);
        xmin = min(xmin, min(x0, x1));
        xmax = max(xmax, max(x0, x1));
      }
    }
    if (leaf) {
      if (nst) cur = stack[--nst];
      else busy = false;
    }

    // the right halves of this step's splits go first to the lanes out of work
    const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !busy);
    const uint32_t donors = __ballot_sync(0xFFFFFFFFu, split);
    const int k = min(__popc(idle), __popc(donors));
    if (split) {
      const int r = __popc(donors & lt);
      if (r < k) {
        TreeXchg& x = xchg[w][r];
#pragma unroll
        for (int i = 0; i < 4; i++) { x.x[i] = right.p[i].x; x.y[i] = right.p[i].y; }
        x.cmd = cmd;
        x.level = uint32_t(right.level);
        x.sign = sign;
      }
      else {
        stack[nst++] = right;
      }
      cur = left;
    }
    __syncwarp();
    if (!busy) {
      const int q = __popc(idle & lt);
      if (q < k) {
        const TreeXchg& x = xchg[w][q];
#pragma unroll
        for (int i = 0; i < 4; i++) cur.p[i] = eb::Pt{x.x[i], x.y[i]};
        cur.level = int(x.level);
        cmd = x.cmd;
        sign = x.sign;
        nst = 0;
        busy = true;
      }
    }
    __syncwarp();
  }
  flush_bounds();
  rows = __reduce_add_sync(0xFFFFFFFFu, rows);
  if (lane == 0 && rows) atomicAdd(f.totals + 1, rows);
}

// Cubic pieces in two kernels: those inside the clip box (most of them) are flattened by
// edge_tree_kernel, whose lanes share the nodes of their subdivision trees; the clipped ones run the
// clipping state machine here. Quadratic and conic pieces all take this kernel.
enum PieceSet : int { kPiecesAll = 0, kPiecesClipped = 2 };

template<int DEG, int SET>
__global__ void __launch_bounds__(kCurveThreads) edge_pieces_kernel(FrameView f) {
  const int lane = threadIdx.x & 31;
  const uint32_t n_cubic = min(f.work_counter[23], f.piece_capacity);
  const uint32_t n_items = SET == kPiecesClipped ? min(f.work_counter[kClipPieces], n_cubic)
                         : DEG == 3 ? n_cubic : min(f.work_counter[25], f.piece_capacity - n_cubic);
  uint32_t* queue = f.work_counter + (SET == kPiecesClipped ? kClipPieces + 2 : DEG == 3 ? 24 : 26);
  eb::Builder b;
  eb::LaneCurve<DEG, eb::CachedStack<DEG>> lc;
  bool busy = false, exhausted = false;
  uint32_t cur = 0, rows = 0;

  for (;;) {
    // hand the next pieces of the list to the idle lanes (one atomic per warp), once enough lanes
    // are idle that the set-up's FP64 instructions serve several pieces at once
    const uint32_t want = __ballot_sync(0xFFFFFFFFu, !busy && !exhausted);
    if (want && (__popc(want) >= kPieceRefillLanes || !__any_sync(0xFFFFFFFFu, busy))) {
      const int leader = __ffs(want) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(queue, uint32_t(__popc(want)));
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      if (!busy && !exhausted) {
        const uint32_t t = base + uint32_t(__popc(want & ((1u << lane) - 1u)));
        if (t >= n_items) {
          exhausted = true;
        }
        else {
          const uint32_t pi = SET == kPiecesClipped ? f.piece_list[f.piece_capacity - 1u - t]
                            : DEG == 3 ? t : f.piece_capacity - 1u - t;
          // a list entry is written only for a piece that fit in the piece array; with a frame
          // that overflowed it (reported by curve_split), an entry may be stale: the lane then
          // stays idle and takes another piece
          if (SET == kPiecesAll || pi < n_cubic) {
            const DevPiece pc = f.pieces[pi];
            cur = pc.cmd;
            init_builder(b, f.canvases[f.cmds[cur].canvas]);
            b.sink.init(f.segs, f.seg_meta, f.totals + 0, f.seg_capacity, cur);
            eb::Pt pts[DEG + 1];
#pragma unroll
            for (int i = 0; i <= DEG; i++) pts[i] = eb::Pt{pc.p[i].x, pc.p[i].y};
            busy = lc.begin_piece(b, pts, pc.any);
            if (!busy) finish_curve(f, b, cur, rows);
          }
        }
      }
    }
    if (__all_sync(0xFFFFFFFFu, !busy && exhausted)) break;   // the list is exhausted
    if (busy) {
      lc.step(b);
      if (lc.state == eb::kLsDone && !lc.next_piece(b, true)) {
        finish_curve(f, b, cur, rows);
        busy = false;
      }
    }
  }
  rows = __reduce_add_sync(0xFFFFFFFFu, rows);
  if (lane == 0 && rows) atomicAdd(f.totals + 1, rows);
}

__global__ void __launch_bounds__(256) edge_items_kernel(FrameView f) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t rows = 0;
  bool emitted = false;                        // the lane built an item whose segments count
  eb::Builder b;
  const uint32_t n_items = min(f.work_counter[1], f.item_capacity);
  if (t < n_items) {
    const DevItem it = f.items[t];
    const DevCmd cmd = f.cmds[it.cmd];
    const DevCanvas cv = f.canvases[cmd.canvas];
    const DevXform xf = f.xforms[cmd.xform];
    init_builder(b, cv);
    b.sink.init(f.segs, f.seg_meta, f.totals + 0, f.seg_capacity, it.cmd);
    eb::Src src;
    src.xy = f.verts + 2ull * cmd.geom_first;
    src.cmd = cmd.geom == kGeomPath ? f.path_cmds + cmd.geom_first : nullptr;
    src.affine = xf.affine != 0;
    src.m00 = xf.m[0]; src.m01 = xf.m[1]; src.m10 = xf.m[2]; src.m11 = xf.m[3]; src.m20 = xf.m[4]; src.m21 = xf.m[5];
    eb::Pt a = src.tf(int(it.a));
    uint32_t a_flags = b.fxy(a);
    int rc = 0;
    if (it.kind == kItemWhole) {
      src.i = 0;
      src.n = int(cmd.geom_count);
      rc = eb::build(b, src);                  // includes done()
    }
    else if (it.kind == kItemLine) {
      src.i = src.n = 0;                       // no further lines: line_to builds exactly this one
      rc = eb::line_to(b, src, a, a_flags, src.tf(int(it.b)));
    }
    else {
      // the source ends right after this curve, so curve_to consumes exactly one
      src.i = int(it.b);
      src.n = int(it.b) + (it.kind == kItemQuad ? 2 : 3);
      if (it.kind == kItemCubic) eb::curve_to<3>(b, src, a, a_flags, false);
      else eb::curve_to<2>(b, src, a, a_flags, it.kind == kItemConic);
    }
    if (rc) {
      atomicOr(&f.cmds_rw[it.cmd].status, kCmdInvalid);
    }
    else {
      if (it.kind != kItemWhole) b.done();
      emitted = true;
    }
  }
  // What is left in the lanes' sinks (a line item's one segment, mostly) goes out with one atomic
  // for the warp, and the command bounds with one set of atomics per command of the warp (the
  // items of a polygon or path sit in consecutive lanes): Sink::flush and finish_curve's work.
  const int lane = threadIdx.x & 31;
  const uint32_t nb = emitted ? uint32_t(b.sink.nb) : 0u;
  uint32_t incl = nb;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += v;
  }
  const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
  if (total) {
    uint32_t base = 0;
    if (lane == 31) base = atomicAdd(f.totals + 0, total);
    base = __shfl_sync(0xFFFFFFFFu, base, 31) + incl - nb;
    for (uint32_t k = 0; k < nb; k++) {
      if (base + k < f.seg_capacity) {
        f.segs[base + k] = b.sink.buf[k];
        f.seg_meta[base + k] = (b.sink.cmd << 1) | b.sink.sbuf[k];
      }
    }
  }
  const bool has = emitted && b.sink.n;
  const uint32_t key = has ? b.sink.cmd : 0xFFFFFFFFu;
  const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
  if (has) {
    const int x0 = __reduce_min_sync(peers, b.sink.xmin), y0 = __reduce_min_sync(peers, b.sink.ymin);
    const int x1 = __reduce_max_sync(peers, b.sink.xmax), y1 = __reduce_max_sync(peers, b.sink.ymax);
    if (lane == __ffs(peers) - 1) {
      int4* bb = f.cmd_bbox + key;
      atomicMin(&bb->x, x0);
      atomicMin(&bb->y, y0);
      atomicMax(&bb->z, x1);
      atomicMax(&bb->w, y1);
      atomicOr(&f.cmds_rw[key].status, kCmdHasSegments);
    }
    rows = b.sink.rows;
  }
  rows = __reduce_add_sync(0xFFFFFFFFu, rows);
  if (lane == 0 && rows) atomicAdd(f.totals + 1, rows);
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

// Between the halves: the sizes the counting half produced must fit the arrays the rendering half
// writes (they always do in an eager run, whose arrays are sized from them; a graph frame's are
// sized by capacities). Otherwise the rendering half is skipped and the host re-runs the frame.
__global__ void frame_gate_kernel(FrameView f) {
  const uint32_t* t = f.totals;
  const bool over = t[0] > min(f.seg_capacity, f.num_segs) || t[1] > f.num_seglist || t[2] > f.num_cmdrows ||
                    t[3] > f.num_row_entries || t[4] > f.num_row_states || t[6] > f.num_row_runs;
  if (over) {
    f.work_counter[kSkipWord] = 1u;
    atomicOr(f.error_flags, kErrCapacity);
  }
}

__device__ __forceinline__ bool frame_skipped(const FrameView& f) { return f.work_counter[kSkipWord] != 0u; }

// Tile ranges of every command (empty commands get 0xFFFFFFFF) and its number of tile rows.
__global__ void cmd_tiles_kernel(FrameView f, uint32_t* cmdrow_counts_per_cmd, uint32_t* row_counts) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= f.counts[kCntCmds]) {
    // entries beyond the frame's commands (up to the capacity the scans run over) count nothing
    if (c < f.num_cmds) { cmdrow_counts_per_cmd[c] = 0; f.rs_count[c] = 0; f.rb_count[c] = 0; }
    return;
  }
  const DevCmd cmd = f.cmds[c];
  const DevCanvas cv = f.canvases[cmd.canvas];
  int x0, y0, x1, y1;   // inclusive pixel range
  bool empty = false;
  if (cmd.kind == kFillAnalytic) {
    // pixel bbox of the coverage: rows [ymin >> 8, (ymax - 1) >> 8], columns [xmin >> 8, xmax >> 8]
    const uint32_t st = cmd.status;
    empty = (st & kCmdInvalid) || !(st & kCmdHasSegments);
    f.cmds_rw[c].status = (st & kCmdInvalid) ? 1u : (empty ? 2u : 0u);
    const int4 bb = f.cmd_bbox[c];
    x0 = max(bb.x >> 8, 0); y0 = max(bb.y >> 8, 0);
    x1 = min(bb.z >> 8, cv.w - 1); y1 = min((bb.w - 1) >> 8, cv.h - 1);
    if (!empty) {
      f.cmds_rw[c].box[0] = x0; f.cmds_rw[c].box[1] = y0;
      f.cmds_rw[c].box[2] = x1; f.cmds_rw[c].box[3] = y1;
    }
  }
  else if (cmd.kind == kFillBoxA || cmd.kind == kFillMaskA) {
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
    f.cmd_xr[c] = 0x0000FFFFu;   // x0 = 65535 > x1 = 0: overlaps nothing
    f.cmd_yr[c] = 0x0000FFFFu;
    cmdrow_counts_per_cmd[c] = 0;
    f.rs_count[c] = 0;
    f.rb_count[c] = 0;
    return;
  }
  const uint32_t fetch = f.styles[cmd.style].fetch;
  f.rs_count[c] = px::has_row_table(fetch) ? uint32_t(y1 - y0 + 1) : 0u;
  // conic row runs: the reference restarts the fetcher at each band of an analytic fill, once for
  // a box fill
  f.rb_count[c] = fetch != kFetchConic ? 0u
                : cmd.kind == kFillAnalytic ? uint32_t(y1 / cv.band_height - y0 / cv.band_height + 1) : 1u;
  f.cmd_xr[c] = uint32_t(x0) | (uint32_t(x1) << 16);
  f.cmd_yr[c] = uint32_t(y0) | (uint32_t(y1) << 16);
  uint32_t tx0 = uint32_t(x0) >> kTileShift, tx1 = uint32_t(x1) >> kTileShift;
  // the command's list rows (1 << list_shift pixel rows each)
  uint32_t ty0 = uint32_t(y0) >> f.list_shift, ty1 = uint32_t(y1) >> f.list_shift;
  f.cmd_tile_x[c] = tx0 | (tx1 << 16);
  f.cmd_tile_y[c] = ty0 | (ty1 << 16);
  // segment lists are kept per (command, strip row, tile column)
  cmdrow_counts_per_cmd[c] = cmd.kind == kFillAnalytic
      ? ((uint32_t(y1) >> kStripShift) - (uint32_t(y0) >> kStripShift) + 1u) * (tx1 - tx0 + 1u) : 0u;

  const uint32_t row_base = cv.row_base << (kTileShift - f.list_shift);
  for (uint32_t r = ty0; r <= ty1; r++) atomicAdd(&row_counts[row_base + r], 1u);
}

// Segments per (command, strip row, tile column) slot: a segment belongs to every slot its cells
// can touch within each strip row. Pass 0 counts the slots' segments and records each slot's
// command; tiles entirely right of a segment get its per-row cover in their backdrop (added once,
// at the first tile right of it; a prefix over tile columns carries it on). Pass 1 writes the
// (segment, mask index) work items, grouped by slot in slot order, so the items of consecutive
// slots with segments are contiguous.
__global__ void __launch_bounds__(256) seg_bin_kernel(FrameView f, int scatter) {
  if (frame_skipped(f)) return;
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  // the segments the edge builders emitted must all have found a place in the segment array
  if (s == 0 && !scatter && f.totals[0] > f.seg_capacity) atomicOr(f.error_flags, kErrSegments);
  if (s >= min(f.totals[0], min(f.seg_capacity, f.num_segs))) return;
  const uint32_t c = f.seg_meta[s] >> 1;
  const uint32_t ctx = f.cmd_tile_x[c];
  if (ctx == 0xFFFFFFFFu) return;
  const uint32_t sm = 0u - (f.seg_meta[s] & 1u);
  const int tx0 = int(ctx & 0xFFFFu), tx1 = int(ctx >> 16), ntx = tx1 - tx0 + 1;
  const uint32_t yr = f.cmd_yr[c];
  const int sr0 = int((yr & 0xFFFFu) >> kStripShift), sr1 = int((yr >> 16) >> kStripShift);
  const DevSeg g = f.segs[s];
  const int ey0 = g.y0 >> 8, ey1 = (g.y1 - 1) >> 8;
  const int r0 = max(ey0 >> kStripShift, sr0), r1 = min(ey1 >> kStripShift, sr1);
  const uint32_t base = f.cmdrow_base[c];
  for (int r = r0; r <= r1; r++) {
    int t_first, t_last;
    strip_tile_range(g, r, t_first, t_last);
    const int t0 = max(t_first, tx0), t1 = min(t_last, tx1);
    const uint32_t row_slot = base + uint32_t(r - sr0) * uint32_t(ntx);
    for (int t = t0; t <= t1; t++) {
      const uint32_t slot = row_slot + uint32_t(t - tx0);
      if (!scatter) {
        atomicAdd(&f.cmdrow_counts[slot], 1u);
        f.slot_cmd[slot] = c;
      }
      else {
        const uint32_t pos = f.slot_first[slot] + atomicSub(&f.cmdrow_counts[slot], 1u) - 1u;
        if (pos >= f.num_seglist) { atomicOr(f.error_flags, kErrSeglist); continue; }
        f.entries[pos] = make_uint2(s, f.slot_mask[slot] - 1u);
      }
    }
    if (!scatter && t_last + 1 <= tx1) {
      uint32_t* bd = f.backdrop + size_t(row_slot + uint32_t(t_last + 1 - tx0)) * kStripRows;
      int ya = max(ey0, r << kStripShift), yb = min(ey1, (r << kStripShift) + kStripRows - 1);
      for (int y = ya; y <= yb; y++) {
        int top = max(g.y0, y << 8), bot = min(g.y1, (y + 1) << 8);
        uint32_t cov = (uint32_t(bot - top) ^ sm) - sm;
        atomicAdd(&bd[y & (kStripRows - 1)], cov << 9);
      }
    }
  }
}

// Slots with segments get a compact mask index: flags for the scan ...
// Slots of the frame: the binning count from the device totals, within the arrays' capacity.
__device__ __forceinline__ uint32_t frame_slots(const FrameView& f) { return min(f.totals[2], f.num_cmdrows); }

__global__ void slot_flags_kernel(FrameView f) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < f.num_cmdrows) f.cmdrow_offsets[i] = (i < frame_slots(f) && f.cmdrow_counts[i]) ? 1u : 0u;
}

// ... and, after the scan, the maps between slots and mask indices.
__global__ void slot_compact_kernel(FrameView f) {
  if (frame_skipped(f)) return;
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t n = frame_slots(f);
  if (i >= n) return;
  if (f.cmdrow_counts[i]) {
    const uint32_t idx = f.cmdrow_offsets[i];
    f.slot_mask[i] = idx + 1u;
    f.mask_slot[idx] = i;
    // what the coverage pass needs of the slot, gathered here where every slot is independent
    const uint32_t c = f.slot_cmd[i];
    const uint32_t ctx = f.cmd_tile_x[c];
    const uint32_t ntx = (ctx >> 16) - (ctx & 0xFFFFu) + 1u;
    const uint32_t local = i - f.cmdrow_base[c];
    const uint32_t sr = ((f.cmd_yr[c] & 0xFFFFu) >> kStripShift) + local / ntx;
    f.mask_info[idx] = make_uint4(((ctx & 0xFFFFu) + local % ntx) << kTileShift, sr << kStripShift,
                                  (f.cmds[c].flags << 16) | f.cmds[c].alpha, i);
  }
  else {
    f.slot_mask[i] = 0u;
  }
  if (i == n - 1) f.totals[5] = f.cmdrow_offsets[i] + (f.cmdrow_counts[i] ? 1u : 0u);
}

// Prefix of the backdrop deltas over the tile columns of every (command, strip row, row): one
// warp per command (most commands are a few strip rows tall), nothing to do for one column.
constexpr uint32_t kPrefixWarps = 8;
__global__ void __launch_bounds__(32 * kPrefixWarps) backdrop_prefix_kernel(FrameView f) {
  if (frame_skipped(f)) return;
  const uint32_t c = blockIdx.x * kPrefixWarps + (threadIdx.x >> 5);
  if (c >= f.counts[kCntCmds]) return;
  const uint32_t ctx = f.cmd_tile_x[c];
  if (ctx == 0xFFFFFFFFu || f.cmds[c].kind != kFillAnalytic) return;
  const uint32_t ntx = (ctx >> 16) - (ctx & 0xFFFFu) + 1u;
  if (ntx == 1) return;
  const uint32_t yr = f.cmd_yr[c];
  const uint32_t nsr = ((yr >> 16) >> kStripShift) - ((yr & 0xFFFFu) >> kStripShift) + 1u;
  const uint32_t base = f.cmdrow_base[c];
  for (uint32_t i = threadIdx.x & 31u; i < nsr * kStripRows; i += 32u) {
    uint32_t sr = i / kStripRows, row = i % kStripRows;
    uint32_t* bd = f.backdrop + size_t(base + sr * ntx) * kStripRows + row;
    uint32_t acc = 0;
    for (uint32_t t = 0; t < ntx; t++) { acc += bd[t * kStripRows]; bd[t * kStripRows] = acc; }
  }
}

// Canvas transfers with page-locked host images: one block column per canvas, one warp per row,
// 4-byte words across the lanes. One launch moves every canvas of a frame, with any strides on
// either side (a DMA copy per canvas pays a per-row cost on the many short rows of small canvases).
__global__ void __launch_bounds__(256) canvas_copy_kernel(const DevXfer* xfers, uint32_t n, int to_host) {
  const uint32_t i = blockIdx.x;
  if (i >= n) return;
  const DevXfer t = xfers[i];
  const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
  for (int y = int(blockIdx.y) * warps + (threadIdx.x >> 5); y < t.h; y += int(gridDim.y) * warps) {
    if (t.a8) {      // strides in bytes
      const uint8_t* src = reinterpret_cast<const uint8_t*>(to_host ? t.dev : t.host) +
                           int64_t(y) * (to_host ? t.dev_stride : t.host_stride);
      uint8_t* dst = reinterpret_cast<uint8_t*>(to_host ? t.host : t.dev) + int64_t(y) * (to_host ? t.host_stride : t.dev_stride);
      for (int x = lane; x < t.w; x += 32) dst[x] = src[x];
      continue;
    }
    const uint32_t* src = to_host ? t.dev + int64_t(y) * t.dev_stride : t.host + int64_t(y) * t.host_stride;
    uint32_t* dst = to_host ? t.host + int64_t(y) * t.host_stride : t.dev + int64_t(y) * t.dev_stride;
    // 16-byte accesses when both rows start at 16-byte boundaries: a quarter of the instructions
    // and of the link transactions, so the copy takes less from the kernels it runs beside
    if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0) {
      const int w4 = t.w >> 2;
      for (int x = lane; x < w4; x += 32)
        reinterpret_cast<uint4*>(dst)[x] = reinterpret_cast<const uint4*>(src)[x];
      for (int x = (w4 << 2) + lane; x < t.w; x += 32) dst[x] = src[x];
    }
    else {
      for (int x = lane; x < t.w; x += 32) dst[x] = src[x];
    }
  }
}

int launch_canvas_copy(const DevXfer* xfers, uint32_t n, int to_host, cudaStream_t st) {
  if (!n) return 0;
  canvas_copy_kernel<<<dim3(n, 16), 256, 0, st>>>(xfers, n, to_host);
  return 1;
}

int launch_frame_gate(const FrameView& f, cudaStream_t st) {
  frame_gate_kernel<<<1, 1, 0, st>>>(f);
  return 1;
}

int launch_backdrop_prefix(const FrameView& f, cudaStream_t st) {
  if (!f.num_cmds || !f.num_cmdrows) return 0;
  backdrop_prefix_kernel<<<(f.num_cmds + kPrefixWarps - 1) / kPrefixWarps, 32 * kPrefixWarps, 0, st>>>(f);
  return 1;
}

constexpr uint32_t kRecSolid = 0x80000000u;   // command-list record: the style is solid, its colour in the record

// Per tile row: commands overlapping the row in painter's order (one block per row).
__global__ void row_fill_kernel(FrameView f, const uint32_t* row_canvas) {
  __shared__ uint32_t smem[32];
  uint32_t row = blockIdx.x;
  const uint32_t log2 = kTileShift - f.list_shift;
  if (row >= (f.counts[kCntRows] << log2) || frame_skipped(f)) return;        // whole blocks leave together
  const DevCanvas cv = f.canvases[row_canvas[row]];
  uint32_t r = row - (cv.row_base << log2);
  uint32_t out = f.row_offsets[row];
  uint32_t copies = 0;
  for (uint32_t base = 0; base < cv.cmd_count; base += blockDim.x) {
    uint32_t c = cv.cmd_first + base + threadIdx.x;
    uint32_t flag = 0;
    if (base + threadIdx.x < cv.cmd_count) {
      uint32_t ty = f.cmd_tile_y[c];
      flag = (ty != 0xFFFFFFFFu && (ty & 0xFFFFu) <= r && (ty >> 16) >= r) ? 1u : 0u;
      copies += flag & f.cmds[c].flags;               // bit 0: SrcCopy
    }
    uint32_t total;
    uint32_t pos = block_exclusive_scan(flag, smem, total);
    if (flag) {
      // everything the composite needs of the command to test it against a strip and find its
      // slot, gathered once here for every strip of the list row
      // A solid fill's colour (DevCmd::color) takes the place of the row-state base it does not
      // use, with bit 31 of the style word saying so: the composite then loads neither the command
      // nor the style.
      const DevCmd& cmd = f.cmds[c];
      const uint32_t ctx = f.cmd_tile_x[c];
      const uint32_t meta = cmd.kind | (cmd.flags << 2) | (cmd.alpha << 4);
      const bool solid = f.styles[cmd.style].fetch == kFetchSolid;
      uint4* rec = f.row_recs + 2u * (out + pos);
      f.row_box[out + pos] = make_uint2(f.cmd_xr[c], f.cmd_yr[c]);
      rec[0] = make_uint4(c, f.cmd_xr[c], f.cmd_yr[c], meta);
      rec[1] = make_uint4(f.cmdrow_base[c], (ctx & 0xFFFFu) | (((ctx >> 16) - (ctx & 0xFFFFu) + 1u) << 16),
                          cmd.style | (solid ? kRecSolid : 0u), solid ? cmd.color : f.rs_base[c]);
    }
    out += total;
  }
  uint32_t total_copies;
  block_exclusive_scan(copies, smem, total_copies);
  if (threadIdx.x == 0) f.row_copies[row] = total_copies;
}

// ---------------------------------------------------------------------------------------------
// K3a - coverage. A slot is (analytic command, strip row, tile column): 4 rows x 32 pixels. One
// block takes kCoverSlots consecutive slots with segments (by mask index), whose work items are
// contiguous: it rasterizes them, a chunk at a time sorted by the DDA path the reference
// rasterizer takes (so a warp's lanes follow the same path), into the slots' cells in shared memory
// (atomicAdd: u32 sums commute) and their left-of-tile cover into the slots' backdrops, then one
// warp per slot sweeps the cells (8-lane shuffle prefix per row from the backdrop) into 128 8-bit
// masks.
// ---------------------------------------------------------------------------------------------

constexpr int kStripsPerTile = kTileH / kStripRows;
constexpr int kFineWarps = kFineThreads / 32;
constexpr int kSlotPixels = kStripRows * kTileW;

// DDA path a segment takes through the reference rasterizer (prepare's classification).
__device__ __forceinline__ uint32_t dda_kind(const DevSeg& g) {
  const int dx = g.x1 - g.x0, adx = dx < 0 ? -dx : dx, dy = g.y1 - g.y0;
  if ((g.x0 >> 8) == (g.x1 >> 8) && ((g.y0 >> 8) == ((g.y1 - 1) >> 8) || adx == 0)) return 0u;
  return dy >= adx ? (dx < 0 ? 2u : 1u) : (dx < 0 ? 4u : 3u);
}

// K slots per group, 4 threads per slot; a round sorts and rasterizes up to 4 items per thread.
template<int K>
__global__ void __launch_bounds__(4 * K) coverage_kernel(FrameView f) {
  constexpr int kCoverThreads = 4 * K;
  constexpr int kCoverChunk = 4 * kCoverThreads;
  __shared__ __align__(16) uint32_t cells[K][kSlotPixels];
  __shared__ uint32_t bd[K][kStripRows];
  __shared__ int2 org[K];                  // x of the slot's first column, its first row
  __shared__ uint32_t meta[K];             // command flags << 16 | alpha
  __shared__ uint2 items[kCoverChunk];
  __shared__ uint32_t kcount[5], kbase[5];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (frame_skipped(f)) return;
  const uint32_t num_masks = min(f.totals[5], f.mask_capacity);
  if (blockIdx.x == 0 && tid == 0 && f.totals[5] > f.mask_capacity) atomicOr(f.error_flags, kErrMasks);
  const uint32_t groups = (num_masks + K - 1) / K;

  for (uint32_t grp = blockIdx.x; grp < groups; grp += gridDim.x) {
    const uint32_t m0 = grp * K;
    const int nk = int(min(uint32_t(K), num_masks - m0));
    if (tid < nk) {
      const uint4 info = f.mask_info[m0 + tid];
      const uint32_t slot = info.w;
      org[tid] = make_int2(int(info.x), int(info.y));
      meta[tid] = info.z;
      const uint4 b4 = *reinterpret_cast<const uint4*>(f.backdrop + size_t(slot) * kStripRows);
      bd[tid][0] = b4.x; bd[tid][1] = b4.y; bd[tid][2] = b4.z; bd[tid][3] = b4.w;
    }
    for (int i = tid; i < K * kSlotPixels / 4; i += kCoverThreads)
      reinterpret_cast<uint4*>(&cells[0][0])[i] = make_uint4(0u, 0u, 0u, 0u);
    const uint32_t e0 = f.slot_first[f.mask_slot[m0]];
    const uint32_t e1 = f.slot_first[f.mask_slot[m0 + uint32_t(nk) - 1u] + 1u];
    __syncthreads();

    for (uint32_t chunk = e0; chunk < e1; chunk += kCoverChunk) {
      const int n = int(min(uint32_t(kCoverChunk), e1 - chunk));
      if (tid < 5) kcount[tid] = 0;
      __syncthreads();
      // sort the chunk's items by DDA kind (counting sort through shared memory)
      uint2 it[kCoverChunk / kCoverThreads];
      uint32_t kind[kCoverChunk / kCoverThreads], pos[kCoverChunk / kCoverThreads];
#pragma unroll
      for (int q = 0; q < kCoverChunk / kCoverThreads; q++) {
        const int i = tid + q * kCoverThreads;
        if (i < n) {
          it[q] = f.entries[chunk + uint32_t(i)];
          kind[q] = dda_kind(f.segs[it[q].x]);
          pos[q] = atomicAdd(&kcount[kind[q]], 1u);
        }
      }
      __syncthreads();
      if (tid == 0) {
        uint32_t acc = 0;
        for (int k = 0; k < 5; k++) { kbase[k] = acc; acc += kcount[k]; }
      }
      __syncthreads();
#pragma unroll
      for (int q = 0; q < kCoverChunk / kCoverThreads; q++) {
        const int i = tid + q * kCoverThreads;
        if (i < n) items[kbase[kind[q]] + pos[q]] = it[q];
      }
      __syncthreads();
      for (int i = tid; i < n; i += kCoverThreads) {
        const uint2 e = items[i];
        const int j = int(e.y - m0);
        ras::WindowSink sink{cells[j], bd[j], org[j].x};
        ras::segment_to_window(f.segs[e.x], f.seg_meta[e.x] & 1u, org[j].y, kStripRows, INT32_MAX, sink);
      }
      __syncthreads();
    }

    // sweep: lane covers row lane / 8, columns (lane % 8) * 4 .. + 3 of the slot
    const int prow = lane >> 3;
    for (int j = warp; j < nk; j += kCoverThreads / 32) {
      const uint32_t flags = meta[j] >> 16, alpha = meta[j] & 0xFFFFu;
      const uint4 cv4 = *reinterpret_cast<const uint4*>(&cells[j][lane * 4]);
      const uint32_t s4 = cv4.x + cv4.y + cv4.z + cv4.w;
      uint32_t inc = s4;
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xFFFFFFFFu, inc, o, 8);
        if ((lane & 7) >= o) inc += v;
      }
      uint32_t cov = (256u << 9) + bd[j][prow] + inc - s4;
      const uint32_t rule = (flags & 2u) ? 0x1FFu : 0xFFFFFFFFu;
      uint32_t m;
      cov += cv4.x; m = px::calc_mask(cov, rule, alpha);
      cov += cv4.y; m |= px::calc_mask(cov, rule, alpha) << 8;
      cov += cv4.z; m |= px::calc_mask(cov, rule, alpha) << 16;
      cov += cv4.w; m |= px::calc_mask(cov, rule, alpha) << 24;
      reinterpret_cast<uint32_t*>(f.masks + size_t(m0 + uint32_t(j)) * kSlotPixels)[lane] = m;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------------
// K3b - composite, persistent. The work unit is a strip of kStripRows x kTileW pixels (one warp,
// 4 pixels per lane held in registers from one 128-bit load to one 128-bit store). Warps pull
// strips from an atomic queue and never wait on each other; the commands of the strip's tile row
// that overlap the strip are applied in painter's order: analytic commands read their 4 masks per
// lane from the coverage pass, box fills compute theirs, then fetch + SrcOver/SrcCopy.
// ---------------------------------------------------------------------------------------------

// The lane's 4 masks of command `ci` in its strip: analytic commands from the slot's masks (or the
// backdrop alone when no segment reaches the slot: `mw` is then the row's backdrop), boxes from
// their rectangles.
__device__ __forceinline__ void strip_masks(const FrameView& f, uint32_t ckind, uint32_t ci, uint32_t cmeta,
                                            uint32_t cnseg, uint32_t mw, int xp, int y, uint32_t m[4]) {
  const uint32_t alpha = cmeta & 0xFFFFu;
  if (ckind == kFillAnalytic) {
    if (cnseg) {
      m[0] = mw & 0xFFu; m[1] = (mw >> 8) & 0xFFu; m[2] = (mw >> 16) & 0xFFu; m[3] = mw >> 24;
    }
    else {
      // no segment reaches this slot: every pixel of a row has the row's carried-in coverage
      const uint32_t rule = ((cmeta >> 16) & 2u) ? 0x1FFu : 0xFFFFFFFFu;
      m[0] = px::calc_mask((256u << 9) + mw, rule, alpha);
      m[1] = m[2] = m[3] = m[0];
    }
  }
  else {
    const DevCmd& cmd = f.cmds[ci];
    if (ckind == kFillBoxA) {
      bool in_y = y >= cmd.box[1] && y < cmd.box[3];
#pragma unroll
      for (int k = 0; k < 4; k++) m[k] = (in_y && xp + k >= cmd.box[0] && xp + k < cmd.box[2]) ? alpha : 0u;
    }
    else if (ckind == kFillMaskA) {
      // FillMask_Base's vmask spans (fillgeneric_p.h:67-162, compopgeneric_p.h:165-183): the mask
      // byte, times the fill alpha below 255 (udiv255)
      const bool in_y = y >= cmd.box[1] && y < cmd.box[3];
      const uint8_t* row = reinterpret_cast<const uint8_t*>(f.images) +
                           ((uint64_t(cmd.xform) << 32) | cmd.geom_first) + int64_t(y - cmd.box[1]) * cmd.geom_count;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        uint32_t v = 0u;
        if (in_y && xp + k >= cmd.box[0] && xp + k < cmd.box[2]) {
          v = __ldg(row + (xp + k - cmd.box[0]));
          if (alpha < 255u) v = ((v * alpha + 0x80u) * 0x101u) >> 16;
        }
        m[k] = v;
      }
    }
    else {
#pragma unroll
      for (int k = 0; k < 4; k++) m[k] = px::box_u_mask(cmd.box, alpha, xp + k, y);
    }
  }
}

// Slot of an analytic command in strip row `strip_row`, tile column tx, from its list records
// (first slot, tx0 | columns << 16, rows y0 | y1 << 16), and its mask index + 1 (0: no segment
// reaches it).
__device__ __forceinline__ uint32_t strip_slot(const FrameView& f, uint32_t slot0, uint32_t tcols, uint32_t yr,
                                               uint32_t strip_row, int tx, uint32_t& nseg) {
  const uint32_t slot = slot0 + (strip_row - ((yr & 0xFFFFu) >> kStripShift)) * (tcols >> 16) + (uint32_t(tx) - (tcols & 0xFFFFu));
  nseg = f.slot_mask[slot];
  return slot;
}

// Occlusion, per strip: a SrcCopy command whose mask is 255 on every pixel of the strip writes its
// source there whatever is below (CompOp_SrcCopy with m = 255 gives the source exactly), so the
// composite pass can start at the last such command of the strip's list. Looked for from the end
// of the list, in rows with SrcCopy commands besides a first clear; 0 elsewhere.
__global__ void __launch_bounds__(kFineThreads) cull_kernel(FrameView f) {
  const int lane = threadIdx.x & 31;
  const int prow = lane >> 3;
  const int pcol = (lane & 7) * 4;
  if (frame_skipped(f)) return;
  const uint32_t num_units = f.counts[kCntTiles] * kStripsPerTile;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t unit = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); unit < num_units; unit += warps) {
    const uint32_t tile = f.tile_order[unit / kStripsPerTile];
    const int strip = int(unit % kStripsPerTile);
    const DevCanvas cv = f.canvases[f.tile_canvas[tile]];
    const uint32_t local = tile - cv.tile_base;
    const int tx = int(local % uint32_t(cv.tiles_x)), ty = int(local / uint32_t(cv.tiles_x));
    const int x_base = tx * kTileW;
    const int row0 = ty * kTileH + strip * kStripRows;
    const uint32_t row_id = (cv.row_base << (kTileShift - f.list_shift)) + (uint32_t(row0) >> f.list_shift);
    if (row0 >= cv.h || f.row_copies[row_id] < 2) {
      if (lane == 0) f.strip_start[unit] = 0;
      continue;
    }
    const uint32_t strip_row = uint32_t(row0) >> kStripShift;
    const int row1 = min(row0 + kStripRows, cv.h) - 1;
    const int y = row0 + prow, xp = x_base + pcol;
    const bool row_ok = y < cv.h;
    const uint32_t list_first = f.row_offsets[row_id];
    const uint32_t list_count = f.row_counts[row_id];
    const uint32_t strip_y = uint32_t(row0) | (uint32_t(row1) << 16);
    const uint32_t strip_x = uint32_t(x_base) | (uint32_t(min(x_base + kTileW, cv.w) - 1) << 16);
    uint32_t start = 0;
    for (int cb = int((list_count - 1u) & ~31u); cb >= 0; cb -= 32) {
      uint4 ra = make_uint4(0u, 0u, 0u, 0u), rb = ra;
      bool cand = false;
      if (uint32_t(cb + lane) < list_count) {
        // the box first; the records only for commands that cover the whole strip
        const uint2 bb = f.row_box[list_first + uint32_t(cb + lane)];
        cand = (bb.x & 0xFFFFu) <= (strip_x & 0xFFFFu) && (bb.x >> 16) >= (strip_x >> 16) &&
               (bb.y & 0xFFFFu) <= (strip_y & 0xFFFFu) && (bb.y >> 16) >= (strip_y >> 16);
        if (cand) {
          const uint4* rec = f.row_recs + 2u * (list_first + uint32_t(cb + lane));
          ra = rec[0];
          rb = rec[1];
          cand = ((ra.w >> 2) & 1u) && (ra.w >> 4) == 255u;
        }
      }
      uint32_t todo = __ballot_sync(0xFFFFFFFFu, cand);
      bool found = false;
      while (todo) {
        const int bit = 31 - __clz(todo);
        todo &= ~(1u << bit);
        const uint32_t ci = __shfl_sync(0xFFFFFFFFu, ra.x, bit);
        const uint32_t rmeta = __shfl_sync(0xFFFFFFFFu, ra.w, bit);
        const uint32_t ckind = rmeta & 3u;
        const uint32_t cmeta = (((rmeta >> 2) & 3u) << 16) | (rmeta >> 4);
        uint32_t cnseg = 0, mw = 0;
        if (ckind == kFillAnalytic) {
          const uint32_t slot = strip_slot(f, __shfl_sync(0xFFFFFFFFu, rb.x, bit), __shfl_sync(0xFFFFFFFFu, rb.y, bit),
                                           __shfl_sync(0xFFFFFFFFu, ra.z, bit), strip_row, tx, cnseg);
          mw = cnseg ? reinterpret_cast<const uint32_t*>(f.masks + size_t(cnseg - 1u) * kSlotPixels)[lane]
                     : f.backdrop[size_t(slot) * kStripRows + prow];
        }
        uint32_t m[4];
        strip_masks(f, ckind, ci, cmeta, cnseg, mw, xp, y, m);
        bool full = true;
#pragma unroll
        for (int k = 0; k < 4; k++) full &= !(row_ok && xp + k < cv.w) || m[k] == 255u;
        if (__all_sync(0xFFFFFFFFu, full)) { start = uint32_t(cb + bit); found = true; break; }
      }
      if (found) break;
    }
    if (lane == 0) f.strip_start[unit] = start;
  }
}

// 5 resident blocks per SM (48 registers, a few spilled): the composite waits on dependent loads,
// and the extra warps hide more of them than the spills cost (curves frame 2.98 -> 2.95 ms; 6
// blocks, 40 registers, measured the same as 5).
__global__ void __launch_bounds__(kFineThreads, 5) fine_kernel(FrameView f) {
  const int lane = threadIdx.x & 31;
  const int prow = lane >> 3;            // row within the strip
  const int pcol = (lane & 7) * 4;       // first of this lane's 4 columns
  uint32_t ops = 0, pat_ops = 0;         // composited pixels of this lane (all strips)
  if (frame_skipped(f)) return;
  const uint32_t num_units = f.counts[kCntTiles] * kStripsPerTile;

  for (;;) {
    uint32_t unit = 0;
    if (lane == 0) unit = atomicAdd(f.work_counter, 1u);
    unit = __shfl_sync(0xFFFFFFFFu, unit, 0);
    if (unit >= num_units) break;
    uint32_t tile = f.tile_order[unit / kStripsPerTile];
    int strip = int(unit % kStripsPerTile);
    const DevCanvas cv = f.canvases[f.tile_canvas[tile]];
    uint32_t local = tile - cv.tile_base;
    int tx = int(local % uint32_t(cv.tiles_x)), ty = int(local / uint32_t(cv.tiles_x));
    int x_base = tx * kTileW;
    int row0 = ty * kTileH + strip * kStripRows;
    if (row0 >= cv.h) continue;
    const uint32_t strip_row = uint32_t(row0) >> kStripShift;
    int row1 = min(row0 + kStripRows, cv.h) - 1;     // last row of the strip inside the canvas
    int y = row0 + prow, xp = x_base + pcol;
    bool row_ok = y < cv.h;
    uint32_t* dst = cv.pixels + int64_t(y) * cv.stride + xp;
    // an A8 canvas: one byte per pixel, composited as the alpha byte of a 32-bit pixel (the
    // reference's P8_Alpha operators are its P32 operators' alpha lane); rows start at 16-byte
    // boundaries and xp is a multiple of 4, so 4 pixels are one aligned word
    uint8_t* dst8 = reinterpret_cast<uint8_t*>(cv.pixels) + int64_t(y) * cv.stride + xp;

    uint32_t pix[4];
    bool full = row_ok && (xp + 3 < cv.w);
    if (cv.a8) {
      if (full) {
        const uint32_t v = *reinterpret_cast<const uint32_t*>(dst8);
#pragma unroll
        for (int k = 0; k < 4; k++) pix[k] = ((v >> (8 * k)) & 0xFFu) << 24;
      }
      else {
#pragma unroll
        for (int k = 0; k < 4; k++) pix[k] = (row_ok && xp + k < cv.w) ? uint32_t(dst8[k]) << 24 : 0u;
      }
    }
    else if (full) {
      uint4 v = *reinterpret_cast<const uint4*>(dst);
      pix[0] = v.x; pix[1] = v.y; pix[2] = v.z; pix[3] = v.w;
    }
    else {
#pragma unroll
      for (int k = 0; k < 4; k++) pix[k] = (row_ok && xp + k < cv.w) ? dst[k] : 0u;
    }

    const uint32_t row_id = (cv.row_base << (kTileShift - f.list_shift)) + (uint32_t(row0) >> f.list_shift);
    uint32_t list_first = f.row_offsets[row_id];
    uint32_t list_count = f.row_counts[row_id];
    const uint32_t strip_y = uint32_t(row0) | (uint32_t(row1) << 16);
    const uint32_t strip_x = uint32_t(x_base) | (uint32_t(min(x_base + kTileW, cv.w) - 1) << 16);

    const uint32_t start = f.strip_start[unit];      // cull_kernel

    for (uint32_t base = start & ~31u; base < list_count; base += 32) {
      // commands of this chunk whose pixel bbox overlaps the strip, in painter's order: one pair
      // of list records per lane holds everything the tests and the slot lookup need
      uint4 ra = make_uint4(0u, 0u, 0u, 0u), rb = ra;
      bool hit = false;
      if (base + lane < list_count && base + lane >= start) {
        // 8 bytes per entry to find the commands over the strip; their records only for those
        const uint2 bb = f.row_box[list_first + base + lane];
        hit = (bb.x & 0xFFFFu) <= (strip_x >> 16) && (bb.x >> 16) >= (strip_x & 0xFFFFu) &&
              (bb.y & 0xFFFFu) <= (strip_y >> 16) && (bb.y >> 16) >= (strip_y & 0xFFFFu);
        if (hit) {
          const uint4* rec = f.row_recs + 2u * (list_first + base + lane);
          ra = rec[0];
          rb = rec[1];
        }
      }
      const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, hit);
      if (!ballot) continue;
      // Each hit lane looks up its command's slot in parallel (one command per lane), so the
      // painter's-order loop below only waits on the mask words.
      uint32_t kind = 0, slot = 0xFFFFFFFFu, nseg = 0, meta = 0;   // meta: flags << 16 | alpha
      if (hit) {
        kind = ra.w & 3u;
        meta = (((ra.w >> 2) & 3u) << 16) | (ra.w >> 4);
        if (kind == kFillAnalytic) slot = strip_slot(f, rb.x, rb.y, ra.z, strip_row, tx, nseg);
      }
      uint32_t todo = ballot;
      // the first command's mask word, then each next one's while the current one composites
      int bit = __ffs(todo) - 1;
      uint32_t next_mw = 0;
      {
        const uint32_t s0 = __shfl_sync(0xFFFFFFFFu, slot, bit), n0 = __shfl_sync(0xFFFFFFFFu, nseg, bit);
        if (s0 != 0xFFFFFFFFu)
          next_mw = n0 ? reinterpret_cast<const uint32_t*>(f.masks + size_t(n0 - 1u) * kSlotPixels)[lane]
                       : f.backdrop[size_t(s0) * kStripRows + prow];
      }
      while (todo) {
        todo &= todo - 1;
        const uint32_t ci = __shfl_sync(0xFFFFFFFFu, ra.x, bit);
        const uint32_t ckind = __shfl_sync(0xFFFFFFFFu, kind, bit);
        const uint32_t cmeta = __shfl_sync(0xFFFFFFFFu, meta, bit);
        const uint32_t cnseg = __shfl_sync(0xFFFFFFFFu, nseg, bit);
        const uint32_t cstyle = __shfl_sync(0xFFFFFFFFu, rb.z, bit);
        const uint32_t crs = __shfl_sync(0xFFFFFFFFu, rb.w, bit);
        const uint32_t cy0 = __shfl_sync(0xFFFFFFFFu, ra.z, bit) & 0xFFFFu;
        const uint32_t mw = next_mw;
        if (todo) {
          const int nb = __ffs(todo) - 1;
          const uint32_t s1 = __shfl_sync(0xFFFFFFFFu, slot, nb), n1 = __shfl_sync(0xFFFFFFFFu, nseg, nb);
          if (s1 != 0xFFFFFFFFu)
            next_mw = n1 ? reinterpret_cast<const uint32_t*>(f.masks + size_t(n1 - 1u) * kSlotPixels)[lane]
                         : f.backdrop[size_t(s1) * kStripRows + prow];
          bit = nb;
        }
        uint32_t m[4];
        strip_masks(f, ckind, ci, cmeta, cnseg, mw, xp, y, m);

        if (row_ok && (m[0] | m[1] | m[2] | m[3]) && (cstyle & kRecSolid)) {
          const bool src_copy = (cmeta >> 16) & 1u;
#pragma unroll
          for (int k = 0; k < 4; k++) {
            if (m[k] && xp + k < cv.w) {
              pix[k] = px::composite(pix[k], crs, m[k], src_copy);
              ops++;
            }
          }
        }
        else if (row_ok && (m[0] | m[1] | m[2] | m[3])) {
          const DevCmd& cmd = f.cmds[ci];
          const DevStyle& st = f.styles[cstyle];
          const bool src_copy = (cmeta >> 16) & 1u;
          px::RowState rs;
          if (px::has_row_table(st.fetch)) {
            const float4 t4 = f.row_states[crs + uint32_t(y - int(cy0))];
            rs.f0 = t4.x; rs.f1 = t4.y; rs.f2 = t4.z;
          }
          else {
            // the reference initializes its fetcher at the start of each band of an analytic fill
            int fetch_y0 = ckind == kFillAnalytic ? max(cmd.box[1], (y / cv.band_height) * cv.band_height) : cmd.fetch_y0;
            rs = px::row_state(st, y, fetch_y0);
          }
          uint32_t n = 0;
          if (px::is_gradient(st.fetch)) {
            // the 4 pixels' LUT indices first, so their 4 table loads are in flight together
            const uint32_t* lut = f.luts + st.lut_offset;
            uint32_t sv[4];
            if (!st.dither) {
#pragma unroll
              for (int k = 0; k < 4; k++) {
                const bool on = m[k] && xp + k < cv.w;
                sv[k] = on ? __ldg(lut + px::gradient_index(st, rs, xp + k)) : 0u;
              }
            }
            else {
              // 64-bit entries (lut_offset is even) + the ordered-dither threshold of each pixel
              uint2 e[4];
#pragma unroll
              for (int k = 0; k < 4; k++) {
                const bool on = m[k] && xp + k < cv.w;
                e[k] = on ? __ldg(reinterpret_cast<const uint2*>(lut) + px::gradient_index(st, rs, xp + k))
                          : make_uint2(0u, 0u);
              }
#pragma unroll
              for (int k = 0; k < 4; k++) sv[k] = px::dither_pixel(e[k], px::dither_threshold(xp + k, y));
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
              if (m[k] && xp + k < cv.w) {
                pix[k] = px::composite(pix[k], sv[k], m[k], src_copy);
                n++;
              }
            }
          }
          else {
            // one copy of the fetch + composite code: the 4 pixels rotate through slot 0
#pragma unroll 1
            for (int k = 0; k < 4; k++) {
              if (m[0] && xp + k < cv.w) {
                uint32_t sv = px::fetch(st, rs, xp + k, f.luts, f.images) | st.src_or;
                pix[0] = px::composite(pix[0], sv, m[0], src_copy);
                n++;
              }
              uint32_t tp = pix[0]; pix[0] = pix[1]; pix[1] = pix[2]; pix[2] = pix[3]; pix[3] = tp;
              uint32_t tm = m[0]; m[0] = m[1]; m[1] = m[2]; m[2] = m[3]; m[3] = tm;
            }
          }
          ops += n;
          pat_ops += st.fetch >= kFetchPatAlignedPad ? n : 0u;
        }
      }
    }

    if (cv.a8) {
      if (full) {
        *reinterpret_cast<uint32_t*>(dst8) = (pix[0] >> 24) | ((pix[1] >> 24) << 8) | ((pix[2] >> 24) << 16) |
                                             (pix[3] & 0xFF000000u);
      }
      else {
#pragma unroll
        for (int k = 0; k < 4; k++) if (row_ok && xp + k < cv.w) dst8[k] = uint8_t(pix[k] >> 24);
      }
    }
    else if (full) {
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

// Gradient row states: one thread per (command, row) of every radial/conic command's bbox.
__global__ void row_state_kernel(FrameView f) {
  if (frame_skipped(f)) return;
  const uint32_t total = min(f.totals[4], f.num_row_states);
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  uint32_t lo = 0, hi = f.counts[kCntCmds] - 1;       // last command whose first row state is <= t
  while (lo < hi) { uint32_t mid = (lo + hi + 1) >> 1; if (f.rs_base[mid] <= t) lo = mid; else hi = mid - 1; }
  const uint32_t c = lo;
  const DevCmd& cmd = f.cmds[c];
  const DevCanvas& cv = f.canvases[cmd.canvas];
  const int y = int(f.cmd_yr[c] & 0xFFFFu) + int(t - f.rs_base[c]);
  // the row the reference initialized its fetcher at (start of the band for analytic fills)
  int fetch_y0 = cmd.kind == kFillAnalytic ? max(cmd.box[1], (y / cv.band_height) * cv.band_height) : cmd.fetch_y0;
  const DevStyle& st = f.styles[cmd.style];
  if (st.fetch == kFetchConic) return;            // conic_rows_kernel
  px::RowState rs = px::row_state(st, y, fetch_y0);
  f.row_states[t] = make_float4(rs.f0, rs.f1, rs.f2, 0.0f);
}

// Conic row values, one thread per run of rows sharing a fetcher start: the reference steps the
// fetcher's FP64 position row by row from there, so a run is one sequential chain (a thread per
// row would repeat the chain's prefix in every row; the FP64 pipe is the scarce one).
__global__ void conic_rows_kernel(FrameView f) {
  if (frame_skipped(f)) return;
  const uint32_t total = min(f.totals[6], f.num_row_runs);
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  uint32_t lo = 0, hi = f.counts[kCntCmds] - 1;       // last command whose first run is <= t
  while (lo < hi) { uint32_t mid = (lo + hi + 1) >> 1; if (f.rb_base[mid] <= t) lo = mid; else hi = mid - 1; }
  const uint32_t c = lo;
  const DevCmd& cmd = f.cmds[c];
  const DevCanvas& cv = f.canvases[cmd.canvas];
  const DevStyle& st = f.styles[cmd.style];
  const int y0 = int(f.cmd_yr[c] & 0xFFFFu), y1 = int(f.cmd_yr[c] >> 16);
  int ya = y0, yb = y1, fs = cmd.fetch_y0;
  if (cmd.kind == kFillAnalytic) {
    const int band = y0 / cv.band_height + int(t - f.rb_base[c]);
    ya = max(y0, band * cv.band_height);
    yb = min(y1, band * cv.band_height + cv.band_height - 1);
    fs = max(cmd.box[1], band * cv.band_height);
  }
  double tx = st.con_tx + st.con_yx * double(fs);
  double ty = st.con_ty + st.con_yy * double(fs);
  int cur = fs;
  float4* out = f.row_states + f.rs_base[c] + uint32_t(ya - y0);
  for (int y = ya; y <= yb; y++) {
    for (; cur < y; cur++) { tx += st.con_yx; ty += st.con_yy; }
    const float ay = float(ty);
    const uint32_t byb = uint32_t(int32_t(__float_as_uint(ay)) >> 31) & __float_as_uint(st.con_n1);
    *out++ = make_float4(float(tx), fabsf(ay), __uint_as_float(byb), 0.0f);
  }
}

// Tile/row bookkeeping: canvas of every global tile and tile row, identity processing order.
__global__ void tile_setup_kernel(FrameView f, uint32_t* row_canvas) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t num_canvases = f.counts[kCntCanvases];
  // binary search the canvas owning tile i / row i
  if (i < f.counts[kCntTiles]) {
    uint32_t lo = 0, hi = num_canvases - 1;
    while (lo < hi) { uint32_t mid = (lo + hi + 1) >> 1; if (f.canvases[mid].tile_base <= i) lo = mid; else hi = mid - 1; }
    f.tile_canvas[i] = lo;
    f.tile_order[i] = i;
  }
  const uint32_t log2 = kTileShift - f.list_shift;
  if (i < (f.counts[kCntRows] << log2)) {
    uint32_t lo = 0, hi = num_canvases - 1;
    while (lo < hi) { uint32_t mid = (lo + hi + 1) >> 1; if ((f.canvases[mid].row_base << log2) <= i) lo = mid; else hi = mid - 1; }
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
  lut_kernel<<<cdiv(f.num_lut_jobs, kLutWarps), 32 * kLutWarps, 0, st>>>(f.lut_jobs, f.stops, f.luts, f.counts);
  return 1;
}

// Device properties the launch shapes depend on, queried once (thread-safe static
// initialization: the runtime's two pipeline lanes launch from two threads).
static int device_sms() {
  static const int v = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  return v;
}
template<typename K>
static int max_blocks_per_sm(K kernel, int threads, size_t dyn_smem = 0) {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, dyn_smem);
  return n > 0 ? n : 1;
}

int launch_edges(const FrameView& f, const LaunchConfig& cfg, cudaStream_t st) {
  if (!f.num_cmds) return 0;
  const int sms = device_sms();
  static const int max_per_sm = max_blocks_per_sm(edge_pieces_kernel<3, kPiecesClipped>, kCurveThreads);
  const int per_sm = cfg.cubic_blocks_per_sm > 0 && cfg.cubic_blocks_per_sm < max_per_sm ? cfg.cubic_blocks_per_sm : max_per_sm;
  const uint32_t eb = cfg.edge_block == 64 || cfg.edge_block == 256 ? uint32_t(cfg.edge_block) : 128u;
  classify_kernel<<<cdiv(f.num_cmds, 128), 128, 0, st>>>(f);
  edge_items_kernel<<<cdiv(f.item_capacity ? f.item_capacity : 1, eb), eb, 0, st>>>(f);
  const uint32_t cubic_grid = uint32_t(sms * per_sm);
  const uint32_t split_grid = cdiv(f.item_capacity ? f.item_capacity : 1, 128);
  curve_split_kernel<3><<<split_grid, 128, 0, st>>>(f);
  curve_split_kernel<2><<<split_grid, 128, 0, st>>>(f);
  const uint32_t pgrid = cdiv(f.piece_capacity ? f.piece_capacity : 1, kCurveThreads);
  const uint32_t pieces_grid = pgrid < cubic_grid ? pgrid : cubic_grid;
  const uint32_t tree_grid = min(pgrid, uint32_t(sms * kTreeBlocksPerSM));
  edge_tree_kernel<<<tree_grid, kCurveThreads, 0, st>>>(f);
  edge_pieces_kernel<3, kPiecesClipped><<<pieces_grid, kCurveThreads, 0, st>>>(f);
  edge_pieces_kernel<2, kPiecesAll><<<pieces_grid, kCurveThreads, 0, st>>>(f);
  return 7;
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
  const uint32_t list_rows = f.num_rows << (kTileShift - f.list_shift);
  uint32_t n = f.num_tiles > list_rows ? f.num_tiles : list_rows;
  if (n) { tile_setup_kernel<<<cdiv(n, 256), 256, 0, st>>>(f, row_canvas); k++; }
  if (list_rows) { row_fill_kernel<<<list_rows, 512, 0, st>>>(f, row_canvas); k++; }
  return k;
}

int fine_grid_size(int blocks_per_sm) {
  const int sms = device_sms();
  static const int max_per_sm = max_blocks_per_sm(fine_kernel, kFineThreads);
  return sms * (blocks_per_sm > 0 && blocks_per_sm < max_per_sm ? blocks_per_sm : max_per_sm);
}

// Coverage pass: compact the slots with segments, lay out their work items slot by slot,
// rasterize and sweep. Called after the binning count pass and the backdrop prefix.
int launch_coverage(const FrameView& f, const LaunchConfig& cfg, uint32_t* scan_tmp, cudaStream_t st) {
  if (!f.num_cmdrows) return 0;
  const int sms = device_sms();
  int k = 0;
  slot_flags_kernel<<<cdiv(f.num_cmdrows, 256), 256, 0, st>>>(f); k++;
  k += exclusive_scan(f.cmdrow_offsets, f.cmdrow_offsets, f.num_cmdrows, scan_tmp, st);
  slot_compact_kernel<<<cdiv(f.num_cmdrows, 256), 256, 0, st>>>(f); k++;
  k += exclusive_scan(f.cmdrow_counts, f.slot_first, f.num_cmdrows + 1, scan_tmp, st);
  k += launch_seg_bin(f, 1, st);
  const int per_sm = cfg.cover_blocks_per_sm > 0 ? cfg.cover_blocks_per_sm : 16;
  // by frame: scenes of long edges (many strip rows per segment) have few work items per slot,
  // where smaller groups keep more of them in flight per SM
  const int slots = cfg.cover_slots ? cfg.cover_slots : (f.num_seglist > 16u * f.num_segs ? 32 : 64);
  if (slots == 16) coverage_kernel<16><<<sms * per_sm, 64, 0, st>>>(f);
  else if (slots == 64) coverage_kernel<64><<<sms * per_sm, 256, 0, st>>>(f);
  else coverage_kernel<32><<<sms * per_sm, 128, 0, st>>>(f);
  return k + 1;
}

int launch_row_states(const FrameView& f, cudaStream_t st) {
  if (!f.num_row_states) return 0;
  row_state_kernel<<<cdiv(f.num_row_states, 128), 128, 0, st>>>(f);
  if (!f.num_row_runs) return 1;
  conic_rows_kernel<<<cdiv(f.num_row_runs, 64), 64, 0, st>>>(f);
  return 2;
}

// work_counter must be zero on entry.
int launch_fine(const FrameView& f, const LaunchConfig& cfg, cudaStream_t st) {
  if (!f.num_tiles) return 0;
  int grid = fine_grid_size(cfg.fine_blocks_per_sm);
  uint32_t max_blocks = (f.num_tiles * kStripsPerTile + kFineWarps - 1) / kFineWarps;
  if (uint32_t(grid) > max_blocks) grid = int(max_blocks);
  if (cfg.no_occlusion_cull) {
    cudaMemsetAsync(f.strip_start, 0, sizeof(uint32_t) * size_t(f.num_tiles) * kStripsPerTile, st);
  }
  else {
    cull_kernel<<<grid, kFineThreads, 0, st>>>(f);
  }
  fine_kernel<<<grid, kFineThreads, 0, st>>>(f);
  return cfg.no_occlusion_cull ? 1 : 2;
}

}  // namespace blgpu
