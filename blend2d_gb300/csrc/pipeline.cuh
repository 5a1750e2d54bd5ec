// pipeline.cuh - per-pixel style fetch and composition for the fine kernel.
//
// The reference walks fetchers along spans (blend2d/pipeline/reference/fetchgeneric_p.h); every
// fetcher's state at pixel (x, y) is a closed-form function of (x, y) - 32.32 fixed-point sums
// wrap mod 2^64, float x positions are exact integers, pattern indices are normalized into a
// unique representative - so each pixel is evaluated directly from (x, y) here. The one stateful
// exception is the conic gradient's row origin, which the reference accumulates in FP64 from the
// row at which its fill call initialized the fetcher; RowState reproduces that accumulation.
//
// Pixel arithmetic follows the reference's 64-bit unpacked form (pixelgeneric_p.h:110-220):
// lanes [A:48 G:32 R:16 B:0], div255 = ((x + 128) + ((x + 128) >> 8)) >> 8 per 16-bit lane.
#pragma once

#include "blgpu_internal.h"
#include "divmagic.h"

namespace blgpu {
namespace px {

constexpr uint64_t kLaneFF = 0x00FF00FF00FF00FFull;

__device__ __forceinline__ uint64_t unpack(uint32_t p) { return uint64_t(p & 0x00FF00FFu) | (uint64_t(p & 0xFF00FF00u) << 24); }
__device__ __forceinline__ uint32_t pack(uint64_t u) { return uint32_t(((u >> 24) | u) & 0xFFFFFFFFu); }
__device__ __forceinline__ uint64_t div255(uint64_t u) {
  u += 0x0080008000800080ull;
  return ((u + ((u >> 8) & kLaneFF)) >> 8) & kLaneFF;
}
__device__ __forceinline__ uint64_t div256(uint64_t u) { return (u >> 8) & kLaneFF; }

// The same per-channel arithmetic on two 16-bit lanes of a 32-bit word (every product and sum
// stays below 2^16, so lanes never carry into each other).
__device__ __forceinline__ uint32_t div255_2x16(uint32_t x) {
  x += 0x00800080u;
  return ((x + ((x >> 8) & 0x00FF00FFu)) >> 8) & 0x00FF00FFu;
}

// CompOp_SrcOver_Op / CompOp_SrcCopy_Op (compopgeneric_p.h:24-63) with a mask m in [0, 255].
__device__ __forceinline__ uint32_t composite(uint32_t d, uint32_t s, uint32_t m, bool src_copy) {
  const uint32_t kM = 0x00FF00FFu;
  if (src_copy) {
    uint32_t im = m ^ 0xFFu;
    uint32_t rb = div255_2x16((d & kM) * im + (s & kM) * m);
    uint32_t ag = div255_2x16(((d >> 8) & kM) * im + ((s >> 8) & kM) * m);
    return rb | (ag << 8);
  }
  uint32_t sm = div255_2x16((s & kM) * m) | (div255_2x16(((s >> 8) & kM) * m) << 8);
  uint32_t ia = (sm >> 24) ^ 0xFFu;
  return sm + (div255_2x16((d & kM) * ia) | (div255_2x16(((d >> 8) & kM) * ia) << 8));
}

// x86 cvttss2si / cvtss2si semantics (INT_MIN for NaN and out-of-range values).
__device__ __forceinline__ int trunc_f(float v) {
  if (!(v >= -2147483648.0f && v < 2147483648.0f)) return INT32_MIN;
  return __float2int_rz(v);
}
__device__ __forceinline__ int nearby_f(float v) {
  if (!(v >= -2147483648.0f && v < 2147483648.0f)) return INT32_MIN;
  return __float2int_rn(v);
}

__device__ __forceinline__ uint32_t grad_index(uint32_t idx, bool pad, uint32_t maxi, uint32_t rori) {
  if (pad) {
    int32_t i = int32_t(idx);
    return uint32_t(i < 0 ? 0 : (i > int32_t(maxi) ? int32_t(maxi) : i));
  }
  uint32_t a = idx & maxi, b = a ^ rori;
  return b < a ? b : a;
}

// Per (command, row) state computed once per thread row.
struct RowState {
  uint64_t a64, b64;     // linear: py | affine: tx, ty of the row
  float f0, f1, f2;      // radial: b, d, dd | conic: tx, |ay|, by
  int32_t r0, r1;        // pattern: source rows (r1 = next row for fx/fy)
};

// Vertical pattern mapping (FetchPatternVertAAExtendCtxAny, fetchgeneric_p.h:78-155).
__device__ __forceinline__ int pat_row(const DevStyle& st, int y) {
  int yy = y + st.pat_ty;
  int h = st.src_h;
  if (st.pat_ry == 0) return yy < 0 ? 0 : (yy > h - 1 ? h - 1 : yy);
  uint32_t m = uint32_t(yy) % uint32_t(st.pat_ry);
  if (int(m) >= h) return 2 * h - 1 - int(m);
  return int(m);
}

// Horizontal pattern mapping (FetchPatternHorzExtendCtx{Pad,Repeat,RoR}).
__device__ __forceinline__ int pat_col(const DevStyle& st, int x, uint32_t kind) {
  int w = st.src_w;
  if (kind == 0) {
    long long xx = (long long)x + st.pat_tx;
    return int(xx < 0 ? 0 : (xx > w - 1 ? w - 1 : xx));
  }
  if (kind == 1) return int(uint32_t(x + st.pat_tx) % uint32_t(w));
  int v = int(uint32_t(x + st.pat_tx) % uint32_t(st.pat_rx));
  if (v >= w) v -= st.pat_rx;
  return v ^ (v >> 31);
}

__device__ __forceinline__ void af_normalize(const DevStyle& s, uint64_t vx, uint64_t vy, uint64_t& ox, uint64_t& oy) {
  uint32_t x = uint32_t(smod_magic(int32_t(vx >> 32), s.af_tw, DivMagic{s.af_tw_m, s.af_tw_s}));
  uint32_t y = uint32_t(smod_magic(int32_t(vy >> 32), s.af_th, DivMagic{s.af_th_m, s.af_th_s}));
  if (int32_t(x) < 0) x += uint32_t(s.af_rx);
  if (int32_t(y) < 0) y += uint32_t(s.af_ry);
  if (int32_t(x) > s.af_ox) x -= uint32_t(s.af_rx);
  if (int32_t(y) > s.af_oy) y -= uint32_t(s.af_ry);
  ox = (uint64_t(x) << 32) | (vx & 0xFFFFFFFFu);
  oy = (uint64_t(y) << 32) | (vy & 0xFFFFFFFFu);
}

__device__ __forceinline__ void af_index(const DevStyle& s, uint64_t px, uint64_t py, int off, uint32_t& ix, uint32_t& iy) {
  int32_t x = int32_t(px >> 32) + off;
  int32_t y = int32_t(py >> 32) + off;
  x = x < s.af_minx ? s.af_minx : x;
  y = y < s.af_miny ? s.af_miny : y;
  if (x > s.af_maxx) x = s.af_corx;
  if (y > s.af_maxy) y = s.af_cory;
  x = x ^ (x >> 31);
  y = y ^ (y >> 31);
  ix = uint32_t(x);
  iy = uint32_t(y);
}

// Row state. `fetch_y0` is the row where the reference initialized its fetcher for this row
// (only the conic gradient depends on it).
// Radial and conic fetchers carry FP64 row state; it is tabulated per (command, row) once per
// frame instead of being recomputed by every lane that composites the row.
__device__ __forceinline__ bool has_row_table(uint32_t fetch) {
  return fetch == kFetchRadialPad || fetch == kFetchRadialRoR || fetch == kFetchConic;
}

__device__ RowState row_state(const DevStyle& st, int y, int fetch_y0) {
  RowState r{};
  switch (st.fetch) {
    case kFetchLinearPad: case kFetchLinearRoR:
      r.a64 = st.lin_pt0 + uint64_t(uint32_t(y)) * st.lin_dy;
      break;
    case kFetchRadialPad: case kFetchRadialRoR: {
      double ry = double(y);
      double ptx = st.rad_yx * ry + st.rad_tx;
      double pty = st.rad_yy * ry + st.rad_ty;
      double b = ry * st.rad_by + st.rad_b0;
      double sq_dist = ptx * ptx + pty * pty;
      r.f0 = float(b * st.rad_inv2a);
      r.f1 = float((st.rad_amul4 * (sq_dist - st.rad_sq_fr) + b * b) * st.rad_sq_inv2a);
      r.f2 = float((ry * st.rad_ddy + st.rad_dd0) * st.rad_sq_inv2a);
      break;
    }
    case kFetchConic: {
      double tx = st.con_tx + st.con_yx * double(fetch_y0);
      double ty = st.con_ty + st.con_yy * double(fetch_y0);
      for (int k = fetch_y0; k < y; k++) { tx += st.con_yx; ty += st.con_yy; }
      float ay = float(ty);
      uint32_t sb = __float_as_uint(ay);
      uint32_t byb = uint32_t(int32_t(sb) >> 31) & __float_as_uint(st.con_n1);
      r.f0 = float(tx);
      r.f1 = fabsf(ay);
      r.f2 = __uint_as_float(byb);
      break;
    }
    case kFetchPatAlignedPad: case kFetchPatAlignedRepeat: case kFetchPatAlignedRoR:
      r.r0 = pat_row(st, y);
      break;
    case kFetchPatFxFyPad: case kFetchPatFxFyRoR:
      r.r0 = pat_row(st, y);
      r.r1 = pat_row(st, y + 1);
      break;
    case kFetchPatAffineNN: case kFetchPatAffineBI:
      r.a64 = st.af_tx + st.af_yx * uint64_t(uint32_t(y));
      r.b64 = st.af_ty + st.af_yy * uint64_t(uint32_t(y));
      break;
    default:
      break;
  }
  return r;
}

__device__ __forceinline__ bool is_gradient(uint32_t fetch) { return fetch >= kFetchLinearPad && fetch <= kFetchConic; }

// Threshold of the 16x16 ordered-dither matrix (bayer_matrix_16x16, tables_p.h:449-473) at canvas
// pixel (x, y), from the matrix's recursive construction instead of a table: the index interleaves
// the bits of row and column, lowest bits most significant, each pair weighted by the 2x2 pattern
// {{0, 3}, {2, 1}} (= 2 * (r ^ c) + c); the entry scales the index from [0, 256) to [0, 255],
// rounding half down.
__device__ __forceinline__ uint32_t dither_threshold(int x, int y) {
  uint32_t c = __brev(uint32_t(x) & 15u) >> 28;               // bit k of x -> bit 3 - k
  uint32_t v = __brev((uint32_t(x) ^ uint32_t(y)) & 15u) >> 28;
  c = (c | (c << 2)) & 0x33u; c = (c | (c << 1)) & 0x55u;      // bit j -> bit 2j
  v = (v | (v << 2)) & 0x33u; v = (v | (v << 1)) & 0x55u;
  return (((v << 1) | c) * 255u + 127u) >> 8;
}

// FetchGradientBase<DITHER>::fetch_pixel (fetchgeneric_p.h:922-933): a 64-bit premultiplied LUT
// entry (lo = g << 16 | b, hi = a << 16 | r) plus the threshold, down to 8 bits, each colour
// channel clamped to alpha.
__device__ __forceinline__ uint32_t dither_pixel(uint2 v, uint32_t dd) {
  const uint32_t a = v.y >> 24;
  const uint32_t r = min(((v.y & 0xFFFFu) + dd) >> 8, a);
  const uint32_t g = min(((v.x >> 16) + dd) >> 8, a);
  const uint32_t b = min(((v.x & 0xFFFFu) + dd) >> 8, a);
  return (a << 24) | (r << 16) | (g << 8) | b;
}

// LUT index of pixel x of a gradient fetcher (linear, radial or conic): the fetchers' per-pixel
// arithmetic up to the table lookup.
__device__ __forceinline__ uint32_t gradient_index(const DevStyle& st, const RowState& r, int x) {
  switch (st.fetch) {
    case kFetchLinearPad: case kFetchLinearRoR: {
      uint64_t pt = r.a64 + uint64_t(uint32_t(x)) * st.lin_dt;
      return grad_index(uint32_t(pt >> 32), st.fetch == kFetchLinearPad, st.maxi, st.rori);
    }
    case kFetchRadialPad: case kFetchRadialRoR: {
      float xf = float(x);
      float sq_x = xf * xf;
      float a = sqrtf(fabsf(sq_x * st.rad_ddd + (xf * r.f2 + r.f1)));
      float v = (xf * st.rad_bd + r.f0) + a;
      return grad_index(uint32_t(trunc_f(v)), st.fetch == kFetchRadialPad, st.maxi, st.rori);
    }
    default: {    // kFetchConic
      float xf = float(x) * st.con_xx + r.f0;
      float ax = fabsf(xf);
      float ay = r.f1;
      float xy_min = ay < ax ? ay : ax;
      float xy_max = ax < ay ? ay : ax;
      float s = __uint_as_float((ax == xy_min ? 0xFFFFFFFFu : 0u) & __float_as_uint(st.con_n4));
      float p = xy_min / xy_max;
      float p_sq = p * p;
      float v = p_sq * st.con_q[3] + st.con_q[2];
      v = v * p_sq + st.con_q[1];
      v = v * p_sq + st.con_q[0];
      v = fabsf(v * p + (-s));
      v = fabsf(v - __uint_as_float(uint32_t(int32_t(__float_as_uint(xf)) >> 31) & __float_as_uint(st.con_n2)));
      v = fabsf(v - r.f2) + st.con_offset;
      int32_t ni = nearby_f(v);
      return uint32_t(ni < st.con_maxi ? ni : st.con_maxi) & uint32_t(st.con_rori);
    }
  }
}

__device__ __forceinline__ uint32_t fetch(const DevStyle& st, const RowState& r, int x,
                                          const uint32_t* __restrict__ luts, const uint32_t* __restrict__ images) {
  switch (st.fetch) {
    case kFetchSolid:
      return st.solid;
    case kFetchLinearPad: case kFetchLinearRoR: case kFetchRadialPad: case kFetchRadialRoR: case kFetchConic:
      // 32-bit LUT only: the fine stage fetches gradients (dithered ones too) on its own path
      return __ldg(luts + st.lut_offset + gradient_index(st, r, x));
    case kFetchPatAlignedPad: case kFetchPatAlignedRepeat: case kFetchPatAlignedRoR: {
      uint32_t kind = st.fetch - kFetchPatAlignedPad;
      int cx = pat_col(st, x, kind);
      return __ldg(images + st.src_offset + int64_t(r.r0) * st.src_stride + cx);
    }
    case kFetchPatFxFyPad: case kFetchPatFxFyRoR: {
      uint32_t kind = st.fetch == kFetchPatFxFyPad ? 0u : 2u;
      int c0 = pat_col(st, x, kind);
      int c1 = pat_col(st, x + 1, kind);
      const uint32_t* l0 = images + st.src_offset + int64_t(r.r0) * st.src_stride;
      const uint32_t* l1 = images + st.src_offset + int64_t(r.r1) * st.src_stride;
      uint64_t acc = unpack(__ldg(l0 + c0)) * st.pat_wa + unpack(__ldg(l1 + c0)) * st.pat_wc;
      uint64_t u = unpack(__ldg(l0 + c1)) * st.pat_wb + unpack(__ldg(l1 + c1)) * st.pat_wd + acc;
      return pack(div256(u));
    }
    case kFetchPatAffineNN: {
      uint64_t px, py;
      af_normalize(st, r.a64 + st.af_xx * uint64_t(uint32_t(x)), r.b64 + st.af_xy * uint64_t(uint32_t(x)), px, py);
      uint32_t ix, iy;
      af_index(st, px, py, 0, ix, iy);
      return __ldg(images + st.src_offset + int64_t(iy) * st.src_stride + ix);
    }
    default: {   // kFetchPatAffineBI
      uint64_t px, py;
      af_normalize(st, r.a64 + st.af_xx * uint64_t(uint32_t(x)), r.b64 + st.af_xy * uint64_t(uint32_t(x)), px, py);
      uint32_t x0, y0, x1, y1;
      af_index(st, px, py, 0, x0, y0);
      af_index(st, px, py, 1, x1, y1);
      uint32_t wx = uint32_t(px & 0xFFFFFFFFu) >> 24;
      uint32_t wy = uint32_t(py & 0xFFFFFFFFu) >> 24;
      uint32_t ix = 256 - wx, iy = 256 - wy;
      const uint32_t* l0 = images + st.src_offset + int64_t(y0) * st.src_stride;
      const uint32_t* l1 = images + st.src_offset + int64_t(y1) * st.src_stride;
      uint64_t p0 = unpack(__ldg(l0 + x0)) * iy + unpack(__ldg(l1 + x0)) * wy;
      uint64_t p1 = unpack(__ldg(l0 + x1)) * iy + unpack(__ldg(l1 + x1)) * wy;
      p0 = div256(p0) * ix;
      p1 = div256(p1) * wx;
      return pack(div256(p0 + p1));
    }
  }
}

// FillAnalytic_Base::calc_mask (fillgeneric_p.h:381-387).
__device__ __forceinline__ uint32_t calc_mask(uint32_t cov, uint32_t rule_mask, uint32_t alpha) {
  uint32_t m = ((uint32_t(int32_t(cov) >> 9)) & rule_mask) - 256u;
  int32_t mi = int32_t(m);
  uint32_t am = uint32_t(mi < 0 ? -mi : mi);
  am = am > 256u ? 256u : am;
  return (am * alpha) >> 8;
}

// Mask of a box with fractional borders (FillData::init_box_u_8bpc_24x8, pipedefs_p.h:644-815).
__device__ __forceinline__ uint32_t box_u_mask(const int32_t* b, uint32_t alpha, int x, int y) {
  uint32_t ax0 = uint32_t(b[0]) >> 8, ay0 = uint32_t(b[1]) >> 8;
  uint32_t ax1 = uint32_t(b[2] + 0xFF) >> 8, ay1 = uint32_t(b[3] + 0xFF) >> 8;
  if (uint32_t(x) < ax0 || uint32_t(x) >= ax1 || uint32_t(y) < ay0 || uint32_t(y) >= ay1) return 0;
  uint32_t fx0 = uint32_t(b[0]) & 0xFFu, fy0 = uint32_t(b[1]) & 0xFFu;
  uint32_t fx1 = (uint32_t(b[2] - 1) & 0xFFu) + 1u, fy1 = (uint32_t(b[3] - 1) & 0xFFu) + 1u;
  uint32_t w = ax1 - ax0, h = ay1 - ay0;
  fy0 = (h == 1 ? fy1 : 256u) - fy0;
  uint32_t fxw;
  if (w == 1) fxw = fx1 - fx0;
  else if (uint32_t(x) == ax0) fxw = 256u - fx0;
  else if (uint32_t(x) == ax1 - 1) fxw = fx1;
  else fxw = 256u;
  if (uint32_t(y) == ay0) return (fxw * (fy0 * alpha)) >> 16;
  if (uint32_t(y) == ay1 - 1) return (fxw * (fy1 * alpha)) >> 16;
  return (fxw * alpha) >> 8;
}

}  // namespace px
}  // namespace blgpu
