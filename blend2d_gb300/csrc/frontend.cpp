// frontend.cpp - host front end: fetch-data setup and numeric helpers (see frontend.h).
// Compiled with -ffp-contract=off: every expression is evaluated unfused, in source order.
#include "frontend.h"
#include "divmagic.h"

#include <math.h>
#include <string.h>

#include <cmath>

#include <algorithm>

namespace blgpu {

// x86 conversion semantics of the reference build (cvttsd2si / cvtsd2si give INT_MIN for NaN and
// out-of-range values; blend2d/support/math_p.h:370-440).
int trunc_to_int(double x) {
  if (!(x > -2147483649.0 && x < 2147483648.0)) return INT32_MIN;
  return int(x);
}
static int64_t trunc_to_int64(double x) {
  if (!(x >= -9223372036854775808.0 && x < 9223372036854775808.0)) return INT64_MIN;
  return int64_t(x);
}
int64_t floor_to_int64(double x) {
  int64_t y = trunc_to_int64(x);
  return y - int64_t(double(y) > x);
}
static int nearby_to_int(double x) {
  if (!(x >= -2147483648.5 && x < 2147483647.5)) return INT32_MIN;
  return int(rint(x));
}
int round_to_int(double x) {
  int y = nearby_to_int(x);
  return y + (double(y) - x == -0.5);
}
static inline double dmin(double a, double b) { return b < a ? b : a; }
static inline double dmax(double a, double b) { return a < b ? b : a; }

// TransformInternal::multiply (blend2d/core/matrix_p.h:57-64).
void mat_multiply(Mat& dst, const Mat& a, const Mat& b) {
  Mat r;
  r.m00 = a.m00 * b.m00 + a.m01 * b.m10;
  r.m01 = a.m00 * b.m01 + a.m01 * b.m11;
  r.m10 = a.m10 * b.m00 + a.m11 * b.m10;
  r.m11 = a.m10 * b.m01 + a.m11 * b.m11;
  r.m20 = a.m20 * b.m00 + a.m21 * b.m10 + b.m20;
  r.m21 = a.m20 * b.m01 + a.m21 * b.m11 + b.m21;
  dst = r;
}

// bl_matrix2d_invert (blend2d/core/matrix.cpp:442-463).
bool mat_invert(Mat& dst, const Mat& s) {
  double d = s.m00 * s.m11 - s.m01 * s.m10;
  if (d == 0.0 || !isfinite(d)) return false;
  double t00 = s.m11, t01 = -s.m01, t10 = -s.m10, t11 = s.m00;
  t00 /= d; t01 /= d; t10 /= d; t11 /= d;
  double t20 = -(s.m20 * t00 + s.m21 * t10);
  double t21 = -(s.m20 * t01 + s.m21 * t11);
  dst = Mat{t00, t01, t10, t11, t20, t21};
  return true;
}

// bl_matrix2d_get_type (blend2d/core/matrix.cpp:133-211).
int mat_type(const Mat& m) {
  unsigned msk = (unsigned(m.m00 != 0.0) << 3) | (unsigned(m.m01 != 0.0) << 2) |
                 (unsigned(m.m10 != 0.0) << 1) | unsigned(m.m11 != 0.0);
  const unsigned valid = (1u << 3) | (1u << 6) | (1u << 7) | (1u << 9) | (1u << 11) | (1u << 12) |
                         (1u << 13) | (1u << 14) | (1u << 15);
  double d = m.m00 * m.m11 - m.m01 * m.m10;
  if (!((1u << msk) & valid) || !isfinite(d) || !isfinite(m.m20) || !isfinite(m.m21)) return kTTInvalid;
  if (msk != 9u) return msk == 6u ? kTTSwap : kTTAffine;
  if (!((m.m00 == 1.0) & (m.m11 == 1.0))) return kTTScale;
  if (!((m.m20 == 0.0) & (m.m21 == 0.0))) return kTTTranslate;
  return kTTIdentity;
}

// cvt_prgb32_8888_from_argb32_8888 (blend2d/pixelops/scalar_p.h:146-157).
uint32_t premultiply(uint32_t c) {
  uint32_t a = c >> 24;
  auto d = [](uint32_t x) { return ((x + 128u) * 257u) >> 16; };
  return (d(255u * a) << 24) | (d(((c >> 16) & 255u) * a) << 16) | (d(((c >> 8) & 255u) * a) << 8) | d((c & 255u) * a);
}

// calculate_band_height for a synchronous context (blend2d/raster/rastercontext.cpp:4154-4193).
int default_band_height(int width) {
  int bh = 64;
  size_t pixel_count = size_t(unsigned(width)) * size_t(bh);
  do {
    if (pixel_count * 4u <= 1024u * 256u) break;
    bh >>= 1;
    pixel_count >>= 1;
  } while (bh > 8);
  return bh;
}

void style_solid(HostStyle& s, uint32_t argb32) {
  s.dev = DevStyle{};
  s.image = -1;
  s.stops.clear();
  s.nop = false;
  s.dev.fetch = kFetchSolid;
  s.dev.solid = premultiply(argb32);
  s.format = argb32 == 0 ? kFmtZERO32 : (argb32 >= 0xFF000000u ? kFmtFRGB32 : kFmtPRGB32);
}

// --- gradients --------------------------------------------------------------------------------

// analyze_stop_array + copy_unsafe_stops (blend2d/core/gradient.cpp:58-173). Returns false when
// an offset is outside [0, 1] (assign_stops then fails and the gradient keeps no stops).
static bool normalize_stops(std::vector<DevStop>& out, const DevStop* src, size_t n) {
  uint32_t result = 0, was_same = 0;
  double prev = -1.0;
  for (size_t i = 0; i < n; i++) {
    double off = src[i].offset;
    if (!((off >= 0.0) & (off <= 1.0))) return false;
    uint32_t same = off == prev;
    result |= off < prev;
    result |= same & was_same;
    was_same = same;
    prev = off;
  }
  out.assign(src, src + n);
  if (result == 0 || n == 0) return true;
  std::vector<size_t> idx(n);
  for (size_t i = 0; i < n; i++) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return src[a].offset < src[b].offset; });
  size_t j = 0;
  double p1 = -1.0, p2 = -1.0;
  out.resize(n);
  for (size_t i = 0; i + 1 < n; i++) {
    double off = src[idx[i]].offset;
    uint64_t rgba = src[idx[i]].rgba64;
    j -= size_t((p1 == p2) & (p2 == off));
    out[j].offset = off;
    out[j].rgba64 = rgba;
    j++;
    p1 = p2;
    p2 = off;
  }
  out.resize(j);
  return true;
}

static uint32_t rgba32_of(uint64_t v) {
  return uint32_t(((v >> 56) & 0xFF) << 24 | ((v >> 40) & 0xFF) << 16 | ((v >> 24) & 0xFF) << 8 | ((v >> 8) & 0xFF));
}

static bool init_linear(DevStyle& d, const double* v, uint32_t extend, const Mat& t) {   // pipedefs.cpp:386-434
  Mat inv;
  if (!mat_invert(inv, t)) return false;
  uint32_t lut_size = d.lut_size;
  uint32_t maxi = extend == 2 ? lut_size * 2u - 1u : lut_size - 1u;
  uint32_t rori = extend == 2 ? maxi : 0u;
  double ax = v[2] - v[0], ay = v[3] - v[1];
  double dist = ax * ax + ay * ay;
  double mx = v[0] * t.m00 + v[1] * t.m10 + t.m20;
  double my = v[0] * t.m01 + v[1] * t.m11 + t.m21;
  double ox = 0.5 - mx, oy = 0.5 - my;
  double dt = ax * inv.m00 + ay * inv.m01;
  double dy = ax * inv.m10 + ay * inv.m11;
  double scale = double(int64_t(uint64_t(lut_size) << 32)) / dist;
  double offset = ox * dt + oy * dy;
  dt *= scale; dy *= scale; offset *= scale;
  d.lin_dy = uint64_t(floor_to_int64(dy));
  d.lin_dt = uint64_t(floor_to_int64(dt));
  d.lin_pt0 = uint64_t(floor_to_int64(offset));
  d.maxi = maxi; d.rori = rori;
  d.fetch = extend != 0 ? kFetchLinearRoR : kFetchLinearPad;
  return true;
}

static bool init_radial(DevStyle& d, const double* v, uint32_t extend, const Mat& t) {   // pipedefs.cpp:480-576
  Mat inv;
  if (!mat_invert(inv, t)) return false;
  uint32_t lut_size = d.lut_size;
  uint32_t maxi = extend == 2 ? lut_size * 2u - 1u : lut_size - 1u;
  d.maxi = maxi;
  d.rori = extend == 2 ? maxi : 0u;
  double cpx = v[0], cpy = v[1], fpx = v[2], fpy = v[3], cr = v[4], fr = v[5];
  double dpx = cpx - fpx, dpy = cpy - fpy;
  double dr = cr - fr;
  double sq_dxdy = dpx * dpx + dpy * dpy;
  double dxdy = sqrt(sq_dxdy);
  const double lim = 0.5;
  if (fabs(dxdy - dr) < lim) {
    double d0x = (dpx * (dr - lim)) / dxdy, d0y = (dpy * (dr - lim)) / dxdy;
    double d1x = (dpx * (dr + lim)) / dxdy, d1y = (dpy * (dr + lim)) / dxdy;
    double e0 = fabs(d0x * d0x + d0y * d0y - sq_dxdy);
    double e1 = fabs(d1x * d1x + d1y * d1y - sq_dxdy);
    if (e0 < e1) { dpx = d0x; dpy = d0y; } else { dpx = d1x; dpy = d1y; }
    fpx = cpx - dpx; fpy = cpy - dpy;
    sq_dxdy = dpx * dpx + dpy * dpy;
  }
  double a = dr * dr - sq_dxdy;
  double sq_fr = fr * fr;
  double scale = double(lut_size);
  double xx = inv.m00, xy = inv.m01, yx = inv.m10, yy = inv.m11;
  double tpx = inv.m20 + (xx + xy) * 0.5 - fpx;
  double tpy = inv.m21 + (yx + yy) * 0.5 - fpy;
  d.rad_tx = tpx; d.rad_ty = tpy; d.rad_yx = yx; d.rad_yy = yy;
  double a_mul_4 = a * 4.0;
  double inv2a = (scale * 0.5) / a;
  double sq_inv2a = inv2a * inv2a;
  d.rad_amul4 = a_mul_4; d.rad_inv2a = inv2a; d.rad_sq_inv2a = sq_inv2a; d.rad_sq_fr = sq_fr;
  double sq_xx_yx = xx * xx + xy * xy;
  double b0 = 2.0 * (dr * fr + tpx * dpx + tpy * dpy);
  double bx = 2.0 * (dpx * xx + dpy * xy);
  double by = 2.0 * (dpx * yx + dpy * yy);
  d.rad_b0 = -b0; d.rad_by = -by;
  double bx2 = bx * 2.0;
  double sq_bx = bx * bx;
  double dd0 = sq_bx + bx2 * b0 + a_mul_4 * (sq_xx_yx + 2.0 * (tpx * xx + tpy * xy));
  double ddy = bx2 * by + a_mul_4 * (2.0 * (xx * yx + yy * xy));
  double ddd_half = (sq_bx + a_mul_4 * sq_xx_yx);
  double ddd_half_inv = ddd_half * sq_inv2a;
  d.rad_dd0 = dd0 - ddd_half;
  d.rad_ddy = ddy;
  d.rad_bd = float(-bx * inv2a);
  d.rad_ddd = float(ddd_half_inv);
  d.fetch = extend != 0 ? kFetchRadialRoR : kFetchRadialPad;
  return true;
}

static bool init_conic(DevStyle& d, const double* v, const Mat& t) {   // pipedefs.cpp:614-671
  static const double q256[4] = {4.071421038552e+1, -1.311160794048e+1, 6.017670215625, -1.623253505085};
  const double kPI_MUL_2 = 6.28318530717958647692;
  double angle = v[2], repeat = v[3];
  double cx = v[0] * t.m00 + v[1] * t.m10 + t.m20;
  double cy = v[0] * t.m01 + v[1] * t.m11 + t.m21;
  cx = 0.5 - cx; cy = 0.5 - cy;
  double vx = 1.0 * t.m00 + 0.0 * t.m10, vy = 1.0 * t.m01 + 0.0 * t.m11;
  double matrix_angle = atan2(vy, vx);
  Mat u = t;
  {
    double ang = -matrix_angle;
    double as = sin(ang), ac = cos(ang);
    double t00 = as * u.m10 + ac * u.m00, t01 = as * u.m11 + ac * u.m01;
    double t10 = ac * u.m10 - as * u.m00, t11 = ac * u.m11 - as * u.m01;
    double ttx = cx - ac * cx + as * cy;
    double tty = cy - as * cx - ac * cy;
    double t20 = ttx * u.m00 + tty * u.m10 + u.m20;
    double t21 = ttx * u.m01 + tty * u.m11 + u.m21;
    u = Mat{t00, t01, t10, t11, t20, t21};
  }
  angle += matrix_angle;
  double fr = angle / -kPI_MUL_2;
  double off = fr - floor(fr);
  if (off != 0.0) off = -1.0 + off;
  Mat inv;
  if (!mat_invert(inv, u)) return false;
  d.con_tx = cx * inv.m00 + cy * inv.m10;
  d.con_ty = cx * inv.m01 + cy * inv.m11;
  d.con_yx = inv.m10;
  d.con_yy = inv.m11;
  double lut = double(int(d.lut_size));
  double rep = lut * repeat;
  double q_scale = rep / 256.0;
  for (int k = 0; k < 4; k++) d.con_q[k] = float(q256[k] * q_scale);
  d.con_n1 = float(rep);
  d.con_n2 = float(rep * 0.5);
  d.con_n4 = float(rep * 0.25);
  d.con_offset = float(off * rep - 0.5);
  d.con_xx = float(inv.m00);
  d.con_maxi = INT32_MAX;
  d.con_rori = int32_t(d.lut_size - 1u);
  d.fetch = kFetchConic;
  return true;
}

// init_non_solid_fetch_data, gradient branch (blend2d/raster/rastercontext.cpp:423-478) with
// GradientInternal::ensure_info (blend2d/core/gradient.cpp:202-287).
// `quality`: BLGradientQuality captured when the style is set (rastercontext.cpp:454-466).
void style_gradient(HostStyle& s, const GradientDesc& g, const Mat& final_transform, uint32_t quality) {
  // reset in place: the stop vector keeps its capacity from style to style
  std::vector<DevStop> stops = std::move(s.stops);
  s.nop = true;
  s.format = kFmtPRGB32;
  s.dev = DevStyle{};
  s.image = -1;
  if (!normalize_stops(stops, g.stops, g.stop_count)) stops.clear();
  Mat tf = final_transform;
  if (g.transform) {
    Mat gm{g.transform[0], g.transform[1], g.transform[2], g.transform[3], g.transform[4], g.transform[5]};
    if (mat_type(gm) != kTTIdentity) mat_multiply(tf, gm, final_transform);
  }
  size_t n = stops.size();
  if (n == 0) { s.nop = true; return; }

  uint32_t flags = 0;
  uint64_t prev = stops[0].rgba64 & 0xFF00FF00FF00FF00ull;
  if (prev < 0xFF00000000000000ull) flags |= 1;
  if (prev > 0x00FFFFFFFFFFFFFFull) flags |= 2;
  for (size_t i = 1; i < n; i++) {
    uint64_t v = stops[i].rgba64 & 0xFF00FF00FF00FF00ull;
    if (v == prev) continue;
    flags |= 4;
    if (v < 0xFF00000000000000ull) flags |= 1;
    if (v > 0x00FFFFFFFFFFFFFFull) flags |= 2;
    prev = v;
  }
  if (!(flags & 2)) flags &= ~4u;
  uint32_t lut_size;
  if (!(flags & 4) || n == 1) lut_size = 256;
  else if (n == 2) lut_size = (stops[1].offset - stops[0].offset >= 0.998) ? 256 : 512;
  else if (n == 3) lut_size = (stops[0].offset <= 0.002 && stops[1].offset == 0.5 && stops[2].offset >= 0.998) ? 512 : 1024;
  else lut_size = 1024;
  s.format = (flags & 1) ? kFmtPRGB32 : kFmtFRGB32;
  s.nop = false;
  if (!(flags & 4)) {
    s.dev.fetch = kFetchSolid;
    s.dev.solid = premultiply(rgba32_of(stops[n - 1].rgba64));
    return;
  }
  if (quality >= 2u) {            // DITHER: lut_size(true) (gradient_p.h:113-120), 64-bit LUT
    lut_size = lut_size * 2u < 1024u ? lut_size * 2u : 1024u;
    s.dev.dither = 1u;
  }
  s.dev.lut_size = lut_size;
  bool ok = g.type == 0 ? init_linear(s.dev, g.values, g.extend, tf)
          : g.type == 1 ? init_radial(s.dev, g.values, g.extend, tf)
                        : init_conic(s.dev, g.values, tf);
  if (!ok) { s.nop = true; return; }
  s.stops = std::move(stops);
}

// --- shapes -------------------------------------------------------------------------------------

// BLPath::add_geometry (path.cpp:1408-1600, direction CW) for circles, ellipses, round rectangles
// and triangles: the path the reference fills or strokes for fill_geometry / stroke_geometry.
bool shape_path(uint32_t type, const double* v, std::vector<uint8_t>& cmd, std::vector<double>& xy) {
  constexpr double kKappa = 0.55228474983;   // mathconst_p.h:52
  cmd.clear();
  xy.clear();
  auto put = [&](uint8_t c, double x, double y) { cmd.push_back(c); xy.push_back(x); xy.push_back(y); };
  auto cubic = [&](double x1, double y1, double x2, double y2, double x3, double y3) {
    put(4, x1, y1); put(4, x2, y2); put(1, x3, y3);
  };
  auto box = [&](double x0, double y0, double x1, double y1) {   // PathAppender::add_box
    put(0, x0, y0); put(1, x1, y0); put(1, x1, y1); put(1, x0, y1); put(5, NAN, NAN);
  };
  switch (type) {
    case kGeometryCircle: case kGeometryEllipse: {
      double x0 = v[0], y0 = v[1], rx = v[2];
      double ry = type == kGeometryCircle ? fabs(rx) : v[3];
      double kx = rx * kKappa, ky = ry * kKappa;
      put(0, x0 + rx, y0);
      cubic(x0 + rx, y0 + ky, x0 + kx, y0 + ry, x0, y0 + ry);
      cubic(x0 - kx, y0 + ry, x0 - rx, y0 + ky, x0 - rx, y0);
      cubic(x0 - rx, y0 - ky, x0 - kx, y0 - ry, x0, y0 - ry);
      cubic(x0 + kx, y0 - ry, x0 + rx, y0 - ky, x0 + rx, y0);
      put(5, NAN, NAN);
      return true;
    }
    case kGeometryRoundRect: {
      double x0 = v[0], y0 = v[1], x1 = v[0] + v[2], y1 = v[1] + v[3];
      double w_half = v[2] * 0.5, h_half = v[3] * 0.5;
      double arx = fabs(v[4]), ary = fabs(v[5]);
      double rx = w_half < arx ? w_half : arx;
      double ry = h_half < ary ? h_half : ary;
      if (!(rx > 1e-14 && ry > 1e-14)) { box(x0, y0, x1, y1); return true; }   // degenerate radii
      double kx = rx * (1.0 - kKappa), ky = ry * (1.0 - kKappa);
      put(0, x0 + rx, y0);
      put(1, x1 - rx, y0);
      cubic(x1 - kx, y0, x1, y0 + ky, x1, y0 + ry);
      put(1, x1, y1 - ry);
      cubic(x1, y1 - ky, x1 - kx, y1, x1 - rx, y1);
      put(1, x0 + rx, y1);
      cubic(x0 + kx, y1, x0, y1 - ky, x0, y1 - ry);
      put(1, x0, y0 + ry);
      cubic(x0, y0 + ky, x0 + kx, y0, x0 + rx, y0);
      put(5, NAN, NAN);
      return true;
    }
    case kGeometryTriangle:
      put(0, v[0], v[1]); put(1, v[2], v[3]); put(1, v[4], v[5]); put(5, NAN, NAN);
      return true;
    case kGeometryArc: case kGeometryChord: case kGeometryPie: {
      // {cx, cy, rx, ry, start, sweep}: arc_to_cubic_spline (path.cpp:503-570), quarter arcs as
      // cubics and the rest as a conic turned into a cubic (PathAppender::conic_to, path_p.h:319)
      const double cx = v[0], cy = v[1], rx = v[2], ry = v[3];
      double sweep = v[5];
      if (type == kGeometryPie) put(0, cx, cy);
      double ss = sin(v[4]), sc = cos(v[4]);
      // make_sin_cos, post_scale(r), post_translate(c)
      double m00 = sc * rx, m01 = ss * ry, m10 = -ss * rx, m11 = sc * ry, m20 = 0.0 * rx + cx, m21 = 0.0 * ry + cy;
      if (sweep < 0) { m10 *= -1.0; m11 *= -1.0; sweep = -sweep; }      // scale(1, -1)
      auto map = [&](double x, double y, double& ox, double& oy) { ox = x * m00 + y * m10 + m20; oy = x * m01 + y * m11 + m21; };
      double v1x = 1.0, v1y = 0.0, vcx = 1.0, vcy = 1.0, v2x, v2y;
      constexpr double kPi2 = 6.28318530717958647692;
      if (sweep >= kPi2 - 1e-14) { sweep = kPi2; v2x = v1x; v2y = v1y; }
      else {
        if (std::isnan(sweep)) { if (type != kGeometryArc) put(5, NAN, NAN); return true; }
        v2x = cos(sweep); v2y = sin(sweep);
      }
      double p0x, p0y;
      map(v1x, v1y, p0x, p0y);
      put(type == kGeometryPie ? 1 : 0, p0x, p0y);
      static const double steps[4] = {1.57079632679489661923, 3.14159265358979323846, 4.71238898038468985769,
                                      6.28318530717958647692};
      size_t i = 0;
      bool full = false;
      while (sweep > steps[i]) {
        double t = v1x; v1x = -v1y; v1y = t;                                 // Geometry::normal
        double p1x, p1y, p2x, p2y;
        map(vcx, vcy, p1x, p1y);
        map(v1x, v1y, p2x, p2y);
        cubic(p0x + (p1x - p0x) * kKappa, p0y + (p1y - p0y) * kKappa, p2x + (p1x - p2x) * kKappa,
              p2y + (p1y - p2y) * kKappa, p2x, p2y);
        if (++i == 4) { full = true; break; }
        t = vcx; vcx = -vcy; vcy = t;
        p0x = p2x; p0y = p2y;
      }
      if (!full) {
        double sx = v1x + v2x, sy = v1y + v2y;
        double dd = sx * sx + sy * sy;
        vcx = 2.0 * sx / dd; vcy = 2.0 * sy / dd;
        double w = sqrt(0.5 * (v1x * v2x + v1y * v2y) + 0.5);
        double k = 4.0 * w / (3.0 * (1.0 + w));
        double p1x, p1y, p2x, p2y;
        map(vcx, vcy, p1x, p1y);
        map(v2x, v2y, p2x, p2y);
        cubic(p0x + (p1x - p0x) * k, p0y + (p1y - p0y) * k, p2x + (p1x - p2x) * k, p2y + (p1y - p2y) * k, p2x, p2y);
      }
      if (type != kGeometryArc) put(5, NAN, NAN);
      return true;
    }
    default:
      return false;
  }
}

// --- patterns ---------------------------------------------------------------------------------

// init_pattern_tx_ty (blend2d/pipeline/pipedefs.cpp:49-110).
static void pattern_simple(DevStyle& d, uint32_t extend, int tx, int ty, bool fractional, bool fxfy) {
  uint32_t ex = extend, ey = extend;
  int rx = 0, ry = 0;
  if (d.src_w <= 1) ex = 0;
  if (d.src_h <= 1) ey = 0;
  if (ex >= 1) {
    rx = d.src_w << int(ex == 2);
    if (unsigned(tx) >= unsigned(rx)) tx %= rx;
    if (tx < 0) tx += rx;
    if (fractional) ex = 1;
  }
  if (ey >= 1) {
    ry = d.src_h << int(ey == 2);
    if (unsigned(ty) >= unsigned(ry)) ty %= ry;
    if (ty < 0) ty += ry;
  }
  d.pat_tx = tx; d.pat_ty = ty; d.pat_rx = rx; d.pat_ry = ry;
  d.ext_y = ey;
  if (fxfy) d.fetch = ex == 0 ? kFetchPatFxFyPad : kFetchPatFxFyRoR;
  else d.fetch = ex == 0 ? kFetchPatAlignedPad : (ex == 1 ? kFetchPatAlignedRepeat : kFetchPatAlignedRoR);
}

// init_pattern_fx_fy (blend2d/pipeline/pipedefs.cpp:116-160).
static void pattern_fx_fy(DevStyle& d, uint32_t extend, uint32_t quality, int64_t tx64, int64_t ty64) {
  uint32_t wx = uint32_t(tx64 & 0xFF), wy = uint32_t(ty64 & 0xFF);
  int tx = -int(tx64 >> 8), ty = -int(ty64 >> 8);
  bool fractional = (wx | wy) != 0;
  bool fxfy = false;
  if (fractional) {
    if (quality == 0) {
      tx -= int(wx >= 128);
      ty -= int(wy >= 128);
      fractional = false;
    }
    else {
      d.pat_wa = (wy * wx) >> 8;
      d.pat_wb = (wy * (256 - wx) + 255) >> 8;
      d.pat_wc = ((256 - wy) * wx) >> 8;
      d.pat_wd = ((256 - wy) * (256 - wx) + 255) >> 8;
      tx--;
      ty--;
      fxfy = true;
    }
  }
  pattern_simple(d, extend, tx, ty, fractional, fxfy);
}

// init_pattern_affine (blend2d/pipeline/pipedefs.cpp:162-381).
static bool pattern_affine(DevStyle& d, uint32_t extend, uint32_t quality, const Mat& t) {
  Mat inv;
  if (!mat_invert(inv, t)) return false;
  int tw = d.src_w, th = d.src_h;
  if (tw == 0) return false;
  double xx = inv.m00, xy = inv.m01, yx = inv.m10, yy = inv.m11;
  if ((fabs(xx - 1.0) <= 1e-14) & (fabs(xy) <= 1e-14) & (fabs(yx) <= 1e-14) & (fabs(yy - 1.0) <= 1e-14)) {
    pattern_fx_fy(d, extend, quality, floor_to_int64(-inv.m20 * 256.0), floor_to_int64(-inv.m21 * 256.0));
    return true;
  }
  d.fetch = quality == 0 ? kFetchPatAffineNN : kFetchPatAffineBI;
  uint32_t ex = extend, ey = extend;
  double tx = inv.m20, ty = inv.m21;
  tx += 0.5 * (xx + yx);
  ty += 0.5 * (xy + yy);
  const double fp_scale = 4294967296.0;
  int ox = INT32_MAX, oy = INT32_MAX, rx = 0, ry = 0;
  d.af_minx = 0; d.af_miny = 0;
  d.af_maxx = tw - 1; d.af_maxy = th - 1;
  d.af_corx = tw - 1; d.af_cory = th - 1;
  if (ex != 0) {
    d.af_minx = INT32_MIN;
    if (ex == 1) d.af_corx = 0;
    ox = tw;
    if (ex == 2) tw *= 2;
    if (xx < 0.0) {
      xx = -xx; yx = -yx; tx = double(tw) - tx;
      if (ex == 1) { ox = 0; d.af_corx = d.af_maxx; d.af_maxx = -1; }
    }
    ox--;
  }
  if (ey != 0) {
    d.af_miny = INT32_MIN;
    if (ey == 1) d.af_cory = 0;
    oy = th;
    if (ey == 2) th *= 2;
    if (xy < 0.0) {
      xy = -xy; yy = -yy; ty = double(th) - ty;
      if (ey == 1) { oy = 0; d.af_cory = d.af_maxy; d.af_maxy = -1; }
    }
    oy--;
  }
  if (quality != 0) { tx -= 0.5; ty -= 0.5; }
  double tw_d = double(tw), th_d = double(th);
  if (ex == 0) tw_d = 2147483647.0;
  else { tx = fmod(tx, tw_d); rx = tw; if (xx >= tw_d) xx = fmod(xx, tw_d); }
  if (ey == 0) th_d = 2147483647.0;
  else { ty = fmod(ty, th_d); ry = th; if (xy >= th_d) xy = fmod(xy, th_d); }
  xx *= fp_scale; xy *= fp_scale; yx *= fp_scale; yy *= fp_scale; tx *= fp_scale; ty *= fp_scale;
  double all_min = dmin(dmin(yy, yx), dmin(xy, xx));
  double all_max = dmax(dmax(xx, xy), dmax(yx, yy));
  all_min = dmin(all_min, dmin(ty, tx));
  all_max = dmax(dmax(tx, ty), all_max);
  if (all_min >= double(INT64_MIN + 1) && all_max <= double(INT64_MAX)) {
    d.af_xx = uint64_t(floor_to_int64(xx)); d.af_xy = uint64_t(floor_to_int64(xy));
    d.af_yx = uint64_t(floor_to_int64(yx)); d.af_yy = uint64_t(floor_to_int64(yy));
    d.af_tx = uint64_t(floor_to_int64(tx)); d.af_ty = uint64_t(floor_to_int64(ty));
  }
  else {
    d.af_xx = d.af_xy = d.af_yx = d.af_yy = d.af_tx = d.af_ty = 0;
  }
  d.af_rx = rx; d.af_ry = ry; d.af_ox = ox; d.af_oy = oy;
  d.af_tw = int32_t(tw_d); d.af_th = int32_t(th_d);
  const DivMagic mw = div_magic(d.af_tw), mh = div_magic(d.af_th);
  d.af_tw_m = mw.m; d.af_tw_s = mw.s; d.af_th_m = mh.m; d.af_th_s = mh.s;
  return true;
}

// init_non_solid_fetch_data, pattern branch (blend2d/raster/rastercontext.cpp:377-421).
// Image blits (rastercontext.cpp:3941-4160): the image area as the style's source, then the
// fetcher the blit sets up. Returns false (style NOP) for an empty area or a singular transform.
static bool blit_source(HostStyle& s, int image, int img_w, const int area[4]) {
  s.nop = true;
  s.dev = DevStyle{};
  s.image = -1;
  s.stops.clear();
  s.format = kFmtPRGB32;
  if (area[2] <= 0 || area[3] <= 0) return false;
  s.image = image;
  s.dev.src_offset = uint64_t(uint32_t(area[1])) * uint64_t(img_w) + uint64_t(uint32_t(area[0]));
  s.dev.src_w = area[2]; s.dev.src_h = area[3]; s.dev.src_stride = img_w;
  return true;
}

// init_pattern_blit (pipedefs_p.h:1070-1076): pixel (x, y) reads the area's (x - x0, y - y0), never
// outside it, which the aligned fetcher with pad extend and translation -x0, -y0 does.
void style_blit_aligned(HostStyle& s, int image, int img_w, const int area[4], int x0, int y0) {
  if (!blit_source(s, image, img_w, area)) return;
  pattern_simple(s.dev, 0u, -x0, -y0, false, false);
  s.nop = false;
}

// setup_pattern_fx_fy with the blit extend (REFLECT, rastercontext_p.h:51).
void style_blit_fx_fy(HostStyle& s, int image, int img_w, const int area[4], uint32_t quality, int64_t tx64, int64_t ty64) {
  if (!blit_source(s, image, img_w, area)) return;
  pattern_fx_fy(s.dev, 2u, quality, tx64, ty64);
  s.nop = false;
}

// setup_pattern_affine with the blit extend.
void style_blit_affine(HostStyle& s, int image, int img_w, const int area[4], uint32_t quality, const Mat& t) {
  if (!blit_source(s, image, img_w, area)) return;
  if (!pattern_affine(s.dev, 2u, quality, t)) { s.nop = true; return; }
  s.nop = false;
}

void style_pattern(HostStyle& s, const PatternDesc& p, uint32_t quality, const Mat& final_transform) {
  s.nop = true;
  s.dev = DevStyle{};
  s.image = -1;
  s.stops.clear();
  s.format = kFmtPRGB32;
  int ax = 0, ay = 0, aw = p.img_w, ah = p.img_h;
  if (p.area[2] > 0) { ax = p.area[0]; ay = p.area[1]; aw = p.area[2]; ah = p.area[3]; }
  if (!aw || !ah) { s.nop = true; return; }
  s.image = p.image;
  s.dev.src_offset = uint64_t(ay) * uint64_t(p.img_w) + uint64_t(ax);   // relative to the image
  s.dev.src_w = aw; s.dev.src_h = ah; s.dev.src_stride = p.img_w;
  Mat tf = final_transform;
  if (p.transform) {
    Mat pm{p.transform[0], p.transform[1], p.transform[2], p.transform[3], p.transform[4], p.transform[5]};
    if (mat_type(pm) != kTTIdentity) mat_multiply(tf, pm, final_transform);
  }
  if (!pattern_affine(s.dev, p.extend, quality, tf)) { s.nop = true; return; }
  s.nop = false;
}

}  // namespace blgpu
