// edge_build.cuh - FP64 edge building on the device (kernel K1).
//
// One thread builds the edges of one analytic fill command: transform, clip against the canvas
// (24.8 fixed-point clip box), split curves into monotonic pieces, flatten them by midpoint
// subdivision and truncate to 24.8 integers - the same arithmetic, in the same order, as the
// reference's EdgeBuilder<int> (blend2d/raster/edgebuilder_p.h:776-2629) and the Bezier splitters
// it calls (blend2d/geometry/bezier_p.h:366-395, :834-920; blend2d/support/math_p.h:574-592).
//
// The reference links polylines into per-band lists; the rasterized result depends only on the
// multiset of non-horizontal segments (cell sums are commutative), so here every polyline point
// appended after the first emits the segment joining it to its predecessor. The translation unit
// is compiled with -fmad=false so every a*b+c stays unfused like the reference's SSE2 build.
#pragma once

#include "blgpu_internal.h"

namespace blgpu {
namespace eb {

struct Pt { double x, y; };

__device__ __forceinline__ double dmin(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double dmax(double a, double b) { return a < b ? b : a; }
__device__ __forceinline__ double dclamp(double a, double lo, double hi) { return dmin(hi, dmax(lo, a)); }

// x86 cvttsd2si: truncation, INT_MIN for NaN / out-of-range (the reference is an x86-64 build).
// Done on the bits with integer instructions: |x| < 1 -> 0; exponent >= 31 (|x| >= 2^31, inf,
// NaN) -> INT_MIN, which is also the right value for the only in-range case there, -2^31 <= x <
// -2^31 + 1; otherwise the mantissa shifted by the exponent, negated for negative x.
__device__ __forceinline__ int trunc_i(double x) {
  const uint64_t b = uint64_t(__double_as_longlong(x));
  const int e = int((b >> 52) & 0x7FFu) - 1023;
  if (e < 0) return 0;
  if (e >= 31) return INT32_MIN;
  const uint32_t v = uint32_t(((b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull) >> (52 - e));
  return (b >> 63) ? -int(v) : int(v);
}

// Segment sink: buffers emitted segments and appends them to the frame's segment array in
// batches (one atomic per batch). Segment order is irrelevant downstream: cell sums commute.
constexpr int kSinkBatch = 16;

struct Sink {
  DevSeg* out;
  uint32_t* meta;
  uint32_t* counter;    // segments appended so far (all builders of the frame)
  uint32_t capacity;    // slots in out/meta; the host re-runs with more when exceeded
  uint32_t cmd;
  uint32_t n;           // segments emitted by this builder
  uint32_t rows;        // bound of the seglist entries of the emitted segments
  int ymin, ymax, xmin, xmax;
  int nb;
  DevSeg buf[kSinkBatch];
  uint32_t sbuf[kSinkBatch];

  __device__ __forceinline__ void init(DevSeg* o, uint32_t* m, uint32_t* ctr, uint32_t cap, uint32_t c) {
    out = o; meta = m; counter = ctr; capacity = cap; cmd = c;
    n = 0; rows = 0; nb = 0;
    ymin = INT32_MAX; ymax = INT32_MIN; xmin = INT32_MAX; xmax = INT32_MIN;
  }
  __device__ void flush() {
    if (!nb) return;
    uint32_t base = atomicAdd(counter, uint32_t(nb));
    for (int k = 0; k < nb; k++) {
      if (base + uint32_t(k) < capacity) {
        out[base + k] = buf[k];
        meta[base + k] = (cmd << 1) | sbuf[k];
      }
    }
    nb = 0;
  }
  __device__ __forceinline__ void emit(int x0, int y0, int x1, int y1, uint32_t sign) {
    if (y0 == y1) return;
    buf[nb] = DevSeg{x0, y0, x1, y1};
    sbuf[nb] = sign;
    if (++nb == kSinkBatch) flush();
    n++;
    // bound of the seglist entries (strip_tile_range summed over the segment's strip rows): the
    // per-strip ranges of a line tile its slackened x extent, overlapping by at most one tile at
    // each strip boundary and widened by at most one tile on each side by the slack
    {
      const uint32_t strips = (uint32_t((y1 - 1) >> 8) >> kStripShift) - (uint32_t(y0 >> 8) >> kStripShift) + 1u;
      const int lo = min(x0, x1) - 256, hi = max(x0, x1) + 256;
      const uint32_t tiles = uint32_t((((hi >> 8) + 1) >> kTileShift) - ((lo >> 8) >> kTileShift) + 1);
      rows += tiles + 3u * strips;
    }
    ymin = min(ymin, y0);
    ymax = max(ymax, y1);
    xmin = min(xmin, min(x0, x1));
    xmax = max(xmax, max(x0, x1));
  }
};

enum { CF_X0 = 1, CF_Y0 = 2, CF_X1 = 4, CF_Y1 = 8 };

struct Builder {
  Sink sink;
  double cx0, cy0, cx1, cy1;
  int icx0, icx1;
  double tol_sq;
  double acc_x0_y0, acc_x0_y1, acc_x1_y0, acc_x1_y1;
  // open polyline
  int px, py;
  uint32_t psign;
  bool pasc;

  __device__ __forceinline__ uint32_t fx0(Pt p) const { return uint32_t(!(p.x >= cx0)) << 0; }
  __device__ __forceinline__ uint32_t fx1(Pt p) const { return uint32_t(!(p.x <= cx1)) << 2; }
  __device__ __forceinline__ uint32_t fy0(Pt p) const { return uint32_t(!(p.y >= cy0)) << 1; }
  __device__ __forceinline__ uint32_t fy1(Pt p) const { return uint32_t(!(p.y <= cy1)) << 3; }
  __device__ __forceinline__ uint32_t fx(Pt p) const { return fx0(p) | fx1(p); }
  __device__ __forceinline__ uint32_t fy(Pt p) const { return fy0(p) | fy1(p); }
  __device__ __forceinline__ uint32_t fxy(Pt p) const { return fx(p) | fy(p); }

  // polylines: descending ones run top-down, ascending ones are collected bottom-up.
  __device__ __forceinline__ void desc_open(int x, int y, uint32_t sign) { px = x; py = y; psign = sign; pasc = false; }
  __device__ __forceinline__ void asc_open(int x, int y) { px = x; py = y; psign = 1; pasc = true; }
  __device__ __forceinline__ void add(int x, int y) {
    if (pasc) sink.emit(x, y, px, py, 1u);
    else sink.emit(px, py, x, y, psign);
    px = x; py = y;
  }

  __device__ void add_line_segment(double x0, double y0, double x1, double y1) {
    int a = trunc_i(x0), b = trunc_i(y0), c = trunc_i(x1), d = trunc_i(y1);
    if (b == d) return;
    if (b < d) sink.emit(a, b, c, d, 0u);
    else sink.emit(c, d, a, b, 1u);
  }

  __device__ void emit_left() {
    int a = trunc_i(acc_x0_y0), b = trunc_i(acc_x0_y1);
    if (a == b) return;
    sink.emit(icx0, min(a, b), icx0, max(a, b), uint32_t(a > b));
  }
  __device__ void emit_right() {
    int a = trunc_i(acc_x1_y0), b = trunc_i(acc_x1_y1);
    if (a == b) return;
    sink.emit(icx1, min(a, b), icx1, max(a, b), uint32_t(a > b));
  }
  __device__ void acc_left(double y0, double y1) {
    if (acc_x0_y1 == y0) { acc_x0_y1 = y1; return; }
    emit_left();
    acc_x0_y0 = y0; acc_x0_y1 = y1;
  }
  __device__ void acc_right(double y0, double y1) {
    if (acc_x1_y1 == y0) { acc_x1_y1 = y1; return; }
    emit_right();
    acc_x1_y0 = y0; acc_x1_y1 = y1;
  }
  __device__ __forceinline__ void acc_left_s(double y0, double y1, uint32_t s) { if (s) acc_left(y1, y0); else acc_left(y0, y1); }
  __device__ __forceinline__ void acc_right_s(double y0, double y1, uint32_t s) { if (s) acc_right(y1, y0); else acc_right(y0, y1); }
  __device__ void done() { emit_left(); emit_right(); }
};

// Vertex source (EdgeSourcePoly / EdgeSourcePath, edgebuilder_p.h:102-270).
struct Src {
  const double* xy;
  const uint8_t* cmd;   // nullptr for polygons
  int i, n;
  bool affine;
  double m00, m01, m10, m11, m20, m21;

  __device__ __forceinline__ Pt tf(int k) const {
    double x = xy[2 * k], y = xy[2 * k + 1];
    if (affine) return Pt{x * m00 + y * m10 + m20, x * m01 + y * m11 + m21};
    return Pt{x * m00 + m20, y * m11 + m21};
  }
  __device__ bool begin(Pt& p) {
    if (!cmd) {
      if (i == n) return false;
      p = tf(i); i++;
      return true;
    }
    for (;;) {
      if (i == n) return false;
      uint8_t c = cmd[i]; i++;
      if (c != 0) continue;
      p = tf(i - 1);
      return true;
    }
  }
  __device__ __forceinline__ bool is_close() const { return cmd && i != n && cmd[i] == 5; }
  __device__ __forceinline__ bool is_line() const { return cmd ? (i != n && cmd[i] == 1) : (i != n); }
  __device__ __forceinline__ bool is_quad() const { return cmd && i <= n - 2 && cmd[i] == 2; }
  __device__ __forceinline__ bool is_conic() const { return cmd && i < n - 2 && cmd[i] == 3; }
  __device__ __forceinline__ bool is_cubic() const { return cmd && i < n - 2 && cmd[i] == 4; }
  __device__ __forceinline__ bool next_line(Pt& p) { if (!is_line()) return false; p = tf(i); i++; return true; }
};

// ---------------------------------------------------------------------------------------------
// line_to (edgebuilder_p.h:1123-1607)
// ---------------------------------------------------------------------------------------------

__device__ int line_to(Builder& eb, Src& src, Pt& A, uint32_t& AF, Pt b) {
  Pt p, d;
  uint32_t b_flags = 0;
  int x0, y0, x1, y1;
  double borY0 = 0.0, borY1;

  do {
    if (!AF) {
      b_flags = eb.fxy(b);
      if (!b_flags) {
        x0 = trunc_i(A.x); y0 = trunc_i(A.y); x1 = trunc_i(b.x); y1 = trunc_i(b.y);
        for (;;) {
          if (y0 < y1) {
DescBegin:
            eb.desc_open(x0, y0, 0u);
            eb.add(x1, y1);
            for (;;) {
DescLoopA:
              if (!src.next_line(A)) { A = b; return 0; }
              b_flags = eb.fxy(A);
              if (b_flags) { Pt t = A; A = b; b = t; goto BeforeClipEnd; }
              x0 = trunc_i(A.x); y0 = trunc_i(A.y);
              if (y0 < y1) { eb.asc_open(x1, y1); eb.add(x0, y0); goto AscLoopB; }
              eb.add(x0, y0);
DescLoopB:
              if (!src.next_line(b)) return 0;
              b_flags = eb.fxy(b);
              if (b_flags) goto BeforeClipEnd;
              x1 = trunc_i(b.x); y1 = trunc_i(b.y);
              if (y1 < y0) { eb.asc_open(x0, y0); eb.add(x1, y1); goto AscLoopA; }
              eb.add(x1, y1);
            }
          }
          else if (y0 > y1) {
AscBegin:
            eb.asc_open(x0, y0);
            eb.add(x1, y1);
            for (;;) {
AscLoopA:
              if (!src.next_line(A)) { A = b; return 0; }
              b_flags = eb.fxy(A);
              if (b_flags) { Pt t = A; A = b; b = t; goto BeforeClipEnd; }
              x0 = trunc_i(A.x); y0 = trunc_i(A.y);
              if (y0 > y1) { eb.desc_open(x1, y1, 0u); eb.add(x0, y0); goto DescLoopB; }
              eb.add(x0, y0);
AscLoopB:
              if (!src.next_line(b)) return 0;
              b_flags = eb.fxy(b);
              if (b_flags) goto BeforeClipEnd;
              x1 = trunc_i(b.x); y1 = trunc_i(b.y);
              if (y1 > y0) { eb.desc_open(x0, y0, 0u); eb.add(x1, y1); goto DescLoopA; }
              eb.add(x1, y1);
            }
          }
          else {
            A = b;
            if (!src.next_line(b)) return 0;
            b_flags = eb.fxy(b);
            if (b_flags) break;
            x0 = x1; y0 = y1;
            x1 = trunc_i(b.x); y1 = trunc_i(b.y);
          }
        }
      }
BeforeClipEnd:
      p = A;
      d = Pt{b.x - A.x, b.y - A.y};
    }
    else {
RestartClip:
      if (AF & CF_Y0) {
        for (;;) {
          if (eb.cy0 < b.y) break;
          A = b;
          if (!src.next_line(b)) { AF = eb.fx(A) | eb.fy0(A); return 0; }
        }
        AF = eb.fx(A) | eb.fy0(A);
        b_flags = eb.fx(b) | eb.fy1(b);
        borY0 = eb.cy0;
        uint32_t common = AF & b_flags;
        if (common) {
          borY1 = dmin(eb.cy1, b.y);
          if (common & CF_X0) eb.acc_left(borY0, borY1); else eb.acc_right(borY0, borY1);
          A = b; AF = b_flags;
          continue;
        }
      }
      else if (AF & CF_Y1) {
        for (;;) {
          if (eb.cy1 > b.y) break;
          A = b;
          if (!src.next_line(b)) { AF = eb.fx(A) | eb.fy1(A); return 0; }
        }
        AF = eb.fx(A) | eb.fy1(A);
        b_flags = eb.fx(b) | eb.fy0(b);
        borY0 = eb.cy1;
        uint32_t common = AF & b_flags;
        if (common) {
          borY1 = dmax(eb.cy0, b.y);
          if (common & CF_X0) eb.acc_left(borY0, borY1); else eb.acc_right(borY0, borY1);
          A = b; AF = b_flags;
          continue;
        }
      }
      else if (AF & CF_X0) {
        borY0 = dclamp(A.y, eb.cy0, eb.cy1);
        for (;;) {
          if (eb.cx0 < b.x) break;
          A = b;
          if (!src.next_line(b)) {
            AF = eb.fy(A) | eb.fx0(A);
            borY1 = dclamp(A.y, eb.cy0, eb.cy1);
            if (borY0 != borY1) eb.acc_left(borY0, borY1);
            return 0;
          }
        }
        borY1 = dclamp(A.y, eb.cy0, eb.cy1);
        if (borY0 != borY1) eb.acc_left(borY0, borY1);
        AF = eb.fx0(A) | eb.fy(A);
        b_flags = eb.fx1(b) | eb.fy(b);
        if (AF & b_flags) goto RestartClip;
        borY0 = borY1;
      }
      else {
        borY0 = dclamp(A.y, eb.cy0, eb.cy1);
        for (;;) {
          if (eb.cx1 > b.x) break;
          A = b;
          if (!src.next_line(b)) {
            AF = eb.fy(A) | eb.fx1(A);
            borY1 = dclamp(A.y, eb.cy0, eb.cy1);
            if (borY0 != borY1) eb.acc_right(borY0, borY1);
            return 0;
          }
        }
        borY1 = dclamp(A.y, eb.cy0, eb.cy1);
        if (borY0 != borY1) eb.acc_right(borY0, borY1);
        AF = eb.fx1(A) | eb.fy(A);
        b_flags = eb.fx0(b) | eb.fy(b);
        if (AF & b_flags) goto RestartClip;
        borY0 = borY1;
      }

      d = Pt{b.x - A.x, b.y - A.y};
      p = Pt{eb.cx1, eb.cy1};
      switch (AF) {
        case 0: p = A; break;
        case CF_X0 | CF_Y0: p.x = eb.cx0; /* fallthrough */
        case CF_X1 | CF_Y0:
          p.y = A.y + (p.x - A.x) * d.y / d.x;
          AF = eb.fy(p);
          if (p.y >= eb.cy0) break;
          /* fallthrough */
        case CF_Y0:
          p.y = eb.cy0;
          p.x = A.x + (p.y - A.y) * d.x / d.y;
          AF = eb.fx(p);
          break;
        case CF_X0 | CF_Y1: p.x = eb.cx0; /* fallthrough */
        case CF_X1 | CF_Y1:
          p.y = A.y + (p.x - A.x) * d.y / d.x;
          AF = eb.fy(p);
          if (p.y <= eb.cy1) break;
          /* fallthrough */
        case CF_Y1:
          p.y = eb.cy1;
          p.x = A.x + (p.y - A.y) * d.x / d.y;
          AF = eb.fx(p);
          break;
        case CF_X0: p.x = eb.cx0; /* fallthrough */
        case CF_X1:
          p.y = A.y + (p.x - A.x) * d.y / d.x;
          AF = eb.fy(p);
          break;
        default:
          return 1;   // NaN: BL_ERROR_INVALID_GEOMETRY
      }

      if (AF) {
        borY1 = dclamp(b.y, eb.cy0, eb.cy1);
        if (p.x <= eb.cx0) eb.acc_left(borY0, borY1);
        else if (p.x >= eb.cx1) eb.acc_right(borY0, borY1);
        A = b; AF = b_flags;
        continue;
      }

      borY1 = dclamp(p.y, eb.cy0, eb.cy1);
      if (borY0 != borY1) {
        if (p.x <= eb.cx0) eb.acc_left(borY0, borY1);
        else eb.acc_right(borY0, borY1);
      }

      if (!b_flags) {
        A = b;
        AF = 0;
        x0 = trunc_i(p.x); y0 = trunc_i(p.y); x1 = trunc_i(b.x); y1 = trunc_i(b.y);
        if (y0 == y1) continue;
        if (y0 < y1) goto DescBegin;
        else goto AscBegin;
      }
    }

    {
      Pt q{eb.cx1, eb.cy1};
      switch (b_flags) {
        case CF_X0 | CF_Y0: q.x = eb.cx0; /* fallthrough */
        case CF_X1 | CF_Y0:
          q.y = A.y + (q.x - A.x) * d.y / d.x;
          if (q.y >= eb.cy0) break;
          /* fallthrough */
        case CF_Y0:
          q.y = eb.cy0;
          q.x = A.x + (q.y - A.y) * d.x / d.y;
          break;
        case CF_X0 | CF_Y1: q.x = eb.cx0; /* fallthrough */
        case CF_X1 | CF_Y1:
          q.y = A.y + (q.x - A.x) * d.y / d.x;
          if (q.y <= eb.cy1) break;
          /* fallthrough */
        case CF_Y1:
          q.y = eb.cy1;
          q.x = A.x + (q.y - A.y) * d.x / d.y;
          break;
        case CF_X0: q.x = eb.cx0; /* fallthrough */
        case CF_X1:
          q.y = A.y + (q.x - A.x) * d.y / d.x;
          break;
        default:
          return 1;
      }
      eb.add_line_segment(p.x, p.y, q.x, q.y);
      double cby = dclamp(b.y, eb.cy0, eb.cy1);
      if (q.y != cby) {
        if (q.x == eb.cx0) eb.acc_left(q.y, cby);
        else eb.acc_right(q.y, cby);
      }
    }

    A = b;
    AF = b_flags;
  } while (src.next_line(b));
  return 0;
}

// ---------------------------------------------------------------------------------------------
// Curve splitting (bezier_p.h) and monotonic flattening (edgebuilder_p.h:426-768, :2029-2445)
// ---------------------------------------------------------------------------------------------

__device__ __forceinline__ double cross(Pt a, Pt b) { return a.x * b.y - a.y * b.x; }
__device__ __forceinline__ double mag_sq(Pt v) { return v.x * v.x + v.y * v.y; }

__device__ int quad_roots(double* dst, double a, double b, double c, double t_min, double t_max) {
  double d = dmax(b * b - 4.0 * a * c, 0.0);
  double s = sqrt(d);
  double q = -0.5 * (b + copysign(s, b));
  double t0 = q / a;
  double t1 = c / q;
  double x0 = dmin(t0, t1);
  double x1 = dmax(t1, t0);
  dst[0] = x0;
  int n = int((x0 >= t_min) & (x0 <= t_max));
  dst[n] = x1;
  n += int((x1 > x0) & (x1 >= t_min) & (x1 <= t_max));
  return n;
}

__device__ int split_quad(Pt* c) {
  Pt c0 = c[0], c1 = c[1], c2 = c[2];
  double ex = (c0.x - c1.x) / (c0.x - c1.x * 2.0 + c2.x);
  double ey = (c0.y - c1.y) / (c0.y - c1.y * 2.0 + c2.y);
  double t0 = dmin(ex, ey), t1 = dmax(ex, ey);
  double ts[3];
  int n = 0;
  ts[n] = t0; n += int((t0 > 0.0) & (t0 < 1.0));
  ts[n] = t1; n += int((t1 > dmax(t0, 0.0)) & (t1 < 1.0));
  if (!n) return 0;
  ts[n++] = 1.0;
  Pt v1{c1.x - c0.x, c1.y - c0.y}, v2{c2.x - c1.x, c2.y - c1.y};
  Pt qa{v2.x - v1.x, v2.y - v1.y}, qb{v1.x + v1.x, v1.y + v1.y}, qc = c0;
  Pt last = c2;
  double t_cut = 0.0;
  Pt* out = c;
  int i = 0;
  do {
    double t = ts[i];
    double dt = (t - t_cut) * 0.5;
    Pt cp{(qa.x * (t * 2.0) + qb.x) * dt, (qa.y * (t * 2.0) + qb.y) * dt};
    Pt tp{(qa.x * t + qb.x) * t + qc.x, (qa.y * t + qb.y) * t + qc.y};
    if (++i == n) tp = last;
    out[1] = Pt{tp.x - cp.x, tp.y - cp.y};
    out[2] = tp;
    out += 2;
    t_cut = t;
  } while (i != n);
  return int(out - c);
}

__device__ int split_cubic(Pt* c) {
  Pt c0 = c[0], c1 = c[1], c2 = c[2], c3 = c[3];
  Pt v1{c1.x - c0.x, c1.y - c0.y}, v2{c2.x - c1.x, c2.y - c1.y}, v3{c3.x - c2.x, c3.y - c2.y};
  Pt ca{v3.x - v2.x - v2.x + v1.x, v3.y - v2.y - v2.y + v1.y};
  Pt cb{3.0 * (v2.x - v1.x), 3.0 * (v2.y - v1.y)};
  Pt cc{3.0 * v1.x, 3.0 * v1.y};
  Pt cd = c0;
  double ts[8];
  int n = 0;
  double q0 = cross(cb, ca), q1 = cross(cc, ca), q2 = cross(cc, cb);
  double t_cusp = (q1 / q0) * -0.5;
  ts[n] = t_cusp; n += int((t_cusp > 0.0) & (t_cusp < 1.0));
  const double kAfter0 = 1e-40, kBefore1 = 0.999999999999999889;
  n += quad_roots(ts + n, q0 * 6.0, q1 * 6.0, q2 * 2.0, kAfter0, kBefore1);
  Pt da{3.0 * (v3.x - v2.x - v2.x + v1.x), 3.0 * (v3.y - v2.y - v2.y + v1.y)};
  Pt db{6.0 * (v2.x - v1.x), 6.0 * (v2.y - v1.y)};
  Pt dc{3.0 * v1.x, 3.0 * v1.y};
  n += quad_roots(ts + n, da.x, db.x, dc.x, kAfter0, kBefore1);
  n += quad_roots(ts + n, da.y, db.y, dc.y, kAfter0, kBefore1);
  if (!n) return 0;
  for (int i = 1; i < n; i++) {
    double v = ts[i];
    int j = i;
    while (j > 0 && v < ts[j - 1]) { ts[j] = ts[j - 1]; j--; }
    ts[j] = v;
  }
  ts[n++] = 1.0;
  Pt last = c3;
  Pt* out = c;
  int i = 0;
  double t_cut = 0.0;
  do {
    double t = ts[i++];
    if (t == t_cut) continue;
    const double k1Div3 = 1.0 / 3.0;
    double dt = (t - t_cut) * k1Div3;
    Pt tp{((ca.x * t + cb.x) * t + cc.x) * t + cd.x, ((ca.y * t + cb.y) * t + cc.y) * t + cd.y};
    if (i == n) tp = last;
    Pt cp1{((ca.x * (t_cut * 3.0) + cb.x * 2.0) * t_cut + cc.x) * dt, ((ca.y * (t_cut * 3.0) + cb.y * 2.0) * t_cut + cc.y) * dt};
    Pt cp2{((ca.x * (t * 3.0) + cb.x * 2.0) * t + cc.x) * dt, ((ca.y * (t * 3.0) + cb.y * 2.0) * t + cc.y) * dt};
    out[1] = Pt{out[0].x + cp1.x, out[0].y + cp1.y};
    out[2] = Pt{tp.x - cp2.x, tp.y - cp2.y};
    out[3] = tp;
    out += 3;
    t_cut = t;
  } while (i != n);
  return int(out - c);
}

struct Step { double value, limit; Pt p01, p12, p23, p012, p123, p0123; };

__device__ __forceinline__ Pt mid(Pt a, Pt b) { return Pt{(a.x + b.x) * 0.5, (a.y + b.y) * 0.5}; }

// v * 0.5 by decrementing the exponent field: exact, and so equal to the multiply, for biased
// exponents 2..0x7FE. `ok` is cleared for the other values (zero, subnormal, the smallest normal
// exponent, inf, NaN), for which the caller falls back to the multiply. This keeps the halvings of
// the subdivision off the FP64 pipe, which bounds the flattening kernels.
__device__ __forceinline__ double half_exp(double v, bool& ok) {
  const int hi = __double2hiint(v), lo = __double2loint(v);
  ok &= ((unsigned(hi) >> 20) & 0x7FFu) - 2u < 0x7FDu;
  return __hiloint2double(hi - 0x100000, lo);
}
__device__ __forceinline__ Pt mid_exp(Pt a, Pt b, bool& ok) { return Pt{half_exp(a.x + b.x, ok), half_exp(a.y + b.y, ok)}; }

// Subdivision stack storage. An entry is the right half of a split still to be flattened, without
// its first point: that is the split point, which is also the last point of everything flattened
// between the push and the pop (the left half's subtree ends there), so the pop takes it from the
// current curve. 32 entries, as the reference's stack.
constexpr int kStackLevels = 32;

template<int DEG>
struct LocalStack {
  Pt e[kStackLevels][DEG];
  // push(lvl, v): entry `lvl` (the stack held lvl entries); pop(lvl, v): takes entry `lvl` (the
  // stack holds lvl entries afterwards).
  __device__ __forceinline__ void push(int lvl, const Pt* v) {
#pragma unroll
    for (int k = 0; k < DEG; k++) e[lvl][k] = v[k];
  }
  __device__ __forceinline__ void pop(int lvl, Pt* v) {
#pragma unroll
    for (int k = 0; k < DEG; k++) v[k] = e[lvl][k];
  }
};

// The same with the top entry held in registers: a pop returns it at once and reloads the entry
// under it, whose load then overlaps the flattening of the popped part instead of stalling it.
template<int DEG>
struct CachedStack {
  Pt top[DEG];
  Pt e[kStackLevels][DEG];
  __device__ __forceinline__ void push(int lvl, const Pt* v) {
#pragma unroll
    for (int k = 0; k < DEG; k++) {
      if (lvl > 0) e[lvl - 1][k] = top[k];
      top[k] = v[k];
    }
  }
  __device__ __forceinline__ void pop(int lvl, Pt* v) {
#pragma unroll
    for (int k = 0; k < DEG; k++) {
      v[k] = top[k];
      if (lvl > 0) top[k] = e[lvl - 1][k];
    }
  }
};

struct NoStack {};

// Monotonic curve with an explicit subdivision stack (FlattenMonoQuad / FlattenMonoCubic).
template<int DEG, class S = LocalStack<DEG>>
struct Mono {
  double tol_sq;
  Pt p[DEG + 1];
  S stack;
  int sp;                      // entries on the stack

  __device__ __forceinline__ void begin(const Pt* src, uint32_t sign) {
    sp = 0;
#pragma unroll
    for (int i = 0; i <= DEG; i++) p[i] = sign ? src[DEG - i] : src[i];
  }
  __device__ __forceinline__ Pt first() const { return p[0]; }
  __device__ __forceinline__ Pt last() const { return p[DEG]; }
  __device__ __forceinline__ bool can_pop() const { return sp != 0; }
  __device__ __forceinline__ bool can_push() const { return sp != kStackLevels; }
  __device__ __forceinline__ bool ltr() const { return p[0].x < p[DEG].x; }
  __device__ __forceinline__ void bound_ltr() {
#pragma unroll
    for (int i = 1; i < DEG; i++) { p[i].x = dclamp(p[i].x, p[0].x, p[DEG].x); p[i].y = dclamp(p[i].y, p[0].y, p[DEG].y); }
  }
  __device__ __forceinline__ void bound_rtl() {
#pragma unroll
    for (int i = 1; i < DEG; i++) { p[i].x = dclamp(p[i].x, p[DEG].x, p[0].x); p[i].y = dclamp(p[i].y, p[0].y, p[DEG].y); }
  }
  __device__ __forceinline__ bool is_flat(Step& s) const {
    if (DEG == 2) {
      Pt v1{p[1].x - p[0].x, p[1].y - p[0].y}, v2{p[2].x - p[0].x, p[2].y - p[0].y};
      double d = cross(v2, v1);
      double len_sq = mag_sq(v2);
      s.value = d * d;
      s.limit = tol_sq * len_sq;
    }
    else {
      Pt v{p[DEG].x - p[0].x, p[DEG].y - p[0].y};
      Pt a{p[1].x - p[0].x, p[1].y - p[0].y}, b{p[2].x - p[0].x, p[2].y - p[0].y};
      double c1 = cross(v, a), c2 = cross(v, b);
      double d1 = c1 * c1, d2 = c2 * c2;
      double len_sq = mag_sq(v);
      s.value = dmax(d1, d2);
      s.limit = tol_sq * len_sq;
    }
    return s.value <= s.limit;
  }
  __device__ __forceinline__ void split(Step& s) const {
    bool ok = true;
    if (DEG == 2) {
      s.p01 = mid_exp(p[0], p[1], ok); s.p12 = mid_exp(p[1], p[2], ok); s.p012 = mid_exp(s.p01, s.p12, ok);
      if (!ok) { s.p01 = mid(p[0], p[1]); s.p12 = mid(p[1], p[2]); s.p012 = mid(s.p01, s.p12); }
    }
    else {
      s.p01 = mid_exp(p[0], p[1], ok); s.p12 = mid_exp(p[1], p[2], ok); s.p23 = mid_exp(p[2], p[DEG], ok);
      s.p012 = mid_exp(s.p01, s.p12, ok); s.p123 = mid_exp(s.p12, s.p23, ok); s.p0123 = mid_exp(s.p012, s.p123, ok);
      if (!ok) {
        s.p01 = mid(p[0], p[1]); s.p12 = mid(p[1], p[2]); s.p23 = mid(p[2], p[DEG]);
        s.p012 = mid(s.p01, s.p12); s.p123 = mid(s.p12, s.p23); s.p0123 = mid(s.p012, s.p123);
      }
    }
  }
  __device__ __forceinline__ Pt step_mid(const Step& s) const { return DEG == 2 ? s.p012 : s.p0123; }
  __device__ __forceinline__ void push(const Step& s) {
    Pt v[DEG];
    if (DEG == 2) {
      v[0] = s.p12; v[DEG - 1] = p[2];
      stack.push(sp, v);
      p[1] = s.p01; p[2] = s.p012;
    }
    else {
      v[0] = s.p123; v[1] = s.p23; v[DEG - 1] = p[DEG];
      stack.push(sp, v);
      p[1] = s.p01; p[2] = s.p012; p[DEG] = s.p0123;
    }
    sp++;
  }
  __device__ __forceinline__ void discard_and_advance(const Step& s) {
    if (DEG == 2) { p[0] = s.p012; p[1] = s.p12; }
    else { p[0] = s.p0123; p[1] = s.p123; p[2] = s.p23; }
  }
  __device__ __forceinline__ void pop() {
    sp--;
    p[0] = p[DEG];
    stack.pop(sp, p + 1);
  }
};

// The subdivision of a monotonic piece inside the clip box as a tree. The loop flattener
// (flatten_safe) walks it depth first with a stack: a node that is not flat and finds the stack with
// room is split, its right half pushed and its left half taken next; any other node is a leaf, whose
// segment (first point to last point, truncated) is emitted, and the next node is popped. A leaf's
// segment depends only on the leaf, and a node's fate only on its points and on its level (the
// stack entries pending while it is processed: one more than its parent's for a left half, the
// parent's for a right half). Taking the nodes in another order, or on other lanes, therefore gives
// the same segments; only their order in the output differs, and nothing downstream depends on it.
template<int DEG>
struct TreeNode {
  Pt p[DEG + 1];
  int level;
};

// The tree's root: the piece oriented and bounded as start_piece does for a piece with no clip flags.
template<int DEG>
__device__ __forceinline__ TreeNode<DEG> tree_root(const Pt* pts, uint32_t& sign) {
  Mono<DEG, NoStack> mc;
  sign = pts[0].y > pts[DEG].y;
  mc.begin(pts, sign);
  if (mc.ltr()) mc.bound_ltr(); else mc.bound_rtl();
  TreeNode<DEG> n;
#pragma unroll
  for (int i = 0; i <= DEG; i++) n.p[i] = mc.p[i];
  n.level = 0;
  return n;
}

// Whether a monotonic piece is flattened exactly as by the safe loop, so that its tree can be
// walked in any order. True for a piece of a curve with no clip flags (`any` 0). For a piece of a
// clipped curve, oriented to increasing y (first point f, last point l), the clipping flattener
// (flatten_unsafe) runs its "inside" loop (LTR_AddLine / RTL_AddLine) with no clip ever firing
// when: its x extent exceeds the vertical-line limit (else it is emitted as one line); it starts
// at or below the clip box's top (else the top loop); it ends above its bottom (y_end is then l.y,
// and no leaf reaches cy1); and it stays between x0 and x1 (its subdivision points lie between f
// and l once the control points are bounded): then that loop is the safe loop, with the same
// desc_open, and finishes with nothing outside to accumulate.
__device__ __forceinline__ bool piece_flattens_safe(const Pt* pts, int deg, uint32_t any, const Builder& eb) {
  if (!any) return true;
  const bool sign = pts[0].y > pts[deg].y;
  const Pt f = sign ? pts[deg] : pts[0], l = sign ? pts[0] : pts[deg];
  if (!(fabs(f.x - l.x) > 0.00390625)) return false;
  if (!(f.y >= eb.cy0) || !(l.y < eb.cy1)) return false;
  return f.x < l.x ? (f.x >= eb.cx0 && l.x <= eb.cx1) : (f.x <= eb.cx1 && l.x >= eb.cx0);
}

// One node: true for a leaf, else its two halves (Mono::is_flat / split / push / pop).
template<int DEG>
__device__ __forceinline__ bool tree_step(const TreeNode<DEG>& n, double tol_sq, TreeNode<DEG>& left, TreeNode<DEG>& right) {
  Mono<DEG, NoStack> mc;
  mc.tol_sq = tol_sq;
#pragma unroll
  for (int i = 0; i <= DEG; i++) mc.p[i] = n.p[i];
  Step st;
  if (mc.is_flat(st) || n.level == kStackLevels) return true;
  mc.split(st);
  if (DEG == 2) {
    left.p[0] = n.p[0]; left.p[1] = st.p01; left.p[2] = st.p012;
    right.p[0] = st.p012; right.p[1] = st.p12; right.p[2] = n.p[2];
  }
  else {
    left.p[0] = n.p[0]; left.p[1] = st.p01; left.p[2] = st.p012; left.p[DEG] = st.p0123;
    right.p[0] = st.p0123; right.p[1] = st.p123; right.p[2] = st.p23; right.p[DEG] = n.p[DEG];
  }
  left.level = n.level + 1;
  right.level = n.level;
  return false;
}

__device__ __forceinline__ double dx_div_dy(Pt a, Pt b) { return (b.x - a.x) / (b.y - a.y); }
__device__ __forceinline__ double dy_div_dx(Pt a, Pt b) { return (b.y - a.y) / (b.x - a.x); }

template<int DEG, class M>
__device__ void flatten_safe(Builder& eb, M& mc, const Pt* src, uint32_t sign) {
  mc.begin(src, sign);
  if (mc.ltr()) mc.bound_ltr(); else mc.bound_rtl();
  eb.desc_open(trunc_i(mc.first().x), trunc_i(mc.first().y), sign);
  for (;;) {
    Step step;
    if (!mc.is_flat(step)) {
      if (mc.can_push()) { mc.split(step); mc.push(step); continue; }
    }
    eb.add(trunc_i(mc.last().x), trunc_i(mc.last().y));
    if (!mc.can_pop()) break;
    mc.pop();
  }
}

template<int DEG, class M>
__device__ void flatten_unsafe(Builder& eb, M& mc, const Pt* src, uint32_t sign) {
  mc.begin(src, sign);
  double y_start = mc.first().y;
  double y_end = dmin(mc.last().y, eb.cy1);
  if ((y_start >= y_end) | (y_end <= eb.cy0)) return;

  const double kDeltaLimit = 0.00390625;
  double x_delta = fabs(mc.first().x - mc.last().x);
  uint32_t out = 0;
  Step step;

  if (x_delta <= kDeltaLimit) {
    y_start = dmax(y_start, eb.cy0);
    double x_min = dmin(mc.first().x, mc.last().x);
    double x_max = dmax(mc.first().x, mc.last().x);
    if (x_max <= eb.cx0) eb.acc_left_s(y_start, y_end, sign);
    else if (x_min >= eb.cx1) eb.acc_right_s(y_start, y_end, sign);
    else {
      eb.desc_open(trunc_i(mc.first().x), trunc_i(y_start), sign);
      eb.add(trunc_i(mc.last().x), trunc_i(y_end));
    }
    return;
  }
  else if (mc.ltr()) {
    mc.bound_ltr();
    if (y_start < eb.cy0) {
      y_start = eb.cy0;
      for (;;) {
        out = (mc.first().x >= eb.cx1);
        if (out) break;
        if (!mc.is_flat(step)) {
          mc.split(step);
          if (mc.step_mid(step).y <= eb.cy0) { mc.discard_and_advance(step); continue; }
          if (mc.can_push()) { mc.push(step); continue; }
        }
        if (mc.last().y > eb.cy0) {
          out = mc.last().x < eb.cx0;
          if (out) goto LTR_BeforeX0_Pop;
          double xc = mc.first().x + (eb.cy0 - mc.first().y) * dx_div_dy(mc.first(), mc.last());
          if (xc <= eb.cx0) goto LTR_BeforeX0_Clip;
          out = (xc >= eb.cx1);
          if (out) break;
          eb.desc_open(trunc_i(xc), trunc_i(eb.cy0), sign);
          goto LTR_AddLine;
        }
        if (!mc.can_pop()) break;
        mc.pop();
      }
      out <<= 2;
    }
    else if (y_start < eb.cy1) {
      if (mc.first().x < eb.cx0) {
        for (;;) {
          out = (mc.first().y >= eb.cy1);
          if (out) break;
          if (!mc.is_flat(step)) {
            mc.split(step);
            if (mc.step_mid(step).x <= eb.cx0) { mc.discard_and_advance(step); continue; }
            if (mc.can_push()) { mc.push(step); continue; }
          }
          if (mc.last().x > eb.cx0) {
LTR_BeforeX0_Clip:
            {
              double yc = mc.first().y + (eb.cx0 - mc.first().x) * dy_div_dx(mc.first(), mc.last());
              out = (yc >= y_end);
              if (out) break;
              if (y_start < yc) eb.acc_left_s(y_start, yc, sign);
              eb.desc_open(trunc_i(eb.cx0), trunc_i(yc), sign);
              goto LTR_AddLine;
            }
          }
          out = (mc.last().y >= y_end);
          if (out) break;
LTR_BeforeX0_Pop:
          if (!mc.can_pop()) break;
          mc.pop();
        }
      }
      else if (mc.first().x < eb.cx1) {
        eb.desc_open(trunc_i(mc.first().x), trunc_i(mc.first().y), sign);
        for (;;) {
          if (!mc.is_flat(step)) {
            mc.split(step);
            if (mc.can_push()) { mc.push(step); continue; }
          }
LTR_AddLine:
          out = mc.last().x > eb.cx1;
          if (out) {
            double yc = mc.first().y + (eb.cx1 - mc.first().x) * dy_div_dx(mc.first(), mc.last());
            if (yc <= y_end) {
              y_start = yc;
              eb.add(trunc_i(eb.cx1), trunc_i(yc));
              break;
            }
          }
          out = mc.last().y >= eb.cy1;
          if (out) {
            double xc = dmin(mc.first().x + (eb.cy1 - mc.first().y) * dx_div_dy(mc.first(), mc.last()), eb.cx1);
            eb.add(trunc_i(xc), trunc_i(eb.cy1));
            out = 0;
            break;
          }
          eb.add(trunc_i(mc.last().x), trunc_i(mc.last().y));
          if (!mc.can_pop()) break;
          mc.pop();
        }
        out <<= 2;
      }
      else {
        out = CF_X1;
      }
    }
  }
  else {
    mc.bound_rtl();
    if (y_start < eb.cy0) {
      y_start = eb.cy0;
      for (;;) {
        out = (mc.first().x <= eb.cx0);
        if (out) break;
        if (!mc.is_flat(step)) {
          mc.split(step);
          if (mc.step_mid(step).y <= eb.cy0) { mc.discard_and_advance(step); continue; }
          if (mc.can_push()) { mc.push(step); continue; }
        }
        if (mc.last().y > eb.cy0) {
          out = mc.last().x > eb.cx1;
          if (out) goto RTL_AfterX1_Pop;
          double xc = mc.first().x + (eb.cy0 - mc.first().y) * dx_div_dy(mc.first(), mc.last());
          if (xc >= eb.cx1) goto RTL_AfterX1_Clip;
          out = (xc <= eb.cx0);
          if (out) break;
          eb.desc_open(trunc_i(xc), trunc_i(eb.cy0), sign);
          goto RTL_AddLine;
        }
        if (!mc.can_pop()) break;
        mc.pop();
      }
    }
    else if (y_start < eb.cy1) {
      if (mc.first().x > eb.cx1) {
        for (;;) {
          out = (mc.first().y >= eb.cy1);
          if (out) break;
          if (!mc.is_flat(step)) {
            mc.split(step);
            if (mc.step_mid(step).x >= eb.cx1) { mc.discard_and_advance(step); continue; }
            if (mc.can_push()) { mc.push(step); continue; }
          }
          if (mc.last().x < eb.cx1) {
RTL_AfterX1_Clip:
            {
              double yc = mc.first().y + (eb.cx1 - mc.first().x) * dy_div_dx(mc.first(), mc.last());
              out = (yc >= y_end);
              if (out) break;
              if (y_start < yc) eb.acc_right_s(y_start, yc, sign);
              eb.desc_open(trunc_i(eb.cx1), trunc_i(yc), sign);
              goto RTL_AddLine;
            }
          }
          out = (mc.last().y >= y_end);
          if (out) break;
RTL_AfterX1_Pop:
          if (!mc.can_pop()) break;
          mc.pop();
        }
        out <<= 2;
      }
      else if (mc.first().x > eb.cx0) {
        eb.desc_open(trunc_i(mc.first().x), trunc_i(mc.first().y), sign);
        for (;;) {
          if (!mc.is_flat(step)) {
            mc.split(step);
            if (mc.can_push()) { mc.push(step); continue; }
          }
RTL_AddLine:
          out = mc.last().x < eb.cx0;
          if (out) {
            double yc = mc.first().y + (eb.cx0 - mc.first().x) * dy_div_dx(mc.first(), mc.last());
            if (yc <= y_end) {
              y_start = yc;
              eb.add(trunc_i(eb.cx0), trunc_i(yc));
              break;
            }
          }
          out = mc.last().y >= eb.cy1;
          if (out) {
            double xc = dmax(mc.first().x + (eb.cy1 - mc.first().y) * dx_div_dy(mc.first(), mc.last()), eb.cx0);
            eb.add(trunc_i(xc), trunc_i(eb.cy1));
            out = 0;
            break;
          }
          eb.add(trunc_i(mc.last().x), trunc_i(mc.last().y));
          if (!mc.can_pop()) break;
          mc.pop();
        }
      }
      else {
        out = CF_X0;
      }
    }
  }

  if (out && y_start < y_end) {
    if (out & CF_X0) eb.acc_left_s(y_start, y_end, sign);
    else eb.acc_right_s(y_start, y_end, sign);
  }
}

// quad_to / cubic_to / conic_to (edgebuilder_p.h:1618-2022); DEG 2 with `conic` reads the conic
// record layout (control point, weight slot, end point) but flattens like a quad, as the
// reference does.
template<int DEG>
__device__ void curve_to(Builder& eb, Src& src, Pt& p0, uint32_t& p0_flags, bool conic) {
  Pt spline[DEG == 3 ? 25 : 7];
  auto next = [&](void) {
    if (DEG == 3) { spline[1] = src.tf(src.i); spline[2] = src.tf(src.i + 1); spline[3] = src.tf(src.i + 2); src.i += 3; }
    else if (conic) { spline[1] = src.tf(src.i); spline[2] = src.tf(src.i + 2); src.i += 2; }
    else { spline[1] = src.tf(src.i); spline[2] = src.tf(src.i + 1); src.i += 2; }
  };
  auto has_next = [&](void) -> bool {
    return DEG == 3 ? src.is_cubic() : (conic ? src.is_conic() : src.is_quad());
  };
  next();
  Mono<DEG> mc;
  mc.tol_sq = eb.tol_sq;

  for (;;) {
    uint32_t fl[DEG + 1];
    uint32_t common = p0_flags;
#pragma unroll
    for (int i = 1; i <= DEG; i++) { fl[i] = eb.fxy(spline[i]); common &= fl[i]; }

    if (common) {
      bool end = false;
      if (common & CF_Y0) {
        for (;;) {
          p0 = spline[DEG];
          end = !has_next();
          if (end) break;
          next();
          bool all = true;
#pragma unroll
          for (int i = 1; i <= DEG; i++) all &= (spline[i].y <= eb.cy0);
          if (!all) break;
        }
      }
      else if (common & CF_Y1) {
        for (;;) {
          p0 = spline[DEG];
          end = !has_next();
          if (end) break;
          next();
          bool all = true;
#pragma unroll
          for (int i = 1; i <= DEG; i++) all &= (spline[i].y >= eb.cy1);
          if (!all) break;
        }
      }
      else {
        double y0 = dclamp(p0.y, eb.cy0, eb.cy1);
        bool left = (common & CF_X0) != 0;
        for (;;) {
          p0 = spline[DEG];
          end = !has_next();
          if (end) break;
          next();
          bool all = true;
#pragma unroll
          for (int i = 1; i <= DEG; i++) all &= left ? (spline[i].x <= eb.cx0) : (spline[i].x >= eb.cx1);
          if (!all) break;
        }
        double y1 = dclamp(p0.y, eb.cy0, eb.cy1);
        if (left) eb.acc_left(y0, y1); else eb.acc_right(y0, y1);
      }
      p0_flags = eb.fxy(p0);
      if (end) return;
      continue;
    }

    spline[0] = p0;
    int nout = DEG == 3 ? split_cubic(spline) : split_quad(spline);
    if (nout == 0) nout = DEG;

    uint32_t any = p0_flags;
#pragma unroll
    for (int i = 1; i <= DEG; i++) any |= fl[i];

    for (int k = 0; k < nout; k += DEG) {
      const Pt* sp = spline + k;
      uint32_t sign = sp[0].y > sp[DEG].y;
      if (any) flatten_unsafe<DEG>(eb, mc, sp, sign);
      else flatten_safe<DEG>(eb, mc, sp, sign);
    }
    p0 = spline[nout];
    if (any) p0_flags = fl[DEG];

    if (!has_next()) return;
    next();
  }
}

// ---------------------------------------------------------------------------------------------
// One curve of an item, flattened one subdivision step per call (the lane-scheduled kernels call
// step() once per iteration of a warp-wide loop, so the FP64 flatness test and split of all lanes
// issue together whatever branch of the clipper each lane is in). The states are the loops of
// flatten_safe / flatten_unsafe above and step() runs one pass of the loop body; the jumps between
// the loops (goto in flatten_unsafe) become state changes taken within the same step. Every
// piece emits the same segments and accumulations as flatten_safe / flatten_unsafe.
// ---------------------------------------------------------------------------------------------

enum : int {
  kLsDone = 0,     // piece finished
  kLsSafe,         // flatten_safe loop
  kLsLTop,         // left-to-right, above the clip box
  kLsLLeft,        // left-to-right, left of the clip box (LTR_BeforeX0)
  kLsLIn,          // left-to-right, inside (LTR_AddLine)
  kLsRTop,         // right-to-left, above the clip box
  kLsRRight,       // right-to-left, right of the clip box (RTL_AfterX1)
  kLsRIn           // right-to-left, inside (RTL_AddLine)
};

template<int DEG, class S = LocalStack<DEG>>
struct LaneCurve {
  Mono<DEG, S> mc;
  Pt spline[DEG == 3 ? 25 : 7];
  int nout, piece, state;
  uint32_t any, sign, out;
  double y_start, y_end;

  // curve_to for a source holding exactly this one curve, up to the flattening: p0 (with its clip
  // flags) and spline[1..DEG] set by the caller. A curve entirely on one side of the clip box is
  // done here; otherwise its monotonic pieces are left in spline[0..nout] (`any`: the curve's clip
  // flags). Returns false when there is nothing to flatten.
  __device__ __forceinline__ bool prepare(Builder& eb, Pt p0, uint32_t p0_flags) {
    mc.tol_sq = eb.tol_sq;
    uint32_t common = p0_flags, fl_any = p0_flags;
#pragma unroll
    for (int i = 1; i <= DEG; i++) { const uint32_t fl = eb.fxy(spline[i]); common &= fl; fl_any |= fl; }
    if (common) {
      if (!(common & (CF_Y0 | CF_Y1))) {
        const double y0 = dclamp(p0.y, eb.cy0, eb.cy1), y1 = dclamp(spline[DEG].y, eb.cy0, eb.cy1);
        if (common & CF_X0) eb.acc_left(y0, y1); else eb.acc_right(y0, y1);
      }
      return false;
    }
    spline[0] = p0;
    nout = DEG == 3 ? split_cubic(spline) : split_quad(spline);
    if (nout == 0) nout = DEG;
    any = fl_any;
    return true;
  }

  // The whole curve: prepare, then the first piece with work.
  __device__ __forceinline__ bool begin_curve(Builder& eb, Pt p0, uint32_t p0_flags) {
    if (!prepare(eb, p0, p0_flags)) return false;
    piece = 0;
    return next_piece(eb, false);
  }

  // One monotonic piece prepared earlier (its DEG + 1 points and its curve's clip flags).
  __device__ __forceinline__ bool begin_piece(Builder& eb, const Pt* pts, uint32_t any_flags) {
    mc.tol_sq = eb.tol_sq;
#pragma unroll
    for (int i = 0; i <= DEG; i++) spline[i] = pts[i];
    nout = DEG;
    any = any_flags;
    piece = 0;
    return next_piece(eb, false);
  }

  // Starts the next piece with work (pieces that finish at their start are skipped). Returns
  // false when the curve is done.
  __device__ __forceinline__ bool next_piece(Builder& eb, bool advance) {
    if (advance) piece += DEG;
    for (; piece < nout; piece += DEG) {
      start_piece(eb);
      if (state != kLsDone) return true;
    }
    return false;
  }

  __device__ __forceinline__ void finish(Builder& eb) {
    if (out && y_start < y_end) {
      if (out & CF_X0) eb.acc_left_s(y_start, y_end, sign);
      else eb.acc_right_s(y_start, y_end, sign);
    }
    state = kLsDone;
  }
  // Leaving a loop: the left-to-right top and inside loops and the right-to-left right loop
  // shift `out` (1 -> CF_X1), the others leave it (1 = CF_X0).
  __device__ __forceinline__ void exit_loop(Builder& eb, bool shift) {
    if (shift) out <<= 2;
    finish(eb);
  }

  __device__ __forceinline__ void start_piece(Builder& eb) {
    const Pt* sp = spline + piece;
    sign = sp[0].y > sp[DEG].y;
    mc.begin(sp, sign);
    if (!any) {
      if (mc.ltr()) mc.bound_ltr(); else mc.bound_rtl();
      eb.desc_open(trunc_i(mc.first().x), trunc_i(mc.first().y), sign);
      state = kLsSafe;
      return;
    }
    state = kLsDone;
    out = 0;
    y_start = mc.first().y;
    y_end = dmin(mc.last().y, eb.cy1);
    if ((y_start >= y_end) | (y_end <= eb.cy0)) return;
    const double kDeltaLimit = 0.00390625;
    const double x_delta = fabs(mc.first().x - mc.last().x);
    if (x_delta <= kDeltaLimit) {
      y_start = dmax(y_start, eb.cy0);
      const double x_min = dmin(mc.first().x, mc.last().x), x_max = dmax(mc.first().x, mc.last().x);
      if (x_max <= eb.cx0) eb.acc_left_s(y_start, y_end, sign);
      else if (x_min >= eb.cx1) eb.acc_right_s(y_start, y_end, sign);
      else {
        eb.desc_open(trunc_i(mc.first().x), trunc_i(y_start), sign);
        eb.add(trunc_i(mc.last().x), trunc_i(y_end));
      }
      return;
    }
    if (mc.ltr()) {
      mc.bound_ltr();
      if (y_start < eb.cy0) { y_start = eb.cy0; state = kLsLTop; }
      else if (y_start < eb.cy1) {
        if (mc.first().x < eb.cx0) state = kLsLLeft;
        else if (mc.first().x < eb.cx1) { eb.desc_open(trunc_i(mc.first().x), trunc_i(mc.first().y), sign); state = kLsLIn; }
        else { out = CF_X1; finish(eb); }
      }
    }
    else {
      mc.bound_rtl();
      if (y_start < eb.cy0) { y_start = eb.cy0; state = kLsRTop; }
      else if (y_start < eb.cy1) {
        if (mc.first().x > eb.cx1) state = kLsRRight;
        else if (mc.first().x > eb.cx0) { eb.desc_open(trunc_i(mc.first().x), trunc_i(mc.first().y), sign); state = kLsRIn; }
        else { out = CF_X0; finish(eb); }
      }
    }
  }

  // One pass of the current loop's body.
  __device__ __forceinline__ void step(Builder& eb) {
    switch (state) {
      case kLsLTop: out = mc.first().x >= eb.cx1; if (out) { exit_loop(eb, true); return; } break;
      case kLsLLeft: out = mc.first().y >= eb.cy1; if (out) { exit_loop(eb, false); return; } break;
      case kLsRTop: out = mc.first().x <= eb.cx0; if (out) { exit_loop(eb, false); return; } break;
      case kLsRRight: out = mc.first().y >= eb.cy1; if (out) { exit_loop(eb, true); return; } break;
      default: break;
    }
    Step st;
    if (!mc.is_flat(st)) {
      mc.split(st);
      const Pt m = mc.step_mid(st);
      const bool discard = ((state == kLsLTop) | (state == kLsRTop)) ? (m.y <= eb.cy0)
                         : state == kLsLLeft ? (m.x <= eb.cx0)
                         : state == kLsRRight ? (m.x >= eb.cx1) : false;
      if (discard) { mc.discard_and_advance(st); return; }
      if (mc.can_push()) { mc.push(st); return; }
    }
    leaf(eb);
  }

  __device__ __forceinline__ void leaf(Builder& eb) {
    const Pt a = mc.first(), b = mc.last();
    switch (state) {
      case kLsSafe:
        eb.add(trunc_i(b.x), trunc_i(b.y));
        if (!mc.can_pop()) { state = kLsDone; return; }
        mc.pop();
        return;
      case kLsLTop:
        if (b.y > eb.cy0) {
          out = b.x < eb.cx0;
          if (out) { l_left_pop(eb); return; }
          const double xc = a.x + (eb.cy0 - a.y) * dx_div_dy(a, b);
          if (xc <= eb.cx0) { l_left_clip(eb); return; }
          out = xc >= eb.cx1;
          if (out) { exit_loop(eb, true); return; }
          eb.desc_open(trunc_i(xc), trunc_i(eb.cy0), sign);
          l_add_line(eb);
          return;
        }
        if (!mc.can_pop()) { exit_loop(eb, true); return; }
        mc.pop();
        return;
      case kLsLLeft:
        if (b.x > eb.cx0) { l_left_clip(eb); return; }
        out = b.y >= y_end;
        if (out) { exit_loop(eb, false); return; }
        l_left_pop(eb);
        return;
      case kLsLIn:
        l_add_line(eb);
        return;
      case kLsRTop:
        if (b.y > eb.cy0) {
          out = b.x > eb.cx1;
          if (out) { r_right_pop(eb); return; }
          const double xc = a.x + (eb.cy0 - a.y) * dx_div_dy(a, b);
          if (xc >= eb.cx1) { r_right_clip(eb); return; }
          out = xc <= eb.cx0;
          if (out) { exit_loop(eb, false); return; }
          eb.desc_open(trunc_i(xc), trunc_i(eb.cy0), sign);
          r_add_line(eb);
          return;
        }
        if (!mc.can_pop()) { exit_loop(eb, false); return; }
        mc.pop();
        return;
      case kLsRRight:
        if (b.x < eb.cx1) { r_right_clip(eb); return; }
        out = b.y >= y_end;
        if (out) { exit_loop(eb, true); return; }
        r_right_pop(eb);
        return;
      case kLsRIn:
        r_add_line(eb);
        return;
      default:
        return;
    }
  }

  __device__ __forceinline__ void l_left_pop(Builder& eb) {           // LTR_BeforeX0_Pop
    state = kLsLLeft;
    if (!mc.can_pop()) { exit_loop(eb, false); return; }
    mc.pop();
  }
  __device__ __forceinline__ void l_left_clip(Builder& eb) {          // LTR_BeforeX0_Clip
    state = kLsLLeft;
    const Pt a = mc.first(), b = mc.last();
    const double yc = a.y + (eb.cx0 - a.x) * dy_div_dx(a, b);
    out = yc >= y_end;
    if (out) { exit_loop(eb, false); return; }
    if (y_start < yc) eb.acc_left_s(y_start, yc, sign);
    eb.desc_open(trunc_i(eb.cx0), trunc_i(yc), sign);
    l_add_line(eb);
  }
  __device__ __forceinline__ void l_add_line(Builder& eb) {           // LTR_AddLine
    state = kLsLIn;
    const Pt a = mc.first(), b = mc.last();
    out = b.x > eb.cx1;
    if (out) {
      const double yc = a.y + (eb.cx1 - a.x) * dy_div_dx(a, b);
      if (yc <= y_end) {
        y_start = yc;
        eb.add(trunc_i(eb.cx1), trunc_i(yc));
        exit_loop(eb, true);
        return;
      }
    }
    out = b.y >= eb.cy1;
    if (out) {
      const double xc = dmin(a.x + (eb.cy1 - a.y) * dx_div_dy(a, b), eb.cx1);
      eb.add(trunc_i(xc), trunc_i(eb.cy1));
      out = 0;
      exit_loop(eb, true);
      return;
    }
    eb.add(trunc_i(b.x), trunc_i(b.y));
    if (!mc.can_pop()) { exit_loop(eb, true); return; }
    mc.pop();
  }
  __device__ __forceinline__ void r_right_pop(Builder& eb) {          // RTL_AfterX1_Pop
    state = kLsRRight;
    if (!mc.can_pop()) { exit_loop(eb, true); return; }
    mc.pop();
  }
  __device__ __forceinline__ void r_right_clip(Builder& eb) {         // RTL_AfterX1_Clip
    state = kLsRRight;
    const Pt a = mc.first(), b = mc.last();
    const double yc = a.y + (eb.cx1 - a.x) * dy_div_dx(a, b);
    out = yc >= y_end;
    if (out) { exit_loop(eb, true); return; }
    if (y_start < yc) eb.acc_right_s(y_start, yc, sign);
    eb.desc_open(trunc_i(eb.cx1), trunc_i(yc), sign);
    r_add_line(eb);
  }
  __device__ __forceinline__ void r_add_line(Builder& eb) {           // RTL_AddLine
    state = kLsRIn;
    const Pt a = mc.first(), b = mc.last();
    out = b.x < eb.cx0;
    if (out) {
      const double yc = a.y + (eb.cx0 - a.x) * dy_div_dx(a, b);
      if (yc <= y_end) {
        y_start = yc;
        eb.add(trunc_i(eb.cx0), trunc_i(yc));
        exit_loop(eb, false);
        return;
      }
    }
    out = b.y >= eb.cy1;
    if (out) {
      const double xc = dmax(a.x + (eb.cy1 - a.y) * dx_div_dy(a, b), eb.cx0);
      eb.add(trunc_i(xc), trunc_i(eb.cy1));
      out = 0;
      exit_loop(eb, false);
      return;
    }
    eb.add(trunc_i(b.x), trunc_i(b.y));
    if (!mc.can_pop()) { exit_loop(eb, false); return; }
    mc.pop();
  }
};

// add_from_source (edgebuilder_p.h:1032-1070) for a closed fill. Returns 0 or 1 (invalid).
__device__ int build(Builder& eb, Src& src) {
  Pt a;
  uint32_t a_flags;
  while (src.begin(a)) {
    Pt start = a, b;
    bool done = false;
    a_flags = eb.fxy(a);
    for (;;) {
      if (src.is_line()) {
        b = src.tf(src.i); src.i++;
LineTo:
        if (line_to(eb, src, a, a_flags, b)) return 1;
        if (done) break;
      }
      else if (src.is_quad()) curve_to<2>(eb, src, a, a_flags, false);
      else if (src.is_cubic()) curve_to<3>(eb, src, a, a_flags, false);
      else if (src.is_conic()) curve_to<2>(eb, src, a, a_flags, true);
      else {
        b = start;
        done = true;
        goto LineTo;
      }
    }
  }
  eb.done();
  return 0;
}

}  // namespace eb
}  // namespace blgpu
