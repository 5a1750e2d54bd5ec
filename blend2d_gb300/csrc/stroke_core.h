// The path stroker, shared by the device (stroke_count_kernel / stroke_emit_kernel, one thread
// per figure) and the host (blgpu_stroke_outline_d). Restates bl::PathInternal::PathStroker
// (blend2d/core/pathstroke.cpp:126-971) and the Bezier helpers it uses
// (blend2d/geometry/bezier_p.h, blend2d/geometry/commons_p.h) operation by operation in double
// precision without FMA contraction (device code is built with -fmad=false, host code with
// -ffp-contract=off), so every expression keeps the reference's operand order.
//
// The reference writes each side of the outline into a growable path and patches vertices it has
// just written. Here a side keeps only its last vertices in a small window (the stroker never
// looks back further than a few vertices, plus the figure's first two) and hands every vertex
// that can no longer change to a sink: a counter in the first pass, the outline buffer in the
// second. So a thread strokes a figure of any length in constant memory.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define SK_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#define SK_HD inline
#endif

namespace blgpu {
namespace sk {

enum : uint8_t { kMove = 0, kOn = 1, kQuad = 2, kCubic = 4, kClose = 5 };
enum : uint32_t { kJoinMiterClip = 0, kJoinMiterBevel = 1, kJoinMiterRound = 2, kJoinBevel = 3, kJoinRound = 4 };
enum : uint32_t { kCapButt = 0, kCapSquare = 1, kCapRound = 2, kCapRoundRev = 3, kCapTriangle = 4, kCapTriangleRev = 5 };

// pathstroke.cpp:22-47, mathconst_p.h:52, path_p.h:89-98 (default approximation options)
constexpr double kMiterMinimum = 1e-10;
constexpr double kLengthEpsilonSq = 1e-10 * 1e-10;
constexpr double kCollinearityEpsilon = 1e-10;
constexpr double kCuspTThreshold = 1e-10;
constexpr double kDegenerateFlatness = 1e-6;
constexpr double kOffsetQuadEpsilonT = 1e-5;
constexpr double kKappa = 0.55228474983;
constexpr double kSimplifyTolerance = 0.05;
constexpr double kOffsetParameter = 0.414213562;

#if defined(__CUDA_ARCH__)
SK_HD double sk_sqrt(double x) { return sqrt(x); }
SK_HD double sk_cbrt(double x) { return cbrt(x); }
SK_HD double sk_pow(double x, double y) { return pow(x, y); }
SK_HD double sk_fabs(double x) { return fabs(x); }
SK_HD bool sk_isfinite(double x) { return isfinite(x); }
SK_HD double sk_nan() { return __longlong_as_double(0x7FF8000000000000LL); }
#else
SK_HD double sk_sqrt(double x) { return std::sqrt(x); }
SK_HD double sk_cbrt(double x) { return std::cbrt(x); }
SK_HD double sk_pow(double x, double y) { return std::pow(x, y); }
SK_HD double sk_fabs(double x) { return std::fabs(x); }
SK_HD bool sk_isfinite(double x) { return std::isfinite(x); }
SK_HD double sk_nan() { return std::nan(""); }
#endif

struct V {
  double x, y;
};
SK_HD V operator+(V a, V b) { return {a.x + b.x, a.y + b.y}; }
SK_HD V operator-(V a, V b) { return {a.x - b.x, a.y - b.y}; }
SK_HD V operator-(V a) { return {-a.x, -a.y}; }
SK_HD V operator*(V a, double s) { return {a.x * s, a.y * s}; }
SK_HD V operator*(double s, V a) { return {s * a.x, s * a.y}; }
SK_HD V operator/(V a, double s) { return {a.x / s, a.y / s}; }
SK_HD bool operator==(V a, V b) { return a.x == b.x && a.y == b.y; }
SK_HD bool operator!=(V a, V b) { return !(a == b); }

SK_HD double dot(V a, V b) { return a.x * b.x + a.y * b.y; }
SK_HD double cross(V a, V b) { return a.x * b.y - a.y * b.x; }
SK_HD double mag_sq(V v) { return v.x * v.x + v.y * v.y; }
SK_HD double mag(V v) { return sk_sqrt(mag_sq(v)); }
SK_HD double dist(V a, V b) { return sk_sqrt(mag_sq(b - a)); }
SK_HD V perp(V v) { return {-v.y, v.x}; }                    // Geometry::normal
SK_HD V unit(V v) { return v / mag(v); }
SK_HD V unit_normal(V v) { return perp(unit(v)); }
SK_HD bool is_zero(V p) { return (p.x == 0) & (p.y == 0); }
SK_HD V lerp(V a, V b, double t) { return (a - t * a) + t * b; }   // Math::lerp (math_p.h:512-520)
SK_HD V mid(V a, V b) { return 0.5 * a + 0.5 * b; }
SK_HD V vmin(V a, V b) { return {b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y}; }
SK_HD V vmax(V a, V b) { return {a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y}; }

// --- quadratic curves (bezier_p.h:190-448) -------------------------------------------------------

SK_HD V quad_point(const V* q, double t) {
  V v1 = q[1] - q[0], v2 = q[2] - q[1];
  V a = v2 - v1, b = v1 + v1;
  return (a * t + b) * t + q[0];
}

SK_HD void quad_derivative(const V* q, V& a, V& b) {
  V v1 = q[1] - q[0], v2 = q[2] - q[1];
  a = 2.0 * v2 - 2.0 * v1;
  b = 2.0 * v1;
}

// Parameter where the tangent has turned by the angle whose tangent is `m`.
SK_HD double quad_angle_step(const V* q, double m) {
  V a, b;
  quad_derivative(q, a, b);
  double aob = dot(a, b), axb = cross(a, b);
  if (aob == 0.0) return 1.0;
  return m * mag_sq(b) / (sk_fabs(axb) - m * aob);
}

// Parameters in (0, 1) where the quad's offset at distance d has a cusp; `ts` has room for one
// more entry after them.
SK_HD uint32_t quad_offset_cusps(const V* q, double d, double ts[3]) {
  V a, b;
  quad_derivative(q, a, b);
  double bxa = cross(b, a), boa = dot(b, a);
  if (bxa == 0.0) return 0;
  double alen2 = mag_sq(a), blen2 = mag_sq(b);
  double fac = -1.0 / alen2;
  double root = sk_sqrt(boa * boa - alen2 * (blen2 - sk_cbrt(d * d * bxa * bxa)));
  double t0 = fac * (boa + root);
  double t1 = fac * (boa - root);
  t0 = t0 < 0.0 ? 0.0 : t0;
  uint32_t n = uint32_t(t0 > 0.0 && t0 < 1.0);
  ts[0] = t0;
  ts[n] = t1;
  return n + uint32_t(t1 > t0 && t1 < 1.0);
}

SK_HD void quad_split(const V* c, V* lo, V* hi, double t) {
  V c0 = c[0], c1 = c[1], c2 = c[2];
  V p01 = lerp(c0, c1, t), p12 = lerp(c1, c2, t), m = lerp(p01, p12, t);
  lo[0] = c0; lo[1] = p01; lo[2] = m;
  hi[0] = m; hi[1] = p12; hi[2] = c2;
}

// A quad's pieces between consecutive parameters (QuadCurveTsIter): each next piece reuses the
// previous split's interpolants.
struct QuadPieces {
  const double* t;
  const double* t_end;
  V in[3], piece[3], i01, i12;

  SK_HD QuadPieces() : t(nullptr), t_end(nullptr) {}
  SK_HD QuadPieces(const V* q, const double* ts, uint32_t n) : t(ts), t_end(ts + n) {
    in[0] = q[0]; in[1] = q[1]; in[2] = q[2];
    double u = *t++;
    i01 = lerp(in[0], in[1], u);
    i12 = lerp(in[1], in[2], u);
    piece[0] = in[0]; piece[1] = i01; piece[2] = lerp(i01, i12, u);
  }
  SK_HD bool next() {
    if (t >= t_end) return false;
    double u = *t++;
    piece[0] = piece[2];
    piece[1] = lerp(i01, i12, u);
    i01 = lerp(in[0], in[1], u);
    i12 = lerp(in[1], in[2], u);
    piece[2] = lerp(i01, i12, u);
    return true;
  }
};

// --- cubic curves (bezier_p.h:617-982) ------------------------------------------------------------

SK_HD V cubic_point(const V* c, double t) {
  V v1 = c[1] - c[0], v2 = c[2] - c[1], v3 = c[3] - c[2];
  V a = v3 - v2 - v2 + v1, b = 3.0 * (v2 - v1), cc = 3.0 * v1;
  return ((a * t + b) * t + cc) * t + c[0];
}

SK_HD V cubic_identity(const V* c) {
  V v1 = c[1] - c[0], v2 = c[2] - c[1], v3 = c[3] - c[2];
  return v3 - v2 - v2 + v1;
}

SK_HD bool cubic_is_flat(const V* c, double f) {
  if (c[3] == c[0]) {
    V v = c[2] - c[1];
    double a = cross(v, c[1] - c[0]);
    return 0.5625 * a * a <= f * f * mag_sq(v);
  }
  V v = c[3] - c[0];
  double a1 = cross(v, c[1] - c[0]), a2 = cross(v, c[2] - c[0]);
  double s1 = a1 * a1, s2 = a2 * a2;
  return 0.5625 * (s1 < s2 ? s2 : s1) <= f * f * mag_sq(v);
}

// Roots of C'(t) x C''(t): tc and the half-distance tl (0 at a cusp, NaN when linear).
SK_HD void cubic_inflections(const V* c, double& tc, double& tl) {
  V v1 = c[1] - c[0], v2 = c[2] - c[1], v3 = c[3] - c[2];
  V da = 3.0 * (v3 - v2 - v2 + v1), db = 6.0 * (v2 - v1), dc = 3.0 * v1;
  double den = cross(db, da);
  if (den != 0) {
    tc = cross(da, dc) / den;
    tl = tc * tc + cross(db, dc) / den;
    if (tl > 0) tl = sk_sqrt(tl);
  }
  else {
    tc = -0.5 * cross(dc, db) / cross(dc, da);
    tl = sk_nan();
  }
}

SK_HD V cubic_start_dir(const V* c) {
  V d = c[1] - c[0], d20 = c[2] - c[0], d30 = c[3] - c[0];
  if (is_zero(d)) d = d20;
  if (is_zero(d)) d = d30;
  return d;
}

SK_HD V cubic_end_dir(const V* c) {
  V d = c[3] - c[2], d31 = c[3] - c[1], d30 = c[3] - c[0];
  if (is_zero(d)) d = d31;
  if (is_zero(d)) d = d30;
  return d;
}

SK_HD V cubic_derivative(const V* c, double t) {
  V p01 = lerp(c[0], c[1], t), p12 = lerp(c[1], c[2], t), p23 = lerp(c[2], c[3], t);
  return 3.0 * (lerp(p12, p23, t) - lerp(p01, p12, t));
}

// Splits at 0.5 (the midpoint form) or at t; inputs are read before any output is written.
SK_HD void cubic_halve(const V* c, V* lo, V* hi) {
  V c0 = c[0], c3 = c[3];
  V p01 = mid(c[0], c[1]), p12 = mid(c[1], c[2]), p23 = mid(c[2], c[3]);
  V l2 = mid(p01, p12), h1 = mid(p12, p23), m = mid(l2, h1);
  lo[0] = c0; lo[1] = p01; lo[2] = l2; lo[3] = m;
  hi[0] = m; hi[1] = h1; hi[2] = p23; hi[3] = c3;
}

SK_HD void cubic_split(const V* c, V* lo, V* hi, double t) {
  V c0 = c[0], c3 = c[3];
  V p01 = lerp(c[0], c[1], t), p12 = lerp(c[1], c[2], t), p23 = lerp(c[2], c[3], t);
  V l2 = lerp(p01, p12, t), h1 = lerp(p12, p23, t), m = lerp(l2, h1, t);
  lo[0] = c0; lo[1] = p01; lo[2] = l2; lo[3] = m;
  hi[0] = m; hi[1] = h1; hi[2] = p23; hi[3] = c3;
}

SK_HD V ray_intersection(V p0, V v0, V p1, V v1) { return p0 + cross(p1 - p0, v1) / cross(v0, v1) * v0; }

// Two quads through the cubic's midpoint estimate (approximate_cubic_with_two_quads).
SK_HD void cubic_two_quads(const V* c, V q[5]) {
  V c1 = lerp(c[0], c[1], 0.75);
  V c2 = lerp(c[3], c[2], 0.75);
  V pm = mid(c1, c2);
  if (c1 == c[0]) c1 = ray_intersection(c[0], cubic_start_dir(c), pm, cubic_derivative(c, 0.5));
  if (c2 == c[3]) c2 = ray_intersection(c[3], cubic_end_dir(c), pm, cubic_derivative(c, 0.5));
  q[0] = c[0]; q[1] = c1; q[2] = pm; q[3] = c2; q[4] = c[3];
}

// --- one side of the outline ---------------------------------------------------------------------

// Receives the vertices of one side as they become final (logical index, command, point); `fix`
// rewrites the figure's first point after it was handed out.
struct NullSink {
  SK_HD void put(uint32_t, uint8_t, V) {}
  SK_HD void fix0(V) {}
};

template <class Sink>
struct Side {
  static constexpr uint32_t kWin = 16;        // window of vertices that may still change
  static constexpr uint32_t kKeep = kWin - 4;
  uint8_t rc[kWin];
  V rp[kWin];
  uint32_t n = 0, done = 0;                   // logical size; [0, done) handed to the sink
  uint8_t first_c[2] = {0, 0};                // the figure's first two vertices
  V first_p[2] = {{0, 0}, {0, 0}};
  Sink sink;

  SK_HD void add(uint8_t c, V p) {
    if (n - done >= kKeep) {
      const uint32_t k = done % kWin;
      sink.put(done, rc[k], rp[k]);
      done++;
    }
    if (n < 2) { first_c[n] = c; first_p[n] = p; }
    rc[n % kWin] = c;
    rp[n % kWin] = p;
    n++;
  }
  SK_HD void move_to(V p) { add(kMove, p); }
  SK_HD void line_to(V p) { add(kOn, p); }
  SK_HD void quad_to(V a, V b) { add(kQuad, a); add(kOn, b); }
  SK_HD void cubic_to(V a, V b, V c) { add(kCubic, a); add(kCubic, b); add(kOn, c); }
  SK_HD void drop(uint32_t k) { n -= k; }
  SK_HD V last(uint32_t k = 1) const { return rp[(n - k) % kWin]; }
  SK_HD uint8_t last_cmd() const { return rc[(n - 1) % kWin]; }
  SK_HD void set_last(V p) {
    rp[(n - 1) % kWin] = p;
    if (n - 1 < 2) first_p[n - 1] = p;
  }
  // The vertex before the last one is an on-point (or the figure's move).
  SK_HD bool prev_on() const { return n >= 2 && rc[(n - 2) % kWin] <= kOn; }
  SK_HD void set_first(V p) {
    first_p[0] = p;
    if (done > 0) sink.fix0(p);
    else rp[0] = p;
  }
  SK_HD void flush() {
    for (; done < n; done++) sink.put(done, rc[done % kWin], rp[done % kWin]);
  }
  SK_HD void quarter_arc_to(V p1, V p2) {     // PathAppender::arc_quadrant_to (path_p.h:374-390)
    V p0 = last();
    cubic_to(p0 + (p1 - p0) * kKappa, p2 + (p1 - p2) * kKappa, p2);
  }
};

// pathstroke.cpp:99-105
SK_HD bool inside_overlap(V a0, V a1, V b0, V b1, V p) {
  V lo = vmax(vmin(a0, a1), vmin(b0, b1));
  V hi = vmin(vmax(a0, a1), vmax(b0, b1));
  return (p.x >= lo.x) & (p.y >= lo.y) & (p.x <= hi.x) & (p.y <= hi.y);
}

// pathstroke.cpp:107-117
template <class S>
SK_HD void arc_through(S& out, V c, V pa, V pb, V corner) {
  V pm = (pa + pb) * 0.5;
  double w = sk_sqrt(mag(c - pm) / mag(c - corner));
  double a = 4 * w / (3.0 * (1.0 + w));
  out.cubic_to(pa + a * (corner - pa), pb + a * (corner - pb), pb);
}

// BLStrokeOptions without the dash array (core/path.h:330-352).
struct Params {
  double width, miter_limit;
  uint32_t join, start_cap, end_cap, pad;
};

// Sizes of one figure's outline: A (offset side), B (other side, reversed on output), C (start
// cap, open figures). The outline is A, then B reversed (for a closed figure a figure of its own
// starting with a move; for an open one continuing from A's end cap, which ends on B's last
// point), then C without its move (it starts on B's first point and ends on A's first).
struct FigureCounts {
  uint32_t a = 0, b = 0, c = 0;
  bool closed = false, b_ok = false;
  SK_HD uint32_t b_out() const { return b_ok ? (closed ? b : b - 1) : 0u; }
  SK_HD uint32_t c_out() const { return closed ? 0u : (b_ok ? c - 1 : c); }
  SK_HD uint32_t total() const { return a + b_out() + c_out(); }
};

// Strokes the figure whose commands are cmd[first, end) (end: where the reference's stroker
// leaves the figure; the commands were validated). Sinks receive A's and B's vertices.
template <class SinkA, class SinkB>
class FigureStroker {
 public:
  Side<SinkA> a;
  Side<SinkB> b;
  Side<NullSink> c;                            // start cap: at most 9 vertices, never handed out

  SK_HD FigureStroker(const Params& p) : opt_(p), join_(p.join) {
    d_[0] = p.width * 0.5; d2_[0] = p.width;
    d_[1] = -d_[0]; d2_[1] = -d2_[0];
    if (join_ <= kJoinMiterRound) {             // the miter joins and their fallbacks
      if (join_ == kJoinMiterBevel) join_ = kJoinBevel;
      else if (join_ == kJoinMiterRound) join_ = kJoinRound;
      miter_ = d_[0] * p.miter_limit;
      miter_sq_ = miter_ * miter_;
    }
    else {
      miter_ = kMiterMinimum;
      miter_sq_ = kMiterMinimum * kMiterMinimum;
    }
  }

  // Returns the figure's counts; A and B are flushed to their sinks.
  SK_HD FigureCounts run(const uint8_t* cmd, const V* vtx, uint32_t first, uint32_t end);

 private:
  const Params& opt_;
  uint32_t join_;
  double d_[2], d2_[2];
  double miter_, miter_sq_;
  V p0_{0, 0}, n0_{0, 0}, p_start_{0, 0}, n_start_{0, 0};
  bool open_ = false, closed_ = false;

  static SK_HD int side_of(V n0, V n1) { return cross(n0, n1) >= 0 ? 1 : 0; }

  // The outer side of a join is A for side 0, B for side 1.
  template <class F>
  SK_HD void on_side(int s, F&& f) {
    if (s == 0) f(a, d_[0], d2_[0]);
    else f(b, d_[1], d2_[1]);
  }
  template <class F>
  SK_HD void on_inner(int s, F&& f) {
    if (s == 0) f(b);
    else f(a);
  }

  // pathstroke.cpp:769-838
  template <class S>
  SK_HD void outer_join(S& out, V n1, V w1, V k, double d, double d2, bool& mitered) {
    V pb = p0_ + w1;
    if (mag_sq(k) <= miter_sq_) {
      out.drop(out.prev_on());
      out.line_to(p0_ + k);
      out.line_to(pb);
      mitered = true;
      return;
    }
    if (join_ == kJoinMiterClip) {
      double b2 = sk_fabs(cross(k, n0_));
      if (b2 > 0) b2 = b2 * miter_ / mag(k);
      else b2 = miter_;
      out.drop(out.prev_on());
      out.line_to(p0_ + d * n0_ - b2 * perp(n0_));
      out.line_to(p0_ + d * n1 + b2 * perp(n1));
      mitered = true;
      out.line_to(pb);
      return;
    }
    if (join_ == kJoinRound) {
      V pa = out.last();
      if (dot(p0_ - pa, p0_ - pb) < 0.0) {       // dull angle: two arcs
        V n2 = unit_normal(pb - pa);
        V m = n0_ + n2;
        V k0 = d2 * m / mag_sq(m);
        V q = d * n2;
        V pc1 = p0_ + k0, pp1 = p0_ + q;
        V pc2 = lerp(pc1, pp1, 2.0);
        arc_through(out, p0_, pa, pp1, pc1);
        arc_through(out, p0_, pp1, pb, pc2);
      }
      else {                                     // acute angle: one arc
        V pm = mid(pa, pb);
        V pi = p0_ + k;
        double w = sk_sqrt(dist(p0_, pm) / dist(p0_, pi));
        double a = 4.0 * w / (3.0 * (1.0 + w));
        out.cubic_to(pa + a * (pi - pa), pb + a * (pi - pb), pb);
      }
      return;
    }
    out.line_to(pb);                             // bevel
  }

  // pathstroke.cpp:841-860: round join around a cusp.
  template <class S>
  SK_HD void cusp_join(S& out, double d, double d2, V w1) {
    V pa = out.last();
    V pb = p0_ + w1;
    V n2 = unit_normal(pb - pa);
    if (!sk_isfinite(n2.x)) return;
    V m = n0_ + n2;
    V k = m * d2 / mag_sq(m);
    V q = n2 * d;
    V pc1 = p0_ + k, pp1 = p0_ + q;
    V pc2 = lerp(pc1, pp1, 2.0);
    arc_through(out, p0_, pa, pp1, pc1);
    arc_through(out, p0_, pp1, pb, pc2);
  }

  // pathstroke.cpp:741-750
  template <class S>
  SK_HD void inner_line_join(S& out, V l0, V l1, V corner) {
    if (out.prev_on() && inside_overlap(out.last(2), out.last(), l0, l1, corner)) {
      out.set_last(corner);
    }
    else {
      out.line_to(p0_);
      out.line_to(l0);
    }
  }

  SK_HD void start_with_line(V p1, V n1) {       // open_line_to (:540-556)
    V w = n1 * d_[0];
    a.move_to(p0_ + w);
    b.move_to(p0_ - w);
    p0_ = p1; n0_ = n1; n_start_ = n1;
    a.line_to(p0_ + w);
    b.line_to(p0_ - w);
    open_ = true;
  }

  SK_HD void line_to(V p1, V n1) {               // join_line_to (:559-598)
    if (n0_ == n1) {
      a.drop(a.prev_on());
      b.drop(b.prev_on());
      V w1 = n1 * d_[0];
      a.line_to(p1 + w1);
      b.line_to(p1 - w1);
    }
    else {
      int s = side_of(n0_, n1);
      V m = n0_ + n1;
      V k = m * d2_[s] / mag_sq(m);
      V w1 = n1 * d_[s];
      on_side(s, [&](auto& outer, double d, double d2) {
        bool mitered = false;
        outer_join(outer, n1, w1, k, d, d2, mitered);
        outer.drop(mitered ? 1u : 0u);
        outer.line_to(p1 + w1);
      });
      on_inner(s, [&](auto& inner) {
        inner_line_join(inner, p0_ - w1, p1 - w1, p0_ - k);
        inner.line_to(p1 - w1);
      });
    }
    p0_ = p1; n0_ = n1;
  }

  SK_HD void start_with_curve(V n) {             // open_curve (:604-616)
    V w = n * d_[0];
    a.move_to(p0_ + w);
    b.move_to(p0_ - w);
    n0_ = n; n_start_ = n;
    open_ = true;
  }

  SK_HD void curve_join(V n1) {                  // join_curve (:619-636)
    if (n0_ == n1) return;
    int s = side_of(n0_, n1);
    V m = n0_ + n1;
    V k = m * d2_[s] / mag_sq(m);
    V w1 = n1 * d_[s];
    on_side(s, [&](auto& outer, double d, double d2) {
      bool unused = false;
      outer_join(outer, n1, w1, k, d, d2, unused);
    });
    on_inner(s, [&](auto& inner) {
      inner.line_to(p0_);
      inner.line_to(p0_ - w1);
    });
    n0_ = n1;
  }

  SK_HD void cusp_curve_join(V n1) {             // join_cusp (:638-647)
    int s = side_of(n0_, n1);
    V w1 = n1 * d_[s];
    on_side(s, [&](auto& outer, double d, double d2) { cusp_join(outer, d, d2, w1); });
    on_inner(s, [&](auto& inner) { inner.line_to(p0_ - w1); });
    n0_ = n1;
  }

  SK_HD void cusp_line_to(V n1, V p1) {          // join_cusp_and_line_to (:649-665)
    int s = side_of(n0_, n1);
    V w1 = n1 * d_[s];
    on_side(s, [&](auto& outer, double d, double d2) {
      cusp_join(outer, d, d2, w1);
      outer.line_to(p1 + w1);
    });
    on_inner(s, [&](auto& inner) {
      inner.line_to(p0_ - w1);
      inner.line_to(p1 - w1);
    });
    n0_ = n1; p0_ = p1;
  }

  SK_HD void poly_to(const V* poly, uint32_t count) {   // smooth_poly_to (:667-694)
    V p1 = poly[0];
    V v1 = p1 - p0_;
    if (mag_sq(v1) < kLengthEpsilonSq) return;
    V n1 = unit_normal(v1);
    if (!open_) start_with_line(p1, n1);
    else line_to(p1, n1);
    for (uint32_t i = 1; i < count; i++) {
      p1 = poly[i];
      v1 = p1 - p0_;
      if (mag_sq(v1) < kLengthEpsilonSq) continue;
      cusp_line_to(unit_normal(v1), p1);
    }
  }

  SK_HD void close_join(V n1) {                  // join_end_point (:697-734)
    if (n0_ == n1) {
      a.drop(a.prev_on());
      b.drop(b.prev_on());
      return;
    }
    int s = side_of(n0_, n1);
    V m = n0_ + n1;
    V w1 = n1 * d_[s];
    V k = m * d2_[s] / mag_sq(m);
    on_side(s, [&](auto& outer, double d, double d2) {
      bool mitered = false;
      outer_join(outer, n1, w1, k, d, d2, mitered);
      // a miter moves the figure's start to the miter point
      if (mitered && outer.first_c[1] == kOn) {
        outer.drop(1);
        outer.set_first(outer.last());
        outer.drop(outer.prev_on());
      }
    });
    on_inner(s, [&](auto& inner) {
      if (inner.first_c[1] <= kOn) {
        V corner = p0_ - k;
        if (inner.prev_on() && inside_overlap(inner.last(2), inner.last(), inner.first_p[0], inner.first_p[1], corner)) {
          inner.set_first(corner);
          inner.drop(1);
        }
        else {
          V start = inner.first_p[0];
          inner.line_to(p0_);
          inner.line_to(start);
        }
      }
    });
  }

  SK_HD void offset_quad_piece(V q0, V q1, V q2) {   // offset_quad_simple (:885-905)
    if (q0 == q2) return;
    V v0 = q1 - q0, v1 = q2 - q1;
    V m0 = unit_normal(q0 != q1 ? v0 : v1);
    V m2 = unit_normal(q1 != q2 ? v1 : v0);
    p0_ = q2; n0_ = m2;
    V m = m0 + m2;
    V k1 = m * d2_[0] / mag_sq(m);
    V k2 = m2 * d_[0];
    a.quad_to(q1 + k1, q2 + k2);
    b.quad_to(q1 - k1, q2 - k2);
  }

  // --- offsetting, one piece per step ------------------------------------------------------
  // offset_quad (:860-883) and approximate_cubic_with_quads (bezier_p.h:943-982) unrolled into a
  // state the figure loop advances by one offset quad piece per iteration, so the lanes of a warp,
  // each on its own figure, issue the piece arithmetic together however many t-steps, quads and
  // pieces their curves need.
  bool cubic_ = false, pieces_ = false;
  uint32_t qn_ = 0, qe_ = 0;                   // quads of the current step start at q_[qn_], end at qe_
  double t_ = 0.0;                             // the cubic's next t-step
  V w_[7];                                     // the cubic's remainder in w_[3..6]
  V q_[5];
  double ts_[3];
  QuadPieces it_;

  SK_HD bool offsetting() const { return pieces_ || qn_ < qe_ || cubic_; }

  SK_HD void begin_quad(const V* q) {
    q_[0] = q[0]; q_[1] = q[1]; q_[2] = q[2];
    qn_ = 0; qe_ = 2;
    cubic_ = false; pieces_ = false;
  }

  SK_HD void begin_cubic(const V* c) {
    double tol = 54.0 * kSimplifyTolerance;
    t_ = sk_pow(tol * tol / mag_sq(cubic_identity(c)), 1.0 / 6.0);
    w_[3] = c[0]; w_[4] = c[1]; w_[5] = c[2]; w_[6] = c[3];
    qn_ = qe_ = 0;
    cubic_ = true; pieces_ = false;
  }

  SK_HD void offset_step() {
    if (!pieces_) {
      if (qn_ >= qe_) {                          // the cubic's next t-step: two quads
        t_ = t_ < 1.0 ? t_ : 1.0;
        if (t_ >= 0.999) t_ = 1.0;
        cubic_split(w_ + 3, w_, w_ + 3, t_);
        cubic_two_quads(w_, q_);
        qn_ = 0; qe_ = 4;
        if (t_ >= 1.0) cubic_ = false;
        else {
          double prev = t_;
          t_ = t_ / (1.0 - t_);
          if (prev - t_ < 1e-3) t_ += 0.01;
        }
      }
      // the next quad, cut at its offset's cusps
      const V* q = q_ + qn_;
      qn_ += 2;
      uint32_t tn = quad_offset_cusps(q, d_[0], ts_);
      ts_[tn++] = 1.0;
      it_ = QuadPieces(q, ts_, tn);
      pieces_ = true;
    }
    double t = quad_angle_step(it_.piece, kOffsetParameter);
    if (!(t > kOffsetQuadEpsilonT && t < 1.0 - kOffsetQuadEpsilonT)) t = 1.0;
    V head[3];
    quad_split(it_.piece, head, it_.piece, t);
    offset_quad_piece(head[0], head[1], head[2]);
    if (t == 1.0 && !it_.next()) pieces_ = false;
  }

  // --- input commands, one per step ----------------------------------------------------------
  bool cusp_pending_ = false;                  // the second half of a cubic split at its cusp
  V cusp_half_[4];

  SK_HD void line_step(V p1) {
    V v1 = p1 - p0_;
    if (mag_sq(v1) < kLengthEpsilonSq) return;
    V n1 = unit_normal(v1);
    if (!open_) start_with_line(p1, n1);
    else line_to(p1, n1);
  }

  // Starts offsetting the cubic p[0..3]; `cusp_join` for the half after a cusp.
  SK_HD void cubic_step(const V* p, bool after_cusp) {
    V v1 = p[1] - p0_;
    if (is_zero(v1)) v1 = p[2] - p0_;
    V n1 = unit_normal(v1);
    if (!open_) start_with_curve(n1);
    else if (!after_cusp) curve_join(n1);
    else cusp_curve_join(n1);
    begin_cubic(p);
  }

  // One command of the figure (PathStroker::stroke's loop body, pathstroke.cpp:266-456); false
  // where that loop ends. Curves leave their offsetting to offset_step.
  SK_HD bool command_step(const uint8_t* cmd, const V* vtx, uint32_t& i, uint32_t end) {
    if (i >= end) return false;
    const uint8_t c = cmd[i];
    const V p1 = vtx[i];
    if (c == kOn) {
      i++;
      line_step(p1);
      return true;
    }
    if (c == kQuad) {
      i += 2;
      const V* q = vtx + i - 3;                  // starts at the input's previous vertex
      V p2 = q[2];
      V v2 = p2 - p1;
      V v1 = p1 - p0_;
      V n1 = unit_normal(v1);
      if (sk_fabs(cross(v2, v1)) <= kCollinearityEpsilon) {
        if (dot(-v1, v2) > 0.0) {                // control point outside: a cusp
          double r1 = dot(p1 - p0_, v1);
          double r2 = dot(p2 - p0_, v1);
          double t = r1 / (2.0 * r1 - r2);
          if (t > 0.0 && t < 1.0) {
            V poly[2] = {quad_point(q, t), p2};
            poly_to(poly, 2);
            return true;
          }
        }
        line_step(p2);
        return true;
      }
      if (mag_sq(v1) < kLengthEpsilonSq || mag_sq(v2) < kLengthEpsilonSq) { line_step(p2); return true; }
      if (!open_) start_with_curve(n1);
      else curve_join(n1);
      begin_quad(q);
      return true;
    }
    if (c == kCubic) {
      i += 3;
      V p[7] = {};
      p[0] = p0_; p[1] = vtx[i - 3]; p[2] = vtx[i - 2]; p[3] = vtx[i - 1];
      if (cubic_is_flat(p, kDegenerateFlatness)) {
        double dot1 = dot(p[0] - p[1], p[3] - p[1]);
        double dot2 = dot(p[0] - p[2], p[3] - p[2]);
        if (!(dot1 < 0.0) || !(dot2 < 0.0)) {    // flat with the controls outside: cusps
          V r = cubic_start_dir(p);
          double r1 = dot(p[1] - p[0], r), r2 = dot(p[2] - p[0], r), r3 = dot(p[3] - p[0], r);
          double aa = 1.0 / (3.0 * r1 - 3.0 * r2 + r3);
          double bb = 2.0 * r1 - r2;
          double sq = sk_sqrt(r2 * (r2 - r1) - r1 * (r3 - r1));
          double t1 = aa * (bb - sq), t2 = aa * (bb + sq);
          V poly[3];
          uint32_t poly_n = 0;
          if (t1 > kCuspTThreshold && t1 < 1.0 - kCuspTThreshold) poly[poly_n++] = cubic_point(p, t1);
          if (t2 > kCuspTThreshold && t2 < 1.0 - kCuspTThreshold) poly[poly_n++] = cubic_point(p, t2);
          if (poly_n == 0) { line_step(p[3]); return true; }
          poly[poly_n++] = p[3];
          poly_to(poly, poly_n);
          return true;
        }
        line_step(p[3]);
        return true;
      }
      double tc, tl;
      cubic_inflections(p, tc, tl);
      if (tl == 0.0 && tc > 0.0 && tc < 1.0) {   // a cusp: the two halves, joined round
        cubic_halve(p, p, p + 3);
        cusp_half_[0] = p[3]; cusp_half_[1] = p[4]; cusp_half_[2] = p[5]; cusp_half_[3] = p[6];
        cusp_pending_ = true;
      }
      cubic_step(p, false);
      return true;
    }
    if (closed_ || c != kClose) return false;
    closed_ = true;
    line_step(p_start_);
    return true;
  }

  template <class S>
  SK_HD void add_cap(S& out, V pivot, V p1, uint32_t cap) {   // pathstroke.cpp:921-969
    V p0 = out.last();
    V q = perp(p1 - p0) * 0.5;
    switch (cap) {
      case kCapSquare: out.line_to(p0 + q); out.line_to(p1 + q); out.line_to(p1); break;
      case kCapRound: out.quarter_arc_to(p0 + q, pivot + q); out.quarter_arc_to(p1 + q, p1); break;
      case kCapRoundRev:
        out.line_to(p0 + q); out.quarter_arc_to(p0, pivot); out.quarter_arc_to(p1, p1 + q); out.line_to(p1);
        break;
      case kCapTriangle: out.line_to(pivot + q); out.line_to(p1); break;
      case kCapTriangleRev: out.line_to(p0 + q); out.line_to(pivot); out.line_to(p1 + q); out.line_to(p1); break;
      default: out.line_to(p1); break;
    }
  }
};

// The figure loop of PathStroker::stroke (pathstroke.cpp:256-478), one unit of work per iteration.
template <class SinkA, class SinkB>
SK_HD FigureCounts FigureStroker<SinkA, SinkB>::run(const uint8_t* cmd, const V* vtx, uint32_t first, uint32_t end) {
  FigureCounts out;
  uint32_t i = first;
  p0_ = vtx[i];
  p_start_ = p0_;
  i++;
  for (;;) {
    if (offsetting()) offset_step();
    else if (cusp_pending_) { cusp_pending_ = false; cubic_step(cusp_half_, true); }
    else if (!command_step(cmd, vtx, i, end)) break;
  }
  if (!open_) return out;
  out.closed = closed_;
  if (closed_) {
    close_join(n_start_);
  }
  else {
    uint32_t start_cap = opt_.start_cap <= kCapTriangleRev ? opt_.start_cap : kCapButt;
    uint32_t end_cap = opt_.end_cap <= kCapTriangleRev ? opt_.end_cap : kCapButt;
    add_cap(a, p0_, b.last(), end_cap);
    c.move_to(b.first_p[0]);
    add_cap(c, p_start_, a.first_p[0], start_cap);
  }
  a.flush();
  b.flush();
  out.a = a.n;
  out.b = b.n;
  out.c = c.n;
  // EdgeSourceReversePathFromStrokeSink::begin (edgebuilder_p.h:322-335) takes B only when it
  // ends on an on-point.
  out.b_ok = b.n > 0 && b.last_cmd() == kOn;
  return out;
}

// --- output -------------------------------------------------------------------------------------

// Writes A forward from `base`.
struct ForwardSink {
  uint8_t* cmd;
  double* xy;
  SK_HD void put(uint32_t i, uint8_t c, V p) { cmd[i] = c; xy[2 * i] = p.x; xy[2 * i + 1] = p.y; }
  SK_HD void fix0(V p) { xy[0] = p.x; xy[1] = p.y; }
};

// Writes B reversed (EdgeSourceReversePathFromStrokeSink, edgebuilder_p.h:287-405): vertex i of
// B lands at n - 1 - i; a vertex keeps its command (control points are symmetric under reversal),
// the move becomes an on-point, and the last vertex starts the reversed figure (closed figures) or
// is dropped (open figures: A's end cap already ends on it).
struct ReverseSink {
  uint8_t* cmd;
  double* xy;
  uint32_t n;       // B's final size
  bool with_move;
  bool enabled;
  SK_HD void put(uint32_t i, uint8_t c, V p) {
    if (!enabled) return;
    uint32_t pos;
    if (with_move) {
      pos = n - 1 - i;
      c = i == n - 1 ? kMove : (c == kMove ? kOn : c);
    }
    else {
      if (i == n - 1) return;
      pos = n - 2 - i;
      c = c == kMove ? kOn : c;
    }
    cmd[pos] = c;
    xy[2 * pos] = p.x;
    xy[2 * pos + 1] = p.y;
  }
  SK_HD void fix0(V p) { put(0, kMove, p); }
};

// Second pass: writes the figure's outline (counts from the first pass) at cmd/xy.
SK_HD void emit_figure(const uint8_t* in_cmd, const V* in_vtx, uint32_t first, uint32_t end, const Params& p,
                       const FigureCounts& fc, uint8_t* out_cmd, double* out_xy) {
  FigureStroker<ForwardSink, ReverseSink> s(p);
  s.a.sink = ForwardSink{out_cmd, out_xy};
  const uint32_t rb = fc.a;
  s.b.sink = ReverseSink{out_cmd + rb, out_xy + 2 * rb, fc.b, fc.closed, fc.b_ok};
  s.run(in_cmd, in_vtx, first, end);
  if (!fc.closed) {
    // C: its move is B's first point where reversed B ends (dropped), or starts a figure when B
    // was not taken
    const uint32_t base = fc.a + fc.b_out();
    const uint32_t skip = fc.b_ok ? 1u : 0u;
    for (uint32_t i = skip; i < s.c.n; i++) {
      const uint32_t pos = base + i - skip;
      out_cmd[pos] = s.c.rc[i];
      out_xy[2 * pos] = s.c.rp[i].x;
      out_xy[2 * pos + 1] = s.c.rp[i].y;
    }
  }
}

// First pass: the figure's outline sizes.
SK_HD FigureCounts count_figure(const uint8_t* in_cmd, const V* in_vtx, uint32_t first, uint32_t end, const Params& p) {
  FigureStroker<NullSink, NullSink> s(p);
  return s.run(in_cmd, in_vtx, first, end);
}

}  // namespace sk
}  // namespace blgpu
