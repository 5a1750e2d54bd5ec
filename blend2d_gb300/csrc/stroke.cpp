// Path stroker. Restates bl::PathInternal::PathStroker (blend2d/core/pathstroke.cpp:126-971) and
// the Bezier helpers it uses (blend2d/geometry/bezier_p.h, blend2d/geometry/commons_p.h): the
// outline is defined by the exact sequence of double operations there (this file is compiled
// with -ffp-contract=off), so every expression keeps the reference's operand order.
#include "stroke.h"

#include <cmath>
#include <cstring>

namespace blgpu {
namespace {

enum : uint8_t { kMove = 0, kOn = 1, kQuad = 2, kConic = 3, kCubic = 4, kClose = 5 };
enum : uint32_t { kJoinMiterClip = 0, kJoinMiterBevel = 1, kJoinMiterRound = 2, kJoinBevel = 3, kJoinRound = 4 };
enum : uint32_t { kCapButt = 0, kCapSquare = 1, kCapRound = 2, kCapRoundRev = 3, kCapTriangle = 4, kCapTriangleRev = 5 };

// pathstroke.cpp:22-47, mathconst_p.h:52
constexpr double kMiterMinimum = 1e-10;
constexpr double kLengthEpsilonSq = 1e-10 * 1e-10;
constexpr double kCollinearityEpsilon = 1e-10;
constexpr double kCuspTThreshold = 1e-10;
constexpr double kDegenerateFlatness = 1e-6;
constexpr double kOffsetQuadEpsilonT = 1e-5;
constexpr double kKappa = 0.55228474983;

struct V {
  double x, y;
  friend V operator+(V a, V b) { return {a.x + b.x, a.y + b.y}; }
  friend V operator-(V a, V b) { return {a.x - b.x, a.y - b.y}; }
  friend V operator-(V a) { return {-a.x, -a.y}; }
  friend V operator*(V a, double s) { return {a.x * s, a.y * s}; }
  friend V operator*(double s, V a) { return {s * a.x, s * a.y}; }
  friend V operator/(V a, double s) { return {a.x / s, a.y / s}; }
  friend bool operator==(V a, V b) { return a.x == b.x && a.y == b.y; }
  friend bool operator!=(V a, V b) { return !(a == b); }
};

inline double dot(V a, V b) { return a.x * b.x + a.y * b.y; }
inline double cross(V a, V b) { return a.x * b.y - a.y * b.x; }
inline double mag_sq(V v) { return v.x * v.x + v.y * v.y; }
inline double mag(V v) { return std::sqrt(mag_sq(v)); }
inline double dist(V a, V b) { return std::sqrt(mag_sq(b - a)); }
inline V perp(V v) { return {-v.y, v.x}; }                    // Geometry::normal
inline V unit(V v) { return v / mag(v); }
inline V unit_normal(V v) { return perp(unit(v)); }
inline bool is_zero(V p) { return (p.x == 0) & (p.y == 0); }
inline V lerp(V a, V b, double t) { return (a - t * a) + t * b; }   // Math::lerp (math_p.h:512-520)
inline V mid(V a, V b) { return 0.5 * a + 0.5 * b; }
inline V vmin(V a, V b) { return {b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y}; }
inline V vmax(V a, V b) { return {a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y}; }

// --- quadratic curves (bezier_p.h:190-448) -------------------------------------------------------

V quad_point(const V* q, double t) {
  V v1 = q[1] - q[0], v2 = q[2] - q[1];
  V a = v2 - v1, b = v1 + v1;
  return (a * t + b) * t + q[0];
}

void quad_derivative(const V* q, V& a, V& b) {
  V v1 = q[1] - q[0], v2 = q[2] - q[1];
  a = 2.0 * v2 - 2.0 * v1;
  b = 2.0 * v1;
}

// Parameter where the tangent has turned by the angle whose tangent is `m`.
double quad_angle_step(const V* q, double m) {
  V a, b;
  quad_derivative(q, a, b);
  double aob = dot(a, b), axb = cross(a, b);
  if (aob == 0.0) return 1.0;
  return m * mag_sq(b) / (std::fabs(axb) - m * aob);
}

// Parameters in (0, 1) where the offset of the quad at distance d has a cusp; `ts` has room for
// one more entry after them.
size_t quad_offset_cusps(const V* q, double d, double ts[3]) {
  V a, b;
  quad_derivative(q, a, b);
  double bxa = cross(b, a), boa = dot(b, a);
  if (bxa == 0.0) return 0;
  double alen2 = mag_sq(a), blen2 = mag_sq(b);
  double fac = -1.0 / alen2;
  double root = std::sqrt(boa * boa - alen2 * (blen2 - std::cbrt(d * d * bxa * bxa)));
  double t0 = fac * (boa + root);
  double t1 = fac * (boa - root);
  t0 = t0 < 0.0 ? 0.0 : t0;
  size_t n = size_t(t0 > 0.0 && t0 < 1.0);
  ts[0] = t0;
  ts[n] = t1;
  return n + size_t(t1 > t0 && t1 < 1.0);
}

void quad_split(const V* c, V* lo, V* hi, double t) {
  V c0 = c[0], c1 = c[1], c2 = c[2];
  V p01 = lerp(c0, c1, t), p12 = lerp(c1, c2, t), m = lerp(p01, p12, t);
  lo[0] = c0; lo[1] = p01; lo[2] = m;
  hi[0] = m; hi[1] = p12; hi[2] = c2;
}

// Walks a quad's pieces between consecutive parameters (the reference's QuadCurveTsIter): each
// next piece reuses the previous split's interpolants.
struct QuadPieces {
  const double* t;
  const double* t_end;
  V in[3], piece[3], i01, i12;

  QuadPieces(const V* q, const double* ts, size_t n) : t(ts), t_end(ts + n) {
    in[0] = q[0]; in[1] = q[1]; in[2] = q[2];
    double u = *t++;
    i01 = lerp(in[0], in[1], u);
    i12 = lerp(in[1], in[2], u);
    piece[0] = in[0]; piece[1] = i01; piece[2] = lerp(i01, i12, u);
  }
  bool next() {
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

V cubic_point(const V* c, double t) {
  V v1 = c[1] - c[0], v2 = c[2] - c[1], v3 = c[3] - c[2];
  V a = v3 - v2 - v2 + v1, b = 3.0 * (v2 - v1), cc = 3.0 * v1;
  return ((a * t + b) * t + cc) * t + c[0];
}

bool cubic_is_flat(const V* c, double f) {
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
void cubic_inflections(const V* c, double& tc, double& tl) {
  V v1 = c[1] - c[0], v2 = c[2] - c[1], v3 = c[3] - c[2];
  V da = 3.0 * (v3 - v2 - v2 + v1), db = 6.0 * (v2 - v1), dc = 3.0 * v1;
  double den = cross(db, da);
  if (den != 0) {
    tc = cross(da, dc) / den;
    tl = tc * tc + cross(db, dc) / den;
    if (tl > 0) tl = std::sqrt(tl);
  }
  else {
    tc = -0.5 * cross(dc, db) / cross(dc, da);
    tl = NAN;
  }
}

V cubic_start_dir(const V* c) {
  V d = c[1] - c[0], d20 = c[2] - c[0], d30 = c[3] - c[0];
  if (is_zero(d)) d = d20;
  if (is_zero(d)) d = d30;
  return d;
}

V cubic_end_dir(const V* c) {
  V d = c[3] - c[2], d31 = c[3] - c[1], d30 = c[3] - c[0];
  if (is_zero(d)) d = d31;
  if (is_zero(d)) d = d30;
  return d;
}

V cubic_derivative(const V* c, double t) {
  V p01 = lerp(c[0], c[1], t), p12 = lerp(c[1], c[2], t), p23 = lerp(c[2], c[3], t);
  return 3.0 * (lerp(p12, p23, t) - lerp(p01, p12, t));
}

// Splits at 0.5 (the midpoint form) or at t; inputs are read before any output is written.
void cubic_halve(const V* c, V* lo, V* hi) {
  V c0 = c[0], c3 = c[3];
  V p01 = mid(c[0], c[1]), p12 = mid(c[1], c[2]), p23 = mid(c[2], c[3]);
  V l2 = mid(p01, p12), h1 = mid(p12, p23), m = mid(l2, h1);
  lo[0] = c0; lo[1] = p01; lo[2] = l2; lo[3] = m;
  hi[0] = m; hi[1] = h1; hi[2] = p23; hi[3] = c3;
}

void cubic_split(const V* c, V* lo, V* hi, double t) {
  V c0 = c[0], c3 = c[3];
  V p01 = lerp(c[0], c[1], t), p12 = lerp(c[1], c[2], t), p23 = lerp(c[2], c[3], t);
  V l2 = lerp(p01, p12, t), h1 = lerp(p12, p23, t), m = lerp(l2, h1, t);
  lo[0] = c0; lo[1] = p01; lo[2] = l2; lo[3] = m;
  hi[0] = m; hi[1] = h1; hi[2] = p23; hi[3] = c3;
}

V ray_intersection(V p0, V v0, V p1, V v1) { return p0 + cross(p1 - p0, v1) / cross(v0, v1) * v0; }

// Two quads through the cubic's midpoint estimate (approximate_cubic_with_two_quads).
void cubic_two_quads(const V* c, V q[5]) {
  V c1 = lerp(c[0], c[1], 0.75);
  V c2 = lerp(c[3], c[2], 0.75);
  V pm = mid(c1, c2);
  if (c1 == c[0]) c1 = ray_intersection(c[0], cubic_start_dir(c), pm, cubic_derivative(c, 0.5));
  if (c2 == c[3]) c2 = ray_intersection(c[3], cubic_end_dir(c), pm, cubic_derivative(c, 0.5));
  q[0] = c[0]; q[1] = c1; q[2] = pm; q[3] = c2; q[4] = c[3];
}

// --- one side's output path -------------------------------------------------------------------------

// An offset path being written: the stroker rewrites and drops the vertices it has just written.
struct Side {
  std::vector<uint8_t> cmd;
  std::vector<V> pt;

  void clear() { cmd.clear(); pt.clear(); }
  size_t size() const { return cmd.size(); }
  void add(uint8_t c, V p) { cmd.push_back(c); pt.push_back(p); }
  void move_to(V p) { add(kMove, p); }
  void line_to(V p) { add(kOn, p); }
  void quad_to(V a, V b) { add(kQuad, a); add(kOn, b); }
  void cubic_to(V a, V b, V c) { add(kCubic, a); add(kCubic, b); add(kOn, c); }
  void close() { add(kClose, V{NAN, NAN}); }
  void drop(size_t n) { cmd.resize(cmd.size() - n); pt.resize(pt.size() - n); }
  V& last(size_t k = 1) { return pt[pt.size() - k]; }
  // The vertex before the last one is an on-point (or the figure's move).
  bool prev_on() const { return cmd.size() >= 2 && cmd[cmd.size() - 2] <= kOn; }
  void quarter_arc_to(V p1, V p2) {            // PathAppender::arc_quadrant_to (path_p.h:374-390)
    V p0 = last();
    cubic_to(p0 + (p1 - p0) * kKappa, p2 + (p1 - p2) * kKappa, p2);
  }
};

// pathstroke.cpp:99-105
bool inside_overlap(V a0, V a1, V b0, V b1, V p) {
  V lo = vmax(vmin(a0, a1), vmin(b0, b1));
  V hi = vmin(vmax(a0, a1), vmax(b0, b1));
  return (p.x >= lo.x) & (p.y >= lo.y) & (p.x <= hi.x) & (p.y <= hi.y);
}

// pathstroke.cpp:107-117
void arc_through(Side& out, V c, V pa, V pb, V corner) {
  V pm = (pa + pb) * 0.5;
  double w = std::sqrt(mag(c - pm) / mag(c - corner));
  double a = 4 * w / (3.0 * (1.0 + w));
  out.cubic_to(pa + a * (corner - pa), pb + a * (corner - pb), pb);
}

class Stroker {
 public:
  Stroker(const StrokeParams& p) : opt_(p), join_(p.join) {
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

  BLGpuResult run(const uint8_t* cmd, const V* vtx, size_t n, std::vector<uint8_t>& out_cmds, std::vector<double>& out_xy);

 private:
  const StrokeParams& opt_;
  uint32_t join_;
  double d_[2], d2_[2];
  double miter_, miter_sq_;
  Side side_[2], cap_;
  V p0_{}, n0_{}, p_start_{}, n_start_{};
  bool open_ = false, closed_ = false;

  static int side_of(V n0, V n1) { return cross(n0, n1) >= 0 ? 1 : 0; }

  // pathstroke.cpp:769-838
  void outer_join(Side& out, V n1, V w1, V k, double d, double d2, bool& mitered) {
    V pb = p0_ + w1;
    if (mag_sq(k) <= miter_sq_) {
      out.drop(out.prev_on());
      out.line_to(p0_ + k);
      out.line_to(pb);
      mitered = true;
      return;
    }
    if (join_ == kJoinMiterClip) {
      double b2 = std::fabs(cross(k, n0_));
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
        double w = std::sqrt(dist(p0_, pm) / dist(p0_, pi));
        double a = 4.0 * w / (3.0 * (1.0 + w));
        out.cubic_to(pa + a * (pi - pa), pb + a * (pi - pb), pb);
      }
      return;
    }
    out.line_to(pb);                             // bevel
  }

  // pathstroke.cpp:841-860: round join around a cusp.
  void cusp_join(Side& out, double d, double d2, V w1) {
    V pa = out.last();
    V pb = p0_ + w1;
    V n2 = unit_normal(pb - pa);
    if (!std::isfinite(n2.x)) return;
    V m = n0_ + n2;
    V k = m * d2 / mag_sq(m);
    V q = n2 * d;
    V pc1 = p0_ + k, pp1 = p0_ + q;
    V pc2 = lerp(pc1, pp1, 2.0);
    arc_through(out, p0_, pa, pp1, pc1);
    arc_through(out, p0_, pp1, pb, pc2);
  }

  // pathstroke.cpp:741-750
  void inner_line_join(Side& out, V l0, V l1, V corner) {
    if (out.prev_on() && inside_overlap(out.last(2), out.last(), l0, l1, corner)) {
      out.last() = corner;
    }
    else {
      out.line_to(p0_);
      out.line_to(l0);
    }
  }

  void start_with_line(V p1, V n1) {            // open_line_to (:540-556)
    V w = n1 * d_[0];
    side_[0].move_to(p0_ + w);
    side_[1].move_to(p0_ - w);
    p0_ = p1; n0_ = n1; n_start_ = n1;
    side_[0].line_to(p0_ + w);
    side_[1].line_to(p0_ - w);
    open_ = true;
  }

  void line_to(V p1, V n1) {                     // join_line_to (:559-598)
    if (n0_ == n1) {
      side_[0].drop(side_[0].prev_on());
      side_[1].drop(side_[1].prev_on());
      V w1 = n1 * d_[0];
      side_[0].line_to(p1 + w1);
      side_[1].line_to(p1 - w1);
    }
    else {
      int s = side_of(n0_, n1);
      V m = n0_ + n1;
      V k = m * d2_[s] / mag_sq(m);
      V w1 = n1 * d_[s];
      bool mitered = false;
      Side& outer = side_[s];
      Side& inner = side_[1 - s];
      outer_join(outer, n1, w1, k, d_[s], d2_[s], mitered);
      outer.drop(mitered ? 1 : 0);
      outer.line_to(p1 + w1);
      inner_line_join(inner, p0_ - w1, p1 - w1, p0_ - k);
      inner.line_to(p1 - w1);
    }
    p0_ = p1; n0_ = n1;
  }

  void start_with_curve(V n) {                   // open_curve (:604-616)
    V w = n * d_[0];
    side_[0].move_to(p0_ + w);
    side_[1].move_to(p0_ - w);
    n0_ = n; n_start_ = n;
    open_ = true;
  }

  void curve_join(V n1) {                        // join_curve (:619-636)
    if (n0_ == n1) return;
    int s = side_of(n0_, n1);
    V m = n0_ + n1;
    V k = m * d2_[s] / mag_sq(m);
    V w1 = n1 * d_[s];
    bool unused = false;
    outer_join(side_[s], n1, w1, k, d_[s], d2_[s], unused);
    side_[1 - s].line_to(p0_);
    side_[1 - s].line_to(p0_ - w1);
    n0_ = n1;
  }

  void cusp_curve_join(V n1) {                   // join_cusp (:638-647)
    int s = side_of(n0_, n1);
    V w1 = n1 * d_[s];
    cusp_join(side_[s], d_[s], d2_[s], w1);
    side_[1 - s].line_to(p0_ - w1);
    n0_ = n1;
  }

  void cusp_line_to(V n1, V p1) {                // join_cusp_and_line_to (:649-665)
    int s = side_of(n0_, n1);
    V w1 = n1 * d_[s];
    cusp_join(side_[s], d_[s], d2_[s], w1);
    side_[s].line_to(p1 + w1);
    side_[1 - s].line_to(p0_ - w1);
    side_[1 - s].line_to(p1 - w1);
    n0_ = n1; p0_ = p1;
  }

  void poly_to(const V* poly, size_t count) {   // smooth_poly_to (:667-694)
    V p1 = poly[0];
    V v1 = p1 - p0_;
    if (mag_sq(v1) < kLengthEpsilonSq) return;
    V n1 = unit_normal(v1);
    if (!open_) start_with_line(p1, n1);
    else line_to(p1, n1);
    for (size_t i = 1; i < count; i++) {
      p1 = poly[i];
      v1 = p1 - p0_;
      if (mag_sq(v1) < kLengthEpsilonSq) continue;
      cusp_line_to(unit_normal(v1), p1);
    }
  }

  void close_join(V n1) {                        // join_end_point (:697-734)
    if (n0_ == n1) {
      side_[0].drop(side_[0].prev_on());
      side_[1].drop(side_[1].prev_on());
      return;
    }
    int s = side_of(n0_, n1);
    V m = n0_ + n1;
    V w1 = n1 * d_[s];
    V k = m * d2_[s] / mag_sq(m);
    bool mitered = false;
    Side& outer = side_[s];
    outer_join(outer, n1, w1, k, d_[s], d2_[s], mitered);
    // a miter moves the figure's start to the miter point
    if (mitered && outer.cmd[1] == kOn) {
      outer.drop(1);
      outer.pt[0] = outer.last();
      outer.drop(outer.prev_on());
    }
    Side& inner = side_[1 - s];
    if (inner.cmd[1] <= kOn) {
      V corner = p0_ - k;
      if (inner.prev_on() && inside_overlap(inner.last(2), inner.last(), inner.pt[0], inner.pt[1], corner)) {
        inner.pt[0] = corner;
        inner.drop(1);
      }
      else {
        V first = inner.pt[0];
        inner.line_to(p0_);
        inner.line_to(first);
      }
    }
  }

  void offset_quad_piece(V q0, V q1, V q2) {    // offset_quad_simple (:885-905)
    if (q0 == q2) return;
    V v0 = q1 - q0, v1 = q2 - q1;
    V m0 = unit_normal(q0 != q1 ? v0 : v1);
    V m2 = unit_normal(q1 != q2 ? v1 : v0);
    p0_ = q2; n0_ = m2;
    V m = m0 + m2;
    V k1 = m * d2_[0] / mag_sq(m);
    V k2 = m2 * d_[0];
    side_[0].quad_to(q1 + k1, q2 + k2);
    side_[1].quad_to(q1 - k1, q2 - k2);
  }

  void offset_quad(const V* q) {                 // offset_quad (:860-883)
    double ts[3];
    size_t tn = quad_offset_cusps(q, d_[0], ts);
    ts[tn++] = 1.0;
    QuadPieces it(q, ts, tn);
    do {
      for (;;) {
        double t = quad_angle_step(it.piece, kOffsetParameter);
        if (!(t > kOffsetQuadEpsilonT && t < 1.0 - kOffsetQuadEpsilonT)) t = 1.0;
        V head[3];
        quad_split(it.piece, head, it.piece, t);
        offset_quad_piece(head[0], head[1], head[2]);
        if (t == 1.0) break;
      }
    } while (it.next());
  }

  void offset_cubic(const V* c) {                // approximate_cubic_with_quads (bezier_p.h:943-982)
    double tol = 54.0 * kSimplifyTolerance;
    double t = std::pow(tol * tol / mag_sq(c[3] - c[2] - (c[2] - c[1]) - (c[2] - c[1]) + (c[1] - c[0])), 1.0 / 6.0);
    V w[7];
    w[3] = c[0]; w[4] = c[1]; w[5] = c[2]; w[6] = c[3];
    for (;;) {
      V q[5];
      t = t < 1.0 ? t : 1.0;
      if (t >= 0.999) t = 1.0;
      cubic_split(w + 3, w, w + 3, t);
      cubic_two_quads(w, q);
      offset_quad(q);
      offset_quad(q + 2);
      if (t >= 1.0) return;
      double prev = t;
      t = t / (1.0 - t);
      if (prev - t < 1e-3) t += 0.01;
    }
  }

  void add_cap(Side& out, V pivot, V p1, uint32_t cap) {   // pathstroke.cpp:921-969
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

  void emit_figure(std::vector<uint8_t>& oc, std::vector<double>& ox);
};

// Appends A forward (without its CLOSE), then B backwards as EdgeSourceReversePathFromStrokeSink
// walks it (edgebuilder_p.h:287-405): the last on-point, then each segment reversed.
void append_forward(const Side& p, size_t first, std::vector<uint8_t>& oc, std::vector<double>& ox) {
  for (size_t i = first; i < p.size(); i++) {
    if (p.cmd[i] == kClose) break;
    oc.push_back(p.cmd[i]);
    ox.push_back(p.pt[i].x);
    ox.push_back(p.pt[i].y);
  }
}

// Returns false when B does not end with an on-point (the reference then adds no B edges).
bool append_reversed(const Side& b, bool with_move, std::vector<uint8_t>& oc, std::vector<double>& ox) {
  size_t n = b.size();
  if (n && b.cmd[n - 1] == kClose) n--;
  if (n == 0 || b.cmd[n - 1] != kOn) return false;
  size_t i = n - 1;
  auto put = [&](uint8_t c, V p) { oc.push_back(c); ox.push_back(p.x); ox.push_back(p.y); };
  if (with_move) put(kMove, b.pt[i]);
  while (i > 0) {
    uint8_t c = b.cmd[i - 1];
    if (c <= kOn) { put(kOn, b.pt[i - 1]); i -= 1; }
    else if (c == kQuad && i >= 2) { put(kQuad, b.pt[i - 1]); put(kOn, b.pt[i - 2]); i -= 2; }
    else if (c == kCubic && i >= 3) { put(kCubic, b.pt[i - 1]); put(kCubic, b.pt[i - 2]); put(kOn, b.pt[i - 3]); i -= 3; }
    else break;
  }
  return true;
}

void Stroker::emit_figure(std::vector<uint8_t>& oc, std::vector<double>& ox) {
  if (closed_) {
    append_forward(side_[0], 0, oc, ox);
    append_reversed(side_[1], true, oc, ox);
    return;
  }
  // A ends on B's last point, B (reversed) ends on its first point where C starts, C ends on
  // A's first point: one loop.
  append_forward(side_[0], 0, oc, ox);
  if (append_reversed(side_[1], false, oc, ox)) {
    append_forward(cap_, 1, oc, ox);
  }
  else {
    append_forward(cap_, 0, oc, ox);
  }
}

// PathStroker::stroke (pathstroke.cpp:224-487).
BLGpuResult Stroker::run(const uint8_t* cmd, const V* vtx, size_t n, std::vector<uint8_t>& oc, std::vector<double>& ox) {
  size_t i = 0;
  while (i < n) {
    if (cmd[i] != kMove) {
      if (cmd[i] != kClose) return BLGPU_ERROR_INVALID_GEOMETRY;
      i++;
      continue;
    }
    side_[0].clear();
    side_[1].clear();
    V poly[4];
    size_t poly_n = 0;
    p0_ = vtx[i];
    p_start_ = p0_;
    open_ = closed_ = false;
    i++;
    while (i < n) {
      uint8_t c = cmd[i];
      V p1 = vtx[i], v1, n1;
      if (c == kOn) {
        i++;
      line:
        v1 = p1 - p0_;
        if (mag_sq(v1) < kLengthEpsilonSq) continue;
        n1 = unit_normal(v1);
        if (!open_) { start_with_line(p1, n1); continue; }
        for (;;) {                               // a run of lines
          line_to(p1, n1);
          if (i >= n) break;
          c = cmd[i];
          p1 = vtx[i];
          if (c != kOn) break;
          i++;
          v1 = p1 - p0_;
          if (mag_sq(v1) < kLengthEpsilonSq) break;
          n1 = unit_normal(v1);
        }
        continue;
      poly:
        poly_to(poly, poly_n);
        continue;
      }
      else if (c == kQuad) {
        i += 2;
        if (i > n) return BLGPU_ERROR_INVALID_GEOMETRY;
        const V* q = vtx + i - 3;                // starts at the input's previous vertex
        V p2 = q[2];
        V v2 = p2 - p1;
        v1 = p1 - p0_;
        n1 = unit_normal(v1);
        if (std::fabs(cross(v2, v1)) <= kCollinearityEpsilon) {
          if (dot(-v1, v2) > 0.0) {              // control point outside: a cusp
            double r1 = dot(p1 - p0_, v1);
            double r2 = dot(p2 - p0_, v1);
            double t = r1 / (2.0 * r1 - r2);
            if (t > 0.0 && t < 1.0) {
              poly[0] = quad_point(q, t);
              poly[1] = p2;
              poly_n = 2;
              goto poly;
            }
          }
          p1 = p2;
          goto line;
        }
        if (mag_sq(v1) < kLengthEpsilonSq || mag_sq(v2) < kLengthEpsilonSq) { p1 = p2; goto line; }
        if (!open_) start_with_curve(n1);
        else curve_join(n1);
        offset_quad(q);
      }
      else if (c == kCubic) {
        i += 3;
        if (i > n) return BLGPU_ERROR_INVALID_GEOMETRY;
        V p[7];
        p[0] = p0_; p[1] = vtx[i - 3]; p[2] = vtx[i - 2]; p[3] = vtx[i - 1];
        int cusp = 0;
        if (cubic_is_flat(p, kDegenerateFlatness)) {
          double dot1 = dot(p[0] - p[1], p[3] - p[1]);
          double dot2 = dot(p[0] - p[2], p[3] - p[2]);
          if (!(dot1 < 0.0) || !(dot2 < 0.0)) {  // flat with the controls outside: cusps
            V r = cubic_start_dir(p);
            double r1 = dot(p[1] - p[0], r), r2 = dot(p[2] - p[0], r), r3 = dot(p[3] - p[0], r);
            double a = 1.0 / (3.0 * r1 - 3.0 * r2 + r3);
            double b = 2.0 * r1 - r2;
            double s = std::sqrt(r2 * (r2 - r1) - r1 * (r3 - r1));
            double t1 = a * (b - s), t2 = a * (b + s);
            poly_n = 0;
            if (t1 > kCuspTThreshold && t1 < 1.0 - kCuspTThreshold) poly[poly_n++] = cubic_point(p, t1);
            if (t2 > kCuspTThreshold && t2 < 1.0 - kCuspTThreshold) poly[poly_n++] = cubic_point(p, t2);
            if (poly_n == 0) { p1 = p[3]; goto line; }
            poly[poly_n++] = p[3];
            goto poly;
          }
          p1 = p[3];
          goto line;
        }
        double tc, tl;
        cubic_inflections(p, tc, tl);
        if (tl == 0.0 && tc > 0.0 && tc < 1.0) {  // a cusp: the two halves, joined round
          cubic_halve(p, p, p + 3);
          cusp = 1;
        }
        for (;;) {
          v1 = p[1] - p0_;
          if (is_zero(v1)) v1 = p[2] - p0_;
          n1 = unit_normal(v1);
          if (!open_) start_with_curve(n1);
          else if (cusp >= 0) curve_join(n1);
          else cusp_curve_join(n1);
          offset_cubic(p);
          if (cusp <= 0) break;
          cusp = -1;
          p[0] = p[3]; p[1] = p[4]; p[2] = p[5]; p[3] = p[6];
        }
      }
      else {
        if (closed_ || c != kClose) break;
        closed_ = true;
        p1 = p_start_;
        goto line;
      }
    }
    i += closed_ ? 1 : 0;
    if (!open_) continue;
    if (closed_) {
      close_join(n_start_);
      side_[0].close();
      side_[1].close();
      cap_.clear();
    }
    else {
      uint32_t start_cap = opt_.start_cap <= kCapTriangleRev ? opt_.start_cap : kCapButt;
      uint32_t end_cap = opt_.end_cap <= kCapTriangleRev ? opt_.end_cap : kCapButt;
      add_cap(side_[0], p0_, side_[1].last(), end_cap);
      cap_.clear();
      cap_.move_to(side_[1].pt[0]);
      add_cap(cap_, p_start_, side_[0].pt[0], start_cap);
    }
    emit_figure(oc, ox);
  }
  return BLGPU_SUCCESS;
}

}  // namespace

BLGpuResult stroke_outline(const uint8_t* cmds, const double* xy, size_t n, const StrokeParams& p,
                           std::vector<uint8_t>& out_cmds, std::vector<double>& out_xy) {
  const size_t c0 = out_cmds.size(), x0 = out_xy.size();
  Stroker s(p);
  BLGpuResult r = s.run(cmds, reinterpret_cast<const V*>(xy), n, out_cmds, out_xy);
  if (r != BLGPU_SUCCESS) {
    out_cmds.resize(c0);
    out_xy.resize(x0);
  }
  return r;
}

}  // namespace blgpu
