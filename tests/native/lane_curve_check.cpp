// Host build of the device edge builder (edge_build.cuh) checking that the lane-stepped curve
// flattener (eb::LaneCurve, one subdivision step per call) emits exactly the segments, in the same
// order, as the loop flattener (eb::curve_to, with the plain local stack) for random cubic, quadratic and conic curves around
// and across the clip box. Usage: lane_curve_check <seed> <curves>; exit status 0 when all match.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <tuple>
#include <vector>

#define __device__
#define __forceinline__ inline
using std::max;
using std::min;
static inline long long __double_as_longlong(double x) { long long v; memcpy(&v, &x, 8); return v; }
static inline int __double2hiint(double x) { return int(uint64_t(__double_as_longlong(x)) >> 32); }
static inline int __double2loint(double x) { return int(uint32_t(uint64_t(__double_as_longlong(x)))); }
static inline double __hiloint2double(int hi, int lo) {
  const uint64_t b = (uint64_t(uint32_t(hi)) << 32) | uint32_t(lo);
  double v; memcpy(&v, &b, 8); return v;
}
static inline uint32_t atomicAdd(uint32_t* p, uint32_t v) { uint32_t o = *p; *p += v; return o; }
#include "edge_build.cuh"

using namespace blgpu;
using namespace blgpu::eb;

struct Out { std::vector<DevSeg> segs; std::vector<uint32_t> meta; uint32_t counter = 0; };

static void init_builder(Builder& b, double w, double h, Out& o) {
  b.cx0 = 0.0; b.cy0 = 0.0; b.cx1 = w * 256.0; b.cy1 = h * 256.0;
  b.icx0 = trunc_i(b.cx0); b.icx1 = trunc_i(b.cx1);
  const double tol = 0.20 * 256.0;
  b.tol_sq = tol * tol;
  b.acc_x0_y0 = b.acc_x0_y1 = b.acc_x1_y0 = b.acc_x1_y1 = b.cy0;
  b.px = b.py = 0; b.psign = 0; b.pasc = false;
  if (o.segs.empty()) { o.segs.resize(1 << 14); o.meta.resize(1 << 14); }
  o.counter = 0;
  b.sink.init(o.segs.data(), o.meta.data(), &o.counter, 1u << 14, 7u);
}

// S: the lane flattener's stack (the kernels use CachedStack, the top entry in registers).
template<int DEG, class S>
static bool same_segments(const double* xy, const uint8_t* cmd, int npts, bool conic, double w, double h) {
  Src src;
  src.xy = xy; src.cmd = cmd; src.affine = false;
  src.m00 = 256.0; src.m01 = 0.0; src.m10 = 0.0; src.m11 = 256.0; src.m20 = 0.0; src.m21 = 0.0;

  static Out o1, o2;
  Builder b1;
  init_builder(b1, w, h, o1);
  Pt p0 = src.tf(0);
  uint32_t f0 = b1.fxy(p0);
  src.i = 1; src.n = npts;
  curve_to<DEG>(b1, src, p0, f0, conic);
  b1.done(); b1.sink.flush();

  Builder b2;
  init_builder(b2, w, h, o2);
  LaneCurve<DEG, S> lc;
  const Pt q0 = src.tf(0);
  lc.spline[1] = src.tf(1);
  if (DEG == 3) { lc.spline[2] = src.tf(2); lc.spline[3] = src.tf(3); }
  else lc.spline[DEG] = src.tf(conic ? 3 : 2);
  bool busy = lc.begin_curve(b2, q0, b2.fxy(q0));
  for (long guard = 0; busy; guard++) {
    if (guard > 10000000) return false;
    lc.step(b2);
    if (lc.state == kLsDone && !lc.next_piece(b2, true)) busy = false;
  }
  b2.done(); b2.sink.flush();

  if (o1.counter != o2.counter || o1.counter > (1u << 14)) return false;
  for (uint32_t i = 0; i < o1.counter; i++) {
    const DevSeg &a = o1.segs[i], &c = o2.segs[i];
    if (a.x0 != c.x0 || a.y0 != c.y0 || a.x1 != c.x1 || a.y1 != c.y1 || o1.meta[i] != o2.meta[i]) return false;
  }
  return true;
}

// The subdivision trees of the tree kernel (edge_tree_kernel) for curves inside the clip box: every
// monotonic piece's tree (eb::tree_root / tree_step) walked in a random order, as lanes sharing
// nodes would, must give the loop flattener's segments, as a multiset. Returns 1 when the curve was
// inside the box and matched, 0 when it was not inside, -1 on a mismatch.
template<int DEG>
static int same_segments_tree(const double* xy, const uint8_t* cmd, int npts, double w, double h, std::mt19937_64& rng) {
  Src src;
  src.xy = xy; src.cmd = cmd; src.affine = false;
  src.m00 = 256.0; src.m01 = 0.0; src.m10 = 0.0; src.m11 = 256.0; src.m20 = 0.0; src.m21 = 0.0;
  static Out o1;
  Builder b1;
  init_builder(b1, w, h, o1);
  Pt p0 = src.tf(0);
  uint32_t f0 = b1.fxy(p0);
  const Pt q0 = p0;
  src.i = 1; src.n = npts;
  curve_to<DEG>(b1, src, p0, f0, false);
  b1.done(); b1.sink.flush();

  Builder b2;
  static Out o2;
  init_builder(b2, w, h, o2);
  LaneCurve<DEG, LocalStack<DEG>> lc;
  lc.spline[1] = src.tf(1);
  if (DEG == 3) { lc.spline[2] = src.tf(2); lc.spline[3] = src.tf(3); }
  else lc.spline[DEG] = src.tf(2);
  if (!lc.prepare(b2, q0, b2.fxy(q0)) || lc.any) return 0;
  struct Seg { int x0, y0, x1, y1; uint32_t meta; };
  std::vector<Seg> want, got;
  for (uint32_t i = 0; i < o1.counter; i++)
    want.push_back(Seg{o1.segs[i].x0, o1.segs[i].y0, o1.segs[i].x1, o1.segs[i].y1, o1.meta[i]});
  for (int piece = 0; piece < lc.nout; piece += DEG) {
    uint32_t sign = 0;
    std::vector<TreeNode<DEG>> pending{tree_root<DEG>(lc.spline + piece, sign)};
    for (long guard = 0; !pending.empty(); guard++) {
      if (guard > 10000000) return -1;
      const size_t pick = size_t(rng() % pending.size());
      const TreeNode<DEG> n = pending[pick];
      pending[pick] = pending.back();
      pending.pop_back();
      TreeNode<DEG> l, r;
      if (tree_step<DEG>(n, b2.tol_sq, l, r)) {
        const int x0 = trunc_i(n.p[0].x), y0 = trunc_i(n.p[0].y), x1 = trunc_i(n.p[DEG].x), y1 = trunc_i(n.p[DEG].y);
        if (y0 != y1) got.push_back(Seg{x0, y0, x1, y1, (7u << 1) | sign});
      }
      else {
        pending.push_back(l);
        pending.push_back(r);
      }
    }
  }
  auto key = [](const Seg& s) { return std::make_tuple(s.x0, s.y0, s.x1, s.y1, s.meta); };
  std::sort(want.begin(), want.end(), [&](const Seg& a, const Seg& c) { return key(a) < key(c); });
  std::sort(got.begin(), got.end(), [&](const Seg& a, const Seg& c) { return key(a) < key(c); });
  if (want.size() != got.size()) return -1;
  for (size_t i = 0; i < want.size(); i++)
    if (key(want[i]) != key(got[i])) return -1;
  return 1;
}

// Pieces routed to the tree flattener (eb::piece_flattens_safe), including pieces of clipped
// curves: each must give, as a multiset, the segments the lane flattener gives for it alone with a
// builder of its own (as edge_pieces_kernel runs it). Returns the number of routed pieces of
// clipped curves compared, or -1 on a mismatch.
static int same_segments_routed(const double* xy, const uint8_t* cmd, double w, double h, std::mt19937_64& rng) {
  Src src;
  src.xy = xy; src.cmd = cmd; src.affine = false;
  src.m00 = 256.0; src.m01 = 0.0; src.m10 = 0.0; src.m11 = 256.0; src.m20 = 0.0; src.m21 = 0.0;
  static Out ob, oa;
  Builder b;
  init_builder(b, w, h, ob);
  LaneCurve<3, CachedStack<3>> lc;
  const Pt q0 = src.tf(0);
  lc.spline[1] = src.tf(1); lc.spline[2] = src.tf(2); lc.spline[3] = src.tf(3);
  if (!lc.prepare(b, q0, b.fxy(q0))) return 0;
  int routed_clipped = 0;
  struct Seg { int x0, y0, x1, y1; uint32_t meta; };
  auto key = [](const Seg& s) { return std::make_tuple(s.x0, s.y0, s.x1, s.y1, s.meta); };
  for (int piece = 0; piece < lc.nout; piece += 3) {
    const Pt* pts = lc.spline + piece;
    if (!piece_flattens_safe(pts, 3, lc.any, b)) continue;
    Builder ba;
    init_builder(ba, w, h, oa);
    LaneCurve<3, CachedStack<3>> la;
    bool busy = la.begin_piece(ba, pts, lc.any);
    for (long guard = 0; busy; guard++) {
      if (guard > 10000000) return -1;
      la.step(ba);
      if (la.state == kLsDone && !la.next_piece(ba, true)) busy = false;
    }
    ba.done(); ba.sink.flush();
    std::vector<Seg> want, got;
    for (uint32_t i = 0; i < oa.counter; i++)
      want.push_back(Seg{oa.segs[i].x0, oa.segs[i].y0, oa.segs[i].x1, oa.segs[i].y1, oa.meta[i]});
    uint32_t sign = 0;
    std::vector<TreeNode<3>> pending{tree_root<3>(pts, sign)};
    for (long guard = 0; !pending.empty(); guard++) {
      if (guard > 10000000) return -1;
      const size_t pick = size_t(rng() % pending.size());
      const TreeNode<3> n = pending[pick];
      pending[pick] = pending.back();
      pending.pop_back();
      TreeNode<3> l, r;
      if (tree_step<3>(n, b.tol_sq, l, r)) {
        const int x0 = trunc_i(n.p[0].x), y0 = trunc_i(n.p[0].y), x1 = trunc_i(n.p[3].x), y1 = trunc_i(n.p[3].y);
        if (y0 != y1) got.push_back(Seg{x0, y0, x1, y1, (7u << 1) | sign});
      }
      else {
        pending.push_back(l);
        pending.push_back(r);
      }
    }
    std::sort(want.begin(), want.end(), [&](const Seg& a, const Seg& c) { return key(a) < key(c); });
    std::sort(got.begin(), got.end(), [&](const Seg& a, const Seg& c) { return key(a) < key(c); });
    if (want.size() != got.size()) return -1;
    for (size_t i = 0; i < want.size(); i++)
      if (key(want[i]) != key(got[i])) return -1;
    if (lc.any) routed_clipped++;
  }
  return routed_clipped;
}

int main(int argc, char** argv) {
  std::mt19937_64 rng(argc > 1 ? strtoull(argv[1], nullptr, 10) : 1);
  const int n = argc > 2 ? atoi(argv[2]) : 100000;
  std::uniform_real_distribution<double> u(0.0, 1.0);
  long fails = 0;
  // half_exp against the multiply, wherever it claims to be exact
  {
    const double specials[] = {0.0, -0.0, 1.0, -1.0, 5e-324, 2.2250738585072014e-308, 4.4501477170144028e-308,
                               1.7976931348623157e308, INFINITY, -INFINITY, NAN, 3.0, 0.75, 65536.0 * 256.0};
    long bad = 0, fast = 0;
    auto one = [&](double v) {
      bool ok = true;
      const double h = half_exp(v, ok);
      const double m = v * 0.5;
      if (ok) { fast++; if (memcmp(&h, &m, 8) != 0) bad++; }
    };
    for (double v : specials) one(v);
    for (int i = 0; i < 2000000; i++) {
      const uint64_t b = rng();
      double v; memcpy(&v, &b, 8);
      one(v);
      one(u(rng) * 1e7 - 5e6);
    }
    printf("half_exp: %ld fast of %d, %ld differ from the multiply\n", fast, 4000000 + 14, bad);
    if (bad) return 1;
  }
  for (int it = 0; it < n; it++) {
    const bool cached = (it & 4) != 0;           // half the curves with each stack
    const double w = 16 + std::floor(u(rng) * 200), h = 16 + std::floor(u(rng) * 200);
    // mostly around the canvas; some points on its borders, on the pixel grid, or far outside
    auto coord = [&](double lim) {
      const double r = u(rng);
      if (r < 0.08) return 0.0;
      if (r < 0.16) return lim;
      if (r < 0.22) return std::floor(u(rng) * lim);
      if (r < 0.26) return -1e6 + 2e6 * u(rng);
      if (r < 0.6) return std::floor(-0.25 * lim + 1.5 * lim * u(rng)) + (u(rng) < 0.5 ? 0.5 : 0.0);
      return -0.5 * lim + 2.0 * lim * u(rng);
    };
    double xy[8];
    for (int k = 0; k < 4; k++) { xy[2 * k] = coord(w); xy[2 * k + 1] = coord(h); }
    if (u(rng) < 0.1) xy[2] = xy[0];
    if (u(rng) < 0.05) xy[7] = xy[1];
    bool ok;
    if (it % 3 == 0) {
      const uint8_t c[4] = {0, 4, 4, 4};
      ok = cached ? same_segments<3, CachedStack<3>>(xy, c, 4, false, w, h) : same_segments<3, LocalStack<3>>(xy, c, 4, false, w, h);
    }
    else if (it % 3 == 1) {
      const uint8_t c[3] = {0, 2, 2};
      ok = cached ? same_segments<2, CachedStack<2>>(xy, c, 3, false, w, h) : same_segments<2, LocalStack<2>>(xy, c, 3, false, w, h);
    }
    else {
      const uint8_t c[4] = {0, 3, 3, 3};
      const double cx[8] = {xy[0], xy[1], xy[2], xy[3], 1.0, 0.0, xy[4], xy[5]};
      ok = cached ? same_segments<2, CachedStack<2>>(cx, c, 4, true, w, h) : same_segments<2, LocalStack<2>>(cx, c, 4, true, w, h);
    }
    if (!ok && ++fails <= 5) printf("mismatch: curve %d (kind %d)\n", it, it % 3);
  }
  // curves inside the clip box (points anywhere on the canvas, borders included) as subdivision
  // trees walked in a random order, cubic and quadratic
  long safe_tested = 0;
  for (int it = 0; it < n; it++) {
    const double span = (it % 4 == 0) ? 4000.0 : 200.0;     // some large curves: deep trees
    const double w = 16 + std::floor(u(rng) * span), h = 16 + std::floor(u(rng) * span);
    auto inside = [&](double lim) {
      const double r = u(rng);
      if (r < 0.05) return 0.0;
      if (r < 0.1) return lim;
      if (r < 0.3) return std::floor(u(rng) * lim) + (u(rng) < 0.5 ? 0.5 : 0.0);
      return lim * u(rng);
    };
    double xy[8];
    for (int k = 0; k < 4; k++) { xy[2 * k] = inside(w); xy[2 * k + 1] = inside(h); }
    if (u(rng) < 0.1) xy[2] = xy[0];
    int r;
    if (it & 1) {
      const uint8_t c[4] = {0, 4, 4, 4};
      r = same_segments_tree<3>(xy, c, 4, w, h, rng);
    }
    else {
      const uint8_t c[3] = {0, 2, 2};
      r = same_segments_tree<2>(xy, c, 3, w, h, rng);
    }
    if (r > 0) safe_tested++;
    if (r < 0 && ++fails <= 10) printf("mismatch: safe curve %d\n", it);
  }
  printf("safe curves %ld\n", safe_tested);
  // cubic curves around and across the clip box: the pieces routed to the tree flattener
  long routed = 0;
  for (int it = 0; it < n; it++) {
    const double w = 16 + std::floor(u(rng) * 200), h = 16 + std::floor(u(rng) * 200);
    auto coord = [&](double lim) {
      const double r = u(rng);
      if (r < 0.08) return 0.0;
      if (r < 0.16) return lim;
      if (r < 0.22) return std::floor(u(rng) * lim);
      if (r < 0.26) return -1e6 + 2e6 * u(rng);
      if (r < 0.6) return std::floor(-0.25 * lim + 1.5 * lim * u(rng)) + (u(rng) < 0.5 ? 0.5 : 0.0);
      return -0.5 * lim + 2.0 * lim * u(rng);
    };
    double xy[8];
    for (int k = 0; k < 4; k++) { xy[2 * k] = coord(w); xy[2 * k + 1] = coord(h); }
    if (u(rng) < 0.1) xy[2] = xy[0];
    const uint8_t c[4] = {0, 4, 4, 4};
    const int r = same_segments_routed(xy, c, w, h, rng);
    if (r < 0 && ++fails <= 15) printf("mismatch: routed piece of curve %d\n", it);
    if (r > 0) routed += r;
  }
  printf("routed pieces of clipped curves %ld\n", routed);
  printf("curves %d mismatches %ld\n", n, fails);
  return fails ? 1 : 0;
}
