/*
 * b2d_oracle_stroke.c - CPU oracle (test infrastructure only): the reference's path stroker.
 *
 * Restates bl::PathInternal::PathStroker (blend2d/core/pathstroke.cpp:126-971) and the Bezier
 * helpers it calls (blend2d/geometry/bezier_p.h, blend2d/geometry/commons_p.h), operation by
 * operation in double precision without FMA contraction, so the A/B/C outline paths it hands to
 * the sink are the reference's to the bit on x86-64. The output appenders follow PathAppender
 * (blend2d/core/path_p.h:191-418): the stroker patches and removes vertices it has already
 * written (`back`, `vtx[-1] = ...`), so they are plain arrays with a size.
 */
#include "b2d_oracle_p.h"
#include "b2d_oracle_stroke.h"

enum { P_MOVE = 0, P_ON = 1, P_QUAD = 2, P_CONIC = 3, P_CUBIC = 4, P_CLOSE = 5 };

/* pathstroke.cpp:22-47 */
static const double kMiterMinimum = 1e-10;
static const double kLengthEpsilonSq = 1e-10 * 1e-10;
static const double kCollinearityEpsilon = 1e-10;
static const double kCuspTThreshold = 1e-10;
static const double kDegenerateFlatness = 1e-6;
static const double kOffsetQuadEpsilonT = 1e-5;
static const double kKappa = 0.55228474983;   /* mathconst_p.h:52 */

/* --- point arithmetic (BLPoint operators, commons_p.h:63-77) ------------------------------- */

static inline OPt P(double x, double y) { OPt r = { x, y }; return r; }
static inline OPt padd(OPt a, OPt b) { return P(a.x + b.x, a.y + b.y); }
static inline OPt psub(OPt a, OPt b) { return P(a.x - b.x, a.y - b.y); }
static inline OPt pmul(OPt a, double s) { return P(a.x * s, a.y * s); }
static inline OPt smul(double s, OPt a) { return P(s * a.x, s * a.y); }
static inline OPt pdiv(OPt a, double s) { return P(a.x / s, a.y / s); }
static inline OPt pneg(OPt a) { return P(-a.x, -a.y); }
static inline int peq(OPt a, OPt b) { return a.x == b.x && a.y == b.y; }
static inline double dot(OPt a, OPt b) { return a.x * b.x + a.y * b.y; }
static inline double cross(OPt a, OPt b) { return a.x * b.y - a.y * b.x; }
static inline double mag_sq(OPt v) { return v.x * v.x + v.y * v.y; }
static inline double mag(OPt v) { return sqrt(mag_sq(v)); }
static inline double length(OPt a, OPt b) { return sqrt(mag_sq(psub(b, a))); }
static inline OPt normal(OPt v) { return P(-v.y, v.x); }
static inline OPt unit_vector(OPt v) { return pdiv(v, mag(v)); }
static inline int is_zero(OPt p) { return (p.x == 0) & (p.y == 0); }
/* Math::lerp: (a - t * a) + t * b, and 0.5 * a + 0.5 * b at t = 0.5 (math_p.h:512-520). */
static inline OPt lerp_t(OPt a, OPt b, double t) { return padd(psub(a, smul(t, a)), smul(t, b)); }
static inline OPt lerp_h(OPt a, OPt b) { return padd(smul(0.5, a), smul(0.5, b)); }
static inline OPt pmin(OPt a, OPt b) { return P(b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y); }
static inline OPt pmax(OPt a, OPt b) { return P(a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y); }

/* --- Bezier helpers (bezier_p.h) ------------------------------------------------------------ */

static OPt quad_eval(const OPt* q, double t) {            /* coefficients_of + evaluate, :190, :207 */
  OPt v1 = psub(q[1], q[0]), v2 = psub(q[2], q[1]);
  OPt a = psub(v2, v1), b = padd(v1, v1), c = q[0];
  return padd(pmul(padd(pmul(a, t), b), t), c);
}

static void quad_deriv(const OPt* q, OPt* a, OPt* b) {    /* derivative_coefficients_of, :197 */
  OPt v1 = psub(q[1], q[0]), v2 = psub(q[2], q[1]);
  *a = psub(smul(2.0, v2), smul(2.0, v1));
  *b = smul(2.0, v1);
}

static double quad_parameter_at_angle(const OPt* q, double m) {   /* :237-253 */
  OPt a, b;
  quad_deriv(q, &a, &b);
  double aob = dot(a, b), axb = cross(a, b);
  if (aob == 0.0) return 1.0;
  return m * mag_sq(b) / (fabs(axb) - m * aob);
}

static size_t quad_offset_cusp_ts(const OPt* q, double d, double t_out[3]) {   /* :255-281 */
  OPt a, b;
  quad_deriv(q, &a, &b);
  double bxa = cross(b, a), boa = dot(b, a);
  if (bxa == 0.0) return 0;
  double alen2 = mag_sq(a), blen2 = mag_sq(b);
  double fac = -1.0 / alen2;
  double sq = sqrt(boa * boa - alen2 * (blen2 - cbrt(d * d * bxa * bxa)));
  double t0 = fac * (boa + sq);
  double t1 = fac * (boa - sq);
  t0 = t0 < 0.0 ? 0.0 : t0;                                 /* bl_max(t0, 0.0) */
  size_t n = (size_t)(t0 > 0.0 && t0 < 1.0);
  t_out[0] = t0;
  t_out[n] = t1;
  return n + (size_t)(t1 > t0 && t1 < 1.0);
}

static void quad_split_t(const OPt* c, OPt* a_out, OPt* b_out, double t) {   /* :296-307 */
  OPt cp0 = c[0], cp1 = c[1], cp2 = c[2];
  OPt p01 = lerp_t(cp0, cp1, t), p12 = lerp_t(cp1, cp2, t), m = lerp_t(p01, p12, t);
  a_out[0] = cp0; a_out[1] = p01; a_out[2] = m;
  b_out[0] = m; b_out[1] = p12; b_out[2] = cp2;
}

/* QuadCurveTsIter (:402-448). */
typedef struct { const double* ts; const double* ts_end; OPt in[3]; OPt part[3]; OPt t01, t12; } QuadTsIter;

static void qti_reset(QuadTsIter* it, const OPt* q, const double* ts, size_t n) {
  it->in[0] = q[0]; it->in[1] = q[1]; it->in[2] = q[2];
  it->ts = ts; it->ts_end = ts + n;
  double t = *it->ts++;
  it->t01 = lerp_t(it->in[0], it->in[1], t);
  it->t12 = lerp_t(it->in[1], it->in[2], t);
  it->part[0] = it->in[0]; it->part[1] = it->t01; it->part[2] = lerp_t(it->t01, it->t12, t);
}

static int qti_next(QuadTsIter* it) {
  if (it->ts >= it->ts_end) return 0;
  double t = *it->ts++;
  it->part[0] = it->part[2];
  it->part[1] = lerp_t(it->t01, it->t12, t);
  it->t01 = lerp_t(it->in[0], it->in[1], t);
  it->t12 = lerp_t(it->in[1], it->in[2], t);
  it->part[2] = lerp_t(it->t01, it->t12, t);
  return 1;
}

static OPt cubic_eval(const OPt* c, double t) {           /* coefficients_of + evaluate, :617-654 */
  OPt v1 = psub(c[1], c[0]), v2 = psub(c[2], c[1]), v3 = psub(c[3], c[2]);
  OPt a = padd(psub(psub(v3, v2), v2), v1);
  OPt b = smul(3.0, psub(v2, v1));
  OPt cc = smul(3.0, v1);
  return padd(pmul(padd(pmul(padd(pmul(a, t), b), t), cc), t), c[0]);
}

static OPt cubic_identity(const OPt* c) {                 /* :700-706 */
  OPt v1 = psub(c[1], c[0]), v2 = psub(c[2], c[1]), v3 = psub(c[3], c[2]);
  return padd(psub(psub(v3, v2), v2), v1);
}

static int is_cubic_flat(const OPt* c, double f) {         /* :708-720 */
  if (peq(c[3], c[0])) {
    OPt v = psub(c[2], c[1]);
    double a = cross(v, psub(c[1], c[0]));
    return 0.5625 * a * a <= f * f * mag_sq(v);
  }
  OPt v = psub(c[3], c[0]);
  double a1 = cross(v, psub(c[1], c[0]));
  double a2 = cross(v, psub(c[2], c[0]));
  double a1s = a1 * a1, a2s = a2 * a2;
  return 0.5625 * (a1s < a2s ? a2s : a1s) <= f * f * mag_sq(v);
}

static void cubic_inflection_parameter(const OPt* c, double* tc, double* tl) {   /* :722-745 */
  OPt v1 = psub(c[1], c[0]), v2 = psub(c[2], c[1]), v3 = psub(c[3], c[2]);
  OPt da = smul(3.0, padd(psub(psub(v3, v2), v2), v1));
  OPt db = smul(6.0, psub(v2, v1));
  OPt dc = smul(3.0, v1);
  double den = cross(db, da);
  if (den != 0) {
    *tc = cross(da, dc) / den;
    *tl = *tc * *tc + cross(db, dc) / den;
    if (*tl > 0) *tl = sqrt(*tl);
  }
  else {
    *tc = -0.5 * cross(dc, db) / cross(dc, da);
    *tl = NAN;
  }
}

static OPt cubic_start_tangent(const OPt* c) {            /* :747-756 */
  OPt out = psub(c[1], c[0]), t20 = psub(c[2], c[0]), t30 = psub(c[3], c[0]);
  if (is_zero(out)) out = t20;
  if (is_zero(out)) out = t30;
  return out;
}

static OPt cubic_end_tangent(const OPt* c) {              /* :758-767 */
  OPt out = psub(c[3], c[2]), t31 = psub(c[3], c[1]), t30 = psub(c[3], c[0]);
  if (is_zero(out)) out = t31;
  if (is_zero(out)) out = t30;
  return out;
}

static OPt cubic_derivative_at(const OPt* c, double t) {  /* :675-681 */
  OPt p01 = lerp_t(c[0], c[1], t), p12 = lerp_t(c[1], c[2], t), p23 = lerp_t(c[2], c[3], t);
  return smul(3.0, psub(lerp_t(p12, p23, t), lerp_t(p01, p12, t)));
}

/* split at 0.5 (:769-783) and at t (:785-799): every output computed from the inputs first, so
 * the in-place uses (a = curve, b = curve + 3) are safe. */
static void cubic_split_half(const OPt* c, OPt* a, OPt* b) {
  OPt c0 = c[0], c3 = c[3];
  OPt p01 = lerp_h(c[0], c[1]), p12 = lerp_h(c[1], c[2]), p23 = lerp_h(c[2], c[3]);
  OPt a2 = lerp_h(p01, p12), b1 = lerp_h(p12, p23), m = lerp_h(a2, b1);
  a[0] = c0; a[1] = p01; a[2] = a2; a[3] = m;
  b[0] = m; b[1] = b1; b[2] = p23; b[3] = c3;
}

static void cubic_split_t(const OPt* c, OPt* a, OPt* b, double t) {
  OPt c0 = c[0], c3 = c[3];
  OPt p01 = lerp_t(c[0], c[1], t), p12 = lerp_t(c[1], c[2], t), p23 = lerp_t(c[2], c[3], t);
  OPt a2 = lerp_t(p01, p12, t), b1 = lerp_t(p12, p23, t), m = lerp_t(a2, b1, t);
  a[0] = c0; a[1] = p01; a[2] = a2; a[3] = m;
  b[0] = m; b[1] = b1; b[2] = p23; b[3] = c3;
}

static OPt line_vector_intersection(OPt p0, OPt v0, OPt p1, OPt v1) {   /* commons_p.h:75-77 */
  return padd(p0, smul(cross(psub(p1, p0), v1) / cross(v0, v1), v0));
}

static void cubic_to_two_quads(const OPt* c, OPt q[5]) {  /* :922-940 */
  OPt c1 = lerp_t(c[0], c[1], 0.75);
  OPt c2 = lerp_t(c[3], c[2], 0.75);
  OPt pm = lerp_h(c1, c2);
  if (peq(c1, c[0])) c1 = line_vector_intersection(c[0], cubic_start_tangent(c), pm, cubic_derivative_at(c, 0.5));
  if (peq(c2, c[3])) c2 = line_vector_intersection(c[3], cubic_end_tangent(c), pm, cubic_derivative_at(c, 0.5));
  q[0] = c[0]; q[1] = c1; q[2] = pm; q[3] = c2; q[4] = c[3];
}

/* --- output paths (PathAppender) -------------------------------------------------------------- */

void o_path_reserve(OPath* p, size_t extra) {
  if (p->n + extra <= p->cap) return;
  size_t cap = p->cap ? p->cap * 2 : 64;
  while (cap < p->n + extra) cap *= 2;
  p->cmd = (uint8_t*)realloc(p->cmd, cap);
  p->vtx = (OPt*)realloc(p->vtx, cap * sizeof(OPt));
  p->cap = cap;
}
void o_path_free(OPath* p) { free(p->cmd); free(p->vtx); memset(p, 0, sizeof(*p)); }

static inline void put(OPath* p, uint8_t c, OPt v) { o_path_reserve(p, 1); p->cmd[p->n] = c; p->vtx[p->n] = v; p->n++; }
static inline void move_to(OPath* p, OPt v) { put(p, P_MOVE, v); }
static inline void line_to(OPath* p, OPt v) { put(p, P_ON, v); }
static inline void quad_to(OPath* p, OPt a, OPt b) { put(p, P_QUAD, a); put(p, P_ON, b); }
static inline void cubic_to(OPath* p, OPt a, OPt b, OPt c) { put(p, P_CUBIC, a); put(p, P_CUBIC, b); put(p, P_ON, c); }
static inline void close_path(OPath* p) { put(p, P_CLOSE, P(NAN, NAN)); }
static inline void back(OPath* p, size_t n) { p->n -= n; }
static inline OPt vtx_back(const OPath* p, size_t k) { return p->vtx[p->n - k]; }
/* `cmd[-2].value <= BL_PATH_CMD_ON`; a path always holds at least a move and one more vertex
 * where the stroker asks. */
static inline int prev_is_on(const OPath* p) { return p->n >= 2 && p->cmd[p->n - 2] <= P_ON; }

static void arc_quadrant_to(OPath* p, OPt p1, OPt p2) {   /* path_p.h:374-390 */
  OPt p0 = vtx_back(p, 1);
  cubic_to(p, padd(p0, pmul(psub(p1, p0), kKappa)), padd(p2, pmul(psub(p1, p2), kKappa)), p2);
}

/* --- the stroker ------------------------------------------------------------------------------ */

enum { SIDE_A = 0, SIDE_B = 1 };
enum { JOIN_MITER_CLIP = 0, JOIN_MITER_BEVEL = 1, JOIN_MITER_ROUND = 2, JOIN_BEVEL = 3, JOIN_ROUND = 4 };
enum { CAP_BUTT = 0, CAP_SQUARE = 1, CAP_ROUND = 2, CAP_ROUND_REV = 3, CAP_TRIANGLE = 4, CAP_TRIANGLE_REV = 5 };

typedef struct {
  const OStrokeOpts* opt;
  double simplify_tolerance, offset_parameter;
  double miter_limit, miter_limit_sq;
  uint32_t join;
  OPath* side[2];              /* A (outer for positive offsets) and B */
  double d[2], d2[2];
  OPt p0, n0, p_initial, n_initial;
  int open, closed;
} Stroker;

static inline int side_from_normals(OPt n0, OPt n1) { return cross(n0, n1) >= 0 ? SIDE_B : SIDE_A; }

static int inner_join_test(OPt a0, OPt a1, OPt b0, OPt b1, OPt join) {   /* pathstroke.cpp:99-105 */
  OPt mn = pmax(pmin(a0, a1), pmin(b0, b1));
  OPt mx = pmin(pmax(a0, a1), pmax(b0, b1));
  return (join.x >= mn.x) & (join.y >= mn.y) & (join.x <= mx.x) & (join.y <= mx.y);
}

static void dull_angle_arc_to(OPath* out, OPt p0, OPt pa, OPt pb, OPt inter) {   /* :107-117 */
  OPt pm = pmul(padd(pa, pb), 0.5);
  double w = sqrt(mag(psub(p0, pm)) / mag(psub(p0, inter)));
  double a = 4 * w / (3.0 * (1.0 + w));
  cubic_to(out, padd(pa, smul(a, psub(inter, pa))), padd(pb, smul(a, psub(inter, pb))), pb);
}

/* outer_join (:769-838) */
static void outer_join(Stroker* s, OPath* out, OPt n1, OPt w1, OPt k, double d, double d2, int* miter_flag) {
  OPt pb = padd(s->p0, w1);
  if (mag_sq(k) <= s->miter_limit_sq) {
    back(out, (size_t)prev_is_on(out));
    line_to(out, padd(s->p0, k));
    line_to(out, pb);
    *miter_flag = 1;
    return;
  }
  if (s->join == JOIN_MITER_CLIP) {
    double b2 = fabs(cross(k, s->n0));
    if (b2 > 0) b2 = b2 * s->miter_limit / mag(k);
    else b2 = s->miter_limit;
    back(out, (size_t)prev_is_on(out));
    line_to(out, psub(padd(s->p0, smul(d, s->n0)), smul(b2, normal(s->n0))));
    line_to(out, padd(padd(s->p0, smul(d, n1)), smul(b2, normal(n1))));
    *miter_flag = 1;
    line_to(out, pb);
    return;
  }
  if (s->join == JOIN_ROUND) {
    OPt pa = vtx_back(out, 1);
    if (dot(psub(s->p0, pa), psub(s->p0, pb)) < 0.0) {
      OPt n2 = normal(unit_vector(psub(pb, pa)));
      OPt m = padd(s->n0, n2);
      OPt k0 = pdiv(smul(d2, m), mag_sq(m));
      OPt q = smul(d, n2);
      OPt pc1 = padd(s->p0, k0);
      OPt pp1 = padd(s->p0, q);
      OPt pc2 = lerp_t(pc1, pp1, 2.0);
      dull_angle_arc_to(out, s->p0, pa, pp1, pc1);
      dull_angle_arc_to(out, s->p0, pp1, pb, pc2);
    }
    else {
      OPt pm = lerp_h(pa, pb);
      OPt pi = padd(s->p0, k);
      double w = sqrt(length(s->p0, pm) / length(s->p0, pi));
      double a = 4.0 * w / (3.0 * (1.0 + w));
      cubic_to(out, padd(pa, smul(a, psub(pi, pa))), padd(pb, smul(a, psub(pi, pb))), pb);
    }
    return;
  }
  line_to(out, pb);   /* bevel */
}

/* dull_round_join (:841-860) */
static void dull_round_join(Stroker* s, OPath* out, double d, double d2, OPt w1) {
  OPt pa = vtx_back(out, 1);
  OPt pb = padd(s->p0, w1);
  OPt n2 = normal(unit_vector(psub(pb, pa)));
  if (!isfinite(n2.x)) return;
  OPt m = padd(s->n0, n2);
  OPt k = pdiv(pmul(m, d2), mag_sq(m));
  OPt q = pmul(n2, d);
  OPt pc1 = padd(s->p0, k);
  OPt pp1 = padd(s->p0, q);
  OPt pc2 = lerp_t(pc1, pp1, 2.0);
  dull_angle_arc_to(out, s->p0, pa, pp1, pc1);
  dull_angle_arc_to(out, s->p0, pp1, pb, pc2);
}

static void inner_join_line_to(Stroker* s, OPath* out, OPt l0, OPt l1, OPt inner_pt) {   /* :741-750 */
  if (prev_is_on(out) && inner_join_test(vtx_back(out, 2), vtx_back(out, 1), l0, l1, inner_pt)) {
    out->vtx[out->n - 1] = inner_pt;
  }
  else {
    line_to(out, s->p0);
    line_to(out, l0);
  }
}

static void open_line_to(Stroker* s, OPt p1, OPt n1) {   /* :540-556 */
  OPt w = pmul(n1, s->d[SIDE_A]);
  move_to(s->side[SIDE_A], padd(s->p0, w));
  move_to(s->side[SIDE_B], psub(s->p0, w));
  s->p0 = p1; s->n0 = n1; s->n_initial = n1;
  line_to(s->side[SIDE_A], padd(s->p0, w));
  line_to(s->side[SIDE_B], psub(s->p0, w));
  s->open = 1;
}

static void join_line_to(Stroker* s, OPt p1, OPt n1) {   /* :559-598 */
  if (peq(s->n0, n1)) {
    OPath* a = s->side[SIDE_A];
    OPath* b = s->side[SIDE_B];
    back(a, (size_t)prev_is_on(a));
    back(b, (size_t)prev_is_on(b));
    OPt w1 = pmul(n1, s->d[SIDE_A]);
    line_to(a, padd(p1, w1));
    line_to(b, psub(p1, w1));
  }
  else {
    int side = side_from_normals(s->n0, n1);
    OPt m = padd(s->n0, n1);
    OPt k = pdiv(pmul(m, s->d2[side]), mag_sq(m));
    OPt w1 = pmul(n1, s->d[side]);
    int miter_flag = 0;
    OPath* outer = s->side[side];
    OPath* inner = s->side[1 - side];
    outer_join(s, outer, n1, w1, k, s->d[side], s->d2[side], &miter_flag);
    back(outer, (size_t)miter_flag);
    line_to(outer, padd(p1, w1));
    inner_join_line_to(s, inner, psub(s->p0, w1), psub(p1, w1), psub(s->p0, k));
    line_to(inner, psub(p1, w1));
  }
  s->p0 = p1; s->n0 = n1;
}

static void open_curve(Stroker* s, OPt n0) {   /* :604-616 */
  OPt w = pmul(n0, s->d[SIDE_A]);
  move_to(s->side[SIDE_A], padd(s->p0, w));
  move_to(s->side[SIDE_B], psub(s->p0, w));
  s->n0 = n0; s->n_initial = n0;
  s->open = 1;
}

static void join_curve(Stroker* s, OPt n1) {   /* :619-636 */
  if (peq(s->n0, n1)) return;
  int side = side_from_normals(s->n0, n1);
  OPt m = padd(s->n0, n1);
  OPt k = pdiv(pmul(m, s->d2[side]), mag_sq(m));
  OPt w1 = pmul(n1, s->d[side]);
  int dummy = 0;
  outer_join(s, s->side[side], n1, w1, k, s->d[side], s->d2[side], &dummy);
  OPath* inner = s->side[1 - side];
  line_to(inner, s->p0);                /* inner_join_curve_to (:736-739) */
  line_to(inner, psub(s->p0, w1));
  s->n0 = n1;
}

static void join_cusp(Stroker* s, OPt n1) {   /* :638-647 */
  int side = side_from_normals(s->n0, n1);
  OPt w1 = pmul(n1, s->d[side]);
  dull_round_join(s, s->side[side], s->d[side], s->d2[side], w1);
  line_to(s->side[1 - side], psub(s->p0, w1));
  s->n0 = n1;
}

static void join_cusp_and_line_to(Stroker* s, OPt n1, OPt p1) {   /* :649-665 */
  int side = side_from_normals(s->n0, n1);
  OPt w1 = pmul(n1, s->d[side]);
  OPath* outer = s->side[side];
  dull_round_join(s, outer, s->d[side], s->d2[side], w1);
  line_to(outer, padd(p1, w1));
  OPath* inner = s->side[1 - side];
  line_to(inner, psub(s->p0, w1));
  line_to(inner, psub(p1, w1));
  s->n0 = n1; s->p0 = p1;
}

static void smooth_poly_to(Stroker* s, const OPt* poly, size_t count) {   /* :667-694 */
  OPt p1 = poly[0];
  OPt v1 = psub(p1, s->p0);
  if (mag_sq(v1) < kLengthEpsilonSq) return;
  OPt n1 = normal(unit_vector(v1));
  if (!s->open) open_line_to(s, p1, n1);
  else join_line_to(s, p1, n1);
  for (size_t i = 1; i < count; i++) {
    p1 = poly[i];
    v1 = psub(p1, s->p0);
    if (mag_sq(v1) < kLengthEpsilonSq) continue;
    n1 = normal(unit_vector(v1));
    join_cusp_and_line_to(s, n1, p1);
  }
}

static void join_end_point(Stroker* s, OPt n1) {   /* :697-734 */
  if (peq(s->n0, n1)) {
    OPath* a = s->side[SIDE_A];
    OPath* b = s->side[SIDE_B];
    back(a, (size_t)prev_is_on(a));
    back(b, (size_t)prev_is_on(b));
    return;
  }
  int side = side_from_normals(s->n0, n1);
  OPt m = padd(s->n0, n1);
  OPt w1 = pmul(n1, s->d[side]);
  OPt k = pdiv(pmul(m, s->d2[side]), mag_sq(m));
  int miter_flag = 0;
  OPath* outer = s->side[side];
  outer_join(s, outer, n1, w1, k, s->d[side], s->d2[side], &miter_flag);
  /* the figure starts at index 0 of both side paths */
  if (miter_flag && outer->cmd[1] == P_ON) {
    back(outer, 1);
    outer->vtx[0] = vtx_back(outer, 1);
    back(outer, (size_t)prev_is_on(outer));
  }
  OPath* inner = s->side[1 - side];
  if (inner->cmd[1] <= P_ON) {
    OPt inner_pt = psub(s->p0, k);   /* inner_join_end_point (:752-761) */
    if (prev_is_on(inner) && inner_join_test(vtx_back(inner, 2), vtx_back(inner, 1), inner->vtx[0], inner->vtx[1], inner_pt)) {
      inner->vtx[0] = inner_pt;
      back(inner, 1);
    }
    else {
      line_to(inner, s->p0);
      line_to(inner, inner->vtx[0]);
    }
  }
}

static void offset_quad_simple(Stroker* s, OPt p0, OPt p1, OPt p2) {   /* :885-905 */
  if (peq(p0, p2)) return;
  OPt v0 = psub(p1, p0), v1 = psub(p2, p1);
  OPt m0 = normal(unit_vector(!peq(p0, p1) ? v0 : v1));
  OPt m2 = normal(unit_vector(!peq(p1, p2) ? v1 : v0));
  s->p0 = p2; s->n0 = m2;
  OPt m = padd(m0, m2);
  OPt k1 = pdiv(pmul(m, s->d2[SIDE_A]), mag_sq(m));
  OPt k2 = pmul(m2, s->d[SIDE_A]);
  quad_to(s->side[SIDE_A], padd(p1, k1), padd(p2, k2));
  quad_to(s->side[SIDE_B], psub(p1, k1), psub(p2, k2));
}

static void offset_quad(Stroker* s, const OPt* bez) {   /* :860-883 */
  double ts[3];
  size_t tn = quad_offset_cusp_ts(bez, s->d[SIDE_A], ts);
  ts[tn++] = 1.0;
  QuadTsIter it;
  qti_reset(&it, bez, ts, tn);
  double m = s->offset_parameter;
  do {
    for (;;) {
      double t = quad_parameter_at_angle(it.part, m);
      if (!(t > kOffsetQuadEpsilonT && t < 1.0 - kOffsetQuadEpsilonT)) t = 1.0;
      OPt part[3];
      quad_split_t(it.part, part, it.part, t);
      offset_quad_simple(s, part[0], part[1], part[2]);
      if (t == 1.0) break;
    }
  } while (qti_next(&it));
}

static void offset_cubic(Stroker* s, const OPt* curve) {   /* approximate_cubic_with_quads (bezier_p.h:943-982) */
  double tol = 54.0 * s->simplify_tolerance;
  double tolerance_sq = tol * tol;
  double t = pow(tolerance_sq / mag_sq(cubic_identity(curve)), 1.0 / 6.0);
  OPt cubic[7];
  cubic[3] = curve[0]; cubic[4] = curve[1]; cubic[5] = curve[2]; cubic[6] = curve[3];
  for (;;) {
    OPt quads[5];
    t = t < 1.0 ? t : 1.0;                                 /* bl_min(1.0, t) */
    if (t >= 0.999) t = 1.0;
    cubic_split_t(cubic + 3, cubic, cubic + 3, t);
    cubic_to_two_quads(cubic, quads);
    offset_quad(s, quads + 0);
    offset_quad(s, quads + 2);
    if (t >= 1.0) return;
    double old_t = t;
    t = t / (1.0 - t);
    if (old_t - t < 1e-3) t += 0.01;
  }
}

static void add_cap(OPath* out, OPt pivot, OPt p1, uint32_t cap) {   /* :921-969 */
  OPt p0 = vtx_back(out, 1);
  OPt q = pmul(normal(psub(p1, p0)), 0.5);
  switch (cap) {
    case CAP_SQUARE: line_to(out, padd(p0, q)); line_to(out, padd(p1, q)); line_to(out, p1); break;
    case CAP_ROUND: arc_quadrant_to(out, padd(p0, q), padd(pivot, q)); arc_quadrant_to(out, padd(p1, q), p1); break;
    case CAP_ROUND_REV:
      line_to(out, padd(p0, q)); arc_quadrant_to(out, p0, pivot); arc_quadrant_to(out, p1, padd(p1, q)); line_to(out, p1);
      break;
    case CAP_TRIANGLE: line_to(out, padd(pivot, q)); line_to(out, p1); break;
    case CAP_TRIANGLE_REV:
      line_to(out, padd(p0, q)); line_to(out, pivot); line_to(out, padd(p1, q)); line_to(out, p1);
      break;
    default: line_to(out, p1); break;   /* butt */
  }
}

/* PathStroker::stroke (:224-487). */
int o_stroke_path(const uint8_t* cmd, const double* xy, size_t n, const OStrokeOpts* opt,
                  double simplify_tolerance, double offset_parameter, OPath* a, OPath* b, OPath* c,
                  OStrokeSink sink, void* user) {
  Stroker s;
  memset(&s, 0, sizeof(s));
  s.opt = opt;
  s.simplify_tolerance = simplify_tolerance;
  s.offset_parameter = offset_parameter;
  s.side[SIDE_A] = a; s.side[SIDE_B] = b;
  s.d[SIDE_A] = opt->width * 0.5; s.d2[SIDE_A] = opt->width;
  s.d[SIDE_B] = -s.d[SIDE_A]; s.d2[SIDE_B] = -s.d2[SIDE_A];
  s.join = opt->join;
  if (s.join == JOIN_MITER_CLIP || s.join == JOIN_MITER_BEVEL || s.join == JOIN_MITER_ROUND) {
    if (s.join == JOIN_MITER_BEVEL) s.join = JOIN_BEVEL;
    else if (s.join == JOIN_MITER_ROUND) s.join = JOIN_ROUND;
    s.miter_limit = s.d[SIDE_A] * opt->miter_limit;
    s.miter_limit_sq = s.miter_limit * s.miter_limit;
  }
  else {
    s.miter_limit = kMiterMinimum;
    s.miter_limit_sq = kMiterMinimum * kMiterMinimum;
  }
  const OPt* vtx = (const OPt*)xy;
  size_t i = 0;
  while (i < n) {
    if (cmd[i] != P_MOVE) {
      if (cmd[i] != P_CLOSE) return 1;                 /* BL_ERROR_INVALID_GEOMETRY */
      i++;
      continue;
    }
    a->n = 0; b->n = 0;
    OPt poly[4];
    size_t poly_size = 0;
    s.p0 = vtx[i]; s.p_initial = s.p0;
    s.open = 0; s.closed = 0;
    i++;
    while (i < n) {
      uint8_t k = cmd[i];
      OPt p1 = vtx[i], v1, n1;
      if (k == P_ON) {
        i++;
LineTo:
        v1 = psub(p1, s.p0);
        if (mag_sq(v1) < kLengthEpsilonSq) continue;
        n1 = normal(unit_vector(v1));
        if (!s.open) { open_line_to(&s, p1, n1); continue; }
        for (;;) {
          join_line_to(&s, p1, n1);
          if (i >= n) break;
          k = cmd[i]; p1 = vtx[i];
          if (k != P_ON) break;
          i++;
          v1 = psub(p1, s.p0);
          if (mag_sq(v1) < kLengthEpsilonSq) break;
          n1 = normal(unit_vector(v1));
        }
        continue;
SmoothPolyTo:
        smooth_poly_to(&s, poly, poly_size);
        continue;
      }
      else if (k == P_QUAD) {
        i += 2;
        if (i > n) return 1;
        const OPt* quad = vtx + i - 3;
        OPt p2 = quad[2];
        OPt v2 = psub(p2, p1);
        v1 = psub(p1, s.p0);
        n1 = normal(unit_vector(v1));
        double cm = cross(v2, v1);
        if (fabs(cm) <= kCollinearityEpsilon) {
          double dd = dot(pneg(v1), v2);
          if (dd > 0.0) {
            double r1 = dot(psub(p1, s.p0), v1);
            double r2 = dot(psub(p2, s.p0), v1);
            double t = r1 / (2.0 * r1 - r2);
            if (t > 0.0 && t < 1.0) {
              poly[0] = quad_eval(quad, t);
              poly[1] = p2;
              poly_size = 2;
              goto SmoothPolyTo;
            }
          }
          p1 = p2;
          goto LineTo;
        }
        if (mag_sq(v1) < kLengthEpsilonSq || mag_sq(v2) < kLengthEpsilonSq) { p1 = p2; goto LineTo; }
        if (!s.open) open_curve(&s, n1);
        else join_curve(&s, n1);
        offset_quad(&s, vtx + i - 3);
      }
      else if (k == P_CUBIC) {
        i += 3;
        if (i > n) return 1;
        OPt p[7];
        int cusp = 0;
        double t_cusp = 0;
        p[0] = s.p0; p[1] = vtx[i - 3]; p[2] = vtx[i - 2]; p[3] = vtx[i - 1];
        if (is_cubic_flat(p, kDegenerateFlatness)) {
          double dot1 = dot(psub(p[0], p[1]), psub(p[3], p[1]));
          double dot2 = dot(psub(p[0], p[2]), psub(p[3], p[2]));
          if (!(dot1 < 0.0) || !(dot2 < 0.0)) {
            OPt r = cubic_start_tangent(p);
            double r1 = dot(psub(p[1], p[0]), r);
            double r2 = dot(psub(p[2], p[0]), r);
            double r3 = dot(psub(p[3], p[0]), r);
            double aa = 1.0 / (3.0 * r1 - 3.0 * r2 + r3);
            double bb = 2.0 * r1 - r2;
            double ss = sqrt(r2 * (r2 - r1) - r1 * (r3 - r1));
            double t1 = aa * (bb - ss);
            double t2 = aa * (bb + ss);
            poly_size = 0;
            if (t1 > kCuspTThreshold && t1 < 1.0 - kCuspTThreshold) poly[poly_size++] = cubic_eval(p, t1);
            if (t2 > kCuspTThreshold && t2 < 1.0 - kCuspTThreshold) poly[poly_size++] = cubic_eval(p, t2);
            if (poly_size == 0) { p1 = p[3]; goto LineTo; }
            poly[poly_size++] = p[3];
            goto SmoothPolyTo;
          }
          p1 = p[3];
          goto LineTo;
        }
        else {
          double tl;
          cubic_inflection_parameter(p, &t_cusp, &tl);
          if (tl == 0.0 && t_cusp > 0.0 && t_cusp < 1.0) {
            cubic_split_half(p, p, p + 3);
            cusp = 1;
          }
        }
        for (;;) {
          v1 = psub(p[1], s.p0);
          if (is_zero(v1)) v1 = psub(p[2], s.p0);
          n1 = normal(unit_vector(v1));
          if (!s.open) open_curve(&s, n1);
          else if (cusp >= 0) join_curve(&s, n1);
          else join_cusp(&s, n1);
          offset_cubic(&s, p);
          if (cusp <= 0) break;
          cusp = -1;
          p[0] = p[3]; p[1] = p[4]; p[2] = p[5]; p[3] = p[6];
        }
      }
      else {
        if (s.closed) break;
        if (k != P_CLOSE) break;
        s.closed = 1;
        p1 = s.p_initial;
        goto LineTo;
      }
    }
    i += (size_t)s.closed;
    if (!s.open) continue;
    if (s.closed) {
      join_end_point(&s, s.n_initial);
      close_path(a);
      close_path(b);
      c->n = 0;
    }
    else {
      uint32_t start_cap = opt->start_cap <= CAP_TRIANGLE_REV ? opt->start_cap : CAP_BUTT;
      uint32_t end_cap = opt->end_cap <= CAP_TRIANGLE_REV ? opt->end_cap : CAP_BUTT;
      add_cap(a, s.p0, vtx_back(b, 1), end_cap);
      c->n = 0;
      move_to(c, b->vtx[0]);
      add_cap(c, s.p_initial, a->vtx[0], start_cap);
    }
    int rc = sink(a, b, c, user);
    if (rc) return rc;
  }
  return 0;
}
