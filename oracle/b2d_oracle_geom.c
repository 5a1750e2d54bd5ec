/*
 * b2d_oracle_geom.c - oracle (test infrastructure): matrices, edge building and the analytic
 * rasterizer band loop, restated from the reference:
 *   matrices        blend2d/core/matrix.cpp:133-211, :442-463, blend2d/core/matrix_p.h:48-64
 *   bezier splits   blend2d/geometry/bezier_p.h:366-395 (quad), :834-920 (cubic)
 *   quad_roots      blend2d/support/math_p.h:574-592
 *   edge builder    blend2d/raster/edgebuilder_p.h:1032-2629
 *   rasterizer      blend2d/raster/analyticrasterizer_p.h:289-1262
 *   band loop       blend2d/raster/rendercommandprocsync_p.h:87-254
 * Compiled with -ffp-contract=off so every a*b+c stays unfused as in the x86-64 reference build.
 */
#include "b2d_oracle_p.h"

/* ============================================================================================
 * Matrices
 * ============================================================================================ */

void o_mat_multiply(OMat* dst, const OMat* a, const OMat* b) {
  OMat r;
  r.m00 = a->m00 * b->m00 + a->m01 * b->m10;
  r.m01 = a->m00 * b->m01 + a->m01 * b->m11;
  r.m10 = a->m10 * b->m00 + a->m11 * b->m10;
  r.m11 = a->m10 * b->m01 + a->m11 * b->m11;
  r.m20 = a->m20 * b->m00 + a->m21 * b->m10 + b->m20;
  r.m21 = a->m20 * b->m01 + a->m21 * b->m11 + b->m21;
  *dst = r;
}

int o_mat_invert(OMat* dst, const OMat* src) {
  double d = src->m00 * src->m11 - src->m01 * src->m10;
  if (d == 0.0 || !isfinite(d))
    return 0;
  double t00 = src->m11, t01 = -src->m01, t10 = -src->m10, t11 = src->m00;
  t00 /= d; t01 /= d; t10 /= d; t11 /= d;
  double t20 = -(src->m20 * t00 + src->m21 * t10);
  double t21 = -(src->m20 * t01 + src->m21 * t11);
  dst->m00 = t00; dst->m01 = t01; dst->m10 = t10; dst->m11 = t11; dst->m20 = t20; dst->m21 = t21;
  return 1;
}

int o_mat_type(const OMat* m) {
  unsigned msk = ((unsigned)(m->m00 != 0.0) << 3) | ((unsigned)(m->m01 != 0.0) << 2) |
                 ((unsigned)(m->m10 != 0.0) << 1) | ((unsigned)(m->m11 != 0.0) << 0);
  /* valid combinations (matrix.cpp:159-174) */
  const unsigned valid = (1u << 3) | (1u << 6) | (1u << 7) | (1u << 9) | (1u << 11) | (1u << 12) |
                         (1u << 13) | (1u << 14) | (1u << 15);
  double d = m->m00 * m->m11 - m->m01 * m->m10;
  if (!((1u << msk) & valid) || !isfinite(d) || !isfinite(m->m20) || !isfinite(m->m21))
    return O_TT_INVALID;
  if (msk != 9u)
    return msk == 6u ? O_TT_SWAP : O_TT_AFFINE;
  if (!((m->m00 == 1.0) & (m->m11 == 1.0)))
    return O_TT_SCALE;
  if (!((m->m20 == 0.0) & (m->m21 == 0.0)))
    return O_TT_TRANSLATE;
  return O_TT_IDENTITY;
}

/* ============================================================================================
 * Edge storage
 * ============================================================================================ */

static int o_ctz(unsigned v) { int n = 0; while (!(v & 1u)) { v >>= 1; n++; } return n; }

void o_storage_init(OEdgeStorage* st, int width, int height, int band_height) {
  (void)width;
  memset(st, 0, sizeof(*st));
  st->band_height = band_height;
  st->shift = o_ctz((unsigned)band_height) + 8;
  st->band_count = (height + band_height - 1) / band_height;
  st->band_first = (int*)malloc(sizeof(int) * (size_t)(st->band_count + 1));
  st->band_last = (int*)malloc(sizeof(int) * (size_t)(st->band_count + 1));
  o_storage_clear(st);
}

void o_storage_free(OEdgeStorage* st) {
  free(st->pts); free(st->edges); free(st->band_first); free(st->band_last);
  memset(st, 0, sizeof(*st));
}

void o_storage_clear(OEdgeStorage* st) {
  st->npts = 0;
  st->nedges = 0;
  for (int i = 0; i <= st->band_count; i++) { st->band_first[i] = -1; st->band_last[i] = -1; }
  st->bbox_y0 = INT_MAX;
  st->bbox_y1 = INT_MIN;
}

static void st_push_pt(OEdgeStorage* st, int x, int y) {
  if (st->npts == st->cap_pts) {
    st->cap_pts = st->cap_pts ? st->cap_pts * 2 : 1024;
    st->pts = (OEdgePt*)realloc(st->pts, st->cap_pts * sizeof(OEdgePt));
  }
  st->pts[st->npts].x = x;
  st->pts[st->npts].y = y;
  st->npts++;
}

/* Links a finished polyline (points top-down) into the band of its first point
 * (EdgeBuilder::_link_edge, edgebuilder_p.h:2535-2539). */
static void st_add_edge(OEdgeStorage* st, const OEdgePt* pts, int count, uint32_t sign) {
  if (st->nedges == st->cap_edges) {
    st->cap_edges = st->cap_edges ? st->cap_edges * 2 : 256;
    st->edges = (OEdge*)realloc(st->edges, st->cap_edges * sizeof(OEdge));
  }
  OEdge* e = &st->edges[st->nedges];
  e->first = (int)st->npts;
  e->count = count;
  e->sign = sign;
  e->next = -1;
  for (int i = 0; i < count; i++)
    st_push_pt(st, pts[i].x, pts[i].y);
  int band = (int)((unsigned)pts[0].y >> st->shift);
  int idx = (int)st->nedges++;
  if (st->band_last[band] < 0) st->band_first[band] = idx;
  else st->edges[st->band_last[band]].next = idx;
  st->band_last[band] = idx;
  st->bbox_y0 = o_imin(st->bbox_y0, pts[0].y);
  st->bbox_y1 = o_imax(st->bbox_y1, pts[count - 1].y);
}

/* ============================================================================================
 * Edge builder
 * ============================================================================================ */

enum { CF_X0 = 1, CF_Y0 = 2, CF_X1 = 4, CF_Y1 = 8 };

static inline uint32_t cf_x0(const OEdgeBuilder* eb, OPt p) { return (uint32_t)(!(p.x >= eb->cx0)) << 0; }
static inline uint32_t cf_x1(const OEdgeBuilder* eb, OPt p) { return (uint32_t)(!(p.x <= eb->cx1)) << 2; }
static inline uint32_t cf_y0(const OEdgeBuilder* eb, OPt p) { return (uint32_t)(!(p.y >= eb->cy0)) << 1; }
static inline uint32_t cf_y1(const OEdgeBuilder* eb, OPt p) { return (uint32_t)(!(p.y <= eb->cy1)) << 3; }
static inline uint32_t cf_x(const OEdgeBuilder* eb, OPt p) { return cf_x0(eb, p) | cf_x1(eb, p); }
static inline uint32_t cf_y(const OEdgeBuilder* eb, OPt p) { return cf_y0(eb, p) | cf_y1(eb, p); }
static inline uint32_t cf_xy(const OEdgeBuilder* eb, OPt p) { return cf_x(eb, p) | cf_y(eb, p); }

void o_eb_init(OEdgeBuilder* eb, OEdgeStorage* st, int width, int height, double tol_sq) {
  memset(eb, 0, sizeof(*eb));
  eb->st = st;
  eb->cx0 = 0.0; eb->cy0 = 0.0; eb->cx1 = (double)width * 256.0; eb->cy1 = (double)height * 256.0;
  eb->icx0 = o_trunc_to_int(eb->cx0); eb->icy0 = o_trunc_to_int(eb->cy0);
  eb->icx1 = o_trunc_to_int(eb->cx1); eb->icy1 = o_trunc_to_int(eb->cy1);
  eb->tol_sq = tol_sq;
  eb->acc_x0_y0 = eb->acc_x0_y1 = eb->acc_x1_y0 = eb->acc_x1_y1 = eb->cy0;
}

void o_eb_free(OEdgeBuilder* eb) { free(eb->tmp); eb->tmp = NULL; }

void o_eb_begin(OEdgeBuilder* eb) {   /* EdgeBuilder::begin (edgebuilder_p.h:934-944) */
  eb->ntmp = 0;
  eb->acc_x0_y0 = eb->acc_x0_y1 = eb->acc_x1_y0 = eb->acc_x1_y1 = eb->cy0;
}

static void tmp_push(OEdgeBuilder* eb, int x, int y) {
  if (eb->ntmp == eb->cap_tmp) {
    eb->cap_tmp = eb->cap_tmp ? eb->cap_tmp * 2 : 256;
    eb->tmp = (OEdgePt*)realloc(eb->tmp, eb->cap_tmp * sizeof(OEdgePt));
  }
  eb->tmp[eb->ntmp].x = x;
  eb->tmp[eb->ntmp].y = y;
  eb->ntmp++;
}

/* Raw polyline building (edgebuilder_p.h:2452-2533). Ascending polylines are collected
 * bottom-up and stored reversed so every stored polyline runs top-down. */
static void desc_open(OEdgeBuilder* eb) { eb->ntmp = 0; eb->ascending = 0; }
static void desc_add(OEdgeBuilder* eb, int x, int y) { tmp_push(eb, x, y); }
static void desc_close(OEdgeBuilder* eb, uint32_t sign) { st_add_edge(eb->st, eb->tmp, (int)eb->ntmp, sign); }
static void asc_open(OEdgeBuilder* eb) { eb->ntmp = 0; eb->ascending = 1; }
static void asc_add(OEdgeBuilder* eb, int x, int y) { tmp_push(eb, x, y); }
static void asc_close(OEdgeBuilder* eb) {
  for (size_t i = 0, j = eb->ntmp - 1; i < j; i++, j--) { OEdgePt t = eb->tmp[i]; eb->tmp[i] = eb->tmp[j]; eb->tmp[j] = t; }
  st_add_edge(eb->st, eb->tmp, (int)eb->ntmp, 1);
}

static void add_closed_line(OEdgeBuilder* eb, int x0, int y0, int x1, int y1, uint32_t sign) {
  OEdgePt p[2] = { { x0, y0 }, { x1, y1 } };
  st_add_edge(eb->st, p, 2, sign);
}

static void add_line_segment(OEdgeBuilder* eb, double x0, double y0, double x1, double y1) {
  int fx0 = o_trunc_to_int(x0), fy0 = o_trunc_to_int(y0), fx1 = o_trunc_to_int(x1), fy1 = o_trunc_to_int(y1);
  if (fy0 == fy1) return;
  if (fy0 < fy1) add_closed_line(eb, fx0, fy0, fx1, fy1, 0);
  else add_closed_line(eb, fx1, fy1, fx0, fy0, 1);
}

/* Border accumulation (edgebuilder_p.h:2546-2622). */
static void emit_left_border(OEdgeBuilder* eb) {
  int a = o_trunc_to_int(eb->acc_x0_y0), b = o_trunc_to_int(eb->acc_x0_y1);
  if (a == b) return;
  add_closed_line(eb, eb->icx0, o_imin(a, b), eb->icx0, o_imax(a, b), (uint32_t)(a > b));
}
static void emit_right_border(OEdgeBuilder* eb) {
  int a = o_trunc_to_int(eb->acc_x1_y0), b = o_trunc_to_int(eb->acc_x1_y1);
  if (a == b) return;
  add_closed_line(eb, eb->icx1, o_imin(a, b), eb->icx1, o_imax(a, b), (uint32_t)(a > b));
}
static void acc_left(OEdgeBuilder* eb, double y0, double y1) {
  if (eb->acc_x0_y1 == y0) { eb->acc_x0_y1 = y1; return; }
  emit_left_border(eb);
  eb->acc_x0_y0 = y0; eb->acc_x0_y1 = y1;
}
static void acc_right(OEdgeBuilder* eb, double y0, double y1) {
  if (eb->acc_x1_y1 == y0) { eb->acc_x1_y1 = y1; return; }
  emit_right_border(eb);
  eb->acc_x1_y0 = y0; eb->acc_x1_y1 = y1;
}
static void acc_left_s(OEdgeBuilder* eb, double y0, double y1, uint32_t sign) {
  if (sign) { double t = y0; y0 = y1; y1 = t; }
  acc_left(eb, y0, y1);
}
static void acc_right_s(OEdgeBuilder* eb, double y0, double y1, uint32_t sign) {
  if (sign) { double t = y0; y0 = y1; y1 = t; }
  acc_right(eb, y0, y1);
}

int o_eb_done(OEdgeBuilder* eb) {
  emit_left_border(eb);
  emit_right_border(eb);
  eb->acc_x0_y0 = eb->acc_x0_y1;
  eb->acc_x1_y0 = eb->acc_x1_y1;
  return 0;
}

/* --- sources (EdgeSourcePoly / EdgeSourcePath, edgebuilder_p.h:102-270) ------------------- */

typedef struct {
  int is_path;
  const double* xy;
  const uint8_t* cmd;
  long i, n;
  int affine;
  OMat m;
} OSrc;

static inline OPt src_tf(const OSrc* s, long k) {
  double x = s->xy[2 * k], y = s->xy[2 * k + 1];
  OPt r;
  if (s->affine) r = o_mat_map(&s->m, x, y);
  else { r.x = x * s->m.m00 + s->m.m20; r.y = y * s->m.m11 + s->m.m21; }
  return r;
}

static int src_begin(OSrc* s, OPt* initial) {
  if (!s->is_path) {
    if (s->i == s->n) return 0;
    *initial = src_tf(s, s->i);
    s->i++;
    return 1;
  }
  for (;;) {
    if (s->i == s->n) return 0;
    uint8_t c = s->cmd[s->i];
    s->i++;
    if (c != 0 /* MOVE */) continue;
    *initial = src_tf(s, s->i - 1);
    return 1;
  }
}
static inline int src_is_close(const OSrc* s) { return s->is_path && s->i != s->n && s->cmd[s->i] == 5; }
static inline int src_is_line_to(const OSrc* s) { return s->is_path ? (s->i != s->n && s->cmd[s->i] == 1) : (s->i != s->n); }
static inline int src_is_quad_to(const OSrc* s) { return s->is_path && s->i <= s->n - 2 && s->cmd[s->i] == 2; }
static inline int src_is_conic_to(const OSrc* s) { return s->is_path && s->i < s->n - 2 && s->cmd[s->i] == 3; }
static inline int src_is_cubic_to(const OSrc* s) { return s->is_path && s->i < s->n - 2 && s->cmd[s->i] == 4; }
static inline void src_next_line_to(OSrc* s, OPt* p) { *p = src_tf(s, s->i); s->i++; }
static inline int src_maybe_next_line_to(OSrc* s, OPt* p) { if (!src_is_line_to(s)) return 0; src_next_line_to(s, p); return 1; }
static inline void src_next_quad_to(OSrc* s, OPt* p1, OPt* p2) { *p1 = src_tf(s, s->i); *p2 = src_tf(s, s->i + 1); s->i += 2; }
static inline void src_next_cubic_to(OSrc* s, OPt* p1, OPt* p2, OPt* p3) {
  *p1 = src_tf(s, s->i); *p2 = src_tf(s, s->i + 1); *p3 = src_tf(s, s->i + 2); s->i += 3;
}
static inline void src_next_conic_to(OSrc* s, OPt* p1, OPt* p2) { *p1 = src_tf(s, s->i); *p2 = src_tf(s, s->i + 2); s->i += 2; }

/* --- line_to (edgebuilder_p.h:1123-1607) ------------------------------------------------ */

#define TR(v) o_trunc_to_int(v)

static int eb_line_to(OEdgeBuilder* eb, OSrc* src, OPt* pa, uint32_t* pa_flags, OPt b) {
#define A (*pa)
#define AF (*pa_flags)
  OPt p, d;
  uint32_t b_flags = 0;
  int fx0, fy0, fx1, fy1;
  double borY0 = 0.0, borY1;

  do {
    if (!AF) {
      b_flags = cf_xy(eb, b);
      if (!b_flags) {
        fx0 = TR(A.x); fy0 = TR(A.y); fx1 = TR(b.x); fy1 = TR(b.y);
        for (;;) {
          if (fy0 < fy1) {
DescendingLineBegin:
            desc_open(eb);
            desc_add(eb, fx0, fy0);
            desc_add(eb, fx1, fy1);
            for (;;) {
DescendingLineLoopA:
              if (!src_maybe_next_line_to(src, &A)) { desc_close(eb, 0); A = b; return 0; }
              b_flags = cf_xy(eb, A);
              if (b_flags) { desc_close(eb, 0); OPt t = A; A = b; b = t; goto BeforeClipEndPoint; }
              fx0 = TR(A.x); fy0 = TR(A.y);
              if (fy0 < fy1) {
                desc_close(eb, 0);
                asc_open(eb); asc_add(eb, fx1, fy1); asc_add(eb, fx0, fy0);
                goto AscendingLineLoopB;
              }
              desc_add(eb, fx0, fy0);
DescendingLineLoopB:
              if (!src_maybe_next_line_to(src, &b)) { desc_close(eb, 0); return 0; }
              b_flags = cf_xy(eb, b);
              if (b_flags) { desc_close(eb, 0); goto BeforeClipEndPoint; }
              fx1 = TR(b.x); fy1 = TR(b.y);
              if (fy1 < fy0) {
                desc_close(eb, 0);
                asc_open(eb); asc_add(eb, fx0, fy0); asc_add(eb, fx1, fy1);
                goto AscendingLineLoopA;
              }
              desc_add(eb, fx1, fy1);
            }
          }
          else if (fy0 > fy1) {
AscendingLineBegin:
            asc_open(eb);
            asc_add(eb, fx0, fy0);
            asc_add(eb, fx1, fy1);
            for (;;) {
AscendingLineLoopA:
              if (!src_maybe_next_line_to(src, &A)) { asc_close(eb); A = b; return 0; }
              b_flags = cf_xy(eb, A);
              if (b_flags) { asc_close(eb); OPt t = A; A = b; b = t; goto BeforeClipEndPoint; }
              fx0 = TR(A.x); fy0 = TR(A.y);
              if (fy0 > fy1) {
                asc_close(eb);
                desc_open(eb); desc_add(eb, fx1, fy1); desc_add(eb, fx0, fy0);
                goto DescendingLineLoopB;
              }
              asc_add(eb, fx0, fy0);
AscendingLineLoopB:
              if (!src_maybe_next_line_to(src, &b)) { asc_close(eb); return 0; }
              b_flags = cf_xy(eb, b);
              if (b_flags) { asc_close(eb); goto BeforeClipEndPoint; }
              fx1 = TR(b.x); fy1 = TR(b.y);
              if (fy1 > fy0) {
                asc_close(eb);
                desc_open(eb); desc_add(eb, fx0, fy0); desc_add(eb, fx1, fy1);
                goto DescendingLineLoopA;
              }
              asc_add(eb, fx1, fy1);
            }
          }
          else {
            A = b;
            if (!src_maybe_next_line_to(src, &b)) return 0;
            b_flags = cf_xy(eb, b);
            if (b_flags) break;
            fx0 = fx1; fy0 = fy1;
            fx1 = TR(b.x); fy1 = TR(b.y);
          }
        }
      }
BeforeClipEndPoint:
      p = A;
      d.x = b.x - A.x; d.y = b.y - A.y;
    }
    else {
RestartClipLoop:
      if (AF & CF_Y0) {
        for (;;) {
          if (eb->cy0 < b.y) break;
          A = b;
          if (!src_maybe_next_line_to(src, &b)) { AF = cf_x(eb, A) | cf_y0(eb, A); return 0; }
        }
        AF = cf_x(eb, A) | cf_y0(eb, A);
        b_flags = cf_x(eb, b) | cf_y1(eb, b);
        borY0 = eb->cy0;
        uint32_t common = AF & b_flags;
        if (common) {
          borY1 = o_min(eb->cy1, b.y);
          if (common & CF_X0) acc_left(eb, borY0, borY1); else acc_right(eb, borY0, borY1);
          A = b; AF = b_flags;
          continue;
        }
      }
      else if (AF & CF_Y1) {
        for (;;) {
          if (eb->cy1 > b.y) break;
          A = b;
          if (!src_maybe_next_line_to(src, &b)) { AF = cf_x(eb, A) | cf_y1(eb, A); return 0; }
        }
        AF = cf_x(eb, A) | cf_y1(eb, A);
        b_flags = cf_x(eb, b) | cf_y0(eb, b);
        borY0 = eb->cy1;
        uint32_t common = AF & b_flags;
        if (common) {
          borY1 = o_max(eb->cy0, b.y);
          if (common & CF_X0) acc_left(eb, borY0, borY1); else acc_right(eb, borY0, borY1);
          A = b; AF = b_flags;
          continue;
        }
      }
      else if (AF & CF_X0) {
        borY0 = o_clamp(A.y, eb->cy0, eb->cy1);
        for (;;) {
          if (eb->cx0 < b.x) break;
          A = b;
          if (!src_maybe_next_line_to(src, &b)) {
            AF = cf_y(eb, A) | cf_x0(eb, A);
            borY1 = o_clamp(A.y, eb->cy0, eb->cy1);
            if (borY0 != borY1) acc_left(eb, borY0, borY1);
            return 0;
          }
        }
        borY1 = o_clamp(A.y, eb->cy0, eb->cy1);
        if (borY0 != borY1) acc_left(eb, borY0, borY1);
        AF = cf_x0(eb, A) | cf_y(eb, A);
        b_flags = cf_x1(eb, b) | cf_y(eb, b);
        if (AF & b_flags) goto RestartClipLoop;
        borY0 = borY1;
      }
      else {
        borY0 = o_clamp(A.y, eb->cy0, eb->cy1);
        for (;;) {
          if (eb->cx1 > b.x) break;
          A = b;
          if (!src_maybe_next_line_to(src, &b)) {
            AF = cf_y(eb, A) | cf_x1(eb, A);
            borY1 = o_clamp(A.y, eb->cy0, eb->cy1);
            if (borY0 != borY1) acc_right(eb, borY0, borY1);
            return 0;
          }
        }
        borY1 = o_clamp(A.y, eb->cy0, eb->cy1);
        if (borY0 != borY1) acc_right(eb, borY0, borY1);
        AF = cf_x1(eb, A) | cf_y(eb, A);
        b_flags = cf_x0(eb, b) | cf_y(eb, b);
        if (AF & b_flags) goto RestartClipLoop;
        borY0 = borY1;
      }

      /* Clip start point. */
      d.x = b.x - A.x; d.y = b.y - A.y;
      p.x = eb->cx1; p.y = eb->cy1;
      switch (AF) {
        case 0: p = A; break;
        case CF_X0 | CF_Y0: p.x = eb->cx0; /* fallthrough */
        case CF_X1 | CF_Y0:
          p.y = A.y + (p.x - A.x) * d.y / d.x;
          AF = cf_y(eb, p);
          if (p.y >= eb->cy0) break;
          /* fallthrough */
        case CF_Y0:
          p.y = eb->cy0;
          p.x = A.x + (p.y - A.y) * d.x / d.y;
          AF = cf_x(eb, p);
          break;
        case CF_X0 | CF_Y1: p.x = eb->cx0; /* fallthrough */
        case CF_X1 | CF_Y1:
          p.y = A.y + (p.x - A.x) * d.y / d.x;
          AF = cf_y(eb, p);
          if (p.y <= eb->cy1) break;
          /* fallthrough */
        case CF_Y1:
          p.y = eb->cy1;
          p.x = A.x + (p.y - A.y) * d.x / d.y;
          AF = cf_x(eb, p);
          break;
        case CF_X0: p.x = eb->cx0; /* fallthrough */
        case CF_X1:
          p.y = A.y + (p.x - A.x) * d.y / d.x;
          AF = cf_y(eb, p);
          break;
        default:
          return -3; /* BL_ERROR_INVALID_GEOMETRY (NaNs) */
      }

      if (AF) {
        borY1 = o_clamp(b.y, eb->cy0, eb->cy1);
        if (p.x <= eb->cx0) acc_left(eb, borY0, borY1);
        else if (p.x >= eb->cx1) acc_right(eb, borY0, borY1);
        A = b; AF = b_flags;
        continue;
      }

      borY1 = o_clamp(p.y, eb->cy0, eb->cy1);
      if (borY0 != borY1) {
        if (p.x <= eb->cx0) acc_left(eb, borY0, borY1);
        else acc_right(eb, borY0, borY1);
      }

      if (!b_flags) {
        A = b;
        AF = 0;
        fx0 = TR(p.x); fy0 = TR(p.y); fx1 = TR(b.x); fy1 = TR(b.y);
        if (fy0 == fy1) continue;
        if (fy0 < fy1) goto DescendingLineBegin;
        else goto AscendingLineBegin;
      }
    }

    {
      /* Clip end point. */
      OPt q = { eb->cx1, eb->cy1 };
      switch (b_flags) {
        case CF_X0 | CF_Y0: q.x = eb->cx0; /* fallthrough */
        case CF_X1 | CF_Y0:
          q.y = A.y + (q.x - A.x) * d.y / d.x;
          if (q.y >= eb->cy0) break;
          /* fallthrough */
        case CF_Y0:
          q.y = eb->cy0;
          q.x = A.x + (q.y - A.y) * d.x / d.y;
          break;
        case CF_X0 | CF_Y1: q.x = eb->cx0; /* fallthrough */
        case CF_X1 | CF_Y1:
          q.y = A.y + (q.x - A.x) * d.y / d.x;
          if (q.y <= eb->cy1) break;
          /* fallthrough */
        case CF_Y1:
          q.y = eb->cy1;
          q.x = A.x + (q.y - A.y) * d.x / d.y;
          break;
        case CF_X0: q.x = eb->cx0; /* fallthrough */
        case CF_X1:
          q.y = A.y + (q.x - A.x) * d.y / d.x;
          break;
        default:
          return -3;
      }
      add_line_segment(eb, p.x, p.y, q.x, q.y);
      double clippedBY = o_clamp(b.y, eb->cy0, eb->cy1);
      if (q.y != clippedBY) {
        if (q.x == eb->cx0) acc_left(eb, q.y, clippedBY);
        else acc_right(eb, q.y, clippedBY);
      }
    }

    A = b;
    AF = b_flags;
  } while (src_maybe_next_line_to(src, &b));

  return 0;
#undef A
#undef AF
}

/* --- Bezier splitting ------------------------------------------------------------------- */

static inline double o_cross(OPt a, OPt b) { return a.x * b.y - a.y * b.x; }
static inline double o_mag_sq(OPt v) { return v.x * v.x + v.y * v.y; }

/* Math::quad_roots (math_p.h:574-592). */
static int o_quad_roots(double dst[2], double a, double b, double c, double t_min, double t_max) {
  double d = o_max(b * b - 4.0 * a * c, 0.0);
  double s = sqrt(d);
  double q = -0.5 * (b + copysign(s, b));
  double t0 = q / a;
  double t1 = c / q;
  double x0 = o_min(t0, t1);
  double x1 = o_max(t1, t0);
  dst[0] = x0;
  int n = (int)((x0 >= t_min) & (x0 <= t_max));
  dst[n] = x1;
  n += (int)((x1 > x0) & (x1 >= t_min) & (x1 <= t_max));
  return n;
}

static const double kAfter0 = 1e-40;
static const double kBefore1 = 0.999999999999999889;

/* split_with_options<kExtremaXY> + split_with_ts (bezier_p.h:331-395). Returns the number of
 * points written past out[0] (0 when the curve needs no split). */
static int o_split_quad(OPt* c) {
  OPt c0 = c[0], c1 = c[1], c2 = c[2];
  double ex = (c0.x - c1.x) / (c0.x - c1.x * 2.0 + c2.x);
  double ey = (c0.y - c1.y) / (c0.y - c1.y * 2.0 + c2.y);
  double t0 = o_min(ex, ey), t1 = o_max(ex, ey);
  double ts[3];
  int n = 0;
  ts[n] = t0; n += (int)((t0 > 0.0) & (t0 < 1.0));
  ts[n] = t1; n += (int)((t1 > o_max(t0, 0.0)) & (t1 < 1.0));
  if (!n) return 0;
  ts[n++] = 1.0;

  OPt v1 = { c1.x - c0.x, c1.y - c0.y }, v2 = { c2.x - c1.x, c2.y - c1.y };
  OPt qa = { v2.x - v1.x, v2.y - v1.y }, qb = { v1.x + v1.x, v1.y + v1.y }, qc = c0;
  OPt last = c2;
  double t_cut = 0.0;
  OPt* out = c;
  int i = 0;
  do {
    double t = ts[i];
    double dt = (t - t_cut) * 0.5;
    OPt cp = { (qa.x * (t * 2.0) + qb.x) * dt, (qa.y * (t * 2.0) + qb.y) * dt };
    OPt tp = { (qa.x * t + qb.x) * t + qc.x, (qa.y * t + qb.y) * t + qc.y };
    if (++i == n) tp = last;
    out[1].x = tp.x - cp.x; out[1].y = tp.y - cp.y;
    out[2] = tp;
    out += 2;
    t_cut = t;
  } while (i != n);
  return (int)(out - c);
}

/* split_cubic_to_spline<kExtremaXYInflectionsCusp> (bezier_p.h:834-920). */
static int o_split_cubic(OPt* c) {
  OPt c0 = c[0], c1 = c[1], c2 = c[2], c3 = c[3];
  OPt v1 = { c1.x - c0.x, c1.y - c0.y }, v2 = { c2.x - c1.x, c2.y - c1.y }, v3 = { c3.x - c2.x, c3.y - c2.y };
  OPt ca = { v3.x - v2.x - v2.x + v1.x, v3.y - v2.y - v2.y + v1.y };
  OPt cb = { 3.0 * (v2.x - v1.x), 3.0 * (v2.y - v1.y) };
  OPt cc = { 3.0 * v1.x, 3.0 * v1.y };
  OPt cd = c0;

  double ts[8];
  int n = 0;
  double q0 = o_cross(cb, ca), q1 = o_cross(cc, ca), q2 = o_cross(cc, cb);
  double t_cusp = (q1 / q0) * -0.5;
  ts[n] = t_cusp; n += (int)((t_cusp > 0.0) & (t_cusp < 1.0));
  n += o_quad_roots(ts + n, q0 * 6.0, q1 * 6.0, q2 * 2.0, kAfter0, kBefore1);

  OPt da = { 3.0 * (v3.x - v2.x - v2.x + v1.x), 3.0 * (v3.y - v2.y - v2.y + v1.y) };
  OPt db = { 6.0 * (v2.x - v1.x), 6.0 * (v2.y - v1.y) };
  OPt dc = { 3.0 * v1.x, 3.0 * v1.y };
  n += o_quad_roots(ts + n, da.x, db.x, dc.x, kAfter0, kBefore1);
  n += o_quad_roots(ts + n, da.y, db.y, dc.y, kAfter0, kBefore1);
  if (!n) return 0;

  for (int i = 1; i < n; i++) {   /* insertion sort */
    double v = ts[i];
    int j = i;
    while (j > 0 && v < ts[j - 1]) { ts[j] = ts[j - 1]; j--; }
    ts[j] = v;
  }
  ts[n++] = 1.0;

  OPt last = c3;
  OPt* out = c;
  int i = 0;
  double t_cut = 0.0;
  do {
    double t = ts[i++];
    if (t == t_cut) continue;
    const double k1Div3 = 1.0 / 3.0;
    double dt = (t - t_cut) * k1Div3;
    OPt tp = { ((ca.x * t + cb.x) * t + cc.x) * t + cd.x, ((ca.y * t + cb.y) * t + cc.y) * t + cd.y };
    if (i == n) tp = last;
    OPt cp1 = { ((ca.x * (t_cut * 3.0) + cb.x * 2.0) * t_cut + cc.x) * dt, ((ca.y * (t_cut * 3.0) + cb.y * 2.0) * t_cut + cc.y) * dt };
    OPt cp2 = { ((ca.x * (t * 3.0) + cb.x * 2.0) * t + cc.x) * dt, ((ca.y * (t * 3.0) + cb.y * 2.0) * t + cc.y) * dt };
    out[1].x = out[0].x + cp1.x; out[1].y = out[0].y + cp1.y;
    out[2].x = tp.x - cp2.x; out[2].y = tp.y - cp2.y;
    out[3] = tp;
    out += 3;
    t_cut = t;
  } while (i != n);
  return (int)(out - c);
}

/* --- monotonic curve flattening (edgebuilder_p.h:426-768) -------------------------------- */

typedef struct {
  int deg;                  /* 2 = quad/conic, 3 = cubic */
  double tol_sq;
  OPt p[4];
  OPt stack[32 * 4];
  int sp;
} OMono;

typedef struct {
  double value, limit;
  OPt p01, p12, p23, p012, p123, p0123;
} OStep;

static inline OPt mid(OPt a, OPt b) { OPt r = { (a.x + b.x) * 0.5, (a.y + b.y) * 0.5 }; return r; }

static void mono_begin(OMono* m, const OPt* src, uint32_t sign) {
  m->sp = 0;
  int n = m->deg + 1;
  for (int i = 0; i < n; i++) m->p[i] = sign ? src[n - 1 - i] : src[i];
}
static inline OPt mono_first(const OMono* m) { return m->p[0]; }
static inline OPt mono_last(const OMono* m) { return m->p[m->deg]; }
static inline int mono_can_pop(const OMono* m) { return m->sp != 0; }
static inline int mono_can_push(const OMono* m) { return m->sp != 32 * (m->deg + 1); }
static inline int mono_is_ltr(const OMono* m) { return mono_first(m).x < mono_last(m).x; }

static void mono_bound_ltr(OMono* m) {
  OPt f = m->p[0], l = m->p[m->deg];
  for (int i = 1; i < m->deg; i++) {
    m->p[i].x = o_clamp(m->p[i].x, f.x, l.x);
    m->p[i].y = o_clamp(m->p[i].y, f.y, l.y);
  }
}
static void mono_bound_rtl(OMono* m) {
  OPt f = m->p[0], l = m->p[m->deg];
  for (int i = 1; i < m->deg; i++) {
    m->p[i].x = o_clamp(m->p[i].x, l.x, f.x);
    m->p[i].y = o_clamp(m->p[i].y, f.y, l.y);
  }
}
static int mono_is_flat(const OMono* m, OStep* s) {
  if (m->deg == 2) {
    OPt v1 = { m->p[1].x - m->p[0].x, m->p[1].y - m->p[0].y };
    OPt v2 = { m->p[2].x - m->p[0].x, m->p[2].y - m->p[0].y };
    double d = o_cross(v2, v1);
    double len_sq = o_mag_sq(v2);
    s->value = d * d;
    s->limit = m->tol_sq * len_sq;
  }
  else {
    OPt v = { m->p[3].x - m->p[0].x, m->p[3].y - m->p[0].y };
    OPt a = { m->p[1].x - m->p[0].x, m->p[1].y - m->p[0].y };
    OPt b = { m->p[2].x - m->p[0].x, m->p[2].y - m->p[0].y };
    double c1 = o_cross(v, a), c2 = o_cross(v, b);
    double d1 = c1 * c1, d2 = c2 * c2;
    double len_sq = o_mag_sq(v);
    s->value = o_max(d1, d2);
    s->limit = m->tol_sq * len_sq;
  }
  return s->value <= s->limit;
}
static void mono_split(const OMono* m, OStep* s) {
  if (m->deg == 2) {
    s->p01 = mid(m->p[0], m->p[1]);
    s->p12 = mid(m->p[1], m->p[2]);
    s->p012 = mid(s->p01, s->p12);
  }
  else {
    s->p01 = mid(m->p[0], m->p[1]);
    s->p12 = mid(m->p[1], m->p[2]);
    s->p23 = mid(m->p[2], m->p[3]);
    s->p012 = mid(s->p01, s->p12);
    s->p123 = mid(s->p12, s->p23);
    s->p0123 = mid(s->p012, s->p123);
  }
}
static inline OPt step_mid(const OMono* m, const OStep* s) { return m->deg == 2 ? s->p012 : s->p0123; }
static void mono_push(OMono* m, const OStep* s) {
  if (m->deg == 2) {
    m->stack[m->sp + 0] = s->p012; m->stack[m->sp + 1] = s->p12; m->stack[m->sp + 2] = m->p[2];
    m->sp += 3;
    m->p[1] = s->p01; m->p[2] = s->p012;
  }
  else {
    m->stack[m->sp + 0] = s->p0123; m->stack[m->sp + 1] = s->p123; m->stack[m->sp + 2] = s->p23; m->stack[m->sp + 3] = m->p[3];
    m->sp += 4;
    m->p[1] = s->p01; m->p[2] = s->p012; m->p[3] = s->p0123;
  }
}
static void mono_discard_and_advance(OMono* m, const OStep* s) {
  if (m->deg == 2) { m->p[0] = s->p012; m->p[1] = s->p12; }
  else { m->p[0] = s->p0123; m->p[1] = s->p123; m->p[2] = s->p23; }
}
static void mono_pop(OMono* m) {
  int n = m->deg + 1;
  m->sp -= n;
  for (int i = 0; i < n; i++) m->p[i] = m->stack[m->sp + i];
}

/* Appender (edgebuilder_p.h:834-877). */
static void app_open_at(OEdgeBuilder* eb, double x, double y) { desc_open(eb); desc_add(eb, TR(x), TR(y)); }
static void app_add_line(OEdgeBuilder* eb, double x, double y) { desc_add(eb, TR(x), TR(y)); }
static void app_close(OEdgeBuilder* eb, uint32_t sign) {
  if (eb->tmp[0].y == eb->tmp[eb->ntmp - 1].y) return; /* degenerate h-line */
  desc_close(eb, sign);
}

static inline double dx_div_dy(OPt a, OPt b) { return (b.x - a.x) / (b.y - a.y); }
static inline double dy_div_dx(OPt a, OPt b) { return (b.y - a.y) / (b.x - a.x); }

static void flatten_safe(OEdgeBuilder* eb, OMono* mc, const OPt* src, uint32_t sign) {
  mono_begin(mc, src, sign);
  if (mono_is_ltr(mc)) mono_bound_ltr(mc); else mono_bound_rtl(mc);
  app_open_at(eb, mono_first(mc).x, mono_first(mc).y);
  for (;;) {
    OStep step;
    if (!mono_is_flat(mc, &step)) {
      if (mono_can_push(mc)) {
        mono_split(mc, &step);
        mono_push(mc, &step);
        continue;
      }
    }
    app_add_line(eb, mono_last(mc).x, mono_last(mc).y);
    if (!mono_can_pop(mc)) break;
    mono_pop(mc);
  }
  app_close(eb, sign);
}

/* flatten_unsafe_mono_curve (edgebuilder_p.h:2071-2445). */
static void flatten_unsafe(OEdgeBuilder* eb, OMono* mc, const OPt* src, uint32_t sign) {
  mono_begin(mc, src, sign);

  double y_start = mono_first(mc).y;
  double y_end = o_min(mono_last(mc).y, eb->cy1);
  if ((y_start >= y_end) | (y_end <= eb->cy0))
    return;

  const double kDeltaLimit = 0.00390625;
  double x_delta = fabs(mono_first(mc).x - mono_last(mc).x);
  uint32_t completely_out = 0;
  OStep step;

  if (x_delta <= kDeltaLimit) {
    y_start = o_max(y_start, eb->cy0);
    double x_min = o_min(mono_first(mc).x, mono_last(mc).x);
    double x_max = o_max(mono_first(mc).x, mono_last(mc).x);
    if (x_max <= eb->cx0) acc_left_s(eb, y_start, y_end, sign);
    else if (x_min >= eb->cx1) acc_right_s(eb, y_start, y_end, sign);
    else {
      app_open_at(eb, mono_first(mc).x, y_start);
      app_add_line(eb, mono_last(mc).x, y_end);
      app_close(eb, sign);
    }
    return;
  }
  else if (mono_is_ltr(mc)) {
    mono_bound_ltr(mc);
    if (y_start < eb->cy0) {
      y_start = eb->cy0;
      for (;;) {
        completely_out = (mono_first(mc).x >= eb->cx1);
        if (completely_out) break;
        if (!mono_is_flat(mc, &step)) {
          mono_split(mc, &step);
          if (step_mid(mc, &step).y <= eb->cy0) { mono_discard_and_advance(mc, &step); continue; }
          if (mono_can_push(mc)) { mono_push(mc, &step); continue; }
        }
        if (mono_last(mc).y > eb->cy0) {
          completely_out = mono_last(mc).x < eb->cx0;
          if (completely_out) goto LeftToRight_BeforeX0_Pop;
          double x_clipped = mono_first(mc).x + (eb->cy0 - mono_first(mc).y) * dx_div_dy(mono_first(mc), mono_last(mc));
          if (x_clipped <= eb->cx0) goto LeftToRight_BeforeX0_Clip;
          completely_out = (x_clipped >= eb->cx1);
          if (completely_out) break;
          app_open_at(eb, x_clipped, eb->cy0);
          goto LeftToRight_AddLine;
        }
        if (!mono_can_pop(mc)) break;
        mono_pop(mc);
      }
      completely_out <<= 2; /* kClipShiftX1 */
    }
    else if (y_start < eb->cy1) {
      if (mono_first(mc).x < eb->cx0) {
        for (;;) {
          completely_out = (mono_first(mc).y >= eb->cy1);
          if (completely_out) break;
          if (!mono_is_flat(mc, &step)) {
            mono_split(mc, &step);
            if (step_mid(mc, &step).x <= eb->cx0) { mono_discard_and_advance(mc, &step); continue; }
            if (mono_can_push(mc)) { mono_push(mc, &step); continue; }
          }
          if (mono_last(mc).x > eb->cx0) {
LeftToRight_BeforeX0_Clip:
            {
              double y_clipped = mono_first(mc).y + (eb->cx0 - mono_first(mc).x) * dy_div_dx(mono_first(mc), mono_last(mc));
              completely_out = (y_clipped >= y_end);
              if (completely_out) break;
              if (y_start < y_clipped) acc_left_s(eb, y_start, y_clipped, sign);
              app_open_at(eb, eb->cx0, y_clipped);
              goto LeftToRight_AddLine;
            }
          }
          completely_out = (mono_last(mc).y >= y_end);
          if (completely_out) break;
LeftToRight_BeforeX0_Pop:
          if (!mono_can_pop(mc)) break;
          mono_pop(mc);
        }
        completely_out <<= 0; /* kClipShiftX0 */
      }
      else if (mono_first(mc).x < eb->cx1) {
        app_open_at(eb, mono_first(mc).x, mono_first(mc).y);
        for (;;) {
          if (!mono_is_flat(mc, &step)) {
            mono_split(mc, &step);
            if (mono_can_push(mc)) { mono_push(mc, &step); continue; }
          }
LeftToRight_AddLine:
          completely_out = mono_last(mc).x > eb->cx1;
          if (completely_out) {
            double y_clipped = mono_first(mc).y + (eb->cx1 - mono_first(mc).x) * dy_div_dx(mono_first(mc), mono_last(mc));
            if (y_clipped <= y_end) {
              y_start = y_clipped;
              app_add_line(eb, eb->cx1, y_clipped);
              break;
            }
          }
          completely_out = mono_last(mc).y >= eb->cy1;
          if (completely_out) {
            double x_clipped = o_min(mono_first(mc).x + (eb->cy1 - mono_first(mc).y) * dx_div_dy(mono_first(mc), mono_last(mc)), eb->cx1);
            app_add_line(eb, x_clipped, eb->cy1);
            completely_out = 0;
            break;
          }
          app_add_line(eb, mono_last(mc).x, mono_last(mc).y);
          if (!mono_can_pop(mc)) break;
          mono_pop(mc);
        }
        app_close(eb, sign);
        completely_out <<= 2;
      }
      else {
        completely_out = CF_X1;
      }
    }
  }
  else {
    mono_bound_rtl(mc);
    if (y_start < eb->cy0) {
      y_start = eb->cy0;
      for (;;) {
        completely_out = (mono_first(mc).x <= eb->cx0);
        if (completely_out) break;
        if (!mono_is_flat(mc, &step)) {
          mono_split(mc, &step);
          if (step_mid(mc, &step).y <= eb->cy0) { mono_discard_and_advance(mc, &step); continue; }
          if (mono_can_push(mc)) { mono_push(mc, &step); continue; }
        }
        if (mono_last(mc).y > eb->cy0) {
          completely_out = mono_last(mc).x > eb->cx1;
          if (completely_out) goto RightToLeft_AfterX1_Pop;
          double x_clipped = mono_first(mc).x + (eb->cy0 - mono_first(mc).y) * dx_div_dy(mono_first(mc), mono_last(mc));
          if (x_clipped >= eb->cx1) goto RightToLeft_AfterX1_Clip;
          completely_out = (x_clipped <= eb->cx0);
          if (completely_out) break;
          app_open_at(eb, x_clipped, eb->cy0);
          goto RightToLeft_AddLine;
        }
        if (!mono_can_pop(mc)) break;
        mono_pop(mc);
      }
      completely_out <<= 0;
    }
    else if (y_start < eb->cy1) {
      if (mono_first(mc).x > eb->cx1) {
        for (;;) {
          completely_out = (mono_first(mc).y >= eb->cy1);
          if (completely_out) break;
          if (!mono_is_flat(mc, &step)) {
            mono_split(mc, &step);
            if (step_mid(mc, &step).x >= eb->cx1) { mono_discard_and_advance(mc, &step); continue; }
            if (mono_can_push(mc)) { mono_push(mc, &step); continue; }
          }
          if (mono_last(mc).x < eb->cx1) {
RightToLeft_AfterX1_Clip:
            {
              double y_clipped = mono_first(mc).y + (eb->cx1 - mono_first(mc).x) * dy_div_dx(mono_first(mc), mono_last(mc));
              completely_out = (y_clipped >= y_end);
              if (completely_out) break;
              if (y_start < y_clipped) acc_right_s(eb, y_start, y_clipped, sign);
              app_open_at(eb, eb->cx1, y_clipped);
              goto RightToLeft_AddLine;
            }
          }
          completely_out = (mono_last(mc).y >= y_end);
          if (completely_out) break;
RightToLeft_AfterX1_Pop:
          if (!mono_can_pop(mc)) break;
          mono_pop(mc);
        }
        completely_out <<= 2;
      }
      else if (mono_first(mc).x > eb->cx0) {
        app_open_at(eb, mono_first(mc).x, mono_first(mc).y);
        for (;;) {
          if (!mono_is_flat(mc, &step)) {
            mono_split(mc, &step);
            if (mono_can_push(mc)) { mono_push(mc, &step); continue; }
          }
RightToLeft_AddLine:
          completely_out = mono_last(mc).x < eb->cx0;
          if (completely_out) {
            double y_clipped = mono_first(mc).y + (eb->cx0 - mono_first(mc).x) * dy_div_dx(mono_first(mc), mono_last(mc));
            if (y_clipped <= y_end) {
              y_start = y_clipped;
              app_add_line(eb, eb->cx0, y_clipped);
              break;
            }
          }
          completely_out = mono_last(mc).y >= eb->cy1;
          if (completely_out) {
            double x_clipped = o_max(mono_first(mc).x + (eb->cy1 - mono_first(mc).y) * dx_div_dy(mono_first(mc), mono_last(mc)), eb->cx0);
            app_add_line(eb, x_clipped, eb->cy1);
            completely_out = 0;
            break;
          }
          app_add_line(eb, mono_last(mc).x, mono_last(mc).y);
          if (!mono_can_pop(mc)) break;
          mono_pop(mc);
        }
        app_close(eb, sign);
        completely_out <<= 0;
      }
      else {
        completely_out = CF_X0;
      }
    }
  }

  if (completely_out && y_start < y_end) {
    if (completely_out & CF_X0) acc_left_s(eb, y_start, y_end, sign);
    else acc_right_s(eb, y_start, y_end, sign);
  }
}

/* --- quad_to / cubic_to / conic_to (edgebuilder_p.h:1618-2022) ------------------------- */

static int eb_curve_to(OEdgeBuilder* eb, OSrc* src, OPt* pa, uint32_t* pa_flags, int deg, int conic) {
  OPt spline[8 * 3 + 1];
  OPt* p0 = pa;
  uint32_t* p0_flags = pa_flags;
  int np = deg + 1;

  if (deg == 3) src_next_cubic_to(src, &spline[1], &spline[2], &spline[3]);
  else if (conic) src_next_conic_to(src, &spline[1], &spline[2]);
  else src_next_quad_to(src, &spline[1], &spline[2]);

  for (;;) {
    uint32_t fl[4];
    uint32_t common = *p0_flags;
    for (int i = 1; i < np; i++) { fl[i] = cf_xy(eb, spline[i]); common &= fl[i]; }
    OPt* pe = &spline[deg];

    if (common) {
      uint32_t end = 0;
      if (common & CF_Y0) {
        for (;;) {
          *p0 = *pe;
          end = deg == 3 ? !src_is_cubic_to(src) : (conic ? !src_is_conic_to(src) : !src_is_quad_to(src));
          if (end) break;
          if (deg == 3) src_next_cubic_to(src, &spline[1], &spline[2], &spline[3]);
          else if (conic) src_next_conic_to(src, &spline[1], &spline[2]);
          else src_next_quad_to(src, &spline[1], &spline[2]);
          int all = 1;
          for (int i = 1; i < np; i++) all &= (spline[i].y <= eb->cy0);
          if (!all) break;
        }
      }
      else if (common & CF_Y1) {
        for (;;) {
          *p0 = *pe;
          end = deg == 3 ? !src_is_cubic_to(src) : (conic ? !src_is_conic_to(src) : !src_is_quad_to(src));
          if (end) break;
          if (deg == 3) src_next_cubic_to(src, &spline[1], &spline[2], &spline[3]);
          else if (conic) src_next_conic_to(src, &spline[1], &spline[2]);
          else src_next_quad_to(src, &spline[1], &spline[2]);
          int all = 1;
          for (int i = 1; i < np; i++) all &= (spline[i].y >= eb->cy1);
          if (!all) break;
        }
      }
      else {
        double y0 = o_clamp(p0->y, eb->cy0, eb->cy1);
        int left = (common & CF_X0) != 0;
        for (;;) {
          *p0 = *pe;
          end = deg == 3 ? !src_is_cubic_to(src) : (conic ? !src_is_conic_to(src) : !src_is_quad_to(src));
          if (end) break;
          if (deg == 3) src_next_cubic_to(src, &spline[1], &spline[2], &spline[3]);
          else if (conic) src_next_conic_to(src, &spline[1], &spline[2]);
          else src_next_quad_to(src, &spline[1], &spline[2]);
          int all = 1;
          for (int i = 1; i < np; i++) all &= left ? (spline[i].x <= eb->cx0) : (spline[i].x >= eb->cx1);
          if (!all) break;
        }
        double y1 = o_clamp(p0->y, eb->cy0, eb->cy1);
        if (left) acc_left(eb, y0, y1); else acc_right(eb, y0, y1);
      }
      *p0_flags = cf_xy(eb, *p0);
      if (end) return 0;
      continue;
    }

    spline[0] = *p0;
    int nout = deg == 3 ? o_split_cubic(spline) : o_split_quad(spline);
    if (nout == 0) nout = deg;
    OPt* sp = spline;
    OPt* se = spline + nout;

    OMono mc;
    mc.deg = deg;
    mc.tol_sq = eb->tol_sq;

    uint32_t any = *p0_flags;
    for (int i = 1; i < np; i++) any |= fl[i];
    if (any) {
      do {
        uint32_t sign = sp[0].y > sp[deg].y;
        flatten_unsafe(eb, &mc, sp, sign);
      } while ((sp += deg) != se);
      *p0 = se[0];
      *p0_flags = fl[deg];
    }
    else {
      do {
        uint32_t sign = sp[0].y > sp[deg].y;
        flatten_safe(eb, &mc, sp, sign);
      } while ((sp += deg) != se);
      *p0 = se[0];
    }

    int more;
    if (deg == 3) { more = src_is_cubic_to(src); if (more) src_next_cubic_to(src, &spline[1], &spline[2], &spline[3]); }
    else if (conic) { more = src_is_conic_to(src); if (more) src_next_conic_to(src, &spline[1], &spline[2]); }
    else { more = src_is_quad_to(src); if (more) src_next_quad_to(src, &spline[1], &spline[2]); }
    if (!more) return 0;
  }
}

/* add_from_source (edgebuilder_p.h:1032-1070). */
static int eb_add_from_source(OEdgeBuilder* eb, OSrc* src, int closed) {
  OPt a;
  uint32_t a_flags;
  while (src_begin(src, &a)) {
    OPt start = a, b;
    int done = 0, rc;
    a_flags = cf_xy(eb, a);
    for (;;) {
      if (src_is_line_to(src)) {
        src_next_line_to(src, &b);
LineTo:
        rc = eb_line_to(eb, src, &a, &a_flags, b);
        if (rc) return rc;
        if (done) break;
      }
      else if (src_is_quad_to(src)) {
        if ((rc = eb_curve_to(eb, src, &a, &a_flags, 2, 0))) return rc;
      }
      else if (src_is_cubic_to(src)) {
        if ((rc = eb_curve_to(eb, src, &a, &a_flags, 3, 0))) return rc;
      }
      else if (src_is_conic_to(src)) {
        if ((rc = eb_curve_to(eb, src, &a, &a_flags, 2, 1))) return rc;
      }
      else {
        b = start;
        done = 1;
        if (closed || src_is_close(src)) goto LineTo;
        break;
      }
    }
  }
  return 0;
}

int o_eb_add_poly(OEdgeBuilder* eb, const double* xy, size_t n, const OMat* m, int ttype) {
  OSrc s;
  memset(&s, 0, sizeof(s));
  s.is_path = 0; s.xy = xy; s.i = 0; s.n = (long)n; s.m = *m; s.affine = ttype > O_TT_SCALE;
  return eb_add_from_source(eb, &s, 1);
}

int o_eb_add_path(OEdgeBuilder* eb, const uint8_t* cmd, const double* xy, size_t n, const OMat* m, int ttype) {
  return o_eb_add_path_ex(eb, cmd, xy, n, m, ttype, 1);
}

/* add_path(view, closed, transform, type) (edgebuilder_p.h:990-1002): `closed` = 0 leaves figures
 * without a CLOSE command open (the stroker's A and C paths). */
int o_eb_add_path_ex(OEdgeBuilder* eb, const uint8_t* cmd, const double* xy, size_t n, const OMat* m, int ttype,
                     int closed) {
  OSrc s;
  memset(&s, 0, sizeof(s));
  s.is_path = 1; s.xy = xy; s.cmd = cmd; s.i = 0; s.n = (long)n; s.m = *m; s.affine = ttype > O_TT_SCALE;
  return eb_add_from_source(eb, &s, closed);
}

/* ============================================================================================
 * Analytic rasterizer (analyticrasterizer_p.h:163-1262)
 * ============================================================================================ */

enum { F_INITIAL = 1, F_VERT_OR_SINGLE = 2, F_RTL = 4 };

typedef struct {
  int ex0, ey0, ex1, ey1, fx0, fy0, fx1, fy1;
  int xErr, yErr, xDlt, yDlt, xRem, yRem, xLift, yLift;
  int dx, dy, savedFy1;
  uint32_t flags;
} ORasState;

typedef struct {
  ORasState s;
  uint64_t* bit_top; size_t bit_stride;   /* in words */
  uint32_t* cell_top; size_t cell_stride; /* in cells */
  uint32_t sign_mask;
  uint32_t band_height, band_offset, band_end;
  uint32_t min_x, max_x;
} ORas;

static inline void acc_err_step_i(int* acc, int* iter, int step, int correction) {
  *iter -= step;
  int mask = *iter >> 31;
  *acc -= mask;
  *iter += mask & correction;
}
static inline void acc_err_step_u(uint32_t* acc, int* iter, int step, int correction) {
  *iter -= step;
  int mask = *iter >> 31;
  *acc -= (uint32_t)mask;
  *iter += mask & correction;
}
static inline void acc_err_multi_step(int* acc, int* iter, int step, int correction, int count) {
  int64_t i = (int64_t)(uint32_t)(*iter);
  i -= (int64_t)((uint64_t)(uint32_t)step * (uint32_t)count);
  if (i < 0) {
    int n = (int)(((uint64_t)(-i) + (uint32_t)correction - 1u) / (uint64_t)(uint32_t)correction);
    *acc += n;
    i += (int64_t)correction * n;
  }
  *iter = (int)i;
}

static inline uint32_t ras_sm(const ORas* r, uint32_t v) { return (v ^ r->sign_mask) - r->sign_mask; }

static inline void cell_merge(uint32_t* row, int x, uint32_t cover, uint32_t area) {
  row[(size_t)(unsigned)x + 0] += (cover << 9) - area;
  row[(size_t)(unsigned)x + 1] += area;
}
static inline void cell_add(uint32_t* row, int x, uint32_t v) { row[(size_t)(unsigned)x] += v; }
static inline void bit_set(uint64_t* row, unsigned i) { row[i / 64u] |= (uint64_t)1 << (i % 64u); }
static void bit_fill(uint64_t* row, unsigned first, unsigned last) {
  size_t ic = first / 64u, ie = last / 64u;
  uint64_t mask = ~(uint64_t)0 << (first % 64u);
  if (ic != ie) {
    row[ic] |= mask;
    mask = ~(uint64_t)0;
    while (++ic != ie) row[ic] = mask;
  }
  mask ^= (~(uint64_t)0 ^ 1u) << (last % 64u);
  row[ic] |= mask;
}
static inline void upd_min(ORas* r, int x) { if ((uint32_t)x < r->min_x) r->min_x = (uint32_t)x; }
static inline void upd_max(ORas* r, int x) { if ((uint32_t)x > r->max_x) r->max_x = (uint32_t)x; }

static int ras_prepare(ORas* r, OEdgePt p0, OEdgePt p1) {
  ORasState* s = &r->s;
  if (p0.y == p1.y) return 0;
  s->dx = p1.x - p0.x;
  s->dy = p1.y - p0.y;
  s->flags = F_INITIAL;
  if (s->dx < 0) { s->flags |= F_RTL; s->dx = -s->dx; }
  s->ex0 = p0.x >> 8; s->ey0 = p0.y >> 8; s->ex1 = p1.x >> 8; s->ey1 = (p1.y - 1) >> 8;
  s->fx0 = p0.x & 255; s->fy0 = p0.y & 255; s->fx1 = p1.x & 255; s->fy1 = ((p1.y - 1) & 255) + 1;
  s->savedFy1 = s->fy1;
  if (s->ey0 != s->ey1) s->fy1 = 256;
  if (s->ex0 == s->ex1 && (s->ey0 == s->ey1 || s->dx == 0)) { s->flags |= F_VERT_OR_SINGLE; return 1; }

  uint64_t x_base = (uint64_t)(uint32_t)s->dx * 256u;
  uint64_t y_base = (uint64_t)(uint32_t)s->dy * 256u;
  s->xLift = (int)(x_base / (unsigned)s->dy);
  s->xRem = (int)(x_base % (unsigned)s->dy);
  s->yLift = (int)(y_base / (unsigned)s->dx);
  s->yRem = (int)(y_base % (unsigned)s->dx);
  s->xDlt = s->dx;
  s->yDlt = s->dy;
  s->xErr = (s->dy >> 1) - 1;
  s->yErr = (s->dx >> 1) - 1;
  if (s->ey0 != s->ey1) {
    uint64_t p = (uint64_t)(256u - (uint32_t)s->fy0) * (uint32_t)s->dx;
    s->xDlt = (int)(p / (unsigned)s->dy);
    s->xErr -= (int)(p % (unsigned)s->dy);
    acc_err_step_i(&s->xDlt, &s->xErr, 0, s->dy);
  }
  if (s->ex0 != s->ex1) {
    uint64_t p = (uint64_t)((s->flags & F_RTL) ? (uint32_t)s->fx0 : 256u - (uint32_t)s->fx0) * (uint32_t)s->dy;
    s->yDlt = (int)(p / (unsigned)s->dx);
    s->yErr -= (int)(p % (unsigned)s->dx);
    acc_err_step_i(&s->yDlt, &s->yErr, 0, s->dx);
  }
  s->yDlt += s->fy0;
  return 1;
}

static void ras_advance_to_y(ORas* r, int y_target) {
  ORasState* s = &r->s;
  if (y_target <= s->ey0) return;
  if (!(s->flags & F_VERT_OR_SINGLE)) {
    int ny = y_target - s->ey0;
    s->xDlt += s->xLift * (ny - 1);
    acc_err_multi_step(&s->xDlt, &s->xErr, s->xRem, s->dy, ny - 1);
    if (s->flags & F_RTL) {
      s->fx0 -= s->xDlt;
      if (s->fx0 < 0) {
        int nx = -(s->fx0 >> 8);
        s->ex0 -= nx;
        s->fx0 &= 255;
        acc_err_multi_step(&s->yDlt, &s->yErr, s->yRem, s->dx, nx);
        s->yDlt += s->yLift * nx;
      }
      if (!(s->dy >= s->dx)) {
        if (!s->fx0) {
          s->fx0 = 256;
          s->ex0--;
          acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
          s->yDlt += s->yLift;
        }
      }
      if (y_target == s->ey1 && s->dy >= s->dx) {
        s->fy1 = s->savedFy1;
        s->xDlt = ((s->ex0 - s->ex1) << 8) + s->fx0 - s->fx1;
      }
      else {
        s->xDlt = s->xLift;
        acc_err_step_i(&s->xDlt, &s->xErr, s->xRem, s->dy);
      }
    }
    else {
      s->fx0 += s->xDlt;
      if (s->fx0 >= 256) {
        int nx = s->fx0 >> 8;
        s->ex0 += nx;
        s->fx0 &= 255;
        acc_err_multi_step(&s->yDlt, &s->yErr, s->yRem, s->dx, nx);
        s->yDlt += s->yLift * nx;
      }
      if (y_target == s->ey1 && s->dy >= s->dx) {
        s->fy1 = s->savedFy1;
        s->xDlt = ((s->ex1 - s->ex0) << 8) + s->fx1 - s->fx0;
      }
      else {
        s->xDlt = s->xLift;
        acc_err_step_i(&s->xDlt, &s->xErr, s->xRem, s->dy);
      }
    }
    if (s->dy >= s->dx) {
      s->yDlt &= 255;
    }
    else {
      int y = ny;
      if (s->flags & F_INITIAL) y--;
      s->yDlt -= y * 256;
    }
  }
  else {
    if (y_target == s->ey1) s->fy1 = s->savedFy1;
  }
  s->fy0 = 0;
  s->ey0 = y_target;
  s->flags &= ~(uint32_t)F_INITIAL;
}

/* rasterize<OPTIONS> with kOptionBandOffset | kOptionRecordMinXMaxX, plus kOptionBandingMode
 * when `banding` is set. Returns 1 when the line is fully rasterized. */
static int ras_rasterize(ORas* r, int banding) {
  ORasState* s = &r->s;
  int ey1_end = s->ey1;
  if (banding) ey1_end = o_imin(ey1_end, (int)r->band_end);

  size_t i = (size_t)((unsigned)ey1_end - (unsigned)s->ey0);
  uint32_t y_offset = (unsigned)s->ey0 - r->band_offset;

  uint64_t* bit_ptr = r->bit_top + (size_t)y_offset * r->bit_stride;
  uint32_t* cell_ptr = r->cell_top + (size_t)y_offset * r->cell_stride;

  if (banding) s->ey0 += (int)i + 1;

  const uint32_t full_cover = ras_sm(r, 256u);

  if (s->flags & F_VERT_OR_SINGLE) {
    uint32_t cover;
    uint32_t area = (uint32_t)s->fx0 + (uint32_t)s->fx1;
    upd_min(r, s->ex0);
    upd_max(r, s->ex0);
    size_t bit_index = (unsigned)s->ex0 / 4u;
    uint64_t bit_mask = (uint64_t)1 << (bit_index % 64u);
    bit_ptr += bit_index / 64u;
    cell_ptr += (unsigned)s->ex0;

    cover = ras_sm(r, (uint32_t)(s->fy1 - s->fy0));
    cell_merge(cell_ptr, 0, cover, cover * area);
    bit_ptr[0] |= bit_mask;

    if (banding) {
      if (!i) {
        if (s->ey0 > s->ey1) return 1;
        s->fy0 = 0;
        s->fy1 = s->ey0 == s->ey1 ? s->savedFy1 : 256;
        return 0;
      }
    }
    else {
      if (!i) return 1;
    }

    bit_ptr += r->bit_stride;
    cell_ptr += r->cell_stride;
    cover = full_cover;
    while (--i) {
      cell_merge(cell_ptr, 0, cover, cover * area);
      cell_ptr += r->cell_stride;
      bit_ptr[0] |= bit_mask;
      bit_ptr += r->bit_stride;
    }

    if (banding) {
      if (s->ey0 <= s->ey1) {
        cell_merge(cell_ptr, 0, cover, cover * area);
        bit_ptr[0] |= bit_mask;
        s->fy0 = 0;
        s->fy1 = s->ey0 == s->ey1 ? s->savedFy1 : 256;
        return 0;
      }
    }

    cover = ras_sm(r, (uint32_t)s->savedFy1);
    cell_merge(cell_ptr, 0, cover, cover * area);
    bit_ptr[0] |= bit_mask;
    return 1;
  }
  else if (s->dy >= s->dx) {
    if (banding) i += (s->ey0 <= s->ey1);

    if (s->flags & F_RTL) {
      upd_max(r, s->ex0);
      for (;;) {
        uint32_t area = (uint32_t)s->fx0;
        uint32_t cov0, cov1;

        s->fx0 -= s->xDlt;
        if (s->fx0 < 0) {
          s->ex0--;
          s->fx0 += 256;
          s->yDlt &= 255;
          if (!area) {
            area = 256;
            acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
            s->yDlt += s->yLift;
            goto VertRightToLeftSingleFirstOrLast;
          }
          bit_set(bit_ptr, (unsigned)(s->ex0 + 0) / 4u);
          bit_set(bit_ptr, (unsigned)(s->ex0 + 1) / 4u);
          cov0 = ras_sm(r, (uint32_t)(s->yDlt - s->fy0));
          area = cov0 * area;
          cell_merge(cell_ptr, s->ex0 + 1, cov0, area);
          cov0 = ras_sm(r, (uint32_t)(s->fy1 - s->yDlt));
          area = cov0 * ((uint32_t)s->fx0 + 256u);
          cell_merge(cell_ptr, s->ex0, cov0, area);
          acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
          s->yDlt += s->yLift;
        }
        else {
VertRightToLeftSingleFirstOrLast:
          bit_set(bit_ptr, (unsigned)s->ex0 / 4u);
          cov0 = ras_sm(r, (uint32_t)(s->fy1 - s->fy0));
          area = cov0 * (area + (uint32_t)s->fx0);
          cell_merge(cell_ptr, s->ex0, cov0, area);
        }

        s->fy0 = 0;
        bit_ptr += r->bit_stride;
        cell_ptr += r->cell_stride;

        if (!i) {
          upd_min(r, s->ex0);
          if (banding) {
            if (s->ey0 > s->ey1) return 1;
            s->xDlt = s->xLift;
            acc_err_step_i(&s->xDlt, &s->xErr, s->xRem, s->dy);
            return 0;
          }
          return 1;
        }

        while (--i) {
          s->xDlt = s->xLift;
          acc_err_step_i(&s->xDlt, &s->xErr, s->xRem, s->dy);
          area = (uint32_t)s->fx0;
          s->fx0 -= s->xDlt;
          if (s->fx0 < 0) {
            s->ex0--;
            s->fx0 += 256;
            s->yDlt &= 255;
            if (!area) {
              area = 256;
              acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
              s->yDlt += s->yLift;
              goto VertRightToLeftSingleInLoop;
            }
            bit_set(bit_ptr, (unsigned)(s->ex0 + 0) / 4u);
            bit_set(bit_ptr, (unsigned)(s->ex0 + 1) / 4u);
            bit_ptr += r->bit_stride;

            cov1 = ras_sm(r, (uint32_t)s->yDlt);
            area = cov1 * area;
            cell_add(cell_ptr, s->ex0 + 2, area);

            cov0 = full_cover - cov1;
            cov1 = (cov1 << 9) - area;
            area = cov0 * ((uint32_t)s->fx0 + 256u);
            cov0 = (cov0 << 9) - area;
            cov1 = cov1 + area;
            cell_add(cell_ptr, s->ex0 + 0, cov0);
            cell_add(cell_ptr, s->ex0 + 1, cov1);
            cell_ptr += r->cell_stride;

            acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
            s->yDlt += s->yLift;
          }
          else {
VertRightToLeftSingleInLoop:
            bit_set(bit_ptr, (unsigned)s->ex0 / 4u);
            bit_ptr += r->bit_stride;
            area = full_cover * (area + (uint32_t)s->fx0);
            cell_merge(cell_ptr, s->ex0, full_cover, area);
            cell_ptr += r->cell_stride;
          }
        }

        if (banding) {
          if (s->ey0 >= s->ey1) {
            s->fy1 = s->savedFy1;
            s->xDlt = ((s->ex0 - s->ex1) << 8) + s->fx0 - s->fx1;
            if (s->ey0 == s->ey1) { upd_min(r, s->ex0); return 0; }
          }
          else {
            upd_min(r, s->ex0);
            s->xDlt = s->xLift;
            acc_err_step_i(&s->xDlt, &s->xErr, s->xRem, s->dy);
            return 0;
          }
        }
        else {
          s->fy1 = s->savedFy1;
          s->xDlt = ((s->ex0 - s->ex1) << 8) + s->fx0 - s->fx1;
        }
      }
    }
    else {
      upd_min(r, s->ex0);
      for (;;) {
        uint32_t area = (uint32_t)s->fx0;
        uint32_t cov0, cov1;

        s->fx0 += s->xDlt;
        bit_set(bit_ptr, (unsigned)s->ex0 / 4u);

        if (s->fx0 <= 256) {
          cov0 = ras_sm(r, (uint32_t)(s->fy1 - s->fy0));
          area = cov0 * (area + (uint32_t)s->fx0);
          cell_merge(cell_ptr, s->ex0, cov0, area);
          if (s->fx0 == 256) {
            s->ex0++;
            s->fx0 = 0;
            s->yDlt += s->yLift;
            acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
          }
        }
        else {
          s->ex0++;
          s->fx0 &= 255;
          s->yDlt &= 255;
          bit_set(bit_ptr, (unsigned)s->ex0 / 4u);
          cov0 = ras_sm(r, (uint32_t)(s->yDlt - s->fy0));
          area = cov0 * (area + 256u);
          cell_merge(cell_ptr, s->ex0 - 1, cov0, area);
          cov0 = ras_sm(r, (uint32_t)(s->fy1 - s->yDlt));
          area = cov0 * (uint32_t)s->fx0;
          cell_merge(cell_ptr, s->ex0, cov0, area);
          s->yDlt += s->yLift;
          acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
        }

        s->fy0 = 0;
        bit_ptr += r->bit_stride;
        cell_ptr += r->cell_stride;

        if (!i) {
          upd_max(r, s->ex0);
          if (banding) {
            if (s->ey0 > s->ey1) return 1;
            s->yDlt += s->yLift;
            acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
            return 0;
          }
          return 1;
        }

        while (--i) {
          s->xDlt = s->xLift;
          acc_err_step_i(&s->xDlt, &s->xErr, s->xRem, s->dy);
          area = (uint32_t)s->fx0;
          s->fx0 += s->xDlt;
          bit_set(bit_ptr, (unsigned)s->ex0 / 4u);

          if (s->fx0 <= 256) {
            bit_ptr += r->bit_stride;
            area = full_cover * (area + (uint32_t)s->fx0);
            cell_merge(cell_ptr, s->ex0, full_cover, area);
            cell_ptr += r->cell_stride;
            if (s->fx0 < 256) continue;
            s->ex0++;
            s->fx0 = 0;
          }
          else {
            s->fx0 &= 255;
            s->yDlt &= 255;
            cov0 = ras_sm(r, (uint32_t)s->yDlt);
            cov1 = cov0 * (area + 256u);
            cov0 = (cov0 << 9) - cov1;
            cell_add(cell_ptr, s->ex0 + 0, cov0);
            s->ex0++;
            cov0 = ras_sm(r, 256u - (uint32_t)s->yDlt);
            area = cov0 * (uint32_t)s->fx0;
            cov0 = (cov0 << 9) - area + cov1;
            cell_add(cell_ptr, s->ex0 + 0, cov0);
            cell_add(cell_ptr, s->ex0 + 1, area);
            cell_ptr += r->cell_stride;
            bit_set(bit_ptr, (unsigned)s->ex0 / 4u);
            bit_ptr += r->bit_stride;
          }
          s->yDlt += s->yLift;
          acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
        }

        if (banding) {
          if (s->ey0 >= s->ey1) {
            s->fy1 = s->savedFy1;
            s->xDlt = ((s->ex1 - s->ex0) << 8) + s->fx1 - s->fx0;
            if (s->ey0 == s->ey1) { upd_max(r, s->ex0); return 0; }
          }
          else {
            upd_max(r, s->ex0);
            s->xDlt = s->xLift;
            acc_err_step_i(&s->xDlt, &s->xErr, s->xRem, s->dy);
            return 0;
          }
        }
        else {
          s->fy1 = s->savedFy1;
          s->xDlt = ((s->ex1 - s->ex0) << 8) + s->fx1 - s->fx0;
        }
      }
    }
  }
  else {
    size_t j = 1;
    int x_local = (s->ex0 << 8) + s->fx0;
    uint32_t cover, area;

    if (s->flags & F_RTL) {
      upd_max(r, s->ex0);
      if (s->flags & F_INITIAL) {
        s->flags &= ~(uint32_t)F_INITIAL;
        j = i;
        i = 1;
        cover = ras_sm(r, (uint32_t)(s->yDlt - s->fy0));
        if (s->fx0 - s->xDlt < 0) goto HorzRightToLeftInside;
        x_local -= s->xDlt;
        bit_set(bit_ptr, (unsigned)s->ex0 / 4u);
        cover = ras_sm(r, (uint32_t)(s->fy1 - s->fy0));
        area = cover * (uint32_t)(s->fx0 * 2 - s->xDlt);
        cell_merge(cell_ptr, s->ex0, cover, area);
        if ((x_local & 255) == 0) {
          s->yDlt += s->yLift;
          acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
        }
        s->xDlt = s->xLift;
        acc_err_step_i(&s->xDlt, &s->xErr, s->xRem, s->dy);
        bit_ptr += r->bit_stride;
        cell_ptr += r->cell_stride;
        i--;
      }

      for (;;) {
        while (i) {
          s->ex0 = ((x_local - 1) >> 8);
          s->fx0 = ((x_local - 1) & 255) + 1;
HorzRightToLeftSkip:
          s->yDlt -= 256;
          cover = ras_sm(r, (uint32_t)s->yDlt);
HorzRightToLeftInside:
          x_local -= s->xDlt;
          {
            int ex_local = x_local >> 8;
            int fx_local = x_local & 255;
            bit_fill(bit_ptr, (unsigned)ex_local / 4u, (unsigned)s->ex0 / 4u);
            area = cover * (uint32_t)s->fx0;
            while (s->ex0 != ex_local) {
              cell_merge(cell_ptr, s->ex0, cover, area);
              cover = (uint32_t)s->yLift;
              acc_err_step_u(&cover, &s->yErr, s->yRem, s->dx);
              s->yDlt += (int32_t)cover;
              cover = ras_sm(r, cover);
              area = cover * 256u;
              s->ex0--;
            }
            cover += ras_sm(r, (uint32_t)(s->fy1 - s->yDlt));
            area = cover * ((uint32_t)fx_local + 256u);
            cell_merge(cell_ptr, s->ex0, cover, area);
            if (fx_local == 0) {
              s->yDlt += s->yLift;
              acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
            }
          }
          s->xDlt = s->xLift;
          acc_err_step_i(&s->xDlt, &s->xErr, s->xRem, s->dy);
          bit_ptr += r->bit_stride;
          cell_ptr += r->cell_stride;
          i--;
        }

        s->fy0 = 0;
        s->fy1 = 256;

        if (banding) {
          if (!j) {
            upd_min(r, s->ex0);
            s->ex0 = ((x_local - 1) >> 8);
            s->fx0 = ((x_local - 1) & 255) + 1;
            return s->ey0 > s->ey1;
          }
        }
        else {
          if (!j) { upd_min(r, s->ex0); return 1; }
        }

        i = j - 1;
        j = 1;

        if (!i) {
          i = 1;
          j = 0;
          int is_last = banding ? (s->ey0 > s->ey1) : 1;
          if (!is_last) continue;

          s->xDlt = x_local - ((s->ex1 << 8) + s->fx1);
          s->fy1 = s->savedFy1;
          s->ex0 = ((x_local - 1) >> 8);
          s->fx0 = ((x_local - 1) & 255) + 1;

          if (s->fx0 - s->xDlt >= 0) {
            cover = ras_sm(r, (uint32_t)s->fy1);
            area = cover * (uint32_t)(s->fx0 * 2 - s->xDlt);
            cell_merge(cell_ptr, s->ex0, cover, area);
            bit_set(bit_ptr, (unsigned)s->ex0 / 4u);
            upd_min(r, s->ex0);
            return 1;
          }
          goto HorzRightToLeftSkip;
        }
      }
    }
    else {
      upd_min(r, s->ex0);
      if (s->flags & F_INITIAL) {
        s->flags &= ~(uint32_t)F_INITIAL;
        j = i;
        i = 1;
        cover = ras_sm(r, (uint32_t)(s->yDlt - s->fy0));
        if (s->fx0 + s->xDlt > 256) goto HorzLeftToRightInside;
        x_local += s->xDlt;
        bit_set(bit_ptr, (unsigned)s->ex0 / 4u);
        cover = ras_sm(r, (uint32_t)(s->fy1 - s->fy0));
        area = cover * ((uint32_t)s->fx0 * 2u + (uint32_t)s->xDlt);
        cell_merge(cell_ptr, s->ex0, cover, area);
        if (s->fx0 + s->xDlt == 256) {
          s->yDlt += s->yLift;
          acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
        }
        s->xDlt = s->xLift;
        acc_err_step_i(&s->xDlt, &s->xErr, s->xRem, s->dy);
        bit_ptr += r->bit_stride;
        cell_ptr += r->cell_stride;
        i--;
      }

      for (;;) {
        while (i) {
          s->ex0 = x_local >> 8;
          s->fx0 = x_local & 255;
HorzLeftToRightSkip:
          s->yDlt -= 256;
          cover = ras_sm(r, (uint32_t)s->yDlt);
HorzLeftToRightInside:
          x_local += s->xDlt;
          {
            int ex_local = (x_local - 1) >> 8;
            int fx_local = ((x_local - 1) & 255) + 1;
            bit_fill(bit_ptr, (unsigned)s->ex0 / 4u, (unsigned)ex_local / 4u);
            area = cover * ((uint32_t)s->fx0 + 256u);
            while (s->ex0 != ex_local) {
              cell_merge(cell_ptr, s->ex0, cover, area);
              cover = (uint32_t)s->yLift;
              acc_err_step_u(&cover, &s->yErr, s->yRem, s->dx);
              s->yDlt += (int32_t)cover;
              cover = ras_sm(r, cover);
              area = cover * 256u;
              s->ex0++;
            }
            cover += ras_sm(r, (uint32_t)(s->fy1 - s->yDlt));
            area = cover * (uint32_t)fx_local;
            cell_merge(cell_ptr, s->ex0, cover, area);
            if (fx_local == 256) {
              s->yDlt += s->yLift;
              acc_err_step_i(&s->yDlt, &s->yErr, s->yRem, s->dx);
            }
          }
          s->xDlt = s->xLift;
          acc_err_step_i(&s->xDlt, &s->xErr, s->xRem, s->dy);
          bit_ptr += r->bit_stride;
          cell_ptr += r->cell_stride;
          i--;
        }

        s->fy0 = 0;
        s->fy1 = 256;

        if (banding) {
          if (!j) {
            upd_max(r, s->ex0);
            s->ex0 = x_local >> 8;
            s->fx0 = x_local & 255;
            return s->ey0 > s->ey1;
          }
        }
        else {
          if (!j) { upd_max(r, s->ex0); return 1; }
        }

        i = j - 1;
        j = 1;

        if (!i) {
          i = 1;
          j = 0;
          int is_last = banding ? (s->ey0 > s->ey1) : 1;
          if (!is_last) continue;

          s->xDlt = ((s->ex1 << 8) + s->fx1) - x_local;
          s->fy1 = s->savedFy1;
          s->ex0 = x_local >> 8;
          s->fx0 = x_local & 255;

          if (s->fx0 + s->xDlt <= 256) {
            cover = ras_sm(r, (uint32_t)s->fy1);
            area = cover * ((uint32_t)s->fx0 * 2u + (uint32_t)s->xDlt);
            cell_merge(cell_ptr, s->ex0, cover, area);
            bit_set(bit_ptr, (unsigned)s->ex0 / 4u);
            upd_max(r, s->ex0);
            return 1;
          }
          goto HorzLeftToRightSkip;
        }
      }
    }
  }
}

/* ============================================================================================
 * Band loop (rendercommandprocsync_p.h:87-254)
 * ============================================================================================ */

typedef struct {
  ORasState state;
  uint32_t sign_bit;
  int cur, end;    /* indices into storage points: `cur` is the end point of the active segment */
} OActive;

int o_fill_analytic(OFillCtx* fc, const OEdgeStorage* st, uint32_t fill_rule) {
  if (st->nedges == 0 || st->bbox_y0 >= st->bbox_y1)
    return 0;

  uint32_t band_height = (uint32_t)st->band_height;
  uint32_t band_height_mask = band_height - 1u;
  const uint32_t y_start = ((uint32_t)st->bbox_y0) >> 8;
  const uint32_t y_end = ((uint32_t)st->bbox_y1 + 255u) >> 8;

  ORas ras;
  memset(&ras, 0, sizeof(ras));
  ras.bit_top = fc->bits; ras.bit_stride = fc->bit_stride;
  ras.cell_top = fc->cells; ras.cell_stride = fc->cell_stride;

  uint32_t band_id = ((unsigned)st->bbox_y0) >> st->shift;
  uint32_t band_end = (uint32_t)o_imin((int)(((unsigned)st->bbox_y1 >> st->shift) + 1), st->band_count);

  ras.band_height = band_height;
  ras.band_offset = y_start;

  OActive* active = (OActive*)malloc(sizeof(OActive) * (st->nedges + 1));
  size_t nactive = 0;
  OActive* next_active = (OActive*)malloc(sizeof(OActive) * (st->nedges + 1));

  do {
    size_t nnext = 0;
    ras.min_x = UINT32_MAX;
    ras.max_x = 0;
    ras.band_end = (uint32_t)o_imin((int)((band_id + 1) * band_height), (int)y_end) - 1u;

    for (size_t k = 0; k < nactive; k++) {
      OActive* cur = &active[k];
      ras.s = cur->state;
      ras.sign_mask = 0u - cur->sign_bit;
      for (;;) {
        if (ras_rasterize(&ras, 1)) {
          int done = 1;
          while (cur->cur != cur->end) {
            cur->cur++;
            if (!ras_prepare(&ras, st->pts[cur->cur - 1], st->pts[cur->cur]))
              continue;
            if ((uint32_t)ras.s.ey0 <= ras.band_end) { done = 0; break; }
            done = 2; break;
          }
          if (done == 0) continue;       /* rasterize the next segment */
          if (done == 1) break;          /* edge fully rasterized: drop it */
        }
        cur->state = ras.s;              /* crosses the band: keep it active */
        next_active[nnext++] = *cur;
        break;
      }
    }

    for (int e = st->band_first[band_id]; e >= 0; e = st->edges[e].next) {
      const OEdge* ed = &st->edges[e];
      int p = ed->first + 1;
      int pend = ed->first + ed->count - 1;   /* index of the last point */
      uint32_t sign_bit = ed->sign;
      ras.sign_mask = 0u - sign_bit;
      for (;;) {
        int ok = ras_prepare(&ras, st->pts[p - 1], st->pts[p]);
        if (ok) {
          if ((uint32_t)ras.s.ey1 <= ras.band_end) {
            ras_rasterize(&ras, 0);
          }
          else {
            OActive a;
            a.sign_bit = sign_bit;
            a.cur = p;
            a.end = pend;
            /* Rasterize within this band (or save) following the reference control flow. */
            for (;;) {
              if ((uint32_t)ras.s.ey0 <= ras.band_end) {
                if (ras_rasterize(&ras, 1)) {
                  int done = 1;
                  while (a.cur != a.end) {
                    a.cur++;
                    if (!ras_prepare(&ras, st->pts[a.cur - 1], st->pts[a.cur]))
                      continue;
                    done = ((uint32_t)ras.s.ey0 <= ras.band_end) ? 0 : 2;
                    break;
                  }
                  if (done == 0) continue;
                  if (done == 1) break;
                }
              }
              a.state = ras.s;
              next_active[nnext++] = a;
              break;
            }
            break; /* the rest of this edge is owned by the active entry */
          }
        }
        if (p == pend) break;
        p++;
      }
    }

    { OActive* t = active; active = next_active; next_active = t; nactive = nnext; }

    if (ras.min_x <= ras.max_x) {
      uint32_t x1a = (ras.max_x + 1u + 3u) & ~3u;
      int box_x1 = (int)((uint32_t)fc->width < x1a ? (uint32_t)fc->width : x1a);
      o_fill_analytic_band(fc, box_x1, (int)ras.band_offset, (int)ras.band_end + 1, fill_rule, fc->bits, fc->cells);
    }

    ras.band_offset = (ras.band_offset + band_height) & ~band_height_mask;
  } while (++band_id < band_end);

  free(active);
  free(next_active);
  return 0;
}

/* Known-answer helper: one line, rows [0, rows), band height `band_height`. */
int b2d_oracle_rasterize_line(int x0, int y0, int x1, int y1, uint32_t sign, uint32_t band_height,
                              int width, int rows, uint32_t* cells) {
  size_t cstride = (size_t)width + 2;
  size_t wwords = ((size_t)width + 2 + 255) / 256 + 1;
  uint64_t* bits = (uint64_t*)calloc((size_t)band_height * wwords, sizeof(uint64_t));
  uint32_t* band_cells = (uint32_t*)calloc((size_t)band_height * cstride, sizeof(uint32_t));
  memset(cells, 0, (size_t)rows * cstride * sizeof(uint32_t));

  ORas ras;
  memset(&ras, 0, sizeof(ras));
  ras.bit_top = bits; ras.bit_stride = wwords;
  ras.cell_top = band_cells; ras.cell_stride = cstride;
  ras.sign_mask = 0u - sign;
  OEdgePt p0 = { x0, y0 }, p1 = { x1, y1 };
  if (!ras_prepare(&ras, p0, p1)) { free(bits); free(band_cells); return 0; }

  uint32_t band_start = (uint32_t)(y0 >> 8) / band_height * band_height;
  ras.band_offset = (uint32_t)(y0 >> 8);
  int done = 0;
  for (uint32_t b = band_start; !done && (int)b < rows; b += band_height) {
    ras.band_end = b + band_height - 1u;
    if ((uint32_t)ras.s.ey0 <= ras.band_end)
      done = ras_rasterize(&ras, 1);
    for (uint32_t yy = 0; yy < band_height && (int)(ras.band_offset + yy) < rows; yy++)
      for (size_t x = 0; x < cstride; x++)
        cells[(ras.band_offset + yy) * cstride + x] += band_cells[yy * cstride + x];
    memset(band_cells, 0, (size_t)band_height * cstride * sizeof(uint32_t));
    ras.band_offset = b + band_height;
  }
  free(bits);
  free(band_cells);
  return 1;
}
