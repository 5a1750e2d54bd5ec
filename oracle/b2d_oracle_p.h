/*
 * b2d_oracle_p.h - private declarations of the CPU oracle (test infrastructure only).
 *
 * Numeric conventions: everything follows x86-64 baseline semantics of the reference build
 * (SSE2 scalar double/float, no FMA contraction: compile with -ffp-contract=off), including
 * the x86 behaviour of float->int conversions for NaN/out-of-range values (INT_MIN).
 */
#ifndef B2D_ORACLE_P_H_INCLUDED
#define B2D_ORACLE_P_H_INCLUDED

#include <limits.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "b2d_oracle.h"

/* --- scalar helpers (blend2d/core/api.h:1742-1752, blend2d/support/math_p.h) ------------------ */

static inline double o_min(double a, double b) { return b < a ? b : a; }
static inline double o_max(double a, double b) { return a < b ? b : a; }
static inline double o_clamp(double a, double lo, double hi) { return o_min(hi, o_max(lo, a)); }
static inline int o_imin(int a, int b) { return b < a ? b : a; }
static inline int o_imax(int a, int b) { return a < b ? b : a; }

/* cvttsd2si: truncation, INT_MIN for NaN / out of range (math_p.h:388 `int(x)` on x86-64). */
static inline int o_trunc_to_int(double x) {
  if (!(x > -2147483649.0 && x < 2147483648.0)) return INT_MIN;
  return (int)x;
}
static inline int64_t o_trunc_to_int64(double x) {
  if (!(x >= -9223372036854775808.0 && x < 9223372036854775808.0)) return INT64_MIN;
  return (int64_t)x;
}
/* cvtsd2si: round-half-even, INT_MIN for NaN / out of range (math_p.h:370-376). */
static inline int o_nearby_to_int(double x) {
  if (!(x >= -2147483648.5 && x < 2147483647.5)) return INT_MIN;
  return (int)rint(x);
}
static inline int o_round_to_int(double x) {   /* math_p.h:404 */
  int y = o_nearby_to_int(x);
  return y + ((double)y - x == -0.5);
}
static inline int64_t o_floor_to_int64(double x) {   /* math_p.h:437 */
  int64_t y = o_trunc_to_int64(x);
  return y - (int64_t)((double)y > x);
}
/* cvtss2si / cvttss2si for float. */
static inline int o_nearby_to_int_f(float x) {
  if (!(x >= -2147483648.0f && x < 2147483648.0f)) return INT_MIN;
  return (int)rintf(x);
}
static inline int o_trunc_to_int_f(float x) {
  if (!(x >= -2147483648.0f && x < 2147483648.0f)) return INT_MIN;
  return (int)x;
}

typedef struct { double x, y; } OPt;
typedef struct { double m00, m01, m10, m11, m20, m21; } OMat;

enum { O_TT_IDENTITY = 0, O_TT_TRANSLATE = 1, O_TT_SCALE = 2, O_TT_SWAP = 3, O_TT_AFFINE = 4, O_TT_INVALID = 5 };

void o_mat_multiply(OMat* dst, const OMat* a, const OMat* b);
int o_mat_invert(OMat* dst, const OMat* src);
int o_mat_type(const OMat* m);
static inline OPt o_mat_map(const OMat* m, double x, double y) {
  OPt r = { x * m->m00 + y * m->m10 + m->m20, x * m->m01 + y * m->m11 + m->m21 };
  return r;
}

/* --- edge storage ------------------------------------------------------------------------- */

typedef struct { int x, y; } OEdgePt;

typedef struct {
  int first;        /* index into pts */
  int count;
  uint32_t sign;
  int next;         /* next edge in the same band list, -1 terminates */
} OEdge;

typedef struct {
  OEdgePt* pts; size_t npts, cap_pts;
  OEdge* edges; size_t nedges, cap_edges;
  int* band_first; int* band_last;
  int band_count;
  int band_height;
  int shift;             /* ctz(band_height) + 8 */
  int bbox_y0, bbox_y1;  /* fixed-point bounding box of linked edges (y only) */
} OEdgeStorage;

typedef struct {
  OEdgeStorage* st;
  double cx0, cy0, cx1, cy1;   /* clip box, fixed point (double) */
  int icx0, icy0, icx1, icy1;  /* clip box, fixed point (int) */
  double tol_sq;
  /* current open polyline */
  OEdgePt* tmp; size_t ntmp, cap_tmp;
  int ascending;
  /* border accumulators (edgebuilder_p.h:813-816) */
  double acc_x0_y0, acc_x0_y1, acc_x1_y0, acc_x1_y1;
} OEdgeBuilder;

void o_storage_init(OEdgeStorage* st, int width, int height, int band_height);
void o_storage_free(OEdgeStorage* st);
void o_storage_clear(OEdgeStorage* st);

void o_eb_init(OEdgeBuilder* eb, OEdgeStorage* st, int width, int height, double tol_sq);
void o_eb_free(OEdgeBuilder* eb);
void o_eb_begin(OEdgeBuilder* eb);
/* Polygon / path edge building (edgebuilder_p.h:959-1070). Returns 0 or an error. */
int o_eb_add_poly(OEdgeBuilder* eb, const double* xy, size_t n, const OMat* m, int ttype);
int o_eb_add_path(OEdgeBuilder* eb, const uint8_t* cmd, const double* xy, size_t n, const OMat* m, int ttype);
int o_eb_add_path_ex(OEdgeBuilder* eb, const uint8_t* cmd, const double* xy, size_t n, const OMat* m, int ttype,
                     int closed);
int o_eb_done(OEdgeBuilder* eb);

/* --- analytic fill --------------------------------------------------------------------- */

struct OFillCtx;
/* Band loop of CommandProcSync::fill_analytic (rendercommandprocsync_p.h:87-254) - calls
 * `o_fill_analytic_band` for each band that received cells. */
int o_fill_analytic(struct OFillCtx* fc, const OEdgeStorage* st, uint32_t fill_rule);

/* --- pipeline ------------------------------------------------------------------------ */

enum {
  O_FT_SOLID = 0,
  O_FT_LINEAR_PAD, O_FT_LINEAR_ROR,
  O_FT_RADIAL_PAD, O_FT_RADIAL_ROR,
  O_FT_CONIC,
  O_FT_PAT_ALIGNED_PAD, O_FT_PAT_ALIGNED_REPEAT, O_FT_PAT_ALIGNED_ROR,
  O_FT_PAT_FXFY_PAD, O_FT_PAT_FXFY_ROR,
  O_FT_PAT_AFFINE_NN, O_FT_PAT_AFFINE_BI
};

enum { O_FMT_PRGB32 = 0, O_FMT_FRGB32 = 1, O_FMT_ZERO32 = 2, O_FMT_XRGB32 = 3 };

typedef struct OStyle {
  int nop;                     /* style resolves to nothing (NoFillStyle) */
  int format;                  /* O_FMT_* of the source */
  int fetch_type;              /* O_FT_* */
  uint32_t solid;              /* premultiplied PRGB32 for O_FT_SOLID */
  /* gradient */
  uint32_t lut[1024];
  uint32_t lut_size;
  int dither;                  /* BL_GRADIENT_QUALITY_DITHER: 64-bit LUT + ordered dither */
  uint64_t lut64[1024];
  uint64_t lin_pt0, lin_dt, lin_dy;
  uint32_t maxi, rori;
  double rad_tx, rad_ty, rad_yx, rad_yy, rad_b0, rad_by, rad_dd0, rad_ddy, rad_inv2a, rad_amul4, rad_sq_inv2a, rad_sq_fr;
  float rad_bd, rad_ddd;
  double con_tx, con_ty, con_yx, con_yy;
  float con_q[4], con_n1, con_n2, con_n4, con_offset, con_xx;
  int32_t con_maxi, con_rori;
  /* pattern source (area origin) */
  const uint32_t* src; int src_w, src_h; intptr_t src_stride; /* stride in pixels */
  /* pattern simple (aligned / fx-fy) */
  int pat_tx, pat_ty, pat_rx, pat_ry;
  uint32_t pat_wa, pat_wb, pat_wc, pat_wd;
  intptr_t vx_stride0, vx_stride1, vx_ystop0, vx_ystop1, vx_ptr_rewind; uintptr_t vx_y_rewind;
  /* pattern affine */
  uint64_t af_xx, af_xy, af_yx, af_yy, af_tx, af_ty;
  int32_t af_ox, af_oy, af_rx, af_ry, af_minx, af_miny, af_maxx, af_maxy, af_corx, af_cory, af_tw, af_th;
} OStyle;

typedef struct OFillCtx {
  uint32_t* dst; int width, height; intptr_t stride;  /* stride in pixels */
  int comp_op;            /* after simplification: 0 SrcOver, 1 SrcCopy */
  uint32_t alpha;         /* 0..255 */
  uint32_t src_or;        /* 0xFF000000 when the pattern fetcher reads its source as XRGB32 */
  const OStyle* style;
  /* scratch for analytic fills */
  uint32_t* cells; uint64_t* bits; size_t cell_stride, bit_stride; /* in elements */
  B2DOracleStats* stats;
} OFillCtx;

void o_fill_box_a(OFillCtx* fc, int x0, int y0, int x1, int y1);
void o_fill_box_u(OFillCtx* fc, int x0, int y0, int x1, int y1);
void o_fill_mask_a(OFillCtx* fc, int x0, int y0, int x1, int y1, const uint8_t* mask, intptr_t mask_stride);
void o_fill_analytic_band(OFillCtx* fc, int box_x1, int y0, int y1, uint32_t fill_rule,
                          uint64_t* bit_top, uint32_t* cell_top);

uint32_t o_premultiply(uint32_t argb32);

#endif /* B2D_ORACLE_P_H_INCLUDED */
