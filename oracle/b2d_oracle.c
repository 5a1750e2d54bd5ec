/*
 * b2d_oracle.c - oracle (test infrastructure): command-stream replay with the reference's
 * synchronous rendering-context front end, restated from:
 *   state & alpha        blend2d/raster/rastercontext.cpp:1919-2027, :4380-4415
 *   transforms           blend2d/raster/rastercontext.cpp:740-800, blend2d/core/matrix.cpp:292-324
 *   style resolution     blend2d/raster/rastercontext.cpp:363-494, :572-695, :1231-1453
 *   comp-op simplify     blend2d/core/compopsimplifyimpl_p.h:86-162
 *   fetch-data setup     blend2d/pipeline/pipedefs.cpp:17-699
 *   gradient info/stops  blend2d/core/gradient.cpp:58-173, :202-287
 *   fill dispatch        blend2d/raster/rastercontext.cpp:2633-2990, :3317-3500
 *   band height          blend2d/raster/rastercontext.cpp:4154-4193
 */
#include "b2d_oracle_p.h"
#include "b2d_oracle_stroke.h"
#include "blgpu_stream.h"

/* ============================================================================================
 * Fetch-data setup
 * ============================================================================================ */

static void o_init_pattern_simple(OStyle* st, uint32_t extend, int tx, int ty, int fractional, int base_is_fxfy) {
  uint32_t ex = extend, ey = extend;   /* simple extend modes only */
  int rx = 0, ry = 0;
  if (st->src_w <= 1) ex = 0;
  if (st->src_h <= 1) ey = 0;
  if (ex >= 1) {
    int is_reflect = ex == 2;
    rx = st->src_w << is_reflect;
    if ((unsigned)tx >= (unsigned)rx) tx %= rx;
    if (tx < 0) tx += rx;
    if (fractional) ex = 1;
  }
  st->vx_stride0 = st->src_stride;
  st->vx_stride1 = 0;
  st->vx_ystop0 = st->src_h;
  st->vx_ystop1 = 0;
  st->vx_y_rewind = 0;
  st->vx_ptr_rewind = (ey != 1 ? 0 : (intptr_t)(st->src_h - 1)) * st->src_stride;
  if (ey >= 1) {
    ry = st->src_h << (ey == 2);
    if ((unsigned)ty >= (unsigned)ry) ty %= ry;
    if (ty < 0) ty += ry;
    st->vx_stride1 = (ey == 1) ? st->src_stride : -st->src_stride;
    st->vx_ystop1 = st->src_h;
    st->vx_y_rewind = (uintptr_t)st->src_h;
  }
  st->pat_tx = tx; st->pat_ty = ty; st->pat_rx = rx; st->pat_ry = ry;
  if (base_is_fxfy) st->fetch_type = ex == 0 ? O_FT_PAT_FXFY_PAD : O_FT_PAT_FXFY_ROR;
  else st->fetch_type = ex == 0 ? O_FT_PAT_ALIGNED_PAD : (ex == 1 ? O_FT_PAT_ALIGNED_REPEAT : O_FT_PAT_ALIGNED_ROR);
}

static void o_init_pattern_fx_fy(OStyle* st, uint32_t extend, uint32_t quality, int64_t tx64, int64_t ty64) {
  int fxfy = 0;
  uint32_t wx = (uint32_t)(tx64 & 0xFF), wy = (uint32_t)(ty64 & 0xFF);
  int tx = -(int)(tx64 >> 8), ty = -(int)(ty64 >> 8);
  int fractional = (wx | wy) != 0;
  if (fractional) {
    if (quality == 0) {
      tx -= (wx >= 128);
      ty -= (wy >= 128);
      fractional = 0;
    }
    else {
      st->pat_wa = ((wy) * (wx)) >> 8;
      st->pat_wb = ((wy) * (256 - wx) + 255) >> 8;
      st->pat_wc = ((256 - wy) * (wx)) >> 8;
      st->pat_wd = ((256 - wy) * (256 - wx) + 255) >> 8;
      tx--;
      ty--;
      fxfy = 1;
    }
  }
  o_init_pattern_simple(st, extend, tx, ty, fractional, fxfy);
}

static int o_is_near(double x, double y) { return fabs(x - y) <= 1e-14; }

/* init_pattern_affine (pipedefs.cpp:162-381). Returns 0 when the pattern is a NOP. */
static int o_init_pattern_affine(OStyle* st, uint32_t extend, uint32_t quality, const OMat* transform) {
  OMat inv;
  if (!o_mat_invert(&inv, transform)) return 0;
  int tw = st->src_w, th = st->src_h;
  if (tw == 0) return 0;

  double xx = inv.m00, xy = inv.m01, yx = inv.m10, yy = inv.m11;
  if (o_is_near(xx, 1.0) & (fabs(xy) <= 1e-14) & (fabs(yx) <= 1e-14) & o_is_near(yy, 1.0)) {
    int64_t tx64 = o_floor_to_int64(-inv.m20 * 256.0);
    int64_t ty64 = o_floor_to_int64(-inv.m21 * 256.0);
    o_init_pattern_fx_fy(st, extend, quality, tx64, ty64);
    return 1;
  }

  st->fetch_type = quality == 0 ? O_FT_PAT_AFFINE_NN : O_FT_PAT_AFFINE_BI;
  uint32_t ex = extend, ey = extend;
  double tx = inv.m20, ty = inv.m21;
  tx += 0.5 * (xx + yx);
  ty += 0.5 * (xy + yy);
  double fp_scale = 4294967296.0;
  int ox = INT32_MAX, oy = INT32_MAX, rx = 0, ry = 0;

  st->af_minx = 0; st->af_miny = 0;
  st->af_maxx = tw - 1; st->af_maxy = th - 1;
  st->af_corx = tw - 1; st->af_cory = th - 1;

  if (ex != 0) {
    st->af_minx = INT32_MIN;
    if (ex == 1) st->af_corx = 0;
    ox = tw;
    if (ex == 2) tw *= 2;
    if (xx < 0.0) {
      xx = -xx; yx = -yx; tx = (double)tw - tx;
      if (ex == 1) { ox = 0; st->af_corx = st->af_maxx; st->af_maxx = -1; }
    }
    ox--;
  }
  if (ey != 0) {
    st->af_miny = INT32_MIN;
    if (ey == 1) st->af_cory = 0;
    oy = th;
    if (ey == 2) th *= 2;
    if (xy < 0.0) {
      xy = -xy; yy = -yy; ty = (double)th - ty;
      if (ey == 1) { oy = 0; st->af_cory = st->af_maxy; st->af_maxy = -1; }
    }
    oy--;
  }
  if (quality != 0) { tx -= 0.5; ty -= 0.5; }

  double tw_d = (double)tw, th_d = (double)th;
  if (ex == 0) tw_d = 2147483647.0;
  else { tx = fmod(tx, tw_d); rx = tw; if (xx >= tw_d) xx = fmod(xx, tw_d); }
  if (ey == 0) th_d = 2147483647.0;
  else { ty = fmod(ty, th_d); ry = th; if (xy >= th_d) xy = fmod(xy, th_d); }

  xx *= fp_scale; xy *= fp_scale; yx *= fp_scale; yy *= fp_scale; tx *= fp_scale; ty *= fp_scale;

  double all_min = o_min(o_min(yy, yx), o_min(xy, xx));
  double all_max = o_max(o_max(xx, xy), o_max(yx, yy));
  all_min = o_min(all_min, o_min(ty, tx));
  all_max = o_max(o_max(tx, ty), all_max);
  if (all_min >= (double)(INT64_MIN + 1) && all_max <= (double)INT64_MAX) {
    st->af_xx = (uint64_t)o_floor_to_int64(xx); st->af_xy = (uint64_t)o_floor_to_int64(xy);
    st->af_yx = (uint64_t)o_floor_to_int64(yx); st->af_yy = (uint64_t)o_floor_to_int64(yy);
    st->af_tx = (uint64_t)o_floor_to_int64(tx); st->af_ty = (uint64_t)o_floor_to_int64(ty);
  }
  else {
    st->af_xx = st->af_xy = st->af_yx = st->af_yy = st->af_tx = st->af_ty = 0;
  }
  st->af_rx = rx; st->af_ry = ry;
  st->af_ox = ox; st->af_oy = oy;
  st->af_tw = (int32_t)tw_d; st->af_th = (int32_t)th_d;
  return 1;
}

typedef struct { double offset; uint64_t rgba; } OGStop;

static int o_init_gradient(OStyle* st, uint32_t type, uint32_t extend, const double* v, const OMat* transform) {
  OMat inv;
  uint32_t lut_size = st->lut_size;
  if (type == 0) {   /* linear (pipedefs.cpp:386-434) */
    if (!o_mat_invert(&inv, transform)) return 0;
    uint32_t maxi = extend == 2 ? lut_size * 2u - 1u : lut_size - 1u;
    uint32_t rori = extend == 2 ? maxi : 0u;
    double ax = v[2] - v[0], ay = v[3] - v[1];
    double dist = ax * ax + ay * ay;
    OPt m = o_mat_map(transform, v[0], v[1]);
    double ox = 0.5 - m.x, oy = 0.5 - m.y;
    double dt = ax * inv.m00 + ay * inv.m01;
    double dy = ax * inv.m10 + ay * inv.m11;
    double scale = (double)(int64_t)((uint64_t)lut_size << 32) / dist;
    double offset = ox * dt + oy * dy;
    dt *= scale; dy *= scale; offset *= scale;
    st->lin_dy = (uint64_t)o_floor_to_int64(dy);
    st->lin_dt = (uint64_t)o_floor_to_int64(dt);
    st->lin_pt0 = (uint64_t)o_floor_to_int64(offset);
    st->maxi = maxi; st->rori = rori;
    st->fetch_type = extend != 0 ? O_FT_LINEAR_ROR : O_FT_LINEAR_PAD;
    return 1;
  }
  if (type == 1) {   /* radial (pipedefs.cpp:480-576) */
    if (!o_mat_invert(&inv, transform)) return 0;
    uint32_t maxi = extend == 2 ? lut_size * 2u - 1u : lut_size - 1u;
    uint32_t rori = extend == 2 ? maxi : 0u;
    st->maxi = maxi; st->rori = rori;
    OPt cp = { v[0], v[1] }, fp = { v[2], v[3] };
    double cr = v[4], fr = v[5];
    OPt dp = { cp.x - fp.x, cp.y - fp.y };
    double dr = cr - fr;
    double sq_dx_plus_dy = dp.x * dp.x + dp.y * dp.y;
    double dx_plus_dy = sqrt(sq_dx_plus_dy);
    double dist_from_border = fabs(dx_plus_dy - dr);
    const double dist_limit = 0.5;
    if (dist_from_border < dist_limit) {
      OPt dp0 = { (dp.x * (dr - dist_limit)) / dx_plus_dy, (dp.y * (dr - dist_limit)) / dx_plus_dy };
      OPt dp1 = { (dp.x * (dr + dist_limit)) / dx_plus_dy, (dp.y * (dr + dist_limit)) / dx_plus_dy };
      double d0 = fabs(dp0.x * dp0.x + dp0.y * dp0.y - sq_dx_plus_dy);
      double d1 = fabs(dp1.x * dp1.x + dp1.y * dp1.y - sq_dx_plus_dy);
      dp = (d0 < d1) ? dp0 : dp1;
      fp.x = cp.x - dp.x; fp.y = cp.y - dp.y;
      sq_dx_plus_dy = dp.x * dp.x + dp.y * dp.y;
    }
    double a = dr * dr - sq_dx_plus_dy;
    double sq_fr = fr * fr;
    double scale = (double)lut_size;
    double xx = inv.m00, xy = inv.m01, yx = inv.m10, yy = inv.m11;
    OPt tp = { inv.m20 + (xx + xy) * 0.5 - fp.x, inv.m21 + (yx + yy) * 0.5 - fp.y };
    st->rad_tx = tp.x; st->rad_ty = tp.y; st->rad_yx = yx; st->rad_yy = yy;
    double a_mul_4 = a * 4.0;
    double inv2a = (scale * 0.5) / a;
    double sq_inv2a = inv2a * inv2a;
    st->rad_amul4 = a_mul_4; st->rad_inv2a = inv2a; st->rad_sq_inv2a = sq_inv2a; st->rad_sq_fr = sq_fr;
    double sq_xx_plus_sq_yx = xx * xx + xy * xy;
    double b0 = 2.0 * (dr * fr + tp.x * dp.x + tp.y * dp.y);
    double bx = 2.0 * (dp.x * xx + dp.y * xy);
    double by = 2.0 * (dp.x * yx + dp.y * yy);
    st->rad_b0 = -b0; st->rad_by = -by;
    double bx_mul_2 = bx * 2.0;
    double sq_bx = bx * bx;
    double dd0 = sq_bx + bx_mul_2 * b0 + a_mul_4 * (sq_xx_plus_sq_yx + 2.0 * (tp.x * xx + tp.y * xy));
    double ddy = bx_mul_2 * by + a_mul_4 * (2.0 * (xx * yx + yy * xy));
    double ddd_half = (sq_bx + a_mul_4 * sq_xx_plus_sq_yx);
    double ddd_half_inv = ddd_half * sq_inv2a;
    st->rad_dd0 = dd0 - ddd_half;
    st->rad_ddy = ddy;
    st->rad_bd = (float)(-bx * inv2a);
    st->rad_ddd = (float)ddd_half_inv;
    st->fetch_type = extend != 0 ? O_FT_RADIAL_ROR : O_FT_RADIAL_PAD;
    return 1;
  }
  /* conic (pipedefs.cpp:614-671) */
  {
    static const double q256[4] = { 4.071421038552e+1, -1.311160794048e+1, 6.017670215625, -1.623253505085 };
    const double kPI_MUL_2 = 6.28318530717958647692;
    double angle = v[2], repeat = v[3];
    OPt c = o_mat_map(transform, v[0], v[1]);
    c.x = 0.5 - c.x; c.y = 0.5 - c.y;
    OPt vv = { 1.0 * transform->m00 + 0.0 * transform->m10, 1.0 * transform->m01 + 0.0 * transform->m11 };
    double matrix_angle = atan2(vv.y, vv.x);
    /* updated_transform = transform.rotate(-matrix_angle, c) (matrix.cpp:292-324) */
    OMat u = *transform;
    {
      double ang = -matrix_angle;
      double as = sin(ang), ac = cos(ang);
      double t00 = as * u.m10 + ac * u.m00;
      double t01 = as * u.m11 + ac * u.m01;
      double t10 = ac * u.m10 - as * u.m00;
      double t11 = ac * u.m11 - as * u.m01;
      double px = c.x, py = c.y;
      double ttx = px - ac * px + as * py;
      double tty = py - as * px - ac * py;
      double t20 = ttx * u.m00 + tty * u.m10 + u.m20;
      double t21 = ttx * u.m01 + tty * u.m11 + u.m21;
      u.m20 = t20; u.m21 = t21;
      u.m00 = t00; u.m01 = t01; u.m10 = t10; u.m11 = t11;
    }
    angle += matrix_angle;
    double fr = angle / -kPI_MUL_2;
    double off = fr - floor(fr);
    if (off != 0.0) off = -1.0 + off;
    if (!o_mat_invert(&inv, &u)) return 0;
    st->con_tx = c.x * inv.m00 + c.y * inv.m10;
    st->con_ty = c.x * inv.m01 + c.y * inv.m11;
    st->con_yx = inv.m10;
    st->con_yy = inv.m11;
    double lutSizeD = (double)(int)lut_size;
    double repeated = lutSizeD * repeat;
    double qScale = repeated / 256.0;
    for (int k = 0; k < 4; k++) st->con_q[k] = (float)(q256[k] * qScale);
    st->con_n1 = (float)repeated;
    st->con_n2 = (float)(repeated * 0.5);
    st->con_n4 = (float)(repeated * 0.25);
    st->con_offset = (float)(off * repeated - 0.5);
    st->con_xx = (float)inv.m00;
    st->con_maxi = INT32_MAX;
    st->con_rori = (int32_t)(lut_size - 1u);
    st->fetch_type = O_FT_CONIC;
    return 1;
  }
}

/* Gradient stop analysis & normalization (gradient.cpp:58-173). Returns the kept count or -1. */
static int o_normalize_stops(OGStop* dst, const BLGpuStreamGradientStop* src, int n) {
  uint32_t result = 0, was_same = 0;
  double prev = -1.0;
  for (int i = 0; i < n; i++) {
    double offset = src[i].offset;
    if (!((offset >= 0.0) & (offset <= 1.0))) return -1;
    uint32_t is_same = (offset == prev);
    result |= (offset < prev);
    result |= is_same & was_same;
    was_same = is_same;
    prev = offset;
  }
  if (result == 0 || n == 0) {
    for (int i = 0; i < n; i++) { dst[i].offset = src[i].offset; dst[i].rgba = src[i].rgba64; }
    return n;
  }
  /* stable sort by offset, then drop the middle of 3+ equal offsets */
  int* idx = (int*)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) idx[i] = i;
  for (int i = 1; i < n; i++) {
    int v = idx[i], j = i;
    while (j > 0 && (src[idx[j - 1]].offset > src[v].offset)) { idx[j] = idx[j - 1]; j--; }
    idx[j] = v;
  }
  int j = 0;
  double prev1 = -1.0, prev2 = -1.0;
  for (int i = 0; i < n - 1; i++) {
    double offset = src[idx[i]].offset;
    uint64_t rgba = src[idx[i]].rgba64;
    j -= (int)((prev1 == prev2) & (prev2 == offset));
    dst[j].offset = offset;
    dst[j].rgba = rgba;
    j++;
    prev1 = prev2;
    prev2 = offset;
  }
  free(idx);
  return j;
}

/* ============================================================================================
 * Context
 * ============================================================================================ */

typedef struct {
  int comp_op, fill_rule;
  double global_alpha, fill_alpha;
  uint32_t global_alpha_i, fill_alpha_i;
  uint32_t gradient_quality, pattern_quality;
  OMat user, final_t, final_fixed;
  int final_type, final_fixed_type;
  int integral_translation, tx_i, ty_i;
  OStyle style;                       /* BL_CONTEXT_STYLE_SLOT_FILL */
  OStyle stroke_style;                /* BL_CONTEXT_STYLE_SLOT_STROKE */
  double stroke_alpha;
  uint32_t stroke_alpha_i;
  OStrokeOpts stroke;
} OState;

typedef struct {
  int w, h;
  uint32_t* pixels;
  uint32_t lut_variant;
  OState s;
  OState* stack; int nstack, cap_stack;
  OEdgeStorage storage;
  OEdgeBuilder eb;
  OFillCtx fc;
  const uint32_t** images; const int* iw; const int* ih;
  const int* ifmt;                    /* O_FMT_PRGB32 / O_FMT_XRGB32 of each image */
  int dst_format;                     /* BLGPU_STREAM_FORMAT_* of the target */
  B2DOracleStats* stats;
} OCtx;

static void on_transform_changed(OCtx* c) {   /* rastercontext.cpp:741-800 */
  OState* s = &c->s;
  OMat id = { 1, 0, 0, 1, 0, 0 };
  o_mat_multiply(&s->final_t, &s->user, &id);
  s->final_fixed = s->final_t;
  s->final_fixed.m00 *= 256.0; s->final_fixed.m01 *= 256.0;
  s->final_fixed.m10 *= 256.0; s->final_fixed.m11 *= 256.0;
  s->final_fixed.m20 *= 256.0; s->final_fixed.m21 *= 256.0;
  s->final_type = o_mat_type(&s->final_t);
  s->final_fixed_type = s->final_type > O_TT_SCALE ? s->final_type : O_TT_SCALE;
  s->integral_translation = 0;
  if (s->final_type <= O_TT_TRANSLATE) {
    double mn = floor((double)(INT32_MIN + 1) * 256.0);
    double mx = floor((double)(INT32_MAX - 1 - (c->w > c->h ? c->w : c->h)) * 256.0);
    const OMat* ft = &s->final_fixed;
    if (ft->m20 >= mn && ft->m20 <= mx && ft->m21 >= mn && ft->m21 <= mx) {
      int64_t tx64 = o_floor_to_int64(ft->m20), ty64 = o_floor_to_int64(ft->m21);
      if (((tx64 | ty64) & 0xFF) == 0) {
        s->tx_i = (int)(tx64 >> 8);
        s->ty_i = (int)(ty64 >> 8);
        s->integral_translation = 1;
      }
    }
  }
}

static inline OStyle* slot_style(OCtx* c, int slot) { return slot ? &c->s.stroke_style : &c->s.style; }

static void set_style_solid(OCtx* c, int slot, uint32_t rgba32) {
  OStyle* st = slot_style(c, slot);
  st->nop = 0;
  st->fetch_type = O_FT_SOLID;
  st->solid = o_premultiply(rgba32);
  st->format = rgba32 == 0 ? O_FMT_ZERO32 : (rgba32 >= 0xFF000000u ? O_FMT_FRGB32 : O_FMT_PRGB32);
}

static void set_style_gradient(OCtx* c, int slot, const uint8_t* p) {
  BLGpuStreamGradient g;
  memcpy(&g, p, sizeof(g));
  OStyle* st = slot_style(c, slot);
  memset(st, 0, sizeof(*st));
  BLGpuStreamGradientStop* raw = (BLGpuStreamGradientStop*)malloc(sizeof(BLGpuStreamGradientStop) * (g.stop_count + 1));
  memcpy(raw, p + sizeof(g), sizeof(BLGpuStreamGradientStop) * g.stop_count);
  OGStop* stops = (OGStop*)malloc(sizeof(OGStop) * (g.stop_count + 1));
  int n = o_normalize_stops(stops, raw, (int)g.stop_count);
  if (n < 0) n = 0;   /* assign_stops failed: the gradient keeps no stops */

  /* transform = gradient.transform x final_transform when the gradient has one */
  OMat tf = c->s.final_t;
  if (g.has_transform) {
    OMat gm = { g.transform[0], g.transform[1], g.transform[2], g.transform[3], g.transform[4], g.transform[5] };
    if (o_mat_type(&gm) != O_TT_IDENTITY) o_mat_multiply(&tf, &gm, &c->s.final_t);
  }

  if (n == 0) { st->nop = 1; goto done; }

  /* ensure_info (gradient.cpp:202-287) */
  {
    uint32_t flags = 0;
    uint64_t prev = stops[0].rgba & 0xFF00FF00FF00FF00ull;
    if (prev < 0xFF00000000000000ull) flags |= 1;
    if (prev > 0x00FFFFFFFFFFFFFFull) flags |= 2;
    for (int i = 1; i < n; i++) {
      uint64_t v = stops[i].rgba & 0xFF00FF00FF00FF00ull;
      if (v == prev) continue;
      flags |= 4;
      if (v < 0xFF00000000000000ull) flags |= 1;
      if (v > 0x00FFFFFFFFFFFFFFull) flags |= 2;
      prev = v;
    }
    if (!(flags & 2)) flags &= ~4u;
    uint32_t lut_size;
    if (!(flags & 4)) lut_size = 256;
    else if (n == 1) lut_size = 256;
    else if (n == 2) lut_size = (stops[1].offset - stops[0].offset >= 0.998) ? 256 : 512;
    else if (n == 3) lut_size = (stops[0].offset <= 0.002 && stops[1].offset == 0.5 && stops[2].offset >= 0.998) ? 512 : 1024;
    else lut_size = 1024;
    st->format = (flags & 1) ? O_FMT_PRGB32 : O_FMT_FRGB32;
    if (!(flags & 4)) {
      uint64_t v = stops[n - 1].rgba;
      uint32_t c32 = (uint32_t)(((v >> 56) & 0xFF) << 24 | ((v >> 40) & 0xFF) << 16 | ((v >> 24) & 0xFF) << 8 | ((v >> 8) & 0xFF));
      st->fetch_type = O_FT_SOLID;
      st->solid = o_premultiply(c32);
      goto done;
    }
    /* gradients are not dithered into A8 targets (rastercontext.cpp:456-458) */
    if (c->s.gradient_quality >= 2u && c->dst_format != BLGPU_STREAM_FORMAT_A8) {
      /* BL_GRADIENT_QUALITY_DITHER: lut_size(true) (gradient_p.h:113-120), ensure_lut64 */
      lut_size = lut_size * 2u < 1024u ? lut_size * 2u : 1024u;
      st->dither = 1;
      b2d_oracle_build_lut64(st->lut64, lut_size, stops, (size_t)n);
    }
    else {
      b2d_oracle_build_lut(st->lut, lut_size, stops, (size_t)n, c->lut_variant);
    }
    st->lut_size = lut_size;
    if (!o_init_gradient(st, g.type, g.extend_mode, g.values, &tf)) st->nop = 1;
  }
done:
  free(raw);
  free(stops);
}

static void set_style_pattern(OCtx* c, int slot, const uint8_t* p) {
  BLGpuStreamPattern pt;
  memcpy(&pt, p, sizeof(pt));
  OStyle* st = slot_style(c, slot);
  memset(st, 0, sizeof(*st));
  int iw = c->iw[pt.image_index], ih = c->ih[pt.image_index];
  int ax = 0, ay = 0, aw = iw, ah = ih;
  if (pt.area[2] > 0) { ax = pt.area[0]; ay = pt.area[1]; aw = pt.area[2]; ah = pt.area[3]; }
  st->format = c->ifmt[pt.image_index];   /* fetch_data->extra.format = the image's (rastercontext.cpp:415) */
  if (!aw || !ah) { st->nop = 1; return; }
  st->src = c->images[pt.image_index] + (intptr_t)ay * iw + ax;
  st->src_w = aw; st->src_h = ah; st->src_stride = iw;

  OMat tf = c->s.final_t;
  if (pt.has_transform) {
    OMat pm = { pt.transform[0], pt.transform[1], pt.transform[2], pt.transform[3], pt.transform[4], pt.transform[5] };
    if (o_mat_type(&pm) != O_TT_IDENTITY) o_mat_multiply(&tf, &pm, &c->s.final_t);
  }
  if (!o_init_pattern_affine(st, pt.extend_mode, c->s.pattern_quality, &tf)) st->nop = 1;
}

static int is_pattern_fetch(int fetch_type) { return fetch_type >= O_FT_PAT_ALIGNED_PAD; }

/* SrcOver / SrcCopy simplified by the destination and source formats (CompOpSimplifyInfoImpl::
 * src_over / src_copy, compopsimplifyimpl_p.h:86-162). Returns -1 for DstCopy (nothing drawn),
 * else the operator (0 SrcOver, 1 SrcCopy); *src_or is 0xFF000000 when the simplified source
 * format is XRGB32 and the fetcher reads an image (solid and gradient fetchers do not look at the
 * source format: fixedpiperuntime.cpp:250-270).
 *   SrcOver: ZERO32 -> DstCopy; FRGB32 -> SrcCopy; XRGB32 -> SrcCopy of XRGB32; PRGB32 -> SrcOver.
 *   SrcCopy: XRGB32 -> SrcCopy of XRGB32; PRGB32 into an XRGB32 target -> SrcCopy of XRGB32.
 * An A8 target's simplifications (opaque alpha, transparent) give the alpha byte these do. */
static int o_simplify(int dst_format, int op, int src_format, int fetch_type, uint32_t* src_or) {
  int xrgb_src = src_format == O_FMT_XRGB32;
  if (op == 0) {
    if (src_format == O_FMT_ZERO32) return -1;
    if (src_format == O_FMT_FRGB32 || xrgb_src) op = 1;
  }
  else if (src_format == O_FMT_PRGB32 && dst_format == BLGPU_STREAM_FORMAT_XRGB32) {
    xrgb_src = 1;
  }
  *src_or = (xrgb_src && is_pattern_fetch(fetch_type)) ? 0xFF000000u : 0u;
  return op;
}

/* Resolve the fill: returns 0 for NOP, else sets comp-op (0/1), alpha and the fill context's
 * src_or (consumed by the fill that follows). */
static int resolve_slot(OCtx* c, int slot, int* comp_op, uint32_t* alpha) {
  OState* s = &c->s;
  const OStyle* st = slot_style(c, slot);
  uint32_t a = slot ? s->stroke_alpha_i : s->fill_alpha_i;
  if (s->global_alpha_i == 0 || a == 0 || st->nop) return 0;
  int op = o_simplify(c->dst_format, s->comp_op, st->format, st->fetch_type, &c->fc.src_or);
  if (op < 0) return 0;
  *comp_op = op;
  *alpha = a;
  return 1;
}
static int resolve_fill(OCtx* c, int* comp_op, uint32_t* alpha) { return resolve_slot(c, 0, comp_op, alpha); }

static void fill_box_a(OCtx* c, int x0, int y0, int x1, int y1) {
  if (c->stats) c->stats->fill_calls++;
  o_fill_box_a(&c->fc, x0, y0, x1, y1);
}

static void fill_clipped_box_f(OCtx* c, int x0, int y0, int x1, int y1) {
  if (((x0 | y0 | x1 | y1) & 0xFF) == 0) { fill_box_a(c, x0 >> 8, y0 >> 8, x1 >> 8, y1 >> 8); return; }
  if (c->stats) c->stats->fill_calls++;
  o_fill_box_u(&c->fc, x0, y0, x1, y1);
}

static void fill_edges(OCtx* c, uint32_t fill_rule) {
  if (c->storage.nedges == 0 || c->storage.bbox_y0 >= c->storage.bbox_y1) return;
  if (c->stats) { c->stats->fill_calls++; c->stats->edge_points += c->storage.npts; }
  o_fill_analytic(&c->fc, &c->storage, fill_rule);
}

static void fill_polygon(OCtx* c, const double* xy, size_t n, uint32_t rule, const OMat* m, int ttype) {
  o_storage_clear(&c->storage);
  o_eb_begin(&c->eb);
  if (o_eb_add_poly(&c->eb, xy, n, m, ttype) == 0) {
    o_eb_done(&c->eb);
    fill_edges(c, rule);
  }
}

static void fill_box_d(OCtx* c, double bx0, double by0, double bx1, double by1) {
  OState* s = &c->s;
  const OMat* t = &s->final_fixed;
  if (s->final_fixed_type <= O_TT_SWAP) {
    double x0 = bx0 * t->m00 + by0 * t->m10 + t->m20;
    double y0 = bx0 * t->m01 + by0 * t->m11 + t->m21;
    double x1 = bx1 * t->m00 + by1 * t->m10 + t->m20;
    double y1 = bx1 * t->m01 + by1 * t->m11 + t->m21;
    double mx0 = o_min(x0, x1), my0 = o_min(y0, y1), mx1 = o_max(x0, x1), my1 = o_max(y0, y1);
    /* Geometry::intersect with the fixed clip box */
    double cx1 = (double)c->w * 256.0, cy1 = (double)c->h * 256.0;
    double ix0 = o_max(mx0, 0.0), iy0 = o_max(my0, 0.0), ix1 = o_min(mx1, cx1), iy1 = o_min(my1, cy1);
    if (!((ix0 < ix1) & (iy0 < iy1))) return;
    int ux0 = o_trunc_to_int(ix0), uy0 = o_trunc_to_int(iy0), ux1 = o_trunc_to_int(ix1), uy1 = o_trunc_to_int(iy1);
    if (ux0 >= ux1 || uy0 >= uy1) return;
    fill_clipped_box_f(c, ux0, uy0, ux1, uy1);
  }
  else {
    double poly[8] = { bx0, by0, bx1, by0, bx1, by1, bx0, by1 };
    fill_polygon(c, poly, 4, 1 /* EVEN_ODD */, t, s->final_fixed_type);
  }
}

/* --- stroking -------------------------------------------------------------------------------
 * stroke_unclipped_geometry / stroke_unclipped_path<kSync> (rastercontext.cpp:3180-3234) with
 * add_stroked_path_edges (rastercontextops_p.h:95-140) and stroke_geometry_sink
 * (rastercontextops.cpp:61-74): the outline of every figure goes into one edge builder - A and C
 * as open paths, B reversed (closed when it ends with CLOSE) - and the edges are filled non-zero
 * with the stroke style. A stroke that fails (invalid geometry) fills nothing. */

typedef struct { OCtx* c; OMat m; int ttype; OPath rev; int failed; } OStrokeEdges;

/* EdgeSourceReversePathFromStrokeSink (edgebuilder_p.h:287-405) as a forward path: the last
 * on-point first, then every segment backwards. Returns the closed flag (must_close). */
static int reverse_stroke_path(const OPath* b, OPath* out) {
  out->n = 0;
  size_t n = b->n;
  int must_close = n > 0 && b->cmd[n - 1] == 5;
  n -= (size_t)must_close;
  if (n == 0 || b->cmd[n - 1] != 1) return must_close;          /* begin(): needs an on-point */
  size_t i = n - 1;
  o_path_reserve(out, n);
  out->cmd[out->n] = 0; out->vtx[out->n++] = b->vtx[i];
  while (i > 0) {
    uint8_t k = b->cmd[i - 1];
    if (k <= 1) { out->cmd[out->n] = 1; out->vtx[out->n++] = b->vtx[i - 1]; i -= 1; }
    else if (k == 2 && i >= 2) {
      out->cmd[out->n] = 2; out->vtx[out->n++] = b->vtx[i - 1];
      out->cmd[out->n] = 1; out->vtx[out->n++] = b->vtx[i - 2];
      i -= 2;
    }
    else if (k == 4 && i >= 3) {
      out->cmd[out->n] = 4; out->vtx[out->n++] = b->vtx[i - 1];
      out->cmd[out->n] = 4; out->vtx[out->n++] = b->vtx[i - 2];
      out->cmd[out->n] = 1; out->vtx[out->n++] = b->vtx[i - 3];
      i -= 3;
    }
    else break;
  }
  return must_close;
}

static int stroke_edges_sink(const OPath* a, const OPath* b, const OPath* cpath, void* user) {
  OStrokeEdges* se = (OStrokeEdges*)user;
  OEdgeBuilder* eb = &se->c->eb;
  if (o_eb_add_path_ex(eb, a->cmd, (const double*)a->vtx, a->n, &se->m, se->ttype, 0)) return 2;
  int closed = reverse_stroke_path(b, &se->rev);
  if (o_eb_add_path_ex(eb, se->rev.cmd, (const double*)se->rev.vtx, se->rev.n, &se->m, se->ttype, closed)) return 2;
  if (cpath->n && o_eb_add_path_ex(eb, cpath->cmd, (const double*)cpath->vtx, cpath->n, &se->m, se->ttype, 0)) return 2;
  return 0;
}

static void stroke_op(OCtx* c, uint32_t op, const uint8_t* p) {
  OState* s = &c->s;
  int cop; uint32_t alpha;
  /* the input path (BLPath::add_geometry, path.cpp:1335-1660; direction CW) */
  OPath in;
  memset(&in, 0, sizeof(in));
  uint32_t n = 0;
  if (op == BLGPU_OP_STROKE_PATH_D || op == BLGPU_OP_STROKE_POLYLINE_D || op == BLGPU_OP_STROKE_POLYGON_D) {
    memcpy(&n, p, 4);
    if (c->stats) c->stats->input_vertices += n;
  }
  if (!resolve_slot(c, 1, &cop, &alpha)) return;
  switch (op) {
    case BLGPU_OP_STROKE_PATH_D: {
      if (n == 0) return;
      o_path_reserve(&in, n);
      memcpy(in.cmd, p + 8, n);
      memcpy(in.vtx, p + 8 + ((n + 7u) & ~7u), sizeof(double) * 2 * n);
      in.n = n;
      break;
    }
    case BLGPU_OP_STROKE_POLYLINE_D: case BLGPU_OP_STROKE_POLYGON_D: {
      if (n == 0) return;
      o_path_reserve(&in, n + 1);
      memcpy(in.vtx, p + 8, sizeof(double) * 2 * n);
      for (uint32_t i = 0; i < n; i++) in.cmd[i] = i ? 1 : 0;
      in.n = n;
      if (op == BLGPU_OP_STROKE_POLYGON_D) { in.cmd[n] = 5; in.vtx[n].x = NAN; in.vtx[n].y = NAN; in.n = n + 1; }
      break;
    }
    case BLGPU_OP_STROKE_LINE_D: {
      double v[4]; memcpy(v, p, sizeof(v));
      o_path_reserve(&in, 2);
      in.cmd[0] = 0; in.vtx[0].x = v[0]; in.vtx[0].y = v[1];
      in.cmd[1] = 1; in.vtx[1].x = v[2]; in.vtx[1].y = v[3];
      in.n = 2;
      break;
    }
    default: {   /* BOX_D, RECT_D: PathAppender::add_box (path_p.h:420-442) */
      double v[4]; memcpy(v, p, sizeof(v));
      double x0 = v[0], y0 = v[1], x1 = v[2], y1 = v[3];
      if (op == BLGPU_OP_STROKE_RECT_D) { x1 = v[2] + v[0]; y1 = v[3] + v[1]; }
      o_path_reserve(&in, 5);
      static const uint8_t box_cmd[5] = { 0, 1, 1, 1, 5 };
      memcpy(in.cmd, box_cmd, 5);
      in.vtx[0].x = x0; in.vtx[0].y = y0; in.vtx[1].x = x1; in.vtx[1].y = y0;
      in.vtx[2].x = x1; in.vtx[2].y = y1; in.vtx[3].x = x0; in.vtx[3].y = y1;
      in.vtx[4].x = NAN; in.vtx[4].y = NAN;
      in.n = 5;
      break;
    }
  }
  OStrokeEdges se;
  memset(&se, 0, sizeof(se));
  se.c = c;
  se.m = s->final_fixed;             /* final_transform_fixed(origin_fixed), origin (0, 0) */
  se.ttype = s->final_fixed_type;
  if (s->stroke.transform_order != 0) {
    /* BEFORE: the path is transformed by the user transform without its translation
     * (DirectStateAccessor::user_transform, rastercontext.cpp:168-171) first; the edges then use
     * the meta transform (identity here, scaled to 24.8) with the final transform's origin. */
    OMat lin = s->user;
    lin.m20 = 0.0; lin.m21 = 0.0;
    for (size_t i = 0; i < in.n; i++) in.vtx[i] = o_mat_map(&lin, in.vtx[i].x, in.vtx[i].y);
    OMat meta = { 256.0, 0.0, 0.0, 256.0, s->final_fixed.m20, s->final_fixed.m21 };
    se.m = meta;
    se.ttype = O_TT_SCALE;
  }
  OPath a, b, cp;
  memset(&a, 0, sizeof(a)); memset(&b, 0, sizeof(b)); memset(&cp, 0, sizeof(cp));
  o_storage_clear(&c->storage);
  o_eb_begin(&c->eb);
  int rc = o_stroke_path(in.cmd, (const double*)in.vtx, in.n, &s->stroke, 0.05, 0.414213562,
                         &a, &b, &cp, stroke_edges_sink, &se);
  if (rc == 0) {
    o_eb_done(&c->eb);
    c->fc.style = &s->stroke_style; c->fc.comp_op = cop; c->fc.alpha = alpha;
    fill_edges(c, 0 /* NON_ZERO */);
  }
  o_path_free(&a); o_path_free(&b); o_path_free(&cp); o_path_free(&se.rev); o_path_free(&in);
}

/* --- image blits (rastercontext.cpp:3941-4160) ----------------------------------------------
 * The image area composited with the comp-op and the global alpha through the blit fetchers. The
 * aligned blit (FetchPatternAlignedBlit, fetchgeneric_p.h:471-534: pixel (x, y) reads the area's
 * (x - x0, y - y0)) is the aligned pad fetcher translated by -x0, -y0: inside the blit box the two
 * read the same pixels. */

/* check_image_area (rastercontext.cpp:2305-2319) */
static int o_image_area(int iw, int ih, const BLGpuStreamBlit* b, int out[4]) {
  out[0] = 0; out[1] = 0; out[2] = iw; out[3] = ih;
  if (b->has_area) {
    unsigned max_w = (unsigned)iw - (unsigned)b->area[0];
    unsigned max_h = (unsigned)ih - (unsigned)b->area[1];
    if ((max_w > (unsigned)iw) | ((unsigned)b->area[2] > max_w) | (max_h > (unsigned)ih) | ((unsigned)b->area[3] > max_h))
      return 0;
    memcpy(out, b->area, sizeof(int) * 4);
  }
  return 1;
}

static int o_blit_source(OCtx* c, OStyle* st, uint32_t image_index, const int a[4]) {
  memset(st, 0, sizeof(*st));
  st->format = c->ifmt[image_index];
  if (a[2] <= 0 || a[3] <= 0) { st->nop = 1; return 0; }
  int iw = c->iw[image_index];
  st->src = c->images[image_index] + (intptr_t)a[1] * iw + a[0];
  st->src_w = a[2]; st->src_h = a[3]; st->src_stride = iw;
  return 1;
}

static void blit_op(OCtx* c, uint32_t op, const uint8_t* p) {
  OState* s = &c->s;
  BLGpuStreamBlit b;
  memcpy(&b, p, sizeof(b));
  int iw = c->iw[b.image_index], ih = c->ih[b.image_index];
  int src[4];
  if (op == BLGPU_OP_BLIT_SCALED_IMAGE_I || op == BLGPU_OP_BLIT_SCALED_IMAGE_D) {
    if (!o_image_area(iw, ih, &b, src)) return;
    if ((b.rect[2] == (double)src[2]) & (b.rect[3] == (double)src[3]))
      op = op == BLGPU_OP_BLIT_SCALED_IMAGE_I ? BLGPU_OP_BLIT_IMAGE_I : BLGPU_OP_BLIT_IMAGE_D;
  }
  if (op == BLGPU_OP_BLIT_IMAGE_I && !s->integral_translation) op = BLGPU_OP_BLIT_IMAGE_D;
  if (!o_image_area(iw, ih, &b, src)) return;
  OStyle* st = (OStyle*)malloc(sizeof(OStyle));
  /* resolve_blit_op (rastercontext.cpp:1331-1342): the comp-op simplified for the image format */
  int bop = o_simplify(c->dst_format, s->comp_op, c->ifmt[b.image_index], O_FT_PAT_ALIGNED_PAD, &c->fc.src_or);
  if (bop < 0) { free(st); return; }
  c->fc.style = st; c->fc.comp_op = bop; c->fc.alpha = s->global_alpha_i;
  if (op == BLGPU_OP_BLIT_IMAGE_I) {
    /* translate_and_clip_rect_to_blit_i (rastercontext.cpp:922-990) */
    int64_t dx = (int64_t)(int32_t)b.rect[0] + s->tx_i, dy = (int64_t)(int32_t)b.rect[1] + s->ty_i;
    int64_t x0 = dx, y0 = dy, x1 = x0 + src[2], y1 = y0 + src[3];
    x0 = x0 < 0 ? 0 : x0; y0 = y0 < 0 ? 0 : y0;
    x1 = x1 > c->w ? c->w : x1; y1 = y1 > c->h ? c->h : y1;
    if ((x0 < x1) & (y0 < y1) & (s->global_alpha_i != 0)) {
      src[0] += (int)(x0 - dx); src[1] += (int)(y0 - dy);
      src[2] = (int)(x1 - x0); src[3] = (int)(y1 - y0);
      if (o_blit_source(c, st, b.image_index, src)) {
        o_init_pattern_simple(st, 0, -(int)x0, -(int)y0, 0, 0);
        fill_box_a(c, (int)x0, (int)y0, (int)x1, (int)y1);
      }
    }
  }
  else if (op == BLGPU_OP_BLIT_IMAGE_D && s->final_type <= O_TT_TRANSLATE) {
    const OMat* t = &s->final_fixed;
    double sx = b.rect[0] * t->m00 + t->m20, sy = b.rect[1] * t->m11 + t->m21;
    double dx0 = o_max(sx, 0.0), dy0 = o_max(sy, 0.0);
    double dx1 = o_min(sx + (double)src[2] * t->m00, (double)c->w * 256.0);
    double dy1 = o_min(sy + (double)src[3] * t->m11, (double)c->h * 256.0);
    if (s->global_alpha_i != 0 && ((dx0 < dx1) & (dy0 < dy1))) {
      int ix0 = o_trunc_to_int(dx0), iy0 = o_trunc_to_int(dy0), ix1 = o_trunc_to_int(dx1), iy1 = o_trunc_to_int(dy1);
      if ((ix0 < ix1) & (iy0 < iy1)) {
        int64_t fx = o_floor_to_int64(sx), fy = o_floor_to_int64(sy);
        int ok;
        if (!((fx | fy) & 0xFF)) {
          int x0 = ix0 >> 8, y0 = iy0 >> 8, x1 = (ix1 + 0xFF) >> 8, y1 = (iy1 + 0xFF) >> 8;
          int tx = (int)(fx >> 8), ty = (int)(fy >> 8);
          src[0] += x0 - tx; src[1] += y0 - ty; src[2] = x1 - x0; src[3] = y1 - y0;
          ok = o_blit_source(c, st, b.image_index, src);
          if (ok) o_init_pattern_simple(st, 0, -x0, -y0, 0, 0);
        }
        else {
          ok = o_blit_source(c, st, b.image_index, src);
          if (ok) o_init_pattern_fx_fy(st, 2 /* REFLECT */, s->pattern_quality, fx, fy);
        }
        if (ok) fill_clipped_box_f(c, ix0, iy0, ix1, iy1);
      }
    }
  }
  else if (s->global_alpha_i != 0) {
    /* affine: BLMatrix2D::translate for a blit, the rectangle's scale x final transform for a
     * scaled blit (TransformInternal::multiply, matrix_p.h:57-64) */
    OMat ft;
    double bx0 = b.rect[0], by0 = b.rect[1], bx1, by1;
    if (op == BLGPU_OP_BLIT_IMAGE_D) {
      ft = s->final_t;
      ft.m20 += b.rect[0] * ft.m00 + b.rect[1] * ft.m10;
      ft.m21 += b.rect[0] * ft.m01 + b.rect[1] * ft.m11;
      bx1 = b.rect[0] + (double)src[2]; by1 = b.rect[1] + (double)src[3];
    }
    else {
      OMat sc = { b.rect[2] / (double)src[2], 0.0, 0.0, b.rect[3] / (double)src[3], b.rect[0], b.rect[1] };
      o_mat_multiply(&ft, &sc, &s->final_t);
      bx1 = b.rect[0] + b.rect[2]; by1 = b.rect[1] + b.rect[3];
    }
    if (o_blit_source(c, st, b.image_index, src) && o_init_pattern_affine(st, 2 /* REFLECT */, s->pattern_quality, &ft))
      fill_box_d(c, bx0, by0, bx1, by1);
  }
  free(st);
}

/* --- masked fills (rastercontext.cpp:3679-3790, fill_unclipped_mask_d :3594-3676) ---------------
 * Only a pixel-aligned mask under a translation renders (the reference returns
 * BL_ERROR_NOT_IMPLEMENTED for the rest). */
static void mask_op(OCtx* c, uint32_t op, const uint8_t* p) {
  OState* s = &c->s;
  BLGpuStreamMask m;
  memcpy(&m, p, sizeof(m));
  const uint8_t* bytes = p + sizeof(m);
  BLGpuStreamBlit area_only;
  memset(&area_only, 0, sizeof(area_only));
  area_only.has_area = m.has_area;
  memcpy(area_only.area, m.area, sizeof(m.area));
  int src[4];
  if (!o_image_area((int)m.width, (int)m.height, &area_only, src)) return;
  int cop; uint32_t alpha;
  int x0, y0, x1, y1;
  if (op == BLGPU_OP_FILL_MASK_I && s->integral_translation) {
    int64_t dx = (int64_t)(int32_t)m.origin[0] + s->tx_i, dy = (int64_t)(int32_t)m.origin[1] + s->ty_i;
    int64_t bx0 = dx, by0 = dy, bx1 = bx0 + src[2], by1 = by0 + src[3];
    bx0 = bx0 < 0 ? 0 : bx0; by0 = by0 < 0 ? 0 : by0;
    bx1 = bx1 > c->w ? c->w : bx1; by1 = by1 > c->h ? c->h : by1;
    if ((bx0 >= bx1) | (by0 >= by1)) return;
    if (!resolve_fill(c, &cop, &alpha)) return;
    src[0] += (int)(bx0 - dx); src[1] += (int)(by0 - dy);
    x0 = (int)bx0; y0 = (int)by0; x1 = (int)bx1; y1 = (int)by1;
  }
  else {
    if (!resolve_fill(c, &cop, &alpha)) return;
    if (s->final_type > O_TT_TRANSLATE) return;
    const OMat* t = &s->final_fixed;
    double sx = m.origin[0] * t->m00 + t->m20, sy = m.origin[1] * t->m11 + t->m21;
    double bx0 = o_max(sx, 0.0), by0 = o_max(sy, 0.0);
    double bx1 = o_min(sx + (double)src[2] * t->m00, (double)c->w * 256.0);
    double by1 = o_min(sy + (double)src[3] * t->m11, (double)c->h * 256.0);
    if (!((bx0 < bx1) & (by0 < by1))) return;
    int64_t fx = o_floor_to_int64(sx), fy = o_floor_to_int64(sy);
    int ux0 = o_trunc_to_int(bx0), uy0 = o_trunc_to_int(by0), ux1 = o_trunc_to_int(bx1), uy1 = o_trunc_to_int(by1);
    if ((fx | fy) & 0xFF) return;
    x0 = ux0 >> 8; y0 = uy0 >> 8; x1 = (ux1 + 0xFF) >> 8; y1 = (uy1 + 0xFF) >> 8;
    src[0] += x0 - (int)(fx >> 8); src[1] += y0 - (int)(fy >> 8);
    if (((ux0 | uy0 | ux1 | uy1) & 0xFF) != 0) return;
  }
  if (c->stats) c->stats->fill_calls++;
  c->fc.style = &s->style; c->fc.comp_op = cop; c->fc.alpha = alpha;
  o_fill_mask_a(&c->fc, x0, y0, x1, y1, bytes + (size_t)src[1] * m.width + (size_t)src[0], (intptr_t)m.width);
}

/* fill_path_d: u32 n, u32 pad, u8 cmd[n] (padded to 8), f64 xy[2n] */
static void fill_path_op(OCtx* c, const uint8_t* p) {
  OState* s = &c->s;
  int cop; uint32_t alpha;
  uint32_t n; memcpy(&n, p, 4);
  if (c->stats) c->stats->input_vertices += n;
  if (!resolve_fill(c, &cop, &alpha)) return;
  if (n == 0) return;
  c->fc.style = &s->style; c->fc.comp_op = cop; c->fc.alpha = alpha;
  const uint8_t* cmd = p + 8;
  double* xy = (double*)malloc(sizeof(double) * 2 * n);
  memcpy(xy, cmd + ((n + 7u) & ~7u), sizeof(double) * 2 * n);
  o_storage_clear(&c->storage);
  o_eb_begin(&c->eb);
  if (o_eb_add_path(&c->eb, cmd, xy, n, &s->final_fixed, s->final_fixed_type) == 0) {
    o_eb_done(&c->eb);
    fill_edges(c, (uint32_t)s->fill_rule);
  }
  free(xy);
}

/* --- shapes: BLPath::add_geometry (path.cpp:1408-1600, direction CW) ----------------------------
 * Returns the vertex count written to cmd/xy (at most 18), 0 for other types. */
static size_t o_shape_path(uint32_t type, const double* v, uint8_t* cmd, double* xy) {
  const double kappa = 0.55228474983;
  size_t n = 0;
#define PUT(c, x, y) do { cmd[n] = (uint8_t)(c); xy[2 * n] = (x); xy[2 * n + 1] = (y); n++; } while (0)
#define CUBIC(a, b, c, d, e, f) do { PUT(4, a, b); PUT(4, c, d); PUT(1, e, f); } while (0)
  if (type == 5 || type == 6) {
    double x0 = v[0], y0 = v[1], rx = v[2];
    double ry = type == 5 ? fabs(rx) : v[3];
    double kx = rx * kappa, ky = ry * kappa;
    PUT(0, x0 + rx, y0);
    CUBIC(x0 + rx, y0 + ky, x0 + kx, y0 + ry, x0, y0 + ry);
    CUBIC(x0 - kx, y0 + ry, x0 - rx, y0 + ky, x0 - rx, y0);
    CUBIC(x0 - rx, y0 - ky, x0 - kx, y0 - ry, x0, y0 - ry);
    CUBIC(x0 + kx, y0 - ry, x0 + rx, y0 - ky, x0 + rx, y0);
    PUT(5, NAN, NAN);
  }
  else if (type == 7) {
    double x0 = v[0], y0 = v[1], x1 = v[0] + v[2], y1 = v[1] + v[3];
    double rx = o_min(fabs(v[4]), v[2] * 0.5), ry = o_min(fabs(v[5]), v[3] * 0.5);
    if (!(rx > 1e-14 && ry > 1e-14)) {
      PUT(0, x0, y0); PUT(1, x1, y0); PUT(1, x1, y1); PUT(1, x0, y1); PUT(5, NAN, NAN);
    }
    else {
      double kx = rx * (1.0 - kappa), ky = ry * (1.0 - kappa);
      PUT(0, x0 + rx, y0);
      PUT(1, x1 - rx, y0);
      CUBIC(x1 - kx, y0, x1, y0 + ky, x1, y0 + ry);
      PUT(1, x1, y1 - ry);
      CUBIC(x1, y1 - ky, x1 - kx, y1, x1 - rx, y1);
      PUT(1, x0 + rx, y1);
      CUBIC(x0 + kx, y1, x0, y1 - ky, x0, y1 - ry);
      PUT(1, x0, y0 + ry);
      CUBIC(x0, y0 + ky, x0 + kx, y0, x0 + rx, y0);
      PUT(5, NAN, NAN);
    }
  }
  else if (type == 12) {
    PUT(0, v[0], v[1]); PUT(1, v[2], v[3]); PUT(1, v[4], v[5]); PUT(5, NAN, NAN);
  }
  else if (type == 8 || type == 9 || type == 10) {
    /* arc_to_cubic_spline (path.cpp:496-570) with PathAppender::conic_to's cubic (path_p.h:319-334) */
    static const double steps[4] = { 1.57079632679489661923, 3.14159265358979323846, 4.71238898038468985769,
                                     6.28318530717958647692 };
    double cx = v[0], cy = v[1], rx = v[2], ry = v[3], sweep = v[5];
    if (type == 10) PUT(0, cx, cy);
    double ss = sin(v[4]), sc = cos(v[4]);
    OMat t = { sc, ss, -ss, sc, 0.0, 0.0 };                  /* make_sin_cos */
    t.m00 *= rx; t.m01 *= ry; t.m10 *= rx; t.m11 *= ry; t.m20 *= rx; t.m21 *= ry;   /* post_scale */
    t.m20 += cx; t.m21 += cy;                               /* post_translate */
    if (sweep < 0) { t.m00 *= 1.0; t.m01 *= 1.0; t.m10 *= -1.0; t.m11 *= -1.0; sweep = -sweep; }
    OPt v1 = { 1.0, 0.0 }, vc = { 1.0, 1.0 }, v2;
    int ok = 1;
    if (sweep >= 6.28318530717958647692 - 1e-14) { sweep = 6.28318530717958647692; v2 = v1; }
    else if (isnan(sweep)) ok = 0;
    else { v2.x = cos(sweep); v2.y = sin(sweep); }
    if (ok) {
      OPt p0 = o_mat_map(&t, v1.x, v1.y);
      PUT(type == 10 ? 1 : 0, p0.x, p0.y);
      int i = 0, full = 0;
      while (sweep > steps[i]) {
        double tmp = v1.x; v1.x = -v1.y; v1.y = tmp;
        OPt p1 = o_mat_map(&t, vc.x, vc.y), p2 = o_mat_map(&t, v1.x, v1.y);
        CUBIC(p0.x + (p1.x - p0.x) * kappa, p0.y + (p1.y - p0.y) * kappa,
              p2.x + (p1.x - p2.x) * kappa, p2.y + (p1.y - p2.y) * kappa, p2.x, p2.y);
        if (++i == 4) { full = 1; break; }
        tmp = vc.x; vc.x = -vc.y; vc.y = tmp;
        p0 = p2;
      }
      if (!full) {
        OPt s2 = { v1.x + v2.x, v1.y + v2.y };
        double dd = s2.x * s2.x + s2.y * s2.y;
        vc.x = 2.0 * s2.x / dd; vc.y = 2.0 * s2.y / dd;
        double w = sqrt(0.5 * (v1.x * v2.x + v1.y * v2.y) + 0.5);
        double k = 4.0 * w / (3.0 * (1.0 + w));
        OPt p1 = o_mat_map(&t, vc.x, vc.y), p2 = o_mat_map(&t, v2.x, v2.y);
        CUBIC(p0.x + (p1.x - p0.x) * k, p0.y + (p1.y - p0.y) * k, p2.x + (p1.x - p2.x) * k, p2.y + (p1.y - p2.y) * k,
              p2.x, p2.y);
      }
    }
    if (type != 8) PUT(5, NAN, NAN);
  }
#undef CUBIC
#undef PUT
  return n;
}

static int replay(OCtx* c, const uint8_t* base, size_t size, size_t off) {
  while (off + 8 <= size) {
    uint32_t op, len;
    memcpy(&op, base + off, 4);
    memcpy(&len, base + off + 4, 4);
    const uint8_t* p = base + off + 8;
    if (off + 8 + len > size) return -1;
    off += 8 + (size_t)len;
    if (op == BLGPU_OP_END) break;
    OState* s = &c->s;
    int cop; uint32_t alpha;

    switch (op) {
      case BLGPU_OP_SET_COMP_OP: { uint32_t v; memcpy(&v, p, 4); s->comp_op = (int)v; break; }
      case BLGPU_OP_SET_FILL_RULE: { uint32_t v; memcpy(&v, p, 4); s->fill_rule = (int)v; break; }
      case BLGPU_OP_SET_GLOBAL_ALPHA: {
        double a; memcpy(&a, p, 8);
        if (isnan(a)) break;
        a = o_clamp(a, 0.0, 1.0);
        double ia = a * 255.0;
        s->global_alpha = a;
        s->global_alpha_i = (uint32_t)o_round_to_int(ia);
        s->fill_alpha_i = (uint32_t)o_round_to_int(ia * s->fill_alpha);
        s->stroke_alpha_i = (uint32_t)o_round_to_int(ia * s->stroke_alpha);
        break;
      }
      case BLGPU_OP_SET_FILL_ALPHA: {
        double a; memcpy(&a, p, 8);
        if (isnan(a)) break;
        a = o_clamp(a, 0.0, 1.0);
        s->fill_alpha = a;
        s->fill_alpha_i = (uint32_t)o_round_to_int(s->global_alpha * 255.0 * a);
        break;
      }
      case BLGPU_OP_SET_HINT: {
        uint32_t h, v; memcpy(&h, p, 4); memcpy(&v, p + 4, 4);
        if (h == BLGPU_HINT_GRADIENT_QUALITY) s->gradient_quality = v;
        else if (h == BLGPU_HINT_PATTERN_QUALITY) s->pattern_quality = v;
        break;
      }
      case BLGPU_OP_SET_TRANSFORM: {
        double m[6]; memcpy(m, p, sizeof(m));
        s->user.m00 = m[0]; s->user.m01 = m[1]; s->user.m10 = m[2]; s->user.m11 = m[3]; s->user.m20 = m[4]; s->user.m21 = m[5];
        on_transform_changed(c);
        break;
      }
      case BLGPU_OP_RESET_TRANSFORM: {
        OMat id = { 1, 0, 0, 1, 0, 0 };
        s->user = id;
        on_transform_changed(c);
        break;
      }
      case BLGPU_OP_STYLE_RGBA32: { uint32_t v; memcpy(&v, p, 4); set_style_solid(c, 0, v); break; }
      case BLGPU_OP_STYLE_GRADIENT: set_style_gradient(c, 0, p); break;
      case BLGPU_OP_STYLE_PATTERN: set_style_pattern(c, 0, p); break;
      case BLGPU_OP_STROKE_STYLE_RGBA32: { uint32_t v; memcpy(&v, p, 4); set_style_solid(c, 1, v); break; }
      case BLGPU_OP_STROKE_STYLE_GRADIENT: set_style_gradient(c, 1, p); break;
      case BLGPU_OP_STROKE_STYLE_PATTERN: set_style_pattern(c, 1, p); break;
      case BLGPU_OP_SET_STROKE_ALPHA: {      /* set_style_alpha (rastercontext.cpp:1920-1939) */
        double a; memcpy(&a, p, 8);
        if (isnan(a)) break;
        a = o_clamp(a, 0.0, 1.0);
        s->stroke_alpha = a;
        s->stroke_alpha_i = (uint32_t)o_round_to_int(s->global_alpha * 255.0 * a);
        break;
      }
      case BLGPU_OP_SET_STROKE_WIDTH: memcpy(&s->stroke.width, p, 8); break;
      case BLGPU_OP_SET_STROKE_MITER_LIMIT: memcpy(&s->stroke.miter_limit, p, 8); break;
      case BLGPU_OP_SET_STROKE_JOIN: { uint32_t v; memcpy(&v, p, 4); if (v <= 4u) s->stroke.join = v; break; }
      case BLGPU_OP_SET_STROKE_CAPS: {
        uint32_t v[2]; memcpy(v, p, 8);
        if (v[0] <= 5u) s->stroke.start_cap = v[0];
        if (v[1] <= 5u) s->stroke.end_cap = v[1];
        break;
      }
      case BLGPU_OP_SET_STROKE_TRANSFORM_ORDER: { uint32_t v; memcpy(&v, p, 4); if (v <= 1u) s->stroke.transform_order = v; break; }
      case BLGPU_OP_STROKE_PATH_D: case BLGPU_OP_STROKE_POLYLINE_D: case BLGPU_OP_STROKE_POLYGON_D:
      case BLGPU_OP_STROKE_BOX_D: case BLGPU_OP_STROKE_RECT_D: case BLGPU_OP_STROKE_LINE_D:
        stroke_op(c, op, p);
        break;
      case BLGPU_OP_BLIT_IMAGE_I: case BLGPU_OP_BLIT_IMAGE_D:
      case BLGPU_OP_BLIT_SCALED_IMAGE_I: case BLGPU_OP_BLIT_SCALED_IMAGE_D:
        blit_op(c, op, p);
        break;
      case BLGPU_OP_FILL_MASK_I: case BLGPU_OP_FILL_MASK_D:
        mask_op(c, op, p);
        break;
      case BLGPU_OP_FILL_GEOMETRY: case BLGPU_OP_STROKE_GEOMETRY: {
        uint32_t type; memcpy(&type, p, 4);
        double v[6]; memcpy(v, p + 8, sizeof(v));
        uint8_t sc[24]; double sxy[48];
        size_t sn = o_shape_path(type, v, sc, sxy);
        if (!sn) break;
        /* the same record layout as FILL_PATH_D / STROKE_PATH_D */
        uint8_t rec[8 + 24 + 48 * 8];
        uint32_t n32 = (uint32_t)sn;
        memset(rec, 0, sizeof(rec));
        memcpy(rec, &n32, 4);
        memcpy(rec + 8, sc, sn);
        memcpy(rec + 8 + ((sn + 7u) & ~7u), sxy, sizeof(double) * 2 * sn);
        if (op == BLGPU_OP_FILL_GEOMETRY) fill_path_op(c, rec);
        else stroke_op(c, BLGPU_OP_STROKE_PATH_D, rec);
        break;
      }

      case BLGPU_OP_CLEAR_ALL: {
        OStyle clear_style;
        memset(&clear_style, 0, sizeof(clear_style));
        clear_style.fetch_type = O_FT_SOLID;
        /* resolve_clear_op (rastercontext.cpp:1230-1242): SrcCopy of the override table's first
         * entry, 0x00000000, whatever the target format */
        c->fc.style = &clear_style;
        c->fc.comp_op = 1;
        c->fc.src_or = 0;
        c->fc.alpha = 255;
        fill_box_a(c, 0, 0, c->w, c->h);
        break;
      }
      case BLGPU_OP_FILL_ALL:
        if (!resolve_fill(c, &cop, &alpha)) break;
        c->fc.style = &s->style; c->fc.comp_op = cop; c->fc.alpha = alpha;
        fill_box_a(c, 0, 0, c->w, c->h);
        break;

      case BLGPU_OP_FILL_RECT_I: {
        int32_t r[4]; memcpy(r, p, sizeof(r));
        if (!resolve_fill(c, &cop, &alpha)) break;
        c->fc.style = &s->style; c->fc.comp_op = cop; c->fc.alpha = alpha;
        if (!s->integral_translation) {
          if ((r[2] <= 0) | (r[3] <= 0)) break;
          fill_box_d(c, (double)r[0], (double)r[1], (double)r[0] + (double)r[2], (double)r[1] + (double)r[3]);
        }
        else {
          int64_t x0 = (int64_t)r[0] + s->tx_i, y0 = (int64_t)r[1] + s->ty_i;
          int64_t x1 = (int64_t)r[2] + x0, y1 = (int64_t)r[3] + y0;
          x0 = x0 < 0 ? 0 : x0; y0 = y0 < 0 ? 0 : y0;
          x1 = x1 > c->w ? c->w : x1; y1 = y1 > c->h ? c->h : y1;
          if ((x0 >= x1) | (y0 >= y1)) break;
          fill_box_a(c, (int)x0, (int)y0, (int)x1, (int)y1);
        }
        break;
      }
      case BLGPU_OP_FILL_RECT_D: {
        double r[4]; memcpy(r, p, sizeof(r));
        if (!resolve_fill(c, &cop, &alpha)) break;
        c->fc.style = &s->style; c->fc.comp_op = cop; c->fc.alpha = alpha;
        fill_box_d(c, r[0], r[1], r[0] + r[2], r[1] + r[3]);
        break;
      }
      case BLGPU_OP_FILL_BOX_D: {
        double b[4]; memcpy(b, p, sizeof(b));
        if (!resolve_fill(c, &cop, &alpha)) break;
        c->fc.style = &s->style; c->fc.comp_op = cop; c->fc.alpha = alpha;
        fill_box_d(c, b[0], b[1], b[2], b[3]);
        break;
      }
      case BLGPU_OP_FILL_POLYGON_D: {
        uint32_t n; memcpy(&n, p, 4);
        if (c->stats) c->stats->input_vertices += n;
        if (!resolve_fill(c, &cop, &alpha)) break;
        if (n < 3) break;
        c->fc.style = &s->style; c->fc.comp_op = cop; c->fc.alpha = alpha;
        double* xy = (double*)malloc(sizeof(double) * 2 * n);
        memcpy(xy, p + 8, sizeof(double) * 2 * n);
        fill_polygon(c, xy, n, (uint32_t)s->fill_rule, &s->final_fixed, s->final_fixed_type);
        free(xy);
        break;
      }
      case BLGPU_OP_FILL_PATH_D:
        fill_path_op(c, p);
        break;
      case BLGPU_OP_SAVE:
        if (c->nstack == c->cap_stack) {
          c->cap_stack = c->cap_stack ? c->cap_stack * 2 : 8;
          c->stack = (OState*)realloc(c->stack, sizeof(OState) * (size_t)c->cap_stack);
        }
        c->stack[c->nstack++] = *s;
        break;
      case BLGPU_OP_RESTORE:
        if (c->nstack) *s = c->stack[--c->nstack];
        break;
      default:
        return -2;
    }
  }
  return 0;
}

static int default_band_height(int w) {   /* calculate_band_height, thread_count = 0 */
  int bh = 64;
  size_t pixel_count = (size_t)(unsigned)w * (size_t)bh;
  do {
    if (pixel_count * 4u <= 1024u * 256u) break;
    bh >>= 1;
    pixel_count >>= 1;
  } while (bh > 8);
  return bh;
}

int b2d_oracle_render(const uint8_t* stream, size_t size, uint32_t* out, const B2DOracleOptions* opt, B2DOracleStats* stats) {
  void* out_a8 = out;
  if (size < sizeof(BLGpuStreamHeader)) return -1;
  BLGpuStreamHeader hdr;
  memcpy(&hdr, stream, sizeof(hdr));
  if (hdr.magic != BLGPU_STREAM_MAGIC || hdr.version != BLGPU_STREAM_VERSION) return -1;

  OCtx c;
  memset(&c, 0, sizeof(c));
  c.w = (int)hdr.width;
  c.h = (int)hdr.height;
  c.dst_format = hdr.format ? (int)hdr.format : BLGPU_STREAM_FORMAT_PRGB32;
  if (c.dst_format < BLGPU_STREAM_FORMAT_PRGB32 || c.dst_format > BLGPU_STREAM_FORMAT_A8) return -1;
  /* An A8 target renders into a 32-bit canvas whose alpha bytes are the A8 pixels: the
   * reference's P8_Alpha operators (compopgeneric_p.h, fetchgeneric_p.h with PixelIO<P8_Alpha, ...>)
   * are its P32 operators' alpha lane, and no P32 lane reads another lane. */
  uint32_t* canvas = out;
  if (c.dst_format == BLGPU_STREAM_FORMAT_A8) {
    canvas = (uint32_t*)calloc((size_t)c.w * (size_t)c.h + 1u, 4u);
    if (!canvas) return -2;
  }
  out = canvas;
  c.pixels = out;
  c.lut_variant = opt ? opt->lut_variant : B2D_ORACLE_LUT_SSE2;
  c.stats = stats;
  if (stats) memset(stats, 0, sizeof(*stats));
  memset(out, 0, (size_t)c.w * (size_t)c.h * 4u);

  size_t off = sizeof(hdr);
  const uint32_t** images = (const uint32_t**)calloc(hdr.image_count + 1, sizeof(void*));
  int* iw = (int*)calloc(hdr.image_count + 1, sizeof(int));
  int* ih = (int*)calloc(hdr.image_count + 1, sizeof(int));
  int* ifmt = (int*)calloc(hdr.image_count + 1, sizeof(int));
  uint32_t** owned = (uint32_t**)calloc(hdr.image_count + 1, sizeof(void*));
  for (uint32_t i = 0; i < hdr.image_count; i++) {
    BLGpuStreamImage im;
    memcpy(&im, stream + off, sizeof(im));
    off += sizeof(im);
    size_t n = (size_t)im.width * im.height;
    owned[i] = (uint32_t*)malloc(n * 4u + 4u);
    memcpy(owned[i], stream + off, n * 4u);
    images[i] = owned[i];
    iw[i] = (int)im.width; ih[i] = (int)im.height;
    ifmt[i] = im.format == BLGPU_STREAM_FORMAT_XRGB32 ? O_FMT_XRGB32 : O_FMT_PRGB32;
    off += (n * 4u + 7u) & ~(size_t)7;
  }
  c.images = images; c.iw = iw; c.ih = ih; c.ifmt = ifmt;

  /* default state (rastercontext.cpp:4380-4415) */
  c.s.comp_op = 0; c.s.fill_rule = 0;
  c.s.global_alpha = 1.0; c.s.fill_alpha = 1.0; c.s.global_alpha_i = 255; c.s.fill_alpha_i = 255;
  c.s.gradient_quality = 0; c.s.pattern_quality = 1;
  OMat id = { 1, 0, 0, 1, 0, 0 };
  c.s.user = id;
  on_transform_changed(&c);
  set_style_solid(&c, 0, 0xFF000000u);
  set_style_solid(&c, 1, 0xFF000000u);
  c.s.stroke_alpha = 1.0; c.s.stroke_alpha_i = 255;
  c.s.stroke.width = 1.0; c.s.stroke.miter_limit = 4.0;   /* bl_stroke_options_init (path.cpp:186-190) */

  int bh = (opt && opt->band_height) ? (int)opt->band_height : default_band_height(c.w);
  o_storage_init(&c.storage, c.w, c.h, bh);
  double tol = 0.20 * 256.0;
  o_eb_init(&c.eb, &c.storage, c.w, c.h, tol * tol);

  size_t required_width = (((size_t)c.w + 1u + 4u) + 3u) & ~(size_t)3u;
  c.fc.dst = out; c.fc.width = c.w; c.fc.height = c.h; c.fc.stride = c.w;
  c.fc.cell_stride = required_width;
  c.fc.bit_stride = ((required_width / 4u) + 63u) / 64u;
  c.fc.cells = (uint32_t*)calloc((size_t)bh * c.fc.cell_stride, 4);
  c.fc.bits = (uint64_t*)calloc((size_t)bh * c.fc.bit_stride, 8);
  c.fc.stats = stats;

  int rc = replay(&c, stream, size, off);

  free(c.fc.cells); free(c.fc.bits);
  o_eb_free(&c.eb);
  o_storage_free(&c.storage);
  free(c.stack);
  for (uint32_t i = 0; i < hdr.image_count; i++) free(owned[i]);
  free(owned); free(images); free(iw); free(ih); free(ifmt);
  if (c.dst_format == BLGPU_STREAM_FORMAT_A8) {
    uint8_t* bytes = (uint8_t*)out_a8;
    for (size_t i = 0, n = (size_t)c.w * (size_t)c.h; i < n; i++) bytes[i] = (uint8_t)(canvas[i] >> 24);
    free(canvas);
  }
  return rc;
}
