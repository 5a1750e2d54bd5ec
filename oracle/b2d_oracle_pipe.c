/*
 * b2d_oracle_pipe.c - oracle (test infrastructure): the fixed pixel pipeline, restated from the
 * reference:
 *   fill loops      blend2d/pipeline/reference/fillgeneric_p.h:22-388
 *   comp-ops        blend2d/pipeline/reference/compopgeneric_p.h:24-184
 *   pixel math      blend2d/pipeline/reference/pixelgeneric_p.h:110-220 (64-bit unpacked form)
 *   fetchers        blend2d/pipeline/reference/fetchgeneric_p.h:25-1254
 *   box-u masks     blend2d/pipeline/pipedefs_p.h:520-815
 *   gradient LUTs   blend2d/pixelops/interpolation.cpp:19-156, interpolation_sse2.cpp:18-171,
 *                   interpolation_avx2.cpp:18-177
 */
#include "b2d_oracle_p.h"

/* ============================================================================================
 * Pixel math: the 64-bit unpacked layout [A:48 G:32 R:16 B:0], 16-bit lanes.
 * ============================================================================================ */

static const uint64_t kLaneFF = 0x00FF00FF00FF00FFull;

static inline uint64_t unpack(uint32_t p) { return (uint64_t)(p & 0x00FF00FFu) | ((uint64_t)(p & 0xFF00FF00u) << 24); }
static inline uint32_t pack(uint64_t u) { return (uint32_t)(((u >> 24) | u) & 0xFFFFFFFFu); }
static inline uint64_t div255(uint64_t u) {
  u += 0x0080008000800080ull;
  return ((u + ((u >> 8) & kLaneFF)) >> 8) & kLaneFF;
}
static inline uint64_t div256(uint64_t u) { return (u >> 8) & kLaneFF; }

uint32_t o_premultiply(uint32_t c) {   /* scalar_p.h:146-157 (SIMD div255 path) */
  uint32_t a = c >> 24;
  uint32_t b = c & 255u, g = (c >> 8) & 255u, r = (c >> 16) & 255u;
  uint32_t rb = ((b * a + 128u) * 257u) >> 16;
  uint32_t gg = ((g * a + 128u) * 257u) >> 16;
  uint32_t rr = ((r * a + 128u) * 257u) >> 16;
  uint32_t aa = ((255u * a + 128u) * 257u) >> 16;
  return (aa << 24) | (rr << 16) | (gg << 8) | rb;
}

static inline uint32_t op_src_over(uint32_t d, uint32_t s) {
  return s + pack(div255(unpack(d) * ((s >> 24) ^ 0xFFu)));
}
static inline uint32_t op_src_over_m(uint32_t d, uint32_t s, uint32_t m) {
  return op_src_over(d, pack(div255(unpack(s) * m)));
}
static inline uint32_t op_src_copy_m(uint32_t d, uint32_t s, uint32_t m) {
  return pack(div255(unpack(d) * (m ^ 0xFFu) + unpack(s) * m));
}

/* ============================================================================================
 * Fetchers
 * ============================================================================================ */

typedef struct {
  const OStyle* s;
  uint32_t solid;
  /* dithered gradients (FetchGradientBase<DITHER>, fetchgeneric_p.h:899-934): matrix row and
     column of the next fetched pixel */
  uint32_t dm_y, dm_x;
  /* linear */
  uint64_t pt, py;
  /* radial */
  double ry;
  float rx, rb, rd, rdd;
  /* conic */
  double tpx, tpy;
  float cx, ctx, cay, cby;
  /* pattern vertical context (FetchPatternVertAAExtendCtxAny) */
  const uint32_t* vptr;
  intptr_t stride0, stride1, ystop0, ystop1, vy, ptr_rewind;
  uintptr_t y_rewind;
  const uint32_t* vptr0;   /* FxFy: pixelPtr0 */
  /* pattern horizontal context */
  intptr_t hx, htx, hmx;
  uintptr_t hw, hrx;
  uint64_t acc;            /* FxFy accumulator (unpacked) */
  /* affine */
  uint64_t tx, ty, px, py_;
} OFetch;

/* 16x16 ordered-dither matrix of the reference (its bayer_matrix_16x16, tables_p.h:449-473),
 * restated from its recursive construction: the index interleaves the bits of the row and column,
 * low bits most significant, each pair weighted by the 2x2 pattern {{0, 3}, {2, 1}}; the entry is
 * the index scaled from [0, 256) to [0, 255] rounding half down. */
static uint8_t o_dither[16][16];
static int o_dither_ready;
static void o_dither_init(void) {
  static const uint32_t p2[2][2] = {{0, 3}, {2, 1}};
  for (uint32_t r = 0; r < 16; r++) {
    for (uint32_t c = 0; c < 16; c++) {
      uint32_t b = 0;
      for (uint32_t k = 0; k < 4; k++) b += p2[(r >> k) & 1u][(c >> k) & 1u] << (2u * (3u - k));
      o_dither[r][c] = (uint8_t)((b * 255u + 127u) >> 8);
    }
  }
  o_dither_ready = 1;
}

static inline uint32_t lut_fetch(OFetch* f, uint32_t idx) {
  if (!f->s->dither) return f->s->lut[idx];
  /* FetchGradientBase<DITHER>::fetch_pixel (fetchgeneric_p.h:922-933) */
  uint64_t v = f->s->lut64[idx];
  uint32_t dd = o_dither[f->dm_y][f->dm_x];
  uint32_t a = (uint32_t)(v >> 48) >> 8;
  uint32_t r = ((uint32_t)(v >> 32) & 0xFFFFu) + dd; r >>= 8; if (r > a) r = a;
  uint32_t g = ((uint32_t)(v >> 16) & 0xFFFFu) + dd; g >>= 8; if (g > a) g = a;
  uint32_t b = ((uint32_t)v & 0xFFFFu) + dd; b >>= 8; if (b > a) b = a;
  f->dm_x = (f->dm_x + 1u) & 15u;
  return (a << 24) | (r << 16) | (g << 8) | b;
}

/* --- pattern vertical context (fetchgeneric_p.h:78-155) --- */
static void vctx_init(OFetch* f, uint32_t y_pos) {
  const OStyle* s = f->s;
  f->vptr = s->src;
  f->stride0 = s->src_stride;
  f->stride1 = f->stride0;
  f->ystop0 = s->src_h;
  f->ystop1 = f->ystop0;
  f->y_rewind = s->vx_y_rewind;
  f->ptr_rewind = s->vx_ptr_rewind;
  f->vy = (intptr_t)y_pos + (intptr_t)s->pat_ty;
  intptr_t ry = s->pat_ry;
  if (ry == 0) {
    intptr_t cy = f->vy < 0 ? 0 : (f->vy > f->ystop0 - 1 ? f->ystop0 - 1 : f->vy);
    f->vptr += cy * f->stride0;
    if (f->vy != cy) { f->stride0 = 0; f->ystop0 = 0; }
    else { f->stride1 = 0; f->ystop1 = 0; }
  }
  else {
    f->vy = (intptr_t)((uint32_t)f->vy % (uint32_t)ry);
    if (f->vy >= f->ystop0) {
      f->vptr += (f->ystop0 - 1) * f->stride0;
      f->stride0 = -f->stride0;
      f->vy -= f->ystop0;
    }
    else if (f->ystop0 != ry) {
      f->stride1 = -f->stride0;
    }
    f->vptr += f->vy * f->stride0;
  }
}
static void vctx_advance(OFetch* f) {
  if (++f->vy == f->ystop0) {
    intptr_t t = f->ystop0; f->ystop0 = f->ystop1; f->ystop1 = t;
    t = f->stride0; f->stride0 = f->stride1; f->stride1 = t;
    f->vy -= (intptr_t)f->y_rewind;
    f->vptr -= f->ptr_rewind;
  }
  else {
    f->vptr += f->stride0;
  }
}

/* --- pattern horizontal contexts (fetchgeneric_p.h:178-352), index in pixels --- */
static inline int hctx_kind(int ft) {   /* 0 pad, 1 repeat, 2 ror */
  if (ft == O_FT_PAT_ALIGNED_PAD || ft == O_FT_PAT_FXFY_PAD) return 0;
  if (ft == O_FT_PAT_ALIGNED_REPEAT) return 1;
  return 2;
}
static inline uintptr_t pmod_u(uintptr_t a, uintptr_t b) { return a % b; }

static void hctx_span_init(OFetch* f) {
  const OStyle* s = f->s;
  switch (hctx_kind(s->fetch_type)) {
    case 0: f->htx = (intptr_t)(uintptr_t)s->pat_tx; f->hmx = (intptr_t)(uintptr_t)(s->src_w - 1); break;
    case 1: f->hw = (uintptr_t)s->src_w; f->htx = (intptr_t)(uintptr_t)s->pat_tx; break;
    default: f->hw = (uintptr_t)s->src_w; f->hrx = (uintptr_t)s->pat_rx; f->htx = (intptr_t)s->pat_tx; break;
  }
}
static void hctx_span_start(OFetch* f, uint32_t x) {
  switch (hctx_kind(f->s->fetch_type)) {
    case 0: f->hx = (intptr_t)(uintptr_t)x + f->htx; break;
    case 1: f->hx = (intptr_t)pmod_u((uintptr_t)x + (uintptr_t)f->htx, f->hw); break;
    default:
      f->hx = (intptr_t)pmod_u((uintptr_t)x + (uintptr_t)f->htx, f->hrx);
      if (f->hx >= (intptr_t)f->hw) f->hx -= (intptr_t)f->hrx;
      break;
  }
}
static void hctx_span_advance(OFetch* f, uint32_t diff) {
  switch (hctx_kind(f->s->fetch_type)) {
    case 0: f->hx += (intptr_t)(uintptr_t)diff; break;
    case 1: {
      uintptr_t x = (uintptr_t)f->hx + diff;
      if (x >= f->hw) x = pmod_u(x, f->hw);
      f->hx = (intptr_t)x;
      break;
    }
    default:
      f->hx += (intptr_t)diff;
      if (f->hx >= (intptr_t)f->hw) {
        f->hx = (intptr_t)pmod_u((uintptr_t)f->hx, f->hrx);
        if (f->hx >= (intptr_t)f->hw) f->hx -= (intptr_t)f->hrx;
      }
      break;
  }
}
static inline size_t hctx_index(const OFetch* f) {
  switch (hctx_kind(f->s->fetch_type)) {
    case 0: return (size_t)(f->hx < 0 ? 0 : (f->hx > f->hmx ? f->hmx : f->hx));
    case 1: return (size_t)f->hx;
    default: { intptr_t m = f->hx >> 63; return (size_t)(f->hx ^ m); }
  }
}
static inline void hctx_advance1(OFetch* f) {
  switch (hctx_kind(f->s->fetch_type)) {
    case 0: f->hx++; break;
    case 1: { uintptr_t x = (uintptr_t)f->hx + 1u; if (x >= f->hw) x = 0; f->hx = (intptr_t)x; break; }
    default: if (++f->hx >= (intptr_t)f->hw) f->hx -= (intptr_t)f->hrx; break;
  }
}

/* --- affine pattern context (fetchgeneric_p.h:354-465) --- */
static inline void af_normalize(const OStyle* s, uint64_t vx, uint64_t vy, uint64_t* ox, uint64_t* oy) {
  uint32_t x = (uint32_t)((int32_t)(vx >> 32) % s->af_tw);
  uint32_t y = (uint32_t)((int32_t)(vy >> 32) % s->af_th);
  if ((int32_t)x < 0) x += (uint32_t)s->af_rx;
  if ((int32_t)y < 0) y += (uint32_t)s->af_ry;
  if ((int32_t)x > s->af_ox) x -= (uint32_t)s->af_rx;
  if ((int32_t)y > s->af_oy) y -= (uint32_t)s->af_ry;
  *ox = ((uint64_t)x << 32) | (vx & 0xFFFFFFFFu);
  *oy = ((uint64_t)y << 32) | (vy & 0xFFFFFFFFu);
}
static inline void af_index(const OStyle* s, uint64_t px, uint64_t py, int offx, int offy, uint32_t* ix, uint32_t* iy) {
  int32_t x = (int32_t)(px >> 32) + offx;
  int32_t y = (int32_t)(py >> 32) + offy;
  x = x < s->af_minx ? s->af_minx : x;
  y = y < s->af_miny ? s->af_miny : y;
  if (x > s->af_maxx) x = s->af_corx;
  if (y > s->af_maxy) y = s->af_cory;
  x = x ^ (x >> 31);
  y = y ^ (y >> 31);
  *ix = (uint32_t)x;
  *iy = (uint32_t)y;
}
static inline void af_advance_x(OFetch* f) {
  const OStyle* s = f->s;
  f->px += s->af_xx;
  f->py_ += s->af_xy;
  int32_t x = (int32_t)(f->px >> 32);
  int32_t y = (int32_t)(f->py_ >> 32);
  x -= (-(int32_t)(x > s->af_ox)) & s->af_rx;
  y -= (-(int32_t)(y > s->af_oy)) & s->af_ry;
  f->px = ((uint64_t)(uint32_t)x << 32) | (f->px & 0xFFFFFFFFu);
  f->py_ = ((uint64_t)(uint32_t)y << 32) | (f->py_ & 0xFFFFFFFFu);
}

/* --- generic fetcher interface --- */

static void conic_begin_scanline(OFetch* f) {
  const OStyle* s = f->s;
  f->ctx = (float)f->tpx;
  f->cay = (float)f->tpy;
  uint32_t sb;
  memcpy(&sb, &f->cay, 4);
  uint32_t nb;
  memcpy(&nb, &s->con_n1, 4);
  uint32_t byb = ((uint32_t)((int32_t)sb >> 31)) & nb;
  memcpy(&f->cby, &byb, 4);
  f->cay = fabsf(f->cay);
}

static void fetch_span_init_y(OFetch* f, uint32_t y) {
  const OStyle* s = f->s;
  f->dm_y = y & 15u;           /* _init_gradient_base: pixel origin (0, 0) */
  switch (s->fetch_type) {
    case O_FT_SOLID: f->solid = s->solid; break;
    case O_FT_LINEAR_PAD: case O_FT_LINEAR_ROR:
      f->pt = 0; f->py = s->lin_pt0; f->py += (uint64_t)y * s->lin_dy; break;
    case O_FT_RADIAL_PAD: case O_FT_RADIAL_ROR:
      f->ry = (double)(int32_t)y; break;
    case O_FT_CONIC:
      f->tpx = s->con_tx + s->con_yx * (double)(int)y;
      f->tpy = s->con_ty + s->con_yy * (double)(int)y;
      break;
    case O_FT_PAT_ALIGNED_PAD: case O_FT_PAT_ALIGNED_REPEAT: case O_FT_PAT_ALIGNED_ROR:
      vctx_init(f, y); hctx_span_init(f); break;
    case O_FT_PAT_FXFY_PAD: case O_FT_PAT_FXFY_ROR:
      vctx_init(f, y); f->vptr0 = f->vptr; vctx_advance(f); hctx_span_init(f); break;
    default: /* affine */
      f->tx = s->af_tx + s->af_yx * (uint64_t)y;
      f->ty = s->af_ty + s->af_yy * (uint64_t)y;
      break;
  }
}

static void fxfy_init_acc(OFetch* f) {
  const OStyle* s = f->s;
  size_t idx = hctx_index(f);
  uint64_t a = unpack(f->vptr0[idx]) * s->pat_wa;
  uint64_t c = unpack(f->vptr[idx]) * s->pat_wc;
  f->acc = a + c;
}

static void fetch_span_start_x(OFetch* f, uint32_t x) {
  const OStyle* s = f->s;
  f->dm_x = x & 15u;           /* _initGradientX */
  switch (s->fetch_type) {
    case O_FT_SOLID: break;
    case O_FT_LINEAR_PAD: case O_FT_LINEAR_ROR: f->pt = f->py + (uint64_t)x * s->lin_dt; break;
    case O_FT_RADIAL_PAD: case O_FT_RADIAL_ROR: {
      double ptx = s->rad_yx * f->ry + s->rad_tx;
      double pty = s->rad_yy * f->ry + s->rad_ty;
      double b = f->ry * s->rad_by + s->rad_b0;
      double sq_dist = ptx * ptx + pty * pty;
      f->rx = (float)(int32_t)x;
      f->rb = (float)(b * s->rad_inv2a);
      f->rd = (float)((s->rad_amul4 * (sq_dist - s->rad_sq_fr) + b * b) * s->rad_sq_inv2a);
      f->rdd = (float)((f->ry * s->rad_ddy + s->rad_dd0) * s->rad_sq_inv2a);
      break;
    }
    case O_FT_CONIC: f->cx = (float)(int)x; conic_begin_scanline(f); break;
    case O_FT_PAT_ALIGNED_PAD: case O_FT_PAT_ALIGNED_REPEAT: case O_FT_PAT_ALIGNED_ROR:
      hctx_span_start(f, x); break;
    case O_FT_PAT_FXFY_PAD: case O_FT_PAT_FXFY_ROR:
      hctx_span_start(f, x); fxfy_init_acc(f); break;
    default:
      af_normalize(s, f->tx + s->af_xx * (uint64_t)x, f->ty + s->af_xy * (uint64_t)x, &f->px, &f->py_);
      break;
  }
}

static void fetch_span_advance_x(OFetch* f, uint32_t x, uint32_t diff) {
  const OStyle* s = f->s;
  f->dm_x = x & 15u;           /* _initGradientX */
  switch (s->fetch_type) {
    case O_FT_SOLID: break;
    case O_FT_LINEAR_PAD: case O_FT_LINEAR_ROR: f->pt += (uint64_t)diff * s->lin_dt; break;
    case O_FT_RADIAL_PAD: case O_FT_RADIAL_ROR: f->rx += (float)(int32_t)diff; break;
    case O_FT_CONIC: f->cx += (float)(int32_t)diff; break;
    case O_FT_PAT_ALIGNED_PAD: case O_FT_PAT_ALIGNED_REPEAT: case O_FT_PAT_ALIGNED_ROR:
      hctx_span_advance(f, diff); break;
    case O_FT_PAT_FXFY_PAD: case O_FT_PAT_FXFY_ROR:
      hctx_span_advance(f, diff); fxfy_init_acc(f); break;
    default:
      af_normalize(s, f->px + s->af_xx * (uint64_t)diff, f->py_ + s->af_xy * (uint64_t)diff, &f->px, &f->py_);
      break;
  }
}

static void fetch_advance_y(OFetch* f) {
  const OStyle* s = f->s;
  f->dm_y = (f->dm_y + 1u) & 15u;   /* _advanceGradientY */
  switch (s->fetch_type) {
    case O_FT_SOLID: break;
    case O_FT_LINEAR_PAD: case O_FT_LINEAR_ROR: f->py += s->lin_dy; break;
    case O_FT_RADIAL_PAD: case O_FT_RADIAL_ROR: f->ry += 1.0; break;
    case O_FT_CONIC: f->tpx += s->con_yx; f->tpy += s->con_yy; break;
    case O_FT_PAT_ALIGNED_PAD: case O_FT_PAT_ALIGNED_REPEAT: case O_FT_PAT_ALIGNED_ROR: vctx_advance(f); break;
    case O_FT_PAT_FXFY_PAD: case O_FT_PAT_FXFY_ROR: f->vptr0 = f->vptr; vctx_advance(f); break;
    default: f->tx += s->af_yx; f->ty += s->af_yy; break;
  }
}

static uint32_t fetch_pixel(OFetch* f) {
  const OStyle* s = f->s;
  switch (s->fetch_type) {
    case O_FT_SOLID: return f->solid;
    case O_FT_LINEAR_PAD: case O_FT_LINEAR_ROR: {
      uint32_t idx = (uint32_t)(f->pt >> 32);
      if (s->fetch_type == O_FT_LINEAR_PAD) {
        int32_t i = (int32_t)idx;
        idx = (uint32_t)(i < 0 ? 0 : (i > (int32_t)s->maxi ? (int32_t)s->maxi : i));
      }
      else {
        uint32_t a = idx & s->maxi, b = a ^ s->rori;
        idx = b < a ? b : a;
      }
      f->pt += s->lin_dt;
      return lut_fetch(f, idx);
    }
    case O_FT_RADIAL_PAD: case O_FT_RADIAL_ROR: {
      float x = f->rx;
      float sq_x = x * x;
      float a = sqrtf(fabsf(sq_x * s->rad_ddd + (x * f->rdd + f->rd)));
      float v = (x * s->rad_bd + f->rb) + a;
      uint32_t idx = (uint32_t)o_trunc_to_int_f(v);
      f->rx += 1.0f;
      if (s->fetch_type == O_FT_RADIAL_PAD) {
        int32_t i = (int32_t)idx;
        idx = (uint32_t)(i < 0 ? 0 : (i > (int32_t)s->maxi ? (int32_t)s->maxi : i));
      }
      else {
        uint32_t aa = idx & s->maxi, bb = aa ^ s->rori;
        idx = bb < aa ? bb : aa;
      }
      return lut_fetch(f, idx);
    }
    case O_FT_CONIC: {
      float x = f->cx * s->con_xx + f->ctx;
      float ax = fabsf(x);
      float xy_min = f->cay < ax ? f->cay : ax;    /* bl_min(ax, ay) */
      float xy_max = ax < f->cay ? f->cay : ax;    /* bl_max(ax, ay) */
      uint32_t smsk = (ax == xy_min) ? 0xFFFFFFFFu : 0u;
      uint32_t n4b; memcpy(&n4b, &s->con_n4, 4);
      uint32_t sb = smsk & n4b; float sv; memcpy(&sv, &sb, 4);
      float p = xy_min / xy_max;
      float p_sq = p * p;
      float v = p_sq * s->con_q[3] + s->con_q[2];
      v = v * p_sq + s->con_q[1];
      v = v * p_sq + s->con_q[0];
      v = fabsf(v * p + (-sv));
      uint32_t xb; memcpy(&xb, &x, 4);
      uint32_t n2b; memcpy(&n2b, &s->con_n2, 4);
      uint32_t mb = ((uint32_t)((int32_t)xb >> 31)) & n2b; float mv; memcpy(&mv, &mb, 4);
      v = fabsf(v - mv);
      v = fabsf(v - f->cby) + s->con_offset;
      int32_t ni = o_nearby_to_int_f(v);
      uint32_t idx = (uint32_t)(ni < s->con_maxi ? ni : s->con_maxi) & (uint32_t)s->con_rori;
      f->cx += 1.0f;
      return lut_fetch(f, idx);
    }
    case O_FT_PAT_ALIGNED_PAD: case O_FT_PAT_ALIGNED_REPEAT: case O_FT_PAT_ALIGNED_ROR: {
      uint32_t p = f->vptr[hctx_index(f)];
      hctx_advance1(f);
      return p;
    }
    case O_FT_PAT_FXFY_PAD: case O_FT_PAT_FXFY_ROR: {
      hctx_advance1(f);
      size_t idx = hctx_index(f);
      uint64_t p0 = unpack(f->vptr0[idx]);
      uint64_t p1 = unpack(f->vptr[idx]);
      uint64_t u = p0 * s->pat_wb + p1 * s->pat_wd + f->acc;
      f->acc = p0 * s->pat_wa + p1 * s->pat_wc;
      return pack(div256(u));
    }
    case O_FT_PAT_AFFINE_NN: {
      uint32_t ix, iy;
      af_index(s, f->px, f->py_, 0, 0, &ix, &iy);
      af_advance_x(f);
      return s->src[(intptr_t)iy * s->src_stride + ix];
    }
    default: {
      uint32_t x0, y0, x1, y1;
      af_index(s, f->px, f->py_, 0, 0, &x0, &y0);
      af_index(s, f->px, f->py_, 1, 1, &x1, &y1);
      uint32_t wx = (uint32_t)(f->px & 0xFFFFFFFFu) >> 24;
      uint32_t wy = (uint32_t)(f->py_ & 0xFFFFFFFFu) >> 24;
      af_advance_x(f);
      uint32_t ix = 256 - wx, iy = 256 - wy;
      const uint32_t* l0 = s->src + (intptr_t)y0 * s->src_stride;
      const uint32_t* l1 = s->src + (intptr_t)y1 * s->src_stride;
      uint64_t p0 = unpack(l0[x0]) * iy + unpack(l1[x0]) * wy;
      uint64_t p1 = unpack(l0[x1]) * iy + unpack(l1[x1]) * wy;
      p0 = div256(p0) * ix;
      p1 = div256(p1) * wx;
      return pack(div256(p0 + p1));
    }
  }
}

/* rect_init_fetch / rectStartX for the box-aligned fill (fetchgeneric_p.h). */
static void fetch_rect_init(OFetch* f, uint32_t x, uint32_t y, uint32_t w) {
  const OStyle* s = f->s;
  (void)w;
  switch (s->fetch_type) {
    case O_FT_LINEAR_PAD: case O_FT_LINEAR_ROR:
      f->dm_y = y & 15u;
      f->pt = 0; f->py = s->lin_pt0; f->py += (uint64_t)y * s->lin_dy + (uint64_t)x * s->lin_dt; break;
    case O_FT_PAT_ALIGNED_PAD: case O_FT_PAT_ALIGNED_REPEAT: case O_FT_PAT_ALIGNED_ROR:
    case O_FT_PAT_FXFY_PAD: case O_FT_PAT_FXFY_ROR: {
      fetch_span_init_y(f, y);
      /* rect_init of the horizontal context folds x into tx (fetchgeneric_p.h:187-279). */
      switch (hctx_kind(s->fetch_type)) {
        case 0: f->htx += (intptr_t)(uintptr_t)x; break;
        case 1: f->htx = (intptr_t)pmod_u((uintptr_t)x + (uintptr_t)f->htx, f->hw); break;
        default:
          f->htx = (intptr_t)pmod_u((uintptr_t)x + (uintptr_t)f->htx, f->hrx);
          if (f->htx >= (intptr_t)f->hw) f->htx -= (intptr_t)f->hrx;
          break;
      }
      break;
    }
    case O_FT_PAT_AFFINE_NN: case O_FT_PAT_AFFINE_BI:
      f->tx = s->af_tx + s->af_yx * (uint64_t)y + s->af_xx * (uint64_t)x;
      f->ty = s->af_ty + s->af_yy * (uint64_t)y + s->af_xy * (uint64_t)x;
      break;
    default:
      fetch_span_init_y(f, y);
      break;
  }
}
static void fetch_rect_start_x(OFetch* f, uint32_t x) {
  const OStyle* s = f->s;
  switch (s->fetch_type) {
    case O_FT_LINEAR_PAD: case O_FT_LINEAR_ROR: f->dm_x = x & 15u; f->pt = f->py; break;
    case O_FT_PAT_ALIGNED_PAD: case O_FT_PAT_ALIGNED_REPEAT: case O_FT_PAT_ALIGNED_ROR:
      f->hx = f->htx; break;
    case O_FT_PAT_FXFY_PAD: case O_FT_PAT_FXFY_ROR:
      f->hx = f->htx; fxfy_init_acc(f); break;
    case O_FT_PAT_AFFINE_NN: case O_FT_PAT_AFFINE_BI:
      af_normalize(s, f->tx, f->ty, &f->px, &f->py_); break;
    default:
      fetch_span_start_x(f, x); break;
  }
}

/* ============================================================================================
 * Compositing helpers
 * ============================================================================================ */

/* src_or: PixelIO<P32_A8R8G8B8, XRGB32>::fetch (pixelgeneric_p.h:650-661) sets the alpha byte of
 * every texel it reads; the bilinear weights are per channel, so setting it after the
 * interpolation gives the same pixel. */
static inline void comp_masked(OFillCtx* fc, OFetch* f, uint32_t* d, uint32_t m) {
  uint32_t s = fetch_pixel(f) | fc->src_or;
  *d = fc->comp_op ? op_src_copy_m(*d, s, m) : op_src_over_m(*d, s, m);
  if (m && fc->stats) fc->stats->composited_pixels++;
}
static inline void comp_opaque(OFillCtx* fc, OFetch* f, uint32_t* d) {
  uint32_t s = fetch_pixel(f) | fc->src_or;
  *d = fc->comp_op ? s : op_src_over(*d, s);
  if (fc->stats) fc->stats->composited_pixels++;
}
static void comp_cspan(OFillCtx* fc, OFetch* f, uint32_t* d, size_t w, uint32_t m) {
  if (fc->comp_op == 1 && m == 255) { for (size_t i = 0; i < w; i++) comp_opaque(fc, f, d + i); }
  else { for (size_t i = 0; i < w; i++) comp_masked(fc, f, d + i, m); }
}

/* ============================================================================================
 * Fill loops
 * ============================================================================================ */

void o_fill_box_a(OFillCtx* fc, int x0, int y0, int x1, int y1) {   /* FillBoxA_Base */
  OFetch f;
  memset(&f, 0, sizeof(f));
  f.s = fc->style;
  uint32_t w = (uint32_t)(x1 - x0), h = (uint32_t)(y1 - y0);
  uint32_t msk = fc->alpha;
  fetch_rect_init(&f, (uint32_t)x0, (uint32_t)y0, w);
  for (uint32_t y = 0; y < h; y++) {
    uint32_t* d = fc->dst + (intptr_t)(y0 + (int)y) * fc->stride + x0;
    fetch_rect_start_x(&f, (uint32_t)x0);
    if (fc->comp_op == 1 && msk == 255) { for (uint32_t i = 0; i < w; i++) comp_opaque(fc, &f, d + i); }
    else { for (uint32_t i = 0; i < w; i++) comp_masked(fc, &f, d + i, msk); }
    fetch_advance_y(&f);
  }
}

/* Masked box fill: fill_box_masked_a (rendercommandprocsync_p.h:65-85), one vmask command per
 * scanline repeated down the box, run by FillMask_Base (fillgeneric_p.h:67-162): the mask byte, or
 * udiv255(mask * alpha) below full alpha (compopgeneric_p.h:165-183). */
void o_fill_mask_a(OFillCtx* fc, int x0, int y0, int x1, int y1, const uint8_t* mask, intptr_t mask_stride) {
  uint32_t alpha = fc->alpha;
  OFetch f;
  memset(&f, 0, sizeof(f));
  f.s = fc->style;
  fetch_span_init_y(&f, (uint32_t)y0);
  for (int y = y0; y < y1; y++) {
    uint32_t* drow = fc->dst + (intptr_t)y * fc->stride;
    const uint8_t* m = mask + (intptr_t)(y - y0) * mask_stride;
    fetch_span_start_x(&f, (uint32_t)x0);
    for (int x = x0; x < x1; x++) {
      uint32_t v = m[x - x0];
      if (alpha < 255u) v = ((v * alpha + 0x80u) * 0x101u) >> 16;   /* Scalar::udiv255 */
      comp_masked(fc, &f, drow + x, v);
    }
    fetch_advance_y(&f);
  }
}

/* Box-unaligned fill: FillData::init_box_u_8bpc_24x8 mask commands (pipedefs_p.h:644-815)
 * executed by FillMask_Base (fillgeneric_p.h:67-162). Each scanline is a list of
 * {x0, x1, cmask | vmask pointer} spans. */
typedef struct { uint32_t x0, x1; int vmask; uint32_t m; const uint8_t* vm; } OMaskSpan;

void o_fill_box_u(OFillCtx* fc, int bx0, int by0, int bx1, int by1) {
  uint32_t alpha = fc->alpha;
  uint32_t ax0 = (uint32_t)bx0 >> 8, ay0 = (uint32_t)by0 >> 8;
  uint32_t ax1 = (uint32_t)(bx1 + 0xFF) >> 8, ay1 = (uint32_t)(by1 + 0xFF) >> 8;
  uint32_t fx0 = (uint32_t)bx0 & 0xFFu, fy0 = (uint32_t)by0 & 0xFFu;
  uint32_t fx1 = ((uint32_t)(bx1 - 1) & 0xFFu) + 1u, fy1 = ((uint32_t)(by1 - 1) & 0xFFu) + 1u;
  uint32_t w = ax1 - ax0, h = ay1 - ay0;
  fy0 = (h == 1 ? fy1 : 256u) - fy0;
  uint32_t fy0_a = fy0 * alpha, fy1_a = fy1 * alpha;

  /* Three row kinds: first (0), middle (1), last (2); each row kind has up to 3 spans. */
  OMaskSpan rows[3][3];
  int nspans[3] = { 0, 0, 0 };
  uint8_t mbuf[3][32];
  int row_y0 = (int)ay0, row_y1 = (int)(ay0 + h);
  int first_row_valid = 1, last_row_valid = 1;

  if (w == 1) {
    uint32_t f = fx1 - fx0;
    uint32_t m0 = (f * fy0_a) >> 16, m1 = (f * alpha) >> 8, m2 = (f * fy1_a) >> 16;
    rows[0][0] = (OMaskSpan){ ax0, ax1, 0, m0, NULL }; nspans[0] = 1;
    rows[1][0] = (OMaskSpan){ ax0, ax1, 0, m1, NULL }; nspans[1] = 1;
    rows[2][0] = (OMaskSpan){ ax0, ax1, 0, m2, NULL }; nspans[2] = 1;
    if (h == 1) { if (!m0) return; }
    else {
      if (!m0) { row_y0++; first_row_valid = 0; }
      if (!m2) { row_y1--; last_row_valid = 0; }
      if (!(row_y0 < row_y1 && m1 != 0)) return;
    }
  }
  else {
    uint32_t m0x1 = fy0_a >> 8, m1x1 = alpha, m2x1 = fy1_a >> 8;
    fx0 = 256 - fx0;
    if ((fx0 & fx1) == 256) {
      rows[0][0] = (OMaskSpan){ ax0, ax1, 0, m0x1, NULL }; nspans[0] = 1;
      rows[1][0] = (OMaskSpan){ ax0, ax1, 0, m1x1, NULL }; nspans[1] = 1;
      rows[2][0] = (OMaskSpan){ ax0, ax1, 0, m2x1, NULL }; nspans[2] = 1;
    }
    else {
      uint32_t mx1[3] = { m0x1, m1x1, m2x1 };
      uint32_t mx0[3] = { (fx0 * fy0_a) >> 16, (fx0 * alpha) >> 8, (fx0 * fy1_a) >> 16 };
      uint32_t mx2[3] = { (fx1 * fy0_a) >> 16, (fx1 * alpha) >> 8, (fx1 * fy1_a) >> 16 };
      for (int k = 0; k < 3; k++) {
        memset(mbuf[k], 0, 4);
        memset(mbuf[k] + 4, (int)mx1[k], 28);
        mbuf[k][4] = (uint8_t)mx0[k];
      }
      uint32_t wAlign = (4u - (w & 3u)) & 3u;
      if (wAlign > ax0) wAlign = 0;
      uint32_t sx0 = ax0 - wAlign;
      uint32_t sw = w + wAlign;
      int base = 4 - (int)wAlign;    /* mask_ptr offset into mbuf */
      if (sw <= 20) {
        for (int k = 0; k < 3; k++) {
          mbuf[k][base + (int)sw - 1] = (uint8_t)mx2[k];
          rows[k][0] = (OMaskSpan){ sx0, ax1, 1, 0, mbuf[k] + base };
          nspans[k] = 1;
        }
      }
      else {
        uint32_t inner_width = (sw - 5u) & ~7u;
        uint32_t inner_end = sx0 + 4u + inner_width;
        uint32_t tail_width = ax1 - inner_end;
        for (int k = 0; k < 3; k++) {
          mbuf[k][base + 15] = (uint8_t)mx2[k];
          rows[k][0] = (OMaskSpan){ sx0, sx0 + 4u, 1, 0, mbuf[k] + base };
          rows[k][1] = (OMaskSpan){ sx0 + 4u, inner_end, 0, mx1[k], NULL };
          rows[k][2] = (OMaskSpan){ inner_end, ax1, 1, 0, mbuf[k] + base + 16 - (int)tail_width };
          nspans[k] = 3;
        }
      }
    }
    if (!m0x1) { row_y0++; first_row_valid = 0; }
    if (!m2x1) { row_y1--; last_row_valid = 0; }
    if (!(row_y0 < row_y1)) return;
  }

  /* FillMask_Base: spanInitY at the (possibly advanced) box y0, then per scanline. */
  OFetch f;
  memset(&f, 0, sizeof(f));
  f.s = fc->style;
  fetch_span_init_y(&f, (uint32_t)row_y0);
  for (int y = row_y0; y < row_y1; y++) {
    int kind;
    if (h == 1) kind = 0;
    else if (y == (int)ay0 && first_row_valid) kind = 0;
    else if (y == (int)(ay0 + h - 1) && last_row_valid) kind = 2;
    else kind = 1;
    uint32_t* drow = fc->dst + (intptr_t)y * fc->stride;
    uint32_t x = rows[kind][0].x0;
    fetch_span_start_x(&f, x);
    for (int k = 0; k < nspans[kind]; k++) {
      OMaskSpan* sp = &rows[kind][k];
      if (x != sp->x0) { fetch_span_advance_x(&f, sp->x0, sp->x0 - x); x = sp->x0; }
      uint32_t n = sp->x1 - sp->x0;
      if (!sp->vmask) comp_cspan(fc, &f, drow + x, n, sp->m);
      else for (uint32_t i = 0; i < n; i++) comp_masked(fc, &f, drow + x + i, sp->vm[i]);
      x += n;
    }
    fetch_advance_y(&f);
  }
}

/* FillAnalytic_Base::fill_func (fillgeneric_p.h:174-388) with 64-bit LSB-first bit words. */
static inline uint32_t calc_mask(uint32_t cov, uint32_t rule_mask, uint32_t alpha) {
  uint32_t m = (((uint32_t)((int32_t)cov >> 9)) & rule_mask) - 256u;
  int32_t mi = (int32_t)m;
  uint32_t am = (uint32_t)(mi < 0 ? -mi : mi);
  if (am > 256u) am = 256u;
  return (am * alpha) >> 8;
}

void o_fill_analytic_band(OFillCtx* fc, int box_x1, int y0, int y1, uint32_t fill_rule,
                          uint64_t* bit_top, uint32_t* cell_top) {
  const size_t kPixelsPerBitWord = 4 * 64;
  uint32_t rule_mask = fill_rule == 0 ? 0xFFFFFFFFu : 0x1FFu;
  uint32_t alpha = fc->alpha;

  OFetch f;
  memset(&f, 0, sizeof(f));
  f.s = fc->style;
  fetch_span_init_y(&f, (uint32_t)y0);

  uint64_t* bit_ptr = bit_top;
  uint64_t* bit_ptr_end = NULL;
  uint32_t* cell_ptr = cell_top;
  uint32_t* dst_row = fc->dst + (intptr_t)y0 * fc->stride;
  uint32_t* dst_ptr = dst_row;
  uint32_t y = (uint32_t)(y1 - y0);

  size_t x0 = 0, x_end = (size_t)box_x1, x_off = 0, i = 0;
  uint32_t cov = 0, msk = 0;
  uint64_t bit_word = 0, bit_word_tmp;

  goto L_Scanline_Init;

L_BitScan_Init:
  x0 = (size_t)__builtin_ctzll(bit_word);
  bit_ptr[-1] = 0;
  bit_word_tmp = ~(uint64_t)0 << x0;
  x0 = x0 * 4 + x_off;
  dst_ptr += x0;
  cell_ptr += x0;
  fetch_span_start_x(&f, (uint32_t)x0);
  if (x0 >= x_end) goto L_Scanline_Done0;
  cov = 256u << 9;
  msk = 0;
  bit_word ^= bit_word_tmp;
  if (bit_word) goto L_BitScan_Match;
  i = 64;
  if (bit_ptr == bit_ptr_end) goto L_BitScan_End;

L_BitScan_Next:
  for (;;) {
    bit_word = ~(uint64_t)0 ^ bit_ptr[0];
    *bit_ptr++ = 0;
    x_off += kPixelsPerBitWord;
    if (bit_word) goto L_BitScan_Match;
    if (bit_ptr == bit_ptr_end) goto L_BitScan_End;
  }

L_BitScan_Match:
  i = (size_t)__builtin_ctzll(bit_word);

L_BitScan_End:
  bit_word_tmp = i >= 64 ? 0 : (~(uint64_t)0 << i);
  i *= 4;
  bit_word ^= bit_word_tmp;
  i += x_off;
  if (i > x_end) i = x_end;
  i -= x0;
  x0 += i;

  goto VLoop_CalcMsk;
  for (;;) {
    i--;
    cell_ptr++;
    comp_masked(fc, &f, dst_ptr, msk);
    dst_ptr++;
VLoop_CalcMsk:
    cov += cell_ptr[0];
    *cell_ptr = 0;
    msk = calc_mask(cov, rule_mask, alpha);
    if (!i) break;
  }

  if (x0 >= x_end) goto L_Scanline_Done1;

  while (!bit_word) {
    x_off += kPixelsPerBitWord;
    if (bit_ptr == bit_ptr_end) goto L_Scanline_Done1;
    bit_word = *bit_ptr++;
  }

  i = (size_t)__builtin_ctzll(bit_word);
  bit_word ^= ~(uint64_t)0 << i;
  bit_ptr[-1] = 0;
  i = i * 4 + x_off - x0;
  x0 += i;
  cell_ptr += i;
  if (!msk) {
    dst_ptr += i;
    fetch_span_advance_x(&f, (uint32_t)x0, (uint32_t)i);
  }
  else {
    comp_cspan(fc, &f, dst_ptr, i, msk);
    dst_ptr += i;
  }
  if (bit_word) goto L_BitScan_Match;
  else goto L_BitScan_Next;

L_Scanline_Done0:
  cell_ptr[0] = 0;

L_Scanline_Done1:
  dst_ptr -= x0;
  cell_ptr -= x0;
  if (--y == 0) return;
  bit_ptr = bit_ptr_end;
  do {
    dst_ptr += fc->stride;
    cell_ptr += fc->cell_stride;
    fetch_advance_y(&f);

L_Scanline_Init:
    x_off = 0;
    bit_word = 0;
    bit_ptr_end = bit_ptr + fc->bit_stride;
    do {
      bit_word |= *bit_ptr++;
      if (bit_word) goto L_BitScan_Init;
      x_off += kPixelsPerBitWord;
    } while (bit_ptr != bit_ptr_end);
  } while (--y);
}

/* ============================================================================================
 * Gradient LUTs
 * ============================================================================================ */

typedef struct { double offset; uint64_t rgba; } OStop;

static inline uint32_t rgba32_from_rgba64(uint64_t v) {
  uint32_t b = (uint32_t)(v >> 8) & 0xFFu, g = (uint32_t)(v >> 24) & 0xFFu;
  uint32_t r = (uint32_t)(v >> 40) & 0xFFu, a = (uint32_t)(v >> 56) & 0xFFu;
  return (a << 24) | (r << 16) | (g << 8) | b;
}

/* div255_u16 of the x86 SIMD layer: ((x + 0x80) * 0x101) >> 16 on a 16-bit lane. */
static inline uint32_t simd_div255(uint32_t x) { return (((x + 0x80u) & 0xFFFFu) * 0x101u) >> 16; }
static inline uint32_t sat_u8(uint32_t v) { return v > 255u ? 255u : v; }

/* Premultiply of an 8-bit [b g r a] lane set the way the SSE2/AVX2 builders do:
 * div255((c | a255) * a) -> [b*a, g*a, r*a, 255*a]. */
static inline uint32_t simd_premul_ok(uint32_t c32) {
  uint32_t a = c32 >> 24;
  uint32_t b = simd_div255((c32 & 255u) * a), g = simd_div255(((c32 >> 8) & 255u) * a);
  uint32_t r = simd_div255(((c32 >> 16) & 255u) * a), aa = simd_div255(255u * a);
  return (sat_u8(aa) << 24) | (sat_u8(r) << 16) | (sat_u8(g) << 8) | sat_u8(b);
}
/* The AVX2 builder's 1-2 entry spans compute `c | (a255 * a)` (operator precedence,
 * interpolation_avx2.cpp:56): colour lanes are div255(c), the alpha lane div255(a | 255*a). */
static inline uint32_t avx2_premul_bug(uint32_t c32) {
  uint32_t a = c32 >> 24;
  uint32_t b = simd_div255(c32 & 255u), g = simd_div255((c32 >> 8) & 255u), r = simd_div255((c32 >> 16) & 255u);
  uint32_t aa = simd_div255(a | (255u * a));
  return (sat_u8(aa) << 24) | (sat_u8(r) << 16) | (sat_u8(g) << 8) | sat_u8(b);
}

static void lut_simd(uint32_t* d, uint32_t d_size, const OStop* s, size_t s_size, int avx2) {
  uint32_t* span = d;
  uint32_t c0 = rgba32_from_rgba64(s[0].rgba), c1;
  uint32_t u0 = 0, u1, i;
  size_t si = (size_t)(s[0].offset == 0.0 && s_size > 1);
  d_size--;
  double fWidth = (double)((int32_t)d_size << 8);
  do {
    c1 = rgba32_from_rgba64(s[si].rgba);
    u1 = (uint32_t)o_round_to_int(s[si].offset * fWidth);
    span = d + (u0 >> 8);
    i = (u1 >> 8) - (u0 >> 8);
    u0 = u1;
    if (i <= 1) {
      uint32_t p0 = avx2 ? avx2_premul_bug(c0) : simd_premul_ok(c0);
      uint32_t p1 = avx2 ? avx2_premul_bug(c1) : simd_premul_ok(c1);
      c0 = c1;
      *span++ = p0;
      if (i == 0) continue;
      *span++ = p1;
    }
    else {
      uint32_t n = i + 1;
      double scale = (double)(1 << 23) / (double)(int)i;
      int32_t cx[4], dx[4];
      for (int k = 0; k < 4; k++) {
        int32_t cc = (int32_t)((c0 >> (8 * k)) & 255u);
        int32_t dd = (int32_t)((c1 >> (8 * k)) & 255u) - cc;
        dx[k] = o_trunc_to_int((double)dd * scale);
        cx[k] = (int32_t)((uint32_t)cc << 23) + (1 << 22);
      }
      for (uint32_t j = 0; j < n; j++) {
        uint32_t v[4];
        for (int k = 0; k < 4; k++) v[k] = (uint32_t)(cx[k] + (int32_t)((uint32_t)dx[k] * j)) >> 23;
        uint32_t a = v[3];
        uint32_t b = simd_div255(v[0] * a), g = simd_div255(v[1] * a), r = simd_div255(v[2] * a), aa = simd_div255(255u * a);
        *span++ = (sat_u8(aa) << 24) | (sat_u8(r) << 16) | (sat_u8(g) << 8) | sat_u8(b);
      }
      c0 = c1;
    }
  } while (++si < s_size);

  i = (uint32_t)((d + d_size + 1) - span);
  uint32_t last = simd_premul_ok(c0);
  uint32_t first = simd_premul_ok(rgba32_from_rgba64(s[0].rgba));
  while (i--) *span++ = last;
  d[0] = first;
}

static inline uint32_t scalar_premul(uint32_t c) {  /* scalar_p.h:134-145 (non-SIMD) */
  uint32_t a = c >> 24;
  uint32_t v = c | 0xFF000000u;
  uint32_t rb = v & 0x00FF00FFu, ag = (v >> 8) & 0x00FF00FFu;
  rb = rb * a + 0x00800080u;
  ag = ag * a + 0x00800080u;
  rb = (rb + ((rb >> 8) & 0x00FF00FFu)) & 0xFF00FF00u;
  ag = (ag + ((ag >> 8) & 0x00FF00FFu)) & 0xFF00FF00u;
  return ag | (rb >> 8);
}

static void lut_scalar(uint32_t* d, uint32_t d_size, const OStop* s, size_t s_size) {
  uint32_t* span = d;
  uint32_t i = d_size;
  uint32_t c0 = rgba32_from_rgba64(s[0].rgba), c1 = c0;
  uint32_t p0 = 0, p1;
  size_t si = 0;
  d_size--;
  double fWidth = (double)((int32_t)d_size << 8);
  uint32_t cp = scalar_premul(c0);
  uint32_t cp_first = cp;

  if (s_size == 1) goto SolidLoop;

  do {
    c1 = rgba32_from_rgba64(s[si].rgba);
    p1 = (uint32_t)o_round_to_int(s[si].offset * fWidth);
    span = d + (p0 >> 8);
    i = (p1 >> 8) - (p0 >> 8);
    if (i == 0) c0 = c1;
    p0 = p1;
    i++;
SolidInit:
    cp = scalar_premul(c0);
    if (c0 == c1) {
SolidLoop:
      do { *span++ = cp; } while (--i);
    }
    else {
      *span++ = cp;
      if (--i) {
        const uint32_t kMask = 0xFFu << 23;
        uint32_t r_pos = (c0 << 7) & kMask, g_pos = (c0 << 15) & kMask, b_pos = (c0 << 23) & kMask;
        uint32_t r_inc = (c1 << 7) & kMask, g_inc = (c1 << 15) & kMask, b_inc = (c1 << 23) & kMask;
        r_inc = (uint32_t)((int32_t)(r_inc - r_pos) / (int32_t)i);
        g_inc = (uint32_t)((int32_t)(g_inc - g_pos) / (int32_t)i);
        b_inc = (uint32_t)((int32_t)(b_inc - b_pos) / (int32_t)i);
        r_pos += 1u << 22; g_pos += 1u << 22; b_pos += 1u << 22;
        if (((c0 & c1) >> 24) == 0xFFu) {
          do {
            r_pos += r_inc; g_pos += g_inc; b_pos += b_inc;
            cp = 0xFF000000u + ((r_pos & kMask) >> 7) + ((g_pos & kMask) >> 15) + ((b_pos & kMask) >> 23);
            *span++ = cp;
          } while (--i);
        }
        else {
          uint32_t a_pos = (c0 >> 1) & kMask, a_inc = (c1 >> 1) & kMask;
          a_inc = (uint32_t)((int32_t)(a_inc - a_pos) / (int32_t)i);
          a_pos += 1u << 22;
          do {
            a_pos += a_inc; r_pos += r_inc; g_pos += g_inc; b_pos += b_inc;
            uint32_t ca, cg;
            cp = ((b_pos & kMask) >> 23) + ((r_pos & kMask) >> 7);
            ca = ((a_pos & kMask) >> 23);
            cg = ((g_pos & kMask) >> 23);
            cp = (cp * ca) + 0x00800080u;
            cg = (cg * ca) + 0x00000080u;
            ca <<= 24;
            cp = ((cp + ((cp & 0xFF00FF00u) >> 8)) & 0xFF00FF00u) >> 8;
            cg = ((cg + ((cg & 0xFF00FF00u) >> 8)) & 0xFF00FF00u);
            cp += cg + ca;
            *span++ = cp;
          } while (--i);
        }
      }
      c0 = c1;
    }
  } while (++si < s_size);

  i = (uint32_t)((d + d_size + 1) - span);
  if (i != 0) goto SolidInit;
  d[0] = cp_first;
}

/* Scalar::udiv65535 and cvt_prgb64_8888_from_argb64_8888 (scalar_p.h:37, :179-222): every
 * channel of an RGBA64 colour times its alpha, divided by 65535 with rounding. */
static inline uint32_t udiv65535(uint32_t x) { return ((x + 0x8000u) + ((x + 0x8000u) >> 16)) >> 16; }
static inline uint64_t premul64(uint64_t c) {
  uint32_t a = (uint32_t)(c >> 48);
  uint32_t r = udiv65535(((uint32_t)(c >> 32) & 0xFFFFu) * a);
  uint32_t g = udiv65535(((uint32_t)(c >> 16) & 0xFFFFu) * a);
  uint32_t b = udiv65535(((uint32_t)c & 0xFFFFu) * a);
  return ((uint64_t)a << 48) | ((uint64_t)r << 32) | ((uint64_t)g << 16) | b;
}

/* interpolate_prgb64 (interpolation.cpp:161-288). */
void b2d_oracle_build_lut64(uint64_t* d, uint32_t d_size, const void* stops, size_t s_size) {
  const OStop* s = (const OStop*)stops;
  if (!o_dither_ready) o_dither_init();
  uint64_t* span = d;
  uint32_t i = d_size;
  uint64_t c0 = s[0].rgba, c1 = c0;
  uint32_t p0 = 0, p1;
  size_t si = 0;
  d_size--;
  double fWidth = (double)((int32_t)d_size << 8);
  uint64_t cp = premul64(c0);
  uint64_t cp_first = cp;

  if (s_size == 1) goto SolidLoop;

  do {
    c1 = s[si].rgba;
    p1 = (uint32_t)o_round_to_int(s[si].offset * fWidth);
    span = d + (p0 >> 8);
    i = (p1 >> 8) - (p0 >> 8);
    if (i == 0) c0 = c1;
    p0 = p1;
    i++;
SolidInit:
    cp = premul64(c0);
    if (c0 == c1) {
SolidLoop:
      do { *span++ = cp; } while (--i);
    }
    else {
      *span++ = cp;
      if (--i) {
        const uint32_t kShift = 15, kMask = 0xFFFFu << 15;
        uint32_t r_pos = (uint32_t)((c0 >> (32 - kShift)) & kMask);
        uint32_t g_pos = (uint32_t)((c0 >> (16 - kShift)) & kMask);
        uint32_t b_pos = (uint32_t)((c0 << kShift) & kMask);
        uint32_t r_inc = (uint32_t)((c1 >> (32 - kShift)) & kMask);
        uint32_t g_inc = (uint32_t)((c1 >> (16 - kShift)) & kMask);
        uint32_t b_inc = (uint32_t)((c1 << kShift) & kMask);
        r_inc = (uint32_t)((int32_t)(r_inc - r_pos) / (int32_t)i);
        g_inc = (uint32_t)((int32_t)(g_inc - g_pos) / (int32_t)i);
        b_inc = (uint32_t)((int32_t)(b_inc - b_pos) / (int32_t)i);
        r_pos += 1u << (kShift - 1); g_pos += 1u << (kShift - 1); b_pos += 1u << (kShift - 1);
        if (((c0 & c1) & 0xFFFF000000000000ull) == 0xFFFF000000000000ull) {
          do {
            r_pos += r_inc; g_pos += g_inc; b_pos += b_inc;
            cp = ((uint64_t)(r_pos & kMask) << (32 - kShift)) | ((uint64_t)(g_pos & kMask) << (16 - kShift)) |
                 ((uint64_t)(b_pos & kMask) >> kShift) | 0xFFFF000000000000ull;
            *span++ = cp;
          } while (--i);
        }
        else {
          uint32_t a_pos = (uint32_t)((c0 >> (48 - kShift)) & kMask);
          uint32_t a_inc = (uint32_t)((c1 >> (48 - kShift)) & kMask);
          a_inc = (uint32_t)((int32_t)(a_inc - a_pos) / (int32_t)i);
          a_pos += 1u << (kShift - 1);
          do {
            a_pos += a_inc; r_pos += r_inc; g_pos += g_inc; b_pos += b_inc;
            uint32_t ca = a_pos >> kShift;
            uint32_t cr = udiv65535((r_pos >> kShift) * ca);
            uint32_t cg = udiv65535((g_pos >> kShift) * ca);
            uint32_t cb = udiv65535((b_pos >> kShift) * ca);
            cp = ((uint64_t)ca << 48) | ((uint64_t)cr << 32) | ((uint64_t)cg << 16) | cb;
            *span++ = cp;
          } while (--i);
        }
      }
      c0 = c1;
    }
  } while (++si < s_size);

  i = (uint32_t)((d + d_size + 1) - span);
  if (i != 0) goto SolidInit;
  d[0] = cp_first;
}

void b2d_oracle_build_lut(uint32_t* lut, uint32_t lut_size, const void* stops, size_t n, uint32_t variant) {
  const OStop* s = (const OStop*)stops;
  if (variant == B2D_ORACLE_LUT_SCALAR) lut_scalar(lut, lut_size, s, n);
  else lut_simd(lut, lut_size, s, n, variant == B2D_ORACLE_LUT_AVX2);
}
