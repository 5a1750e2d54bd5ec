// raster.cuh - the reference's analytic cell rasterizer, run per (segment, window of rows).
//
// The cell values come from the reference's integer DDA (AnalyticRasterizer::prepare_ref,
// advanceToY and rasterize<kOptionBandingMode>, blend2d/raster/analyticrasterizer_p.h:289-1166):
// cell[x] += (cover << 9) - area, cell[x+1] += area, with the same error accumulators. A window of
// rows is one rasterizer band: a segment that starts above it is jumped to the window's first row
// with advanceToY (the reference's own unit test pins advanceToY to the banded state), then
// rasterized in banding mode for the window's rows. Cells left of the window are summed into a
// per-row backdrop (the coverage carried in from the left), cells right of it are dropped. All sums
// are modular u32, so the per-window partial sums equal the reference's band sums.
#pragma once

#include "blgpu_internal.h"

namespace blgpu {
namespace ras {

enum : uint32_t { kInitial = 1, kVertOrSingle = 2, kRTL = 4 };

struct State {
  int ex0, ey0, ex1, ey1, fx0, fy0, fx1, fy1;
  int xErr, yErr, xDlt, yDlt, xRem, yRem, xLift, yLift;
  int dx, dy, savedFy1;
  uint32_t flags;
};

// Destination of cell contributions for one window of `kWindowRows` rows x kTileW columns:
// shared-memory cells plus a per-row backdrop that receives every contribution left of it.
struct WindowSink {
  uint32_t* cells;
  uint32_t* backdrop;
  int tx0;
  __device__ __forceinline__ void add(int row, int x, uint32_t v) {
    int cx = x - tx0;
    if (cx < 0) atomicAdd(&backdrop[row], v);
    else if (cx < kTileW) atomicAdd(&cells[row * kTileW + cx], v);
  }
  __device__ __forceinline__ void merge(int row, int x, uint32_t cover, uint32_t area) {
    add(row, x, (cover << 9) - area);
    add(row, x + 1, area);
  }
};

__device__ __forceinline__ void acc_step(int& acc, int& iter, int step, int corr) {
  iter -= step;
  int m = iter >> 31;
  acc -= m;
  iter += m & corr;
}
__device__ __forceinline__ void acc_step_u(uint32_t& acc, int& iter, int step, int corr) {
  iter -= step;
  int m = iter >> 31;
  acc -= uint32_t(m);
  iter += m & corr;
}
// 64-by-32-bit unsigned division with a 32-bit fast path (the common case: short segments).
__device__ __forceinline__ uint64_t udiv64(uint64_t n, uint32_t d) {
  if ((n >> 32) == 0) return uint32_t(n) / d;
  return n / d;
}
__device__ __forceinline__ uint64_t umod64(uint64_t n, uint32_t d) {
  if ((n >> 32) == 0) return uint32_t(n) % d;
  return n % d;
}

__device__ __forceinline__ void acc_multi_step(int& acc, int& iter, int step, int corr, int count) {
  int64_t i = int64_t(uint32_t(iter));
  i -= int64_t(uint64_t(uint32_t(step)) * uint32_t(count));
  if (i < 0) {
    int n = int(udiv64(uint64_t(-i) + uint32_t(corr) - 1u, uint32_t(corr)));
    acc += n;
    i += int64_t(corr) * n;
  }
  iter = int(i);
}

__device__ bool prepare(State& s, int x0, int y0, int x1, int y1) {
  if (y0 == y1) return false;
  s.dx = x1 - x0;
  s.dy = y1 - y0;
  s.flags = kInitial;
  if (s.dx < 0) { s.flags |= kRTL; s.dx = -s.dx; }
  s.ex0 = x0 >> 8; s.ey0 = y0 >> 8; s.ex1 = x1 >> 8; s.ey1 = (y1 - 1) >> 8;
  s.fx0 = x0 & 255; s.fy0 = y0 & 255; s.fx1 = x1 & 255; s.fy1 = ((y1 - 1) & 255) + 1;
  s.savedFy1 = s.fy1;
  s.xErr = s.yErr = s.xDlt = s.yDlt = s.xRem = s.yRem = s.xLift = s.yLift = 0;
  if (s.ey0 != s.ey1) s.fy1 = 256;
  if (s.ex0 == s.ex1 && (s.ey0 == s.ey1 || s.dx == 0)) { s.flags |= kVertOrSingle; return true; }
  uint64_t xb = uint64_t(uint32_t(s.dx)) * 256u;
  uint64_t yb = uint64_t(uint32_t(s.dy)) * 256u;
  s.xLift = int(udiv64(xb, unsigned(s.dy))); s.xRem = int(umod64(xb, unsigned(s.dy)));
  s.yLift = int(udiv64(yb, unsigned(s.dx))); s.yRem = int(umod64(yb, unsigned(s.dx)));
  s.xDlt = s.dx; s.yDlt = s.dy;
  s.xErr = (s.dy >> 1) - 1;
  s.yErr = (s.dx >> 1) - 1;
  if (s.ey0 != s.ey1) {
    uint64_t p = uint64_t(256u - uint32_t(s.fy0)) * uint32_t(s.dx);
    s.xDlt = int(udiv64(p, unsigned(s.dy)));
    s.xErr -= int(umod64(p, unsigned(s.dy)));
    acc_step(s.xDlt, s.xErr, 0, s.dy);
  }
  if (s.ex0 != s.ex1) {
    uint64_t p = uint64_t((s.flags & kRTL) ? uint32_t(s.fx0) : 256u - uint32_t(s.fx0)) * uint32_t(s.dy);
    s.yDlt = int(udiv64(p, unsigned(s.dx)));
    s.yErr -= int(umod64(p, unsigned(s.dx)));
    acc_step(s.yDlt, s.yErr, 0, s.dx);
  }
  s.yDlt += s.fy0;
  return true;
}

__device__ void advance_to_y(State& s, int y_target) {
  if (y_target <= s.ey0) return;
  if (!(s.flags & kVertOrSingle)) {
    int ny = y_target - s.ey0;
    s.xDlt += s.xLift * (ny - 1);
    acc_multi_step(s.xDlt, s.xErr, s.xRem, s.dy, ny - 1);
    if (s.flags & kRTL) {
      s.fx0 -= s.xDlt;
      if (s.fx0 < 0) {
        int nx = -(s.fx0 >> 8);
        s.ex0 -= nx;
        s.fx0 &= 255;
        acc_multi_step(s.yDlt, s.yErr, s.yRem, s.dx, nx);
        s.yDlt += s.yLift * nx;
      }
      if (!(s.dy >= s.dx)) {
        if (!s.fx0) {
          s.fx0 = 256;
          s.ex0--;
          acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
          s.yDlt += s.yLift;
        }
      }
      if (y_target == s.ey1 && s.dy >= s.dx) {
        s.fy1 = s.savedFy1;
        s.xDlt = ((s.ex0 - s.ex1) << 8) + s.fx0 - s.fx1;
      }
      else {
        s.xDlt = s.xLift;
        acc_step(s.xDlt, s.xErr, s.xRem, s.dy);
      }
    }
    else {
      s.fx0 += s.xDlt;
      if (s.fx0 >= 256) {
        int nx = s.fx0 >> 8;
        s.ex0 += nx;
        s.fx0 &= 255;
        acc_multi_step(s.yDlt, s.yErr, s.yRem, s.dx, nx);
        s.yDlt += s.yLift * nx;
      }
      if (y_target == s.ey1 && s.dy >= s.dx) {
        s.fy1 = s.savedFy1;
        s.xDlt = ((s.ex1 - s.ex0) << 8) + s.fx1 - s.fx0;
      }
      else {
        s.xDlt = s.xLift;
        acc_step(s.xDlt, s.xErr, s.xRem, s.dy);
      }
    }
    if (s.dy >= s.dx) s.yDlt &= 255;
    else {
      int y = ny;
      if (s.flags & kInitial) y--;
      s.yDlt -= y * 256;
    }
  }
  else {
    if (y_target == s.ey1) s.fy1 = s.savedFy1;
  }
  s.fy0 = 0;
  s.ey0 = y_target;
  s.flags &= ~uint32_t(kInitial);
}

// rasterize<kOptionBandOffset | kOptionBandingMode> for the band [band_offset, band_end].
__device__ void rasterize(State& s, uint32_t sm, uint32_t band_offset, uint32_t band_end, WindowSink& cs) {
  auto SM = [sm](uint32_t v) -> uint32_t { return (v ^ sm) - sm; };
  int ey1_end = min(s.ey1, int(band_end));
  uint32_t i = unsigned(ey1_end) - unsigned(s.ey0);
  int row = int(unsigned(s.ey0) - band_offset);
  s.ey0 += int(i) + 1;
  const uint32_t full_cover = SM(256u);

  if (s.flags & kVertOrSingle) {
    uint32_t area = uint32_t(s.fx0) + uint32_t(s.fx1);
    uint32_t cover = SM(uint32_t(s.fy1 - s.fy0));
    cs.merge(row, s.ex0, cover, cover * area);
    if (!i) {
      if (s.ey0 > s.ey1) return;
      s.fy0 = 0;
      s.fy1 = s.ey0 == s.ey1 ? s.savedFy1 : 256;
      return;
    }
    row++;
    cover = full_cover;
    while (--i) { cs.merge(row, s.ex0, cover, cover * area); row++; }
    if (s.ey0 <= s.ey1) {
      cs.merge(row, s.ex0, cover, cover * area);
      s.fy0 = 0;
      s.fy1 = s.ey0 == s.ey1 ? s.savedFy1 : 256;
      return;
    }
    cover = SM(uint32_t(s.savedFy1));
    cs.merge(row, s.ex0, cover, cover * area);
    return;
  }
  else if (s.dy >= s.dx) {
    i += (s.ey0 <= s.ey1);
    if (s.flags & kRTL) {
      for (;;) {
        uint32_t area = uint32_t(s.fx0);
        uint32_t cov0, cov1;
        s.fx0 -= s.xDlt;
        if (s.fx0 < 0) {
          s.ex0--;
          s.fx0 += 256;
          s.yDlt &= 255;
          if (!area) {
            area = 256;
            acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
            s.yDlt += s.yLift;
            goto VRTLFirst;
          }
          cov0 = SM(uint32_t(s.yDlt - s.fy0));
          area = cov0 * area;
          cs.merge(row, s.ex0 + 1, cov0, area);
          cov0 = SM(uint32_t(s.fy1 - s.yDlt));
          area = cov0 * (uint32_t(s.fx0) + 256u);
          cs.merge(row, s.ex0, cov0, area);
          acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
          s.yDlt += s.yLift;
        }
        else {
VRTLFirst:
          cov0 = SM(uint32_t(s.fy1 - s.fy0));
          area = cov0 * (area + uint32_t(s.fx0));
          cs.merge(row, s.ex0, cov0, area);
        }
        s.fy0 = 0;
        row++;
        if (!i) {
          if (s.ey0 > s.ey1) return;
          s.xDlt = s.xLift;
          acc_step(s.xDlt, s.xErr, s.xRem, s.dy);
          return;
        }
        while (--i) {
          s.xDlt = s.xLift;
          acc_step(s.xDlt, s.xErr, s.xRem, s.dy);
          area = uint32_t(s.fx0);
          s.fx0 -= s.xDlt;
          if (s.fx0 < 0) {
            s.ex0--;
            s.fx0 += 256;
            s.yDlt &= 255;
            if (!area) {
              area = 256;
              acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
              s.yDlt += s.yLift;
              goto VRTLInLoop;
            }
            cov1 = SM(uint32_t(s.yDlt));
            area = cov1 * area;
            cs.add(row, s.ex0 + 2, area);
            cov0 = full_cover - cov1;
            cov1 = (cov1 << 9) - area;
            area = cov0 * (uint32_t(s.fx0) + 256u);
            cov0 = (cov0 << 9) - area;
            cov1 = cov1 + area;
            cs.add(row, s.ex0 + 0, cov0);
            cs.add(row, s.ex0 + 1, cov1);
            row++;
            acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
            s.yDlt += s.yLift;
          }
          else {
VRTLInLoop:
            area = full_cover * (area + uint32_t(s.fx0));
            cs.merge(row, s.ex0, full_cover, area);
            row++;
          }
        }
        if (s.ey0 >= s.ey1) {
          s.fy1 = s.savedFy1;
          s.xDlt = ((s.ex0 - s.ex1) << 8) + s.fx0 - s.fx1;
          if (s.ey0 == s.ey1) return;
        }
        else {
          s.xDlt = s.xLift;
          acc_step(s.xDlt, s.xErr, s.xRem, s.dy);
          return;
        }
      }
    }
    else {
      for (;;) {
        uint32_t area = uint32_t(s.fx0);
        uint32_t cov0, cov1;
        s.fx0 += s.xDlt;
        if (s.fx0 <= 256) {
          cov0 = SM(uint32_t(s.fy1 - s.fy0));
          area = cov0 * (area + uint32_t(s.fx0));
          cs.merge(row, s.ex0, cov0, area);
          if (s.fx0 == 256) {
            s.ex0++;
            s.fx0 = 0;
            s.yDlt += s.yLift;
            acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
          }
        }
        else {
          s.ex0++;
          s.fx0 &= 255;
          s.yDlt &= 255;
          cov0 = SM(uint32_t(s.yDlt - s.fy0));
          area = cov0 * (area + 256u);
          cs.merge(row, s.ex0 - 1, cov0, area);
          cov0 = SM(uint32_t(s.fy1 - s.yDlt));
          area = cov0 * uint32_t(s.fx0);
          cs.merge(row, s.ex0, cov0, area);
          s.yDlt += s.yLift;
          acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
        }
        s.fy0 = 0;
        row++;
        if (!i) {
          if (s.ey0 > s.ey1) return;
          s.yDlt += s.yLift;
          acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
          return;
        }
        while (--i) {
          s.xDlt = s.xLift;
          acc_step(s.xDlt, s.xErr, s.xRem, s.dy);
          area = uint32_t(s.fx0);
          s.fx0 += s.xDlt;
          if (s.fx0 <= 256) {
            area = full_cover * (area + uint32_t(s.fx0));
            cs.merge(row, s.ex0, full_cover, area);
            row++;
            if (s.fx0 < 256) continue;
            s.ex0++;
            s.fx0 = 0;
          }
          else {
            s.fx0 &= 255;
            s.yDlt &= 255;
            cov0 = SM(uint32_t(s.yDlt));
            cov1 = cov0 * (area + 256u);
            cov0 = (cov0 << 9) - cov1;
            cs.add(row, s.ex0 + 0, cov0);
            s.ex0++;
            cov0 = SM(256u - uint32_t(s.yDlt));
            area = cov0 * uint32_t(s.fx0);
            cov0 = (cov0 << 9) - area + cov1;
            cs.add(row, s.ex0 + 0, cov0);
            cs.add(row, s.ex0 + 1, area);
            row++;
          }
          s.yDlt += s.yLift;
          acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
        }
        if (s.ey0 >= s.ey1) {
          s.fy1 = s.savedFy1;
          s.xDlt = ((s.ex1 - s.ex0) << 8) + s.fx1 - s.fx0;
          if (s.ey0 == s.ey1) return;
        }
        else {
          s.xDlt = s.xLift;
          acc_step(s.xDlt, s.xErr, s.xRem, s.dy);
          return;
        }
      }
    }
  }
  else {
    uint32_t j = 1;
    int x_local = (s.ex0 << 8) + s.fx0;
    uint32_t cover, area;
    if (s.flags & kRTL) {
      if (s.flags & kInitial) {
        s.flags &= ~uint32_t(kInitial);
        j = i;
        i = 1;
        cover = SM(uint32_t(s.yDlt - s.fy0));
        if (s.fx0 - s.xDlt < 0) goto HRTLInside;
        x_local -= s.xDlt;
        cover = SM(uint32_t(s.fy1 - s.fy0));
        area = cover * uint32_t(s.fx0 * 2 - s.xDlt);
        cs.merge(row, s.ex0, cover, area);
        if ((x_local & 255) == 0) {
          s.yDlt += s.yLift;
          acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
        }
        s.xDlt = s.xLift;
        acc_step(s.xDlt, s.xErr, s.xRem, s.dy);
        row++;
        i--;
      }
      for (;;) {
        while (i) {
          s.ex0 = ((x_local - 1) >> 8);
          s.fx0 = ((x_local - 1) & 255) + 1;
HRTLSkip:
          s.yDlt -= 256;
          cover = SM(uint32_t(s.yDlt));
HRTLInside:
          x_local -= s.xDlt;
          {
            int ex_local = x_local >> 8;
            int fx_local = x_local & 255;
            area = cover * uint32_t(s.fx0);
            while (s.ex0 != ex_local) {
              cs.merge(row, s.ex0, cover, area);
              cover = uint32_t(s.yLift);
              acc_step_u(cover, s.yErr, s.yRem, s.dx);
              s.yDlt += int32_t(cover);
              cover = SM(cover);
              area = cover * 256u;
              s.ex0--;
            }
            cover += SM(uint32_t(s.fy1 - s.yDlt));
            area = cover * (uint32_t(fx_local) + 256u);
            cs.merge(row, s.ex0, cover, area);
            if (fx_local == 0) {
              s.yDlt += s.yLift;
              acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
            }
          }
          s.xDlt = s.xLift;
          acc_step(s.xDlt, s.xErr, s.xRem, s.dy);
          row++;
          i--;
        }
        s.fy0 = 0;
        s.fy1 = 256;
        if (!j) {
          s.ex0 = ((x_local - 1) >> 8);
          s.fx0 = ((x_local - 1) & 255) + 1;
          return;
        }
        i = j - 1;
        j = 1;
        if (!i) {
          i = 1;
          j = 0;
          if (!(s.ey0 > s.ey1)) continue;
          s.xDlt = x_local - ((s.ex1 << 8) + s.fx1);
          s.fy1 = s.savedFy1;
          s.ex0 = ((x_local - 1) >> 8);
          s.fx0 = ((x_local - 1) & 255) + 1;
          if (s.fx0 - s.xDlt >= 0) {
            cover = SM(uint32_t(s.fy1));
            area = cover * uint32_t(s.fx0 * 2 - s.xDlt);
            cs.merge(row, s.ex0, cover, area);
            return;
          }
          goto HRTLSkip;
        }
      }
    }
    else {
      if (s.flags & kInitial) {
        s.flags &= ~uint32_t(kInitial);
        j = i;
        i = 1;
        cover = SM(uint32_t(s.yDlt - s.fy0));
        if (s.fx0 + s.xDlt > 256) goto HLTRInside;
        x_local += s.xDlt;
        cover = SM(uint32_t(s.fy1 - s.fy0));
        area = cover * (uint32_t(s.fx0) * 2u + uint32_t(s.xDlt));
        cs.merge(row, s.ex0, cover, area);
        if (s.fx0 + s.xDlt == 256) {
          s.yDlt += s.yLift;
          acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
        }
        s.xDlt = s.xLift;
        acc_step(s.xDlt, s.xErr, s.xRem, s.dy);
        row++;
        i--;
      }
      for (;;) {
        while (i) {
          s.ex0 = x_local >> 8;
          s.fx0 = x_local & 255;
HLTRSkip:
          s.yDlt -= 256;
          cover = SM(uint32_t(s.yDlt));
HLTRInside:
          x_local += s.xDlt;
          {
            int ex_local = (x_local - 1) >> 8;
            int fx_local = ((x_local - 1) & 255) + 1;
            area = cover * (uint32_t(s.fx0) + 256u);
            while (s.ex0 != ex_local) {
              cs.merge(row, s.ex0, cover, area);
              cover = uint32_t(s.yLift);
              acc_step_u(cover, s.yErr, s.yRem, s.dx);
              s.yDlt += int32_t(cover);
              cover = SM(cover);
              area = cover * 256u;
              s.ex0++;
            }
            cover += SM(uint32_t(s.fy1 - s.yDlt));
            area = cover * uint32_t(fx_local);
            cs.merge(row, s.ex0, cover, area);
            if (fx_local == 256) {
              s.yDlt += s.yLift;
              acc_step(s.yDlt, s.yErr, s.yRem, s.dx);
            }
          }
          s.xDlt = s.xLift;
          acc_step(s.xDlt, s.xErr, s.xRem, s.dy);
          row++;
          i--;
        }
        s.fy0 = 0;
        s.fy1 = 256;
        if (!j) {
          s.ex0 = x_local >> 8;
          s.fx0 = x_local & 255;
          return;
        }
        i = j - 1;
        j = 1;
        if (!i) {
          i = 1;
          j = 0;
          if (!(s.ey0 > s.ey1)) continue;
          s.xDlt = ((s.ex1 << 8) + s.fx1) - x_local;
          s.fy1 = s.savedFy1;
          s.ex0 = x_local >> 8;
          s.fx0 = x_local & 255;
          if (s.fx0 + s.xDlt <= 256) {
            cover = SM(uint32_t(s.fy1));
            area = cover * (uint32_t(s.fx0) * 2u + uint32_t(s.xDlt));
            cs.merge(row, s.ex0, cover, area);
            return;
          }
          goto HLTRSkip;
        }
      }
    }
  }
}

// All cells of one segment for the window rows [row0, row0 + rows) (clipped to `last_row`).
// Segments entirely left of the window only add their per-row cover (cells sum to cover << 9 per
// row, analyticrasterizer_p.h:1203-1211); segments right of it contribute nothing.
__device__ __forceinline__ void segment_to_window(const DevSeg& g, uint32_t sign, int row0, int rows, int last_row,
                                                  WindowSink& cs) {
  int ey0 = g.y0 >> 8;
  int ey1 = (g.y1 - 1) >> 8;
  int band_end = min(row0 + rows - 1, last_row);
  if (ey1 < row0 || ey0 > band_end) return;
  int min_x = min(g.x0, g.x1) >> 8;
  if (min_x >= cs.tx0 + kTileW) return;
  uint32_t sm = 0u - sign;
  int max_x = max(g.x0, g.x1) >> 8;
  if (max_x + 2 < cs.tx0) {
    int r0 = max(ey0, row0), r1 = min(ey1, band_end);
    for (int r = r0; r <= r1; r++) {
      int top = max(g.y0, r << 8);
      int bot = min(g.y1, (r + 1) << 8);
      uint32_t cov = (uint32_t(bot - top) ^ sm) - sm;
      atomicAdd(&cs.backdrop[r - row0], cov << 9);
    }
    return;
  }
  State s;
  if (!prepare(s, g.x0, g.y0, g.x1, g.y1)) return;
  if (s.ey0 < row0) advance_to_y(s, row0);
  rasterize(s, sm, uint32_t(row0), uint32_t(band_end), cs);
}

}  // namespace ras
}  // namespace blgpu
