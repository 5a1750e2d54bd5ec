// ref_raster.cpp - analytic-rasterizer known answers from the reference's own rasterizer
// (blend2d/raster/analyticrasterizer_p.h), driven band by band like CommandProcSync::fill_analytic
// and like the reference's unit test (blend2d/raster/analyticrasterizer_test.cpp:34-155).
// Test infrastructure, built by oracle/ref.mk.
//
// stdin : lines "width rows band_height x0 y0 x1 y1 sign" (24.8 fixed-point line, y0 < y1)
// stdout: per line the dense cell grid [rows x (width+2)] as one hex string of u32 (row-major)
#include <blend2d/core/api-build_p.h>
#include <blend2d/pipeline/pipedefs_p.h>
#include <blend2d/raster/analyticrasterizer_p.h>
#include <blend2d/support/intops_p.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace bl;
using namespace bl::RasterEngine;

int main() {
  int w, rows, x0, y0, x1, y1;
  unsigned bh, sign;
  while (scanf("%d %d %u %d %d %d %d %u", &w, &rows, &bh, &x0, &y0, &x1, &y1, &sign) == 8) {
    size_t required_width = IntOps::align_up(uint32_t(w) + 1u + BL_PIPE_PIXELS_PER_ONE_BIT, BL_PIPE_PIXELS_PER_ONE_BIT);
    size_t bit_stride = IntOps::word_count_from_bit_count<BLBitWord>(required_width / BL_PIPE_PIXELS_PER_ONE_BIT) * sizeof(BLBitWord);
    size_t cell_stride = required_width * sizeof(uint32_t);
    std::vector<BLBitWord> bits(bh * bit_stride / sizeof(BLBitWord) + 8, 0);
    std::vector<uint32_t> cells(bh * required_width + 16, 0);
    std::vector<uint32_t> grid(size_t(rows) * size_t(w + 2), 0);

    uint32_t y_start = uint32_t(y0 >> 8);
    uint32_t y_end = uint32_t((y1 + 255) >> 8);
    uint32_t band = y_start / bh;

    AnalyticRasterizer ras;
    ras.init(bits.data(), bit_stride, cells.data(), cell_stride, band * bh, bh);
    ras._band_offset = y_start;
    ras.set_sign_mask_from_bit(sign);
    bool prepared = ras.prepare(EdgePoint<int>{x0, y0}, EdgePoint<int>{x1, y1});
    bool done = !prepared;
    while (!done) {
      ras._band_end = bl_min((band + 1) * bh, y_end) - 1;
      if (uint32_t(ras._ey0) <= ras._band_end)
        done = ras.template rasterize<AnalyticRasterizer::kOptionBandOffset | AnalyticRasterizer::kOptionBandingMode>();
      for (uint32_t r = 0; r < bh; r++) {
        uint32_t y = ras._band_offset + r;
        for (int x = 0; x < w + 2; x++) {
          if (y < uint32_t(rows)) grid[size_t(y) * size_t(w + 2) + size_t(x)] += cells[r * required_width + size_t(x)];
        }
      }
      std::fill(cells.begin(), cells.end(), 0u);
      std::fill(bits.begin(), bits.end(), BLBitWord(0));
      ras._band_offset = (band + 1) * bh;
      band++;
      if (ras._band_offset >= y_end) break;
    }
    for (uint32_t v : grid) printf("%08x", v);
    printf("\n");
  }
  return 0;
}
