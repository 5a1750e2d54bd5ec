// ref_lut.cpp - gradient-LUT known answers from the reference's three builders
// (blend2d/pixelops/interpolation.cpp, interpolation_sse2.cpp, interpolation_avx2.cpp), called
// directly. Test infrastructure, built by oracle/ref.mk.
//
// stdin : lines "lut_size n off0 rgba64_0 off1 rgba64_1 ..." (offsets as %a hex floats)
// stdout: per line "scalar-hex sse2-hex avx2-hex" (each the LUT as packed little-endian hex)
#include <blend2d/blend2d.h>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <vector>

namespace bl { namespace PixelOps { namespace Interpolation {
void interpolate_prgb32(uint32_t*, uint32_t, const BLGradientStop*, size_t) noexcept;
void interpolate_prgb32_sse2(uint32_t*, uint32_t, const BLGradientStop*, size_t) noexcept;
void interpolate_prgb32_avx2(uint32_t*, uint32_t, const BLGradientStop*, size_t) noexcept;
}}}

static void dump(const std::vector<uint32_t>& v) {
  for (uint32_t x : v) printf("%08x", x);
}

int main() {
  unsigned lut_size, n;
  while (scanf("%u %u", &lut_size, &n) == 2) {
    std::vector<BLGradientStop> stops(n);
    for (unsigned i = 0; i < n; i++) {
      double off; unsigned long long c;
      if (scanf("%la %llx", &off, &c) != 2) return 2;
      stops[i] = BLGradientStop(off, BLRgba64(uint64_t(c)));
    }
    std::vector<uint32_t> a(lut_size), b(lut_size), c(lut_size);
    bl::PixelOps::Interpolation::interpolate_prgb32(a.data(), lut_size, stops.data(), n);
    bl::PixelOps::Interpolation::interpolate_prgb32_sse2(b.data(), lut_size, stops.data(), n);
    bl::PixelOps::Interpolation::interpolate_prgb32_avx2(c.data(), lut_size, stops.data(), n);
    dump(a); printf(" "); dump(b); printf(" "); dump(c); printf("\n");
  }
  return 0;
}
