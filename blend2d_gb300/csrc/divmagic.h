// divmagic.h - signed 32-bit division and remainder by a divisor fixed per style, through a
// multiply-high with a precomputed magic number (Warren, "Hacker's Delight", section 10-1: signed
// division by constants). Exact for every int32 dividend, with C's truncating semantics, so it
// replaces `n % d` bit for bit while keeping the per-pixel remainder off the slow division path.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define BLGPU_HD __host__ __device__ __forceinline__
#else
#define BLGPU_HD inline
#endif

namespace blgpu {

struct DivMagic {
  int32_t m;       // magic multiplier
  int32_t s;       // post-shift; -1: the divisor is 1 (remainder 0)
};

// Magic number and shift for a divisor d >= 1.
inline DivMagic div_magic(int32_t d) {
  if (d == 1) return DivMagic{0, -1};
  const uint32_t two31 = 0x80000000u;
  const uint32_t ad = uint32_t(d);
  const uint32_t anc = two31 - 1u - two31 % ad;    // |nc|
  int p = 31;
  uint32_t q1 = two31 / anc, r1 = two31 - q1 * anc;
  uint32_t q2 = two31 / ad, r2 = two31 - q2 * ad;
  uint32_t delta;
  do {
    p++;
    q1 *= 2u; r1 *= 2u;
    if (r1 >= anc) { q1++; r1 -= anc; }
    q2 *= 2u; r2 *= 2u;
    if (r2 >= ad) { q2++; r2 -= ad; }
    delta = ad - r2;
  } while (q1 < delta || (q1 == delta && r1 == 0));
  return DivMagic{int32_t(q2 + 1u), p - 32};
}

BLGPU_HD int32_t mulhi_s32(int32_t a, int32_t b) {
#if defined(__CUDA_ARCH__)
  return __mulhi(a, b);
#else
  return int32_t((int64_t(a) * int64_t(b)) >> 32);
#endif
}

// n % d (C semantics) for d >= 1 with dm = div_magic(d).
BLGPU_HD int32_t smod_magic(int32_t n, int32_t d, DivMagic dm) {
  if (dm.s < 0) return 0;
  int32_t q = mulhi_s32(dm.m, n);
  if (dm.m < 0) q += n;
  q >>= dm.s;
  q += int32_t(uint32_t(n) >> 31);
  return int32_t(uint32_t(n) - uint32_t(q) * uint32_t(d));
}

}  // namespace blgpu
