// Host check of smod_magic (divmagic.h) against the % operator: edge divisors and dividends plus
// random ones. Exit status 0 when every remainder matches.
#include <cstdint>
#include <cstdio>
#include <random>
#include "divmagic.h"

int main() {
  using namespace blgpu;
  std::mt19937_64 rng(12345);
  const int32_t divisors[] = {1, 2, 3, 5, 6, 7, 9, 10, 16, 100, 255, 256, 257, 511, 512, 640, 1000, 1024, 4096,
                              65535, 65536, 65537, 1 << 20, 1 << 30, 2147483646, 2147483647};
  const int32_t edges[] = {0, 1, -1, 2, -2, INT32_MAX, INT32_MIN, INT32_MIN + 1, INT32_MAX - 1, 255, -255, 256, -256};
  long bad = 0, n_checked = 0;
  auto check = [&](int32_t n, int32_t d, DivMagic dm) {
    n_checked++;
    if (smod_magic(n, d, dm) != n % d) {
      if (++bad <= 5) printf("mismatch: %d %% %d: %d vs %d\n", n, d, smod_magic(n, d, dm), n % d);
    }
  };
  for (int32_t d : divisors) {
    const DivMagic dm = div_magic(d);
    for (int32_t n : edges) check(n, d, dm);
    for (int i = 0; i < 200000; i++) check(int32_t(uint32_t(rng())), d, dm);
    for (int i = -3000; i <= 3000; i++) check(i, d, dm);
  }
  for (int k = 0; k < 2000; k++) {
    const int32_t d = int32_t(1 + rng() % (k < 1000 ? 5000 : 2147483646u));
    const DivMagic dm = div_magic(d);
    for (int32_t n : edges) check(n, d, dm);
    for (int i = 0; i < 2000; i++) check(int32_t(uint32_t(rng())), d, dm);
  }
  printf("checked %ld remainders, %ld mismatches\n", n_checked, bad);
  return bad ? 1 : 0;
}
