/* b2d_oracle_render - CLI around the CPU oracle (test infrastructure): renders a command stream
 * and writes raw PRGB32 pixels; with --frames K prints the median frame time as JSON. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "b2d_oracle.h"
#include "blgpu_stream.h"

static double now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}
static int cmp_d(const void* a, const void* b) {
  double x = *(const double*)a, y = *(const double*)b;
  return x < y ? -1 : x > y;
}

int main(int argc, char** argv) {
  if (argc < 3) { fprintf(stderr, "usage: %s stream.bin out.raw|- [--frames K] [--lut avx2|sse2|scalar]\n", argv[0]); return 2; }
  int frames = 0;
  B2DOracleOptions opt;
  memset(&opt, 0, sizeof(opt));
  for (int i = 3; i + 1 < argc; i += 2) {
    if (!strcmp(argv[i], "--frames")) frames = atoi(argv[i + 1]);
    else if (!strcmp(argv[i], "--lut")) opt.lut_variant = !strcmp(argv[i + 1], "avx2") ? B2D_ORACLE_LUT_AVX2 : (!strcmp(argv[i + 1], "scalar") ? B2D_ORACLE_LUT_SCALAR : B2D_ORACLE_LUT_SSE2);
  }
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 2;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  unsigned char* buf = (unsigned char*)malloc((size_t)n);
  if (fread(buf, 1, (size_t)n, f) != (size_t)n) return 2;
  fclose(f);
  BLGpuStreamHeader hdr;
  memcpy(&hdr, buf, sizeof(hdr));
  uint32_t* px = (uint32_t*)malloc((size_t)hdr.width * hdr.height * 4u);
  B2DOracleStats st;
  int rc = b2d_oracle_render(buf, (size_t)n, px, &opt, &st);
  if (rc) { fprintf(stderr, "render failed %d\n", rc); return 1; }
  if (frames > 0) {
    double* ms = (double*)malloc(sizeof(double) * (size_t)frames);
    for (int k = 0; k < frames; k++) { double t0 = now_ms(); b2d_oracle_render(buf, (size_t)n, px, &opt, NULL); ms[k] = now_ms() - t0; }
    qsort(ms, (size_t)frames, sizeof(double), cmp_d);
    printf("{\"frames\": %d, \"median_ms\": %.4f, \"min_ms\": %.4f, \"composited_pixels\": %llu, \"fill_calls\": %llu}\n",
           frames, ms[frames / 2], ms[0], (unsigned long long)st.composited_pixels, (unsigned long long)st.fill_calls);
  }
  if (strcmp(argv[2], "-")) { FILE* o = fopen(argv[2], "wb"); fwrite(px, 4, (size_t)hdr.width * hdr.height, o); fclose(o); }
  return 0;
}
