/*
 * b2d_oracle.h - CPU oracle for the blgpu raster backend (TEST INFRASTRUCTURE ONLY).
 *
 * A sequential C restatement of the reference's synchronous fill pipeline (Blend2D fixed
 * pipeline: the raster, pipeline/reference and pixelops directories of blend2d). It replays a
 * command stream (include/blgpu_stream.h) and produces the PRGB32 pixels the reference would.
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use it, as the checker.
 */
#ifndef B2D_ORACLE_H_INCLUDED
#define B2D_ORACLE_H_INCLUDED

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Gradient LUT builder variant (blend2d/pixelops/funcs.cpp:22-34). A no-JIT x86-64 build of
 * the reference never detects CPU features (blend2d/core/runtime.cpp:127-180) and selects the
 * SSE2 builder; a no-JIT build on other hosts selects the portable one; AVX2 is what JIT builds
 * with runtime feature detection select on AVX2 machines. */
enum {
  B2D_ORACLE_LUT_SSE2 = 0,   /* interpolate_prgb32_sse2 (default) */
  B2D_ORACLE_LUT_AVX2 = 1,   /* interpolate_prgb32_avx2 */
  B2D_ORACLE_LUT_SCALAR = 2  /* interpolate_prgb32 (portable) */
};

typedef struct B2DOracleOptions {
  uint32_t lut_variant;      /* B2D_ORACLE_LUT_* */
  uint32_t band_height;      /* 0 = the reference's synchronous-context default for the width */
  uint32_t reserved[6];
} B2DOracleOptions;

typedef struct B2DOracleStats {
  uint64_t fill_calls;       /* fill records that reached the pipeline (not NOP) */
  uint64_t composited_pixels;/* pixels composited with a non-zero mask */
  uint64_t edge_points;      /* edge points emitted by the edge builder */
  uint64_t input_vertices;   /* vertices read from polygon/path records */
} B2DOracleStats;

/* Renders `stream` into `out_pixels`: width*height 32-bit pixels (PRGB32 or XRGB32 targets) or
 * width*height bytes (A8 targets), tightly packed. The canvas starts zeroed. Returns 0 on
 * success, a negative value for a malformed stream. */
int b2d_oracle_render(const uint8_t* stream, size_t size, uint32_t* out_pixels,
                      const B2DOracleOptions* options, B2DOracleStats* stats);

/* Builds a gradient LUT of `lut_size` entries from `n` stops {double offset; uint64 rgba64}. */
void b2d_oracle_build_lut(uint32_t* lut, uint32_t lut_size, const void* stops, size_t n, uint32_t variant);
/* The 64-bit (premultiplied RGBA64) LUT of dithered gradients (interpolate_prgb64). */
void b2d_oracle_build_lut64(uint64_t* lut, uint32_t lut_size, const void* stops, size_t n);

/* Analytic-rasterizer known-answer support: rasterizes one 24.8 line into a dense cell grid
 * [rows x (width+2)] using banded rasterization with `band_height`, starting at row 0. */
int b2d_oracle_rasterize_line(int x0, int y0, int x1, int y1, uint32_t sign, uint32_t band_height,
                              int width, int rows, uint32_t* cells);

#ifdef __cplusplus
}
#endif

#endif /* B2D_ORACLE_H_INCLUDED */
