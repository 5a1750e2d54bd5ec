/*
 * b2d_oracle_stroke.h - CPU oracle (test infrastructure only): path stroker declarations.
 */
#ifndef B2D_ORACLE_STROKE_H_INCLUDED
#define B2D_ORACLE_STROKE_H_INCLUDED

#include <stddef.h>
#include <stdint.h>

/* A path under construction: BLPathCmd bytes and their vertices (PathAppender's view). */
typedef struct {
  uint8_t* cmd;
  OPt* vtx;
  size_t n, cap;
} OPath;

/* BLStrokeOptions (blend2d/core/path.h:330-352), without the dash array the stroker ignores. */
typedef struct {
  double width, miter_limit;
  uint32_t join, start_cap, end_cap, transform_order;
} OStrokeOpts;

/* Receives the outline of one figure: A (offset + end cap), B (offset to be reversed) and C
 * (start cap; empty for a closed figure). BLPathStrokeSinkFunc (blend2d/core/path.h:372). */
typedef int (*OStrokeSink)(const OPath* a, const OPath* b, const OPath* c, void* user);

void o_path_reserve(OPath* p, size_t extra);
void o_path_free(OPath* p);

/* Returns 0, 1 for BL_ERROR_INVALID_GEOMETRY, or the sink's non-zero result. Figures already
 * passed to the sink stay passed when a later one fails, as in the reference. */
int o_stroke_path(const uint8_t* cmd, const double* xy, size_t n, const OStrokeOpts* opt,
                  double simplify_tolerance, double offset_parameter, OPath* a, OPath* b, OPath* c,
                  OStrokeSink sink, void* user);

#endif
