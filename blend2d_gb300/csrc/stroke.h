// Path stroking on the recording thread: a stroke becomes the non-zero fill of its outline, which
// the device pipeline then builds, rasterizes and composites like any analytic fill.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "blgpu.h"

namespace blgpu {

// BLStrokeOptions (blend2d/core/path.h:330-352); the dash array is not part of the reference's
// stroker and is not kept.
struct StrokeParams {
  double width = 1.0;
  double miter_limit = 4.0;
  uint32_t join = 0;              // BLStrokeJoin, MITER_CLIP
  uint32_t start_cap = 0;         // BLStrokeCap, BUTT
  uint32_t end_cap = 0;
  uint32_t transform_order = 0;   // BLStrokeTransformOrder, AFTER
};

// BLApproximationOptions defaults (blend2d/core/path_p.h:89-98) the stroker reads.
constexpr double kSimplifyTolerance = 0.05;
constexpr double kOffsetParameter = 0.414213562;

// Strokes the path (BLPathCmd bytes + vertices) and appends its outline to `cmds`/`xy` as
// implicitly closed figures for a non-zero fill: per closed input figure its two offset paths
// (A, and B reversed); per open figure one loop A + end cap + reversed B + start cap. The
// segments are exactly those the reference's stroke sink hands its edge builder
// (rastercontextops.cpp:61-74): an open A or C path ends where the next part starts, and the
// zero-length closing line of the joined loop adds nothing. Returns BLGPU_SUCCESS, or
// BLGPU_ERROR_INVALID_GEOMETRY with nothing appended (the reference then fills nothing).
BLGpuResult stroke_outline(const uint8_t* cmds, const double* xy, size_t n, const StrokeParams& p,
                           std::vector<uint8_t>& out_cmds, std::vector<double>& out_xy);

}  // namespace blgpu
