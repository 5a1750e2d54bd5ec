// Path stroking. The stroker itself (stroke_core.h) runs on the device, one thread per figure;
// the recording thread only splits a stroked path into the figures the reference's stroker visits
// and validates it.
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

// The figures PathStroker::stroke (pathstroke.cpp:224-487) strokes, as [first, end) command
// ranges appended to `ranges` (figures with a move only are left out: they stroke to nothing).
// Returns BLGPU_ERROR_INVALID_GEOMETRY where the reference's stroke fails (a command other than
// a move or close between figures, a curve running past the path's end): it then draws nothing.
BLGpuResult stroke_figures(const uint8_t* cmds, size_t n, std::vector<uint32_t>& ranges);

// The outline a stroke fills non-zero, on the host with the same stroker: per closed figure its
// two offset figures, per open figure one loop (see stroke_core.h). Used by
// blgpu_stroke_outline_d; rendering strokes the figures on the device.
BLGpuResult stroke_outline(const uint8_t* cmds, const double* xy, size_t n, const StrokeParams& p,
                           std::vector<uint8_t>& out_cmds, std::vector<double>& out_xy);

}  // namespace blgpu
