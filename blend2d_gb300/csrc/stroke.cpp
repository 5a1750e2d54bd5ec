// Host side of stroking: figure extents and validation, and the host outline export.
#include "stroke.h"

#include "stroke_core.h"

namespace blgpu {

BLGpuResult stroke_figures(const uint8_t* cmd, size_t n, std::vector<uint32_t>& ranges) {
  const size_t mark = ranges.size();
  size_t i = 0;
  while (i < n) {
    if (cmd[i] != sk::kMove) {
      if (cmd[i] != sk::kClose) { ranges.resize(mark); return BLGPU_ERROR_INVALID_GEOMETRY; }
      i++;
      continue;
    }
    const size_t first = i++;
    // the figure's commands as the stroker consumes them: lines one vertex, curves their two or
    // three vertices whatever their commands, a close ends the figure and is consumed, anything
    // else ends it
    while (i < n) {
      const uint8_t c = cmd[i];
      if (c == sk::kOn) { i++; continue; }
      if (c == sk::kQuad || c == sk::kCubic) {
        i += c == sk::kQuad ? 2 : 3;
        if (i > n) { ranges.resize(mark); return BLGPU_ERROR_INVALID_GEOMETRY; }
        continue;
      }
      if (c == sk::kClose) i++;
      break;
    }
    if (i - first >= 2) {
      ranges.push_back(uint32_t(first));
      ranges.push_back(uint32_t(i));
    }
  }
  return BLGPU_SUCCESS;
}

BLGpuResult stroke_outline(const uint8_t* cmds, const double* xy, size_t n, const StrokeParams& p,
                           std::vector<uint8_t>& out_cmds, std::vector<double>& out_xy) {
  std::vector<uint32_t> ranges;
  BLGpuResult r = stroke_figures(cmds, n, ranges);
  if (r) return r;
  const sk::Params sp{p.width, p.miter_limit, p.join, p.start_cap, p.end_cap, 0u};
  const sk::V* vtx = reinterpret_cast<const sk::V*>(xy);
  std::vector<sk::FigureCounts> counts(ranges.size() / 2);
  size_t total = 0;
  for (size_t f = 0; f < counts.size(); f++) {
    counts[f] = sk::count_figure(cmds, vtx, ranges[2 * f], ranges[2 * f + 1], sp);
    total += counts[f].total();
  }
  size_t at = out_cmds.size();
  out_cmds.resize(at + total);
  out_xy.resize(2 * (at + total));
  for (size_t f = 0; f < counts.size(); f++) {
    if (!counts[f].total()) continue;
    sk::emit_figure(cmds, vtx, ranges[2 * f], ranges[2 * f + 1], sp, counts[f], out_cmds.data() + at, out_xy.data() + 2 * at);
    at += counts[f].total();
  }
  return BLGPU_SUCCESS;
}

}  // namespace blgpu
