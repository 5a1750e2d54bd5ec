// Device stroking: one thread per figure of every stroke command in the frame (threads take the
// figures in an order that puts figures with alike control flow side by side). The first kernel
// runs the stroker to count the figure's outline vertices, an exclusive scan places the figures'
// outlines after the frame's recorded vertices, and the second kernel runs the stroker again to
// write them; the stroke command then reads its outline like any analytic fill's path.
#include "blgpu_internal.h"
#include "launch.h"
#include "stroke_core.h"

namespace blgpu {

namespace {

constexpr int kStrokeThreads = 64;

__global__ void __launch_bounds__(kStrokeThreads) stroke_count_kernel(FrameView f) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= f.counts[kCntStrokeFigs]) {
    if (t < f.num_stroke_figs) f.stroke_totals[t] = 0;   // beyond the frame's figures: nothing to scan
    return;
  }
  const uint32_t i = f.stroke_order[t];
  const DevStrokeFig fg = f.stroke_figs[i];
  const DevStrokeParams dp = f.stroke_params[fg.param];
  const sk::Params p{dp.width, dp.miter_limit, dp.join, dp.start_cap, dp.end_cap, 0u};
  const sk::FigureCounts fc =
      sk::count_figure(f.stroke_cmds, reinterpret_cast<const sk::V*>(f.stroke_xy), fg.first, fg.end, p);
  f.stroke_counts[i] = make_uint4(fc.total(), fc.a, fc.b,
                                  fc.c | (fc.closed ? 1u << 30 : 0u) | (fc.b_ok ? 1u << 31 : 0u));
  f.stroke_totals[i] = fc.total();
}

__global__ void __launch_bounds__(kStrokeThreads) stroke_emit_kernel(FrameView f) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= f.counts[kCntStrokeFigs]) return;
  const uint32_t i = f.stroke_order[t];
  const DevStrokeFig fg = f.stroke_figs[i];
  const uint32_t off = f.stroke_offsets[i];
  const uint32_t vb = f.counts[kCntStrokeVertBase] + off;
  if (fg.cmd_figs) {
    DevCmd& c = f.cmds_rw[fg.cmd];
    c.geom_first = vb;
    c.geom_count = f.stroke_offsets[i + fg.cmd_figs] - off;
  }
  const uint4 cnt = f.stroke_counts[i];
  if (!cnt.x) return;
  sk::FigureCounts fc;
  fc.a = cnt.y;
  fc.b = cnt.z;
  fc.c = cnt.w & 0x3FFFFFFFu;
  fc.closed = (cnt.w >> 30) & 1u;
  fc.b_ok = (cnt.w >> 31) & 1u;
  const DevStrokeParams dp = f.stroke_params[fg.param];
  const sk::Params p{dp.width, dp.miter_limit, dp.join, dp.start_cap, dp.end_cap, 0u};
  // the frame's vertex and command arrays are written here, before any kernel reads them
  uint8_t* out_cmd = const_cast<uint8_t*>(f.path_cmds) + vb;
  double* out_xy = const_cast<double*>(f.verts) + 2ull * vb;
  sk::emit_figure(f.stroke_cmds, reinterpret_cast<const sk::V*>(f.stroke_xy), fg.first, fg.end, p, fc, out_cmd, out_xy);
}

}  // namespace

int launch_stroke_count(const FrameView& f, cudaStream_t st) {
  if (!f.num_stroke_figs) return 0;
  const uint32_t n = f.num_stroke_figs;
  stroke_count_kernel<<<(n + kStrokeThreads - 1) / kStrokeThreads, kStrokeThreads, 0, st>>>(f);
  int k = 1;
  k += exclusive_scan(f.stroke_totals, f.stroke_offsets, n, f.stroke_scan_tmp, st);
  k += launch_total(f.stroke_totals, f.stroke_offsets, n, f.stroke_offsets + n, st);
  return k;
}

int launch_stroke_emit(const FrameView& f, cudaStream_t st) {
  if (!f.num_stroke_figs) return 0;
  const uint32_t n = f.num_stroke_figs;
  stroke_emit_kernel<<<(n + kStrokeThreads - 1) / kStrokeThreads, kStrokeThreads, 0, st>>>(f);
  return 1;
}

}  // namespace blgpu
