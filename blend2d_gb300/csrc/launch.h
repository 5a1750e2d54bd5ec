// launch.h - host entry points of the device pipeline (kernels.cu, stroke.cu). Each returns
// the number of kernels it launched on `st`.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "blgpu_internal.h"

namespace blgpu {

// Launch shapes the autotuner chooses between (0 = the default for that field).
struct LaunchConfig {
  int cover_slots = 0;            // slots with segments per coverage block (16, 32 or 64; 0 = by frame)
  int cover_blocks_per_sm = 0;    // coverage grid: blocks per SM (0 = as many as fit)
  int fine_blocks_per_sm = 0;     // composite grid: blocks per SM (0 = as many as fit)
  int edge_block = 128;           // threads per block of the per-item edge builder (64/128/256)
  int cubic_blocks_per_sm = 3;    // lane-scheduled curve-piece flattener: blocks per SM (0 = as many as fit)
  int no_occlusion_cull = 0;      // 1: the composite starts every strip at its first command
  int max_segments = 0;           // > 0: cap of the segment array (frames needing more fail)
  int graph_frames = 0;           // 1: frames run as a captured graph over capacity-sized arrays
  int list_rows = 32;             // pixel rows per command list (4, 8, 16 or 32)
  int device_order = 0;           // 1: pipelines of runtimes that set it run one after another on the device
};

// log2 of the list-row height a launch config selects.
inline uint32_t list_shift_of(const LaunchConfig& c) {
  return c.list_rows == 4 ? 2u : c.list_rows == 8 ? 3u : c.list_rows == 16 ? 4u : 5u;
}

int exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* tmp, cudaStream_t st);
uint32_t scan_temp_words(uint32_t n);
int launch_total(const uint32_t* counts, const uint32_t* offsets, uint32_t n, uint32_t* total, cudaStream_t st);
int launch_sum(const uint32_t* in, uint32_t n, uint32_t* total, cudaStream_t st);

int launch_lut(const FrameView& f, cudaStream_t st);
int launch_edges(const FrameView& f, const LaunchConfig& cfg, cudaStream_t st);
int launch_cmd_tiles(const FrameView& f, uint32_t* cmdrow_counts_per_cmd, cudaStream_t st);
int launch_seg_bin(const FrameView& f, int scatter, cudaStream_t st);
int launch_rows_and_tiles(const FrameView& f, uint32_t* row_canvas, cudaStream_t st);
int launch_fine(const FrameView& f, const LaunchConfig& cfg, cudaStream_t st);
int launch_row_states(const FrameView& f, cudaStream_t st);
int launch_backdrop_prefix(const FrameView& f, cudaStream_t st);
int launch_frame_gate(const FrameView& f, cudaStream_t st);
// Copies the `n` canvases of `xfers` (device memory) to their host images (to_host) or back.
int launch_canvas_copy(const DevXfer* xfers, uint32_t n, int to_host, cudaStream_t st);
int launch_coverage(const FrameView& f, const LaunchConfig& cfg, uint32_t* scan_tmp, cudaStream_t st);
int fine_grid_size(int blocks_per_sm);
// Stroking: per-figure outline sizes and their exclusive scan (stroke_offsets), then the outlines.
int launch_stroke_count(const FrameView& f, cudaStream_t st);
int launch_stroke_emit(const FrameView& f, cudaStream_t st);

}  // namespace blgpu
