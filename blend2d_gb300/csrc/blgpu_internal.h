// blgpu_internal.h - data layout shared by the host front end and the sm_103a kernels.
//
// A *frame* is everything recorded between two flushes of one or more canvases: fill commands in
// painter's order, their styles (fetch parameters prepared on the host with the reference's
// formulas), input geometry in double precision, transforms, gradient LUT requests and pattern
// images. The device pipeline turns it into pixels:
//
//   K0 lut_build    - gradient LUTs (one thread per entry, reference builder semantics)
//   K1 edge_build   - FP64 edge building per analytic command (count pass + emit pass) producing
//                     24.8 fixed-point segments, exactly the reference's EdgeBuilder output
//   K2 binning      - per command tile ranges, per (command, tile row) segment lists, per tile row
//                     command lists in painter's order
//   K3 fine         - persistent tile kernel: tile pixels stay in registers while every command
//                     touching the tile is rasterized into shared-memory cells, swept and composited
//
// Everything here is POD so a frame can be uploaded with one copy.
#pragma once

#include <stdint.h>
#include <vector_types.h>

namespace blgpu {

constexpr int kTileW = 32;          // tile width in pixels
constexpr int kTileH = 32;          // tile height in pixels (also the rasterizer band)
constexpr int kTileShift = 5;
constexpr int kFineThreads = 256;   // 8 warps per block
constexpr int kStripRows = 4;       // a strip (one warp: 32 lanes x 4 pixels) is 4 rows of a tile
constexpr int kStripShift = 2;
constexpr int kMaxListLog2 = kTileShift - kStripShift;   // list rows down to one strip (4 rows)

enum FillKind : uint32_t {
  kFillAnalytic = 0,   // edges -> analytic coverage (FillAnalytic_Base)
  kFillBoxA = 1,       // pixel-aligned box (FillBoxA_Base)
  kFillBoxU = 2,       // 24.8 box with fractional borders (FillData::init_box_u_8bpc_24x8)
  kFillMaskA = 3       // pixel-aligned box with an A8 mask (fill_box_masked_a): geom_first / xform =
                       // low / high 32 bits of the mask's byte offset in the image pool at the box's
                       // top-left pixel, geom_count = the mask's row pitch in bytes
};

enum GeomKind : uint32_t { kGeomPolygon = 0, kGeomPath = 1 };

// Bits of FrameView::error_flags[0]: a work array of the frame was too small for what the device
// produced (the frame's pixels are then not valid and the host reports an error). The host sizes
// every array from a bound, so none of them is expected; a replay whose data changed could meet
// one.
enum ErrorFlag : uint32_t {
  kErrItems = 1u,        // lines / curves of the analytic commands (bound: one per vertex)
  kErrPieces = 2u,       // monotonic curve pieces (bound: 3 per curve vertex)
  kErrSeglist = 4u,      // coverage work items (sized by the binning count pass)
  kErrMasks = 8u,        // slot masks (sized by the binning count pass)
  kErrSegments = 16u,    // segments (the segment array is grown and the frame re-run)
  kErrCapacity = 32u     // a work array sized by capacity (graph frames) is too small: the render
                         // half was skipped
};

// FrameView::work_counter[kSkipWord] != 0: the binning and composite passes do nothing (their
// inputs would not fit the arrays they write; set by frame_gate_kernel).
constexpr int kSkipWord = 27;

enum FetchKind : uint32_t {
  kFetchSolid = 0,
  kFetchLinearPad, kFetchLinearRoR,
  kFetchRadialPad, kFetchRadialRoR,
  kFetchConic,
  kFetchPatAlignedPad, kFetchPatAlignedRepeat, kFetchPatAlignedRoR,
  kFetchPatFxFyPad, kFetchPatFxFyRoR,
  kFetchPatAffineNN, kFetchPatAffineBI
};

enum LutVariant : uint32_t { kLutSSE2 = 0, kLutAVX2 = 1, kLutScalar = 2,
                             kLut64 = 3 };   // kLut64: the 64-bit LUT of dithered gradients (interpolate_prgb64)

// Fetch parameters of one style, set up on the host exactly like the reference's
// Pipeline::FetchUtils (blend2d/pipeline/pipedefs.cpp). The three gradient kinds' parameters share
// one block, since a style reads only its own kind's (every reader dispatches on `fetch`); its
// largest member (radial) comes first, so a value-initialized DevStyle{} has every byte zero. The
// pattern parameters stay outside it: the composite measured about 10 % slower with them in the
// shared block too (the layout changes how the fetch code is compiled).
struct alignas(16) DevStyle {
  uint32_t fetch;          // FetchKind
  uint32_t solid;          // premultiplied PRGB32 (kFetchSolid)
  uint32_t lut_offset;     // first entry in the LUT pool
  uint32_t lut_size;
  uint32_t maxi, rori;
  int32_t con_maxi, con_rori;
  union {
    struct {
      // radial
      double rad_tx, rad_ty, rad_yx, rad_yy, rad_b0, rad_by, rad_dd0, rad_ddy;
      double rad_inv2a, rad_amul4, rad_sq_inv2a, rad_sq_fr;
      float rad_bd, rad_ddd;
    };
    struct {
      // linear (32.32 fixed point)
      uint64_t lin_pt0, lin_dt, lin_dy;
    };
    struct {
      // conic
      float con_q[4];
      float con_n1, con_n2, con_n4, con_offset, con_xx;
      float pad0;
      double con_tx, con_ty, con_yx, con_yy;
    };
  };
  // pattern source (area origin inside the image pool)
  uint64_t src_offset;     // in pixels
  int32_t src_w, src_h, src_stride, pad1;
  // pattern aligned / fx-fy
  int32_t pat_tx, pat_ty, pat_rx, pat_ry;
  uint32_t pat_wa, pat_wb, pat_wc, pat_wd;
  uint32_t ext_y;          // vertical extend: 0 pad, 1 repeat, 2 reflect
  uint32_t dither;         // gradient quality DITHER: 64-bit LUT (2 words per entry) + ordered dither
  uint32_t src_or;         // OR-ed into every pattern fetch: 0xFF000000 when the source is read as XRGB32
  uint32_t pad2;
  // pattern affine (32.32 fixed point)
  uint64_t af_xx, af_xy, af_yx, af_yy, af_tx, af_ty;
  int32_t af_ox, af_oy, af_rx, af_ry;
  int32_t af_minx, af_miny, af_maxx, af_maxy;
  int32_t af_corx, af_cory, af_tw, af_th;
  int32_t af_tw_m, af_tw_s, af_th_m, af_th_s;   // div_magic of af_tw / af_th (divmagic.h)
};
static_assert(sizeof(DevStyle) == 320, "DevStyle: 32-byte common part, 104-byte gradient block, pattern fields");

struct alignas(16) DevXform {
  double m[6];             // m00 m01 m10 m11 m20 m21 (final transform x 256)
  uint32_t affine;         // 1 = EdgeTransformAffine, 0 = EdgeTransformScale
  uint32_t pad[3];
};

struct alignas(16) DevCmd {
  uint32_t kind;           // FillKind
  uint32_t canvas;         // canvas index
  uint32_t style;          // DevStyle index
  uint32_t flags;          // bit0 SrcCopy, bit1 EvenOdd
  uint32_t alpha;          // 0..255
  uint32_t geom;           // GeomKind
  uint32_t geom_first;     // first vertex
  uint32_t geom_count;     // vertex count
  uint32_t xform;          // DevXform index
  int32_t fetch_y0;        // box fills: first row the reference's fetcher is initialized at
  int32_t box[4];          // BoxA: pixels; BoxU: 24.8; analytic: pixel bbox written by K1
  uint32_t seg_first;      // K1 output
  uint32_t seg_count;
  uint32_t status;         // after binning: 0 ok, 1 invalid geometry (NaN), 2 nothing to render
  uint32_t color;          // solid styles: the premultiplied colour (their style entry is shared and carries none)
};

struct alignas(16) DevCanvas {
  uint32_t* pixels;        // device pointer to the canvas's first pixel
  int32_t w, h, stride;    // stride in pixels
  int32_t band_height;     // reference band height (conic fetch start rows)
  int32_t tiles_x, tiles_y;
  uint32_t tile_base;      // first global tile index
  uint32_t row_base;       // first global tile-row index (command-list rows: row_base << list_log2)
  uint32_t cmd_first, cmd_count;
  uint32_t a8;             // 1: one byte per pixel (A8 target); pixels/stride then count bytes
  uint32_t pad;
};

struct alignas(16) DevLutJob {
  uint32_t style;          // DevStyle index (receives the LUT)
  uint32_t stop_first;     // first stop in the stop pool
  uint32_t stop_count;
  uint32_t lut_offset;
  uint32_t lut_size;
  uint32_t variant;        // LutVariant
  uint32_t pad[2];
};

struct DevStop {
  double offset;
  uint64_t rgba64;
};

struct DevSeg {            // one non-horizontal 24.8 segment, y0 < y1
  int32_t x0, y0, x1, y1;
};

enum ItemKind : uint32_t { kItemLine = 0, kItemQuad = 1, kItemCubic = 2, kItemConic = 3, kItemWhole = 4 };

// A canvas copied between the runtime's canvas pool and a page-locked host image by a kernel (the
// device reaches page-locked memory directly): rows of w pixels, strides in pixels (one byte each
// for an A8 canvas).
struct DevXfer {
  uint32_t* dev;
  uint32_t* host;              // the host image's device-accessible address
  int32_t w, h;
  int32_t dev_stride, host_stride;
  int32_t a8, pad;
};

// One line, curve or closing line of an analytic command, built independently of the command's
// other items. Vertex indices are relative to geom_first.
struct DevItem {
  uint32_t cmd;
  uint32_t kind;           // ItemKind
  uint32_t a;              // start point (the previous curve's end point)
  uint32_t b;              // first control point (line: end point)
};

#ifdef __CUDACC__
// Tile columns whose cells a segment can touch within strip row `r` (pixel rows [4r, 4r + 3]):
// the line's x at the strip's clipped y extent, one pixel of slack on both sides (the integer DDA
// stays within a 24.8 unit of the exact line) and 16 units more for the FP32 evaluation (segments
// are clipped to the canvas, so |dx|, |dy| < 2^24 are exact floats and the product and quotient
// are off by a few units at most), clamped to the segment's own x extent, plus the cell right of
// the last one (area). `t_last` is the last such column; columns after it only see the segment's
// full row cover. A wider range only adds work items (whose cells the window clipping keeps
// exact); FP32 keeps this off the FP64 pipe that 64-bit integer division would use.
__device__ __forceinline__ void strip_tile_range(const DevSeg& g, int r, int& t0, int& t_last) {
  int ya = max(g.y0, (r << kStripShift) << 8);
  int yb = min(g.y1, ((r + 1) << kStripShift) << 8);
  const float slope = float(g.x1 - g.x0) / float(g.y1 - g.y0);
  int xa = g.x0 + int(slope * float(ya - g.y0));
  int xb = g.x0 + int(slope * float(yb - g.y0));
  int lo = max(min(xa, xb) - (256 + 16), min(g.x0, g.x1));
  int hi = min(max(xa, xb) + (256 + 16), max(g.x0, g.x1));
  t0 = (lo >> 8) >> kTileShift;
  t_last = ((hi >> 8) + 1) >> kTileShift;
}
#endif

// One monotonic piece of a curve, split off by curve_split_kernel and flattened by
// edge_pieces_kernel: its DEG + 1 points (transformed, 24.8 scale), its command and its curve's
// clip flags (0: the curve lies inside the clip box).
struct alignas(16) DevPiece {
  double2 p[4];
  uint32_t cmd;
  uint32_t any;
  uint32_t pad[2];
};

// One figure of a stroked path: commands [first, end) of the frame's stroke input (the extent the
// reference's stroker walks), the stroke command whose outline it adds to, and its options.
struct DevStrokeFig {
  uint32_t first, end;
  uint32_t cmd;            // DevCmd index
  uint32_t cmd_figs;       // on the command's first figure: its figure count; else 0
  uint32_t param;          // stroke parameter index
};

// Width, miter limit, join and caps of a stroke (BLStrokeOptions without the dash array).
struct DevStrokeParams {
  double width, miter_limit;
  uint32_t join, start_cap, end_cap, pad;
};

// The frame's sizes in device memory (FrameView::counts), uploaded with its data: kernels read
// them there, so launches sized by capacities serve any frame that fits (a captured CUDA graph can
// render new frames).
enum CountIndex : uint32_t {
  kCntCmds = 0, kCntCanvases = 1, kCntTiles = 2, kCntRows = 3, kCntLutJobs = 4, kCntStrokeFigs = 5,
  kCntStrokeVertBase = 6, kCntWords = 8
};

// Device-side view of a frame (pointers into one device arena). The num_* fields are the
// capacities the arrays are sized by (the frame's own sizes in an eager run): launches are sized by
// them, and kernels take the actual sizes from `counts` and from the device totals.
struct FrameView {
  const uint32_t* counts;      // [kCntWords] CountIndex
  const DevCmd* cmds;
  DevCmd* cmds_rw;
  const DevStyle* styles;
  const DevXform* xforms;
  const DevCanvas* canvases;
  const double* verts;         // xy pairs
  const uint8_t* path_cmds;    // one command byte per vertex
  const DevLutJob* lut_jobs;
  const DevStop* stops;
  uint32_t* luts;
  const uint32_t* images;
  uint32_t* pixels;
  // K1
  DevItem* items;              // lines and curves of every analytic command (any order)
  DevItem* curve_items;        // cubic curves from the front, quadratic / conic curves from the back
  DevPiece* pieces;            // their monotonic pieces, cubic from the front, quadratic from the back
  uint32_t* piece_list;        // cubic piece indices: inside the clip box from the front, clipped from the back
  uint32_t piece_capacity;
  int4* cmd_bbox;              // [num_cmds] 24.8 bbox of the emitted segments: xmin, ymin, xmax, ymax
  DevSeg* segs;                // emitted segments (any order)
  uint32_t* seg_meta;          // cmd << 1 | sign
  uint32_t seg_capacity;       // slots in segs / seg_meta
  uint32_t item_capacity;      // upper bound of the number of items
  // K2
  uint32_t* cmd_tile_x;        // tx0 | tx1 << 16 (0xFFFFFFFF = nothing)
  uint32_t* cmd_tile_y;        // ty0 | ty1 << 16
  uint32_t* cmd_xr;            // pixel columns x0 | x1 << 16 (inclusive; x0 > x1 = nothing)
  uint32_t* cmd_yr;            // pixel rows y0 | y1 << 16
  uint32_t* cmdrow_base;       // [num_cmds + 1]: first (cmd, strip row, tile column) slot
  uint32_t* cmdrow_counts;     // [num_cmdrows + 1]
  uint32_t* cmdrow_offsets;    // scratch for the scan of non-empty slots
  uint32_t* slot_cmd;          // [num_cmdrows] command of each slot with segments
  uint32_t* slot_mask;         // [num_cmdrows + 1] 1 + index of the slot's masks, 0 = no segments
  uint32_t* mask_slot;         // [non-empty slots] slot of each compact mask index
  uint4* mask_info;            // [non-empty slots] {x of the slot's first column, its first row, flags << 16 | alpha, slot}
  uint32_t* slot_first;        // [num_cmdrows + 1] first work item of each slot (exclusive scan of the counts)
  uint2* entries;              // coverage work items {segment, mask index}, grouped by slot in slot order
  uint32_t mask_capacity;      // slots the masks array holds
  uint8_t* masks;              // [non-empty slots][kStripRows * kTileW]: analytic masks from the coverage pass
  uint32_t* backdrop;          // [num_cmdrows][kStripRows]: coverage carried into the slot's tile
                               //   from segments entirely left of it (cover << 9 per row)
  uint32_t* row_counts;        // [num_rows + 1]
  uint32_t* row_offsets;
  uint2* row_box;              // per list entry: its command's pixel columns x0 | x1 << 16 and rows
                               //   y0 | y1 << 16, what a strip tests before it reads the records
  uint4* row_recs;             // command lists per list row, painter's order: two records per entry,
                               //   {command, pixel columns x0 | x1 << 16, rows y0 | y1 << 16, meta}
                               //   {first slot, tile column tx0 | columns << 16, style, first row state}
                               //   with meta = kind | flags << 2 | alpha << 4; for a solid style the
                               //   style word has bit 31 set and the colour replaces the row state
  uint32_t* row_copies;        // [num_rows] SrcCopy commands in each tile row's list
  uint32_t* strip_start;       // [num_tiles * strips per tile] first list entry the composite needs (occlusion)
  uint32_t* tile_order;        // tile processing order for the persistent fine kernel
  uint32_t* tile_canvas;       // canvas index per global tile
  uint32_t* work_counter;      // [0] fine work queue, [1] items, [2] cubics, [3] their queue, [21] quads, [22] their queue,
                               //   [23] cubic pieces, [24] their queue, [25] quadratic pieces, [26] their queue,
                               //   [28] / [29] cubic pieces inside the clip box / clipped, [30] / [31] their queues
  uint32_t* totals;            // [8] segments, seglist bound, (cmd,strip) slots, row entries, gradient rows,
                               //   slots with segments, conic row runs
  uint32_t* rs_count;          // [num_cmds + 1] gradient row states per command (radial/conic styles)
  uint32_t* rs_base;           // exclusive scan of rs_count
  float4* row_states;          // per (command, row): the fetcher's row values f0, f1, f2
  uint32_t* rb_count;          // [num_cmds + 1] conic styles: runs of rows sharing one fetcher start
  uint32_t* rb_base;           // exclusive scan of rb_count
  uint32_t* error_flags;
  unsigned long long* pixel_ops;   // [2] composited pixels (mask != 0), of which pattern-fetched
  uint32_t num_cmds;
  uint32_t num_canvases;
  uint32_t num_tiles;
  uint32_t num_rows;
  uint32_t num_lut_jobs;
  // Stroking: the stroke input paths, one thread per figure counts (stroke_counts: total, A, B,
  // C | closed << 30 | B taken << 31) and then writes the figure's outline at
  // verts / path_cmds[stroke_vert_base + stroke_offsets[fig]].
  const DevStrokeFig* stroke_figs;
  const uint32_t* stroke_order;   // thread -> figure: figures with alike work side by side
  const DevStrokeParams* stroke_params;
  const double* stroke_xy;
  const uint8_t* stroke_cmds;
  uint4* stroke_counts;
  uint32_t* stroke_totals;
  uint32_t* stroke_offsets;   // num_stroke_figs + 1 (the last one: the outline's size)
  uint32_t* stroke_scan_tmp;
  uint32_t num_stroke_figs;
  uint32_t stroke_vert_base;
  uint32_t num_segs;
  uint32_t num_cmdrows;
  uint32_t num_seglist;
  uint32_t num_row_states;
  uint32_t num_row_runs;       // conic row runs (sum of rb_count)
  uint32_t num_row_entries;    // row list entries (sum of row_counts)
  // Command lists are kept per list row of 1 << list_shift pixel rows (4 to 32; tunable): a canvas
  // of tiles_y tile rows has tiles_y << list_log2 list rows (list_log2 = 5 - list_shift), from
  // list row row_base << list_log2 on; rows past the canvas's bottom stay empty.
  uint32_t list_shift;
};

}  // namespace blgpu
