// frontend.h - host-side rendering-context front end (the part of BLRasterContextImpl that stays
// on the CPU in the reference too): state, transforms, style resolution and fetch-data setup.
//
// Every formula follows the reference (file:line at each function in frontend.cpp) and runs in
// IEEE double with no FMA contraction (-ffp-contract=off), so the fetch parameters the kernels
// consume are bit-identical to the ones the reference pipeline consumes.
#pragma once

#include <stdint.h>

#include <vector>

#include "blgpu_internal.h"

namespace blgpu {

struct Mat { double m00, m01, m10, m11, m20, m21; };

enum TransformType : int { kTTIdentity = 0, kTTTranslate, kTTScale, kTTSwap, kTTAffine, kTTInvalid };
enum SrcFormat : int { kFmtPRGB32 = 0, kFmtFRGB32 = 1, kFmtZERO32 = 2, kFmtXRGB32 = 3 };

int trunc_to_int(double x);
int64_t floor_to_int64(double x);
int round_to_int(double x);
void mat_multiply(Mat& dst, const Mat& a, const Mat& b);
bool mat_invert(Mat& dst, const Mat& src);
int mat_type(const Mat& m);
uint32_t premultiply(uint32_t argb32);

// A resolved fill style: fetch parameters plus what the frame must provide (LUT, image).
struct HostStyle {
  bool nop = true;                  // NoFillStyle
  int format = kFmtPRGB32;          // source format for comp-op simplification
  DevStyle dev{};
  std::vector<DevStop> stops;       // gradient stops (LUT to build) when dev.lut_size != 0
  int image = -1;                   // frame image index for patterns
};

struct GradientDesc {
  uint32_t type, extend;
  double values[6];
  const DevStop* stops;
  size_t stop_count;
  const double* transform;
};

// Pattern source as seen by the front end: the image is already registered in the frame.
struct PatternDesc {
  int image;                        // frame image index
  int img_w, img_h;
  int area[4];
  uint32_t extend;
  const double* transform;
};

// BLGeometryType values of the shapes shape_path builds.
constexpr uint32_t kGeometryCircle = 5, kGeometryEllipse = 6, kGeometryRoundRect = 7, kGeometryArc = 8,
                   kGeometryChord = 9, kGeometryPie = 10, kGeometryTriangle = 12;
// The path BLPath::add_geometry makes of a circle {cx, cy, r}, ellipse {cx, cy, rx, ry}, round
// rectangle {x, y, w, h, rx, ry}, triangle {x0, y0, x1, y1, x2, y2} or arc / chord / pie
// {cx, cy, rx, ry, start, sweep}; false for other types.
bool shape_path(uint32_t type, const double* v, std::vector<uint8_t>& cmd, std::vector<double>& xy);

void style_solid(HostStyle& s, uint32_t argb32);
void style_gradient(HostStyle& s, const GradientDesc& g, const Mat& final_transform, uint32_t quality = 0);
void style_pattern(HostStyle& s, const PatternDesc& p, uint32_t pattern_quality, const Mat& final_transform);
// Blit fetchers over the image area {x, y, w, h} (image = frame image index).
void style_blit_aligned(HostStyle& s, int image, int img_w, const int area[4], int x0, int y0);
void style_blit_fx_fy(HostStyle& s, int image, int img_w, const int area[4], uint32_t quality, int64_t tx64, int64_t ty64);
void style_blit_affine(HostStyle& s, int image, int img_w, const int area[4], uint32_t quality, const Mat& t);

int default_band_height(int width);

}  // namespace blgpu
