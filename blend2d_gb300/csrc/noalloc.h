// noalloc.h - fixed-size device scratch area for the no-allocation render entry point.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include <mutex>

namespace blgpu {

// 32 MiB per device: enough for a frame of a few thousand fills on a canvas up to 2048 x 2048
// (frame data, gradient LUTs, pattern images, segments and binning lists all live in it). Frames
// that need more are rejected with BLGPU_ERROR_DATA_TOO_LARGE.
constexpr size_t kNoAllocArenaBytes = size_t(32) << 20;
constexpr int kNoAllocMaxDevices = 64;

// Device address of the scratch area of `device`, which must be the current device. Looked up
// with cudaGetSymbolAddress on the first call per device and cached for the life of the process
// (a cudaDeviceReset after that first call is not supported: the cached address belongs to the
// context the reset destroys).
cudaError_t noalloc_arena(int device, void** out);

// The lock that serializes calls of this process on `device`'s scratch area.
std::mutex& noalloc_lock(int device);

}  // namespace blgpu
