// noalloc.cu - the fixed device scratch area of blgpu_render_stream_noalloc.
//
// One statically allocated, 256-byte aligned array per device (it exists from module load on; no
// allocating call ever creates or grows it). Its address is looked up once per device with
// cudaGetSymbolAddress while that device is current.
#include <cuda_runtime.h>

#include <mutex>

#include "noalloc.h"

namespace blgpu {

__device__ __align__(256) unsigned char g_noalloc_arena[kNoAllocArenaBytes];

cudaError_t noalloc_arena(int device, void** out) {
  static std::mutex lock;
  static void* addr[kNoAllocMaxDevices] = {};
  if (device < 0 || device >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> guard(lock);
  if (!addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_arena);
    if (e != cudaSuccess) return e;
    addr[device] = p;
  }
  *out = addr[device];
  return cudaSuccess;
}

std::mutex& noalloc_lock(int device) {
  static std::mutex locks[kNoAllocMaxDevices];
  static std::mutex fallback;
  return device >= 0 && device < kNoAllocMaxDevices ? locks[device] : fallback;
}

}  // namespace blgpu
