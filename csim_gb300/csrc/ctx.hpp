// Context object behind the C ABI: device, stream, owned allocations and the
// device status word that bounded waits write on time-out.
#pragma once
#include <cuda_runtime.h>
#include <mutex>
#include <set>

#include "common.cuh"

struct csg_ctx {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  int* status = nullptr;            // device int, 0 = ok
  std::set<void*> allocations;
  int sm_count = 0;
};

namespace csg {

// RAII guard that makes the context's device current for the call.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

// Grow-only device scratch owned by a plan.
struct Scratch {
  void* ptr = nullptr;
  size_t bytes = 0;
  int ensure(size_t need) {
    if (need <= bytes) return CSG_OK;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    if (cudaMalloc(&ptr, need) != cudaSuccess) {
      cudaGetLastError();
      set_error("scratch allocation failed");
      return CSG_E_NOMEM;
    }
    bytes = need;
    return CSG_OK;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
};

}  // namespace csg
