// Context object behind the C ABI: device, stream, owned allocations and the
// device status word that bounded waits write on time-out.
#pragma once
#include <cuda_runtime.h>
#include <mutex>
#include <set>

#include "common.cuh"

#include <atomic>
#include <map>
#include <tuple>
#include <string>
#include <vector>

namespace csg {
struct ProfPending {
  std::string name;
  cudaEvent_t a, b;
  double flops, bytes;
};
struct ProfAcc {
  long long count = 0;
  double ms = 0, flops = 0, bytes = 0;
};
// Kernel launches made by the library's host code (all contexts).
extern std::atomic<unsigned long long> g_launches;
}  // namespace csg

struct csg_ctx {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  int* status = nullptr;            // device int, 0 = ok
  long long wait_budget = 0;        // bounded-wait cycles of the GEMMs (0: default)
  std::set<void*> allocations;
  int sm_count = 0;
  // pipelined readout (csg_readout_d2h): two device staging buffers, each
  // copied to the host on copy_stream while the context's stream runs on
  cudaStream_t copy_stream = nullptr;
  void* ro_buf[2] = {nullptr, nullptr};
  size_t ro_cap[2] = {0, 0};
  cudaEvent_t ro_ready[2] = {nullptr, nullptr};  // staging filled (context stream)
  cudaEvent_t ro_done[2] = {nullptr, nullptr};   // staging copied out (copy stream)
  int ro_next = 0;
  // DFT plans of non-power-of-two 2-D transforms, by (n, sign, precision),
  // and their spectrum scratch (grow-only)
  std::map<std::tuple<int, int, int>, csg_mft*> dft_plans;
  void* dft_scratch = nullptr;
  size_t dft_scratch_bytes = 0;
  int* dft_zero = nullptr;  // operator slot 0 for every field
  int dft_zero_n = 0;
  // opt-in per-kernel timing (CUDA events on the launching stream)
  bool prof = false;
  std::vector<csg::ProfPending> pending;
  std::map<std::string, csg::ProfAcc> acc;
};

namespace csg {

// Records CUDA events around the launches inside its scope when profiling is
// on (never inside graph capture: csg_profile refuses while capturing).
struct ProfScope {
  csg_ctx* c;
  ProfPending p;
  bool on;
  ProfScope(csg_ctx* ctx, const char* name, double flops = 0, double bytes = 0)
      : c(ctx), on(ctx && ctx->prof) {
    if (!on) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(ctx->stream, &cs);
    if (cs != cudaStreamCaptureStatusNone) {
      on = false;
      return;
    }
    p.name = name;
    p.flops = flops;
    p.bytes = bytes;
    cudaEventCreate(&p.a);
    cudaEventCreate(&p.b);
    cudaEventRecord(p.a, ctx->stream);
  }
  ~ProfScope() {
    if (!on) return;
    cudaEventRecord(p.b, c->stream);
    c->pending.push_back(p);
  }
};

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
