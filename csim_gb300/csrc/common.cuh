// Shared helpers for the csim GB300 kernels: status codes, error capture,
// bounded mbarrier waits and the bf16 three-way split.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/csimgpu.h"

namespace csg {

// Per-thread last error message (the C ABI exposes it through csg_last_error).
void set_error(const std::string& msg);
const char* get_error();

#define CSG_CUDA(call)                                                          \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      ::csg::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));    \
      return CSG_E_CUDA;                                                        \
    }                                                                           \
  } while (0)

#define CSG_CHECK(cond, code, msg)                                              \
  do {                                                                          \
    if (!(cond)) {                                                              \
      ::csg::set_error(msg);                                                    \
      return (code);                                                            \
    }                                                                           \
  } while (0)

#define CSG_LAUNCH_CHECK()                                                      \
  do {                                                                          \
    ::csg::count_launch();                                                      \
    cudaError_t e_ = cudaGetLastError();                                        \
    if (e_ != cudaSuccess) {                                                    \
      ::csg::set_error(std::string("kernel launch: ") + cudaGetErrorString(e_)); \
      return CSG_E_CUDA;                                                        \
    }                                                                           \
  } while (0)

// Counts kernel launches made by the library (csg_launch_count).
void count_launch();

// ~1 s at 2 GHz: no legitimate wait inside a kernel comes close.
constexpr long long kWaitBudgetCycles = 2000000000LL;

__device__ __forceinline__ void split3(float v, __nv_bfloat16& a, __nv_bfloat16& b,
                                       __nv_bfloat16& c) {
  // v = a + b + c to ~24 bits: each residual is exact in fp32.
  a = __float2bfloat16_rn(v);
  float r = v - __bfloat162float(a);
  b = __float2bfloat16_rn(r);
  float r2 = r - __bfloat162float(b);
  c = __float2bfloat16_rn(r2);
}

inline int grid_for(long long n, int block, int cap = 152 * 32) {
  long long g = (n + block - 1) / block;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace csg
