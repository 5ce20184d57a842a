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

// split3 of two values at once (paired bf16 conversions, one instruction per
// part), bit-identical to split3 on each: h0, h1, h2 hold the parts of x0 in
// their low and of x1 in their high halves.
__device__ __forceinline__ void split3_pair(float x0, float x1, uint32_t& h0, uint32_t& h1,
                                            uint32_t& h2) {
  const __nv_bfloat162 a = __floats2bfloat162_rn(x0, x1);
  const float2 fa = __bfloat1622float2(a);
  const float r0 = x0 - fa.x, r1 = x1 - fa.y;
  const __nv_bfloat162 b = __floats2bfloat162_rn(r0, r1);
  const float2 fb = __bfloat1622float2(b);
  const __nv_bfloat162 c = __floats2bfloat162_rn(r0 - fb.x, r1 - fb.y);
  h0 = *reinterpret_cast<const uint32_t*>(&a);
  h1 = *reinterpret_cast<const uint32_t*>(&b);
  h2 = *reinterpret_cast<const uint32_t*>(&c);
}

inline int grid_for(long long n, int block, int cap = 152 * 32) {
  long long g = (n + block - 1) / block;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace csg
