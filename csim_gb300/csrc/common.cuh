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

// Exponent-aligned three-way split (CSG_PREC_HIGH). All values of one
// 64-wide K group of an operand row share the grid g = 2^(e - 8), where
// 2^e bounds the group's largest magnitude: hi = rint(v / g) g is an integer
// multiple of g with |hi / g| <= 256 (exact in bf16), and mid, lo are the
// ordinary bf16 rounding of what is left (v - hi is exact in fp32). Every
// hi x hi product of one K group then lies on the grid g_a g_b and a group's
// sum (at most 64 * 2^16 grid units) is an integer below 2^24 units, so the
// tensor core accumulates it without any rounding.
struct Grid {
  float g, inv;
};
// Grid of a group whose largest |value| has the fp32 bit pattern maxbits
// (non-negative). Groups below 2^-100 use the grid of 2^-100.
__device__ __forceinline__ Grid grid_of(uint32_t maxbits) {
  int e = (int)(maxbits >> 23);  // biased exponent: max < 2^(e - 126)
  e = e < 27 ? 27 : e;
  Grid r;
  r.g = __int_as_float((e - 7) << 23);     // 2^(e - 134)
  r.inv = __int_as_float((261 - e) << 23);  // 2^(134 - e)
  return r;
}
__device__ __forceinline__ uint32_t absbits(float v) { return __float_as_uint(v) & 0x7fffffffu; }

__device__ __forceinline__ void split3_aligned(float v, const Grid& gr, __nv_bfloat16& a,
                                               __nv_bfloat16& b, __nv_bfloat16& c) {
  const float h = rintf(v * gr.inv) * gr.g;
  a = __float2bfloat16_rn(h);
  const float r = v - h;
  b = __float2bfloat16_rn(r);
  c = __float2bfloat16_rn(r - __bfloat162float(b));
}
// The same for a two-float value v + w (|w| below half an ulp of v): the
// low word joins the remainder.
__device__ __forceinline__ void split3_aligned2(float v, float w, const Grid& gr,
                                                __nv_bfloat16& a, __nv_bfloat16& b,
                                                __nv_bfloat16& c) {
  const float h = rintf(v * gr.inv) * gr.g;
  a = __float2bfloat16_rn(h);
  const float r = (v - h) + w;
  b = __float2bfloat16_rn(r);
  c = __float2bfloat16_rn(r - __bfloat162float(b));
}
// Two values on one grid, packed as split3_pair packs them.
__device__ __forceinline__ void split3_aligned_pair(float x0, float x1, const Grid& gr,
                                                    uint32_t& h0, uint32_t& h1, uint32_t& h2) {
  const float a0 = rintf(x0 * gr.inv) * gr.g, a1 = rintf(x1 * gr.inv) * gr.g;
  const __nv_bfloat162 a = __floats2bfloat162_rn(a0, a1);
  const float r0 = x0 - a0, r1 = x1 - a1;
  const __nv_bfloat162 b = __floats2bfloat162_rn(r0, r1);
  const float2 fb = __bfloat1622float2(b);
  const __nv_bfloat162 c = __floats2bfloat162_rn(r0 - fb.x, r1 - fb.y);
  h0 = *reinterpret_cast<const uint32_t*>(&a);
  h1 = *reinterpret_cast<const uint32_t*>(&b);
  h2 = *reinterpret_cast<const uint32_t*>(&c);
}

// Error-free sum: s + e = a + b exactly (Knuth's TwoSum, no ordering needed).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Whether every value of a host array is finite (CSG_E_NAN checks).
inline bool all_finite(const double* v, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!(v[i] - v[i] == 0.0)) return false;
  return true;
}

inline int grid_for(long long n, int block, int cap = 152 * 32) {
  long long g = (n + block - 1) / block;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace csg
