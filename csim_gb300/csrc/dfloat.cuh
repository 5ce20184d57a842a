// Double-float ("two-float") arithmetic for the CSG_PREC_HIGH transforms.
//
// A value is the unevaluated sum h + l of two fp32 words with |l| at most
// half an ulp of h, about 48 significant bits. Sums use Knuth's TwoSum and a
// fast renormalisation, products fmaf's exact product error (the classical
// double-single algorithms of Dekker and Knuth, as in Hida, Li and Bailey's
// double-double library, applied to fp32). A sum costs 11 fp32 operations
// and a product by a two-float constant 7, against 1 and 1 in fp32; a
// complex twiddle product 2 x 19.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace csg {

struct dfl {
  float h, l;
};

__device__ __forceinline__ dfl df_from(float v) { return dfl{v, 0.f}; }
__device__ __forceinline__ float df_round(dfl a) { return a.h + a.l; }

// s + e = a + b exactly, for |a| >= |b| (or a == 0).
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  dfl r;
  fast_two_sum(s, e, r.h, r.l);
  return r;
}
// a0 + b0 and a1 + b1 (or a - b) with the same operations as df_add, on
// packed fp32 pairs (add.rn.f32x2 / sub.rn.f32x2: the same round-to-nearest
// results per lane, one instruction for both sums).
__device__ __forceinline__ void df_add2(dfl a0, dfl a1, dfl b0, dfl b1, dfl& r0, dfl& r1) {
  asm("{\n\t.reg .b64 ah, al, bh, bl, s, bb, t, u, e, rh, rl;\n\t"
      "mov.b64 ah, {%4, %5};\n\tmov.b64 al, {%6, %7};\n\t"
      "mov.b64 bh, {%8, %9};\n\tmov.b64 bl, {%10, %11};\n\t"
      "add.rn.f32x2 s, ah, bh;\n\t"   // TwoSum(ah, bh)
      "sub.rn.f32x2 bb, s, ah;\n\t"
      "sub.rn.f32x2 t, s, bb;\n\t"
      "sub.rn.f32x2 t, ah, t;\n\t"
      "sub.rn.f32x2 u, bh, bb;\n\t"
      "add.rn.f32x2 e, t, u;\n\t"
      "add.rn.f32x2 u, al, bl;\n\t"   // + (al + bl)
      "add.rn.f32x2 e, e, u;\n\t"
      "add.rn.f32x2 rh, s, e;\n\t"    // fast TwoSum renormalisation
      "sub.rn.f32x2 u, rh, s;\n\t"
      "sub.rn.f32x2 rl, e, u;\n\t"
      "mov.b64 {%0, %1}, rh;\n\tmov.b64 {%2, %3}, rl;\n\t}"
      : "=f"(r0.h), "=f"(r1.h), "=f"(r0.l), "=f"(r1.l)
      : "f"(a0.h), "f"(a1.h), "f"(a0.l), "f"(a1.l), "f"(b0.h), "f"(b1.h), "f"(b0.l), "f"(b1.l));
}
__device__ __forceinline__ void df_sub2(dfl a0, dfl a1, dfl b0, dfl b1, dfl& r0, dfl& r1) {
  asm("{\n\t.reg .b64 ah, al, bh, bl, s, bb, t, u, e, rh, rl;\n\t"
      "mov.b64 ah, {%4, %5};\n\tmov.b64 al, {%6, %7};\n\t"
      "mov.b64 bh, {%8, %9};\n\tmov.b64 bl, {%10, %11};\n\t"
      "sub.rn.f32x2 s, ah, bh;\n\t"   // TwoSum(ah, -bh)
      "sub.rn.f32x2 bb, s, ah;\n\t"
      "sub.rn.f32x2 t, s, bb;\n\t"
      "sub.rn.f32x2 t, ah, t;\n\t"
      "add.rn.f32x2 u, bh, bb;\n\t"   // (-bh - bb) = -(bh + bb)
      "sub.rn.f32x2 e, t, u;\n\t"
      "sub.rn.f32x2 u, al, bl;\n\t"   // + (al - bl)
      "add.rn.f32x2 e, e, u;\n\t"
      "add.rn.f32x2 rh, s, e;\n\t"
      "sub.rn.f32x2 u, rh, s;\n\t"
      "sub.rn.f32x2 rl, e, u;\n\t"
      "mov.b64 {%0, %1}, rh;\n\tmov.b64 {%2, %3}, rl;\n\t}"
      : "=f"(r0.h), "=f"(r1.h), "=f"(r0.l), "=f"(r1.l)
      : "f"(a0.h), "f"(a1.h), "f"(a0.l), "f"(a1.l), "f"(b0.h), "f"(b1.h), "f"(b0.l), "f"(b1.l));
}
__device__ __forceinline__ dfl df_neg(dfl a) { return dfl{-a.h, -a.l}; }
__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ dfl df_scale(dfl a, float p2) { return dfl{a.h * p2, a.l * p2}; }

// (ar + i ai) (c + i s) with two-float c and s.
__device__ __forceinline__ void df_cmul(dfl ar, dfl ai, dfl c, dfl s, dfl& orr, dfl& oi) {
  {
    const float p1 = __fmul_rn(ar.h, c.h), p2 = __fmul_rn(ai.h, s.h);
    const float e1 = fmaf(ar.h, c.h, -p1), e2 = fmaf(ai.h, s.h, -p2);
    float S, E;
    two_sum(p1, -p2, S, E);
    E = __fadd_rn(E, __fsub_rn(e1, e2));
    E = fmaf(ar.h, c.l, E);
    E = fmaf(ar.l, c.h, E);
    E = fmaf(-ai.h, s.l, E);
    E = fmaf(-ai.l, s.h, E);
    fast_two_sum(S, E, orr.h, orr.l);
  }
  {
    const float p1 = __fmul_rn(ar.h, s.h), p2 = __fmul_rn(ai.h, c.h);
    const float e1 = fmaf(ar.h, s.h, -p1), e2 = fmaf(ai.h, c.h, -p2);
    float S, E;
    two_sum(p1, p2, S, E);
    E = __fadd_rn(E, __fadd_rn(e1, e2));
    E = fmaf(ar.h, s.l, E);
    E = fmaf(ar.l, s.h, E);
    E = fmaf(ai.h, c.l, E);
    E = fmaf(ai.l, c.h, E);
    fast_two_sum(S, E, oi.h, oi.l);
  }
}

// FP64 value -> two-float (hi the fp32 rounding, lo the fp32 rounding of the rest).
__host__ __device__ inline float2 split_f64(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}

}  // namespace csg
