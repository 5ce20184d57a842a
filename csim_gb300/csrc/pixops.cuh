// Per-pixel element operations fused into the prologue or epilogue of the
// pass that already reads or writes the field (FFT passes, the MFT operand
// split, or one standalone elementwise pass). Each op is one reference
// element applied to one pixel:
//   OP_SOURCE  efield::init_point_sources (efield.cpp:179-206): replaces the
//              pixel by amp exp(2 pi i (2 x tip / Lx + 2 y tilt / Ly))
//   OP_MASK    mask::execute (mask.cpp:38-46): * m, or * (m + i m)
//   OP_PHASE   mirror / deformableMirror: * exp(-sign 4 pi i sag / lambda)
//   OP_CMASK   complexMask (complexMask.cpp:24-55): centred amp exp(-i ph)
// Phases are products of an fp32 datum and an FP64 per-field constant held
// as an fp32 (hi, lo) pair, reduced modulo one turn with the product's
// rounding error folded back (fmaf).
#pragma once
#include "common.cuh"

namespace csg {

// OP_PHASOR multiplies by a precomputed per-wavelength phasor table
// (float2 [slot][R][C], the reference's mirrorPhase cube, mirror.cpp:66-72),
// indexed by the field's wavelength slot.
enum PixOpKind { OP_SOURCE = 1, OP_MASK = 2, OP_PHASE = 3, OP_CMASK = 4, OP_PHASOR = 5 };
constexpr int MAX_PIXOPS = 6;

struct PixOps {
  int n = 0;
  int kind[MAX_PIXOPS] = {};
  const float* a[MAX_PIXOPS] = {};  // mask, sag or amplitude
  const float* b[MAX_PIXOPS] = {};  // phase of a complex mask
  float param[MAX_PIXOPS] = {};     // OP_MASK: quirk flag; OP_PHASE: mirror sign
  int mr[MAX_PIXOPS] = {}, mc[MAX_PIXOPS] = {};
};

// Per-field inputs the ops need (device arrays indexed by field).
struct FieldInfo {
  const double* lam = nullptr;
  const double* amp = nullptr;
  const double* tip = nullptr;
  const double* tilt = nullptr;
  const int* slot = nullptr;  // wavelength slot (OP_PHASOR tables)
};

// Per-field constants, computed once per CTA.
struct PixConsts {
  float khi[MAX_PIXOPS], klo[MAX_PIXOPS];  // OP_PHASE turns per metre
  float sxh, sxl, syh, syl, amp;           // OP_SOURCE
  int slot;                                // OP_PHASOR table
};

__device__ __forceinline__ float frac_prod(float a, float khi, float klo) {
  const float p = a * khi;
  float e = fmaf(a, khi, -p);
  e = fmaf(a, klo, e);
  return (p - rintf(p)) + e;
}

__device__ __forceinline__ void split_f64_pair(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

__device__ __forceinline__ void pix_consts(const PixOps& ops, const FieldInfo& fi, int f, int R,
                                           int C, PixConsts& k) {
  k.slot = fi.slot ? fi.slot[f] : 0;
#pragma unroll
  for (int i = 0; i < MAX_PIXOPS; ++i) {
    if (i >= ops.n) break;
    if (ops.kind[i] == OP_PHASE) {
      split_f64_pair(-(double)ops.param[i] * 2.0 / fi.lam[f], k.khi[i], k.klo[i]);
    } else if (ops.kind[i] == OP_SOURCE) {
      split_f64_pair(2.0 * fi.tip[f] / (double)C, k.sxh, k.sxl);
      split_f64_pair(2.0 * fi.tilt[f] / (double)R, k.syh, k.syl);
      k.amp = (float)fi.amp[f];
    }
  }
}

// CTA-wide per-field constants: one thread evaluates the FP64 expressions,
// the rest read them after a barrier (every thread of the CTA must call it,
// and the CTA must cover a single field).
__device__ __forceinline__ void pix_consts_cta(const PixOps& ops, const FieldInfo& fi, int f, int R,
                                               int C, PixConsts& k, PixConsts* shared) {
  if (threadIdx.x == 0) pix_consts(ops, fi, f, R, C, *shared);
  __syncthreads();
  k = *shared;
}

__device__ __forceinline__ float pick(const float* v, int i) {
  float x = v[0];
#pragma unroll
  for (int j = 1; j < MAX_PIXOPS; ++j)
    if (i == j) x = v[j];
  return x;
}

// OP_SOURCE for NE pixels (r + e dr, c + e dc): replaces them by the point
// source's field (flat for an on-axis source).
template <int NE>
__device__ __forceinline__ void pix_source_n(const PixConsts& k, int r, int c, int dr, int dc,
                                             int R, int C, float* re, float* im) {
  if (k.sxh == 0.f && k.syh == 0.f && k.sxl == 0.f && k.syl == 0.f) {
#pragma unroll
    for (int e = 0; e < NE; ++e) re[e] = k.amp, im[e] = 0.f;
  } else {
#pragma unroll
    for (int e = 0; e < NE; ++e) {
      const float xc = (float)(c + e * dc) - 0.5f * (float)(C - 1);
      const float yr = (float)(r + e * dr) - 0.5f * (float)(R - 1);
      float t = frac_prod(xc, k.sxh, k.sxl) + frac_prod(yr, k.syh, k.syl);
      t -= rintf(t);
      float s, co;
      sincospif(2.f * t, &s, &co);
      re[e] = k.amp * co;
      im[e] = k.amp * s;
    }
  }
}

// Apply the ops to NE pixels (r + e dr, c + e dc), e < NE, of an R x C field
// held in registers. Ops are applied one at a time over all NE pixels, so
// each op's NE table reads are issued together. OP_SOURCE is only ever the
// first op (it replaces the pixel) and is applied before the op loop: its
// per-pixel phase does not depend on the op, and inside the loop the
// compiler would hoist that arithmetic out of it and evaluate it for every
// op program, with or without a source.
template <int NE>
__device__ __forceinline__ void pix_apply_n(const PixOps& ops, const PixConsts& k, int r, int c,
                                            int dr, int dc, int R, int C, float* re, float* im) {
  int i0 = 0;
  if (ops.n && ops.kind[0] == OP_SOURCE) {
    pix_source_n<NE>(k, r, c, dr, dc, R, C, re, im);
    i0 = 1;
  }
#pragma unroll 1
  for (int i = i0; i < ops.n; ++i) {
    const int kind = ops.kind[i];
    const float* a = ops.a[i];
    if (kind == OP_SOURCE) {
      continue;  // never past the first op
    } else if (kind == OP_MASK) {
      float m[NE];
#pragma unroll
      for (int e = 0; e < NE; ++e) m[e] = __ldg(&a[(size_t)(r + e * dr) * C + c + e * dc]);
      if (ops.param[i] != 0.f) {
#pragma unroll
        for (int e = 0; e < NE; ++e) {
          const float t = m[e] * (re[e] - im[e]);
          im[e] = m[e] * (re[e] + im[e]);
          re[e] = t;
        }
      } else {
#pragma unroll
        for (int e = 0; e < NE; ++e) re[e] *= m[e], im[e] *= m[e];
      }
    } else if (kind == OP_PHASE) {
      const float khi = pick(k.khi, i), klo = pick(k.klo, i);
      float sg[NE];
#pragma unroll
      for (int e = 0; e < NE; ++e) sg[e] = __ldg(&a[(size_t)(r + e * dr) * C + c + e * dc]);
#pragma unroll
      for (int e = 0; e < NE; ++e) {
        float s, co;
        sincospif(2.f * frac_prod(sg[e], khi, klo), &s, &co);
        const float xr = re[e];
        re[e] = xr * co - im[e] * s;
        im[e] = xr * s + im[e] * co;
      }
    } else if (kind == OP_PHASOR) {
      const float2* w = reinterpret_cast<const float2*>(a) + (size_t)k.slot * R * C;
      float2 wv[NE];
#pragma unroll
      for (int e = 0; e < NE; ++e) wv[e] = __ldg(&w[(size_t)(r + e * dr) * C + c + e * dc]);
#pragma unroll
      for (int e = 0; e < NE; ++e) {
        const float xr = re[e];
        re[e] = xr * wv[e].x - im[e] * wv[e].y;
        im[e] = xr * wv[e].y + im[e] * wv[e].x;
      }
    } else if (kind == OP_CMASK) {
      const int r0 = R / 2 - ops.mr[i] / 2, c0 = C / 2 - ops.mc[i] / 2;
#pragma unroll
      for (int e = 0; e < NE; ++e) {
        const int rr = r + e * dr - r0, cc = c + e * dc - c0;
        if (rr >= 0 && rr < ops.mr[i] && cc >= 0 && cc < ops.mc[i]) {
          const size_t o = (size_t)rr * ops.mc[i] + cc;
          float s, co;
          sincosf(-ops.b[i][o], &s, &co);
          const float am = a[o];
          const float xr = re[e];
          re[e] = am * (xr * co - im[e] * s);
          im[e] = am * (xr * s + im[e] * co);
        }
      }
    }
  }
}

// Apply the ops to pixel (r, c) of an R x C field.
__device__ __forceinline__ void pix_apply(const PixOps& ops, const PixConsts& k, int r, int c,
                                          int R, int C, float& re, float& im) {
#pragma unroll
  for (int i = 0; i < MAX_PIXOPS; ++i) {  // static indices keep k in registers
    if (i >= ops.n) break;
    const int kind = ops.kind[i];
    if (kind == OP_SOURCE && k.sxh == 0.f && k.syh == 0.f && k.sxl == 0.f && k.syl == 0.f) {
      re = k.amp;  // on-axis source: flat phase
      im = 0.f;
    } else if (kind == OP_SOURCE) {
      const float xc = (float)c - 0.5f * (float)(C - 1);
      const float yr = (float)r - 0.5f * (float)(R - 1);
      float t = frac_prod(xc, k.sxh, k.sxl) + frac_prod(yr, k.syh, k.syl);
      t -= rintf(t);
      float s, co;
      sincospif(2.f * t, &s, &co);
      re = k.amp * co;
      im = k.amp * s;
    } else if (kind == OP_MASK) {
      const float m = ops.a[i][(size_t)r * C + c];
      if (ops.param[i] != 0.f) {
        const float t = m * (re - im);
        im = m * (re + im);
        re = t;
      } else {
        re *= m;
        im *= m;
      }
    } else if (kind == OP_PHASE) {
      const float t = frac_prod(ops.a[i][(size_t)r * C + c], k.khi[i], k.klo[i]);
      float s, co;
      sincospif(2.f * t, &s, &co);
      const float xr = re;
      re = xr * co - im * s;
      im = xr * s + im * co;
    } else if (kind == OP_PHASOR) {
      const float2 w = reinterpret_cast<const float2*>(ops.a[i])[((size_t)k.slot * R + r) * C + c];
      const float xr = re;
      re = xr * w.x - im * w.y;
      im = xr * w.y + im * w.x;
    } else if (kind == OP_CMASK) {
      const int r0 = R / 2 - ops.mr[i] / 2, c0 = C / 2 - ops.mc[i] / 2;
      const int rr = r - r0, cc = c - c0;
      if (rr >= 0 && rr < ops.mr[i] && cc >= 0 && cc < ops.mc[i]) {
        const size_t o = (size_t)rr * ops.mc[i] + cc;
        float s, co;
        sincosf(-ops.b[i][o], &s, &co);
        const float a = ops.a[i][o];
        const float xr = re;
        re = a * (xr * co - im * s);
        im = a * (xr * s + im * co);
      }
    }
  }
}

// Standalone pass: field [F][2][R][C] <- ops(field).
int pixops_pass(cudaStream_t st, float* field, int F, int R, int C, const PixOps& ops,
                const FieldInfo& fi);

// out [F][2][P][P] <- n x n fields ops(in) embedded at the centre of zeros;
// crop: out [F][2][n][n] <- the centred n x n block of P x P fields.
int pad_center_pass(cudaStream_t st, const float* in, float* out, int F, int n, int P,
                    const PixOps& ops, const FieldInfo& fi);
int crop_center_pass(cudaStream_t st, const float* in, float* out, int F, int n, int P);

struct FresnelArgs {
  const double* lambda;           // per field
  double z;
  double ap_rad;
  const float2* H = nullptr;      // optional transfer-function table [slot][N][N]
  const int* slot = nullptr;      // per field, with H or H4
  // two-float transfer-function table [slot][N][N] (cos hi, cos lo, sin hi,
  // sin lo): required by the two-float (CSG_PREC_HIGH) passes
  const float4* H4 = nullptr;
};

// Per-wavelength tables, built once per chain in FP64-reduced phases:
// mirror phasors exp(-sign 4 pi i sag / lambda_s) and Fresnel transfer
// functions H_s (same arithmetic as the in-kernel evaluations).
int build_phasor_table(cudaStream_t st, const float* sag, int R, int C, const double* lam,
                       int n_slot, double sign, float2* out);
int build_fresnel_table(cudaStream_t st, int N, const double* lam, int n_slot, double z,
                        double ap_rad, float2* out);
// The same in FP64, stored two-float (the CSG_PREC_HIGH Fresnel).
int build_fresnel_table_df(cudaStream_t st, int N, const double* lam, int n_slot, double z,
                           double ap_rad, float4* out);
// Two-float copy (low words zero) of an fp32 complex table of n values.
int table_to_df(cudaStream_t st, const float2* in, float4* out, long long n);

// Band-limited padded transform (with fa only): the n x n field src sits at
// rows and columns [lo, lo + n) of zero-padded N x N fields. The first row
// pass transforms only those rows, reading them straight from src (the zero
// columns are generated); the column pass loads and stores only the band's
// rows (the others are zero on input and unused on output); the last row
// pass transforms the band's rows and writes their centre columns straight
// to dst (n x n). lo and n must be multiples of the transform's threads per
// row and column.
struct FftBand {
  int lo = 0, n = 0;
  const float* src = nullptr;
  float* dst = nullptr;
  // inverse row pass only: also store the three-part bf16 split of the
  // result, [F][3][2][N][N] (an MFT's operand layout), beside the fp32 field
  __nv_bfloat16* split = nullptr;
};

// 2-D FFT (direction -1 / +1) or, with fa, Fresnel propagation of F square
// N x N fields with element ops fused before (pro) and after (epi).
// support (with fa only; lo and n, no src or dst): the field is zero outside
// rows [lo, lo + n) once pro is applied (a mask's support), so the first row
// pass transforms only those rows and the column pass reads only them; the
// other rows of the field are not read before they are overwritten.
// split_out (with fa, without band): the last pass also writes the result's
// three-part bf16 split in the layout of an N x N MFT's input (mft_split_buffer).
// high: the transforms run in two-float arithmetic (CSG_PREC_HIGH; a Fresnel
// then reads fa->H4 and split_out is not available).
int fft2d_fused(csg_ctx* ctx, float* field, int F, int n, int direction, const FresnelArgs* fa,
                const PixOps& pro, const PixOps& epi, const FieldInfo& fi,
                const FftBand* band = nullptr, const FftBand* support = nullptr,
                __nv_bfloat16* split_out = nullptr, bool high = false);
// Sizes that are not powers of two: the 2-D DFT runs as a matrix Fourier
// transform; dft_prepare creates its plans and buffers for F fields
// (allocates, so before any graph capture).
bool fft_is_dft_size(int n);
int dft_prepare(csg_ctx* ctx, int n, int F, bool high);
// Whether fft2d_fused can run an N-point padded transform band-limited to
// [lo, lo + n) (fp32 or two-float passes).
bool fft_band_supported(int N, int lo, int n, bool high = false);
// Rows [r0, r1) widened to a band fft2d_fused accepts as a row support
// (false: none).
bool fft_row_support(int N, int r0, int r1, int* lo, int* n, bool high = false);

// A window of a field: rows x cols of the transform start at (r0, c0) of
// planes that are `rows` x `pitch`.
struct MftWindow {
  int r0, c0, rows, pitch;
};

// MFT with element ops applied to the input in the operand split; the input
// and output may be windows of larger fields (nullptr: the whole plane), and
// output field f may read input field in_idx[f] (device, nullptr: f).
int mft_execute_ops(csg_ctx* ctx, csg_mft* m, const float* in, float* out, int n_fields,
                    const int* slot, int accumulate, const float* in_mul, const int* mul_idx,
                    const PixOps& pre, const FieldInfo& fi, const MftWindow* iw = nullptr,
                    const MftWindow* ow = nullptr, const int* in_idx = nullptr,
                    bool presplit = false, float* out_lo = nullptr);
// Whether a plan runs at CSG_PREC_HIGH (its input split is exponent-aligned,
// so a producer must not hand it a plain split).
bool mft_is_high(const csg_mft* m);
// The plan's input split buffer, [n_fields][3][2][ny][nx] bf16, grown to
// n_fields (nullptr: allocation failed). A producer that writes it lets
// mft_execute_ops run with presplit = true, which skips the split pass.
__nv_bfloat16* mft_split_buffer(csg_mft* m, int n_fields);
// Input rows and columns of a plan.
void mft_input_shape(const csg_mft* m, int* ny, int* nx);

}  // namespace csg
