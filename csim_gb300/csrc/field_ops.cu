// Element field operations (HBM-bound elementwise / gather kernels) and the
// intensity / dark-hole reductions.
//
// The single-element calls (point source, mask, mirror phase, complex mask)
// are one standalone pass of the fused element machinery (pixops.cuh); the
// chain executor instead folds them into the FFT and MFT passes.
#include "ctx.hpp"
#include "pixops.cuh"

namespace csg {

// ----------------------------------------------------- standalone element pass
// 4 consecutive pixels per thread (float4 when the row length allows).
__global__ void k_pixops(float* __restrict__ field, int R, int C, PixOps ops, FieldInfo fi) {
  const int f = blockIdx.y;
  const int plane = R * C;
  PixConsts k;
  pix_consts(ops, fi, f, R, C, k);
  float* re = field + (size_t)f * 2 * plane;
  float* im = re + plane;
  const bool gen = ops.n && ops.kind[0] == OP_SOURCE;
  if ((C & 3) == 0) {
    const int nv = plane / 4;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
      float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
      if (!gen) {
        a = reinterpret_cast<const float4*>(re)[v];
        b = reinterpret_cast<const float4*>(im)[v];
      }
      const int e0 = 4 * v, r = e0 / C, c = e0 % C;
      float xr[4] = {a.x, a.y, a.z, a.w}, xi[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int q = 0; q < 4; ++q) pix_apply(ops, k, r, c + q, R, C, xr[q], xi[q]);
      reinterpret_cast<float4*>(re)[v] = make_float4(xr[0], xr[1], xr[2], xr[3]);
      reinterpret_cast<float4*>(im)[v] = make_float4(xi[0], xi[1], xi[2], xi[3]);
    }
  } else {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += gridDim.x * blockDim.x) {
      float xr = gen ? 0.f : re[i], xi = gen ? 0.f : im[i];
      pix_apply(ops, k, i / C, i % C, R, C, xr, xi);
      re[i] = xr;
      im[i] = xi;
    }
  }
}

// Mirror phasor table [slot][R][C]: exp(-sign 4 pi i sag / lambda_s), the
// same fp32 arithmetic as OP_PHASE.
__global__ void k_phasor_table(const float* __restrict__ sag, int plane, const double* lam,
                               double sign, float2* __restrict__ out) {
  const int s = blockIdx.y;
  float kh, kl;
  split_f64_pair(-sign * 2.0 / lam[s], kh, kl);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += gridDim.x * blockDim.x) {
    const float t = frac_prod(sag[i], kh, kl);
    float sn, cs;
    sincospif(2.f * t, &sn, &cs);
    out[(size_t)s * plane + i] = make_float2(cs, sn);
  }
}

int build_phasor_table(cudaStream_t st, const float* sag, int R, int C, const double* lam,
                       int n_slot, double sign, float2* out) {
  dim3 grid(grid_for((long long)R * C, 256, 1024), n_slot);
  k_phasor_table<<<grid, 256, 0, st>>>(sag, R * C, lam, sign, out);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

// Zero-padded embedding: out [F][2][P][P] = 0 except the centred n x n block
// at offset o = (P - n) / 2, which holds ops(in) (the ops see the n x n
// field's own coordinates). fpmPupToLyot.cpp:112-118 embeds at [N/2, 3N/2)
// the same way for P = 2N. Four pixels per thread (n, P multiples of 4).
__global__ void k_pad_center(const float* __restrict__ in, float* __restrict__ out, int n,
                             int lp, PixOps ops, FieldInfo fi) {
  const int f = blockIdx.y;
  const int P = 1 << lp, o = (P - n) / 2;
  const size_t pplane = (size_t)P * P, nplane = (size_t)n * n;
  PixConsts k;
  if (ops.n) pix_consts(ops, fi, f, n, n, k);
  const bool gen = ops.n && ops.kind[0] == OP_SOURCE;
  const float* ire = in + (size_t)f * 2 * nplane;
  const float* iim = ire + nplane;
  float* ore = out + (size_t)f * 2 * pplane;
  float* oim = ore + pplane;
  const long long nv = (long long)pplane / 4;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv;
       v += (long long)gridDim.x * blockDim.x) {
    const int r = (int)((4 * v) >> lp), c = (int)((4 * v) & (P - 1));
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    const int rr = r - o, cc = c - o;
    if (rr >= 0 && rr < n && cc >= 0 && cc < n) {
      if (!gen) {
        a = *reinterpret_cast<const float4*>(ire + (size_t)rr * n + cc);
        b = *reinterpret_cast<const float4*>(iim + (size_t)rr * n + cc);
      }
      if (ops.n) {
        float xr[4] = {a.x, a.y, a.z, a.w}, xi[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) pix_apply(ops, k, rr, cc + q, n, n, xr[q], xi[q]);
        a = make_float4(xr[0], xr[1], xr[2], xr[3]);
        b = make_float4(xi[0], xi[1], xi[2], xi[3]);
      }
    }
    reinterpret_cast<float4*>(ore)[v] = a;
    reinterpret_cast<float4*>(oim)[v] = b;
  }
}

// The centred n x n block of P x P fields (fpmPupToLyot.cpp:154-157).
__global__ void k_crop_center(const float* __restrict__ in, float* __restrict__ out, int n,
                              int P) {
  const int f = blockIdx.y;
  const int o = (P - n) / 2;
  const size_t pplane = (size_t)P * P, nplane = (size_t)n * n;
  const long long nv = (long long)nplane / 4 * 2;  // both planes
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv;
       v += (long long)gridDim.x * blockDim.x) {
    const int d = (int)(v / (nplane / 4));
    const long long e0 = 4 * (v % (long long)(nplane / 4));
    const int r = (int)(e0 / n), c = (int)(e0 % n);
    const float4 x = *reinterpret_cast<const float4*>(in + ((size_t)f * 2 + d) * pplane +
                                                      (size_t)(r + o) * P + c + o);
    *reinterpret_cast<float4*>(out + ((size_t)f * 2 + d) * nplane + e0) = x;
  }
}

int pad_center_pass(cudaStream_t st, const float* in, float* out, int F, int n, int P,
                    const PixOps& ops, const FieldInfo& fi) {
  CSG_CHECK(F > 0 && F < 65536 && n % 4 == 0 && P >= n && (P & (P - 1)) == 0 && (P - n) % 8 == 0,
            CSG_E_SHAPE, "pad: bad shape");
  int lp = 0;
  while ((1 << lp) < P) ++lp;
  dim3 grid(grid_for((long long)P * P / 4, 256, 2048), F);
  k_pad_center<<<grid, 256, 0, st>>>(in, out, n, lp, ops, fi);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

int crop_center_pass(cudaStream_t st, const float* in, float* out, int F, int n, int P) {
  CSG_CHECK(F > 0 && F < 65536 && n % 4 == 0 && P >= n && (P - n) % 8 == 0, CSG_E_SHAPE,
            "crop: bad shape");
  dim3 grid(grid_for((long long)n * n / 2, 256, 1024), F);
  k_crop_center<<<grid, 256, 0, st>>>(in, out, n, P);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

int pixops_pass(cudaStream_t st, float* field, int F, int R, int C, const PixOps& ops,
                const FieldInfo& fi) {
  if (!ops.n) return CSG_OK;
  CSG_CHECK(F > 0 && F < 65536 && (long long)R * C < (1LL << 31), CSG_E_SHAPE,
            "element pass: bad shape");
  dim3 grid(grid_for((long long)R * C / 4 + 1, 256, 1024), F);
  k_pixops<<<grid, 256, 0, st>>>(field, R, C, ops, fi);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

// ------------------------------------------------------------- hex FPM
// Per (output j, hex h): cis(phaseSign * 2 * sag / lambda turns) in FP64;
// slot n_hex holds the value for pixels outside every hex (sag 0 -> 1).
__global__ void k_hex_phasors(float2* __restrict__ ph, const double* __restrict__ sags, int n_hex,
                              int n_out, const int* __restrict__ cand,
                              const double* __restrict__ lambda, double phase_sign) {
  const long long n = (long long)n_out * (n_hex + 1);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(i / (n_hex + 1)), h = (int)(i % (n_hex + 1));
    double sag = h < n_hex ? sags[(long long)cand[j] * n_hex + h] : 0.0;
    double t = phase_sign * 2.0 * sag / lambda[j];
    t -= rint(t);
    double s, c;
    sincospi(2.0 * t, &s, &c);
    ph[i] = make_float2((float)c, (float)s);
  }
}

__global__ void k_hex_mask(const int16_t* __restrict__ hex_id, const uint16_t* __restrict__ count,
                           int S, float inv_nsub2, const float2* __restrict__ ph, int n_hex,
                           int n_out, int flip, float subtract, int only, float* __restrict__ out) {
  const long long plane = (long long)S * S;
  const long long n = plane * n_out;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(i / plane);
    const long long o = i % plane;
    const int r = (int)(o / S), c = (int)(o % S);
    const long long src = (long long)r * S + (flip ? (S - 1 - c) : c);
    float mr = 0.f, mi = 0.f;
    const float2* phj = ph + (long long)j * (n_hex + 1);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int id = hex_id[k * plane + src];
      float w = (float)count[k * plane + src];
      if (only >= 0) {
        const bool keep = (id == only) || (only == n_hex && id == -1);
        if (!keep) w = 0.f;
      }
      if (w != 0.f) {
        const float2 p = phj[id >= 0 ? id : n_hex];
        mr += w * p.x;
        mi += w * p.y;
      }
    }
    float* base = out + (long long)j * 2 * plane + o;
    base[0] = mr * inv_nsub2 - subtract;
    base[plane] = mi * inv_nsub2;
  }
}

// --------------------------------------------------------- reductions
template <typename T>
__device__ T block_reduce_sum(T v, T* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = threadIdx.x < nw ? sh[threadIdx.x] : T(0);
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ T block_reduce_max(T v, T* sh) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = threadIdx.x < nw ? sh[threadIdx.x] : T(0);
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// One CTA per group: I = sum over the group's fields of |E|^2 at the region
// pixels, reduced by mean (mode 0) or max (mode 1), FP64.
__global__ void k_region_reduce(const float* __restrict__ field, long long plane, int per_group,
                                const int* __restrict__ pix, int n_pix, int mode, double scale,
                                double* __restrict__ out) {
  __shared__ double sh[32];
  const int g = blockIdx.x;
  double acc = 0.0;
  for (int p = threadIdx.x; p < n_pix; p += blockDim.x) {
    const long long o = pix[p];
    double ip = 0.0;
    for (int k = 0; k < per_group; ++k) {
      const float* re = field + ((long long)g * per_group + k) * 2 * plane;
      const double a = re[o], b = re[plane + o];
      ip += a * a + b * b;
    }
    acc = mode == 0 ? acc + ip : fmax(acc, ip);
  }
  acc = mode == 0 ? block_reduce_sum(acc, sh) : block_reduce_max(acc, sh);
  if (threadIdx.x == 0) out[g] = (mode == 0 ? acc / (double)n_pix : acc) * scale;
}

__global__ void k_intensity(const float* __restrict__ field, long long plane, int F,
                            double* __restrict__ out, unsigned long long* __restrict__ out_max) {
  __shared__ double sh[32];
  double m = 0.0;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < plane;
       o += (long long)gridDim.x * blockDim.x) {
    double ip = 0.0;
    for (int f = 0; f < F; ++f) {
      const float* re = field + (long long)f * 2 * plane;
      const double a = re[o], b = re[plane + o];
      ip += a * a + b * b;
    }
    out[o] = ip;
    m = fmax(m, ip);
  }
  m = block_reduce_max(m, sh);
  // non-negative doubles order like their bit patterns
  if (threadIdx.x == 0 && out_max) atomicMax(out_max, (unsigned long long)__double_as_longlong(m));
}

// Hex mask with a caller-provided phasor buffer [n_out][n_hex + 1] (used by
// the chain executor, which owns that buffer).
// The mask on a sub-rectangle [r0, r0 + RR) x [c0, c0 + CC) of the (flipped)
// S x S mask grid, written as [n_out][2][RR][CC]: the chain evaluates the
// Babinet term only where fliplr(M) - 1 can be nonzero.
__global__ void k_hex_mask_region(const int16_t* __restrict__ hex_id,
                                  const uint16_t* __restrict__ count, int S, int r0, int c0, int RR,
                                  int CC, float inv_nsub2, const float2* __restrict__ ph, int n_hex,
                                  int flip, float subtract, float* __restrict__ out) {
  const int j = blockIdx.y;
  const int plane = RR * CC;
  const size_t splane = (size_t)S * S;
  const float2* phj = ph + (size_t)j * (n_hex + 1);
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < plane; o += gridDim.x * blockDim.x) {
    const int r = r0 + o / CC, c = c0 + o % CC;
    const size_t src = (size_t)r * S + (flip ? (S - 1 - c) : c);
    float mr = 0.f, mi = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int id = hex_id[k * splane + src];
      const float w = (float)count[k * splane + src];
      if (w != 0.f) {
        const float2 p = phj[id >= 0 ? id : n_hex];
        mr += w * p.x;
        mi += w * p.y;
      }
    }
    float* base = out + (size_t)j * 2 * plane + o;
    base[0] = mr * inv_nsub2 - subtract;
    base[plane] = mi * inv_nsub2;
  }
}

int hex_mask_region(csg_ctx* ctx, const int16_t* hex_id, const uint16_t* count, int S, int r0,
                    int c0, int RR, int CC, int n_sub, const double* sags, int n_hex, int n_out,
                    const int* cand, const double* lambda, double phase_sign, int flip,
                    double subtract, float* out, float2* phasors) {
  cudaStream_t st = ctx->stream;
  k_hex_phasors<<<grid_for((long long)n_out * (n_hex + 1), 256), 256, 0, st>>>(
      phasors, sags, n_hex, n_out, cand, lambda, phase_sign);
  CSG_LAUNCH_CHECK();
  dim3 grid(grid_for((long long)RR * CC, 256, 256), n_out);
  k_hex_mask_region<<<grid, 256, 0, st>>>(hex_id, count, S, r0, c0, RR, CC,
                                          1.f / (float)(n_sub * n_sub), phasors, n_hex, flip,
                                          (float)subtract, out);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

int hex_mask_with_phasor_buffer(csg_ctx* ctx, const int16_t* hex_id, const uint16_t* count, int S,
                                int n_sub, const double* sags, int n_hex, int n_out,
                                const int* cand, const double* lambda, double phase_sign, int flip,
                                double subtract, int use_only_hex, float* out, float2* phasors) {
  cudaStream_t st = ctx->stream;
  k_hex_phasors<<<grid_for((long long)n_out * (n_hex + 1), 256), 256, 0, st>>>(
      phasors, sags, n_hex, n_out, cand, lambda, phase_sign);
  CSG_LAUNCH_CHECK();
  k_hex_mask<<<grid_for((long long)S * S * n_out, 256), 256, 0, st>>>(
      hex_id, count, S, 1.f / (float)(n_sub * n_sub), phasors, n_hex, n_out, flip,
      (float)subtract, use_only_hex, out);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

}  // namespace csg

using namespace csg;

extern "C" {

int csg_point_source(csg_ctx* ctx, float* field, int n_fields, int rows, int cols, double dx,
                     double dy, const double* amp, const double* tip, const double* tilt) {
  CSG_CHECK(ctx && field && amp && tip && tilt, CSG_E_ARG, "csg_point_source: null argument");
  CSG_CHECK(n_fields > 0 && rows > 0 && cols > 0, CSG_E_SHAPE, "csg_point_source: bad shape");
  (void)dx;
  (void)dy;  // the phase depends on the pixel index only (x / Lx = index / C)
  DeviceGuard g(ctx->device);
  PixOps ops;
  ops.n = 1;
  ops.kind[0] = OP_SOURCE;
  FieldInfo fi;
  fi.amp = amp;
  fi.tip = tip;
  fi.tilt = tilt;
  return pixops_pass(ctx->stream, field, n_fields, rows, cols, ops, fi);
}

int csg_mask_real(csg_ctx* ctx, float* field, int n_fields, int rows, int cols, const float* mask,
                  int ref_quirk) {
  CSG_CHECK(ctx && field && mask, CSG_E_ARG, "csg_mask_real: null argument");
  CSG_CHECK(n_fields > 0 && rows > 0 && cols > 0, CSG_E_SHAPE, "csg_mask_real: bad shape");
  DeviceGuard g(ctx->device);
  PixOps ops;
  ops.n = 1;
  ops.kind[0] = OP_MASK;
  ops.a[0] = mask;
  ops.param[0] = ref_quirk ? 1.f : 0.f;
  return pixops_pass(ctx->stream, field, n_fields, rows, cols, ops, FieldInfo());
}

int csg_phase_screen(csg_ctx* ctx, float* field, int n_fields, int rows, int cols, const float* sag,
                     const double* lambda, double sign) {
  CSG_CHECK(ctx && field && sag && lambda, CSG_E_ARG, "csg_phase_screen: null argument");
  CSG_CHECK(n_fields > 0 && rows > 0 && cols > 0, CSG_E_SHAPE, "csg_phase_screen: bad shape");
  DeviceGuard g(ctx->device);
  PixOps ops;
  ops.n = 1;
  ops.kind[0] = OP_PHASE;
  ops.a[0] = sag;
  ops.param[0] = (float)sign;
  FieldInfo fi;
  fi.lam = lambda;
  return pixops_pass(ctx->stream, field, n_fields, rows, cols, ops, fi);
}

int csg_complex_mask(csg_ctx* ctx, float* field, int n_fields, int rows, int cols,
                     const float* amp, const float* ph, int mrows, int mcols) {
  CSG_CHECK(ctx && field && amp && ph, CSG_E_ARG, "csg_complex_mask: null argument");
  CSG_CHECK(n_fields > 0 && mrows > 0 && mcols > 0 && mrows <= rows && mcols <= cols,
            CSG_E_SHAPE, "csg_complex_mask: mask larger than field");
  DeviceGuard g(ctx->device);
  PixOps ops;
  ops.n = 1;
  ops.kind[0] = OP_CMASK;
  ops.a[0] = amp;
  ops.b[0] = ph;
  ops.mr[0] = mrows;
  ops.mc[0] = mcols;
  return pixops_pass(ctx->stream, field, n_fields, rows, cols, ops, FieldInfo());
}

int csg_hex_mask(csg_ctx* ctx, const int16_t* hex_id, const uint16_t* count, int S, int n_sub,
                 const double* sags, int n_hex, int n_out, const int* cand, const double* lambda,
                 double phase_sign, int flip, double subtract, int use_only_hex, float* out) {
  CSG_CHECK(ctx && hex_id && count && sags && cand && lambda && out, CSG_E_ARG,
            "csg_hex_mask: null argument");
  CSG_CHECK(S > 0 && n_sub > 0 && n_hex > 0 && n_hex < 32767 && n_out > 0, CSG_E_SHAPE,
            "csg_hex_mask: bad shape");
  CSG_CHECK(use_only_hex >= -1 && use_only_hex <= n_hex, CSG_E_ARG,
            "csg_hex_mask: use_only_hex out of range");
  DeviceGuard g(ctx->device);
  float2* ph = nullptr;
  const size_t bytes = (size_t)n_out * (n_hex + 1) * sizeof(float2);
  CSG_CUDA(cudaMallocAsync((void**)&ph, bytes, ctx->stream));
  int rc = hex_mask_with_phasor_buffer(ctx, hex_id, count, S, n_sub, sags, n_hex, n_out, cand,
                                       lambda, phase_sign, flip, subtract, use_only_hex, out, ph);
  cudaFreeAsync(ph, ctx->stream);
  return rc;
}

int csg_region_reduce(csg_ctx* ctx, const float* field, int rows, int cols, int n_groups,
                      int per_group, const int* pix_idx, int n_pix, int mode, double scale,
                      double* out) {
  CSG_CHECK(ctx && field && pix_idx && out, CSG_E_ARG, "csg_region_reduce: null argument");
  CSG_CHECK(n_groups > 0 && per_group > 0 && n_pix > 0, CSG_E_SHAPE,
            "csg_region_reduce: empty region or batch");
  CSG_CHECK(mode == 0 || mode == 1, CSG_E_ARG, "csg_region_reduce: mode must be 0 or 1");
  DeviceGuard g(ctx->device);
  k_region_reduce<<<n_groups, 256, 0, ctx->stream>>>(field, (long long)rows * cols, per_group,
                                                     pix_idx, n_pix, mode, scale, out);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

int csg_intensity(csg_ctx* ctx, const float* field, int rows, int cols, int n_fields, double* out,
                  double* out_max) {
  CSG_CHECK(ctx && field && out, CSG_E_ARG, "csg_intensity: null argument");
  CSG_CHECK(n_fields > 0 && rows > 0 && cols > 0, CSG_E_SHAPE, "csg_intensity: bad shape");
  DeviceGuard g(ctx->device);
  const long long plane = (long long)rows * cols;
  if (out_max) CSG_CUDA(cudaMemsetAsync(out_max, 0, sizeof(double), ctx->stream));
  k_intensity<<<grid_for(plane, 256), 256, 0, ctx->stream>>>(
      field, plane, n_fields, out, reinterpret_cast<unsigned long long*>(out_max));
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

}  // extern "C"
