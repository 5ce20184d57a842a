// Element field operations (HBM-bound elementwise / gather kernels) and the
// intensity / dark-hole reductions.
//
// Phases: a per-pixel phase is the product of an fp32 datum (sag, pixel
// offset) and an FP64 constant. The constant is carried as an fp32 pair
// (hi + lo) and the product is reduced modulo one turn with the rounding
// error of the leading product folded back (fmaf), which keeps ~2^-40 turns
// of accuracy without FP64 arithmetic per pixel.
#include "ctx.hpp"

namespace csg {

__device__ __forceinline__ float frac_mul2(float a, float khi, float klo) {
  const float p = a * khi;
  float e = fmaf(a, khi, -p);
  e = fmaf(a, klo, e);
  return (p - rintf(p)) + e;
}

__device__ __forceinline__ void split_f64(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// ------------------------------------------------------------ point source
__global__ void k_point_source(float* __restrict__ field, int F, int R, int C, double dx, double dy,
                               const double* __restrict__ amp, const double* __restrict__ tip,
                               const double* __restrict__ tilt) {
  const long long plane = (long long)R * C;
  const int f = blockIdx.y;
  if (f >= F) return;
  // turns = 2 x tip / Lx + 2 y tilt / Ly, x = (c - (C-1)/2) dx, Lx = C dx
  float kxh, kxl, kyh, kyl;
  split_f64(2.0 * tip[f] / (double)C, kxh, kxl);
  split_f64(2.0 * tilt[f] / (double)R, kyh, kyl);
  const float a = (float)amp[f];
  float* re = field + (long long)f * 2 * plane;
  float* im = re + plane;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < plane;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C), r = (int)(i / C);
    const float xc = (float)c - 0.5f * (float)(C - 1);  // exact half-integers
    const float yr = (float)r - 0.5f * (float)(R - 1);
    float t = frac_mul2(xc, kxh, kxl) + frac_mul2(yr, kyh, kyl);
    t -= rintf(t);
    float s, co;
    sincospif(2.f * t, &s, &co);
    re[i] = a * co;
    im[i] = a * s;
  }
}

// -------------------------------------------------------------- masks
__global__ void k_mask_real(float* __restrict__ field, int F, long long plane,
                            const float* __restrict__ mask, int quirk) {
  const long long n = plane * F;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long f = i / plane, o = i % plane;
    float* re = field + f * 2 * plane + o;
    float* im = re + plane;
    const float m = mask[o];
    const float xr = *re, xi = *im;
    if (quirk) {  // (xr + i xi)(m + i m)
      *re = m * (xr - xi);
      *im = m * (xr + xi);
    } else {
      *re = xr * m;
      *im = xi * m;
    }
  }
}

__global__ void k_phase_screen(float* __restrict__ field, int F, long long plane,
                               const float* __restrict__ sag, const double* __restrict__ lambda,
                               double sign) {
  const int f = blockIdx.y;
  if (f >= F) return;
  float kh, kl;  // turns per metre of sag: -sign * 2 / lambda
  split_f64(-sign * 2.0 / lambda[f], kh, kl);
  float* re = field + (long long)f * 2 * plane;
  float* im = re + plane;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < plane;
       i += (long long)gridDim.x * blockDim.x) {
    float t = frac_mul2(sag[i], kh, kl);
    float s, c;
    sincospif(2.f * t, &s, &c);
    const float xr = re[i], xi = im[i];
    re[i] = xr * c - xi * s;
    im[i] = xr * s + xi * c;
  }
}

__global__ void k_complex_mask(float* __restrict__ field, int F, int R, int C,
                               const float* __restrict__ amp, const float* __restrict__ ph,
                               int mr, int mc) {
  const long long plane = (long long)R * C;
  const long long mplane = (long long)mr * mc;
  const int r0 = R / 2 - mr / 2, c0 = C / 2 - mc / 2;
  const long long n = mplane * F;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long f = i / mplane, o = i % mplane;
    const int r = (int)(o / mc), c = (int)(o % mc);
    float s, co;
    sincosf(-ph[o], &s, &co);
    const float a = amp[o];
    float* re = field + f * 2 * plane + (long long)(r0 + r) * C + (c0 + c);
    float* im = re + plane;
    const float xr = *re, xi = *im;
    *re = a * (xr * co - xi * s);
    *im = a * (xr * s + xi * co);
  }
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
  CSG_CHECK(n_fields > 0 && n_fields < 65536 && rows > 0 && cols > 0, CSG_E_SHAPE,
            "csg_point_source: bad shape");
  (void)dx;
  (void)dy;  // the phase only depends on the pixel index (x / Lx = index / C)
  DeviceGuard g(ctx->device);
  dim3 grid(grid_for((long long)rows * cols, 256, 512), n_fields);
  k_point_source<<<grid, 256, 0, ctx->stream>>>(field, n_fields, rows, cols, dx, dy, amp, tip,
                                                tilt);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

int csg_mask_real(csg_ctx* ctx, float* field, int n_fields, int rows, int cols, const float* mask,
                  int ref_quirk) {
  CSG_CHECK(ctx && field && mask, CSG_E_ARG, "csg_mask_real: null argument");
  CSG_CHECK(n_fields > 0 && rows > 0 && cols > 0, CSG_E_SHAPE, "csg_mask_real: bad shape");
  DeviceGuard g(ctx->device);
  const long long plane = (long long)rows * cols;
  k_mask_real<<<grid_for(plane * n_fields, 256), 256, 0, ctx->stream>>>(field, n_fields, plane,
                                                                        mask, ref_quirk);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

int csg_phase_screen(csg_ctx* ctx, float* field, int n_fields, int rows, int cols, const float* sag,
                     const double* lambda, double sign) {
  CSG_CHECK(ctx && field && sag && lambda, CSG_E_ARG, "csg_phase_screen: null argument");
  CSG_CHECK(n_fields > 0 && n_fields < 65536 && rows > 0 && cols > 0, CSG_E_SHAPE,
            "csg_phase_screen: bad shape");
  DeviceGuard g(ctx->device);
  const long long plane = (long long)rows * cols;
  dim3 grid(grid_for(plane, 256, 512), n_fields);
  k_phase_screen<<<grid, 256, 0, ctx->stream>>>(field, n_fields, plane, sag, lambda, sign);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

int csg_complex_mask(csg_ctx* ctx, float* field, int n_fields, int rows, int cols,
                     const float* amp, const float* ph, int mrows, int mcols) {
  CSG_CHECK(ctx && field && amp && ph, CSG_E_ARG, "csg_complex_mask: null argument");
  CSG_CHECK(n_fields > 0 && mrows > 0 && mcols > 0 && mrows <= rows && mcols <= cols,
            CSG_E_SHAPE, "csg_complex_mask: mask larger than field");
  DeviceGuard g(ctx->device);
  k_complex_mask<<<grid_for((long long)mrows * mcols * n_fields, 256), 256, 0, ctx->stream>>>(
      field, n_fields, rows, cols, amp, ph, mrows, mcols);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
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
