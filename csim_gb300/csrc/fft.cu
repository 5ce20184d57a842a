// Shared-memory Stockham FFTs for square N x N planar fp32 fields and the
// fused angular-spectrum Fresnel pipeline.
//
// A 2-D transform is two HBM passes: a row pass (rows per CTA, coalesced
// row loads) and a column pass (a [N][COLS] tile per CTA, coalesced row
// segments). Each pass reads and writes the field once; every butterfly stage
// runs in shared memory with the stage's inputs held in registers so the
// transform is done in place (one buffer). Stages are radix 4 (one radix-2
// stage first when log2 N is odd). Twiddles come from an FP64-generated
// table of N entries.
//
// Fresnel (csim_fft.cpp:371-392) runs as: row FFT | column FFT x H x column
// IFFT | row IFFT / N^2, i.e. three passes instead of four, with H generated
// in-kernel from the integer frequency index (no N^2 exp table).
#include <map>
#include <mutex>

#include "ctx.hpp"

namespace csg {

// ----------------------------------------------------------- twiddles
__global__ void k_twiddles(float2* tw, int n) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)m / (double)n, &s, &c);
    tw[m] = make_float2((float)c, (float)s);
  }
}

// One immutable table per (device, N); kept for the life of the process.
static const float2* twiddles(int device, int n, cudaStream_t st) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, float2*> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(device, n);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  float2* p = nullptr;
  if (cudaMalloc(&p, sizeof(float2) * n) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  k_twiddles<<<(n + 255) / 256, 256, 0, st>>>(p, n);
  cudaStreamSynchronize(st);
  cache[key] = p;
  return p;
}

// ------------------------------------------------------- in-smem FFT
// ntr transforms of length N; element m of transform t at t*ts + m*es.
// Requires blockDim.x == ntr * N / 16. TF: transform index fastest across
// threads (columns) or butterfly index fastest (rows).
template <bool INV, bool TF>
__device__ void smem_fft(float* __restrict__ re, float* __restrict__ im, int N, int log2n, int ntr,
                         int es, int ts, const float2* __restrict__ tw) {
  const int T = blockDim.x;
  const int tid = threadIdx.x;
  const float sg = INV ? 1.f : -1.f;
  float vr[16], vi[16];
  int L = 1;
  int first = 1;
  while (L < N) {
    const int R = (first && (log2n & 1)) ? 2 : 4;
    first = 0;
    const int nbf = N / R;          // butterflies per transform
    const int per = (ntr * nbf) / T;  // butterflies per thread (4 or 8)
    const int stride_in = nbf;      // N / R
    const int twstep = N / (L * R);
    // gather + compute into registers
    for (int i = 0; i < per; ++i) {
      const int b = tid + i * T;
      int t, j;
      if (TF) { t = b % ntr; j = b / ntr; }
      else    { j = b % nbf; t = b / nbf; }
      const int k = j % L, g = j / L;
      const int src = t * ts + (g * L + k) * es;
      if (R == 4) {
        float ar[4], ai[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int idx = src + q * stride_in * es;
          float xr = re[idx], xi = im[idx];
          if (q) {
            const float2 w = __ldg(&tw[k * q * twstep]);
            const float wi = sg * w.y;
            const float tr = xr * w.x - xi * wi;
            xi = xr * wi + xi * w.x;
            xr = tr;
          }
          ar[q] = xr; ai[q] = xi;
        }
        const float s02r = ar[0] + ar[2], s02i = ai[0] + ai[2];
        const float d02r = ar[0] - ar[2], d02i = ai[0] - ai[2];
        const float s13r = ar[1] + ar[3], s13i = ai[1] + ai[3];
        const float d13r = ar[1] - ar[3], d13i = ai[1] - ai[3];
        // y1 = d02 + sg*i*d13, y3 = d02 - sg*i*d13
        vr[4 * i + 0] = s02r + s13r;        vi[4 * i + 0] = s02i + s13i;
        vr[4 * i + 1] = d02r - sg * d13i;   vi[4 * i + 1] = d02i + sg * d13r;
        vr[4 * i + 2] = s02r - s13r;        vi[4 * i + 2] = s02i - s13i;
        vr[4 * i + 3] = d02r + sg * d13i;   vi[4 * i + 3] = d02i - sg * d13r;
      } else {
        const int i0 = src, i1 = src + stride_in * es;
        float xr = re[i1], xi = im[i1];
        const float2 w = __ldg(&tw[k * twstep]);
        const float wi = sg * w.y;
        const float tr = xr * w.x - xi * wi;
        xi = xr * wi + xi * w.x;
        xr = tr;
        const float ar = re[i0], ai = im[i0];
        vr[2 * i + 0] = ar + xr; vi[2 * i + 0] = ai + xi;
        vr[2 * i + 1] = ar - xr; vi[2 * i + 1] = ai - xi;
      }
    }
    __syncthreads();
    for (int i = 0; i < per; ++i) {
      const int b = tid + i * T;
      int t, j;
      if (TF) { t = b % ntr; j = b / ntr; }
      else    { j = b % nbf; t = b / nbf; }
      const int k = j % L, g = j / L;
      const int dst = t * ts + (g * L * R + k) * es;
      for (int q = 0; q < R; ++q) {
        re[dst + q * L * es] = vr[R * i + q];
        im[dst + q * L * es] = vi[R * i + q];
      }
    }
    __syncthreads();
    L *= R;
  }
}

// Row pass: blockDim = rows * N / 16; each CTA transforms `rows` rows.
template <bool INV>
__global__ void k_fft_rows(float* __restrict__ field, int F, int N, int log2n, int rows,
                           float scale, const float2* __restrict__ tw) {
  extern __shared__ float sm[];
  float* re = sm;
  float* im = sm + rows * N;
  const int ctas_per_field = N / rows;
  const int f = blockIdx.x / ctas_per_field;
  const int r0 = (blockIdx.x % ctas_per_field) * rows;
  const long long plane = (long long)N * N;
  float* fre = field + (long long)f * 2 * plane + (long long)r0 * N;
  float* fim = fre + plane;
  const int n = rows * N;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    re[i] = fre[i];
    im[i] = fim[i];
  }
  __syncthreads();
  smem_fft<INV, false>(re, im, N, log2n, rows, 1, N, tw);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    fre[i] = re[i] * scale;
    fim[i] = im[i] * scale;
  }
}

struct FresnelArgs {
  const double* lambda;  // per field, nullptr = plain column pass
  double z;
  double ap_rad;
};

__device__ __forceinline__ float frac_mul(float a, float khi, float klo) {
  // a * (khi + klo) modulo 1, with the product error folded back in
  const float p = a * khi;
  float e = fmaf(a, khi, -p);
  e = fmaf(a, klo, e);
  return (p - rintf(p)) + e;
}

// Column pass: blockDim = cols * N / 16; tile [N][cols] of one field.
// MODE 0: forward, 1: inverse, 2: forward * H(lambda_f) * inverse.
template <int MODE>
__global__ void k_fft_cols(float* __restrict__ field, int F, int N, int log2n, int cols,
                           const float2* __restrict__ tw, FresnelArgs fa) {
  extern __shared__ float sm[];
  float* re = sm;
  float* im = sm + cols * N;
  const int ctas_per_field = N / cols;
  const int f = blockIdx.x / ctas_per_field;
  const int c0 = (blockIdx.x % ctas_per_field) * cols;
  const long long plane = (long long)N * N;
  float* fre = field + (long long)f * 2 * plane + c0;
  float* fim = fre + plane;
  const int n = cols * N;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int r = i / cols, c = i % cols;
    re[i] = fre[(long long)r * N + c];
    im[i] = fim[(long long)r * N + c];
  }
  __syncthreads();
  if (MODE == 1) {
    smem_fft<true, true>(re, im, N, log2n, cols, cols, 1, tw);
  } else {
    smem_fft<false, true>(re, im, N, log2n, cols, cols, 1, tw);
  }
  if (MODE == 2) {
    // H = exp(2 pi i [z/lambda sqrt(1 - eps)]), eps = (lambda/apRad)^2 f^2 / 4
    //   turns = z/lambda - K f^2 / 2 - K f^2 h,  K = z lambda / (4 apRad^2),
    //   h = eps / (2 (1 + sqrt(1 - eps))^2)
    const double lam = fa.lambda[f];
    double t0 = fa.z / lam;
    t0 -= rint(t0);
    const double K = fa.z * lam / (4.0 * fa.ap_rad * fa.ap_rad);
    const double kh = 0.5 * K;
    const float khi = (float)kh, klo = (float)(kh - (double)khi);
    const float Kf = (float)K;
    const float c_eps = (float)(0.25 * (lam / fa.ap_rad) * (lam / fa.ap_rad));
    const float t0f = (float)t0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int r = i / cols, c = c0 + i % cols;
      const int fr = r < N / 2 ? r : r - N;
      const int fc = c < N / 2 ? c : c - N;
      const float f2 = (float)(fr * fr + fc * fc);  // exact: < 2^24
      const float eps = c_eps * f2;
      const float s = sqrtf(1.f - eps);
      const float h = eps / (2.f * (1.f + s) * (1.f + s));
      float t = t0f - frac_mul(f2, khi, klo) - Kf * f2 * h;
      t -= rintf(t);
      float sn, cs;
      sincospif(2.f * t, &sn, &cs);
      const float xr = re[i], xi = im[i];
      re[i] = xr * cs - xi * sn;
      im[i] = xr * sn + xi * cs;
    }
    __syncthreads();
    smem_fft<true, true>(re, im, N, log2n, cols, cols, 1, tw);
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int r = i / cols, c = i % cols;
    fre[(long long)r * N + c] = re[i];
    fim[(long long)r * N + c] = im[i];
  }
}

static int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}

static int rows_for(int n) { return n >= 4096 ? 1 : (4096 / n > 16 ? 16 : 4096 / n); }
static int cols_for(int n) { return n >= 2048 ? 8 * 2048 / n : (n >= 64 ? 16 : 16); }

template <typename K>
static int prep_smem(K kern, size_t bytes) {
  CSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return CSG_OK;
}

int fft2d_launch(csg_ctx* ctx, float* field, int F, int n, int direction, const double* lambda,
                 double ap_rad, double z, bool fresnel) {
  CSG_CHECK(n >= 64 && n <= 4096 && (n & (n - 1)) == 0, CSG_E_SHAPE,
            "FFT size must be a power of two in [64, 4096]");
  CSG_CHECK(F > 0, CSG_E_SHAPE, "FFT needs at least one field");
  cudaStream_t st = ctx->stream;
  const float2* tw = twiddles(ctx->device, n, st);
  CSG_CHECK(tw != nullptr, CSG_E_NOMEM, "twiddle table allocation failed");
  const int lg = ilog2(n);
  const int rows = rows_for(n), cols = cols_for(n);
  const size_t rsm = (size_t)rows * n * 8, csm = (size_t)cols * n * 8;
  const int rthreads = rows * n / 16, cthreads = cols * n / 16;
  const long long rgrid = (long long)F * (n / rows), cgrid = (long long)F * (n / cols);
  CSG_CHECK(rgrid < (1LL << 31) && cgrid < (1LL << 31), CSG_E_SHAPE, "too many fields");
  FresnelArgs fa{lambda, z, ap_rad};
  int rc;
  const bool inv = direction > 0;
  const float inv_scale = 1.f / ((float)n * (float)n);
  // one compulsory read + write of the planar fp32 field per pass
  const double pass_bytes = (double)F * n * n * 16.0;
  ProfScope ps(ctx, fresnel ? "fresnel_3pass" : "fft2d_2pass", 0,
               pass_bytes * (fresnel ? 3.0 : 2.0));
  if (!fresnel) {
    if (!inv) {
      if ((rc = prep_smem(k_fft_rows<false>, rsm))) return rc;
      k_fft_rows<false><<<(int)rgrid, rthreads, rsm, st>>>(field, F, n, lg, rows, 1.f, tw);
      CSG_LAUNCH_CHECK();
      if ((rc = prep_smem(k_fft_cols<0>, csm))) return rc;
      k_fft_cols<0><<<(int)cgrid, cthreads, csm, st>>>(field, F, n, lg, cols, tw, fa);
      CSG_LAUNCH_CHECK();
    } else {
      if ((rc = prep_smem(k_fft_cols<1>, csm))) return rc;
      k_fft_cols<1><<<(int)cgrid, cthreads, csm, st>>>(field, F, n, lg, cols, tw, fa);
      CSG_LAUNCH_CHECK();
      if ((rc = prep_smem(k_fft_rows<true>, rsm))) return rc;
      k_fft_rows<true><<<(int)rgrid, rthreads, rsm, st>>>(field, F, n, lg, rows, inv_scale, tw);
      CSG_LAUNCH_CHECK();
    }
  } else {
    if ((rc = prep_smem(k_fft_rows<false>, rsm))) return rc;
    k_fft_rows<false><<<(int)rgrid, rthreads, rsm, st>>>(field, F, n, lg, rows, 1.f, tw);
    CSG_LAUNCH_CHECK();
    if ((rc = prep_smem(k_fft_cols<2>, csm))) return rc;
    k_fft_cols<2><<<(int)cgrid, cthreads, csm, st>>>(field, F, n, lg, cols, tw, fa);
    CSG_LAUNCH_CHECK();
    if ((rc = prep_smem(k_fft_rows<true>, rsm))) return rc;
    k_fft_rows<true><<<(int)rgrid, rthreads, rsm, st>>>(field, F, n, lg, rows, inv_scale, tw);
    CSG_LAUNCH_CHECK();
  }
  return CSG_OK;
}

}  // namespace csg

using namespace csg;

extern "C" {

int csg_fft2d(csg_ctx* ctx, float* field, int n_fields, int n, int direction) {
  CSG_CHECK(ctx && field, CSG_E_ARG, "csg_fft2d: null argument");
  CSG_CHECK(direction == -1 || direction == 1, CSG_E_ARG, "csg_fft2d: direction must be -1 or +1");
  DeviceGuard g(ctx->device);
  return fft2d_launch(ctx, field, n_fields, n, direction, nullptr, 0, 0, false);
}

int csg_fresnel(csg_ctx* ctx, float* field, int n_fields, int n, const double* lambda,
                double ap_rad, double z) {
  CSG_CHECK(ctx && field && lambda, CSG_E_ARG, "csg_fresnel: null argument");
  CSG_CHECK(ap_rad > 0, CSG_E_ARG, "csg_fresnel: apRad must be positive");
  DeviceGuard g(ctx->device);
  return fft2d_launch(ctx, field, n_fields, n, -1, lambda, ap_rad, z, true);
}

}  // extern "C"
