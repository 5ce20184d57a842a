// Callers around the propagation: the contrast curve (radial profile of the
// normalised image) and the finite-difference Jacobian of the dark-hole
// field over a batch of perturbed candidates.
#include "ctx.hpp"
#include "common.cuh"

namespace csg {

// contrastCurve::make_contrast_curve (contrastCurve.cpp:127-140): bin i
// (1 <= i <= K-2) averages the normalised intensity over pixels with
// s[i-1] < R < s[i+1], R = |pixel centre| / loD on the n x n output grid
// (pixel centres -(d n - d) / 2 + k d, csim_geom.cpp:130-135). A pixel falls
// in at most two bins, found around floor(R / step) and checked exactly.
__global__ void k_contrast_curve(const double* __restrict__ inten, int n, double d, double lod,
                                 double scale, const double* __restrict__ s, int K,
                                 double* __restrict__ sum, double* __restrict__ cnt) {
  const long long plane = (long long)n * n;
  const double x0 = -(d * n - d) / 2.0;
  const double step = s[K - 1] / (double)(K - 1);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < plane;
       p += (long long)gridDim.x * blockDim.x) {
    const double x = x0 + (double)(p % n) * d, y = x0 + (double)(p / n) * d;
    const double R = sqrt(x * x + y * y) / lod;
    const double v = inten[p] * scale;
    const int j = step > 0 ? (int)floor(R / step) : 0;
    for (int i = max(1, j - 1); i <= min(K - 2, j + 2); ++i)
      if (s[i - 1] < R && R < s[i + 1]) {
        atomicAdd(&sum[i - 1], v);
        atomicAdd(&cnt[i - 1], 1.0);
      }
  }
}

__global__ void k_bin_mean(const double* __restrict__ sum, const double* __restrict__ cnt, int nb,
                           double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nb) out[i] = cnt[i] > 0 ? sum[i] / cnt[i] : nan("");
}

// linearOptimizer::compute_jacobian (linearOptimizer.cpp:420-495): column i
// of the Jacobian is (E_i - E_0) / dx at the region pixels, rows ordered by
// base field b (source, polarisation, wavelength in the reference's order)
// as [Re over the pixels; Im over the pixels]. Fields are candidate-major:
// field c * n_base + b is base field b of candidate c; candidate 0 is the
// unperturbed one, candidate i + 1 perturbs variable i.
__global__ void k_fd_jacobian(const float* __restrict__ img, int plane, int n_base, int n_var,
                              const int* __restrict__ pix, int n_pix, double inv_dx,
                              double* __restrict__ jac) {
  const long long rows = 2LL * n_base * n_pix;
  const long long total = rows * n_var;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int var = (int)(t / rows);
    const long long r = t % rows;
    const int b = (int)(r / (2LL * n_pix));
    const int comp = (int)((r / n_pix) % 2);
    const int k = (int)(r % n_pix);
    const long long q = (long long)comp * plane + pix[k];
    const double e0 = img[(size_t)b * 2 * plane + q];
    const double e1 = img[((size_t)(var + 1) * n_base + b) * 2 * plane + q];
    jac[r * n_var + var] = (e1 - e0) * inv_dx;  // row-major [rows][n_var]
  }
}

}  // namespace csg

using namespace csg;

extern "C" {

int csg_contrast_curve(csg_ctx* ctx, const double* intensity, int n, double pixel, double lod,
                       double scale, const double* samples, int n_samples, double* work,
                       double* out_mean) {
  CSG_CHECK(ctx && intensity && samples && work && out_mean, CSG_E_ARG,
            "csg_contrast_curve: null argument");
  CSG_CHECK(n > 0 && n_samples >= 3 && pixel > 0 && lod > 0, CSG_E_SHAPE,
            "csg_contrast_curve: bad geometry");
  DeviceGuard g(ctx->device);
  const int nb = n_samples - 2;
  CSG_CUDA(cudaMemsetAsync(work, 0, sizeof(double) * 2 * nb, ctx->stream));
  k_contrast_curve<<<grid_for((long long)n * n, 256), 256, 0, ctx->stream>>>(
      intensity, n, pixel, lod, scale, samples, n_samples, work, work + nb);
  CSG_LAUNCH_CHECK();
  k_bin_mean<<<(nb + 255) / 256, 256, 0, ctx->stream>>>(work, work + nb, nb, out_mean);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

int csg_fd_jacobian(csg_ctx* ctx, const float* image, int n_out, int n_base, int n_var,
                    const int* pix_idx, int n_pix, double dx, double* jac) {
  CSG_CHECK(ctx && image && pix_idx && jac, CSG_E_ARG, "csg_fd_jacobian: null argument");
  CSG_CHECK(n_out > 0 && n_base > 0 && n_var > 0 && n_pix > 0 && dx != 0, CSG_E_SHAPE,
            "csg_fd_jacobian: bad shape");
  DeviceGuard g(ctx->device);
  const long long total = 2LL * n_base * n_pix * n_var;
  k_fd_jacobian<<<grid_for(total, 256), 256, 0, ctx->stream>>>(
      image, n_out * n_out, n_base, n_var, pix_idx, n_pix, 1.0 / dx, jac);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

}  // extern "C"
