// Hex focal-plane-mask interpolation tables on the GPU: the reference's
// make_hex_array (complexHexMaskFPM.cpp:317-366) and make_interpolation_data
// (:372-469). Every FP64 expression is written with explicit _rn intrinsics
// so no multiply-add is contracted and sub-pixel samples land on exactly the
// design-array cells the reference's x86-64 build selects.
#include "ctx.hpp"

namespace csg {

__global__ void k_hex_design(const double* __restrict__ hx, const double* __restrict__ hy,
                             int n_hex, int A, double step_pix, double radius, double close_sq,
                             int* __restrict__ design) {
  const int h = blockIdx.x;
  if (h >= n_hex) return;
  const double vx = 0.86602540378443864676, vy = 0.5;  // sqrt(3)/2, 1/2
  const double cx = __dadd_rn(0.5 * A, __dmul_rn(hx[h], step_pix));
  const double cy = __dadd_rn(0.5 * A, __dmul_rn(hy[h], step_pix));
  const double outer = sqrt(close_sq);
  int i0 = (int)floor(cy - outer) - 1, i1 = (int)ceil(cy + outer) + 1;
  int j0 = (int)floor(cx - outer) - 1, j1 = (int)ceil(cx + outer) + 1;
  i0 = max(i0, 0); j0 = max(j0, 0);
  i1 = min(i1, A - 1); j1 = min(j1, A - 1);
  const int w = j1 - j0 + 1, n = (i1 - i0 + 1) * w;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int ii = i0 + t / w, jj = j0 + t % w;
    const double dx = __dsub_rn((double)jj, cx);
    const double dy = __dsub_rn((double)ii, cy);
    const double r2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    if (r2 > close_sq) continue;
    const double dpx = __dmul_rn(dx, vx), dpy = __dmul_rn(dy, vy);
    if (fabs(dy) < radius && fabs(__dadd_rn(dpx, dpy)) < radius &&
        fabs(__dsub_rn(dpx, dpy)) < radius)
      atomicMax(&design[ii * A + jj], h);
  }
}

// Row / column index of every sub-pixel sample: the sample coordinate only
// depends on (pixel, sub-pixel) along one axis.
__global__ void k_hex_sample_index(int S, int n_sub, int A, double pixel_scale, double ac1,
                                   double xc1, int* __restrict__ idx) {
  const int n = S * n_sub;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int i = t / n_sub, s = t % n_sub;
    const double frac = __ddiv_rn(__dadd_rn(0.5, (double)s), (double)n_sub);
    const double x = __dmul_rn(__dadd_rn(__dadd_rn((double)i, ac1), frac), pixel_scale);
    idx[t] = (int)__dadd_rn(__dmul_rn(__dadd_rn(0.5, __dmul_rn(x, xc1)), (double)A), 0.5);
  }
}

// stale != 0: the reference's row check as its loop runs on one OpenMP
// thread (complexHexMaskFPM.cpp:395-423): the check's row index is the
// midpoint's until the row's first passing cell and afterwards the one left
// by the last sub-sample of the cell before. The sample indices grow with
// the pixel index, so in a row whose midpoint index is on the array the
// first passing cell is the first column whose midpoint index is; after it
// the check uses the last sub-sample's row index.
__global__ void k_hex_interp(const int* __restrict__ design, int A, int S, int n_sub,
                             const int* __restrict__ sidx, int16_t* __restrict__ hex_id,
                             uint16_t* __restrict__ count, int* __restrict__ overflow,
                             int stale) {
  const long long plane = (long long)S * S;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < plane;
       p += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(p / S), j = (int)(p % S);
    const int* ri = sidx + i * n_sub;
    const int* rj = sidx + j * n_sub;
    const int c = n_sub / 2;
    int list[3] = {-1, -1, -1};
    unsigned cnt[3] = {0, 0, 0};
    int nl = 0, over = 0;
    bool inside = ri[c] >= 0 && ri[c] < A && rj[c] >= 0 && rj[c] < A;
    if (stale && inside) {
      const int jp = j > 0 ? sidx[(j - 1) * n_sub + c] : -1;
      const bool first = j == 0 || jp < 0 || jp >= A;
      const bool last_on = ri[n_sub - 1] >= 0 && ri[n_sub - 1] < A;
      inside = first || last_on;
    }
    if (inside) {
      for (int a = 0; a < n_sub; ++a) {
        const int ii1 = ri[a];
        const bool row_ok = ii1 >= 0 && ii1 < A;
        for (int b = 0; b < n_sub; ++b) {
          const int jj1 = rj[b];
          if (!row_ok || jj1 < 0 || jj1 >= A) {
            cnt[0]++;
            continue;
          }
          const int h = design[ii1 * A + jj1];
          if (h < 0) {
            cnt[0]++;
            continue;
          }
          int k = 0;
          while (k < nl && list[k] != h) ++k;
          if (k == nl) {
            if (nl == 3) {
              over = 1;
              cnt[0]++;
              continue;
            }
            list[nl++] = h;
          }
          cnt[k]++;
        }
      }
    }
    if (cnt[0] + cnt[1] + cnt[2] == 0) cnt[0] = (unsigned)(n_sub * n_sub);
    for (int k = 0; k < 3; ++k) {
      hex_id[k * plane + p] = (int16_t)(k < nl ? list[k] : -1);
      count[k * plane + p] = (uint16_t)cnt[k];
    }
    if (over) atomicAdd(overflow, 1);
  }
}

}  // namespace csg

using namespace csg;

extern "C" int csg_hex_tables(csg_ctx* ctx, const double* hex_x, const double* hex_y, int n_hex,
                              int n_rings, int design_size, double fpm_scale_factor,
                              double hex_gap, double pitch, int S, int n_sub, double pixel_scale,
                              double fpm_radius, int16_t* hex_id, uint16_t* count,
                              int* n_overflow, int reference_single_thread) {
  CSG_CHECK(ctx && hex_x && hex_y && hex_id && count, CSG_E_ARG, "csg_hex_tables: null argument");
  CSG_CHECK(n_hex > 0 && n_hex < 32767 && n_rings > 0 && design_size > 0 && S > 0 && n_sub > 0 &&
                n_sub * n_sub < 65536,
            CSG_E_SHAPE, "csg_hex_tables: bad size");
  CSG_CHECK(pixel_scale > 0 && fpm_radius > 0 && pitch > 0 && fpm_scale_factor > 0, CSG_E_ARG,
            "csg_hex_tables: non-positive scale");
  DeviceGuard g(ctx->device);
  cudaStream_t st = ctx->stream;
  const int A = design_size;
  int *design = nullptr, *sidx = nullptr, *over = nullptr;
  CSG_CUDA(cudaMallocAsync((void**)&design, sizeof(int) * (size_t)A * A, st));
  CSG_CUDA(cudaMallocAsync((void**)&sidx, sizeof(int) * (size_t)S * n_sub, st));
  CSG_CUDA(cudaMallocAsync((void**)&over, sizeof(int), st));
  CSG_CUDA(cudaMemsetAsync(design, 0xFF, sizeof(int) * (size_t)A * A, st));
  CSG_CUDA(cudaMemsetAsync(over, 0, sizeof(int), st));
  // host FP64 set-up, same expressions as the reference
  const double step_pix = (0.5 * A) / n_rings * fpm_scale_factor;
  const double radius = step_pix * (1.0 - hex_gap) * (pitch / 2.0);
  const double outer = 2.0 * radius / sqrt(3.0);
  k_hex_design<<<n_hex, 256, 0, st>>>(hex_x, hex_y, n_hex, A, step_pix, radius, outer * outer,
                                      design);
  CSG_LAUNCH_CHECK();
  const double ac1 = -S / 2.0 - 0.5;
  const double xc1 = (0.5 / fpm_radius) * fpm_scale_factor;
  k_hex_sample_index<<<grid_for((long long)S * n_sub, 256), 256, 0, st>>>(S, n_sub, A,
                                                                            pixel_scale, ac1, xc1,
                                                                            sidx);
  CSG_LAUNCH_CHECK();
  k_hex_interp<<<grid_for((long long)S * S, 128), 128, 0, st>>>(
      design, A, S, n_sub, sidx, hex_id, count, over, reference_single_thread ? 1 : 0);
  CSG_LAUNCH_CHECK();
  int h_over = 0;
  CSG_CUDA(cudaMemcpyAsync(&h_over, over, sizeof(int), cudaMemcpyDeviceToHost, st));
  cudaFreeAsync(design, st);
  cudaFreeAsync(sidx, st);
  cudaFreeAsync(over, st);
  CSG_CUDA(cudaStreamSynchronize(st));
  if (n_overflow) *n_overflow = h_over;
  return CSG_OK;
}
