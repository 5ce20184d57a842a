// Deformable-mirror surface (deformableMirror.cpp:205-270).
//
// The reference places the nA x nA actuator strokes as delta points on a
// U x U grid (U = nA ceil((N+1)/nA)), FFTs it, applies the half-cell shift
// phase, truncates the spectrum to N x N with Nyquist averaging
// (fft_truncate, csim_fft.cpp:322-367), multiplies by the FFT of the
// Gaussian influence function, inverse-FFTs and keeps the real part. Every
// step is separable (the influence exp(-4 ln2 (x^2 + y^2) / s^2) is a
// product of two 1-D Gaussians on the pixel grid, and the truncation, the
// shift phase and the delta upsampling act on rows and columns
// independently), so the surface is exactly
//     surface = Re(M A M^T),   M[x][a] = (1/N) sum_k' X[k'][a] e^{+2 pi i k' x / N}
//     X[k'][a] = g_hat[k'] (T Y)[k'][a],  Y[k][a] = Phi[k] e^{-2 pi i k a / nA}
// with g_hat the N-point FFT of the 1-D Gaussian, T the 1-D truncation
// (N x U) and Phi[k] = e^{2 pi i f[k] N (1 - 1/nA) / 2}, f[k] the signed
// frequency over N. X and g_hat are built on the host in FP64; the N x nA
// basis M (once per geometry) and the surface (per actuator update) are FP64
// GPU products, the surface is stored as fp32 metres.
#include <cmath>
#include <complex>
#include <vector>

#include "ctx.hpp"

struct csg_dm {
  csg_ctx* ctx = nullptr;
  int n = 0, n_act = 0;
  double2* basis = nullptr;  // M [n][n_act]
  double2* tmp = nullptr;    // A M^T: [n_act][n]
};

namespace csg {

// M[x][a] = (1/N) sum_k X[k][a] tw[(k x) mod N], tw[j] = e^{2 pi i j / N}.
__global__ void k_dm_basis(const double2* __restrict__ X, const double2* __restrict__ tw, int n,
                           int n_act, double2* __restrict__ M) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * n_act) return;
  const int x = i / n_act, a = i % n_act;
  double re = 0.0, im = 0.0;
  for (int k = 0; k < n; ++k) {
    const double2 v = X[(size_t)k * n_act + a];
    const double2 w = tw[((long long)k * x) & (n - 1)];
    re = fma(v.x, w.x, fma(-v.y, w.y, re));
    im = fma(v.x, w.y, fma(v.y, w.x, im));
  }
  M[i] = make_double2(re / n, im / n);
}

// T[a][x] = sum_b A[a][b] M[x][b]
__global__ void k_dm_right(const double* __restrict__ A, const double2* __restrict__ M, int n,
                           int n_act, double2* __restrict__ T) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * n_act) return;
  const int a = i / n, x = i % n;
  double re = 0.0, im = 0.0;
  for (int b = 0; b < n_act; ++b) {
    const double s = A[a * n_act + b];
    const double2 m = M[(size_t)x * n_act + b];
    re = fma(s, m.x, re);
    im = fma(s, m.y, im);
  }
  T[(size_t)a * n + x] = make_double2(re, im);
}

// surface[y][x] = Re sum_a M[y][a] T[a][x]
__global__ void k_dm_left(const double2* __restrict__ M, const double2* __restrict__ T, int n,
                          int n_act, float* __restrict__ surf) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)n * n) return;
  const int y = (int)(i / n), x = (int)(i % n);
  double re = 0.0;
  for (int a = 0; a < n_act; ++a) {
    const double2 m = M[(size_t)y * n_act + a];
    const double2 t = T[(size_t)a * n + x];
    re = fma(m.x, t.x, fma(-m.y, t.y, re));
  }
  surf[i] = (float)re;
}

}  // namespace csg

using namespace csg;

extern "C" {

// Surface generator for an N x N mirror with n_act x n_act actuators and
// influence width sigma (in actuator pitches; influenceSigma = sigma
// physicalSize / nActuatorRows, deformableMirror.cpp:205-214).
int csg_dm_create(csg_ctx* ctx, csg_dm** out, int n, int n_act, double sigma) {
  CSG_CHECK(ctx && out, CSG_E_ARG, "csg_dm_create: null argument");
  CSG_CHECK(n >= 8 && n <= 8192 && (n & (n - 1)) == 0 && n_act >= 2 && n_act <= n && sigma > 0,
            CSG_E_SHAPE, "csg_dm_create: N must be a power of two, 2 <= n_act <= N, sigma > 0");
  using cd = std::complex<double>;
  const double two_pi = 2.0 * M_PI;
  const int N = n, nA = n_act;
  const int ur = (N + 1 + nA - 1) / nA;  // ceil((N + 1) / nA)
  const long long U = (long long)ur * nA;
  // the reference's shift-frequency vectors have 2 floor(U/2) entries, so it
  // only runs for an even upsampled size
  CSG_CHECK(U % 2 == 0, CSG_E_SHAPE, "csg_dm_create: upsampled actuator grid must be even");
  // 1-D Gaussian on the pixel centres, in pixel units: s = sigma N / nA pixels
  const double s = sigma * N / nA;
  std::vector<cd> twN(N);
  for (int j = 0; j < N; ++j) twN[j] = std::polar(1.0, two_pi * j / N);
  std::vector<double> g(N);
  for (int r = 0; r < N; ++r) {
    const double y = -(N - 1) / 2.0 + r;
    g[r] = std::exp(-4.0 * std::log(2.0) * y * y / (s * s));
  }
  std::vector<cd> ghat(N);
  for (int k = 0; k < N; ++k) {
    cd acc = 0.0;
    for (int r = 0; r < N; ++r) acc += g[r] * std::conj(twN[((long long)k * r) & (N - 1)]);
    ghat[k] = acc;
  }
  // Y[k][a] at the U-grid frequencies the truncation keeps
  const double h = N * (1.0 - 1.0 / nA) / 2.0;
  auto Y = [&](long long k, int a) {
    const double f = (double)(k < U / 2 ? k : k - U) / N;
    const double ph = f * h - (double)((k * a) % nA) / nA;  // turns
    return std::polar(1.0, two_pi * (ph - std::rint(ph)));
  };
  std::vector<double2> X((size_t)N * nA);
  for (int kp = 0; kp < N; ++kp)
    for (int a = 0; a < nA; ++a) {
      cd v;
      if (kp < N / 2) {
        v = Y(kp, a);
      } else if (kp == N / 2) {  // Nyquist: average of +N/2 and -N/2
        v = 0.5 * (Y(N / 2, a) + Y(U - N / 2, a));
      } else {
        v = Y(U - N + kp, a);
      }
      v *= ghat[kp];
      X[(size_t)kp * nA + a] = make_double2(v.real(), v.imag());
    }
  DeviceGuard dg(ctx->device);
  cudaStream_t st = ctx->stream;
  csg_dm* d = new csg_dm();
  d->ctx = ctx;
  d->n = N;
  d->n_act = nA;
  double2 *dX = nullptr, *dtw = nullptr;
  std::vector<double2> tw(N);
  for (int j = 0; j < N; ++j) tw[j] = make_double2(twN[j].real(), twN[j].imag());
  if (cudaMalloc(&d->basis, sizeof(double2) * N * nA) != cudaSuccess ||
      cudaMalloc(&d->tmp, sizeof(double2) * N * nA) != cudaSuccess ||
      cudaMalloc(&dX, sizeof(double2) * N * nA) != cudaSuccess ||
      cudaMalloc(&dtw, sizeof(double2) * N) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(d->basis);
    cudaFree(d->tmp);
    cudaFree(dX);
    cudaFree(dtw);
    delete d;
    set_error("csg_dm_create: allocation failed");
    return CSG_E_NOMEM;
  }
  CSG_CUDA(cudaMemcpyAsync(dX, X.data(), sizeof(double2) * N * nA, cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(dtw, tw.data(), sizeof(double2) * N, cudaMemcpyHostToDevice, st));
  k_dm_basis<<<(N * nA + 127) / 128, 128, 0, st>>>(dX, dtw, N, nA, d->basis);
  CSG_LAUNCH_CHECK();
  CSG_CUDA(cudaStreamSynchronize(st));
  cudaFree(dX);
  cudaFree(dtw);
  *out = d;
  return CSG_OK;
}

int csg_dm_destroy(csg_dm* d) {
  if (!d) return CSG_OK;
  DeviceGuard dg(d->ctx->device);
  cudaStreamSynchronize(d->ctx->stream);
  cudaFree(d->basis);
  cudaFree(d->tmp);
  delete d;
  return CSG_OK;
}

// surface [N][N] (device fp32, metres) from device FP64 strokes
// [n_act][n_act] (row-major, rows = y): compute_deformable_mirror_surface.
int csg_dm_surface(csg_dm* d, const double* act, float* surface) {
  CSG_CHECK(d && act && surface, CSG_E_ARG, "csg_dm_surface: null argument");
  DeviceGuard dg(d->ctx->device);
  cudaStream_t st = d->ctx->stream;
  const int N = d->n, nA = d->n_act;
  {
    ProfScope ps(d->ctx, "dm_surface", 0, 0);
    k_dm_right<<<(N * nA + 255) / 256, 256, 0, st>>>(act, d->basis, N, nA, d->tmp);
    CSG_LAUNCH_CHECK();
    k_dm_left<<<(unsigned)(((long long)N * N + 255) / 256), 256, 0, st>>>(d->basis, d->tmp, N,
                                                                         nA, surface);
    CSG_LAUNCH_CHECK();
  }
  return CSG_OK;
}

}  // extern "C"
