// Shared-memory Stockham FFTs for square N x N planar fp32 fields and the
// fused angular-spectrum Fresnel pipeline.
//
// A 2-D transform is two HBM passes: a row pass (4096/N rows per CTA, float4
// row loads) and a column pass (a [N][COLS] tile per CTA, coalesced row
// segments). Each pass reads and writes the field once. Inside a pass every
// thread owns 16 elements of one transform in registers; stages are radix 16
// (one radix 2/4/8 stage first when log2 N is not a multiple of 4), so a
// 1024-point transform is 3 shared-memory exchanges. The radix-R butterflies
// are unrolled radix-2 decimation-in-frequency networks with exact W16
// constants; inter-stage twiddles come from an FP64-generated table. Row
// transforms are padded in shared memory (one float per 16) so the
// stride-16 stores of the first stage are conflict-free.
//
// Element ops (point source, masks, mirrors) ride along in the row passes'
// prologue and epilogue (pixops.cuh), so they cost no extra HBM pass.
//
// Fresnel (csim_fft.cpp:371-392) is row FFT | column FFT x H x column IFFT |
// row IFFT / N^2: three passes, H generated in-kernel from the integer
// frequency index.
#include <map>
#include <mutex>

#include "ctx.hpp"
#include "pixops.cuh"

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

// ------------------------------------------------ in-register butterflies
// cos and sin of 2 pi m / 16.
__device__ __forceinline__ float w16c(int m) {
  constexpr float c[16] = {1.0f, 0.92387953251128674f, 0.70710678118654752f, 0.38268343236508977f,
                           0.0f, -0.38268343236508977f, -0.70710678118654752f, -0.92387953251128674f,
                           -1.0f, -0.92387953251128674f, -0.70710678118654752f, -0.38268343236508977f,
                           0.0f, 0.38268343236508977f, 0.70710678118654752f, 0.92387953251128674f};
  return c[m];
}
__device__ __forceinline__ float w16s(int m) { return w16c((m + 12) & 15); }  // sin = cos(. - pi/2)

constexpr int bitrev(int q, int bits) {
  int r = 0;
  for (int i = 0; i < bits; ++i) r |= ((q >> i) & 1) << (bits - 1 - i);
  return r;
}
constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

// Radix-2 decimation-in-frequency network on R register values (natural
// order in, bit-reversed order out). sg = -1 forward, +1 inverse.
template <int R, int HALF, bool INV>
__device__ __forceinline__ void dif_stage(float* xr, float* xi) {
  if constexpr (HALF >= 1) {
#pragma unroll
    for (int base = 0; base < R; base += 2 * HALF) {
#pragma unroll
      for (int k = 0; k < HALF; ++k) {
        const float ar = xr[base + k], ai = xi[base + k];
        const float br = xr[base + k + HALF], bi = xi[base + k + HALF];
        xr[base + k] = ar + br;
        xi[base + k] = ai + bi;
        const float dr = ar - br, di = ai - bi;
        constexpr int step = 16 / (2 * HALF);
        const int m = k * step;
        if (m == 0) {
          xr[base + k + HALF] = dr;
          xi[base + k + HALF] = di;
        } else if (m == 4) {  // times -i (forward) or +i (inverse)
          xr[base + k + HALF] = INV ? -di : di;
          xi[base + k + HALF] = INV ? dr : -dr;
        } else {
          const float c = w16c(m), s = INV ? w16s(m) : -w16s(m);
          xr[base + k + HALF] = dr * c - di * s;
          xi[base + k + HALF] = dr * s + di * c;
        }
      }
    }
    dif_stage<R, HALF / 2, INV>(xr, xi);
  }
}

// Shared-memory swizzle: word address s is stored at s ^ ((s >> 4) & 31).
// It permutes words within each aligned 32-word row, and it makes every
// access of these transforms (32 consecutive elements, the stride-16 stores
// of a radix-16 stage, the (g, k) scatter of the later stages, and the
// column tile's 16-column rows) hit 32 distinct banks (checked exhaustively
// for N = 256..4096).
__device__ __forceinline__ int swz(int s) { return s ^ ((s >> 4) & 31); }

// Row layout: transform t at t * N.
template <int N>
struct RowAddr {
  static constexpr int NP = N;
  __device__ __forceinline__ static int at(int t, int m) { return t * N + swz(m); }
};
// Column layout: element m of column t at m * COLS + t.
template <int COLS>
struct ColAddr {
  static constexpr int PITCH = COLS;
  __device__ __forceinline__ static int at(int t, int m) { return swz(m * COLS + t); }
};

// One Stockham stage of radix R at sub-length L; each thread owns 16 / R
// butterflies j = u + i N / 16.
template <int N, int R, int L, bool INV, class A>
__device__ __forceinline__ void stockham_stage(float* __restrict__ re, float* __restrict__ im,
                                               int t, int u, const float2* __restrict__ tw) {
  constexpr int TPT = N / 16;
  constexpr int BPT = 16 / R;
  constexpr int STRIDE = N / R;
  constexpr int TWSTEP = N / (L * R);
  float xr[16], xi[16];
#pragma unroll
  for (int i = 0; i < BPT; ++i) {
    const int j = u + i * TPT;
    const int k = j % L, g = j / L;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int m = g * L + k + q * STRIDE;
      float a = re[A::at(t, m)], b = im[A::at(t, m)];
      if (L > 1 && q > 0) {
        const float2 w = __ldg(&tw[k * q * TWSTEP]);
        const float ws = INV ? w.y : -w.y;
        const float tr = a * w.x - b * ws;
        b = a * ws + b * w.x;
        a = tr;
      }
      xr[i * R + q] = a;
      xi[i * R + q] = b;
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < BPT; ++i) {
    dif_stage<R, R / 2, INV>(&xr[i * R], &xi[i * R]);
    const int j = u + i * TPT;
    const int k = j % L, g = j / L;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int m = g * L * R + k + q * L;
      constexpr int bits = ilog2c(R);
      re[A::at(t, m)] = xr[i * R + bitrev(q, bits)];
      im[A::at(t, m)] = xi[i * R + bitrev(q, bits)];
    }
  }
  __syncthreads();
}

// Full transform: radix-16 stages first, then one radix 2^(log2 N mod 4)
// stage if needed. (Radix 16 first keeps every stage's stores either
// contiguous or at stride 16, which the one-in-16 padding makes
// conflict-free.)
template <int N, int L, bool INV, class A>
__device__ __forceinline__ void stockham_from(float* re, float* im, int t, int u,
                                              const float2* tw) {
  if constexpr (L * 16 <= N) {
    stockham_stage<N, 16, L, INV, A>(re, im, t, u, tw);
    stockham_from<N, L * 16, INV, A>(re, im, t, u, tw);
  } else if constexpr (L < N) {
    stockham_stage<N, N / L, L, INV, A>(re, im, t, u, tw);
  }
}

template <int N, bool INV, class A>
__device__ __forceinline__ void smem_fft(float* re, float* im, int t, int u, const float2* tw) {
  stockham_from<N, 1, INV, A>(re, im, t, u, tw);
}

template <int N>
struct RowCfg {
  static constexpr int TPT = N / 16;
  static constexpr int ROWS = 4096 / N > 0 ? 4096 / N : 1;  // 256 threads per CTA
  static constexpr int THREADS = ROWS * TPT;
  static constexpr size_t SMEM = (size_t)ROWS * RowAddr<N>::NP * 8;
};
template <int N>
struct ColCfg {
  static constexpr int TPT = N / 16;
  static constexpr int COLS = N >= 2048 ? 16 * 1024 / N : 16;
  static constexpr int THREADS = COLS * TPT;
  static constexpr size_t SMEM = (size_t)COLS * N * 8;
};

// Row pass with fused element prologue / epilogue.
template <int N, bool INV>
__global__ void __launch_bounds__(RowCfg<N>::THREADS, 3)
    k_fft_rows(float* __restrict__ field, float scale, const float2* __restrict__ tw, PixOps pro,
               PixOps epi, FieldInfo fi) {
  using CF = RowCfg<N>;
  using A = RowAddr<N>;
  extern __shared__ float sm[];
  float* re = sm;
  float* im = sm + CF::ROWS * A::NP;
  constexpr int CPF = N / CF::ROWS;  // CTAs per field
  const int f = blockIdx.x / CPF;
  const int r0 = (blockIdx.x % CPF) * CF::ROWS;
  const size_t plane = (size_t)N * N;
  float* fre = field + (size_t)f * 2 * plane + (size_t)r0 * N;
  float* fim = fre + plane;
  PixConsts kp, ke;
  if (pro.n) pix_consts(pro, fi, f, N, N, kp);
  if (epi.n) pix_consts(epi, fi, f, N, N, ke);
  const bool gen = pro.n && pro.kind[0] == OP_SOURCE;  // source overwrites: skip the read
  // one element per thread per instruction: coalesced global access and
  // consecutive (conflict-free) shared-memory addresses
  constexpr int NE = CF::ROWS * N;
#pragma unroll 4
  for (int e = threadIdx.x; e < NE; e += CF::THREADS) {
    const int t = e / N, m = e % N;
    float xr = 0.f, xi = 0.f;
    if (!gen) {
      xr = fre[e];
      xi = fim[e];
    }
    if (pro.n) pix_apply(pro, kp, r0 + t, m, N, N, xr, xi);
    re[A::at(t, m)] = xr;
    im[A::at(t, m)] = xi;
  }
  __syncthreads();
  const int t = threadIdx.x / CF::TPT, u = threadIdx.x % CF::TPT;
  smem_fft<N, INV, A>(re, im, t, u, tw);
#pragma unroll 4
  for (int e = threadIdx.x; e < NE; e += CF::THREADS) {
    const int tt = e / N, m = e % N;
    float xr = re[A::at(tt, m)] * scale, xi = im[A::at(tt, m)] * scale;
    if (epi.n) pix_apply(epi, ke, r0 + tt, m, N, N, xr, xi);
    fre[e] = xr;
    fim[e] = xi;
  }
}

// Angular-spectrum transfer function (csim_fft.cpp:377-386):
//   H = exp(2 pi i [z/lambda sqrt(1 - eps)]), eps = (lambda/apRad)^2 f^2 / 4
//   turns = z/lambda - K f^2 / 2 - K f^2 h,  K = z lambda / (4 apRad^2),
//   h = eps / (2 (1 + sqrt(1 - eps))^2)
// with f^2 the fftshifted integer frequency index squared. The large terms
// are reduced in FP64 (z/lambda) and double-float (K f^2 / 2); eps > 1
// (evanescent) gives NaN like the reference's real sqrt.
struct FresnelConsts {
  float t0, khi, klo, K, c_eps;
};

__device__ __forceinline__ FresnelConsts fresnel_consts(double lam, double z, double ap_rad) {
  FresnelConsts c;
  double t0 = z / lam;
  t0 -= rint(t0);
  const double K = z * lam / (4.0 * ap_rad * ap_rad);
  split_f64_pair(0.5 * K, c.khi, c.klo);
  c.K = (float)K;
  c.c_eps = (float)(0.25 * (lam / ap_rad) * (lam / ap_rad));
  c.t0 = (float)t0;
  return c;
}

__device__ __forceinline__ float2 fresnel_h(int N, int r, int c, const FresnelConsts& k) {
  const int fr = r < N / 2 ? r : r - N;
  const int fc = c < N / 2 ? c : c - N;
  const float f2 = (float)(fr * fr + fc * fc);  // exact: < 2^24
  const float eps = k.c_eps * f2;
  const float s = sqrtf(1.f - eps);
  const float h = eps / (2.f * (1.f + s) * (1.f + s));
  float tt = k.t0 - frac_prod(f2, k.khi, k.klo) - k.K * f2 * h;
  tt -= rintf(tt);
  float sn, cs;
  sincospif(2.f * tt, &sn, &cs);
  return make_float2(cs, sn);
}

__global__ void k_fresnel_table(int N, const double* lam, double z, double ap_rad,
                                float2* __restrict__ out) {
  const int s = blockIdx.y;
  const FresnelConsts fc = fresnel_consts(lam[s], z, ap_rad);
  const int plane = N * N;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += gridDim.x * blockDim.x)
    out[(size_t)s * plane + i] = fresnel_h(N, i / N, i % N, fc);
}

int build_fresnel_table(cudaStream_t st, int N, const double* lam, int n_slot, double z,
                        double ap_rad, float2* out) {
  dim3 grid(grid_for((long long)N * N, 256, 1024), n_slot);
  k_fresnel_table<<<grid, 256, 0, st>>>(N, lam, z, ap_rad, out);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

// Column pass; MODE 0: forward, 1: inverse, 2: forward * H(lambda_f) * inverse.
template <int N, int MODE>
__global__ void __launch_bounds__(ColCfg<N>::THREADS)
    k_fft_cols(float* __restrict__ field, const float2* __restrict__ tw, FresnelArgs fa) {
  using CF = ColCfg<N>;
  using A = ColAddr<CF::COLS>;
  extern __shared__ float sm[];
  float* re = sm;
  float* im = sm + A::PITCH * N;
  constexpr int CPF = N / CF::COLS;
  const int f = blockIdx.x / CPF;
  const int c0 = (blockIdx.x % CPF) * CF::COLS;
  const size_t plane = (size_t)N * N;
  float* fre = field + (size_t)f * 2 * plane + c0;
  float* fim = fre + plane;
  constexpr int NE = CF::COLS * N;
#pragma unroll 4
  for (int i = threadIdx.x; i < NE; i += CF::THREADS) {
    const int r = i / CF::COLS, c = i % CF::COLS;
    re[A::at(c, r)] = fre[(size_t)r * N + c];
    im[A::at(c, r)] = fim[(size_t)r * N + c];
  }
  __syncthreads();
  const int t = threadIdx.x % CF::COLS, u = threadIdx.x / CF::COLS;
  smem_fft<N, MODE == 1, A>(re, im, t, u, tw);
  if (MODE == 2) {
    if (fa.H) {  // per-wavelength table (L2-resident, shared by the batch)
      const float2* Hs = fa.H + (size_t)fa.slot[f] * N * N + c0;
#pragma unroll 4
      for (int i = threadIdx.x; i < NE; i += CF::THREADS) {
        const int r = i / CF::COLS, cl = i % CF::COLS;
        const float2 w = Hs[(size_t)r * N + cl];
        const int a = A::at(cl, r);
        const float xr = re[a], xi = im[a];
        re[a] = xr * w.x - xi * w.y;
        im[a] = xr * w.y + xi * w.x;
      }
    } else {
      const FresnelConsts fc = fresnel_consts(fa.lambda[f], fa.z, fa.ap_rad);
      for (int i = threadIdx.x; i < NE; i += CF::THREADS) {
        const int r = i / CF::COLS, cl = i % CF::COLS;
        const float2 w = fresnel_h(N, r, c0 + cl, fc);
        const int a = A::at(cl, r);
        const float xr = re[a], xi = im[a];
        re[a] = xr * w.x - xi * w.y;
        im[a] = xr * w.y + xi * w.x;
      }
    }
    __syncthreads();
    smem_fft<N, true, A>(re, im, t, u, tw);
  }
#pragma unroll 4
  for (int i = threadIdx.x; i < NE; i += CF::THREADS) {
    const int r = i / CF::COLS, c = i % CF::COLS;
    fre[(size_t)r * N + c] = re[A::at(c, r)];
    fim[(size_t)r * N + c] = im[A::at(c, r)];
  }
}

template <typename K>
static int prep_smem(K kern, size_t bytes) {
  CSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  // optional shared-memory carveout preference (percent), for tuning
  static const char* cv = getenv("CSG_FFT_CARVEOUT");
  if (cv) CSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, atoi(cv)));
  return CSG_OK;
}

template <int N>
static int run_fft(csg_ctx* ctx, float* field, int F, int direction, const FresnelArgs* fa,
                   const PixOps& pro, const PixOps& epi, const FieldInfo& fi, const float2* tw) {
  using RC = RowCfg<N>;
  using CC = ColCfg<N>;
  cudaStream_t st = ctx->stream;
  const int rgrid = F * (N / RC::ROWS), cgrid = F * (N / CC::COLS);
  const float inv_scale = 1.f / ((float)N * (float)N);
  const double pass_bytes = (double)F * N * N * 16.0;
  const PixOps none;
  int rc;
  auto rows = [&](bool inv, float scale, const PixOps& p, const PixOps& e) -> int {
    const bool gen = p.n && p.kind[0] == OP_SOURCE;
    ProfScope ps(ctx, inv ? "fft_rows_inv" : "fft_rows_fwd", 0, pass_bytes * (gen ? 0.5 : 1.0));
    if (inv) {
      if ((rc = prep_smem(k_fft_rows<N, true>, RC::SMEM))) return rc;
      k_fft_rows<N, true><<<rgrid, RC::THREADS, RC::SMEM, st>>>(field, scale, tw, p, e, fi);
    } else {
      if ((rc = prep_smem(k_fft_rows<N, false>, RC::SMEM))) return rc;
      k_fft_rows<N, false><<<rgrid, RC::THREADS, RC::SMEM, st>>>(field, scale, tw, p, e, fi);
    }
    CSG_LAUNCH_CHECK();
    return CSG_OK;
  };
  auto cols = [&](int mode) -> int {
    ProfScope ps(ctx, mode == 2 ? "fft_cols_fresnel" : "fft_cols", 0, pass_bytes);
    if (mode == 2) {
      if ((rc = prep_smem(k_fft_cols<N, 2>, CC::SMEM))) return rc;
      k_fft_cols<N, 2><<<cgrid, CC::THREADS, CC::SMEM, st>>>(field, tw, *fa);
    } else if (mode == 1) {
      if ((rc = prep_smem(k_fft_cols<N, 1>, CC::SMEM))) return rc;
      k_fft_cols<N, 1><<<cgrid, CC::THREADS, CC::SMEM, st>>>(field, tw, FresnelArgs{});
    } else {
      if ((rc = prep_smem(k_fft_cols<N, 0>, CC::SMEM))) return rc;
      k_fft_cols<N, 0><<<cgrid, CC::THREADS, CC::SMEM, st>>>(field, tw, FresnelArgs{});
    }
    CSG_LAUNCH_CHECK();
    return CSG_OK;
  };
  if (fa) {
    if ((rc = rows(false, 1.f, pro, none))) return rc;
    if ((rc = cols(2))) return rc;
    return rows(true, inv_scale, none, epi);
  } else if (direction < 0) {
    if ((rc = rows(false, 1.f, pro, none))) return rc;
    if ((rc = cols(0))) return rc;
    if (epi.n) return pixops_pass(st, field, F, N, N, epi, fi);
  } else {
    if (pro.n && (rc = pixops_pass(st, field, F, N, N, pro, fi))) return rc;
    if ((rc = cols(1))) return rc;
    return rows(true, inv_scale, none, epi);
  }
  return CSG_OK;
}

// 2-D FFT or Fresnel propagation of F square N x N fields with fused element
// ops (pro before the transform, epi after it).
int fft2d_fused(csg_ctx* ctx, float* field, int F, int n, int direction, const FresnelArgs* fa,
                const PixOps& pro, const PixOps& epi, const FieldInfo& fi) {
  CSG_CHECK(n >= 64 && n <= 4096 && (n & (n - 1)) == 0, CSG_E_SHAPE,
            "FFT size must be a power of two in [64, 4096]");
  CSG_CHECK(F > 0 && (long long)F * n < (1LL << 31), CSG_E_SHAPE, "FFT: bad field count");
  cudaStream_t st = ctx->stream;
  const float2* tw = twiddles(ctx->device, n, st);
  CSG_CHECK(tw != nullptr, CSG_E_NOMEM, "twiddle table allocation failed");
  const double pass_bytes = (double)F * n * n * 16.0;
  const bool gen = pro.n && pro.kind[0] == OP_SOURCE;  // the first pass only writes
  ProfScope ps(ctx, fa ? "fresnel_3pass" : "fft2d_2pass", 0,
               pass_bytes * ((fa ? 3.0 : 2.0) - (gen ? 0.5 : 0.0)));
  switch (n) {
    case 64: return run_fft<64>(ctx, field, F, direction, fa, pro, epi, fi, tw);
    case 128: return run_fft<128>(ctx, field, F, direction, fa, pro, epi, fi, tw);
    case 256: return run_fft<256>(ctx, field, F, direction, fa, pro, epi, fi, tw);
    case 512: return run_fft<512>(ctx, field, F, direction, fa, pro, epi, fi, tw);
    case 1024: return run_fft<1024>(ctx, field, F, direction, fa, pro, epi, fi, tw);
    case 2048: return run_fft<2048>(ctx, field, F, direction, fa, pro, epi, fi, tw);
    default: return run_fft<4096>(ctx, field, F, direction, fa, pro, epi, fi, tw);
  }
}

}  // namespace csg

using namespace csg;

extern "C" {

int csg_fft2d(csg_ctx* ctx, float* field, int n_fields, int n, int direction) {
  CSG_CHECK(ctx && field, CSG_E_ARG, "csg_fft2d: null argument");
  CSG_CHECK(direction == -1 || direction == 1, CSG_E_ARG, "csg_fft2d: direction must be -1 or +1");
  DeviceGuard g(ctx->device);
  return fft2d_fused(ctx, field, n_fields, n, direction, nullptr, PixOps(), PixOps(), FieldInfo());
}

int csg_fresnel(csg_ctx* ctx, float* field, int n_fields, int n, const double* lambda,
                double ap_rad, double z) {
  CSG_CHECK(ctx && field && lambda, CSG_E_ARG, "csg_fresnel: null argument");
  CSG_CHECK(ap_rad > 0, CSG_E_ARG, "csg_fresnel: apRad must be positive");
  DeviceGuard g(ctx->device);
  FresnelArgs fa{lambda, z, ap_rad};
  return fft2d_fused(ctx, field, n_fields, n, -1, &fa, PixOps(), PixOps(), FieldInfo());
}

}  // extern "C"
