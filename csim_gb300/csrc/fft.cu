// Register-resident Stockham FFTs for square N x N planar fp32 fields and
// the fused angular-spectrum Fresnel pipeline.
//
// A 2-D transform is two HBM passes: a row pass (256 threads: 256 E / N
// rows per CTA) and a column pass (COLS columns per CTA). Each pass reads
// and writes the field once. Every thread owns E elements of one transform
// (E = 32 from N = 512 up, 16 below), u + s N/E, which it loads straight
// from global memory and stores straight back: the first stage runs on the
// registers as loaded and the last stage leaves its outputs in the same
// natural order, so shared memory carries only the exchanges between stages
// (one for N = 1024: radix 32 x 32). The radix-R butterflies are unrolled
// radix-2 decimation-in-frequency networks with exact W32 constants;
// inter-stage twiddles come from an FP64-generated table. Shared memory is
// XOR-swizzled (swz) so every stage access is bank-conflict-free.
//
// Element ops (point source, masks, mirrors) ride along in the row passes'
// prologue and epilogue (pixops.cuh), so they cost no extra HBM pass.
//
// Fresnel (csim_fft.cpp:371-392) is row FFT | column FFT x H x column IFFT |
// row IFFT / N^2: three passes; H comes from a per-wavelength table or is
// generated in-kernel from the integer frequency index.
#include <map>
#include <mutex>
#include <type_traits>
#include <vector>

#include "ctx.hpp"
#include "dfloat.cuh"
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

// Two-float twiddles: (cos hi, cos lo, sin hi, sin lo).
__global__ void k_twiddles_df(float4* tw, int n) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)m / (double)n, &s, &c);
    const float2 a = split_f64(c), b = split_f64(s);
    tw[m] = make_float4(a.x, a.y, b.x, b.y);
  }
}

static const float4* twiddles_df(int device, int n, cudaStream_t st) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, float4*> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(device, n);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  float4* p = nullptr;
  if (cudaMalloc(&p, sizeof(float4) * n) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  k_twiddles_df<<<(n + 255) / 256, 256, 0, st>>>(p, n);
  cudaStreamSynchronize(st);
  cache[key] = p;
  return p;
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
// cos and sin of 2 pi m / 32.
__device__ __forceinline__ float w32c(int m) {
  constexpr float c[32] = {
      1.0f,  0.98078528040323043f,  0.92387953251128674f,  0.83146961230254524f,
      0.70710678118654757f,  0.55557023301960218f,  0.38268343236508978f,  0.19509032201612828f,
      0.0f, -0.19509032201612828f, -0.38268343236508978f, -0.55557023301960218f,
      -0.70710678118654757f, -0.83146961230254524f, -0.92387953251128674f, -0.98078528040323043f,
      -1.0f, -0.98078528040323043f, -0.92387953251128674f, -0.83146961230254524f,
      -0.70710678118654757f, -0.55557023301960218f, -0.38268343236508978f, -0.19509032201612828f,
      0.0f,  0.19509032201612828f,  0.38268343236508978f,  0.55557023301960218f,
      0.70710678118654757f,  0.83146961230254524f,  0.92387953251128674f,  0.98078528040323043f};
  return c[m];
}
__device__ __forceinline__ float w32s(int m) { return w32c((m + 24) & 31); }  // sin = cos(. - pi/2)
// The same as two-float constants (fp32 rounding of cos(pi m / 16) and of
// the rest), symmetric by construction.
__device__ __forceinline__ dfl w32c_df(int m) {
  constexpr float h[32] = {
      1.0f, 0.9807852506637573f, 0.9238795042037964f, 0.8314695954322815f, 0.7071067690849304f,
      0.5555702447891235f, 0.3826834261417389f, 0.19509032368659973f, 0.0f,
      -0.19509032368659973f, -0.3826834261417389f, -0.5555702447891235f, -0.7071067690849304f,
      -0.8314695954322815f, -0.9238795042037964f, -0.9807852506637573f, -1.0f,
      -0.9807852506637573f, -0.9238795042037964f, -0.8314695954322815f, -0.7071067690849304f,
      -0.5555702447891235f, -0.3826834261417389f, -0.19509032368659973f, 0.0f,
      0.19509032368659973f, 0.3826834261417389f, 0.5555702447891235f, 0.7071067690849304f,
      0.8314695954322815f, 0.9238795042037964f, 0.9807852506637573f};
  constexpr float l[32] = {
      0.0f, 2.9739473106360492e-08f, 2.830748968563057e-08f, 1.687026340846387e-08f,
      1.2101617485882343e-08f, -1.1769521357507529e-08f, 6.2233507236442165e-09f,
      -1.670471427850373e-09f, 0.0f, 1.670471427850373e-09f, -6.2233507236442165e-09f,
      1.1769521357507529e-08f, -1.2101617485882343e-08f, -1.687026340846387e-08f,
      -2.830748968563057e-08f, -2.9739473106360492e-08f, 0.0f, -2.9739473106360492e-08f,
      -2.830748968563057e-08f, -1.687026340846387e-08f, -1.2101617485882343e-08f,
      1.1769521357507529e-08f, -6.2233507236442165e-09f, 1.670471427850373e-09f, 0.0f,
      -1.670471427850373e-09f, 6.2233507236442165e-09f, -1.1769521357507529e-08f,
      1.2101617485882343e-08f, 1.687026340846387e-08f, 2.830748968563057e-08f,
      2.9739473106360492e-08f};
  return dfl{h[m], l[m]};
}
__device__ __forceinline__ dfl w32s_df(int m) { return w32c_df((m + 24) & 31); }

// Arithmetic of the transforms: fp32, or two-float (CSG_PREC_HIGH).
__device__ __forceinline__ float vadd(float a, float b) { return a + b; }
__device__ __forceinline__ float vsub(float a, float b) { return a - b; }
__device__ __forceinline__ float vneg(float a) { return -a; }
__device__ __forceinline__ dfl vadd(dfl a, dfl b) { return df_add(a, b); }
__device__ __forceinline__ dfl vsub(dfl a, dfl b) { return df_sub(a, b); }
__device__ __forceinline__ dfl vneg(dfl a) { return df_neg(a); }

// (dr + i di) times W_32^m (forward e^-i, inverse e^+i) for m != 0, 8.
template <bool INV>
__device__ __forceinline__ void mul_w32(float dr, float di, int m, float& orr, float& oi) {
  const float c = w32c(m), s = INV ? w32s(m) : -w32s(m);
  orr = dr * c - di * s;
  oi = dr * s + di * c;
}
template <bool INV>
__device__ __forceinline__ void mul_w32(dfl dr, dfl di, int m, dfl& orr, dfl& oi) {
  const dfl c = w32c_df(m), s = INV ? w32s_df(m) : df_neg(w32s_df(m));
  df_cmul(dr, di, c, s, orr, oi);
}

// Twiddle tables: cos, sin of 2 pi m / N as float2 (fp32) or float4
// (two-float: cos hi, cos lo, sin hi, sin lo), both generated in FP64.
template <class T> struct TwOf;
template <> struct TwOf<float> { using type = float2; };
template <> struct TwOf<dfl> { using type = float4; };

template <bool INV>
__device__ __forceinline__ void mul_tw(const float2* tw, int idx, float& a, float& b) {
  const float2 w = __ldg(&tw[idx]);
  const float ws = INV ? w.y : -w.y;
  const float tr = a * w.x - b * ws;
  b = a * ws + b * w.x;
  a = tr;
}
template <bool INV>
__device__ __forceinline__ void mul_tw(const float4* tw, int idx, dfl& a, dfl& b) {
  const float4 w = __ldg(&tw[idx]);
  const dfl c{w.x, w.y};
  const dfl s = INV ? dfl{w.z, w.w} : dfl{-w.z, -w.w};
  dfl ra, rb;
  df_cmul(a, b, c, s, ra, rb);
  a = ra;
  b = rb;
}

// Shared-memory words of one value: fp32 values take one word; two-float
// values keep their low words LO words further on (their own planes).
template <int LO>
__device__ __forceinline__ void sld(const float* p, int i, float& v) { v = p[i]; }
template <int LO>
__device__ __forceinline__ void sld(const float* p, int i, dfl& v) { v = dfl{p[i], p[i + LO]}; }
template <int LO>
__device__ __forceinline__ void sst(float* p, int i, float v) { p[i] = v; }
template <int LO>
__device__ __forceinline__ void sst(float* p, int i, dfl v) {
  p[i] = v.h;
  p[i + LO] = v.l;
}

constexpr int bitrev(int q, int bits) {
  int r = 0;
  for (int i = 0; i < bits; ++i) r |= ((q >> i) & 1) << (bits - 1 - i);
  return r;
}
constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

// Packed fp32 pairs: one add.f32x2 / sub.f32x2 instruction for two sums
// (the register pairs are formed and split by mov.b64, which costs nothing
// when the two values sit in adjacent registers).
__device__ __forceinline__ void add2(float a0, float a1, float b0, float b1, float& s0, float& s1) {
  asm("{\n\t.reg .b64 x, y, r;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\t"
      "add.rn.f32x2 r, x, y;\n\tmov.b64 {%0, %1}, r;\n\t}"
      : "=f"(s0), "=f"(s1)
      : "f"(a0), "f"(a1), "f"(b0), "f"(b1));
}
__device__ __forceinline__ void sub2(float a0, float a1, float b0, float b1, float& s0, float& s1) {
  asm("{\n\t.reg .b64 x, y, r;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\t"
      "sub.rn.f32x2 r, x, y;\n\tmov.b64 {%0, %1}, r;\n\t}"
      : "=f"(s0), "=f"(s1)
      : "f"(a0), "f"(a1), "f"(b0), "f"(b1));
}

// Sums and differences of two values at once (packed pairs).
__device__ __forceinline__ void pair_add(float a0, float a1, float b0, float b1, float& r0,
                                         float& r1) {
  add2(a0, a1, b0, b1, r0, r1);
}
__device__ __forceinline__ void pair_sub(float a0, float a1, float b0, float b1, float& r0,
                                         float& r1) {
  sub2(a0, a1, b0, b1, r0, r1);
}
__device__ __forceinline__ void pair_add(dfl a0, dfl a1, dfl b0, dfl b1, dfl& r0, dfl& r1) {
  df_add2(a0, a1, b0, b1, r0, r1);
}
__device__ __forceinline__ void pair_sub(dfl a0, dfl a1, dfl b0, dfl b1, dfl& r0, dfl& r1) {
  df_sub2(a0, a1, b0, b1, r0, r1);
}

// Radix-2 decimation-in-frequency network on R register values (natural
// order in, bit-reversed order out). sg = -1 forward, +1 inverse. The sums
// and differences of butterflies k and k + 1 (HALF >= 2) go through packed
// pairs (fp32 or two-float): the same round-to-nearest results, half the
// adds issued.
template <int R, int HALF, bool INV, class T>
__device__ __forceinline__ void dif_stage(T* xr, T* xi) {
  if constexpr (HALF >= 1) {
    constexpr bool PAIRED = HALF >= 2;
#pragma unroll
    for (int base = 0; base < R; base += 2 * HALF) {
      T dpr[HALF], dpi[HALF];  // differences (paired path)
      if constexpr (PAIRED) {
#pragma unroll
        for (int k = 0; k < HALF; k += 2) {
          const int a = base + k, b = base + k + HALF;
          T sr0, sr1, si0, si1;
          pair_sub(xr[a], xr[a + 1], xr[b], xr[b + 1], dpr[k], dpr[k + 1]);
          pair_sub(xi[a], xi[a + 1], xi[b], xi[b + 1], dpi[k], dpi[k + 1]);
          pair_add(xr[a], xr[a + 1], xr[b], xr[b + 1], sr0, sr1);
          pair_add(xi[a], xi[a + 1], xi[b], xi[b + 1], si0, si1);
          xr[a] = sr0, xr[a + 1] = sr1, xi[a] = si0, xi[a + 1] = si1;
        }
      }
#pragma unroll
      for (int k = 0; k < HALF; ++k) {
        T dr, di;
        if constexpr (PAIRED) {
          dr = dpr[k];
          di = dpi[k];
        } else {
          const T ar = xr[base + k], ai = xi[base + k];
          const T br = xr[base + k + HALF], bi = xi[base + k + HALF];
          xr[base + k] = vadd(ar, br);
          xi[base + k] = vadd(ai, bi);
          dr = vsub(ar, br);
          di = vsub(ai, bi);
        }
        constexpr int step = 32 / (2 * HALF);  // twiddle W_{2 HALF}^k = W_32^(k step)
        const int m = k * step;
        if (m == 0) {
          xr[base + k + HALF] = dr;
          xi[base + k + HALF] = di;
        } else if (m == 8) {  // times -i (forward) or +i (inverse)
          xr[base + k + HALF] = INV ? vneg(di) : di;
          xi[base + k + HALF] = INV ? dr : vneg(dr);
        } else {
          mul_w32<INV>(dr, di, m, xr[base + k + HALF], xi[base + k + HALF]);
        }
      }
    }
    dif_stage<R, HALF / 2, INV, T>(xr, xi);
  }
}

// Shared-memory swizzle for E elements per thread: word address s is stored
// at s ^ ((s >> log2 E) & 31), a bijection that permutes words within each
// aligned 32-word row. It makes every shared-memory access of these
// transforms (the stride-E stores of the first stage, the (g, k) gathers and
// scatters of the later stages, for rows of any N and for column tiles of 4,
// 8 or 16 columns) hit 32 distinct banks; checked exhaustively for
// N = 64..4096, E = 16 and 32.
template <int E>
__device__ __forceinline__ int swz(int s) {
  return s ^ ((s >> ilog2c(E)) & 31);
}

// Row layout: element m of transform t at t * N + m.
template <int N, int E>
struct RowAddr {
  __device__ __forceinline__ static int at(int t, int m) { return swz<E>(t * N + m); }
};
// Column layout: element m of column t at m * COLS + t.
template <int COLS, int E>
struct ColAddr {
  static constexpr int PITCH = COLS;
  __device__ __forceinline__ static int at(int t, int m) { return swz<E>(m * COLS + t); }
};

// Stockham stages of radix R at sub-length L. Each thread owns E / R
// butterflies j = u + i N / E of one transform (index t of the tile).
// stage_read gathers a stage's inputs (with the inter-stage twiddles) into
// registers, stage_write scatters its outputs. LO: offset of the low-word
// planes (two-float values).
template <int N, int E, int R, int L, bool INV, class A, int LO, class T, class TW>
__device__ __forceinline__ void stage_read(const float* __restrict__ re,
                                           const float* __restrict__ im, int t, int u,
                                           const TW* __restrict__ tw, T* xr, T* xi) {
  constexpr int TPT = N / E, BPT = E / R, STRIDE = N / R, TWSTEP = N / (L * R);
#pragma unroll
  for (int i = 0; i < BPT; ++i) {
    const int j = u + i * TPT;
    const int k = j % L, g = j / L;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int m = g * L + k + q * STRIDE;
      T a, b;
      sld<LO>(re, A::at(t, m), a);
      sld<LO>(im, A::at(t, m), b);
      if (L > 1 && q > 0) mul_tw<INV>(tw, k * q * TWSTEP, a, b);
      xr[i * R + q] = a;
      xi[i * R + q] = b;
    }
  }
}

template <int E, int R, bool INV, class T>
__device__ __forceinline__ void stage_butterflies(T* xr, T* xi) {
#pragma unroll
  for (int i = 0; i < E / R; ++i) dif_stage<R, R / 2, INV, T>(&xr[i * R], &xi[i * R]);
}

template <int N, int E, int R, int L, class A, int LO, class T>
__device__ __forceinline__ void stage_write(float* __restrict__ re, float* __restrict__ im, int t,
                                            int u, const T* xr, const T* xi) {
  constexpr int TPT = N / E, BPT = E / R, bits = ilog2c(R);
#pragma unroll
  for (int i = 0; i < BPT; ++i) {
    const int j = u + i * TPT;
    const int k = j % L, g = j / L;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int m = g * L * R + k + q * L;
      sst<LO>(re, A::at(t, m), xr[i * R + bitrev(q, bits)]);
      sst<LO>(im, A::at(t, m), xi[i * R + bitrev(q, bits)]);
    }
  }
}

// Stages from sub-length L on: shared memory holds the output of the stages
// before L. Radix E while E L < N, then one final stage of radix N / L
// whose outputs stay in registers in natural order.
template <int N, int E, int L, bool INV, class A, int LO, class T, class TW>
__device__ __forceinline__ void fft_tail(T* xr, T* xi, float* re, float* im, int t, int u,
                                         const TW* tw) {
  if constexpr (L * E < N) {
    stage_read<N, E, E, L, INV, A, LO>(re, im, t, u, tw, xr, xi);
    __syncthreads();
    stage_butterflies<E, E, INV>(xr, xi);
    stage_write<N, E, E, L, A, LO>(re, im, t, u, xr, xi);
    __syncthreads();
    fft_tail<N, E, L * E, INV, A, LO>(xr, xi, re, im, t, u, tw);
  } else {
    constexpr int R = N / L, BPT = E / R, bits = ilog2c(R);
    T yr[E], yi[E];
    stage_read<N, E, R, L, INV, A, LO>(re, im, t, u, tw, yr, yi);
    stage_butterflies<E, R, INV>(yr, yi);
    // the last stage writes element k + q L with k = j = u + i N/E and
    // L = BPT N/E: element u + (i + q BPT) N/E
#pragma unroll
    for (int i = 0; i < BPT; ++i)
#pragma unroll
      for (int q = 0; q < R; ++q) {
        xr[i + q * BPT] = yr[i * R + bitrev(q, bits)];
        xi[i + q * BPT] = yi[i * R + bitrev(q, bits)];
      }
  }
}

// Length-N transform held by N/E threads: on entry and on exit register s
// of thread u holds element u + s N/E (natural order). The first stage
// (radix E, no twiddles) runs on the registers as loaded, so the caller
// loads straight from global memory and stores the result straight back;
// shared memory carries only the exchanges between stages. The caller
// synchronises before shared memory is reused by another transform.
template <int N, int E, bool INV, class A, int LO, class T, class TW>
__device__ __forceinline__ void fft_regs(T* xr, T* xi, float* re, float* im, int t, int u,
                                         const TW* tw) {
  stage_butterflies<E, E, INV>(xr, xi);
  stage_write<N, E, E, 1, A, LO>(re, im, t, u, xr, xi);
  __syncthreads();
  fft_tail<N, E, E, INV, A, LO>(xr, xi, re, im, t, u, tw);
}

// Elements per thread: 32 (radix-32 stages, one shared-memory exchange at
// N = 1024, 128 registers) from N = 512 up, 16 below; two-float transforms
// always 16 (64 registers of values).
constexpr int default_e(int n) { return n >= 512 ? 32 : 16; }
template <class T>
constexpr int elems_for(int n) {
  return std::is_same<T, dfl>::value ? 16 : default_e(n);
}
// CTAs per SM the register budget is sized for: 128 registers per thread at
// E = 32, 64-85 at E = 16; two-float row passes 128 at 256 threads.
constexpr int min_blocks(int e, int threads) {
  return e == 32 ? (threads >= 512 ? 1 : 512 / threads)
                 : (threads >= 1024 ? 1 : (threads >= 512 ? 2 : 3));
}
template <class T>
constexpr int min_blocks_t(int e, int threads) {
  return std::is_same<T, dfl>::value ? (threads >= 512 ? 1 : (threads >= 256 ? 2 : 4))
                                     : min_blocks(e, threads);
}
// Words per value in shared memory.
template <class T>
constexpr int words_of() {
  return std::is_same<T, dfl>::value ? 2 : 1;
}

template <int N, int E, class T = float>
struct RowCfg {
  static constexpr int TPT = N / E;
  static constexpr int ROWS = 256 / TPT > 0 ? 256 / TPT : 1;  // 256 threads per CTA
  static constexpr int THREADS = ROWS * TPT;
  static constexpr int MIN_BLOCKS = min_blocks_t<T>(E, THREADS);
  static constexpr int PLANE = ROWS * N;  // words of one component plane
  static constexpr size_t SMEM = (size_t)ROWS * N * 8 * words_of<T>();
};
// Column tile width: 8 columns (32-byte row segments) at N = 1024. Two-float
// tiles hold 256 threads (4 columns at N = 1024, 64 KB of shared memory),
// two CTAs per SM within 128 registers: the transfer-function pass fits
// without spilling once the inverse transform's indices are opaque (see
// k_fft_cols). Measured on the 152-field PIAACMC step at CSG_PREC_HIGH, the
// Fresnel column pass per step: 10.1 ms at one 256-thread CTA per SM (255
// registers), 7.2 ms at three 128-thread CTAs (168 registers, 336 bytes of
// spills), 4.4 ms at two 256-thread CTAs with the opaque indices (5.1 ms at
// four 128-thread CTAs).
constexpr int default_cols(int n) { return n <= 512 ? 16 : (n == 1024 ? 8 : 4); }
template <class T>
constexpr int cols_for(int n) {
  return std::is_same<T, dfl>::value ? (256 / (n / 16) > 0 ? 256 / (n / 16) : 1)
                                     : default_cols(n);
}
template <int N, int E, int COLS, class T = float>
struct ColCfg {
  static constexpr int TPT = N / E;
  static constexpr int THREADS = COLS * TPT;
  static constexpr int MIN_BLOCKS =
      std::is_same<T, dfl>::value ? (THREADS <= 128 ? 4 : 2) : min_blocks_t<T>(E, THREADS);
  static constexpr int PLANE = COLS * N;
  static constexpr size_t SMEM = (size_t)COLS * N * 8 * words_of<T>();
};

// Row pass with fused element prologue / epilogue. Two-float passes (T =
// dfl) apply the element ops in fp32 on the pupil-plane values as loaded and
// as rounded for the store; the transform itself runs in two-float.
template <int N, int E, bool INV, class T>
__global__ void __launch_bounds__(RowCfg<N, E, T>::THREADS, RowCfg<N, E, T>::MIN_BLOCKS)
    k_fft_rows(float* __restrict__ field, float scale,
               const typename TwOf<T>::type* __restrict__ tw,
               const __grid_constant__ PixOps pro, const __grid_constant__ PixOps epi,
               const __grid_constant__ FieldInfo fi, const FftBand band) {
  using CF = RowCfg<N, E, T>;
  using A = RowAddr<N, E>;
  constexpr int LO = 2 * CF::PLANE;
  constexpr bool DF = std::is_same<T, dfl>::value;
  extern __shared__ float sm[];
  __shared__ PixConsts shk[2];
  float* re = sm;
  float* im = sm + CF::PLANE;
  constexpr int TPT = CF::TPT;
  const int cpf = band.n ? band.n / CF::ROWS : N / CF::ROWS;  // CTAs per field
  const int f = blockIdx.x / cpf;
  const int t = threadIdx.x / TPT, u = threadIdx.x % TPT;
  const int row = band.lo + (blockIdx.x % cpf) * CF::ROWS + t;
  const size_t plane = (size_t)N * N;
  float* fre = field + (size_t)f * 2 * plane + (size_t)row * N + u;
  float* fim = fre + plane;
  // thread u of row t owns elements u + s N/E: each load and store
  // instruction of a warp covers 32 consecutive floats of a row
  float xr[E], xi[E];
  // band: element s is in the n-wide centre iff s0 <= s < s1
  const int s0 = band.lo / TPT, s1 = (band.lo + band.n) / TPT;
  const bool gen = pro.n && pro.kind[0] == OP_SOURCE;  // source overwrites: skip the read
  if (band.n && band.src && !INV) {  // rows of the n x n source, zero outside its columns
    const size_t np = (size_t)band.n * band.n;
    const float* sre = band.src + (size_t)f * 2 * np + (size_t)(row - band.lo) * band.n + u -
                       band.lo;
#pragma unroll
    for (int s = 0; s < E; ++s) {
      const bool in = s >= s0 && s < s1;
      xr[s] = in ? sre[s * TPT] : 0.f;
      xi[s] = in ? sre[np + s * TPT] : 0.f;
    }
  } else if (!gen) {
#pragma unroll
    for (int s = 0; s < E; ++s) {
      xr[s] = fre[s * TPT];
      xi[s] = fim[s * TPT];
    }
  } else {
#pragma unroll
    for (int s = 0; s < E; ++s) xr[s] = xi[s] = 0.f;
  }
  PixConsts kp, ke;
  if (pro.n) pix_consts_cta(pro, fi, f, N, N, kp, &shk[0]);
  if (epi.n) pix_consts_cta(epi, fi, f, N, N, ke, &shk[1]);
  // element ops in groups (bounds the live table values; the prologue's
  // wider groups put more table loads in flight at once)
  if (pro.n) {
    constexpr int G = E >= 16 ? 16 : E;
#pragma unroll
    for (int h = 0; h < E; h += G)
      pix_apply_n<G>(pro, kp, row, u + h * TPT, 0, TPT, N, N, xr + h, xi + h);
  }
  if constexpr (DF) {
    dfl yr[E], yi[E];
#pragma unroll
    for (int s = 0; s < E; ++s) {
      yr[s] = df_from(xr[s]);
      yi[s] = df_from(xi[s]);
    }
    fft_regs<N, E, INV, A, LO>(yr, yi, re, im, t, u, tw);
#pragma unroll
    for (int s = 0; s < E; ++s) {
      xr[s] = df_round(df_scale(yr[s], scale));  // scale: a power of two
      xi[s] = df_round(df_scale(yi[s], scale));
    }
  } else {
    fft_regs<N, E, INV, A, LO>(xr, xi, re, im, t, u, tw);
#pragma unroll
    for (int s = 0; s < E; ++s) xr[s] *= scale, xi[s] *= scale;
  }
  if (epi.n) {
#pragma unroll
    for (int h = 0; h < E; h += 8)
      pix_apply_n<8>(epi, ke, row, u + h * TPT, 0, TPT, N, N, xr + h, xi + h);
  }
  if (band.n && band.dst && INV) {  // the centre n columns straight to the n x n field
    const size_t np = (size_t)band.n * band.n;
    float* dre = band.dst + (size_t)f * 2 * np + (size_t)(row - band.lo) * band.n + u - band.lo;
#pragma unroll
    for (int s = 0; s < E; ++s)
      if (s >= s0 && s < s1) {
        dre[s * TPT] = xr[s];
        dre[np + s * TPT] = xi[s];
      }
    return;
  }
#pragma unroll
  for (int s = 0; s < E; ++s) {
    fre[s * TPT] = xr[s];
    fim[s * TPT] = xi[s];
  }
  if constexpr (INV && !DF) {
    if (band.split) {
      // The next MFT's operand parts, straight from the registers. Lane pairs
      // (u, u ^ 1) swap one value per two slots so that each lane holds two
      // adjacent columns of one slot (the even lane of slot s, the odd lane
      // of slot s + 1) and stores every part as one bf16x2 word. TPT is even
      // and a warp holds whole rows, so the pair is in the same row.
      const int odd = u & 1;
      const size_t plane2 = plane / 2;
      uint32_t* sp = reinterpret_cast<uint32_t*>(band.split) +
                     ((size_t)f * 6 * plane + (size_t)row * N + (u - odd)) / 2;
#pragma unroll
      for (int s = 0; s < E; s += 2) {
        const float rr = __shfl_xor_sync(0xffffffffu, odd ? xr[s] : xr[s + 1], 1);
        const float ri = __shfl_xor_sync(0xffffffffu, odd ? xi[s] : xi[s + 1], 1);
        const float ar = odd ? rr : xr[s], br = odd ? xr[s + 1] : rr;  // columns c, c + 1
        const float ai = odd ? ri : xi[s], bi = odd ? xi[s + 1] : ri;
        uint32_t hr[3], hi[3];
        split3_pair(ar, br, hr[0], hr[1], hr[2]);
        split3_pair(ai, bi, hi[0], hi[1], hi[2]);
        const size_t w = (size_t)(odd ? s + 1 : s) * (TPT / 2);
#pragma unroll
        for (int p = 0; p < 3; ++p) {
          sp[(size_t)(2 * p) * plane2 + w] = hr[p];
          sp[(size_t)(2 * p + 1) * plane2 + w] = hi[p];
        }
      }
    }
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

// The transfer function of the two-float Fresnel (CSG_PREC_HIGH), evaluated
// in FP64: turns = t0 - (z / lambda) eps / (1 + sqrt(1 - eps)) with
// t0 = z / lambda reduced first, so the phase is exact to ~1e-13 turns;
// stored as (cos hi, cos lo, sin hi, sin lo).
__global__ void k_fresnel_table_df(int N, const double* lam, double z, double ap_rad,
                                   float4* __restrict__ out) {
  const int s = blockIdx.y;
  const double zl = z / lam[s];
  const double t0 = zl - rint(zl);
  const double ce = 0.25 * (lam[s] / ap_rad) * (lam[s] / ap_rad);
  const int plane = N * N;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += gridDim.x * blockDim.x) {
    const int r = i / N, c = i % N;
    const int fr = r < N / 2 ? r : r - N;
    const int fc = c < N / 2 ? c : c - N;
    const double eps = ce * (double)(fr * fr + fc * fc);
    double t = t0 - zl * eps / (1.0 + sqrt(1.0 - eps));
    t -= rint(t);
    double sn, cs;
    sincospi(2.0 * t, &sn, &cs);
    const float2 a = split_f64(cs), b = split_f64(sn);
    out[(size_t)s * plane + i] = make_float4(a.x, a.y, b.x, b.y);
  }
}

int build_fresnel_table(cudaStream_t st, int N, const double* lam, int n_slot, double z,
                        double ap_rad, float2* out) {
  dim3 grid(grid_for((long long)N * N, 256, 1024), n_slot);
  k_fresnel_table<<<grid, 256, 0, st>>>(N, lam, z, ap_rad, out);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

int build_fresnel_table_df(cudaStream_t st, int N, const double* lam, int n_slot, double z,
                           double ap_rad, float4* out) {
  dim3 grid(grid_for((long long)N * N, 256, 1024), n_slot);
  k_fresnel_table_df<<<grid, 256, 0, st>>>(N, lam, z, ap_rad, out);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

// A two-float table from an fp32 one (masks used as transfer functions).
__global__ void k_table_to_df(const float2* __restrict__ in, float4* __restrict__ out,
                              long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float2 v = in[i];
    out[i] = make_float4(v.x, 0.f, v.y, 0.f);
  }
}
int table_to_df(cudaStream_t st, const float2* in, float4* out, long long n) {
  k_table_to_df<<<grid_for(n, 256, 1024), 256, 0, st>>>(in, out, n);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

// Column pass; MODE 0: forward, 1: inverse, 2: forward * H(lambda_f) * inverse.
// Thread (t, u) = (threadIdx % COLS, threadIdx / COLS) owns rows u + s N/16
// of column c0 + t: a warp's load or store covers 32/COLS rows x COLS
// consecutive floats. In MODE 2 the forward transform leaves each thread
// holding exactly the elements the inverse transform's first stage needs,
// so H is applied in registers and the inverse starts without a
// shared-memory exchange. Two-float passes read the two-float table H4.
template <int N, int E, int MODE, int COLS, class T>
__global__ void __launch_bounds__(ColCfg<N, E, COLS, T>::THREADS,
                                  ColCfg<N, E, COLS, T>::MIN_BLOCKS)
    k_fft_cols(float* __restrict__ field, const typename TwOf<T>::type* __restrict__ tw,
               const __grid_constant__ FresnelArgs fa, int band_lo, int band_n, int store_all) {
  using CF = ColCfg<N, E, COLS, T>;
  using A = ColAddr<COLS, E>;
  constexpr int LO = 2 * CF::PLANE;
  constexpr bool DF = std::is_same<T, dfl>::value;
  constexpr int TPT = CF::TPT;
  extern __shared__ float sm[];
  float* re = sm;
  float* im = sm + CF::PLANE;
  constexpr int CPF = N / COLS;
  const int f = blockIdx.x / CPF;
  const int c0 = (blockIdx.x % CPF) * COLS;
  const int t = threadIdx.x % COLS, u = threadIdx.x / COLS;
  const size_t plane = (size_t)N * N;
  float* fre = field + (size_t)f * 2 * plane + (size_t)u * N + c0 + t;
  float* fim = fre + plane;
  T xr[E], xi[E];
  // band: rows u + s N/E outside [band_lo, band_lo + band_n) are zero on
  // input and, unless store_all, not stored (band_n = 0: every row)
  const int s0 = band_n ? band_lo / TPT : 0, s1 = band_n ? (band_lo + band_n) / TPT : E;
  const int w0 = store_all ? 0 : s0, w1 = store_all ? E : s1;
#pragma unroll
  for (int s = 0; s < E; ++s) {
    const bool in = s >= s0 && s < s1;
    const float a = in ? fre[(size_t)s * TPT * N] : 0.f;
    const float b = in ? fim[(size_t)s * TPT * N] : 0.f;
    if constexpr (DF) {
      xr[s] = df_from(a);
      xi[s] = df_from(b);
    } else {
      xr[s] = a;
      xi[s] = b;
    }
  }
  fft_regs<N, E, MODE == 1, A, LO>(xr, xi, re, im, t, u, tw);
  if (MODE == 2) {
    if constexpr (DF) {
      const float4* Hs = fa.H4 + (size_t)fa.slot[f] * plane + (size_t)u * N + c0 + t;
#pragma unroll
      for (int h = 0; h < E; h += 4) {
        float4 w[4];
#pragma unroll
        for (int s = 0; s < 4; ++s) w[s] = __ldg(&Hs[(size_t)(h + s) * TPT * N]);
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          dfl orr, oi;
          df_cmul(xr[h + s], xi[h + s], dfl{w[s].x, w[s].y}, dfl{w[s].z, w[s].w}, orr, oi);
          xr[h + s] = orr;
          xi[h + s] = oi;
        }
      }
    } else if (fa.H) {  // per-wavelength table (L2-resident, shared by the batch)
      const float2* Hs = fa.H + (size_t)fa.slot[f] * plane + (size_t)u * N + c0 + t;
#pragma unroll
      for (int h = 0; h < E; h += 8) {  // in groups of 8 (bounds the live table values)
        float2 w[8];
#pragma unroll
        for (int s = 0; s < 8; ++s) w[s] = __ldg(&Hs[(size_t)(h + s) * TPT * N]);
#pragma unroll
        for (int s = 0; s < 8; ++s) {
          const float a = xr[h + s];
          xr[h + s] = a * w[s].x - xi[h + s] * w[s].y;
          xi[h + s] = a * w[s].y + xi[h + s] * w[s].x;
        }
      }
    } else {
      __shared__ FresnelConsts shc;
      if (threadIdx.x == 0) shc = fresnel_consts(fa.lambda[f], fa.z, fa.ap_rad);
      __syncthreads();
      const FresnelConsts fc = shc;
#pragma unroll
      for (int s = 0; s < E; ++s) {
        const float2 w = fresnel_h(N, u + s * TPT, c0 + t, fc);
        const float a = xr[s];
        xr[s] = a * w.x - xi[s] * w.y;
        xi[s] = a * w.y + xi[s] * w.x;
      }
    }
    __syncthreads();  // the forward transform's last reads precede the inverse's writes
    // the inverse's indices pass through an opaque copy, so its address
    // arithmetic is not computed ahead (and held) across the forward
    // transform and the product
    int t2 = t, u2 = u;
    asm volatile("" : "+r"(t2), "+r"(u2));
    fft_regs<N, E, true, A, LO>(xr, xi, re, im, t2, u2, tw);
  }
#pragma unroll
  for (int s = 0; s < E; ++s)
    if (s >= w0 && s < w1) {
      if constexpr (DF) {
        fre[(size_t)s * TPT * N] = df_round(xr[s]);
        fim[(size_t)s * TPT * N] = df_round(xi[s]);
      } else {
        fre[(size_t)s * TPT * N] = xr[s];
        fim[(size_t)s * TPT * N] = xi[s];
      }
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

template <int N, int E, int COLS, class T>
static int launch_cols(cudaStream_t st, float* field, int F, int mode,
                       const typename TwOf<T>::type* tw, const FresnelArgs* fa,
                       const FftBand& band, int store_all) {
  using CC = ColCfg<N, E, COLS, T>;
  const int grid = F * (N / COLS);
  int rc;
  if (mode == 2) {
    if ((rc = prep_smem(k_fft_cols<N, E, 2, COLS, T>, CC::SMEM))) return rc;
    k_fft_cols<N, E, 2, COLS, T><<<grid, CC::THREADS, CC::SMEM, st>>>(field, tw, *fa, band.lo,
                                                                      band.n, store_all);
  } else if (mode == 1) {
    if ((rc = prep_smem(k_fft_cols<N, E, 1, COLS, T>, CC::SMEM))) return rc;
    k_fft_cols<N, E, 1, COLS, T><<<grid, CC::THREADS, CC::SMEM, st>>>(field, tw, FresnelArgs{},
                                                                      0, 0, 0);
  } else {
    if ((rc = prep_smem(k_fft_cols<N, E, 0, COLS, T>, CC::SMEM))) return rc;
    k_fft_cols<N, E, 0, COLS, T><<<grid, CC::THREADS, CC::SMEM, st>>>(field, tw, FresnelArgs{},
                                                                      0, 0, 0);
  }
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

template <int N, int E, class T>
static int launch_rows(cudaStream_t st, float* field, int F, bool inv, float scale,
                       const typename TwOf<T>::type* tw, const PixOps& p, const PixOps& e,
                       const FieldInfo& fi, const FftBand& band) {
  using RC = RowCfg<N, E, T>;
  const int grid = F * ((band.n ? band.n : N) / RC::ROWS);
  int rc;
  if (inv) {
    if ((rc = prep_smem(k_fft_rows<N, E, true, T>, RC::SMEM))) return rc;
    k_fft_rows<N, E, true, T><<<grid, RC::THREADS, RC::SMEM, st>>>(field, scale, tw, p, e, fi,
                                                                   band);
  } else {
    if ((rc = prep_smem(k_fft_rows<N, E, false, T>, RC::SMEM))) return rc;
    k_fft_rows<N, E, false, T><<<grid, RC::THREADS, RC::SMEM, st>>>(field, scale, tw, p, e, fi,
                                                                    band);
  }
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

// Tuning overrides for N = 1024: CSG_FFT_COLS (4, 8 or 16 columns per
// column-pass CTA) and CSG_FFT_E (16 elements per thread instead of 32).
static int env_choice(const char* name, std::initializer_list<int> allowed) {
  const char* s = getenv(name);
  const int c = s ? atoi(s) : 0;
  for (int a : allowed)
    if (c == a) return c;
  return 0;
}

template <int N, class T>
static int run_fft(csg_ctx* ctx, float* field, int F, int direction, const FresnelArgs* fa,
                   const PixOps& pro, const PixOps& epi, const FieldInfo& fi,
                   const typename TwOf<T>::type* tw, const FftBand& band, const FftBand& sup,
                   __nv_bfloat16* split_out) {
  constexpr bool DF = std::is_same<T, dfl>::value;
  cudaStream_t st = ctx->stream;
  const float inv_scale = 1.f / ((float)N * (float)N);
  // a band-limited pass moves n rows of N (the first and last touch n x n)
  const double pass_bytes = (double)F * N * (band.n ? band.n : N) * 16.0;
  const double edge_bytes = band.n ? (double)F * band.n * (N + band.n) * 8.0 : pass_bytes;
  const PixOps none;
  const bool e16 =
      !DF && (N == 1024) && !band.n && !sup.n && env_choice("CSG_FFT_E", {16}) == 16;
  const int c_over = DF ? 0 : env_choice("CSG_FFT_COLS", {4, 16});
  int rc;
  auto rows = [&](bool inv, float scale, const PixOps& p, const PixOps& e,
                  const FftBand& bd) -> int {
    const bool gen = p.n && p.kind[0] == OP_SOURCE;
    const double bytes = (bd.n && !bd.src && !bd.dst ? (double)F * N * bd.n * 16.0 : edge_bytes) *
                             (gen ? 0.5 : 1.0) +
                         (bd.split ? (double)F * N * N * 12.0 : 0.0);
    ProfScope ps(ctx, inv ? "fft_rows_inv" : "fft_rows_fwd", 0, bytes);
    if constexpr (N == 1024 && !DF)
      if (e16) return launch_rows<N, 16, T>(st, field, F, inv, scale, tw, p, e, fi, bd);
    return launch_rows<N, elems_for<T>(N), T>(st, field, F, inv, scale, tw, p, e, fi, bd);
  };
  auto cols = [&](int mode, const FftBand& bd, int store_all) -> int {
    const double bytes = store_all ? (double)F * N * (N + bd.n) * 8.0 : pass_bytes;
    ProfScope ps(ctx, mode == 2 ? "fft_cols_fresnel" : "fft_cols", 0, bytes);
    if constexpr (N == 1024 && !DF) {
      if (e16) return launch_cols<N, 16, 8, T>(st, field, F, mode, tw, fa, bd, store_all);
      if (c_over == 4) return launch_cols<N, 32, 4, T>(st, field, F, mode, tw, fa, bd, store_all);
      if (c_over == 16)
        return launch_cols<N, 32, 16, T>(st, field, F, mode, tw, fa, bd, store_all);
    }
    return launch_cols<N, elems_for<T>(N), cols_for<T>(N), T>(st, field, F, mode, tw, fa, bd,
                                                               store_all);
  };
  FftBand whole, last = band;
  whole.split = last.split = split_out;  // the last pass also writes the split
  if (fa && sup.n) {
    // rows outside the prologue's support are zero: the first row pass
    // skips them (leaving them unwritten) and the column pass reads only
    // the support's rows and writes every row
    if ((rc = rows(false, 1.f, pro, none, sup))) return rc;
    if ((rc = cols(2, sup, 1))) return rc;
    return rows(true, inv_scale, none, epi, whole);
  } else if (fa) {
    if ((rc = rows(false, 1.f, pro, none, band))) return rc;
    if ((rc = cols(2, band, 0))) return rc;
    return rows(true, inv_scale, none, epi, last);
  } else if (direction < 0) {
    if ((rc = rows(false, 1.f, pro, none, band))) return rc;
    if ((rc = cols(0, band, 0))) return rc;
    if (epi.n) return pixops_pass(st, field, F, N, N, epi, fi);
  } else {
    if (pro.n && (rc = pixops_pass(st, field, F, N, N, pro, fi))) return rc;
    if ((rc = cols(1, band, 0))) return rc;
    return rows(true, inv_scale, none, epi, band);
  }
  return CSG_OK;
}

// Threads per transform of the row and column passes (fp32 or two-float).
static int fft_tpt(int N, bool high) { return N / (high ? 16 : default_e(N)); }

bool fft_band_supported(int N, int lo, int n, bool high) {
  const int TPT = fft_tpt(N, high), rows = 256 / TPT > 0 ? 256 / TPT : 1;
  return n > 0 && lo >= 0 && lo + n <= N && lo % TPT == 0 && n % TPT == 0 && n % rows == 0;
}

bool fft_row_support(int N, int r0, int r1, int* lo, int* n, bool high) {
  const int TPT = fft_tpt(N, high);
  if (r0 < 0 || r1 > N || r0 >= r1) return false;
  *lo = r0 / TPT * TPT;
  *n = (r1 + TPT - 1) / TPT * TPT - *lo;
  return fft_band_supported(N, *lo, *n, high);
}

template <class T>
static int run_fft_n(csg_ctx* ctx, float* field, int F, int n, int direction,
                     const FresnelArgs* fa, const PixOps& pro, const PixOps& epi,
                     const FieldInfo& fi, const typename TwOf<T>::type* tw, const FftBand& bd,
                     const FftBand& sp, __nv_bfloat16* so) {
  switch (n) {
    case 64: return run_fft<64, T>(ctx, field, F, direction, fa, pro, epi, fi, tw, bd, sp, so);
    case 128: return run_fft<128, T>(ctx, field, F, direction, fa, pro, epi, fi, tw, bd, sp, so);
    case 256: return run_fft<256, T>(ctx, field, F, direction, fa, pro, epi, fi, tw, bd, sp, so);
    case 512: return run_fft<512, T>(ctx, field, F, direction, fa, pro, epi, fi, tw, bd, sp, so);
    case 1024:
      return run_fft<1024, T>(ctx, field, F, direction, fa, pro, epi, fi, tw, bd, sp, so);
    case 2048:
      return run_fft<2048, T>(ctx, field, F, direction, fa, pro, epi, fi, tw, bd, sp, so);
    default:
      return run_fft<4096, T>(ctx, field, F, direction, fa, pro, epi, fi, tw, bd, sp, so);
  }
}

// ------------------------------------ sizes that are not powers of two
// The reference plans FFTW for any size (csim_fft.cpp:111-115). Sizes the
// register FFT does not cover (multiples of 8 that are not powers of two, up
// to 8192) run the 2-D DFT as a matrix Fourier transform on the tensor cores:
// X[k1][k2] = sum x[n1][n2] exp(-+2 pi i (n1 k1 + n2 k2) / N), i.e. integer
// coordinates and lambda f = N, so every operator phase is exact in FP64;
// the inverse carries the 1 / N^2. A Fresnel propagation multiplies the
// spectrum by the transfer function between the two (in FFT order, the
// table of its wavelength slot or evaluated in place). O(N^3) work instead
// of O(N^2 log N), on the tensor cores.
static int dft_plan(csg_ctx* ctx, int n, int sgn, int precision, csg_mft** out) {
  const auto key = std::make_tuple(n, sgn, precision);
  auto it = ctx->dft_plans.find(key);
  if (it != ctx->dft_plans.end()) {
    *out = it->second;
    return CSG_OK;
  }
  std::vector<double> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = (double)i;
  const double lf = (double)n;
  const double pref[2] = {sgn > 0 ? 1.0 / ((double)n * (double)n) : 1.0, 0.0};
  csg_mft* m = nullptr;
  const int rc = csg_mft_create(ctx, &m, n, n, n, n, idx.data(), idx.data(), idx.data(),
                                idx.data(), 1, &lf, pref, (double)sgn, precision);
  if (rc) return rc;
  ctx->dft_plans[key] = m;
  *out = m;
  return CSG_OK;
}

// The DFT-product Fresnel factors the transfer function as H = c H' with
// c = exp(2 pi i z / lambda) (H at zero frequency) and propagates
//   E' = c (E + IDFT[DFT(E) (H' - 1)]):
// H' - 1 vanishes at zero frequency and stays small where the spectrum of a
// smooth field is concentrated, so the inverse transform's input has a far
// smaller dynamic range than DFT(E) H (whose zero-frequency term dominates
// every 64-element group it sits in and sets the rounding of the rest).

// c of each field, FP64-evaluated (cos, sin; two-float as (hi, lo) pairs).
__device__ __forceinline__ void fresnel_unit(double lam, double z, dfl& cr, dfl& ci) {
  const double zl = z / lam;
  double sn, cs;
  sincospi(2.0 * (zl - rint(zl)), &sn, &cs);
  const float2 a = split_f64(cs), b = split_f64(sn);
  cr = dfl{a.x, a.y};
  ci = dfl{b.x, b.y};
}

// The spectrum times H' - 1 of each field's wavelength (FFT order), from
// the table (H conj(c) - 1) or evaluated here (exp(2 pi i tau) - 1 with
// tau the phase past z / lambda: (-2 sin^2(pi tau), sin(2 pi tau))).
__global__ void k_fresnel_mul(float* __restrict__ spec, int N, const __grid_constant__ FresnelArgs fa) {
  const int f = blockIdx.y;
  const size_t plane = (size_t)N * N;
  float* re = spec + (size_t)f * 2 * plane;
  float* im = re + plane;
  __shared__ FresnelConsts shc;
  __shared__ float2 shu;
  if (threadIdx.x == 0) {
    shc = fresnel_consts(fa.lambda[f], fa.z, fa.ap_rad);
    shc.t0 = 0.f;  // the in-place evaluation gives H' itself
    dfl cr, ci;
    fresnel_unit(fa.lambda[f], fa.z, cr, ci);
    shu = make_float2(cr.h, ci.h);
  }
  __syncthreads();
  const float2 u = shu;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < plane;
       i += (size_t)gridDim.x * blockDim.x) {
    float2 w;  // H' - 1
    if (fa.H4 || fa.H) {
      float2 h;
      if (fa.H4) {
        const float4 q = fa.H4[(size_t)fa.slot[f] * plane + i];
        h = make_float2(q.x + q.y, q.z + q.w);
      } else {
        h = fa.H[(size_t)fa.slot[f] * plane + i];
      }
      w = make_float2(fmaf(h.x, u.x, fmaf(h.y, u.y, -1.f)), fmaf(h.y, u.x, -h.x * u.y));
    } else {
      const int r = (int)(i / N), c = (int)(i % N);
      const int fr = r < N / 2 ? r : r - N;
      const int fc = c < N / 2 ? c : c - N;
      const float f2 = (float)(fr * fr + fc * fc);
      const float eps = shc.c_eps * f2;
      const float sq = sqrtf(1.f - eps);
      const float hh = eps / (2.f * (1.f + sq) * (1.f + sq));
      float tt = -frac_prod(f2, shc.khi, shc.klo) - shc.K * f2 * hh;
      tt -= rintf(tt);
      float s1, c1, s2, c2;
      sincospif(tt, &s1, &c1);
      sincospif(2.f * tt, &s2, &c2);
      w = make_float2(-2.f * s1 * s1, s2);
    }
    const float a = re[i], b = im[i];
    re[i] = a * w.x - b * w.y;
    im[i] = a * w.y + b * w.x;
  }
}

// Each field times its c (the last step of E' = c (E + ...)).
__global__ void k_fresnel_unit(float* __restrict__ field, int N, const double* __restrict__ lambda,
                               double z) {
  const int f = blockIdx.y;
  const size_t plane = (size_t)N * N;
  float* re = field + (size_t)f * 2 * plane;
  float* im = re + plane;
  __shared__ float2 shu;
  if (threadIdx.x == 0) {
    dfl cr, ci;
    fresnel_unit(lambda[f], z, cr, ci);
    shu = make_float2(cr.h, ci.h);
  }
  __syncthreads();
  const float2 u = shu;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < plane;
       i += (size_t)gridDim.x * blockDim.x) {
    const float a = re[i], b = im[i];
    re[i] = a * u.x - b * u.y;
    im[i] = a * u.y + b * u.x;
  }
}

// Plans, spectrum scratch and the all-zero slot vector of F fields of size n
// (allocates: called before any capture; the chain calls it when planning).
int dft_prepare(csg_ctx* ctx, int n, int F, bool high) {
  CSG_CHECK(n % 8 == 0 && n <= 8192, CSG_E_SHAPE,
            "FFT: sizes that are not powers of two must be multiples of 8, at most 8192");
  const int prec = high ? CSG_PREC_HIGH : CSG_PREC_BF16X6;
  csg_mft* m = nullptr;
  int rc = dft_plan(ctx, n, -1, prec, &m);
  if (!rc) rc = dft_plan(ctx, n, +1, prec, &m);
  if (rc) return rc;
  const size_t bytes = (size_t)F * 2 * n * n * sizeof(float);
  if (ctx->dft_scratch_bytes < bytes) {
    if (ctx->dft_scratch) cudaFree(ctx->dft_scratch);
    ctx->dft_scratch = nullptr;
    ctx->dft_scratch_bytes = 0;
    CSG_CUDA(cudaMalloc(&ctx->dft_scratch, bytes));
    ctx->dft_scratch_bytes = bytes;
  }
  if (ctx->dft_zero_n < F) {
    if (ctx->dft_zero) cudaFree(ctx->dft_zero);
    ctx->dft_zero = nullptr;
    ctx->dft_zero_n = 0;
    CSG_CUDA(cudaMalloc((void**)&ctx->dft_zero, sizeof(int) * F));
    CSG_CUDA(cudaMemset(ctx->dft_zero, 0, sizeof(int) * F));
    ctx->dft_zero_n = F;
  }
  for (int i = 0; i < F; i += 65535) {  // the split kernels' grid.y bound
    csg_mft* p = nullptr;
    dft_plan(ctx, n, -1, prec, &p);
    if ((rc = csg_mft_reserve(p, std::min(F - i, 65535)))) return rc;
    dft_plan(ctx, n, +1, prec, &p);
    if ((rc = csg_mft_reserve(p, std::min(F - i, 65535)))) return rc;
  }
  return CSG_OK;
}

static int dft2d_mft(csg_ctx* ctx, float* field, int F, int n, int direction,
                     const FresnelArgs* fa, const PixOps& pro, const PixOps& epi,
                     const FieldInfo& fi, bool high) {
  cudaStream_t st = ctx->stream;
  const int prec = high ? CSG_PREC_HIGH : CSG_PREC_BF16X6;
  const size_t bytes = (size_t)F * 2 * n * n * sizeof(float);
  auto fit = ctx->dft_plans.find(std::make_tuple(n, -1, prec));
  auto iit = ctx->dft_plans.find(std::make_tuple(n, +1, prec));
  CSG_CHECK(fit != ctx->dft_plans.end() && iit != ctx->dft_plans.end() &&
                ctx->dft_scratch_bytes >= bytes && ctx->dft_zero_n >= F,
            CSG_E_STATE, "FFT: the DFT of this size was not prepared (dft_prepare)");
  int rc = CSG_OK;
  if (pro.n && (rc = pixops_pass(st, field, F, n, n, pro, fi))) return rc;
  float* tmp = static_cast<float*>(ctx->dft_scratch);
  const int* zero = ctx->dft_zero;  // every field on operator slot 0
  csg_mft *fwd = fit->second, *inv = iit->second;
  {
    if (fa) {
      // E' = c (E + IDFT[DFT(E) (H' - 1)]): the inverse accumulates into the
      // field, which still holds E
      const dim3 grid(grid_for((long long)n * n, 256, 512), F);
      rc = mft_execute_ops(ctx, fwd, field, tmp, F, zero, 0, nullptr, nullptr, PixOps(), fi);
      if (!rc) {
        k_fresnel_mul<<<grid, 256, 0, st>>>(tmp, n, *fa);
        CSG_LAUNCH_CHECK();
      }
      if (!rc)
        rc = mft_execute_ops(ctx, inv, tmp, field, F, zero, 1, nullptr, nullptr, PixOps(), fi);
      if (!rc) {
        k_fresnel_unit<<<grid, 256, 0, st>>>(field, n, fa->lambda, fa->z);
        CSG_LAUNCH_CHECK();
      }
    } else {
      rc = mft_execute_ops(ctx, direction < 0 ? fwd : inv, field, tmp, F, zero, 0, nullptr,
                           nullptr, PixOps(), fi);
      if (!rc && cudaMemcpyAsync(field, tmp, bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
        set_error("FFT: copy failed");
        rc = CSG_E_CUDA;
      }
    }
  }
  if (!rc && epi.n) rc = pixops_pass(st, field, F, n, n, epi, fi);
  return rc;
}

bool fft_is_dft_size(int n) { return n >= 8 && (n & (n - 1)) != 0; }

// 2-D FFT or Fresnel propagation of F square N x N fields with fused element
// ops (pro before the transform, epi after it); high: two-float arithmetic.
int fft2d_fused(csg_ctx* ctx, float* field, int F, int n, int direction, const FresnelArgs* fa,
                const PixOps& pro, const PixOps& epi, const FieldInfo& fi, const FftBand* band,
                const FftBand* support, __nv_bfloat16* split_out, bool high) {
  CSG_CHECK(F > 0 && (long long)F * n < (1LL << 31), CSG_E_SHAPE, "FFT: bad field count");
  if (fft_is_dft_size(n)) {
    CSG_CHECK(!band && !support && !split_out, CSG_E_ARG,
              "FFT: band, support and split outputs need a power-of-two size");
    return dft2d_mft(ctx, field, F, n, direction, fa, pro, epi, fi, high);
  }
  CSG_CHECK(n >= 64 && n <= 4096, CSG_E_SHAPE,
            "FFT: power-of-two sizes must be in [64, 4096]");
  FftBand bd, sp;
  if (band) {
    CSG_CHECK(fa && !pro.n && !epi.n && band->src && band->dst && !band->split && !support &&
                  fft_band_supported(n, band->lo, band->n, high),
              CSG_E_ARG, "FFT: unsupported band-limited transform");
    bd = *band;
  }
  CSG_CHECK(!split_out || (fa && !band && !high), CSG_E_ARG,
            "FFT: the split output needs an fp32 Fresnel pass over the whole field");
  CSG_CHECK(!high || !fa || fa->H4, CSG_E_ARG,
            "FFT: a two-float Fresnel pass needs the two-float transfer-function table");
  if (support) {
    CSG_CHECK(fa && !support->src && !support->dst && !support->split &&
                  fft_band_supported(n, support->lo, support->n, high),
              CSG_E_ARG, "FFT: unsupported row support");
    sp = *support;
  }
  cudaStream_t st = ctx->stream;
  const double pass_bytes = (double)F * n * n * 16.0;
  const bool gen = pro.n && pro.kind[0] == OP_SOURCE;  // the first pass only writes
  double total = pass_bytes * ((fa ? 3.0 : 2.0) - (gen ? 0.5 : 0.0));
  if (band)
    total = (double)F * band->n * (n + band->n) * 16.0 + (double)F * n * band->n * 16.0;
  else if (support)
    total = (double)F * n * support->n * 16.0 * (gen ? 0.5 : 1.0) +
            (double)F * n * (n + support->n) * 8.0 + pass_bytes;
  if (split_out) total += (double)F * n * n * 12.0;
  ProfScope ps(ctx, fa ? (high ? "fresnel_3pass_df" : "fresnel_3pass") : "fft2d_2pass", 0, total);
  if (high) {
    const float4* tw = twiddles_df(ctx->device, n, st);
    CSG_CHECK(tw != nullptr, CSG_E_NOMEM, "twiddle table allocation failed");
    return run_fft_n<dfl>(ctx, field, F, n, direction, fa, pro, epi, fi, tw, bd, sp, nullptr);
  }
  const float2* tw = twiddles(ctx->device, n, st);
  CSG_CHECK(tw != nullptr, CSG_E_NOMEM, "twiddle table allocation failed");
  return run_fft_n<float>(ctx, field, F, n, direction, fa, pro, epi, fi, tw, bd, sp, split_out);
}

}  // namespace csg

using namespace csg;

extern "C" {

int csg_fft2d(csg_ctx* ctx, float* field, int n_fields, int n, int direction) {
  CSG_CHECK(ctx && field, CSG_E_ARG, "csg_fft2d: null argument");
  CSG_CHECK(direction == -1 || direction == 1, CSG_E_ARG, "csg_fft2d: direction must be -1 or +1");
  DeviceGuard g(ctx->device);
  if (fft_is_dft_size(n)) {
    const int rc = dft_prepare(ctx, n, n_fields, false);
    if (rc) return rc;
  }
  return fft2d_fused(ctx, field, n_fields, n, direction, nullptr, PixOps(), PixOps(), FieldInfo());
}

int csg_fft2d_prec(csg_ctx* ctx, float* field, int n_fields, int n, int direction,
                   int precision) {
  CSG_CHECK(precision == CSG_PREC_BF16X6 || precision == CSG_PREC_BF16X3 ||
                precision == CSG_PREC_HIGH,
            CSG_E_ARG, "csg_fft2d_prec: bad precision");
  CSG_CHECK(ctx && field, CSG_E_ARG, "csg_fft2d_prec: null argument");
  CSG_CHECK(direction == -1 || direction == 1, CSG_E_ARG,
            "csg_fft2d_prec: direction must be -1 or +1");
  DeviceGuard g(ctx->device);
  if (fft_is_dft_size(n)) {
    const int rc = dft_prepare(ctx, n, n_fields, precision == CSG_PREC_HIGH);
    if (rc) return rc;
  }
  return fft2d_fused(ctx, field, n_fields, n, direction, nullptr, PixOps(), PixOps(), FieldInfo(),
                     nullptr, nullptr, nullptr, precision == CSG_PREC_HIGH);
}

int csg_fresnel(csg_ctx* ctx, float* field, int n_fields, int n, const double* lambda,
                double ap_rad, double z) {
  CSG_CHECK(ctx && field && lambda, CSG_E_ARG, "csg_fresnel: null argument");
  CSG_CHECK(all_finite(&z, 1) && all_finite(&ap_rad, 1), CSG_E_NAN,
            "csg_fresnel: non-finite distance or aperture radius");
  CSG_CHECK(ap_rad > 0, CSG_E_ARG, "csg_fresnel: apRad must be positive");
  DeviceGuard g(ctx->device);
  if (fft_is_dft_size(n)) {
    const int rc = dft_prepare(ctx, n, n_fields, false);
    if (rc) return rc;
  }
  FresnelArgs fa{lambda, z, ap_rad};
  return fft2d_fused(ctx, field, n_fields, n, -1, &fa, PixOps(), PixOps(), FieldInfo());
}

int csg_fresnel_prec(csg_ctx* ctx, float* field, int n_fields, int n, const double* lambda,
                     double ap_rad, double z, int precision) {
  CSG_CHECK(precision == CSG_PREC_BF16X6 || precision == CSG_PREC_BF16X3 ||
                precision == CSG_PREC_HIGH,
            CSG_E_ARG, "csg_fresnel_prec: bad precision");
  if (precision != CSG_PREC_HIGH) return csg_fresnel(ctx, field, n_fields, n, lambda, ap_rad, z);
  CSG_CHECK(ctx && field && lambda, CSG_E_ARG, "csg_fresnel_prec: null argument");
  CSG_CHECK(all_finite(&z, 1) && all_finite(&ap_rad, 1), CSG_E_NAN,
            "csg_fresnel_prec: non-finite distance or aperture radius");
  CSG_CHECK(ap_rad > 0, CSG_E_ARG, "csg_fresnel_prec: apRad must be positive");
  CSG_CHECK(n_fields > 0, CSG_E_SHAPE, "csg_fresnel_prec: n_fields must be positive");
  DeviceGuard g(ctx->device);
  if (fft_is_dft_size(n)) {
    const int rc = dft_prepare(ctx, n, n_fields, true);
    if (rc) return rc;
  } else {
    CSG_CHECK(n >= 64 && n <= 4096, CSG_E_SHAPE, "FFT: power-of-two sizes must be in [64, 4096]");
  }
  cudaStream_t st = ctx->stream;
  // one two-float transfer function per field (its own wavelength), built in
  // FP64 for this call: the fields' slot is their own index
  const size_t plane = (size_t)n * n;
  float4* H4 = nullptr;
  int* slot = nullptr;
  if (cudaMallocAsync(&H4, plane * n_fields * sizeof(float4), st) != cudaSuccess ||
      cudaMallocAsync(&slot, n_fields * sizeof(int), st) != cudaSuccess) {
    cudaGetLastError();
    if (H4) cudaFreeAsync(H4, st);
    set_error("csg_fresnel_prec: allocation failed");
    return CSG_E_NOMEM;
  }
  std::vector<int> idx(n_fields);
  for (int i = 0; i < n_fields; ++i) idx[i] = i;
  int rc = CSG_OK;
  if (cudaMemcpyAsync(slot, idx.data(), n_fields * sizeof(int), cudaMemcpyHostToDevice, st) !=
      cudaSuccess) {
    set_error("csg_fresnel_prec: copy failed");
    rc = CSG_E_CUDA;
  }
  if (!rc) rc = build_fresnel_table_df(st, n, lambda, n_fields, z, ap_rad, H4);
  if (!rc) {
    FresnelArgs fa{lambda, z, ap_rad, nullptr, slot, H4};
    rc = fft2d_fused(ctx, field, n_fields, n, -1, &fa, PixOps(), PixOps(), FieldInfo(), nullptr,
                     nullptr, nullptr, true);
  }
  cudaStreamSynchronize(st);  // the host index vector and the tables
  cudaFreeAsync(H4, st);
  cudaFreeAsync(slot, st);
  return rc;
}

}  // extern "C"
