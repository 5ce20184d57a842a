// Surrogate MLP for hex-FPM sag vectors (no reference counterpart): a
// fully connected network n_in -> hidden... -> 1 with exact-erf GELU,
// bf16 weights and activations, fp32 accumulation, fp32 master weights and
// Adam. Every matrix product is one tcgen05 GEMM kernel (k_mlp_gemm) with
// both operands K-major (A [M][K], B [N][K], C = A B^T) and a fused epilogue:
//   forward   Z = H W^T + b, H' = gelu(Z)        (bf16 H' and H'^T stored)
//   backward  dW = dZ^T H   (A = dZ^T, B = H^T)   fp32
//             dH = dZ W     (A = dZ,  B = W^T)   times gelu'(Z) -> dZ (bf16, and dZ^T)
// The one-output last layer, the loss, bias gradients and Adam are small
// CUDA-core kernels. Accumulation is a single fp32 chain in tensor memory
// (training tolerates the truncation the MFT cannot).
#include <cmath>
#include <random>
#include <vector>

#include "ctx.hpp"
#include "tc_gemm.cuh"

namespace csg {
int make_map(CUtensorMap* m, const void* base, int k, int rows, long long planes, int box_rows);

namespace mlp {

using namespace tc;
constexpr int MBN = 128;        // N tile
constexpr int MSTAGES = 4;
constexpr int EPI_WARPS = 4;
constexpr int MTHREADS = (EPI_WARPS + 2) * 32;
constexpr uint32_t MA_BYTES = BM * BK * 2, MB_BYTES = MBN * BK * 2;
constexpr size_t MSMEM = (size_t)MSTAGES * (MA_BYTES + MB_BYTES) + 1024 + 256;

struct GemmParams {
  int M, N, k_blocks;
  const float* bias;     // [N] or null
  const float* aux;      // dgelu: Z [M][N] fp32
  int act;               // 0 none, 1 gelu (store Z in out_f32), 2 times gelu'(aux)
  float* out_f32;        // [M][N] or null
  __nv_bfloat16* out_bf16;   // [M][ld_bf16] or null
  __nv_bfloat16* out_bf16t;  // [N][ld_bf16t] (transposed) or null
  int ld_bf16, ld_bf16t;
  int* status;
};

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678f)); }
__device__ __forceinline__ float gelu_d(float z) {
  return 0.5f * (1.f + erff(z * 0.70710678f)) + z * 0.39894228f * expf(-0.5f * z * z);
}

__global__ void __launch_bounds__(MTHREADS, 1)
    k_mlp_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               const GemmParams p) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  uint8_t* sbase = smem_raw + (base - smem_u32(smem_raw));
  uint8_t* sA = sbase;
  uint8_t* sB = sbase + MSTAGES * MA_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + MSTAGES * MB_BYTES);
  uint64_t* empty = full + MSTAGES;
  uint64_t* done = empty + MSTAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_tiles = (p.N + MBN - 1) / MBN;
  const int mt = blockIdx.x / n_tiles, nt = blockIdx.x % n_tiles;
  const int row0 = mt * BM, col0 = nt * MBN;
  if (threadIdx.x == 0) {
    for (int s = 0; s < MSTAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(MBN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  if (warp == EPI_WARPS) {  // producer
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      for (int kb = 0; kb < p.k_blocks; ++kb) {
        if (kb >= MSTAGES && !mbar_wait(&empty[stage], phase ^ 1)) {
          atomicExch(p.status, 11);
          *abort_flag = 1;
          break;
        }
        if (*abort_flag) break;
        mbar_expect_tx(&full[stage], MA_BYTES + MB_BYTES);
        tma_load_3d(sA + stage * MA_BYTES, &tmA, &full[stage], kb * BK, row0, 0);
        tma_load_3d(sB + stage * MB_BYTES, &tmB, &full[stage], kb * BK, col0, 0);
        if (++stage == MSTAGES) {
          stage = 0;
          phase ^= 1;
        }
      }
    }
    __syncwarp();
  } else if (warp == EPI_WARPS + 1) {  // MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = instr_desc(BM, MBN);
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true;
      for (int kb = 0; kb < p.k_blocks; ++kb) {
        ok = mbar_wait(&full[stage], phase);
        if (!ok || *abort_flag) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t a0 = smem_u32(sA + stage * MA_BYTES), b0 = smem_u32(sB + stage * MB_BYTES);
#pragma unroll
        for (int k = 0; k < BK / 16; ++k)
          umma(tmem, smem_desc(a0 + k * 32), smem_desc(b0 + k * 32), idesc,
               (kb > 0 || k > 0) ? 1u : 0u);
        umma_commit(&empty[stage]);
        if (++stage == MSTAGES) {
          stage = 0;
          phase ^= 1;
        }
      }
      if (!ok) {
        atomicExch(p.status, 12);
        *abort_flag = 1;
      }
      umma_commit(done);  // also releases the epilogue after an abort
    }
    __syncwarp();
  } else {  // epilogue: warp q owns rows q*32 .. q*32+31
    const bool ok = mbar_wait(done, 0) && !*abort_flag;
    if (!ok) {
      if (lane == 0) atomicExch(p.status, 13);
    } else {
      tc_fence_after();
      const int m = row0 + warp * 32 + lane;
      for (int cb = 0; cb < MBN; cb += 32) {
        uint32_t r[32];
        tmem_ld32_nowait(tmem + ((uint32_t)(warp * 32) << 16) + cb, r);
        tmem_wait_ld();
        if (col0 + cb >= p.N) break;
#pragma unroll 4
        for (int j = 0; j < 32; ++j) {
          const int n = col0 + cb + j;
          if (m >= p.M || n >= p.N) continue;
          float v = __uint_as_float(r[j]);
          if (p.bias) v += p.bias[n];
          float outv = v;
          if (p.act == 1) {
            outv = gelu(v);
          } else if (p.act == 2) {
            v = v * gelu_d(p.aux[(size_t)m * p.N + n]);
            outv = v;
          }
          if (p.out_f32) p.out_f32[(size_t)m * p.N + n] = v;
          if (p.out_bf16) p.out_bf16[(size_t)m * p.ld_bf16 + n] = __float2bfloat16_rn(outv);
          if (p.out_bf16t) p.out_bf16t[(size_t)n * p.ld_bf16t + m] = __float2bfloat16_rn(outv);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(MBN));
  }
}

// ------------------------------------------------------------- small kernels
// features, mode 0: x[b][i] = sags[b][i] / sag_scale (i < n_var); mode 1
// (phasor): x[b][2i], x[b][2i+1] = cos, sin(4 pi sag / lambda) (the hex
// phasor of complexHexMaskFPM.cpp:87 with phaseSign sag_scale); then
// (lam[b] - lam0) / lam_scale and zeros; bf16 [B][K] and transposed [K][B].
__global__ void k_features(const double* __restrict__ sags, int n_var, const double* __restrict__ lam,
                           double sag_scale, double lam0, double lam_scale, int B, int K,
                           int mode, __nv_bfloat16* __restrict__ x,
                           __nv_bfloat16* __restrict__ xt) {
  const long long n = (long long)B * K;
  const int nf = mode == 1 ? 2 * n_var : n_var;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(t / K), i = (int)(t % K);
    double v = 0.0;
    if (i < nf && mode == 1) {
      double turns = sag_scale * 2.0 * sags[(size_t)b * n_var + i / 2] / lam[b];
      turns -= rint(turns);
      double s, c;
      sincospi(2.0 * turns, &s, &c);
      v = (i & 1) ? s : c;
    } else if (i < nf) {
      v = sags[(size_t)b * n_var + i] / sag_scale;
    } else if (i == nf) {
      v = (lam[b] - lam0) / lam_scale;
    }
    const __nv_bfloat16 h = __float2bfloat16_rn((float)v);
    x[t] = h;
    xt[(size_t)i * B + b] = h;
  }
}

// raw fp32 input [B][n_in] -> bf16 [B][K] and [K][B] (zero padded)
__global__ void k_set_input(const float* __restrict__ in, int n_in, int B, int K,
                            __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ xt) {
  const long long n = (long long)B * K;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(t / K), i = (int)(t % K);
    const __nv_bfloat16 h = __float2bfloat16_rn(i < n_in ? in[(size_t)b * n_in + i] : 0.f);
    x[t] = h;
    xt[(size_t)i * B + b] = h;
  }
}

// y[b] = sum_i H[b][i] w[i] + b0 (one warp per row)
__global__ void k_last_forward(const __nv_bfloat16* __restrict__ H, int K, int B,
                               const float* __restrict__ w, const float* __restrict__ b0,
                               float* __restrict__ y) {
  const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
  if (row >= B) return;
  float acc = 0.f;
  for (int i = lane; i < K; i += 32)
    acc += __bfloat162float(H[(size_t)row * K + i]) * __bfloat162float(__float2bfloat16_rn(w[i]));
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) y[row] = acc + b0[0];
}

// MSE loss: dy = 2 (y - t) / B; loss = mean (y - t)^2 (one block)
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, int B,
                      float* __restrict__ dy, float* __restrict__ loss) {
  __shared__ float red[32];
  float acc = 0.f;
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    const float d = y[b] - t[b];
    dy[b] = 2.f * d / B;
    acc += d * d;
  }
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x / 32] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0.f;
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && loss) *loss = v / B;
  }
}

// last layer backward: dW[i] = sum_b dy[b] H[b][i], db = sum_b dy[b];
// dZ[b][i] = dy[b] w[i] gelu'(Z[b][i]) -> bf16 [B][K] and [K][B]
__global__ void k_last_backward(const __nv_bfloat16* __restrict__ H, const float* __restrict__ Z,
                                int K, int B, const float* __restrict__ w,
                                const float* __restrict__ dy, float* __restrict__ dw,
                                float* __restrict__ db, __nv_bfloat16* __restrict__ dz,
                                __nv_bfloat16* __restrict__ dzt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < K) {
    float acc = 0.f;
    for (int b = 0; b < B; ++b) acc += dy[b] * __bfloat162float(H[(size_t)b * K + i]);
    dw[i] = acc;
    const float wi = __bfloat162float(__float2bfloat16_rn(w[i]));
    for (int b = 0; b < B; ++b) {
      const __nv_bfloat16 h = __float2bfloat16_rn(dy[b] * wi * gelu_d(Z[(size_t)b * K + i]));
      dz[(size_t)b * K + i] = h;
      dzt[(size_t)i * B + b] = h;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    float s = 0.f;
    for (int b = 0; b < B; ++b) s += dy[b];
    db[0] = s;
  }
}

// db[o] = sum_b dZ[b][o] (from the transposed copy: rows contiguous)
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ dzt, int N, int B,
                            float* __restrict__ db) {
  const int o = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
  if (o >= N) return;
  float acc = 0.f;
  for (int b = lane; b < B; b += 32) acc += __bfloat162float(dzt[(size_t)o * B + b]);
  for (int s = 16; s; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
  if (lane == 0) db[o] = acc;
}

// Adam on fp32 masters; refreshes the bf16 copy [rows][cols] and its
// transpose [cols][rows] (null for vectors).
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, long long n, float lr, float b1, float b2, float eps,
                       float c1, float c2, __nv_bfloat16* __restrict__ w16,
                       __nv_bfloat16* __restrict__ w16t, int rows, int cols, int ldk) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    if (w16) {
      const int r = (int)(i / cols), c = (int)(i % cols);
      const __nv_bfloat16 h = __float2bfloat16_rn(pi);
      w16[(size_t)r * ldk + c] = h;
      w16t[(size_t)c * rows + r] = h;
    }
  }
}

}  // namespace mlp
}  // namespace csg

using namespace csg;
using namespace csg::mlp;

struct csg_mlp {
  csg_ctx* ctx = nullptr;
  int L = 0;                 // linear layers (the last one has one output)
  std::vector<int> dim;      // dim[0] = n_in ... dim[L] = 1
  std::vector<int> kpad;     // padded input width of layer l (multiple of 8)
  int max_batch = 0;
  long long step = 0;
  // per layer: fp32 masters, grads, Adam moments; bf16 W [out][kpad], W^T [kpad][out]
  std::vector<float*> W, b, gW, gb, mW, vW, mb, vb;
  std::vector<__nv_bfloat16*> W16, W16t;
  // activations: H[l] bf16 [B][kpad[l]] (H[0] = input), Ht[l] [kpad[l]][B], Z[l] fp32 [B][dim[l]]
  std::vector<__nv_bfloat16*> H, Ht, dZ, dZt;
  std::vector<float*> Z;
  float* y = nullptr;
  float* dy = nullptr;
  float* loss = nullptr;
  std::vector<void*> owned;
};

template <typename T>
static T* mlp_alloc(csg_mlp* m, size_t n) {
  void* p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  cudaMemsetAsync(p, 0, std::max<size_t>(n, 1) * sizeof(T), m->ctx->stream);
  m->owned.push_back(p);
  return static_cast<T*>(p);
}

static int launch_mlp_gemm(csg_mlp* m, const __nv_bfloat16* A, int M, const __nv_bfloat16* Bm,
                           int N, int K, const GemmParams& gp0) {
  CUtensorMap ta, tb;
  int rc = make_map(&ta, A, K, M, 1, BM);
  if (!rc) rc = make_map(&tb, Bm, K, N, 1, MBN);
  if (rc) return rc;
  GemmParams gp = gp0;
  gp.M = M;
  gp.N = N;
  gp.k_blocks = (K + BK - 1) / BK;
  gp.status = m->ctx->status;
  static bool attr = false;
  if (!attr) {
    CSG_CUDA(cudaFuncSetAttribute(k_mlp_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)MSMEM));
    attr = true;
  }
  const int grid = ((M + BM - 1) / BM) * ((N + MBN - 1) / MBN);
  k_mlp_gemm<<<grid, MTHREADS, MSMEM, m->ctx->stream>>>(ta, tb, gp);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

static int mlp_forward(csg_mlp* m, int B) {
  for (int l = 0; l + 1 < m->L; ++l) {
    GemmParams gp{};
    gp.bias = m->b[l];
    gp.act = 1;
    gp.out_f32 = m->Z[l + 1];
    gp.out_bf16 = m->H[l + 1];
    gp.out_bf16t = m->Ht[l + 1];
    gp.ld_bf16 = m->kpad[l + 1];
    gp.ld_bf16t = B;
    int rc = launch_mlp_gemm(m, m->H[l], B, m->W16[l], m->dim[l + 1], m->kpad[l], gp);
    if (rc) return rc;
  }
  const int l = m->L - 1;
  k_last_forward<<<(B + 7) / 8, 256, 0, m->ctx->stream>>>(m->H[l], m->kpad[l], B, m->W[l],
                                                          m->b[l], m->y);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

extern "C" {

// Network n_in -> hidden[0] -> ... -> hidden[n_hidden-1] -> 1, He-style
// uniform initialisation from `seed`, buffers for batches up to max_batch
// (a multiple of 8).
int csg_mlp_create(csg_ctx* ctx, csg_mlp** out, int n_in, int n_hidden, const int* hidden,
                   int max_batch, unsigned long long seed) {
  CSG_CHECK(ctx && out && hidden && n_in > 0 && n_hidden > 0, CSG_E_ARG,
            "csg_mlp_create: bad argument");
  CSG_CHECK(max_batch > 0 && max_batch % 8 == 0, CSG_E_SHAPE,
            "csg_mlp_create: max_batch must be a positive multiple of 8");
  for (int i = 0; i < n_hidden; ++i)
    CSG_CHECK(hidden[i] > 0 && hidden[i] % 8 == 0, CSG_E_SHAPE,
              "csg_mlp_create: hidden widths must be multiples of 8");
  DeviceGuard g(ctx->device);
  csg_mlp* m = new csg_mlp();
  m->ctx = ctx;
  m->dim.push_back(n_in);
  for (int i = 0; i < n_hidden; ++i) m->dim.push_back(hidden[i]);
  m->dim.push_back(1);
  m->L = n_hidden + 1;
  m->max_batch = max_batch;
  for (int l = 0; l <= m->L; ++l) m->kpad.push_back((m->dim[l] + 7) / 8 * 8);
  std::mt19937_64 rng(seed);
  const int B = max_batch;
  bool ok = true;
  m->H.resize(m->L + 1);
  m->Ht.resize(m->L + 1);
  m->dZ.resize(m->L + 1);
  m->dZt.resize(m->L + 1);
  m->Z.resize(m->L + 1);
  for (int l = 0; l < m->L; ++l) {
    const int o = m->dim[l + 1], k = m->kpad[l], ki = m->dim[l];
    std::vector<float> w((size_t)o * ki), wb(o, 0.f);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    const float a = std::sqrt(6.f / ki);
    for (auto& x : w) x = a * u(rng);
    float* W = mlp_alloc<float>(m, w.size());
    float* bb = mlp_alloc<float>(m, o);
    ok &= W && bb;
    if (!ok) break;
    cudaMemcpyAsync(W, w.data(), w.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    m->W.push_back(W);
    m->b.push_back(bb);
    m->gW.push_back(mlp_alloc<float>(m, w.size()));
    m->gb.push_back(mlp_alloc<float>(m, o));
    m->mW.push_back(mlp_alloc<float>(m, w.size()));
    m->vW.push_back(mlp_alloc<float>(m, w.size()));
    m->mb.push_back(mlp_alloc<float>(m, o));
    m->vb.push_back(mlp_alloc<float>(m, o));
    m->W16.push_back(mlp_alloc<__nv_bfloat16>(m, (size_t)o * k));
    m->W16t.push_back(mlp_alloc<__nv_bfloat16>(m, (size_t)k * o));
    // bf16 copies of the initial weights (lr = 0 Adam pass writes them)
    CSG_CUDA(cudaStreamSynchronize(ctx->stream));
    k_adam<<<grid_for((long long)w.size(), 256), 256, 0, ctx->stream>>>(
        W, m->gW.back(), m->mW.back(), m->vW.back(), (long long)w.size(), 0.f, 0.f, 0.f, 1.f,
        1.f, 1.f, m->W16.back(), m->W16t.back(), o, ki, k);
  }
  for (int l = 0; l <= m->L && ok; ++l) {
    m->H[l] = mlp_alloc<__nv_bfloat16>(m, (size_t)B * m->kpad[l]);
    m->Ht[l] = mlp_alloc<__nv_bfloat16>(m, (size_t)B * m->kpad[l]);
    m->dZ[l] = mlp_alloc<__nv_bfloat16>(m, (size_t)B * m->kpad[l]);
    m->dZt[l] = mlp_alloc<__nv_bfloat16>(m, (size_t)B * m->kpad[l]);
    m->Z[l] = mlp_alloc<float>(m, (size_t)B * m->dim[l]);
    ok &= m->H[l] && m->Ht[l] && m->dZ[l] && m->dZt[l] && m->Z[l];
  }
  m->y = mlp_alloc<float>(m, B);
  m->dy = mlp_alloc<float>(m, B);
  m->loss = mlp_alloc<float>(m, 1);
  ok &= m->y && m->dy && m->loss;
  for (auto p : m->gW) ok &= p != nullptr;
  if (!ok) {
    for (void* p : m->owned) cudaFree(p);
    delete m;
    set_error("csg_mlp_create: allocation failed");
    return CSG_E_NOMEM;
  }
  CSG_CUDA(cudaStreamSynchronize(ctx->stream));
  *out = m;
  return CSG_OK;
}

int csg_mlp_destroy(csg_mlp* m) {
  if (!m) return CSG_OK;
  DeviceGuard g(m->ctx->device);
  cudaStreamSynchronize(m->ctx->stream);
  for (void* p : m->owned) cudaFree(p);
  delete m;
  return CSG_OK;
}

// Input batch from candidate sags (device FP64 [B][n_var]) and per-sample
// wavelengths (device FP64 [B]): mode 0 x = sag / sag_scale; mode 1 the hex
// phasors cos, sin(4 pi sag_scale sag / lambda) (sag_scale = phaseSign);
// then (lambda - lam0) / lam_scale.
int csg_mlp_features(csg_mlp* m, const double* sags, int n_var, const double* lam,
                     double sag_scale, double lam0, double lam_scale, int B, int mode) {
  CSG_CHECK(m && sags && lam && B > 0 && B <= m->max_batch && B % 8 == 0 && (mode == 0 || mode == 1),
            CSG_E_ARG, "csg_mlp_features: bad argument");
  CSG_CHECK((mode == 1 ? 2 * n_var : n_var) + 1 <= m->dim[0], CSG_E_SHAPE,
            "csg_mlp_features: the network input is too narrow for these features");
  DeviceGuard g(m->ctx->device);
  const int K = m->kpad[0];
  k_features<<<grid_for((long long)B * K, 256), 256, 0, m->ctx->stream>>>(
      sags, n_var, lam, sag_scale, lam0, lam_scale, B, K, mode, m->H[0], m->Ht[0]);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

// Input batch from raw fp32 features [B][n_in] (device).
int csg_mlp_set_input(csg_mlp* m, const float* x, int B) {
  CSG_CHECK(m && x && B > 0 && B <= m->max_batch && B % 8 == 0, CSG_E_ARG,
            "csg_mlp_set_input: bad argument");
  DeviceGuard g(m->ctx->device);
  const int K = m->kpad[0];
  k_set_input<<<grid_for((long long)B * K, 256), 256, 0, m->ctx->stream>>>(x, m->dim[0], B, K,
                                                                           m->H[0], m->Ht[0]);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

// Forward pass of the current input batch; y (device fp32 [B]) may be null
// (the prediction stays in the network's output buffer).
int csg_mlp_forward(csg_mlp* m, int B, float* y) {
  CSG_CHECK(m && B > 0 && B <= m->max_batch && B % 8 == 0, CSG_E_ARG,
            "csg_mlp_forward: bad batch");
  DeviceGuard g(m->ctx->device);
  int rc = mlp_forward(m, B);
  if (!rc && y)
    CSG_CUDA(cudaMemcpyAsync(y, m->y, sizeof(float) * B, cudaMemcpyDeviceToDevice, m->ctx->stream));
  return rc;
}

// One training step on the current input batch against targets t (device
// fp32 [B]): forward, MSE loss (device scalar *loss if non-null), backward,
// Adam (lr; beta 0.9 / 0.999, eps 1e-8). lr = 0 computes gradients only
// (csg_mlp_param exposes them).
int csg_mlp_train_step(csg_mlp* m, int B, const float* t, float lr, float* loss) {
  CSG_CHECK(m && t && B > 0 && B <= m->max_batch && B % 8 == 0, CSG_E_ARG,
            "csg_mlp_train_step: bad argument");
  DeviceGuard g(m->ctx->device);
  cudaStream_t st = m->ctx->stream;
  int rc = mlp_forward(m, B);
  if (rc) return rc;
  k_mse<<<1, 256, 0, st>>>(m->y, t, B, m->dy, m->loss);
  CSG_LAUNCH_CHECK();
  if (loss) CSG_CUDA(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToDevice, st));
  const int L = m->L;
  {
    const int l = L - 1, K = m->kpad[l];
    k_last_backward<<<(K + 127) / 128, 128, 0, st>>>(m->H[l], m->Z[l], K, B, m->W[l], m->dy,
                                                     m->gW[l], m->gb[l], m->dZ[l], m->dZt[l]);
    CSG_LAUNCH_CHECK();
  }
  for (int l = L - 2; l >= 0; --l) {
    const int o = m->dim[l + 1], ki = m->dim[l], kp = m->kpad[l];
    // dW = dZ^T H: A = dZ^T [o][B], B-operand = H^T [kp][B]
    GemmParams gw{};
    gw.out_f32 = m->gW[l];
    rc = launch_mlp_gemm(m, m->dZt[l + 1], o, m->Ht[l], ki, B, gw);
    if (rc) return rc;
    k_bias_grad<<<(o + 7) / 8, 256, 0, st>>>(m->dZt[l + 1], o, B, m->gb[l]);
    CSG_LAUNCH_CHECK();
    if (l > 0) {  // dH = dZ W (A = dZ [B][o], B-operand = W^T [kp][o]) times gelu'(Z)
      GemmParams gh{};
      gh.aux = m->Z[l];
      gh.act = 2;
      gh.out_bf16 = m->dZ[l];
      gh.out_bf16t = m->dZt[l];
      gh.ld_bf16 = kp;
      gh.ld_bf16t = B;
      rc = launch_mlp_gemm(m, m->dZ[l + 1], B, m->W16t[l], ki, o, gh);
      if (rc) return rc;
    }
  }
  ++m->step;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = lr > 0 ? 1.f - std::pow(b1, (float)m->step) : 1.f;
  const float c2 = lr > 0 ? 1.f - std::pow(b2, (float)m->step) : 1.f;
  for (int l = 0; l < L && lr > 0; ++l) {
    const int o = m->dim[l + 1], ki = m->dim[l];
    const long long nw = (long long)o * ki;
    k_adam<<<grid_for(nw, 256), 256, 0, st>>>(m->W[l], m->gW[l], m->mW[l], m->vW[l], nw, lr, b1,
                                              b2, 1e-8f, c1, c2, m->W16[l], m->W16t[l], o, ki,
                                              m->kpad[l]);
    CSG_LAUNCH_CHECK();
    k_adam<<<grid_for(o, 256), 256, 0, st>>>(m->b[l], m->gb[l], m->mb[l], m->vb[l], o, lr, b1,
                                             b2, 1e-8f, c1, c2, nullptr, nullptr, 0, 1, 0);
    CSG_LAUNCH_CHECK();
  }
  return CSG_OK;
}

// Device pointers of layer l: fp32 weights [out][in], bias [out], and their
// gradients from the last training step.
int csg_mlp_param(csg_mlp* m, int l, float** w, float** b, float** gw, float** gb) {
  CSG_CHECK(m && l >= 0 && l < m->L, CSG_E_ARG, "csg_mlp_param: bad layer");
  if (w) *w = m->W[l];
  if (b) *b = m->b[l];
  if (gw) *gw = m->gW[l];
  if (gb) *gb = m->gb[l];
  return CSG_OK;
}

}  // extern "C"
