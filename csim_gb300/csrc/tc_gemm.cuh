// tcgen05 split-bf16 GEMM for the matrix Fourier transforms.
//
// One launch computes, for a batch of fields, the real-ified complex product
//   C = sum_{terms (pa,pb)} sum_{comp c} A[pa, sel] * B[pb, sel]^T
// with both operands K-major bf16 tiles staged by TMA (128B swizzle) into a
// shared-memory ring, multiplied by a single issuing thread
// (tcgen05.mma.cta_group::1.kind::f16, M = 128, N = BN, K = 16 per
// instruction) into rotating tensor-memory slots, and drained by eight warps
// (tcgen05.ld.32x32b) into fp32 register accumulators.
//
// Operand roles: one operand is a field ("data", indexed by field and split
// part) and the other an MFT operator ("op", indexed by the field's slot and
// split part). Complex arithmetic is real-ified: each tile produces one
// output component d (re or im), and each K segment pairs data component c
// with operator plane sel(d, c) in {re, im, -im}:
//   (d,c) = (re,re): re   (re,im): -im   (im,re): im   (im,im): re
#pragma once
#include <cuda.h>
#include "common.cuh"

namespace csg {
namespace tc {

constexpr int BM = 128;
constexpr int BK = 64;  // bf16 elements per 128-byte swizzled row

enum Epi { EPI_T_SPLIT = 0, EPI_F32 = 1 };

struct Params {
  int n_fields;
  int m_tiles;      // tiles along M (stage 2 counts both components)
  int n_tiles;      // tiles along N (stage 1 counts both components)
  int m_half;       // stage 2: tiles per component along M
  int n_half;       // stage 1: tiles per component along N
  int rows_valid;   // stage 1: Ny (data rows); stage 2: Mo (operator rows per comp)
  int cols_valid;   // No (valid output columns)
  int k_blocks;     // ceil(K / BK)
  int n_terms;
  int term_a[8];
  int term_b[8];
  const int* slot;  // [n_fields] operator slot of each field
  void* out;
  int out_rows;     // EPI_T_SPLIT: No (rows of T^T); EPI_F32: Mo
  int out_cols;     // EPI_T_SPLIT: Ny; EPI_F32: No
  int accumulate;   // EPI_F32 only
  // EPI_F32 output window: element (v, u) of a field's component plane is
  // stored at (out_r0 + v) * out_pitch + out_c0 + u of planes that are
  // out_plane_rows x out_pitch (a sub-rectangle of a larger field).
  int out_pitch, out_plane_rows, out_r0, out_c0;
  int* status;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ uint32_t mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok;
}

// Bounded wait: false once the cycle budget is spent.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  if (mbar_try_wait(a, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(a, parity)) {
    if (clock64() - t0 > kWaitBudgetCycles) return false;
  }
  return true;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, uint64_t* bar,
                                            int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// K-major, 128-byte swizzle, 8-row atoms of 1024 bytes stacked along M/N.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;                 // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;       // stride byte offset: next 8-row atom
  d |= (uint64_t)1 << 46;                 // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                 // SWIZZLE_128B
  return d;
}

// kind::f16 instruction descriptor: bf16 x bf16 -> f32, both K-major.
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
  return (1u << 4)                 // D format f32
         | (1u << 7)               // A format bf16
         | (1u << 10)              // B format bf16
         | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                     uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 32 lanes x 32 columns of fp32 from tensor memory (no wait).
__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ int sel_plane(int d, int c) {
  // (re,re)->0 re, (re,im)->2 -im, (im,re)->1 im, (im,im)->0 re
  return d == 0 ? (c == 0 ? 0 : 2) : (c == 0 ? 1 : 0);
}


// Accumulation and precision. Tensor-core fp32 accumulation truncates at
// every instruction, so a long chain of the dominant product in tensor
// memory would shrink the result by ~2^-24 per instruction. The products of
// the three-way split are therefore grouped by magnitude (part indices
// pa + pb): group 0 (hi x hi) goes to a fresh tensor-memory slot every K
// block (two slots rotate) and eight drain warps add each finished slot into
// fp32 registers with round-to-nearest adds while the next block is
// multiplied; group 1 (hi x mid, mid x hi, 2^-8 of the result) and group 2
// (the 2^-16 terms) accumulate over the whole K range in two persistent
// slots, where the truncation is relative to their own small magnitude, and
// are added once at the end.
//
// Operand traffic. A pipeline stage holds every split part of the A and B
// tiles of one K block (3 + 3 tiles for bf16x6), and all the products of
// that block are issued from it, so each part tile crosses L2 once per K
// block (instead of once per product).
constexpr int DRAIN_WARPS = 8;
constexpr int THREADS = (DRAIN_WARPS + 2) * 32;  // + TMA producer warp + MMA warp
constexpr int PRODUCER_WARP = DRAIN_WARPS;
constexpr int MMA_WARP = DRAIN_WARPS + 1;
constexpr int MAX_PARTS = 3;

template <int BN>
struct Cfg {
  static_assert(BN == 64 || BN == 128, "N tile must be 64 or 128");
  static constexpr uint32_t A_BYTES = BM * BK * 2;
  static constexpr uint32_t B_BYTES = BN * BK * 2;
  static constexpr uint32_t STAGE_BYTES = MAX_PARTS * (A_BYTES + B_BYTES);
  static constexpr int STAGES = BN == 128 ? 2 : 3;  // 192 KB / 216 KB of operand ring
  static constexpr int TMEM_COLS = 4 * BN;          // group 1, group 2, two rotating slots
  static constexpr int COLS_PER_WARP = BN / 2;      // two warps share a lane quadrant
  static constexpr size_t SMEM = (size_t)STAGES * STAGE_BYTES + 1024 + 512;
};

template <int BN>
constexpr size_t smem_bytes() {
  return Cfg<BN>::SMEM;
}

// Drain one lane quadrant's CPW columns at taddr into acc (+=).
template <int CPW>
__device__ __forceinline__ void drain_add(uint32_t taddr, float* acc) {
#pragma unroll
  for (int cb = 0; cb < CPW; cb += 64) {
    uint32_t r[64];
    tmem_ld32_nowait(taddr + cb, r);
    if (cb + 32 < CPW) tmem_ld32_nowait(taddr + cb + 32, r + 32);
    tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < 64; ++j)
      if (cb + j < CPW) acc[cb + j] += __uint_as_float(r[j]);
  }
}

// OP_IS_A = false: stage 1 (A = data rows y, B = operator rows u, d from N tile)
// OP_IS_A = true : stage 2 (A = operator rows v, B = data rows u, d from M tile)
template <int BN, bool OP_IS_A, int EPI>
__global__ void __launch_bounds__(THREADS, 1)
    k_split_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                 const Params p) {
  using CF = Cfg<BN>;
  constexpr int STAGES = CF::STAGES;
  constexpr int NSLOT = 2;  // rotating group-0 slots
  constexpr int CPW = CF::COLS_PER_WARP;
  extern __shared__ uint8_t smem_raw[];

  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  uint8_t* sbase = smem_raw + (base - smem_u32(smem_raw));
  uint64_t* full = reinterpret_cast<uint64_t*>(sbase + STAGES * CF::STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;   // slot filled by the MMA warp
  uint64_t* tempty = tfull + NSLOT;   // slot drained by the drain warps
  uint64_t* quiesce = tempty + NSLOT;  // abort path: in-flight products done
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(quiesce + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  int t = blockIdx.x;
  const int nt = t % p.n_tiles;
  t /= p.n_tiles;
  const int mt = t % p.m_tiles;
  const int field = t / p.m_tiles;
  if (field >= p.n_fields) return;
  const int slot = p.slot[field];

  int d, row_a0, row_b0;
  if (!OP_IS_A) {
    d = nt / p.n_half;
    row_a0 = mt * BM;
    row_b0 = (nt % p.n_half) * BN;
  } else {
    d = mt / p.m_half;
    row_a0 = (mt % p.m_half) * BM;
    row_b0 = nt * BN;
  }
  int n_parts = 1;
  for (int i = 0; i < p.n_terms; ++i)
    n_parts = max(n_parts, 1 + max(p.term_a[i], p.term_b[i]));

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int s = 0; s < NSLOT; ++s) {
      mbar_init(&tfull[s], 1);
      mbar_init(&tempty[s], DRAIN_WARPS);
    }
    mbar_init(quiesce, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(CF::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t t_g1 = tmem, t_g2 = tmem + BN, t_rot = tmem + 2 * BN;

  const int k_iters = 2 * p.k_blocks;  // (data component c, K block)

  if (warp == PRODUCER_WARP) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      for (int it = 0; it < k_iters; ++it) {
        if (it >= STAGES && !mbar_wait(&empty[stage], phase ^ 1)) {
          atomicExch(p.status, 1);
          *abort_flag = 1;
          break;
        }
        if (*abort_flag) break;
        const int kb = it % p.k_blocks;
        const int c = it / p.k_blocks;
        uint8_t* sA = sbase + stage * CF::STAGE_BYTES;
        uint8_t* sB = sA + MAX_PARTS * CF::A_BYTES;
        mbar_expect_tx(&full[stage], n_parts * (CF::A_BYTES + CF::B_BYTES));
        for (int pp = 0; pp < n_parts; ++pp) {
          int za, zb;
          if (!OP_IS_A) {
            za = (field * 3 + pp) * 2 + c;
            zb = (slot * 3 + pp) * 3 + sel_plane(d, c);
          } else {
            za = (slot * 3 + pp) * 3 + sel_plane(d, c);
            zb = (field * 3 + pp) * 2 + c;
          }
          tma_load_3d(sA + pp * CF::A_BYTES, &tmA, &full[stage], kb * BK, row_a0, za);
          tma_load_3d(sB + pp * CF::B_BYTES, &tmB, &full[stage], kb * BK, row_b0, zb);
        }
        if (++stage == STAGES) {
          stage = 0;
          phase ^= 1;
        }
      }
    }
    __syncwarp();
  } else if (warp == MMA_WARP) {
    if (lane == 0) {
      constexpr uint32_t idesc = instr_desc(BM, BN);
      int stage = 0;
      uint32_t phase = 0;
      bool g1_on = false, g2_on = false;  // persistent groups hold data
      for (int it = 0; it < k_iters; ++it) {
        const int ts = it % NSLOT;
        const uint32_t round = (uint32_t)(it / NSLOT);
        bool ok = true;
        if (it >= NSLOT) ok = mbar_wait(&tempty[ts], (round & 1u) ^ 1u);
        if (ok) ok = mbar_wait(&full[stage], phase);
        if (!ok || *abort_flag) {
          atomicExch(p.status, 2);
          *abort_flag = 1;
          // let the products already issued finish before tensor memory is
          // released (bounded wait), then release every drain wait so nobody
          // waits for the full budget again
          umma_commit(quiesce);
          mbar_wait(quiesce, 0);
          for (int s = 0; s < NSLOT; ++s)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tfull[s]))
                         : "memory");
          break;
        }
        tc_fence_after();
        const uint32_t a0 = smem_u32(sbase + stage * CF::STAGE_BYTES);
        const uint32_t b0 = a0 + MAX_PARTS * CF::A_BYTES;
        for (int i = 0; i < p.n_terms; ++i) {
          const int pa = p.term_a[i], pb = p.term_b[i];
          const int g = min(pa + pb, 2);
          const uint32_t dcol = g == 0 ? t_rot + (uint32_t)(ts * BN) : (g == 1 ? t_g1 : t_g2);
          bool on = g == 0 ? false : (g == 1 ? g1_on : g2_on);
          const uint32_t aa = a0 + pa * CF::A_BYTES, bb = b0 + pb * CF::B_BYTES;
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
            umma(dcol, smem_desc(aa + k * 32), smem_desc(bb + k * 32), idesc, on ? 1u : 0u);
            on = true;
          }
          if (g == 1) g1_on = true;
          if (g == 2) g2_on = true;
        }
        umma_commit(&empty[stage]);
        umma_commit(&tfull[ts]);
        if (++stage == STAGES) {
          stage = 0;
          phase ^= 1;
        }
      }
    }
    __syncwarp();
  } else {
    // ---------------- drain warps: quadrant q of the 128 rows, half h of the columns
    const int q = warp & 3, h = warp >> 2;
    const int row = q * 32 + lane;
    const uint32_t lane_off = ((uint32_t)(q * 32) << 16) + (uint32_t)(h * CPW);
    float acc[CPW];
#pragma unroll
    for (int j = 0; j < CPW; ++j) acc[j] = 0.f;
    bool ok = true;
    for (int it = 0; it < k_iters; ++it) {
      const int ts = it % NSLOT;
      const uint32_t round = (uint32_t)(it / NSLOT);
      ok = mbar_wait(&tfull[ts], round & 1u);
      ok = __all_sync(0xffffffffu, ok && !*abort_flag);
      if (!ok) break;
      tc_fence_after();
      drain_add<CPW>(t_rot + (uint32_t)(ts * BN) + lane_off, acc);
      tc_fence_before();
      __syncwarp();
      if (lane == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[ts]))
                     : "memory");
    }
    if (ok) {
      // the last commit covered every product: add the persistent groups
      // (smaller first: g2 into g1, then into the accumulator)
      tc_fence_after();
      float gsum[CPW];
#pragma unroll
      for (int j = 0; j < CPW; ++j) gsum[j] = 0.f;
      drain_add<CPW>(t_g2 + lane_off, gsum);
      drain_add<CPW>(t_g1 + lane_off, gsum);
#pragma unroll
      for (int j = 0; j < CPW; ++j) acc[j] += gsum[j];
    }
    if (!ok) {
      atomicExch(p.status, 3);
    } else if (EPI == EPI_T_SPLIT) {
      // C[y][u] -> T^T parts [field][part][d][u][y] (bf16)
      const int y = row_a0 + row;
      if (y < p.out_cols) {
        __nv_bfloat16* out = reinterpret_cast<__nv_bfloat16*>(p.out);
        const size_t plane = (size_t)p.out_rows * p.out_cols;
        const int u0 = row_b0 + h * CPW;
#pragma unroll
        for (int j = 0; j < CPW; ++j) {
          const int u = u0 + j;
          if (u < p.cols_valid) {
            __nv_bfloat16 h0, h1, h2;
            split3(acc[j], h0, h1, h2);
            const size_t off = (size_t)u * p.out_cols + y;
            out[((size_t)(field * 3 + 0) * 2 + d) * plane + off] = h0;
            out[((size_t)(field * 3 + 1) * 2 + d) * plane + off] = h1;
            out[((size_t)(field * 3 + 2) * 2 + d) * plane + off] = h2;
          }
        }
      }
    } else {
      // C[v][u] -> out fp32 [field][d][out_r0 + v][out_c0 + u] (pitch out_pitch)
      const int v = row_a0 + row;
      if (v < p.rows_valid) {
        float* out = reinterpret_cast<float*>(p.out) +
                     ((size_t)(field * 2 + d) * p.out_plane_rows + p.out_r0 + v) * p.out_pitch +
                     p.out_c0;
        const int u0 = row_b0 + h * CPW;
        if (u0 + CPW <= p.cols_valid && ((p.out_pitch | p.out_c0) & 3) == 0) {
          float4* o4 = reinterpret_cast<float4*>(out + u0);
#pragma unroll
          for (int j = 0; j < CPW / 4; ++j) {
            float4 val = make_float4(acc[4 * j], acc[4 * j + 1], acc[4 * j + 2], acc[4 * j + 3]);
            if (p.accumulate) {
              const float4 old = o4[j];
              val.x += old.x; val.y += old.y; val.z += old.z; val.w += old.w;
            }
            o4[j] = val;
          }
        } else {
#pragma unroll
          for (int j = 0; j < CPW; ++j) {
            const int u = u0 + j;
            if (u < p.cols_valid) {
              float val = acc[j];
              if (p.accumulate) val += out[u];
              out[u] = val;
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(CF::TMEM_COLS));
  }
}

}  // namespace tc
}  // namespace csg
