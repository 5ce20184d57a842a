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
  int k_blocks;     // ceil(K / K block): 64 elements, 32 for N = 256 tiles
  int n_terms;      // products of the split issued (6: bf16x6, 3: bf16x3; see term_a)
  const int* slot;  // [n_fields] operator slot of each field
  void* out;
  int out_rows;     // EPI_T_SPLIT: No (rows of T^T); EPI_F32: Mo
  int out_cols;     // EPI_T_SPLIT: Ny; EPI_F32: No
  int accumulate;   // EPI_F32 only
  // EPI_F32 output window: element (v, u) of a field's component plane is
  // stored at (out_r0 + v) * out_pitch + out_c0 + u of planes that are
  // out_plane_rows x out_pitch (a sub-rectangle of a larger field).
  int out_pitch, out_plane_rows, out_r0, out_c0;
  // EPI_F32 through the output tensor map (fp32, origin at the window's
  // (out_r0, out_c0), box 32 x 32, 128B swizzle): tiles are staged in the
  // free operand ring and written by TMA stores, or by TMA add-reductions
  // when accumulating. 0: per-thread stores.
  int tma_out;
  // ragged plans: slot s's outputs are zero beyond valid[s] rows and columns
  // (its operator rows there are zero), so tiles starting beyond it are not
  // computed (stage 2 writes their zeros); nullptr: every tile
  const int* valid;
  int* status;
  // high precision, EPI_F32: the low words of the two-float results, stored
  // per thread beside `out` (same window and pitch); null: not written
  float* out_lo;
  // cycles a role waits for another before the tile walk gives up (the
  // context's csg_set_wait_budget; 0: kWaitBudgetCycles). The clean-up after
  // a give-up always waits with the full budget.
  long long wait_budget;
  // K blocks ahead at which the producer prefetches the field operand's
  // parts into L2 (0: no prefetch)
  int prefetch;
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
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          long long budget = kWaitBudgetCycles) {
  const uint32_t a = smem_u32(bar);
  if (mbar_try_wait(a, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(a, parity)) {
    if (clock64() - t0 > budget) return false;
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

// L2 prefetch of one box at (x, y, z) (no shared memory, no completion).
__device__ __forceinline__ void tma_prefetch_3d(const CUtensorMap* tm, int x, int y, int z) {
  asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"(
                   reinterpret_cast<uint64_t>(tm)),
               "r"(x), "r"(y), "r"(z)
               : "memory");
}

// Shared -> global tile store, or element-wise fp32 add into global (the
// reduction is applied at L2), of one box at (x, y, z); bulk-group completion.
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* tm, const void* src, int x, int y,
                                             int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
          reinterpret_cast<uint64_t>(tm)),
      "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
      : "memory");
}
__device__ __forceinline__ void tma_reduce_add_3d(const CUtensorMap* tm, const void* src, int x,
                                                  int y, int z) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.tile.bulk_group"
      " [%0, {%2, %3, %4}], [%1];" ::"l"(reinterpret_cast<uint64_t>(tm)),
      "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// Waits until the committed bulk copies have finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// Orders this thread's generic-proxy shared-memory writes before later
// async-proxy (TMA) reads.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
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

// K-major, 64-byte swizzle: 8-row atoms of 512 bytes (32-wide K blocks).
__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(512 >> 4) << 32;        // stride byte offset: next 8-row atom
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)4 << 61;                 // SWIZZLE_64B
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
// pa + pb): hi x hi goes to a fresh tensor-memory slot every K block (three
// slots rotate) and eight drain warps add each finished slot into fp32
// registers with round-to-nearest adds while the rest of the block and the
// next blocks are multiplied (each block issues hi x hi first and commits
// its slot before the smaller products); the smaller products (hi x mid,
// mid x hi: 2^-8 of the result; the 2^-16 terms) accumulate over the whole K
// range in one persistent slot, where the truncation is relative to their
// own small magnitude (the 2^-16 terms lose only bits below 2^-32 of the
// result there), and are added once at the end of the tile.
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

// Persistent CTAs: each CTA walks the tiles blockIdx.x, blockIdx.x + grid,
// ... with the operand ring, the rotating slots and their barriers running
// on across tiles, so the producer loads the next tile while the current
// one finishes and its epilogue runs. The fp32 epilogue stages its boxes in
// a region of its own (4 KB per drain warp), apart from the ring.
//
// N = 256 tiles issue 256-wide products (which keep the tensor pipe busier
// than 128-wide ones for the same shared-memory operand traffic per FLOP).
// Their three-part stages use 32-wide K blocks (64-byte swizzle) to leave
// room for two or three stages, and tensor memory holds one 256-column
// rotating hi x hi slot beside the small products' slot: hi x hi is
// committed first, so its drain overlaps the rest of the block.
//
// KB_ selects the K block explicitly (0: 64, or 32 for 256-wide tiles).
// Measured on the 1024^2 PIAACMC chain at 76 fields: 128-wide tiles with
// four 32-wide-K stages kept the tensor pipe 55% busy against 66% for two
// 64-wide ones (twice the per-block barrier, commit and drain overhead for
// no gain in operand latency), so the 64-wide blocks stay the default.
template <int BN, int EPI, bool HP = false, int KB_ = 0>
struct Cfg {
  static_assert(BN == 64 || BN == 128 || BN == 256, "N tile must be 64, 128 or 256");
  static_assert(!HP || BN <= 128, "high precision: N tile 64 or 128");
  static_assert(KB_ == 0 || KB_ == 32 || KB_ == 64, "K block: 32 or 64 elements");
  static constexpr int KB = KB_ ? KB_ : (BN == 256 ? 32 : BK);  // K elements per stage
  static_assert(BN != 256 || KB == 32, "256-wide tiles use 32-wide K blocks");
  static constexpr uint32_t A_BYTES = BM * KB * 2;
  static constexpr uint32_t B_BYTES = BN * KB * 2;
  static constexpr uint32_t STAGE_BYTES = MAX_PARTS * (A_BYTES + B_BYTES);
  // fp32 epilogue: 4 KB box per drain warp; high-precision split epilogue:
  // the per-column group maxima of each warp, double-buffered by tile
  static constexpr uint32_t STAGING_BYTES =
      EPI == 1 ? DRAIN_WARPS * 4096 : (HP ? 2 * DRAIN_WARPS * (BN / 2) * 4 : 0);
  // as many operand stages as fit beside the staging region and the
  // barriers (at most four): two 96 KB stages at N = 128 with 64-wide K
  // blocks, four 48 KB stages with 32-wide ones
  static constexpr int STAGES_FIT = (int)((232448u - STAGING_BYTES - 1536u) / STAGE_BYTES);
  static constexpr int STAGES = STAGES_FIT < 4 ? STAGES_FIT : 4;
  static_assert(STAGES >= 2, "at least two operand stages");
  static constexpr int NSLOT = BN == 256 ? 1 : 3;  // rotating hi x hi slots
  static constexpr int TMEM_COLS = BN * (1 + NSLOT);  // small products + rotating
  static constexpr int COLS_PER_WARP = BN / 2;      // two warps share a lane quadrant
  static constexpr int BN_ = BN;
  static constexpr size_t SMEM = (size_t)STAGES * STAGE_BYTES + STAGING_BYTES + 1024 + 512;
  static_assert(SMEM <= 232448, "shared memory per CTA");
};

template <int BN, int EPI, bool HP = false, int KB_ = 0>
constexpr size_t smem_bytes() {
  return Cfg<BN, EPI, HP, KB_>::SMEM;
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

// High precision: each K block's exact hi x hi sum joins a two-float
// register accumulator (acc, lo) through an error-free TwoSum. The low word
// only gathers rounding errors of the fp32 word (each below half its ulp),
// so it is kept in bf16 pairs: its own 2^-9 relative rounding is 2^-33 of
// the result, and both words of 64 columns fit the drain warps' registers.
template <int CPW>
__device__ __forceinline__ void drain_add2(uint32_t taddr, float* acc, __nv_bfloat162* lo) {
#pragma unroll
  for (int cb = 0; cb < CPW; cb += 32) {
    uint32_t r[32];
    tmem_ld32_nowait(taddr + cb, r);
    tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < 32; j += 2) {
      float s0, e0, s1, e1;
      two_sum(acc[cb + j], __uint_as_float(r[j]), s0, e0);
      two_sum(acc[cb + j + 1], __uint_as_float(r[j + 1]), s1, e1);
      acc[cb + j] = s0;
      acc[cb + j + 1] = s1;
      lo[(cb + j) / 2] = __hadd2(lo[(cb + j) / 2], __floats2bfloat162_rn(e0, e1));
    }
  }
}

// The end of a high-precision tile: the smaller products' slot (fp32) and
// the low words join, and (acc, lo) become the renormalised pair: acc the
// fp32 rounding of the result, lo the rest.
template <int CPW>
__device__ __forceinline__ void drain_final2(uint32_t taddr, float* acc, __nv_bfloat162* lo) {
#pragma unroll
  for (int cb = 0; cb < CPW; cb += 32) {
    uint32_t r[32];
    tmem_ld32_nowait(taddr + cb, r);
    tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < 32; j += 2) {
      const float2 l = __bfloat1622float2(lo[(cb + j) / 2]);
      float s0, e0, s1, e1;
      two_sum(acc[cb + j], __uint_as_float(r[j]) + l.x, s0, e0);
      two_sum(acc[cb + j + 1], __uint_as_float(r[j + 1]) + l.y, s1, e1);
      acc[cb + j] = s0;
      acc[cb + j + 1] = s1;
      lo[(cb + j) / 2] = __floats2bfloat162_rn(e0, e1);
    }
  }
}

// Split products in issue order: (A part, B part), hi x hi first, then
// the 2^-8 group and the 2^-16 group. n_terms = 6 (bf16x6) or 3 (bf16x3)
// takes a prefix.
// (0,0) (0,1) (1,0) (0,2) (1,1) (2,0)
__host__ __device__ constexpr int term_a(int i) { return i == 2 || i == 4 ? 1 : (i == 5 ? 2 : 0); }
__host__ __device__ constexpr int term_b(int i) { return i == 1 || i == 4 ? 1 : (i == 3 ? 2 : 0); }
// hi x hi (group 0) and the smaller products (groups 1 and 2, one slot)
__host__ __device__ constexpr int term_group(int i) { return term_a(i) + term_b(i) == 0 ? 0 : 1; }
__host__ __device__ constexpr bool first_of_group(int i) {
  for (int j = 0; j < i; ++j)
    if (term_group(j) == term_group(i)) return false;
  return true;
}

// Every product of one K block: group 0 into the block's rotating slot d0
// (fresh), the smaller products into the persistent slot t_gs (fresh only
// for the first of them in the first block).
template <int I0, int NT, class CF>
__device__ __forceinline__ void issue_block(uint64_t da, uint64_t db, uint32_t d0, uint32_t t_gs,
                                            bool first_block) {
  constexpr uint32_t idesc = instr_desc(BM, CF::BN_);
#pragma unroll
  for (int i = I0; i < NT; ++i) {
    const int g = term_group(i);
    const uint32_t dcol = g == 0 ? d0 : t_gs;
    const uint64_t dA = da + (uint64_t)((term_a(i) * CF::A_BYTES) >> 4);
    const uint64_t dB = db + (uint64_t)((term_b(i) * CF::B_BYTES) >> 4);
#pragma unroll
    for (int k = 0; k < CF::KB / 16; ++k) {
      const bool fresh = k == 0 && (g == 0 || (first_of_group(i) && first_block));
      umma(dcol, dA + 2 * k, dB + 2 * k, idesc, fresh ? 0u : 1u);
    }
  }
}

// OP_IS_A = false: stage 1 (A = data rows y, B = operator rows u, d from N tile)
// OP_IS_A = true : stage 2 (A = operator rows v, B = data rows u, d from M tile)
struct TileCoord {
  int field, d, row_a0, row_b0;
};

// Whether a tile of a ragged plan lies wholly beyond its slot's outputs:
// stage 1 by its output columns (rows of T), stage 2 by its output rows or
// columns.
template <bool OP_IS_A>
__device__ __forceinline__ bool tile_beyond(const Params& p, const TileCoord& tc) {
  if (!p.valid) return false;
  const int v = p.valid[p.slot[tc.field]];
  return OP_IS_A ? (tc.row_a0 >= v || tc.row_b0 >= v) : tc.row_b0 >= v;
}
template <int BN, bool OP_IS_A>
__device__ __forceinline__ TileCoord tile_coord(const Params& p, int t) {
  TileCoord c;
  const int nt = t % p.n_tiles;
  t /= p.n_tiles;
  const int mt = t % p.m_tiles;
  c.field = t / p.m_tiles;
  if (!OP_IS_A) {
    c.d = nt / p.n_half;
    c.row_a0 = mt * BM;
    c.row_b0 = (nt % p.n_half) * BN;
  } else {
    c.d = mt / p.m_half;
    c.row_a0 = (mt % p.m_half) * BM;
    c.row_b0 = nt * BN;
  }
  return c;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

template <int BN, bool OP_IS_A, int EPI, bool HP = false, int KB_ = 0>
__global__ void __launch_bounds__(THREADS, 1)
    k_split_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                 const __grid_constant__ CUtensorMap tmO, const Params p) {
  using CF = Cfg<BN, EPI, HP, KB_>;
  constexpr int STAGES = CF::STAGES;
  constexpr int NSLOT = CF::NSLOT;  // rotating group-0 slots
  constexpr int CPW = CF::COLS_PER_WARP;
  extern __shared__ uint8_t smem_raw[];

  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  uint8_t* sbase = smem_raw + (base - smem_u32(smem_raw));
  uint8_t* staging = sbase + STAGES * CF::STAGE_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(staging + CF::STAGING_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;   // slot filled by the MMA warp
  uint64_t* tempty = tfull + NSLOT;   // slot drained by the drain warps
  uint64_t* gdone = tempty + NSLOT;   // a tile's products all complete (per tile)
  uint64_t* gfree = gdone + 1;        // a tile's persistent slot read (per tile)
  uint64_t* quiesce = gfree + 1;      // abort path: in-flight products done
  uint64_t* pairbar = quiesce + 1;    // HP split epilogue: warp pairs' maxima written (4)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(pairbar + DRAIN_WARPS / 2);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int n_tiles_total = p.n_fields * p.m_tiles * p.n_tiles;
  const int n_parts = p.n_terms > 3 ? 3 : 2;  // parts the issued products read
  const int k_iters = 2 * p.k_blocks;         // (data component c, K block) per tile
  const long long wb = p.wait_budget > 0 ? p.wait_budget : kWaitBudgetCycles;
  long long g_issued = 0;  // producer lane: loads issued (their stages' phases)

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int s = 0; s < NSLOT; ++s) {
      mbar_init(&tfull[s], 1);
      mbar_init(&tempty[s], DRAIN_WARPS);
    }
    mbar_init(gdone, 1);
    mbar_init(gfree, DRAIN_WARPS);
    mbar_init(quiesce, 1);
    for (int q = 0; q < DRAIN_WARPS / 2; ++q) mbar_init(&pairbar[q], 64);
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
  const uint32_t t_gs = tmem, t_rot = tmem + BN;

  if (warp == PRODUCER_WARP) {
    if (lane == 0) {
      long long g = 0;  // iterations over all of this CTA's tiles
      for (int t = blockIdx.x; t < n_tiles_total && !*abort_flag; t += gridDim.x) {
        const TileCoord tc = tile_coord<BN, OP_IS_A>(p, t);
        if (tile_beyond<OP_IS_A>(p, tc)) continue;
        const int slot = p.slot[tc.field];
        for (int it = 0; it < k_iters; ++it, ++g) {
          const int stage = (int)(g % STAGES);
          const uint32_t phase = (uint32_t)((g / STAGES) & 1);
          if (g >= STAGES && !mbar_wait(&empty[stage], phase ^ 1, wb)) {
            atomicExch(p.status, 1);
            *abort_flag = 1;
          }
          if (*abort_flag) break;
          g_issued = g + 1;
          const int kb = it % p.k_blocks;
          const int c = it / p.k_blocks;
          uint8_t* sA = sbase + stage * CF::STAGE_BYTES;
          uint8_t* sB = sA + MAX_PARTS * CF::A_BYTES;
          mbar_expect_tx(&full[stage], n_parts * (CF::A_BYTES + CF::B_BYTES));
          for (int pp = 0; pp < n_parts; ++pp) {
            int za, zb;
            if (!OP_IS_A) {
              za = (tc.field * 3 + pp) * 2 + c;
              zb = (slot * 3 + pp) * 3 + sel_plane(tc.d, c);
            } else {
              za = (slot * 3 + pp) * 3 + sel_plane(tc.d, c);
              zb = (tc.field * 3 + pp) * 2 + c;
            }
            tma_load_3d(sA + pp * CF::A_BYTES, &tmA, &full[stage], kb * CF::KB, tc.row_a0, za);
            tma_load_3d(sB + pp * CF::B_BYTES, &tmB, &full[stage], kb * CF::KB, tc.row_b0, zb);
          }
          // The field operand streams from DRAM (the operator stays in L2):
          // its parts for block it + PF are prefetched into L2 now, so that
          // their loads, issued with only one stage of lead, find them there.
          const int PF = p.prefetch;
          if (PF > 0 && it + PF < k_iters) {
            const int kbp = (it + PF) % p.k_blocks, cp = (it + PF) / p.k_blocks;
            for (int pp = 0; pp < n_parts; ++pp) {
              const int zd = (tc.field * 3 + pp) * 2 + cp;
              if (!OP_IS_A)
                tma_prefetch_3d(&tmA, kbp * CF::KB, tc.row_a0, zd);
              else
                tma_prefetch_3d(&tmB, kbp * CF::KB, tc.row_b0, zd);
            }
          }
        }
      }
    }
    __syncwarp();
  } else if (warp == MMA_WARP) {
    if (lane == 0) {
      long long g = 0;
      int j = 0;  // tiles done by this CTA
      bool ok = true;
      for (int t = blockIdx.x; t < n_tiles_total && ok; t += gridDim.x) {
        if (tile_beyond<OP_IS_A>(p, tile_coord<BN, OP_IS_A>(p, t))) continue;
        for (int it = 0; it < k_iters; ++it, ++g) {
          const int stage = (int)(g % STAGES);
          const uint32_t phase = (uint32_t)((g / STAGES) & 1);
          const int ts = (int)(g % NSLOT);
          const uint32_t round = (uint32_t)((g / NSLOT) & 1);
          if (g >= NSLOT) ok = mbar_wait(&tempty[ts], round ^ 1u, wb);
          if (ok) ok = mbar_wait(&full[stage], phase, wb);
          // the previous tile's persistent slot must be read before this
          // tile's first products overwrite them
          if (ok && it == 0 && j > 0) ok = mbar_wait(gfree, (uint32_t)((j - 1) & 1), wb);
          if (!ok || *abort_flag) {
            ok = false;
            atomicExch(p.status, 2);
            *abort_flag = 1;
            // release the drain warps' waits (they see the flag and stop);
            // the products already issued are waited out at the end
            for (int s = 0; s < NSLOT; ++s) mbar_arrive(&tfull[s]);
            mbar_arrive(gdone);
            break;
          }
          tc_fence_after();
          // descriptors of the stage's part tiles: the start-address field is
          // (address >> 4), so offsets are added to it directly (shared
          // addresses stay below 2^18: no carry out of the 14-bit field)
          const uint32_t a0 = smem_u32(sbase + stage * CF::STAGE_BYTES);
          const uint32_t b0 = a0 + MAX_PARTS * CF::A_BYTES;
          const uint64_t da = CF::KB == 64 ? smem_desc(a0) : smem_desc_sw64(a0);
          const uint64_t db = CF::KB == 64 ? smem_desc(b0) : smem_desc_sw64(b0);
          // One thread issues every product of the block, so the issue loop
          // is fully unrolled over the fixed term order (descriptor offsets
          // and accumulate flags are constants; only the first smaller
          // product depends on it). hi x hi goes first and its slot is
          // committed to the drain warps while the smaller products are
          // multiplied.
          const uint32_t d0 = t_rot + (uint32_t)(ts * BN);
          issue_block<0, 1, CF>(da, db, d0, t_gs, it == 0);
          umma_commit(&tfull[ts]);
          if (p.n_terms == 6)
            issue_block<1, 6, CF>(da, db, d0, t_gs, it == 0);
          else
            issue_block<1, 3, CF>(da, db, d0, t_gs, it == 0);
          umma_commit(&empty[stage]);
        }
        if (ok) umma_commit(gdone);  // the tile's persistent slot is final
        ++j;
      }
    }
    __syncwarp();
  } else {
    // ---------------- drain warps: quadrant q of the 128 rows, half h of the columns
    const int q = warp & 3, h = warp >> 2;
    const int row = q * 32 + lane;
    const uint32_t lane_off = ((uint32_t)(q * 32) << 16) + (uint32_t)(h * CPW);
    uint8_t* stage_w = staging + warp * 4096;  // this warp's fp32 box
    long long g = 0;
    int j = 0;
    int xt = 0;  // HP split epilogue: exchanges of group maxima done by this warp
    bool ok = true;
    for (int t = blockIdx.x; t < n_tiles_total && ok; t += gridDim.x) {
      const TileCoord tc = tile_coord<BN, OP_IS_A>(p, t);
      const int field = tc.field, d = tc.d, row_a0 = tc.row_a0, row_b0 = tc.row_b0;
      float acc[CPW];
      // HP: low words of the two-float accumulators, in pairs (unused otherwise)
      __nv_bfloat162 lo[HP ? CPW / 2 : 1];
#pragma unroll
      for (int jj = 0; jj < CPW; ++jj) acc[jj] = 0.f;
#pragma unroll
      for (int jj = 0; jj < (HP ? CPW / 2 : 1); ++jj) lo[jj] = __floats2bfloat162_rn(0.f, 0.f);
      // a ragged tile beyond its slot: nothing computed; stage 2 stores zeros
      const bool beyond = tile_beyond<OP_IS_A>(p, tc);
      if (beyond && EPI == EPI_T_SPLIT) continue;
      for (int it = 0; it < (beyond ? 0 : k_iters); ++it, ++g) {
        const int ts = (int)(g % NSLOT);
        const uint32_t round = (uint32_t)((g / NSLOT) & 1);
        ok = mbar_wait(&tfull[ts], round, wb);
        ok = __all_sync(0xffffffffu, ok && !*abort_flag);
        if (!ok) break;
        tc_fence_after();
        if constexpr (HP)
          drain_add2<CPW>(t_rot + (uint32_t)(ts * BN) + lane_off, acc, lo);
        else
          drain_add<CPW>(t_rot + (uint32_t)(ts * BN) + lane_off, acc);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&tempty[ts]);
      }
      if (ok && !beyond) {
        // the tile's persistent slot is complete once its last commit lands
        ok = mbar_wait(gdone, (uint32_t)(j & 1), wb);
        ok = __all_sync(0xffffffffu, ok && !*abort_flag);
      }
      if (!ok) {
        atomicExch(p.status, 3);
        *abort_flag = 1;
        break;
      }
      if (!beyond) {
        // add the persistent slot of the smaller products, then hand it to
        // the next tile
        tc_fence_after();
        if constexpr (HP)
          drain_final2<CPW>(t_gs + lane_off, acc, lo);
        else
          drain_add<CPW>(t_gs + lane_off, acc);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(gfree);
        ++j;
      }
      if (EPI == EPI_T_SPLIT && HP) {
        // C[y][u] -> T^T parts [field][part][d][u][y] (bf16), split on the
        // grid of each column's 64-row group (quadrant pair q, q ^ 1): this
        // warp's per-column maxima go to shared memory, the pair meets at a
        // bounded barrier, and both take the larger of the two.
        uint32_t* xown =
            reinterpret_cast<uint32_t*>(staging) + ((xt & 1) * DRAIN_WARPS + warp) * CPW;
        const uint32_t* xpar = reinterpret_cast<const uint32_t*>(staging) +
                               ((xt & 1) * DRAIN_WARPS + (warp ^ 1)) * CPW;
#pragma unroll
        for (int jj = 0; jj < CPW; ++jj) {
          const uint32_t m = __reduce_max_sync(0xffffffffu, absbits(acc[jj]));
          if (lane == (jj & 31)) xown[jj] = m;
        }
        mbar_arrive(&pairbar[warp >> 1]);  // every lane of both warps (release)
        ok = mbar_wait(&pairbar[warp >> 1], (uint32_t)(xt & 1), wb);
        ok = __all_sync(0xffffffffu, ok && !*abort_flag);
        ++xt;
        if (!ok) {
          atomicExch(p.status, 4);
          *abort_flag = 1;
          break;
        }
        const int y = row_a0 + row;
        if ((p.out_cols & 1) == 0) {
          __nv_bfloat162* out = reinterpret_cast<__nv_bfloat162*>(p.out);
          const size_t plane2 = (size_t)p.out_rows * p.out_cols / 2;
          const int odd = lane & 1;
          const int ye = y - odd;
          const int u0 = row_b0 + h * CPW + odd;
#pragma unroll
          for (int jj = 0; jj < CPW; jj += 2) {
            const float recv = __shfl_xor_sync(0xffffffffu, odd ? acc[jj] : acc[jj + 1], 1);
            const float2 l = __bfloat1622float2(lo[jj / 2]);
            const float recvl = __shfl_xor_sync(0xffffffffu, odd ? l.x : l.y, 1);
            const float v0 = odd ? recv : acc[jj], w0 = odd ? recvl : l.x;
            const float v1 = odd ? acc[jj + 1] : recv, w1 = odd ? l.y : recvl;
            const int col = jj + odd;
            const Grid gr = grid_of(max(xown[col], xpar[col]));
            const int u = u0 + jj;
            if (ye < p.out_cols && u < p.cols_valid) {
              __nv_bfloat16 a0, a1, a2, b0, b1, b2;
              split3_aligned2(v0, w0, gr, a0, a1, a2);
              split3_aligned2(v1, w1, gr, b0, b1, b2);
              const size_t off = ((size_t)u * p.out_cols + ye) / 2;
              out[((size_t)(field * 3 + 0) * 2 + d) * plane2 + off] = __halves2bfloat162(a0, b0);
              out[((size_t)(field * 3 + 1) * 2 + d) * plane2 + off] = __halves2bfloat162(a1, b1);
              out[((size_t)(field * 3 + 2) * 2 + d) * plane2 + off] = __halves2bfloat162(a2, b2);
            }
          }
        } else if (y < p.out_cols) {
          __nv_bfloat16* out = reinterpret_cast<__nv_bfloat16*>(p.out);
          const size_t plane = (size_t)p.out_rows * p.out_cols;
          const int u0 = row_b0 + h * CPW;
#pragma unroll
          for (int jj = 0; jj < CPW; ++jj) {
            const int u = u0 + jj;
            if (u < p.cols_valid) {
              const Grid gr = grid_of(max(xown[jj], xpar[jj]));
              const float2 l = __bfloat1622float2(lo[jj / 2]);
              __nv_bfloat16 h0, h1, h2;
              split3_aligned2(acc[jj], (jj & 1) ? l.y : l.x, gr, h0, h1, h2);
              const size_t off = (size_t)u * p.out_cols + y;
              out[((size_t)(field * 3 + 0) * 2 + d) * plane + off] = h0;
              out[((size_t)(field * 3 + 1) * 2 + d) * plane + off] = h1;
              out[((size_t)(field * 3 + 2) * 2 + d) * plane + off] = h2;
            }
          }
        }
      } else if (EPI == EPI_T_SPLIT) {
        // C[y][u] -> T^T parts [field][part][d][u][y] (bf16)
        const int y = row_a0 + row;
        if ((p.out_cols & 1) == 0) {
          // Lane pairs (y, y + 1) swap one value per two columns, so each
          // lane holds both rows of one column and stores them as one bf16x2
          // word: the even lane column u0 + jj, the odd lane column
          // u0 + jj + 1. With an even row count y + 1 is in range whenever
          // the even y is.
          __nv_bfloat162* out = reinterpret_cast<__nv_bfloat162*>(p.out);
          const size_t plane2 = (size_t)p.out_rows * p.out_cols / 2;
          const int odd = lane & 1;
          const int ye = y - odd;
          const int u0 = row_b0 + h * CPW + odd;
#pragma unroll
          for (int jj = 0; jj < CPW; jj += 2) {
            const float send = odd ? acc[jj] : acc[jj + 1];
            const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
            const float lo = odd ? recv : acc[jj];
            const float hi = odd ? acc[jj + 1] : recv;
            const int u = u0 + jj;
            if (ye < p.out_cols && u < p.cols_valid) {
              __nv_bfloat16 a0, a1, a2, b0, b1, b2;
              split3(lo, a0, a1, a2);
              split3(hi, b0, b1, b2);
              const size_t off = ((size_t)u * p.out_cols + ye) / 2;
              out[((size_t)(field * 3 + 0) * 2 + d) * plane2 + off] = __halves2bfloat162(a0, b0);
              out[((size_t)(field * 3 + 1) * 2 + d) * plane2 + off] = __halves2bfloat162(a1, b1);
              out[((size_t)(field * 3 + 2) * 2 + d) * plane2 + off] = __halves2bfloat162(a2, b2);
            }
          }
        } else if (y < p.out_cols) {
          __nv_bfloat16* out = reinterpret_cast<__nv_bfloat16*>(p.out);
          const size_t plane = (size_t)p.out_rows * p.out_cols;
          const int u0 = row_b0 + h * CPW;
#pragma unroll
          for (int jj = 0; jj < CPW; ++jj) {
            const int u = u0 + jj;
            if (u < p.cols_valid) {
              __nv_bfloat16 h0, h1, h2;
              split3(acc[jj], h0, h1, h2);
              const size_t off = (size_t)u * p.out_cols + y;
              out[((size_t)(field * 3 + 0) * 2 + d) * plane + off] = h0;
              out[((size_t)(field * 3 + 1) * 2 + d) * plane + off] = h1;
              out[((size_t)(field * 3 + 2) * 2 + d) * plane + off] = h2;
            }
          }
        }
      }
      if (EPI == EPI_F32 && HP && p.out_lo) {
        // low words of the two-float results, per thread, beside `out`
        const int v = row_a0 + row;
        if (v < p.rows_valid) {
          float* out = p.out_lo +
                       ((size_t)(field * 2 + d) * p.out_plane_rows + p.out_r0 + v) * p.out_pitch +
                       p.out_c0;
          const int u0 = row_b0 + h * CPW;
#pragma unroll
          for (int jj = 0; jj < CPW; jj += 2) {
            const float2 l = __bfloat1622float2(lo[jj / 2]);
            if (u0 + jj < p.cols_valid) out[u0 + jj] = l.x;
            if (u0 + jj + 1 < p.cols_valid) out[u0 + jj + 1] = l.y;
          }
        }
      }
      if (EPI == EPI_T_SPLIT) {
      } else if (p.tma_out) {
        // Each warp stages its 32 x CPW block one 32 x 32 fp32 box at a time
        // in its own 4 KB of the staging region, in the TMA 128B-swizzled
        // layout (16-byte chunk c of row r at chunk c ^ (r & 7):
        // conflict-free), and one lane stores the box (or adds it into the
        // window), clipped to the window; the box is rewritten only after
        // the previous copy has read it.
#pragma unroll
        for (int b = 0; b < CPW / 32; ++b) {
          if (lane == 0) bulk_wait_read_all();
          __syncwarp();
          uint8_t* box = stage_w + lane * 128;
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            const float* a = acc + b * 32 + c * 4;
            *reinterpret_cast<float4*>(box + ((c ^ (lane & 7)) << 4)) =
                make_float4(a[0], a[1], a[2], a[3]);
          }
          fence_proxy_async_smem();
          __syncwarp();
          if (lane == 0) {
            const int u = row_b0 + h * CPW + b * 32;
            const int v0 = row_a0 + q * 32, z = field * 2 + d;
            if (p.accumulate)
              tma_reduce_add_3d(&tmO, stage_w, u, v0, z);
            else
              tma_store_3d(&tmO, stage_w, u, v0, z);
            bulk_commit();
          }
        }
      } else {
        // C[v][u] -> out fp32 [field][d][out_r0 + v][out_c0 + u] (pitch out_pitch)
        const int v = row_a0 + row;
        if (v < p.rows_valid) {
          float* out = reinterpret_cast<float*>(p.out) +
                       ((size_t)(field * 2 + d) * p.out_plane_rows + p.out_r0 + v) *
                           p.out_pitch +
                       p.out_c0;
          const int u0 = row_b0 + h * CPW;
          if (u0 + CPW <= p.cols_valid && ((p.out_pitch | p.out_c0) & 3) == 0) {
            float4* o4 = reinterpret_cast<float4*>(out + u0);
#pragma unroll
            for (int jj = 0; jj < CPW / 4; ++jj) {
              float4 val = make_float4(acc[4 * jj], acc[4 * jj + 1], acc[4 * jj + 2],
                                       acc[4 * jj + 3]);
              if (p.accumulate) {
                const float4 old = o4[jj];
                val.x += old.x; val.y += old.y; val.z += old.z; val.w += old.w;
              }
              o4[jj] = val;
            }
          } else {
#pragma unroll
            for (int jj = 0; jj < CPW; ++jj) {
              const int u = u0 + jj;
              if (u < p.cols_valid) {
                float val = acc[jj];
                if (p.accumulate) val += out[u];
                out[u] = val;
              }
            }
          }
        }
      }
    }
    // the staged boxes must be read before the CTA's shared memory goes
    if (EPI == EPI_F32 && lane == 0) bulk_wait_read_all();
    __syncwarp();
  }
  tc_fence_before();
  __syncthreads();
  // After a give-up (the flag is settled: every role has stopped), nothing
  // asynchronous may outlive the CTA: the MMA thread waits for the products
  // it issued (tensor memory is released next) and the producer for the
  // operand loads still in flight, which complete their stages' full
  // barriers when the bytes land (only the last STAGES loads can be pending:
  // each was issued after the one STAGES before it had been consumed).
  if (*abort_flag) {
    if (warp == MMA_WARP && lane == 0) {
      umma_commit(quiesce);
      mbar_wait(quiesce, 0);
    }
    if (warp == PRODUCER_WARP && lane == 0) {
      for (long long i = g_issued > STAGES ? g_issued - STAGES : 0; i < g_issued; ++i)
        mbar_wait(&full[(int)(i % STAGES)], (uint32_t)((i / STAGES) & 1));
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
