// Matrix Fourier transform (the reference's zoomFft / chirp-Z zoom) on
// tcgen05 tensor cores.
//
//   out = pref * A_y . in . B_x^T,  A_y[v][y] = e^{sgn 2 pi i yin_y yout_v / lf},
//                                  B_x[u][x] = e^{sgn 2 pi i xin_x xout_u / lf}
//
// Stage 1 contracts x: T[y][u] = sum_x in[y][x] B_x[u][x]; the epilogue writes
// T transposed and already split into three bf16 parts.
// Stage 2 contracts y: out[v][u] = sum_y (pref A_y)[v][y] T^T[u][y] in fp32.
// Operators are generated once per plan in FP64 (phase reduced in turns) and
// stored split as [slot][part][sel: re, im, -im][rows][K] bf16.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>
#include <vector>

#include "ctx.hpp"
#include "pixops.cuh"
#include "tc_gemm.cuh"

namespace csg {

// ------------------------------------------------------------ tensor maps
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

static int get_encoder() {
  static std::once_flag once;
  static int rc = CSG_OK;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
      rc = CSG_E_CUDA;
    } else {
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
  });
  if (rc != CSG_OK) set_error("cuTensorMapEncodeTiled entry point unavailable");
  return rc;
}

// 3-D bf16 map: (k inner, rows, planes), box (box_k, box_rows, 1), with the
// swizzle of a box_k-wide row: 128 bytes (64 elements) or 64 bytes (32).
int make_map_k(CUtensorMap* m, const void* base, int k, int rows, long long planes,
               int box_rows, int box_k) {
  int rc = get_encoder();
  if (rc) return rc;
  CSG_CHECK(((uintptr_t)base & 15) == 0, CSG_E_ARG, "TMA base not 16-byte aligned");
  CSG_CHECK((k % 8) == 0, CSG_E_SHAPE, "TMA inner extent must be a multiple of 8 elements");
  CSG_CHECK(box_k == 64 || box_k == 32, CSG_E_ARG, "TMA box K must be 64 or 32");
  cuuint64_t dims[3] = {(cuuint64_t)k, (cuuint64_t)rows, (cuuint64_t)planes};
  cuuint64_t strides[2] = {(cuuint64_t)k * 2, (cuuint64_t)k * 2 * rows};
  cuuint32_t box[3] = {(cuuint32_t)box_k, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        box_k == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  CSG_CHECK(r == CUDA_SUCCESS, CSG_E_CUDA,
            "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return CSG_OK;
}

// The same with 64-wide K boxes (128B swizzle).
int make_map(CUtensorMap* m, const void* base, int k, int rows, long long planes,
             int box_rows) {
  return make_map_k(m, base, k, rows, planes, box_rows, tc::BK);
}

// 3-D fp32 map of an output window for the GEMM epilogue: (cols, rows,
// planes) with origin base, row pitch `pitch` and plane stride
// plane_rows * pitch elements; box (32, 32, 1), 128B swizzle. Returns false
// (and leaves m unused) when the window breaks a TMA rule: the origin must
// be 16-byte aligned and the pitch a multiple of 4 elements.
bool make_map_f32_out(CUtensorMap* m, float* base, int cols, int rows, long long planes,
                      int pitch, int plane_rows) {
  if (get_encoder() != CSG_OK) return false;
  if (((uintptr_t)base & 15) != 0 || (pitch & 3) != 0 || cols <= 0 || rows <= 0) return false;
  cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, (cuuint64_t)planes};
  cuuint64_t strides[2] = {(cuuint64_t)pitch * 4, (cuuint64_t)pitch * 4 * plane_rows};
  cuuint32_t box[3] = {32, 32, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// ------------------------------------------------------------ kernels
// Operator generator: op[slot][part][sel][r][k] for r < rows, k < K.
// value = pref_s * exp(sgn 2 pi i frac(cout_r cin_k / lf_s)); sel 0/1/2 = re/im/-im.
// Ragged plans: slot s reads its output coordinates at cout + s * cstride
// and its rows r >= valid[s] are zero.
__global__ void k_build_operator(__nv_bfloat16* __restrict__ op, const double* __restrict__ cout,
                                 const double* __restrict__ cin, int rows, int K, int n_slots,
                                 const double* __restrict__ lf, const double* __restrict__ pref,
                                 double sgn, int cstride, const int* __restrict__ valid) {
  const long long n = (long long)n_slots * rows * K;
  const long long plane = (long long)rows * K;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i % K);
    const long long t = i / K;
    const int r = (int)(t % rows);
    const int s = (int)(t / rows);
    double turns = cout[(long long)s * cstride + r] * cin[k] / lf[s];
    turns -= rint(turns);  // exact in FP64 for |turns| < 2^52
    double sn, cs;
    sincospi(2.0 * sgn * turns, &sn, &cs);
    double pr = 1.0, pi = 0.0;
    if (pref) {
      pr = pref[2 * s];
      pi = pref[2 * s + 1];
    }
    if (valid && r >= valid[s]) pr = pi = 0.0;
    const double re = pr * cs - pi * sn;
    const double im = pr * sn + pi * cs;
    __nv_bfloat16 a0, a1, a2, b0, b1, b2;
    split3((float)re, a0, a1, a2);
    split3((float)im, b0, b1, b2);
    const long long off = (long long)r * K + k;
    const __nv_bfloat16 pre[3] = {a0, a1, a2};
    const __nv_bfloat16 pim[3] = {b0, b1, b2};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      __nv_bfloat16* base = op + ((long long)(s * 3 + q) * 3) * plane + off;
      base[0] = pre[q];
      base[plane] = pim[q];
      base[2 * plane] = __hneg(pim[q]);
    }
  }
}

// The operator of CSG_PREC_HIGH: the same values, split on one grid per
// 64-wide K group of each row and plane (split3_aligned). One warp per
// (slot, row, group); lane l computes elements 64 g + l and 64 g + 32 + l.
__global__ void k_build_operator_aligned(__nv_bfloat16* __restrict__ op,
                                         const double* __restrict__ cout,
                                         const double* __restrict__ cin, int rows, int K,
                                         int n_slots, const double* __restrict__ lf,
                                         const double* __restrict__ pref, double sgn, int cstride,
                                         const int* __restrict__ valid) {
  const int groups = (K + 63) / 64;
  const long long nw = (long long)n_slots * rows * groups;
  const long long plane = (long long)rows * K;
  const int lane = threadIdx.x & 31;
  for (long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nw;
       w += ((long long)gridDim.x * blockDim.x) >> 5) {
    const int gi = (int)(w % groups);
    const long long t = w / groups;
    const int r = (int)(t % rows);
    const int s = (int)(t / rows);
    float vre[2], vim[2];
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const int k = gi * 64 + hh * 32 + lane;
      vre[hh] = vim[hh] = 0.f;
      if (k < K) {
        double turns = cout[(long long)s * cstride + r] * cin[k] / lf[s];
        turns -= rint(turns);
        double sn, cs;
        sincospi(2.0 * sgn * turns, &sn, &cs);
        double pr = 1.0, pi = 0.0;
        if (pref) {
          pr = pref[2 * s];
          pi = pref[2 * s + 1];
        }
        if (valid && r >= valid[s]) pr = pi = 0.0;
        vre[hh] = (float)(pr * cs - pi * sn);
        vim[hh] = (float)(pr * sn + pi * cs);
      }
    }
    const Grid gre = grid_of(__reduce_max_sync(0xffffffffu, max(absbits(vre[0]), absbits(vre[1]))));
    const Grid gim = grid_of(__reduce_max_sync(0xffffffffu, max(absbits(vim[0]), absbits(vim[1]))));
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const int k = gi * 64 + hh * 32 + lane;
      if (k >= K) continue;
      __nv_bfloat16 pre[3], pim[3];
      split3_aligned(vre[hh], gre, pre[0], pre[1], pre[2]);
      split3_aligned(vim[hh], gim, pim[0], pim[1], pim[2]);
      const long long off = (long long)r * K + k;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        __nv_bfloat16* base = op + ((long long)(s * 3 + q) * 3) * plane + off;
        base[0] = pre[q];
        base[plane] = pim[q];
        base[2 * plane] = __hneg(pim[q]);
      }
    }
  }
}

// Data split: planar fp32 [F][2][R][C] -> (element ops `pre`) -> (times a
// complex multiplier [n_mul][2][R][C] chosen by mul_idx[f]) -> bf16
// [F][3][2][R][C]. Eight pixels of one row per thread (C is a multiple of
// 8); grid.y is the field; field f reads input field in_idx[f] (f when
// in_idx is null). The input is the R x C window at (r0, c0) of fields whose
// planes are RT x PT (the element ops see the field's own coordinates and
// size). The parts come from paired bf16 conversions (split3_pair, two
// values per instruction), bit-identical to split3.
__global__ void k_split_field(const float* __restrict__ in, __nv_bfloat16* __restrict__ out, int R,
                              int C, int r0, int c0, int RT, int PT,
                              const float* __restrict__ mul,
                              const int* __restrict__ mul_idx,
                              const __grid_constant__ PixOps pre, const __grid_constant__ FieldInfo fi,
                              const int* __restrict__ in_idx) {
  __shared__ PixConsts shk;
  const int f = blockIdx.y;
  const int plane = R * C;
  const size_t fplane = (size_t)RT * PT;
  PixConsts k;
  if (pre.n) pix_consts_cta(pre, fi, f, RT, PT, k, &shk);
  const float* ire = in + (size_t)(in_idx ? in_idx[f] : f) * 2 * fplane;
  const float* iim = ire + fplane;
  const float* mre = mul ? mul + (size_t)mul_idx[f] * 2 * plane : nullptr;
  const int groups = C / 8;
  const int ng = R * groups;
  for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ng; gi += gridDim.x * blockDim.x) {
    const int r = gi / groups, c = (gi - r * groups) * 8;
    const size_t g = (size_t)(r0 + r) * PT + c0 + c;  // 16-byte aligned: c0, C, PT % 4 == 0
    float xr[8], xi[8];
    {
      const float4 a0 = *reinterpret_cast<const float4*>(ire + g);
      const float4 a1 = *reinterpret_cast<const float4*>(ire + g + 4);
      const float4 b0 = *reinterpret_cast<const float4*>(iim + g);
      const float4 b1 = *reinterpret_cast<const float4*>(iim + g + 4);
      xr[0] = a0.x, xr[1] = a0.y, xr[2] = a0.z, xr[3] = a0.w;
      xr[4] = a1.x, xr[5] = a1.y, xr[6] = a1.z, xr[7] = a1.w;
      xi[0] = b0.x, xi[1] = b0.y, xi[2] = b0.z, xi[3] = b0.w;
      xi[4] = b1.x, xi[5] = b1.y, xi[6] = b1.z, xi[7] = b1.w;
    }
    if (pre.n) pix_apply_n<8>(pre, k, r0 + r, c0 + c, 0, 1, RT, PT, xr, xi);
    const int e0 = r * C + c;
    if (mre) {
      float mr[8], mi[8];
      const float4* m4 = reinterpret_cast<const float4*>(mre + e0);
      const float4* n4 = reinterpret_cast<const float4*>(mre + plane + e0);
      const float4 m0 = m4[0], m1 = m4[1], q0 = n4[0], q1 = n4[1];
      mr[0] = m0.x, mr[1] = m0.y, mr[2] = m0.z, mr[3] = m0.w;
      mr[4] = m1.x, mr[5] = m1.y, mr[6] = m1.z, mr[7] = m1.w;
      mi[0] = q0.x, mi[1] = q0.y, mi[2] = q0.z, mi[3] = q0.w;
      mi[4] = q1.x, mi[5] = q1.y, mi[6] = q1.z, mi[7] = q1.w;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float tr = xr[q] * mr[q] - xi[q] * mi[q];
        xi[q] = xr[q] * mi[q] + xi[q] * mr[q];
        xr[q] = tr;
      }
    }
    uint32_t hr[3][4], hi[3][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      split3_pair(xr[2 * q], xr[2 * q + 1], hr[0][q], hr[1][q], hr[2][q]);
      split3_pair(xi[2 * q], xi[2 * q + 1], hi[0][q], hi[1][q], hi[2][q]);
    }
#pragma unroll
    for (int p = 0; p < 3; ++p) {
      __nv_bfloat16* o = out + ((size_t)(f * 3 + p) * 2) * plane + e0;
      *reinterpret_cast<uint4*>(o) = make_uint4(hr[p][0], hr[p][1], hr[p][2], hr[p][3]);
      *reinterpret_cast<uint4*>(o + plane) = make_uint4(hi[p][0], hi[p][1], hi[p][2], hi[p][3]);
    }
  }
}

// The data split of CSG_PREC_HIGH: as k_split_field, with every 64-column
// group of a row split on one grid (split3_aligned). One warp per (row,
// 256-column chunk): lane l holds columns 8 l .. 8 l + 7 of the chunk, so
// the eight lanes 8 m .. 8 m + 7 hold one group and exchange their maxima.
__global__ void k_split_field_aligned(const float* __restrict__ in,
                                      __nv_bfloat16* __restrict__ out, int R, int C, int r0,
                                      int c0, int RT, int PT, const float* __restrict__ mul,
                                      const int* __restrict__ mul_idx,
                                      const __grid_constant__ PixOps pre,
                                      const __grid_constant__ FieldInfo fi,
                                      const int* __restrict__ in_idx) {
  __shared__ PixConsts shk;
  const int f = blockIdx.y;
  const int plane = R * C;
  const size_t fplane = (size_t)RT * PT;
  PixConsts k;
  if (pre.n) pix_consts_cta(pre, fi, f, RT, PT, k, &shk);
  const float* ire = in + (size_t)(in_idx ? in_idx[f] : f) * 2 * fplane;
  const float* iim = ire + fplane;
  const float* mre = mul ? mul + (size_t)mul_idx[f] * 2 * plane : nullptr;
  const int chunks = (C + 255) / 256;
  const int nw = R * chunks;
  const int lane = threadIdx.x & 31;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nw;
       w += (gridDim.x * blockDim.x) >> 5) {
    const int r = w / chunks, c = (w - r * chunks) * 256 + lane * 8;
    const bool act = c < C;  // C is a multiple of 8
    float xr[8], xi[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) xr[q] = xi[q] = 0.f;
    const size_t g = (size_t)(r0 + r) * PT + c0 + c;
    const int e0 = r * C + c;
    if (act) {
      const float4 a0 = *reinterpret_cast<const float4*>(ire + g);
      const float4 a1 = *reinterpret_cast<const float4*>(ire + g + 4);
      const float4 b0 = *reinterpret_cast<const float4*>(iim + g);
      const float4 b1 = *reinterpret_cast<const float4*>(iim + g + 4);
      xr[0] = a0.x, xr[1] = a0.y, xr[2] = a0.z, xr[3] = a0.w;
      xr[4] = a1.x, xr[5] = a1.y, xr[6] = a1.z, xr[7] = a1.w;
      xi[0] = b0.x, xi[1] = b0.y, xi[2] = b0.z, xi[3] = b0.w;
      xi[4] = b1.x, xi[5] = b1.y, xi[6] = b1.z, xi[7] = b1.w;
      if (pre.n) pix_apply_n<8>(pre, k, r0 + r, c0 + c, 0, 1, RT, PT, xr, xi);
      if (mre) {
        const float4* m4 = reinterpret_cast<const float4*>(mre + e0);
        const float4* n4 = reinterpret_cast<const float4*>(mre + plane + e0);
        const float4 m0 = m4[0], m1 = m4[1], q0 = n4[0], q1 = n4[1];
        const float mr[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
        const float mi[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const float tr = xr[q] * mr[q] - xi[q] * mi[q];
          xi[q] = xr[q] * mi[q] + xi[q] * mr[q];
          xr[q] = tr;
        }
      }
    }
    uint32_t br = 0, bi = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      br = max(br, absbits(xr[q]));
      bi = max(bi, absbits(xi[q]));
    }
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      br = max(br, __shfl_xor_sync(0xffffffffu, br, o));
      bi = max(bi, __shfl_xor_sync(0xffffffffu, bi, o));
    }
    if (!act) continue;
    const Grid gre = grid_of(br), gim = grid_of(bi);
    uint32_t hr[3][4], hi[3][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      split3_aligned_pair(xr[2 * q], xr[2 * q + 1], gre, hr[0][q], hr[1][q], hr[2][q]);
      split3_aligned_pair(xi[2 * q], xi[2 * q + 1], gim, hi[0][q], hi[1][q], hi[2][q]);
    }
#pragma unroll
    for (int p = 0; p < 3; ++p) {
      __nv_bfloat16* o = out + ((size_t)(f * 3 + p) * 2) * plane + e0;
      *reinterpret_cast<uint4*>(o) = make_uint4(hr[p][0], hr[p][1], hr[p][2], hr[p][3]);
      *reinterpret_cast<uint4*>(o + plane) = make_uint4(hi[p][0], hi[p][1], hi[p][2], hi[p][3]);
    }
  }
}

// L2 prefetch distance of the GEMM's field operand, in K blocks (tuning
// override CSG_GEMM_PREFETCH, 0 to 16; default 0: off).
static int gemm_prefetch() {
  static const int pf = [] {
    const char* e = getenv("CSG_GEMM_PREFETCH");
    const int v = e ? atoi(e) : 0;
    return v < 0 ? 0 : (v > 16 ? 16 : v);
  }();
  return pf;
}

// The GEMM issues a prefix of its fixed product order (tc::term_a, tc::term_b):
// all six products for bf16x6, the three largest for bf16x3.
void terms_for(int precision, tc::Params& p) {
  p.n_terms = precision == CSG_PREC_BF16X3 ? 3 : 6;
}

template <int BN, bool OP_IS_A, int EPI, bool HP = false, int KB = 0>
static int launch_gemm(const CUtensorMap& a, const CUtensorMap& b, const tc::Params& p,
                       int grid, cudaStream_t st, const CUtensorMap* o = nullptr) {
  auto kern = tc::k_split_gemm<BN, OP_IS_A, EPI, HP, KB>;
  constexpr size_t smem = tc::smem_bytes<BN, EPI, HP, KB>();
  static bool attr_set = false;  // per template instance
  if (!attr_set) {
    CSG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  CSG_CHECK(o || !p.tma_out, CSG_E_ARG, "GEMM: TMA output without a tensor map");
  static const CUtensorMap unused{};  // read only when p.tma_out
  // persistent CTAs, one per SM (the kernel walks tiles with a grid stride)
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    CSG_CUDA(cudaGetDevice(&dev));
    CSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  kern<<<std::min(grid, sms), tc::THREADS, smem, st>>>(a, b, o ? *o : unused, p);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

// Data (A, rows of the fields) x operator (B) with an fp32 output
// [field][re/im][rows][cols]: the response-matrix objective's product.
int launch_gemm_data_op_f32(int bn, const CUtensorMap& a, const CUtensorMap& b,
                            const tc::Params& p, int grid, cudaStream_t st) {
  return bn == 64 ? launch_gemm<64, false, tc::EPI_F32>(a, b, p, grid, st)
                  : launch_gemm<128, false, tc::EPI_F32>(a, b, p, grid, st);
}

}  // namespace csg

using namespace csg;

struct csg_mft {
  csg_ctx* ctx = nullptr;
  int ny = 0, nx = 0, mo = 0, no = 0, n_slots = 0, precision = 6;
  __nv_bfloat16* op1 = nullptr;  // [slot][3][3][no][nx]
  __nv_bfloat16* op2 = nullptr;  // [slot][3][3][mo][ny]
  Scratch split_in;               // [F][3][2][ny][nx] bf16
  Scratch tt;                     // [F][3][2][no][ny] bf16
  int* valid = nullptr;           // ragged plans: outputs per slot (device)
  int bn = 0;                     // tile width chosen by the autotuner (0: default)
  int tuned_fields = 0;           // batch size the choice was measured at (-1: fixed)
  float tuned_ms[3] = {0, 0, 0};  // measured time of BN = 128, 64, 256 (0: not tried)
};

namespace {
std::string g_tune_log;

// Tile autotuner: times the transform with N-tile widths 128 and 64 at the
// batch size it will run at (zero input, every field on slot 0) and keeps the
// faster. Runs outside graph capture (csg_mft_reserve is called before).
int autotune(csg_mft* m, int F) {
  if (m->tuned_fields == F || m->tuned_fields == -1) return CSG_OK;
  const char* env = getenv("CSG_MFT_AUTOTUNE");
  if (env && env[0] == '0') {
    m->bn = 0;
    m->tuned_fields = F;
    return CSG_OK;
  }
  cudaStream_t st = m->ctx->stream;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cs);
  if (cs != cudaStreamCaptureStatusNone) return CSG_OK;
  float *in = nullptr, *out = nullptr;
  int* slot = nullptr;
  const size_t in_b = (size_t)F * 2 * m->ny * m->nx * 4, out_b = (size_t)F * 2 * m->mo * m->no * 4;
  if (cudaMalloc(&in, in_b) != cudaSuccess || cudaMalloc(&out, out_b) != cudaSuccess ||
      cudaMalloc(&slot, (size_t)F * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(in);
    cudaFree(out);
    cudaFree(slot);
    return CSG_OK;  // keep the default tile on allocation pressure
  }
  cudaMemsetAsync(in, 0, in_b, st);
  cudaMemsetAsync(slot, 0, (size_t)F * sizeof(int), st);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int cand[3] = {128, 64, 256};
  float best = 1e30f;
  int best_bn = 0, rc = CSG_OK;
  const bool prof = m->ctx->prof;
  m->ctx->prof = false;
  // 256-wide tiles only where the output is at least that wide per component
  const int n_cand = m->no >= 256 && m->precision != CSG_PREC_HIGH ? 3 : 2;
  m->tuned_ms[2] = 0;
  for (int i = 0; i < n_cand && !rc; ++i) {
    m->bn = cand[i];
    rc = mft_execute_ops(m->ctx, m, in, out, F, slot, 0, nullptr, nullptr, PixOps(), FieldInfo());
    cudaEventRecord(a, st);
    for (int r = 0; r < 2 && !rc; ++r)
      rc = mft_execute_ops(m->ctx, m, in, out, F, slot, 0, nullptr, nullptr, PixOps(),
                           FieldInfo());
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    m->tuned_ms[i] = ms / 2;
    if (ms < best) {
      best = ms;
      best_bn = cand[i];
    }
  }
  m->ctx->prof = prof;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(in);
  cudaFree(out);
  cudaFree(slot);
  m->bn = best_bn;
  m->tuned_fields = F;
  char line[200];
  snprintf(line, sizeof(line), "%s{\"in\": [%d, %d], \"out\": [%d, %d], \"fields\": %d, "
           "\"bn\": %d, \"ms_bn128\": %.4f, \"ms_bn64\": %.4f, \"ms_bn256\": %.4f}",
           g_tune_log.empty() ? "" : ", ", m->ny, m->nx, m->mo, m->no, F, best_bn,
           m->tuned_ms[0], m->tuned_ms[1], m->tuned_ms[2]);
  g_tune_log += line;
  return rc;
}
}  // namespace

// JSON list of every autotuning decision made in this process.
extern "C" int csg_mft_tuning_log(char* buf, size_t len) {
  CSG_CHECK(buf && len > 0, CSG_E_ARG, "csg_mft_tuning_log: bad buffer");
  const std::string s = "[" + g_tune_log + "]";
  CSG_CHECK(s.size() + 1 <= len, CSG_E_ARG, "csg_mft_tuning_log: buffer too small");
  memcpy(buf, s.c_str(), s.size() + 1);
  return CSG_OK;
}

extern "C" {

// Shared body of csg_mft_create and csg_mft_create_ragged: with n_out
// non-null, slot s has its own n_out[s] output coordinates at yout/xout +
// s * n_out_y (n_out_y = n_out_x = the largest size).
static int create_plan(csg_ctx* ctx, csg_mft** plan, int n_in_y, int n_in_x, int n_out_y,
                       int n_out_x, const double* yin, const double* xin, const double* yout,
                       const double* xout, int n_slots, const double* lf, const double* pref,
                       double sgn, int precision, const int* n_out) {
  CSG_CHECK(ctx && plan && yin && xin && yout && xout && lf, CSG_E_ARG,
            "csg_mft_create: null argument");
  CSG_CHECK(n_in_y > 0 && n_in_x > 0 && n_out_y > 0 && n_out_x > 0 && n_slots > 0, CSG_E_SHAPE,
            "csg_mft_create: non-positive size");
  CSG_CHECK(n_in_x % 8 == 0 && n_in_y % 8 == 0, CSG_E_SHAPE,
            "csg_mft_create: input sizes must be multiples of 8");
  CSG_CHECK(precision == CSG_PREC_BF16X6 || precision == CSG_PREC_BF16X3 ||
                precision == CSG_PREC_HIGH,
            CSG_E_ARG,
            "csg_mft_create: precision must be CSG_PREC_BF16X6, CSG_PREC_BF16X3 or CSG_PREC_HIGH");
  for (int s = 0; s < n_slots; ++s)
    CSG_CHECK(lf[s] != 0.0, CSG_E_ARG, "csg_mft_create: zero lambda*f");
  {
    const int rs = n_out ? n_slots : 1;
    CSG_CHECK(all_finite(yin, n_in_y) && all_finite(xin, n_in_x) &&
                  all_finite(yout, (size_t)rs * n_out_y) && all_finite(xout, (size_t)rs * n_out_x) &&
                  all_finite(lf, n_slots) && (!pref || all_finite(pref, 2 * (size_t)n_slots)),
              CSG_E_NAN, "csg_mft_create: non-finite coordinate, lambda*f or prefactor");
  }
  DeviceGuard g(ctx->device);
  csg_mft* m = new csg_mft();
  m->ctx = ctx;
  m->ny = n_in_y;
  m->nx = n_in_x;
  m->mo = n_out_y;
  m->no = n_out_x;
  m->n_slots = n_slots;
  m->precision = precision;
  const size_t op1_elems = (size_t)n_slots * 9 * n_out_x * n_in_x;
  const size_t op2_elems = (size_t)n_slots * 9 * n_out_y * n_in_y;
  double* dvec = nullptr;
  const int rs = n_out ? n_slots : 1;  // output coordinate sets
  const size_t nvec = (size_t)n_in_y + n_in_x + (size_t)rs * (n_out_y + n_out_x) + 3 * n_slots +
                      (n_out ? (n_slots + 1) / 2 : 0);
  if (cudaMalloc(&m->op1, op1_elems * 2) != cudaSuccess ||
      cudaMalloc(&m->op2, op2_elems * 2) != cudaSuccess ||
      cudaMalloc(&dvec, nvec * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(m->op1);
    cudaFree(m->op2);
    cudaFree(dvec);
    delete m;
    set_error("csg_mft_create: operator allocation failed");
    return CSG_E_NOMEM;
  }
  std::vector<double> h(nvec, 0.0);
  size_t o = 0;
  const size_t o_yin = o; for (int i = 0; i < n_in_y; ++i) h[o++] = yin[i];
  const size_t o_xin = o; for (int i = 0; i < n_in_x; ++i) h[o++] = xin[i];
  const size_t o_yout = o; for (size_t i = 0; i < (size_t)rs * n_out_y; ++i) h[o++] = yout[i];
  const size_t o_xout = o; for (size_t i = 0; i < (size_t)rs * n_out_x; ++i) h[o++] = xout[i];
  const size_t o_lf = o; for (int i = 0; i < n_slots; ++i) h[o++] = lf[i];
  const size_t o_pref = o;
  for (int i = 0; i < n_slots; ++i) {
    h[o++] = pref ? pref[2 * i] : 1.0;
    h[o++] = pref ? pref[2 * i + 1] : 0.0;
  }
  const size_t o_valid = o;  // int32 per slot, packed into the FP64 vector
  if (n_out) memcpy(&h[o_valid], n_out, sizeof(int) * n_slots);
  const int* valid = n_out ? reinterpret_cast<const int*>(dvec + o_valid) : nullptr;
  cudaStream_t st = ctx->stream;
  CSG_CUDA(cudaMemcpyAsync(dvec, h.data(), nvec * sizeof(double), cudaMemcpyHostToDevice, st));
  // stage-1 operator: rows u (xout), K = x (xin), no prefactor;
  // stage-2 operator: rows v (yout), K = y (yin), carries the prefactor
  if (precision == CSG_PREC_HIGH) {
    k_build_operator_aligned<<<grid_for((long long)n_slots * n_out_x * ((n_in_x + 63) / 64), 8),
                               256, 0, st>>>(m->op1, dvec + o_xout, dvec + o_xin, n_out_x,
                                             n_in_x, n_slots, dvec + o_lf, nullptr, sgn,
                                             n_out ? n_out_x : 0, valid);
    CSG_LAUNCH_CHECK();
    k_build_operator_aligned<<<grid_for((long long)n_slots * n_out_y * ((n_in_y + 63) / 64), 8),
                               256, 0, st>>>(m->op2, dvec + o_yout, dvec + o_yin, n_out_y,
                                             n_in_y, n_slots, dvec + o_lf, dvec + o_pref, sgn,
                                             n_out ? n_out_y : 0, valid);
    CSG_LAUNCH_CHECK();
  } else {
    k_build_operator<<<grid_for((long long)n_slots * n_out_x * n_in_x, 256), 256, 0, st>>>(
        m->op1, dvec + o_xout, dvec + o_xin, n_out_x, n_in_x, n_slots, dvec + o_lf, nullptr, sgn,
        n_out ? n_out_x : 0, valid);
    CSG_LAUNCH_CHECK();
    k_build_operator<<<grid_for((long long)n_slots * n_out_y * n_in_y, 256), 256, 0, st>>>(
        m->op2, dvec + o_yout, dvec + o_yin, n_out_y, n_in_y, n_slots, dvec + o_lf,
        dvec + o_pref, sgn, n_out ? n_out_y : 0, valid);
    CSG_LAUNCH_CHECK();
  }
  CSG_CUDA(cudaStreamSynchronize(st));
  cudaFree(dvec);
  if (n_out) {  // per-slot output extents, for skipping the all-zero tiles
    if (cudaMalloc(&m->valid, sizeof(int) * n_slots) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(m->op1);
      cudaFree(m->op2);
      delete m;
      set_error("csg_mft_create: allocation failed");
      return CSG_E_NOMEM;
    }
    CSG_CUDA(cudaMemcpy(m->valid, n_out, sizeof(int) * n_slots, cudaMemcpyHostToDevice));
  }
  *plan = m;
  return CSG_OK;
}

int csg_mft_create(csg_ctx* ctx, csg_mft** plan, int n_in_y, int n_in_x, int n_out_y,
                   int n_out_x, const double* yin, const double* xin, const double* yout,
                   const double* xout, int n_slots, const double* lf, const double* pref,
                   double sgn, int precision) {
  return create_plan(ctx, plan, n_in_y, n_in_x, n_out_y, n_out_x, yin, xin, yout, xout, n_slots,
                     lf, pref, sgn, precision, nullptr);
}

// Ragged batch (one plan, one launch, fields of every size): slot s maps to
// an n_out[s] x n_out[s] grid at yout/xout[s][0 .. n_out[s]); outputs are
// n_out_max^2 planes whose leading n_out[s] rows and columns hold the slot's
// transform and the rest is zero.
int csg_mft_create_ragged(csg_ctx* ctx, csg_mft** plan, int n_in_y, int n_in_x, int n_out_max,
                          const int* n_out, const double* yin, const double* xin,
                          const double* yout, const double* xout, int n_slots, const double* lf,
                          const double* pref, double sgn, int precision) {
  CSG_CHECK(n_out && n_slots > 0, CSG_E_ARG, "csg_mft_create_ragged: null n_out");
  for (int s = 0; s < n_slots; ++s)
    CSG_CHECK(n_out[s] > 0 && n_out[s] <= n_out_max, CSG_E_SHAPE,
              "csg_mft_create_ragged: n_out[s] must be in [1, n_out_max]");
  return create_plan(ctx, plan, n_in_y, n_in_x, n_out_max, n_out_max, yin, xin, yout, xout,
                     n_slots, lf, pref, sgn, precision, n_out);
}

int csg_mft_destroy(csg_mft* m) {
  if (!m) return CSG_OK;
  DeviceGuard g(m->ctx->device);
  cudaStreamSynchronize(m->ctx->stream);
  cudaFree(m->op1);
  cudaFree(m->op2);
  cudaFree(m->valid);
  m->split_in.release();
  m->tt.release();
  delete m;
  return CSG_OK;
}

int csg_mft_reserve(csg_mft* m, int n_fields) {
  CSG_CHECK(m && n_fields > 0, CSG_E_ARG, "csg_mft_reserve: bad argument");
  DeviceGuard g(m->ctx->device);
  int rc = m->split_in.ensure((size_t)n_fields * 12 * m->ny * m->nx);
  if (!rc) rc = m->tt.ensure((size_t)n_fields * 12 * m->no * m->ny);
  if (!rc) rc = autotune(m, n_fields);
  return rc;
}

int csg_mft_set_tile(csg_mft* m, int bn) {
  CSG_CHECK(m, CSG_E_ARG, "csg_mft_set_tile: null plan");
  CSG_CHECK(bn == 0 || bn == 64 || bn == 128 || bn == 256, CSG_E_ARG,
            "csg_mft_set_tile: width must be 0, 64, 128 or 256");
  CSG_CHECK(bn != 256 || m->no >= 256, CSG_E_ARG,
            "csg_mft_set_tile: 256-wide tiles need at least 256 output columns");
  CSG_CHECK(bn != 256 || m->precision != CSG_PREC_HIGH, CSG_E_ARG,
            "csg_mft_set_tile: CSG_PREC_HIGH runs 64- or 128-wide tiles");
  m->bn = bn;
  m->tuned_fields = bn ? -1 : 0;  // -1: fixed by the caller, never retuned
  return CSG_OK;
}

// Tile width the autotuner chose for the last reserved batch size and the
// times it measured (ms per transform for widths 128 and 256).
int csg_mft_tuning(csg_mft* m, int* bn, float* ms128, float* ms64) {
  CSG_CHECK(m && bn, CSG_E_ARG, "csg_mft_tuning: null argument");
  *bn = m->bn;
  if (ms128) *ms128 = m->tuned_ms[0];
  if (ms64) *ms64 = m->tuned_ms[1];
  return CSG_OK;
}

size_t csg_mft_workspace_bytes(csg_mft* m, int n_fields) {
  if (!m) return 0;
  return (size_t)n_fields * 12 * ((size_t)m->ny * m->nx + (size_t)m->no * m->ny);
}

}  // extern "C"

// MFT with element ops applied to the input pixels in the operand split
// (the chain executor fuses the elements before a transform here).
int csg::mft_execute_ops(csg_ctx* ctx, csg_mft* m, const float* in, float* out, int n_fields,
                         const int* slot, int accumulate, const float* in_mul, const int* mul_idx,
                         const PixOps& pre, const FieldInfo& fi, const MftWindow* iw,
                         const MftWindow* ow, const int* in_idx, bool presplit,
                         float* out_lo) {
  CSG_CHECK(ctx && m && in && out && slot, CSG_E_ARG, "csg_mft_execute: null argument");
  CSG_CHECK(n_fields > 0, CSG_E_SHAPE, "csg_mft_execute: n_fields must be positive");
  CSG_CHECK(!in_mul || mul_idx, CSG_E_ARG, "csg_mft_execute: in_mul needs mul_idx");
  const MftWindow inw = iw ? *iw : MftWindow{0, 0, m->ny, m->nx};
  const MftWindow outw = ow ? *ow : MftWindow{0, 0, m->mo, m->no};
  CSG_CHECK(inw.r0 >= 0 && inw.c0 >= 0 && inw.r0 + m->ny <= inw.rows && inw.c0 + m->nx <= inw.pitch &&
                ((inw.c0 | inw.pitch) & 3) == 0,
            CSG_E_SHAPE, "csg_mft_execute: input window outside the field or misaligned");
  CSG_CHECK(outw.r0 >= 0 && outw.c0 >= 0 && outw.r0 + m->mo <= outw.rows &&
                outw.c0 + m->no <= outw.pitch,
            CSG_E_SHAPE, "csg_mft_execute: output window outside the field");
  DeviceGuard g(ctx->device);
  cudaStream_t st = ctx->stream;
  int rc;
  if ((rc = m->split_in.ensure((size_t)n_fields * 12 * m->ny * m->nx))) return rc;
  if ((rc = m->tt.ensure((size_t)n_fields * 12 * m->no * m->ny))) return rc;
  auto* sin = static_cast<__nv_bfloat16*>(m->split_in.ptr);
  auto* tt = static_cast<__nv_bfloat16*>(m->tt.ptr);

  const double F = n_fields;
  CSG_CHECK(!presplit || (!in_mul && !pre.n && !iw && !in_idx), CSG_E_ARG,
            "csg_mft_execute: a split input takes no input ops, window or index");
  const bool hp = m->precision == CSG_PREC_HIGH;
  CSG_CHECK(!out_lo || (hp && !accumulate), CSG_E_ARG,
            "csg_mft_execute: a low-order output plane needs CSG_PREC_HIGH and no accumulation");
  if (!presplit) {  // else the producer of the input wrote split_in
    ProfScope ps(ctx, "mft_split", 0, F * m->ny * m->nx * (8.0 + 12.0 + (in_mul ? 8.0 : 0.0)));
    CSG_CHECK(n_fields < 65536, CSG_E_SHAPE, "csg_mft_execute: too many fields in one call");
    if (hp) {
      const long long warps = (long long)m->ny * ((m->nx + 255) / 256);
      dim3 grid(grid_for(warps, 8, 1024), n_fields);
      k_split_field_aligned<<<grid, 256, 0, st>>>(in, sin, m->ny, m->nx, inw.r0, inw.c0,
                                                  inw.rows, inw.pitch, in_mul, mul_idx, pre, fi,
                                                  in_idx);
    } else {
      dim3 grid(grid_for((long long)m->ny * m->nx / 8, 256, 1024), n_fields);
      k_split_field<<<grid, 256, 0, st>>>(in, sin, m->ny, m->nx, inw.r0, inw.c0, inw.rows,
                                          inw.pitch, in_mul, mul_idx, pre, fi, in_idx);
    }
    CSG_LAUNCH_CHECK();
  }

  const int bn1 = m->bn && !(hp && m->bn == 256) ? m->bn : 128;
  const int kb = bn1 == 256 ? 32 : tc::BK;  // K block of the tile width
  // ---- stage 1: T^T = split(in . B_x^T)^T
  {
    CUtensorMap ta, tb;
    if ((rc = make_map_k(&ta, sin, m->nx, m->ny, (long long)n_fields * 6, tc::BM, kb))) return rc;
    if ((rc = make_map_k(&tb, m->op1, m->nx, m->no, (long long)m->n_slots * 9, bn1, kb)))
      return rc;
    tc::Params p{};
    p.n_fields = n_fields;
    p.m_tiles = (m->ny + tc::BM - 1) / tc::BM;
    p.n_half = (m->no + bn1 - 1) / bn1;
    p.n_tiles = 2 * p.n_half;
    p.m_half = p.m_tiles;
    p.rows_valid = m->ny;
    p.cols_valid = m->no;
    p.k_blocks = (m->nx + kb - 1) / kb;
    terms_for(m->precision, p);
    p.slot = slot;
    p.out = tt;
    p.out_rows = m->no;
    p.out_cols = m->ny;
    p.accumulate = 0;
    p.status = ctx->status;
    p.valid = m->valid;
    p.wait_budget = ctx->wait_budget;
    p.prefetch = gemm_prefetch();
    const int grid = n_fields * p.m_tiles * p.n_tiles;
    // algorithmic work: 8 flops per complex multiply-add of the contraction
    ProfScope ps(ctx, "mft_gemm", 8.0 * F * m->ny * m->no * m->nx);
    if (hp)
      rc = bn1 == 64 ? launch_gemm<64, false, tc::EPI_T_SPLIT, true>(ta, tb, p, grid, st)
                     : launch_gemm<128, false, tc::EPI_T_SPLIT, true>(ta, tb, p, grid, st);
    else
      rc = bn1 == 64    ? launch_gemm<64, false, tc::EPI_T_SPLIT>(ta, tb, p, grid, st)
           : bn1 == 256 ? launch_gemm<256, false, tc::EPI_T_SPLIT>(ta, tb, p, grid, st)
                        : launch_gemm<128, false, tc::EPI_T_SPLIT>(ta, tb, p, grid, st);
    if (rc) return rc;
  }
  // ---- stage 2: out = (pref A_y) . T
  {
    CUtensorMap ta, tb;
    if ((rc = make_map_k(&ta, m->op2, m->ny, m->mo, (long long)m->n_slots * 9, tc::BM, kb)))
      return rc;
    if ((rc = make_map_k(&tb, tt, m->ny, m->no, (long long)n_fields * 6, bn1, kb))) return rc;
    tc::Params p{};
    p.n_fields = n_fields;
    p.m_half = (m->mo + tc::BM - 1) / tc::BM;
    p.m_tiles = 2 * p.m_half;
    p.n_tiles = (m->no + bn1 - 1) / bn1;
    p.n_half = p.n_tiles;
    p.rows_valid = m->mo;
    p.cols_valid = m->no;
    p.k_blocks = (m->ny + kb - 1) / kb;
    terms_for(m->precision, p);
    p.slot = slot;
    p.out = out;
    p.out_rows = m->mo;
    p.out_cols = m->no;
    p.out_pitch = outw.pitch;
    p.out_plane_rows = outw.rows;
    p.out_r0 = outw.r0;
    p.out_c0 = outw.c0;
    p.accumulate = accumulate;
    p.status = ctx->status;
    p.valid = m->valid;
    p.wait_budget = ctx->wait_budget;
    p.prefetch = gemm_prefetch();
    p.out_lo = out_lo;
    CUtensorMap to;
    p.tma_out = make_map_f32_out(&to, out + (size_t)outw.r0 * outw.pitch + outw.c0, m->no, m->mo,
                                 (long long)n_fields * 2, outw.pitch, outw.rows)
                    ? 1
                    : 0;
    const CUtensorMap* tmo = p.tma_out ? &to : nullptr;
    const int grid = n_fields * p.m_tiles * p.n_tiles;
    ProfScope ps(ctx, "mft_gemm", 8.0 * F * m->mo * m->no * m->ny);
    if (hp)
      rc = bn1 == 64 ? launch_gemm<64, true, tc::EPI_F32, true>(ta, tb, p, grid, st, tmo)
                     : launch_gemm<128, true, tc::EPI_F32, true>(ta, tb, p, grid, st, tmo);
    else
      rc = bn1 == 64    ? launch_gemm<64, true, tc::EPI_F32>(ta, tb, p, grid, st, tmo)
           : bn1 == 256 ? launch_gemm<256, true, tc::EPI_F32>(ta, tb, p, grid, st, tmo)
                        : launch_gemm<128, true, tc::EPI_F32>(ta, tb, p, grid, st, tmo);
    if (rc) return rc;
  }
  return CSG_OK;
}

__nv_bfloat16* csg::mft_split_buffer(csg_mft* m, int n_fields) {
  if (!m || n_fields <= 0) return nullptr;
  if (m->split_in.ensure((size_t)n_fields * 12 * m->ny * m->nx)) return nullptr;
  return static_cast<__nv_bfloat16*>(m->split_in.ptr);
}

bool csg::mft_is_high(const csg_mft* m) { return m && m->precision == CSG_PREC_HIGH; }

void csg::mft_input_shape(const csg_mft* m, int* ny, int* nx) {
  *ny = m->ny;
  *nx = m->nx;
}

extern "C" int csg_mft_execute(csg_ctx* ctx, csg_mft* m, const float* in, float* out,
                               int n_fields, const int* slot, int accumulate, const float* in_mul,
                               const int* mul_idx) {
  return mft_execute_ops(ctx, m, in, out, n_fields, slot, accumulate, in_mul, mul_idx, PixOps(),
                         FieldInfo());
}

extern "C" int csg_mft_execute_lo(csg_ctx* ctx, csg_mft* m, const float* in, float* out,
                                  float* out_lo, int n_fields, const int* slot) {
  CSG_CHECK(out_lo, CSG_E_ARG, "csg_mft_execute_lo: null low-order output");
  return mft_execute_ops(ctx, m, in, out, n_fields, slot, 0, nullptr, nullptr, PixOps(),
                         FieldInfo(), nullptr, nullptr, nullptr, false, out_lo);
}
