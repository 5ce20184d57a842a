// Response-matrix objective (optHexRespObjective, optObjective.cpp:24-69)
// on tcgen05 tensor cores.
//
//   X~ = [X; 0],  P_l = exp(i phaseSign 4 pi / lambda_l X~)      (per wavelength)
//   E_m = M_m P_l(m)                (complex GEMM, every (s, p, lambda) matrix)
//   pix = sum_m |E_m|^2,  f = mean_pix (or max_pix) / calib
//
// M is uploaded once and split into three bf16 parts; P is generated per call
// from FP64 phases (reduced in turns) straight into split operator planes; one
// launch of the split-bf16 GEMM (fp32 output) covers every matrix, and one
// reduction kernel turns |E|^2 into the objective of every candidate.
#include <cuda.h>

#include <map>
#include <vector>

#include "ctx.hpp"
#include "tc_gemm.cuh"

namespace csg {
int make_map(CUtensorMap* m, const void* base, int k, int rows, long long planes, int box_rows);
void terms_for(int precision, tc::Params& p);
int launch_gemm_data_op_f32(int bn, const CUtensorMap& a, const CUtensorMap& b,
                            const tc::Params& p, int grid, cudaStream_t st);

// M (complex<double>, row-major [n_mat][npix][ncol]) -> bf16 parts
// [n_mat][3][2][npix][kpad], zero in the padding columns.
__global__ void k_split_matrix(const double2* __restrict__ m, __nv_bfloat16* __restrict__ out,
                               int n_mat, int npix, int ncol, int kpad) {
  const long long plane = (long long)npix * kpad;
  const long long n = plane * n_mat;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int mat = (int)(i / plane);
    const long long o = i % plane;
    const int p = (int)(o / kpad), k = (int)(o % kpad);
    double2 v = make_double2(0.0, 0.0);
    if (k < ncol) v = m[((long long)mat * npix + p) * ncol + k];
    __nv_bfloat16 a[3], b[3];
    split3((float)v.x, a[0], a[1], a[2]);
    split3((float)v.y, b[0], b[1], b[2]);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      out[((long long)(mat * 3 + q) * 2 + 0) * plane + o] = a[q];
      out[((long long)(mat * 3 + q) * 2 + 1) * plane + o] = b[q];
    }
  }
}

// P[slot][part][sel][pop][kpad]: exp(i phaseSign 4 pi x / lambda) with x the
// candidate's sag (x = 0 for the last column, the Babinet term, and 0 in the
// padding columns); sel 0/1/2 = re, im, -im.
__global__ void k_phase_operator(const double* __restrict__ x, int pop, int nvar, int kpad,
                                 const double* __restrict__ lam, int n_slot, double phase_sign,
                                 __nv_bfloat16* __restrict__ out) {
  const long long plane = (long long)pop * kpad;
  const long long n = plane * n_slot;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(i / plane);
    const long long o = i % plane;
    const int c = (int)(o / kpad), k = (int)(o % kpad);
    float re = 0.f, im = 0.f;
    if (k <= nvar) {
      const double xv = k < nvar ? x[(long long)c * nvar + k] : 0.0;
      double t = phase_sign * 2.0 * xv / lam[s];  // 4 pi x / lambda rad = 2 x / lambda turns
      t -= rint(t);
      double sn, cs;
      sincospi(2.0 * t, &sn, &cs);
      re = (float)cs;
      im = (float)sn;
    }
    __nv_bfloat16 a[3], b[3];
    split3(re, a[0], a[1], a[2]);
    split3(im, b[0], b[1], b[2]);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      __nv_bfloat16* base = out + ((long long)(s * 3 + q) * 3) * plane + o;
      base[0] = a[q];
      base[plane] = b[q];
      base[2 * plane] = __hneg(b[q]);
    }
  }
}

// One block column of 32 candidates per blockIdx.x; threads.y split the
// pixels. pix = sum_mat |E|^2 in FP64, then mean or max over pixels.
__global__ void k_objective(const float* __restrict__ e, int n_mat, int npix, int pop, int mode,
                            double inv_calib, double* __restrict__ out) {
  __shared__ double red[8][33];
  const int q = blockIdx.x * 32 + threadIdx.x;
  double acc = 0.0;
  if (q < pop) {
    for (int p = threadIdx.y; p < npix; p += blockDim.y) {
      double ip = 0.0;
      for (int m = 0; m < n_mat; ++m) {
        const float* re = e + ((size_t)(m * 2) * npix + p) * pop;
        const float* im = re + (size_t)npix * pop;
        const double a = re[q], b = im[q];
        ip += a * a + b * b;
      }
      acc = mode == 0 ? acc + ip : fmax(acc, ip);
    }
  }
  red[threadIdx.y][threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.y == 0 && q < pop) {
    double v = red[0][threadIdx.x];
    for (int y = 1; y < blockDim.y; ++y)
      v = mode == 0 ? v + red[y][threadIdx.x] : fmax(v, red[y][threadIdx.x]);
    out[q] = (mode == 0 ? v / (double)npix : v) * inv_calib;
  }
}

}  // namespace csg

using namespace csg;

struct csg_respobj {
  csg_ctx* ctx = nullptr;
  int n_mat = 0, npix = 0, ncol = 0, kpad = 0, n_slot = 0, mode = 0, precision = 6;
  double calib = 1.0, phase_sign = 1.0;
  __nv_bfloat16* msplit = nullptr;  // [n_mat][3][2][npix][kpad]
  int* slot = nullptr;              // [n_mat] wavelength slot of each matrix
  double* lam = nullptr;            // [n_slot]
  Scratch psplit;                   // [n_slot][3][3][pop][kpad]
  Scratch eout;                     // [n_mat][2][npix][pop] fp32
};

extern "C" {

int csg_respobj_create(csg_ctx* ctx, csg_respobj** obj, const double* m_host, int n_mat,
                       int npix, int ncol, const double* wavelength, double calib,
                       double phase_sign, int objective) {
  CSG_CHECK(ctx && obj && m_host && wavelength, CSG_E_ARG, "csg_respobj_create: null argument");
  CSG_CHECK(n_mat > 0 && npix > 0 && ncol > 1, CSG_E_SHAPE, "csg_respobj_create: bad shape");
  CSG_CHECK(objective == 0 || objective == 1, CSG_E_ARG, "csg_respobj_create: objective 0 or 1");
  CSG_CHECK(all_finite(&calib, 1) && all_finite(wavelength, n_mat) &&
                all_finite(m_host, (size_t)n_mat * npix * ncol * 2),
            CSG_E_NAN, "csg_respobj_create: non-finite response matrix, wavelength or calibration");
  CSG_CHECK(calib > 0, CSG_E_ARG, "csg_respobj_create: calibration must be positive");
  DeviceGuard g(ctx->device);
  cudaStream_t st = ctx->stream;
  csg_respobj* o = new csg_respobj();
  o->ctx = ctx;
  o->n_mat = n_mat;
  o->npix = npix;
  o->ncol = ncol;
  o->kpad = (ncol + 7) / 8 * 8;
  o->calib = calib;
  o->phase_sign = phase_sign;
  o->mode = objective;
  std::map<double, int> slots;
  std::vector<int> slot(n_mat);
  std::vector<double> lam;
  for (int m = 0; m < n_mat; ++m) {
    CSG_CHECK(wavelength[m] > 0, CSG_E_ARG, "csg_respobj_create: non-positive wavelength");
    auto it = slots.find(wavelength[m]);
    if (it == slots.end()) {
      it = slots.emplace(wavelength[m], (int)lam.size()).first;
      lam.push_back(wavelength[m]);
    }
    slot[m] = it->second;
  }
  o->n_slot = (int)lam.size();
  const size_t mbytes = (size_t)n_mat * npix * ncol * 16;
  double2* staging = nullptr;
  if (cudaMalloc(&o->msplit, (size_t)n_mat * 12 * npix * o->kpad) != cudaSuccess ||
      cudaMalloc(&o->slot, n_mat * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&o->lam, lam.size() * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&staging, mbytes) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(o->msplit);
    cudaFree(o->slot);
    cudaFree(o->lam);
    cudaFree(staging);
    delete o;
    set_error("csg_respobj_create: allocation failed");
    return CSG_E_NOMEM;
  }
  CSG_CUDA(cudaMemcpyAsync(staging, m_host, mbytes, cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(o->slot, slot.data(), n_mat * sizeof(int), cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(o->lam, lam.data(), lam.size() * sizeof(double), cudaMemcpyHostToDevice,
                           st));
  k_split_matrix<<<grid_for((long long)n_mat * npix * o->kpad, 256), 256, 0, st>>>(
      staging, o->msplit, n_mat, npix, ncol, o->kpad);
  CSG_LAUNCH_CHECK();
  CSG_CUDA(cudaStreamSynchronize(st));
  cudaFree(staging);
  *obj = o;
  return CSG_OK;
}

int csg_respobj_destroy(csg_respobj* o) {
  if (!o) return CSG_OK;
  DeviceGuard g(o->ctx->device);
  cudaStreamSynchronize(o->ctx->stream);
  cudaFree(o->msplit);
  cudaFree(o->slot);
  cudaFree(o->lam);
  o->psplit.release();
  o->eout.release();
  delete o;
  return CSG_OK;
}

int csg_respobj_execute(csg_respobj* o, const double* x, int pop, double* out) {
  CSG_CHECK(o && x && out, CSG_E_ARG, "csg_respobj_execute: null argument");
  CSG_CHECK(pop > 0, CSG_E_SHAPE, "csg_respobj_execute: empty population");
  csg_ctx* ctx = o->ctx;
  DeviceGuard g(ctx->device);
  cudaStream_t st = ctx->stream;
  int rc;
  if ((rc = o->psplit.ensure((size_t)o->n_slot * 9 * pop * o->kpad * 2))) return rc;
  if ((rc = o->eout.ensure((size_t)o->n_mat * 2 * o->npix * pop * 4))) return rc;
  auto* ps = static_cast<__nv_bfloat16*>(o->psplit.ptr);
  auto* eo = static_cast<float*>(o->eout.ptr);
  k_phase_operator<<<grid_for((long long)o->n_slot * pop * o->kpad, 256), 256, 0, st>>>(
      x, pop, o->ncol - 1, o->kpad, o->lam, o->n_slot, o->phase_sign, ps);
  CSG_LAUNCH_CHECK();
  const int bn = pop <= 64 ? 64 : 128;
  CUtensorMap ta, tb;
  if ((rc = make_map(&ta, o->msplit, o->kpad, o->npix, (long long)o->n_mat * 6, tc::BM))) return rc;
  if ((rc = make_map(&tb, ps, o->kpad, pop, (long long)o->n_slot * 9, bn))) return rc;
  tc::Params p{};
  p.n_fields = o->n_mat;
  p.m_tiles = (o->npix + tc::BM - 1) / tc::BM;
  p.n_half = (pop + bn - 1) / bn;
  p.n_tiles = 2 * p.n_half;
  p.m_half = p.m_tiles;
  p.rows_valid = o->npix;
  p.cols_valid = pop;
  p.k_blocks = (o->kpad + tc::BK - 1) / tc::BK;
  terms_for(o->precision, p);
  p.slot = o->slot;
  p.out = eo;
  p.out_rows = o->npix;
  p.out_cols = pop;
  p.accumulate = 0;
  p.out_pitch = pop;
  p.out_plane_rows = o->npix;
  p.out_r0 = 0;
  p.out_c0 = 0;
  p.status = ctx->status;
  {
    ProfScope ps2(ctx, "respobj_gemm", 8.0 * o->n_mat * o->npix * (double)pop * o->ncol);
    rc = launch_gemm_data_op_f32(bn, ta, tb, p, o->n_mat * p.m_tiles * p.n_tiles, st);
    if (rc) return rc;
  }
  dim3 blk(32, 8), grd((pop + 31) / 32);
  k_objective<<<grd, blk, 0, st>>>(eo, o->n_mat, o->npix, pop, o->mode, 1.0 / o->calib, out);
  CSG_LAUNCH_CHECK();
  return CSG_OK;
}

}  // extern "C"
