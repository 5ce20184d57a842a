// Batched coronagraph executor: the reference's element walk
// (coronagraph::execute, coronagraph.cpp:175-200) over a batch of fields,
// each field one (wavelength, source, candidate) triple. Elements are added in
// optical order; execute() launches each element once for the whole batch on
// the context's stream, so the walk can be captured into a CUDA graph and
// replayed (csg_chain_capture / csg_chain_replay).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

#include "ctx.hpp"
#include "pixops.cuh"

extern "C" {
int csg_mft_create(csg_ctx*, csg_mft**, int, int, int, int, const double*, const double*,
                   const double*, const double*, int, const double*, const double*, double, int);
int csg_mft_create_ragged(csg_ctx*, csg_mft**, int, int, int, const int*, const double*,
                          const double*, const double*, const double*, int, const double*,
                          const double*, double, int);
int csg_mft_destroy(csg_mft*);
int csg_mft_execute(csg_ctx*, csg_mft*, const float*, float*, int, const int*, int, const float*,
                    const int*);
int csg_mft_reserve(csg_mft*, int);
int csg_mask_real(csg_ctx*, float*, int, int, int, const float*, int);
int csg_phase_screen(csg_ctx*, float*, int, int, int, const float*, const double*, double);
int csg_complex_mask(csg_ctx*, float*, int, int, int, const float*, const float*, int, int);
int csg_fresnel(csg_ctx*, float*, int, int, const double*, double, double);
int csg_intensity(csg_ctx*, const float*, int, int, int, double*, double*);
int csg_point_source(csg_ctx*, float*, int, int, int, double, double, const double*,
                     const double*, const double*);
}

namespace csg {
int hex_mask_region(csg_ctx* ctx, const int16_t* hex_id, const uint16_t* count, int S, int r0,
                    int c0, int RR, int CC, int n_sub, const double* sags, int n_hex, int n_out,
                    const int* cand, const double* lambda, double phase_sign, int flip,
                    double subtract, float* out, float2* phasors);
int hex_mask_with_phasor_buffer(csg_ctx* ctx, const int16_t* hex_id, const uint16_t* count, int S,
                                int n_sub, const double* sags, int n_hex, int n_out,
                                const int* cand, const double* lambda, double phase_sign, int flip,
                                double subtract, int use_only_hex, float* out, float2* phasors);

enum ElemKind {
  E_MASK,
  E_MIRROR,
  E_FRESNEL,
  E_CMASK,
  E_FPM_HEX,
  E_FRAUNHOFER,
  E_FFT_FPM,
  E_FPM_HEX_DOUBLE,
  E_FPM_MASK
};

template <typename T>
static T* dev_copy(const T* h, size_t n, cudaStream_t st) {
  T* d = nullptr;
  if (cudaMalloc(&d, n * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (h) cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, st);
  return d;
}

static std::vector<double> pixel_centres(int n, double d, double shift = 0.0) {
  // set_xy: -(n d - d)/2 + i d - origin (csim_geom.cpp:113-142)
  std::vector<double> v(n);
  for (int i = 0; i < n; ++i) v[i] = -(d * n - d) / 2.0 + i * d + shift;
  return v;
}

struct Elem {
  ElemKind kind;
  std::string name;
  int disable_for_calibration = 0;
  // mask / mirror / complex mask
  float* a = nullptr;
  float* b = nullptr;
  int mrows = 0, mcols = 0;
  int quirk = 0;
  double sign = 1.0;
  // fresnel
  double z = 0, ap_rad = 0;
  // hex FPM
  int16_t* hex_id = nullptr;
  uint16_t* count = nullptr;
  int S = 0, n_sub = 0, n_hex = 0;
  int r0 = 0, c0 = 0, RR = 0, CC = 0;  // transformed box of the S x S mask grid
  double phase_sign = 1.0;
  csg_mft* mft1 = nullptr;
  csg_mft* mft2 = nullptr;
  // double-Fraunhofer FPM: mft1 field -> zoom grid, mft2 zoom grid -> field,
  // mft3 the mask block of the zoom grid -> field; nz x nz zoom grid with the
  // RR x CC block at (zr0, zc0); the mask is the hex mask (hex_id set) or
  // the fixed dmask (M - 1 per wavelength slot)
  csg_mft* mft3 = nullptr;
  int nz = 0, zr0 = 0, zc0 = 0;
  // fraunhofer
  csg_mft* mft = nullptr;
  int n_out = 0;
  std::vector<int> n_out_l;  // ragged: per-wavelength image size (n_out = the largest)
  // padded-FFT focal-plane mask: P x P grid
  int P = 0;
  // its Babinet form: 1 - M vanishes outside the mask-index box
  // [br0, br0 + bR) x [bc0, bc0 + bC); bab = 1 runs it as a pair of MFTs
  // (mft1: field -> box spectrum, mft2: back, times 1 - M, subtracted),
  // bab = 2: M = 1 everywhere (the identity), bab = 0: the padded FFT
  int bab = 0;
  int br0 = 0, bc0 = 0, bR = 0, bC = 0;
  float* dmask = nullptr;  // [L][2][bR][bC] planar: 1 - M on the box
  // fixed-mask fpmPupToLyot: cmask the calibration mask (M - 1 or M like
  // dmask, [L][2][RR][CC]); null when calibration leaves the field as it is
  float* cmask = nullptr;
  // per-wavelength tables (mirror phasors, Fresnel transfer function)
  float2* tab = nullptr;
  // CSG_PREC_HIGH: the transfer function (Fresnel, padded-FFT mask) two-float
  float4* tab4 = nullptr;
  // mirror right after a real mask: the mask times the phasor table
  float2* tab_m = nullptr;
  // real mask: bounding box [sr0, sr1) x [sc0, sc1) of its nonzero pixels
  int sr0 = 0, sr1 = 0, sc0 = 0, sc1 = 0;
  // lazily built transforms: wavelength-f products, prefactors, window
  std::vector<double> lf, pref;
  double dm = 0, out_pixel = 0;
  MftWindow win{0, 0, 0, 0};  // window origin in the n x n field
  int win_rows = 0, win_cols = 0;
};

}  // namespace csg

using namespace csg;

struct csg_chain {
  csg_ctx* ctx = nullptr;
  int n = 0;
  double dx = 0;
  int n_lambda = 0;
  std::vector<double> lambda;
  double* lam_slots = nullptr;  // device copy of lambda (one per slot)
  int precision = 6;
  bool crop_support = true;
  bool fft_fpm_babinet = true;  // padded-FFT occulters in Babinet form when compact
  // fixed-mask FPMs without Babinet: calibrate the first wavelength only, as
  // the reference's compute-once calibration hat does
  bool ref_calibration = false;
  bool planned = false;  // lazily built transforms are up to date
  std::vector<Elem> elems;
  // batch description (device)
  int n_fields = 0, cap_fields = 0;
  int* slot = nullptr;          // wavelength index per field
  double* lam_f = nullptr;      // wavelength per field
  double* amp = nullptr;
  double* tip = nullptr;
  double* tilt = nullptr;
  int* cand = nullptr;          // candidate per field
  int* ident = nullptr;         // 0..F-1
  // buffers
  float* field = nullptr;       // [F][2][n][n]
  float* fpm = nullptr;         // [F][2][S][S]
  float* fpm_mask = nullptr;    // [F][2][S][S]
  float2* phasors = nullptr;    // [F][n_hex+1]
  float* image = nullptr;       // [F][2][n_out][n_out]
  float* image_lo = nullptr;    // CSG_PREC_HIGH: low-order words of the image
  float* padbuf = nullptr;      // [F][2][P][P] (padded-FFT focal-plane masks)
  double* sags = nullptr;       // [n_cand][n_hex]
  int n_cand = 0, sag_hex = 0;
  size_t fpm_cap = 0, img_cap = 0, ph_cap = 0, pad_cap = 0, img_lo_cap = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_calib = -1;
};

static int ensure_buf(float** p, size_t& cap, size_t need) {
  if (need <= cap) return CSG_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  cap = 0;
  if (cudaMalloc(p, need) != cudaSuccess) {
    cudaGetLastError();
    set_error("chain buffer allocation failed");
    return CSG_E_NOMEM;
  }
  cap = need;
  return CSG_OK;
}

static void drop_graph(csg_chain* c) {
  if (c->exec) cudaGraphExecDestroy(c->exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->exec = nullptr;
  c->graph = nullptr;
  c->graph_calib = -1;
}

extern "C" {

int csg_chain_create(csg_ctx* ctx, csg_chain** out, int n, double pixel_scale, int n_lambda,
                     const double* lambda, int precision) {
  CSG_CHECK(ctx && out && lambda, CSG_E_ARG, "csg_chain_create: null argument");
  CSG_CHECK(n >= 64 && n <= 4096 && n % 8 == 0, CSG_E_SHAPE,
            "csg_chain_create: the field must be N x N with N a multiple of 8 in [64, 4096]");
  CSG_CHECK(n_lambda > 0 && pixel_scale > 0, CSG_E_ARG, "csg_chain_create: bad parameters");
  CSG_CHECK(precision == CSG_PREC_BF16X6 || precision == CSG_PREC_BF16X3 ||
                precision == CSG_PREC_HIGH,
            CSG_E_ARG, "csg_chain_create: precision must be a CSG_PREC_* value");
  CSG_CHECK(all_finite(lambda, n_lambda) && all_finite(&pixel_scale, 1), CSG_E_NAN,
            "csg_chain_create: non-finite wavelength or pixel scale");
  csg_chain* c = new csg_chain();
  c->ctx = ctx;
  c->n = n;
  c->dx = pixel_scale;
  c->n_lambda = n_lambda;
  c->lambda.assign(lambda, lambda + n_lambda);
  {
    DeviceGuard g(ctx->device);
    c->lam_slots = dev_copy(lambda, n_lambda, ctx->stream);
    if (!c->lam_slots) {
      delete c;
      set_error("csg_chain_create: allocation failed");
      return CSG_E_NOMEM;
    }
  }
  c->precision = precision;
  *out = c;
  return CSG_OK;
}

int csg_chain_destroy(csg_chain* c) {
  if (!c) return CSG_OK;
  DeviceGuard g(c->ctx->device);
  cudaStreamSynchronize(c->ctx->stream);
  drop_graph(c);
  for (auto& e : c->elems) {
    cudaFree(e.a);
    cudaFree(e.b);
    cudaFree(e.hex_id);
    cudaFree(e.count);
    cudaFree(e.tab);
    cudaFree(e.tab4);
    cudaFree(e.tab_m);
    cudaFree(e.dmask);
    cudaFree(e.cmask);
    csg_mft_destroy(e.mft1);
    csg_mft_destroy(e.mft2);
    csg_mft_destroy(e.mft3);
    csg_mft_destroy(e.mft);
  }
  for (void* p : {(void*)c->slot, (void*)c->lam_f, (void*)c->amp, (void*)c->tip, (void*)c->tilt,
                  (void*)c->cand, (void*)c->ident, (void*)c->field, (void*)c->fpm,
                  (void*)c->fpm_mask, (void*)c->phasors, (void*)c->image, (void*)c->image_lo,
                  (void*)c->sags,
                  (void*)c->lam_slots, (void*)c->padbuf})
    cudaFree(p);
  delete c;
  return CSG_OK;
}

// mask element (mask.cpp:23-58): real mask N x N (host fp32), ref_quirk as
// csg_mask_real.
int csg_chain_add_mask(csg_chain* c, const float* mask, int ref_quirk, int disable_for_calibration) {
  CSG_CHECK(c && mask, CSG_E_ARG, "csg_chain_add_mask: null argument");
  DeviceGuard g(c->ctx->device);
  Elem e;
  e.kind = E_MASK;
  e.quirk = ref_quirk;
  e.disable_for_calibration = disable_for_calibration;
  e.a = dev_copy(mask, (size_t)c->n * c->n, c->ctx->stream);
  CSG_CHECK(e.a, CSG_E_NOMEM, "csg_chain_add_mask: allocation failed");
  // support of the mask (where it is nonzero)
  e.sr0 = e.sc0 = c->n;
  e.sr1 = e.sc1 = 0;
  for (int r = 0; r < c->n; ++r)
    for (int cc = 0; cc < c->n; ++cc)
      if (mask[(size_t)r * c->n + cc] != 0.f) {
        e.sr0 = std::min(e.sr0, r);
        e.sr1 = std::max(e.sr1, r + 1);
        e.sc0 = std::min(e.sc0, cc);
        e.sc1 = std::max(e.sc1, cc + 1);
      }
  c->elems.push_back(e);
  c->planned = false;
  drop_graph(c);
  return CSG_OK;
}

// out[s][p] = mask[p] * tab[s][p] for every wavelength slot s; with quirk
// the mask multiplies as m (1 + i), as the mask element applies it.
__global__ void k_mask_times_table(const float* __restrict__ mask, const float2* __restrict__ tab,
                                   long long plane, long long total, int quirk,
                                   float2* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const float m = mask[i % plane];
    const float2 w = tab[i];
    out[i] = quirk ? make_float2(m * (w.x - w.y), m * (w.x + w.y)) : make_float2(m * w.x, m * w.y);
  }
}

// mirror element (mirror.cpp:23-72): sag N x N (host fp32, metres).
int csg_chain_add_mirror(csg_chain* c, const float* sag, double sign) {
  CSG_CHECK(c && sag, CSG_E_ARG, "csg_chain_add_mirror: null argument");
  DeviceGuard g(c->ctx->device);
  Elem e;
  e.kind = E_MIRROR;
  e.sign = sign;
  e.a = dev_copy(sag, (size_t)c->n * c->n, c->ctx->stream);
  CSG_CHECK(e.a, CSG_E_NOMEM, "csg_chain_add_mirror: allocation failed");
  // per-wavelength phasors, as the reference's mirrorPhase cube (mirror.cpp:66-72)
  const size_t plane = (size_t)c->n * c->n;
  e.tab = dev_copy<float2>(nullptr, plane * c->n_lambda, c->ctx->stream);
  CSG_CHECK(e.tab, CSG_E_NOMEM, "csg_chain_add_mirror: allocation failed");
  int rc = build_phasor_table(c->ctx->stream, e.a, c->n, c->n, c->lam_slots, c->n_lambda, sign,
                              e.tab);
  if (rc) return rc;
  // after a real mask the walk applies both with one table read per pixel
  if (!c->elems.empty() && c->elems.back().kind == E_MASK) {
    e.tab_m = dev_copy<float2>(nullptr, plane * c->n_lambda, c->ctx->stream);
    CSG_CHECK(e.tab_m, CSG_E_NOMEM, "csg_chain_add_mirror: allocation failed");
    const long long total = (long long)plane * c->n_lambda;
    k_mask_times_table<<<grid_for(total, 256), 256, 0, c->ctx->stream>>>(
        c->elems.back().a, e.tab, (long long)plane, total, c->elems.back().quirk, e.tab_m);
    CSG_LAUNCH_CHECK();
  }
  c->elems.push_back(e);
  c->planned = false;
  drop_graph(c);
  return CSG_OK;
}

// fresnelPropagator (fresnelPropagator.cpp:23-61, pad factor 1): z is the
// signed distance, ap_rad the efield's arrayRadiusPhysical. The transfer
// function of every wavelength is tabulated once here (the reference rebuilds
// it on every call, csim_fft.cpp:386).
int csg_chain_add_fresnel(csg_chain* c, double z, double ap_rad) {
  CSG_CHECK(c && ap_rad > 0, CSG_E_ARG, "csg_chain_add_fresnel: bad argument");
  CSG_CHECK(all_finite(&z, 1) && all_finite(&ap_rad, 1), CSG_E_NAN,
            "csg_chain_add_fresnel: non-finite distance or aperture radius");
  DeviceGuard g(c->ctx->device);
  Elem e;
  e.kind = E_FRESNEL;
  e.z = z;
  e.ap_rad = ap_rad;
  e.tab = dev_copy<float2>(nullptr, (size_t)c->n * c->n * c->n_lambda, c->ctx->stream);
  CSG_CHECK(e.tab, CSG_E_NOMEM, "csg_chain_add_fresnel: allocation failed");
  int rc = build_fresnel_table(c->ctx->stream, c->n, c->lam_slots, c->n_lambda, z, ap_rad, e.tab);
  if (!rc && c->precision == CSG_PREC_HIGH) {
    e.tab4 = dev_copy<float4>(nullptr, (size_t)c->n * c->n * c->n_lambda, c->ctx->stream);
    if (!e.tab4) {
      cudaFree(e.tab);
      set_error("csg_chain_add_fresnel: allocation failed");
      return CSG_E_NOMEM;
    }
    rc = build_fresnel_table_df(c->ctx->stream, c->n, c->lam_slots, c->n_lambda, z, ap_rad,
                                e.tab4);
  }
  if (rc) {
    cudaFree(e.tab);
    cudaFree(e.tab4);
    return rc;
  }
  c->elems.push_back(e);
  c->planned = false;
  drop_graph(c);
  return CSG_OK;
}

// fresnelPropagator with padFactor != 1 (fresnelPropagator.cpp:41-54): the
// field embedded at [N/2, 3N/2) of a 2N x 2N zero array, propagated with the
// aperture radius padFactor apRad, and the centre cropped. It runs as the
// padded-FFT element's band-limited passes with the Fresnel transfer
// function of the 2N grid as the table: the first row pass reads the N field
// rows straight from the field, the column pass moves only those rows, and
// the last row pass writes the centre straight back (exact: the padding is
// zero, and the crop only needs the centre rows and columns).
int csg_chain_add_fresnel_padded(csg_chain* c, double z, double ap_rad, double pad_factor) {
  CSG_CHECK(c && ap_rad > 0 && pad_factor > 0, CSG_E_ARG,
            "csg_chain_add_fresnel_padded: bad argument");
  CSG_CHECK(all_finite(&z, 1) && all_finite(&ap_rad, 1) && all_finite(&pad_factor, 1),
            CSG_E_NAN, "csg_chain_add_fresnel_padded: non-finite argument");
  if (pad_factor == 1.0) return csg_chain_add_fresnel(c, z, ap_rad);
  const int P = 2 * c->n;
  CSG_CHECK(P <= 4096 && (P & (P - 1)) == 0, CSG_E_SHAPE,
            "csg_chain_add_fresnel_padded: 2N must be a power of two, at most 4096");
  DeviceGuard g(c->ctx->device);
  Elem e;
  e.kind = E_FFT_FPM;
  e.name = "fresnel_padded";
  e.P = P;
  e.bab = 0;
  e.z = z;
  e.ap_rad = ap_rad * pad_factor;
  const size_t n_tab = (size_t)P * P * c->n_lambda;
  e.tab = dev_copy<float2>(nullptr, n_tab, c->ctx->stream);
  CSG_CHECK(e.tab, CSG_E_NOMEM, "csg_chain_add_fresnel_padded: allocation failed");
  int rc = build_fresnel_table(c->ctx->stream, P, c->lam_slots, c->n_lambda, z, e.ap_rad, e.tab);
  if (!rc && c->precision == CSG_PREC_HIGH) {
    e.tab4 = dev_copy<float4>(nullptr, n_tab, c->ctx->stream);
    if (!e.tab4) {
      cudaFree(e.tab);
      set_error("csg_chain_add_fresnel_padded: allocation failed");
      return CSG_E_NOMEM;
    }
    rc = build_fresnel_table_df(c->ctx->stream, P, c->lam_slots, c->n_lambda, z, e.ap_rad,
                                e.tab4);
  }
  if (rc) {
    cudaFree(e.tab);
    cudaFree(e.tab4);
    return rc;
  }
  c->elems.push_back(e);
  c->planned = false;
  drop_graph(c);
  return CSG_OK;
}

// complexMask (complexMask.cpp:24-66): centred amp exp(-i ph), host fp32.
int csg_chain_add_complex_mask(csg_chain* c, const float* amp, const float* ph, int mrows,
                               int mcols, int disable_for_calibration) {
  CSG_CHECK(c && amp && ph && mrows > 0 && mcols > 0 && mrows <= c->n && mcols <= c->n, CSG_E_ARG,
            "csg_chain_add_complex_mask: bad argument");
  DeviceGuard g(c->ctx->device);
  Elem e;
  e.kind = E_CMASK;
  e.mrows = mrows;
  e.mcols = mcols;
  e.disable_for_calibration = disable_for_calibration;
  e.a = dev_copy(amp, (size_t)mrows * mcols, c->ctx->stream);
  e.b = dev_copy(ph, (size_t)mrows * mcols, c->ctx->stream);
  CSG_CHECK(e.a && e.b, CSG_E_NOMEM, "csg_chain_add_complex_mask: allocation failed");
  c->elems.push_back(e);
  c->planned = false;
  drop_graph(c);
  return CSG_OK;
}

// fpmPupToLyot with fpmIntHexCMCForPupToLyot (fpmPupToLyot.cpp:24-167,
// 419-455) in matrix-Fourier form:
//   E <- E + c MFT2[(fliplr(M) - 1) . MFT1[E]]
// MFT1: pupil -> mask grid, kernel e^{+2 pi i xm x / lf'};
// MFT2: mask grid -> pupil grid shifted by +dx/2, kernel e^{-2 pi i ...};
// lf' = fRatioSign lambda focalRatio 2 beamRadius,
// c = zoomFftSign dm^2 / (i lf') * dx^2 / (-i fRatioSign lf').
// This is the reference's 2N circular-convolution operator exactly (the
// convolution never wraps and fft_shift by N puts the kernel origin at +dx/2).
// hex_id/count: host [3][S][S] tables; dm: mask pixel size (metres).
int csg_chain_add_fpm_hex(csg_chain* c, const int16_t* hex_id, const uint16_t* count, int S,
                          int n_sub, int n_hex, double dm, double focal_ratio, double beam_radius,
                          double f_ratio_sign, double zoom_fft_sign, double phase_sign,
                          int disable_for_calibration) {
  CSG_CHECK(c && hex_id && count, CSG_E_ARG, "csg_chain_add_fpm_hex: null argument");
  CSG_CHECK(S >= 8 && S % 8 == 0 && n_sub > 0 && n_hex > 0, CSG_E_SHAPE,
            "csg_chain_add_fpm_hex: S must be a multiple of 8");
  DeviceGuard g(c->ctx->device);
  cudaStream_t st = c->ctx->stream;
  Elem e;
  e.kind = E_FPM_HEX;
  e.S = S;
  e.n_sub = n_sub;
  e.n_hex = n_hex;
  e.phase_sign = phase_sign;
  e.disable_for_calibration = disable_for_calibration;
  e.hex_id = dev_copy(hex_id, (size_t)3 * S * S, st);
  e.count = dev_copy(count, (size_t)3 * S * S, st);
  CSG_CHECK(e.hex_id && e.count, CSG_E_NOMEM, "csg_chain_add_fpm_hex: allocation failed");
  const int n = c->n, L = c->n_lambda;
  std::vector<double> lf(L), pref1(2 * L), pref2(2 * L);
  for (int l = 0; l < L; ++l) {
    lf[l] = f_ratio_sign * c->lambda[l] * focal_ratio * 2.0 * beam_radius;
    pref1[2 * l] = 1.0;
    pref1[2 * l + 1] = 0.0;
    // c = s dm^2/(i lf) * dx^2/(-i fr lf) = s dm^2 dx^2 / (fr lf^2)   (i * -i = 1)
    pref2[2 * l] = zoom_fft_sign * dm * dm * c->dx * c->dx / (f_ratio_sign * lf[l] * lf[l]);
    pref2[2 * l + 1] = 0.0;
  }
  // Support of fliplr(M) - 1: M = sum_k n_k e^{i phi_k} / nSub^2 with
  // sum_k n_k = nSub^2, so M - 1 vanishes wherever no sub-pixel falls in a hex,
  // for every choice of sags. Both transforms run on the bounding box of that
  // support (rounded out to multiples of 8), which gives exactly the
  // full-grid result.
  int rmin = S, rmax = -1, cmin = S, cmax = -1;
  if (c->crop_support) {
    const size_t plane = (size_t)S * S;
    for (int r = 0; r < S; ++r)
      for (int cc = 0; cc < S; ++cc) {
        const size_t src = (size_t)r * S + (S - 1 - cc);  // flipped column
        bool in = false;
        for (int k = 0; k < 3; ++k) in |= count[k * plane + src] > 0 && hex_id[k * plane + src] >= 0;
        if (in) {
          rmin = std::min(rmin, r);
          rmax = std::max(rmax, r);
          cmin = std::min(cmin, cc);
          cmax = std::max(cmax, cc);
        }
      }
  }
  if (rmax < 0) {  // no cropping (or an empty mask): the full grid
    rmin = cmin = 0;
    rmax = cmax = S - 1;
  }
  // box sides rounded up to multiples of 128 (the tensor-core tile), centred
  // on the support and kept inside the grid
  auto place = [S](int lo, int hi, int& o, int& len) {
    len = std::min(S, (hi - lo + 1 + 127) / 128 * 128);
    o = std::max(0, std::min(S - len, (lo + hi + 1) / 2 - len / 2));
  };
  place(rmin, rmax, e.r0, e.RR);
  place(cmin, cmax, e.c0, e.CC);
  std::vector<double> xp = pixel_centres(n, c->dx), xm = pixel_centres(S, dm);
  std::vector<double> xps = pixel_centres(n, c->dx, c->dx / 2.0);
  const double* ym_c = xm.data() + e.r0;  // rows of the box (y)
  const double* xm_c = xm.data() + e.c0;  // columns of the box (x)
  int rc = csg_mft_create(c->ctx, &e.mft1, n, n, e.RR, e.CC, xp.data(), xp.data(), ym_c, xm_c, L,
                          lf.data(), pref1.data(), +1.0, c->precision);
  if (rc) return rc;
  // the return transform is built once the elements after it are known
  // (its output may be limited to the support of the following stops)
  e.lf = lf;
  e.pref = pref2;
  e.dm = dm;
  c->elems.push_back(e);
  c->planned = false;
  drop_graph(c);
  return CSG_OK;
}

// fpmPupToLyot with a fixed mask (the CMC and binary adapters,
// fpmPupToLyot.cpp:303-367, 521-557): the hex element's transform pair with
// the mask uploaded once per wavelength instead of built from sags.
int csg_chain_add_fpm_mask(csg_chain* c, const float* mask_re, const float* mask_im, int n_mask,
                           int mask_index, int rows, int cols, double mask_pixel, const double* lf,
                           double f_ratio_sign, double zoom_fft_sign, int babinet,
                           const float* calib_re, const float* calib_im,
                           int disable_for_calibration) {
  CSG_CHECK(c && mask_re && lf, CSG_E_ARG, "csg_chain_add_fpm_mask: null argument");
  const int n = c->n, L = c->n_lambda;
  CSG_CHECK(rows >= 8 && cols >= 8 && rows % 8 == 0 && cols % 8 == 0 && n_mask >= 1 &&
                mask_pixel > 0.0,
            CSG_E_SHAPE,
            "csg_chain_add_fpm_mask: rows and cols must be multiples of 8 and n_mask >= 1");
  CSG_CHECK(mask_index >= -1 && mask_index < n_mask, CSG_E_ARG,
            "csg_chain_add_fpm_mask: mask_index must be -1 or a slice of the mask cube");
  // the reference applies one slice to every wavelength: maskIndex, or the
  // first slice it processes when the script leaves it at -1
  // (fpmCMCForPupToLyot::set_fpmMatAmp, fpmPupToLyot.cpp:355-360)
  const int slice = mask_index < 0 ? 0 : mask_index;
  DeviceGuard g(c->ctx->device);
  cudaStream_t st = c->ctx->stream;
  Elem e;
  e.kind = E_FPM_MASK;
  e.disable_for_calibration = disable_for_calibration;
  e.bab = babinet ? 1 : 0;
  e.r0 = e.c0 = 0;
  e.RR = rows;
  e.CC = cols;
  e.dm = mask_pixel;
  // planar per-wavelength multipliers: M - 1 (Babinet) or M
  const size_t plane = (size_t)rows * cols;
  // the calibration mask is a single plane ([rows][cols], the binary
  // adapter's calibMat) applied at every wavelength
  auto planes = [&](const float* re, const float* im, bool ones, size_t src) {
    std::vector<float> d((size_t)L * 2 * plane);
    for (int l = 0; l < L; ++l) {
      for (size_t p = 0; p < plane; ++p) {
        const float mr = ones ? 1.f : re[src + p], mi = ones || !im ? 0.f : im[src + p];
        d[(size_t)l * 2 * plane + p] = e.bab ? mr - 1.f : mr;
        d[(size_t)l * 2 * plane + plane + p] = mi;
      }
    }
    return d;
  };
  std::vector<float> d = planes(mask_re, mask_im, false, (size_t)slice * plane);
  e.dmask = dev_copy(d.data(), d.size(), st);
  CSG_CHECK(e.dmask, CSG_E_NOMEM, "csg_chain_add_fpm_mask: allocation failed");
  // the calibration mask, unless it leaves the field as it is (ones with Babinet)
  if (disable_for_calibration && (calib_re || !e.bab)) {
    std::vector<float> cd = planes(calib_re, calib_im, calib_re == nullptr, 0);
    if (c->ref_calibration && !e.bab) {
      // the reference's calibration transform exists for the first
      // wavelength only; the others keep a zero mask hat, so their
      // calibration fields are zero (fpmPupToLyot.cpp:56, 86-92)
      std::fill(cd.begin() + 2 * plane, cd.end(), 0.f);
    }
    e.cmask = dev_copy(cd.data(), cd.size(), st);
    if (!e.cmask) {
      cudaFree(e.dmask);
      set_error("csg_chain_add_fpm_mask: allocation failed");
      return CSG_E_NOMEM;
    }
  }
  std::vector<double> lfv(lf, lf + L), pref1(2 * L, 0.0), pref2(2 * L, 0.0);
  for (int l = 0; l < L; ++l) {
    pref1[2 * l] = 1.0;
    pref2[2 * l] = zoom_fft_sign * mask_pixel * mask_pixel * c->dx * c->dx /
                   (f_ratio_sign * lf[l] * lf[l]);
  }
  std::vector<double> xp = pixel_centres(n, c->dx), yr = pixel_centres(rows, mask_pixel),
                      xc = pixel_centres(cols, mask_pixel);
  int rc = csg_mft_create(c->ctx, &e.mft1, n, n, rows, cols, xp.data(), xp.data(), yr.data(),
                          xc.data(), L, lfv.data(), pref1.data(), +1.0, c->precision);
  if (rc) {
    cudaFree(e.dmask);
    cudaFree(e.cmask);
    return rc;
  }
  e.lf = lfv;
  e.pref = pref2;
  c->elems.push_back(e);
  c->planned = false;
  drop_graph(c);
  return CSG_OK;
}

// The double-Fraunhofer elements (doubleFraunhoferInterpFPM.cpp:24-65 with
// geometry :86-121 and complexHexMaskFPM.cpp:25-42; doubleFraunhoferFPM.cpp:
// 23-110): zoom FFT to an nz x nz grid of pixel zpx[l] at lambda f =
// lf_factor lambda, a mask on the centred rows x cols block (the rest of the
// grid left as it is), zoom FFT back at -lf_factor lambda. So E_out =
// MFT_out[Z] + MFT_out restricted to the block[(M - 1) Z]. The zoom grid's
// coordinates (i - nz/2) zpx[l] enter the phases as integers over
// lambda f / zpx[l], so one plan serves every wavelength's pixel size.
static int add_double_fraunhofer(csg_chain* c, Elem& e, int rows, int cols, const double* zpx,
                                 double pad_factor, double lf_factor) {
  const int n = c->n, L = c->n_lambda;
  const int nz = (int)(pad_factor * n);  // int nRows = padFactor * nRowsE
  CSG_CHECK(rows >= 8 && cols >= 8 && rows % 8 == 0 && cols % 8 == 0 && nz % 8 == 0 &&
                nz >= rows && nz >= cols && lf_factor != 0.0,
            CSG_E_SHAPE,
            "double-Fraunhofer FPM: mask sides and pad_factor N must be multiples of 8, "
            "pad_factor N at least the mask");
  for (int l = 0; l < L; ++l)
    CSG_CHECK(zpx[l] > 0.0, CSG_E_ARG, "double-Fraunhofer FPM: zoom pixel must be positive");
  e.nz = nz;
  e.zr0 = nz / 2 - rows / 2;  // tcMat.n_rows / 2 - mask.n_rows / 2
  e.zc0 = nz / 2 - cols / 2;
  e.r0 = e.c0 = 0;
  e.RR = rows;
  e.CC = cols;
  std::vector<double> zi(nz), xp = pixel_centres(n, c->dx);
  for (int i = 0; i < nz; ++i) zi[i] = (double)i - (double)nz / 2.0;
  std::vector<double> lf_in(L), lf_out(L), pin(2 * L), pout(2 * L);
  for (int l = 0; l < L; ++l) {
    const double lf = lf_factor * c->lambda[l];
    lf_in[l] = lf / zpx[l];
    lf_out[l] = -lf / zpx[l];
    // zoomFft prefactor dx_in dy_in / (i lambda f) (csim_fft.cpp:794-801)
    pin[2 * l] = 0.0;
    pin[2 * l + 1] = -c->dx * c->dx / lf;
    pout[2 * l] = 0.0;
    pout[2 * l + 1] = zpx[l] * zpx[l] / lf;
  }
  int rc = csg_mft_create(c->ctx, &e.mft1, n, n, nz, nz, xp.data(), xp.data(), zi.data(),
                          zi.data(), L, lf_in.data(), pin.data(), -1.0, c->precision);
  if (!rc)
    rc = csg_mft_create(c->ctx, &e.mft2, nz, nz, n, n, zi.data(), zi.data(), xp.data(), xp.data(),
                        L, lf_out.data(), pout.data(), -1.0, c->precision);
  if (!rc)
    rc = csg_mft_create(c->ctx, &e.mft3, rows, cols, n, n, zi.data() + e.zr0, zi.data() + e.zc0,
                        xp.data(), xp.data(), L, lf_out.data(), pout.data(), -1.0, c->precision);
  if (rc) {
    csg_mft_destroy(e.mft1);
    csg_mft_destroy(e.mft2);
    csg_mft_destroy(e.mft3);
    return rc;
  }
  return CSG_OK;
}

int csg_chain_add_fpm_hex_double(csg_chain* c, const int16_t* hex_id, const uint16_t* count,
                                 int S, int n_sub, int n_hex, double fpm_scale, double pad_factor,
                                 double lf_factor, double phase_sign,
                                 int disable_for_calibration) {
  CSG_CHECK(c && hex_id && count, CSG_E_ARG, "csg_chain_add_fpm_hex_double: null argument");
  CSG_CHECK(S >= 8 && S % 8 == 0 && n_sub > 0 && n_hex > 0 && fpm_scale > 0.0, CSG_E_SHAPE,
            "csg_chain_add_fpm_hex_double: bad mask size, sub-pixel count or scale");
  DeviceGuard g(c->ctx->device);
  cudaStream_t st = c->ctx->stream;
  Elem e;
  e.kind = E_FPM_HEX_DOUBLE;
  e.S = S;
  e.n_sub = n_sub;
  e.n_hex = n_hex;
  e.phase_sign = phase_sign;
  e.disable_for_calibration = disable_for_calibration;
  std::vector<double> zpx(c->n_lambda, fpm_scale);  // the hex mask's fpmScale
  int rc = add_double_fraunhofer(c, e, S, S, zpx.data(), pad_factor, lf_factor);
  if (rc) return rc;
  e.hex_id = dev_copy(hex_id, (size_t)3 * S * S, st);
  e.count = dev_copy(count, (size_t)3 * S * S, st);
  if (!e.hex_id || !e.count) {
    cudaFree(e.hex_id);
    cudaFree(e.count);
    csg_mft_destroy(e.mft1);
    csg_mft_destroy(e.mft2);
    csg_mft_destroy(e.mft3);
    CSG_CHECK(false, CSG_E_NOMEM, "csg_chain_add_fpm_hex_double: allocation failed");
  }
  c->elems.push_back(e);
  c->planned = false;
  drop_graph(c);
  return CSG_OK;
}

int csg_chain_add_fpm_double_mask(csg_chain* c, const float* mask_re, const float* mask_im,
                                  int rows, int cols, const double* zoom_pixel, double pad_factor,
                                  double lf_factor, int disable_for_calibration) {
  CSG_CHECK(c && mask_re && zoom_pixel, CSG_E_ARG, "csg_chain_add_fpm_double_mask: null argument");
  DeviceGuard g(c->ctx->device);
  Elem e;
  e.kind = E_FPM_HEX_DOUBLE;  // the same walk step, with a fixed mask
  e.disable_for_calibration = disable_for_calibration;
  int rc = add_double_fraunhofer(c, e, rows, cols, zoom_pixel, pad_factor, lf_factor);
  if (rc) return rc;
  // M - 1 per wavelength slot (one mask for every wavelength)
  const int L = c->n_lambda;
  const size_t plane = (size_t)rows * cols;
  std::vector<float> d((size_t)L * 2 * plane);
  for (int l = 0; l < L; ++l)
    for (size_t p = 0; p < plane; ++p) {
      d[(size_t)l * 2 * plane + p] = mask_re[p] - 1.f;
      d[(size_t)l * 2 * plane + plane + p] = mask_im ? mask_im[p] : 0.f;
    }
  e.dmask = dev_copy(d.data(), d.size(), c->ctx->stream);
  if (!e.dmask) {
    csg_mft_destroy(e.mft1);
    csg_mft_destroy(e.mft2);
    csg_mft_destroy(e.mft3);
    CSG_CHECK(false, CSG_E_NOMEM, "csg_chain_add_fpm_double_mask: allocation failed");
  }
  c->elems.push_back(e);
  c->planned = false;
  drop_graph(c);
  return CSG_OK;
}

// Padded-FFT focal-plane mask (the plain Lyot coronagraph's occulter): the
// n x n field is embedded at the centre of a zeroed pad x pad grid (as
// fpmPupToLyot.cpp:112-118 does for pad = 2n), transformed by a pad^2 FFT,
// multiplied by the focal-plane mask, transformed back (ifft / pad^2) and
// cropped to its centre. mask_re / mask_im: host [n_lambda][pad][pad] in
// centred focal coordinates (row pad/2, column pad/2 is zero frequency);
// mask_im may be null for a real mask. Stored in FFT order, one table per
// wavelength, and applied between the column transforms (the same three
// passes as a Fresnel propagation).
int csg_chain_add_fft_fpm(csg_chain* c, int pad, const float* mask_re, const float* mask_im,
                          int disable_for_calibration) {
  CSG_CHECK(c && mask_re, CSG_E_ARG, "csg_chain_add_fft_fpm: null argument");
  CSG_CHECK(pad >= c->n && pad <= 4096 && (pad & (pad - 1)) == 0, CSG_E_SHAPE,
            "csg_chain_add_fft_fpm: pad must be a power of two in [n, 4096]");
  DeviceGuard g(c->ctx->device);
  Elem e;
  e.kind = E_FFT_FPM;
  e.P = pad;
  e.disable_for_calibration = disable_for_calibration;
  const size_t plane = (size_t)pad * pad;
  std::vector<float2> h(plane * c->n_lambda);
  const int half = pad / 2;
  for (int l = 0; l < c->n_lambda; ++l)
    for (int r = 0; r < pad; ++r)
      for (int cc = 0; cc < pad; ++cc) {
        const size_t src = l * plane + (size_t)r * pad + cc;
        const size_t dst = l * plane + (size_t)((r + half) % pad) * pad + (cc + half) % pad;
        h[dst] = make_float2(mask_re[src], mask_im ? mask_im[src] : 0.f);
      }
  e.tab = dev_copy(h.data(), h.size(), c->ctx->stream);
  CSG_CHECK(e.tab, CSG_E_NOMEM, "csg_chain_add_fft_fpm: allocation failed");
  if (c->precision == CSG_PREC_HIGH) {  // the two-float passes read a two-float table
    e.tab4 = dev_copy<float4>(nullptr, h.size(), c->ctx->stream);
    if (!e.tab4) {
      cudaFree(e.tab);
      set_error("csg_chain_add_fft_fpm: allocation failed");
      return CSG_E_NOMEM;
    }
    const int rc4 = table_to_df(c->ctx->stream, e.tab, e.tab4, (long long)h.size());
    if (rc4) {
      cudaFree(e.tab);
      cudaFree(e.tab4);
      return rc4;
    }
  }
  if (c->fft_fpm_babinet) {
    // Babinet form: E - crop(ifft((1 - M) fft(embed(E)))). Where 1 - M has a
    // small support only those frequencies enter, and both transforms are
    // exact DFT sums over them: an MFT from the field's padded-grid pixels
    // to the support box and one back (integer coordinates, period pad).
    int r0 = pad, r1 = 0, c0 = pad, c1 = 0;
    for (int l = 0; l < c->n_lambda; ++l)
      for (int r = 0; r < pad; ++r)
        for (int cc = 0; cc < pad; ++cc) {
          const size_t src = l * plane + (size_t)r * pad + cc;
          if (mask_re[src] != 1.f || (mask_im && mask_im[src] != 0.f)) {
            r0 = std::min(r0, r);
            r1 = std::max(r1, r + 1);
            c0 = std::min(c0, cc);
            c1 = std::max(c1, cc + 1);
          }
        }
    if (r1 <= r0) {
      e.bab = 2;
    } else {
      // box sides rounded up to multiples of 8 (the transforms' TMA extents)
      const int R = std::min(pad, (r1 - r0 + 7) / 8 * 8), C = std::min(pad, (c1 - c0 + 7) / 8 * 8);
      r0 = std::min(r0, pad - R);
      c0 = std::min(c0, pad - C);
      if ((size_t)R * C * 16 <= plane && R <= 1024 && C <= 1024) {
        e.bab = 1;
        e.br0 = r0;
        e.bc0 = c0;
        e.bR = R;
        e.bC = C;
        const int L = c->n_lambda;
        std::vector<float> d((size_t)L * 2 * R * C);
        for (int l = 0; l < L; ++l)
          for (int r = 0; r < R; ++r)
            for (int cc = 0; cc < C; ++cc) {
              const size_t src = l * plane + (size_t)(r0 + r) * pad + (c0 + cc);
              const size_t o = ((size_t)l * 2 * R + r) * C + cc;
              d[o] = (float)(1.0 - (double)mask_re[src]);
              d[o + (size_t)R * C] = mask_im ? -mask_im[src] : 0.f;
            }
        e.dmask = dev_copy(d.data(), d.size(), c->ctx->stream);
        CSG_CHECK(e.dmask, CSG_E_NOMEM, "csg_chain_add_fft_fpm: allocation failed");
        // field pixel y sits at padded index (pad - n)/2 + y; mask index j is
        // frequency j - pad/2
        const int n = c->n, lo = (pad - n) / 2;
        std::vector<double> pin(n), fy(R), fx(C), lf(L, (double)pad), pref(2 * L, 0.0);
        for (int y = 0; y < n; ++y) pin[y] = lo + y;
        for (int r = 0; r < R; ++r) fy[r] = r0 + r - pad / 2;
        for (int cc = 0; cc < C; ++cc) fx[cc] = c0 + cc - pad / 2;
        for (int l = 0; l < L; ++l) pref[2 * l] = 1.0;
        int rc = csg_mft_create(c->ctx, &e.mft1, n, n, R, C, pin.data(), pin.data(), fy.data(),
                                fx.data(), L, lf.data(), pref.data(), -1.0, c->precision);
        if (rc) return rc;
      }
    }
  }
  CSG_CUDA(cudaStreamSynchronize(c->ctx->stream));  // the host staging buffers go away
  c->elems.push_back(e);
  c->planned = false;
  drop_graph(c);
  return CSG_OK;
}

// Whether hex focal-plane masks added after this call run their transforms on
// the mask's support only (default on; the result is the same either way).
int csg_chain_set_fft_fpm_babinet(csg_chain* c, int enable) {
  CSG_CHECK(c, CSG_E_ARG, "csg_chain_set_fft_fpm_babinet: null chain");
  c->fft_fpm_babinet = enable != 0;
  return CSG_OK;
}

int csg_chain_set_support_crop(csg_chain* c, int enable) {
  CSG_CHECK(c, CSG_E_ARG, "csg_chain_set_support_crop: null chain");
  c->crop_support = enable != 0;
  c->planned = false;
  drop_graph(c);
  return CSG_OK;
}

// The FPM grid actually transformed by the idx-th hex FPM element.
int csg_chain_fpm_region(csg_chain* c, int idx, int* r0, int* c0, int* rows, int* cols) {
  CSG_CHECK(c && r0 && c0 && rows && cols, CSG_E_ARG, "csg_chain_fpm_region: null argument");
  int k = 0;
  for (auto& e : c->elems)
    if (e.kind == E_FPM_HEX && k++ == idx) {
      *r0 = e.r0;
      *c0 = e.c0;
      *rows = e.RR;
      *cols = e.CC;
      return CSG_OK;
    }
  set_error("csg_chain_fpm_region: no such element");
  return CSG_E_ARG;
}

// fraunhoferFocal (fraunhoferFocal.cpp:23-72): zoomFft to n_out x n_out at
// out_pixel, lambda f = lambda * lf_scale (lf_scale = 2 beamRadius
// primaryfRatio), prefactor dx^2 / (i lambda f).
int csg_chain_add_fraunhofer(csg_chain* c, int n_out, double out_pixel, double lf_scale) {
  CSG_CHECK(c && n_out > 0 && out_pixel > 0 && lf_scale != 0, CSG_E_ARG,
            "csg_chain_add_fraunhofer: bad argument");
  DeviceGuard g(c->ctx->device);
  Elem e;
  e.kind = E_FRAUNHOFER;
  e.n_out = n_out;
  const int n = c->n, L = c->n_lambda;
  std::vector<double> lf(L), pref(2 * L);
  for (int l = 0; l < L; ++l) {
    lf[l] = c->lambda[l] * lf_scale;
    // dx dy / (i lf) = -i dx^2 / lf
    pref[2 * l] = 0.0;
    pref[2 * l + 1] = -c->dx * c->dx / lf[l];
  }
  (void)n;
  e.lf = lf;
  e.pref = pref;
  e.out_pixel = out_pixel;
  c->elems.push_back(e);  // the transform is built with the rest of the walk
  c->planned = false;
  drop_graph(c);
  return CSG_OK;
}

int csg_chain_add_fraunhofer_ragged(csg_chain* c, const int* n_out, double out_pixel,
                                    double lf_scale) {
  CSG_CHECK(c && n_out, CSG_E_ARG, "csg_chain_add_fraunhofer_ragged: null argument");
  int n_max = 0;
  for (int l = 0; l < c->n_lambda; ++l) {
    CSG_CHECK(n_out[l] > 0, CSG_E_SHAPE, "csg_chain_add_fraunhofer_ragged: bad size");
    n_max = std::max(n_max, n_out[l]);
  }
  int rc = csg_chain_add_fraunhofer(c, n_max, out_pixel, lf_scale);
  if (rc) return rc;
  c->elems.back().n_out_l.assign(n_out, n_out + c->n_lambda);
  return CSG_OK;
}

// Window of the field that the transform after elements (lo, hi) needs:
// the intersection of the supports of the real masks applied in between
// (also in calibration), rounded out to multiples of 32; the whole field when
// there is none or cropping is off.
static MftWindow stop_window(const csg_chain* c, int lo, int hi) {
  const int n = c->n;
  int r0 = 0, r1 = n, c0 = 0, c1 = n;
  if (c->crop_support) {
    for (int k = lo + 1; k < hi; ++k) {
      const Elem& m = c->elems[k];
      if (m.kind != E_MASK || m.disable_for_calibration) continue;
      r0 = std::max(r0, m.sr0);
      r1 = std::min(r1, m.sr1);
      c0 = std::max(c0, m.sc0);
      c1 = std::min(c1, m.sc1);
    }
    if (r1 <= r0 || c1 <= c0) r0 = c0 = 0, r1 = c1 = 32;  // an all-zero stop
  }
  r0 = r0 / 32 * 32;
  c0 = c0 / 32 * 32;
  r1 = std::min(n, (r1 + 31) / 32 * 32);
  c1 = std::min(n, (c1 + 31) / 32 * 32);
  return MftWindow{r0, c0, r1 - r0, c1 - c0};
}

static bool is_pointwise(ElemKind k) { return k == E_MASK || k == E_MIRROR || k == E_CMASK; }

// Build the transforms whose shape depends on the elements around them: the
// hex FPM's return transform and the final-image transform run on the
// window of the stops between them.
static int build_plans(csg_chain* c) {
  if (c->planned) return CSG_OK;
  const int n = c->n, L = c->n_lambda;
  const int ne = (int)c->elems.size();
  std::vector<double> xp = pixel_centres(n, c->dx), xps = pixel_centres(n, c->dx, c->dx / 2.0);
  for (int i = 0; i < ne; ++i) {
    Elem& e = c->elems[i];
    if (e.kind == E_FPM_HEX) {
      int j = i + 1;
      while (j < ne && is_pointwise(c->elems[j].kind)) ++j;
      MftWindow w = (j < ne && c->elems[j].kind == E_FRAUNHOFER) ? stop_window(c, i, j)
                                                                 : MftWindow{0, 0, n, n};
      std::vector<double> xm = pixel_centres(e.S, e.dm);
      csg_mft_destroy(e.mft2);
      e.mft2 = nullptr;
      int rc = csg_mft_create(c->ctx, &e.mft2, e.RR, e.CC, w.rows, w.pitch, xm.data() + e.r0,
                              xm.data() + e.c0, xps.data() + w.r0, xps.data() + w.c0, L,
                              e.lf.data(), e.pref.data(), -1.0, c->precision);
      if (rc) return rc;
      e.win = MftWindow{w.r0, w.c0, n, n};  // output window of the n x n field
      e.win_rows = w.rows;
      e.win_cols = w.pitch;
    } else if (e.kind == E_FPM_MASK) {
      int j = i + 1;
      while (j < ne && is_pointwise(c->elems[j].kind)) ++j;
      MftWindow w = (j < ne && c->elems[j].kind == E_FRAUNHOFER) ? stop_window(c, i, j)
                                                                 : MftWindow{0, 0, n, n};
      std::vector<double> yr = pixel_centres(e.RR, e.dm), xc = pixel_centres(e.CC, e.dm);
      csg_mft_destroy(e.mft2);
      e.mft2 = nullptr;
      int rc = csg_mft_create(c->ctx, &e.mft2, e.RR, e.CC, w.rows, w.pitch, yr.data(), xc.data(),
                              xps.data() + w.r0, xps.data() + w.c0, L, e.lf.data(),
                              e.pref.data(), -1.0, c->precision);
      if (rc) return rc;
      e.win = MftWindow{w.r0, w.c0, n, n};  // output window of the n x n field
    } else if (e.kind == E_FFT_FPM && e.bab == 1) {
      int j = i + 1;
      while (j < ne && is_pointwise(c->elems[j].kind)) ++j;
      MftWindow w = (j < ne && c->elems[j].kind == E_FRAUNHOFER) ? stop_window(c, i, j)
                                                                 : MftWindow{0, 0, n, n};
      const int lo = (e.P - n) / 2;
      std::vector<double> fy(e.bR), fx(e.bC), py(w.rows), px(w.pitch), lf(L, (double)e.P);
      std::vector<double> pref(2 * L, 0.0);
      for (int r = 0; r < e.bR; ++r) fy[r] = e.br0 + r - e.P / 2;
      for (int cc = 0; cc < e.bC; ++cc) fx[cc] = e.bc0 + cc - e.P / 2;
      for (int r = 0; r < w.rows; ++r) py[r] = lo + w.r0 + r;
      for (int cc = 0; cc < w.pitch; ++cc) px[cc] = lo + w.c0 + cc;
      for (int l = 0; l < L; ++l) pref[2 * l] = -1.0 / ((double)e.P * e.P);  // E - ifft(...)
      csg_mft_destroy(e.mft2);
      e.mft2 = nullptr;
      int rc = csg_mft_create(c->ctx, &e.mft2, e.bR, e.bC, w.rows, w.pitch, fy.data(), fx.data(),
                              py.data(), px.data(), L, lf.data(), pref.data(), +1.0,
                              c->precision);
      if (rc) return rc;
      e.win = MftWindow{w.r0, w.c0, n, n};  // output window of the n x n field
    } else if (e.kind == E_FRAUNHOFER) {
      int k = i - 1;
      while (k >= 0 && is_pointwise(c->elems[k].kind)) --k;
      const MftWindow w = stop_window(c, k, i);
      std::vector<double> xo = pixel_centres(e.n_out, e.out_pixel);
      csg_mft_destroy(e.mft);
      e.mft = nullptr;
      int rc;
      if (e.n_out_l.empty()) {
        rc = csg_mft_create(c->ctx, &e.mft, w.rows, w.pitch, e.n_out, e.n_out, xp.data() + w.r0,
                            xp.data() + w.c0, xo.data(), xo.data(), L, e.lf.data(),
                            e.pref.data(), -1.0, c->precision);
      } else {  // each wavelength's own grid, centred, at the same pixel scale
        std::vector<double> xr((size_t)L * e.n_out, 0.0);
        for (int l = 0; l < L; ++l) {
          std::vector<double> v = pixel_centres(e.n_out_l[l], e.out_pixel);
          std::copy(v.begin(), v.end(), xr.begin() + (size_t)l * e.n_out);
        }
        rc = csg_mft_create_ragged(c->ctx, &e.mft, w.rows, w.pitch, e.n_out, e.n_out_l.data(),
                                   xp.data() + w.r0, xp.data() + w.c0, xr.data(), xr.data(), L,
                                   e.lf.data(), e.pref.data(), -1.0, c->precision);
      }
      if (rc) return rc;
      e.win = MftWindow{w.r0, w.c0, n, n};  // input window of the n x n field
      e.win_rows = w.rows;
      e.win_cols = w.pitch;
    }
  }
  c->planned = true;
  return CSG_OK;
}

// Batch of n_fields fields: wavelength index, point-source amplitude
// (sqrt(flux)) and tip/tilt (already times magnification), and the candidate
// whose sags drive the hex FPM (efield.cpp:179-206, :295-304).
int csg_chain_set_batch(csg_chain* c, int n_fields, const int* lambda_idx, const double* amp,
                        const double* tip, const double* tilt, const int* cand) {
  CSG_CHECK(c && lambda_idx && amp && tip && tilt && cand, CSG_E_ARG,
            "csg_chain_set_batch: null argument");
  CSG_CHECK(n_fields > 0 && n_fields < 65536, CSG_E_SHAPE, "csg_chain_set_batch: bad batch size");
  for (int f = 0; f < n_fields; ++f)
    CSG_CHECK(lambda_idx[f] >= 0 && lambda_idx[f] < c->n_lambda && cand[f] >= 0, CSG_E_ARG,
              "csg_chain_set_batch: wavelength index or candidate out of range");
  DeviceGuard g(c->ctx->device);
  cudaStream_t st = c->ctx->stream;
  CSG_CUDA(cudaStreamSynchronize(st));
  if (n_fields > c->cap_fields) {
    for (void* p : {(void*)c->slot, (void*)c->lam_f, (void*)c->amp, (void*)c->tip,
                    (void*)c->tilt, (void*)c->cand, (void*)c->ident, (void*)c->field})
      cudaFree(p);
    c->slot = dev_copy<int>(nullptr, n_fields, st);
    c->lam_f = dev_copy<double>(nullptr, n_fields, st);
    c->amp = dev_copy<double>(nullptr, n_fields, st);
    c->tip = dev_copy<double>(nullptr, n_fields, st);
    c->tilt = dev_copy<double>(nullptr, n_fields, st);
    c->cand = dev_copy<int>(nullptr, n_fields, st);
    c->ident = dev_copy<int>(nullptr, n_fields, st);
    c->field = dev_copy<float>(nullptr, (size_t)n_fields * 2 * c->n * c->n, st);
    CSG_CHECK(c->slot && c->lam_f && c->amp && c->tip && c->tilt && c->cand && c->ident &&
                  c->field,
              CSG_E_NOMEM, "csg_chain_set_batch: allocation failed");
    c->cap_fields = n_fields;
  }
  std::vector<double> lam(n_fields);
  std::vector<int> id(n_fields);
  for (int f = 0; f < n_fields; ++f) {
    lam[f] = c->lambda[lambda_idx[f]];
    id[f] = f;
  }
  CSG_CUDA(cudaMemcpyAsync(c->slot, lambda_idx, n_fields * sizeof(int), cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(c->lam_f, lam.data(), n_fields * sizeof(double), cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(c->amp, amp, n_fields * sizeof(double), cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(c->tip, tip, n_fields * sizeof(double), cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(c->tilt, tilt, n_fields * sizeof(double), cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(c->cand, cand, n_fields * sizeof(int), cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(c->ident, id.data(), n_fields * sizeof(int), cudaMemcpyHostToDevice, st));
  CSG_CUDA(cudaStreamSynchronize(st));
  c->n_fields = n_fields;
  drop_graph(c);
  return CSG_OK;
}

// Device FP64 arrays [n_fields] of the batch's source amplitude, tip and tilt:
// writing them in place between executions changes the sources without a new
// batch (or a new graph).
int csg_chain_batch_buffers(csg_chain* c, double** amp, double** tip, double** tilt) {
  CSG_CHECK(c, CSG_E_ARG, "csg_chain_batch_buffers: null chain");
  CSG_CHECK(c->n_fields > 0, CSG_E_STATE, "csg_chain_batch_buffers: no batch");
  if (amp) *amp = c->amp;
  if (tip) *tip = c->tip;
  if (tilt) *tilt = c->tilt;
  return CSG_OK;
}

// Device buffer of candidate sags [n_cand][n_hex] (FP64 metres), allocated on
// first use; the caller (or the DE kernels) writes it in place.
int csg_chain_sags(csg_chain* c, int n_cand, int n_hex, double** dev_sags) {
  CSG_CHECK(c && dev_sags && n_cand > 0 && n_hex > 0, CSG_E_ARG, "csg_chain_sags: bad argument");
  DeviceGuard g(c->ctx->device);
  if (!c->sags || n_cand != c->n_cand || n_hex != c->sag_hex) {
    cudaStreamSynchronize(c->ctx->stream);
    cudaFree(c->sags);
    c->sags = dev_copy<double>(nullptr, (size_t)n_cand * n_hex, c->ctx->stream);
    CSG_CHECK(c->sags, CSG_E_NOMEM, "csg_chain_sags: allocation failed");
    CSG_CUDA(cudaMemsetAsync(c->sags, 0, sizeof(double) * n_cand * n_hex, c->ctx->stream));
    c->n_cand = n_cand;
    c->sag_hex = n_hex;
    drop_graph(c);
  }
  *dev_sags = c->sags;
  return CSG_OK;
}

static int prepare(csg_chain* c) {
  int prc = build_plans(c);
  if (prc) return prc;
  const size_t F = (size_t)c->n_fields;
  size_t fpm_need = 0, ph_need = 0, img_need = 0, pad_need = 0;
  for (auto& e : c->elems) {
    if (e.kind == E_FRESNEL && fft_is_dft_size(c->n)) {
      // a size that is not a power of two: the Fresnel runs as DFT transforms
      const int rc = dft_prepare(c->ctx, c->n, c->n_fields, c->precision == CSG_PREC_HIGH);
      if (rc) return rc;
    } else if (e.kind == E_FPM_HEX) {
      fpm_need = std::max(fpm_need, F * 2 * e.RR * e.CC * sizeof(float));
      ph_need = std::max(ph_need, F * (e.n_hex + 1) * sizeof(float2));
      int rc = csg_mft_reserve(e.mft1, c->n_fields);
      if (!rc) rc = csg_mft_reserve(e.mft2, c->n_fields);
      if (rc) return rc;
    } else if (e.kind == E_FFT_FPM && e.bab == 1) {
      fpm_need = std::max(fpm_need, F * 2 * (size_t)e.bR * e.bC * sizeof(float));
      int rc = csg_mft_reserve(e.mft1, c->n_fields);
      if (!rc) rc = csg_mft_reserve(e.mft2, c->n_fields);
      if (rc) return rc;
    } else if (e.kind == E_FPM_MASK) {
      fpm_need = std::max(fpm_need, F * 2 * (size_t)e.RR * e.CC * sizeof(float));
      int rc = csg_mft_reserve(e.mft1, c->n_fields);
      if (!rc) rc = csg_mft_reserve(e.mft2, c->n_fields);
      if (rc) return rc;
    } else if (e.kind == E_FPM_HEX_DOUBLE) {
      fpm_need = std::max(fpm_need, F * 2 * (size_t)e.RR * e.CC * sizeof(float));
      ph_need = std::max(ph_need, F * (e.n_hex + 1) * sizeof(float2));
      pad_need = std::max(pad_need, F * 2 * (size_t)e.nz * e.nz * sizeof(float));  // zoom grid
      int rc = csg_mft_reserve(e.mft1, c->n_fields);
      if (!rc) rc = csg_mft_reserve(e.mft2, c->n_fields);
      if (!rc) rc = csg_mft_reserve(e.mft3, c->n_fields);
      if (rc) return rc;
    } else if (e.kind == E_FFT_FPM && e.bab == 0) {
      pad_need = std::max(pad_need, F * 2 * (size_t)e.P * e.P * sizeof(float));
    } else if (e.kind == E_FRAUNHOFER) {
      img_need = std::max(img_need, F * 2 * e.n_out * e.n_out * sizeof(float));
      int rc = csg_mft_reserve(e.mft, c->n_fields);
      if (rc) return rc;
    }
  }
  size_t mask_cap = c->fpm_cap;
  int rc = ensure_buf(&c->fpm, c->fpm_cap, fpm_need);
  if (!rc) rc = ensure_buf(&c->fpm_mask, mask_cap, fpm_need);
  if (!rc) rc = ensure_buf(reinterpret_cast<float**>(&c->phasors), c->ph_cap, ph_need);
  if (!rc) rc = ensure_buf(&c->image, c->img_cap, img_need);
  if (!rc && c->precision == CSG_PREC_HIGH) rc = ensure_buf(&c->image_lo, c->img_lo_cap, img_need);
  if (!rc) rc = ensure_buf(&c->padbuf, c->pad_cap, pad_need);
  return rc;
}

// The walk as fused passes: elementwise elements (the point source, masks,
// mirrors, complex masks) never get a pass of their own when a transform can
// carry them. Ops before a Fresnel propagation ride in its first row pass,
// ops right after it in its last row pass, ops before the final MFT in its
// operand split; only ops with no such neighbour get one standalone pass.
struct Step {
  enum Kind { PIX, FRESNEL, FPM, FINAL, FFT_FPM, FPM_DOUBLE } kind;
  PixOps pro, epi;
  const Elem* e = nullptr;
  int sup0 = 0, sup1 = 1 << 30;  // FRESNEL: rows that can be nonzero on input
  bool calib = false;            // FPM with a fixed mask: apply its calibration mask
  // FRESNEL followed by a hex FPM: the last row pass also writes the FPM's
  // forward-transform operand split (split_to), and the FPM skips its split
  csg_mft* split_to = nullptr;
  bool presplit = false;
};

static bool push_op(PixOps& o, int kind, const float* a, const float* b, float param, int mr,
                    int mc) {
  if (o.n >= MAX_PIXOPS) return false;
  o.kind[o.n] = kind;
  o.a[o.n] = a;
  o.b[o.n] = b;
  o.param[o.n] = param;
  o.mr[o.n] = mr;
  o.mc[o.n] = mc;
  ++o.n;
  return true;
}

static std::vector<Step> plan_walk(const csg_chain* c, int calibrating) {
  std::vector<Step> prog;
  PixOps pend;
  push_op(pend, OP_SOURCE, nullptr, nullptr, 0.f, 0, 0);
  bool epi_open = false;  // the last step is a Fresnel that can still take ops
  // rows of the field that can be nonzero: real masks applied since the last
  // transform zero everything outside their row support
  int sup0 = 0, sup1 = c->n;
  const size_t ne = c->elems.size();
  for (size_t ei = 0; ei < ne; ++ei) {
    const Elem& e = c->elems[ei];
    // disabled for calibration: skipped, or a fixed-mask FPM's calibration mask
    const bool calib_mask = calibrating && e.disable_for_calibration && e.kind == E_FPM_MASK;
    if (calibrating && e.disable_for_calibration && !(calib_mask && e.cmask)) continue;
    int kind = 0;
    float param = 0.f;
    const float* a = e.a;
    if (e.kind == E_MASK) {
      kind = OP_MASK;
      param = e.quirk ? 1.f : 0.f;
      sup0 = std::max(sup0, e.sr0);
      sup1 = std::min(sup1, e.sr1);
      // a real mask followed by a mirror: one op with the mirror's
      // mask-multiplied phasor table
      if (ei + 1 < ne && c->elems[ei + 1].kind == E_MIRROR && c->elems[ei + 1].tab_m &&
          !(calibrating && c->elems[ei + 1].disable_for_calibration)) {
        kind = OP_PHASOR;
        param = 0.f;
        a = reinterpret_cast<const float*>(c->elems[ei + 1].tab_m);
        ++ei;
      }
    } else if (e.kind == E_MIRROR) {
      kind = OP_PHASOR;  // reads the element's per-wavelength phasor table
      a = reinterpret_cast<const float*>(e.tab);
    } else if (e.kind == E_CMASK) {
      kind = OP_CMASK;
    }
    if (kind) {
      const float* b = kind == OP_PHASOR ? nullptr : e.b;
      if (epi_open && push_op(prog.back().epi, kind, a, b, param, e.mrows, e.mcols)) continue;
      epi_open = false;
      if (!push_op(pend, kind, a, b, param, e.mrows, e.mcols)) {
        Step s{Step::PIX, pend, PixOps(), nullptr};
        prog.push_back(s);
        pend = PixOps();
        push_op(pend, kind, a, b, param, e.mrows, e.mcols);
      }
      continue;
    }
    if (e.kind == E_FRESNEL) {
      Step s{Step::FRESNEL, pend, PixOps(), &e};
      s.sup0 = sup0;
      s.sup1 = sup1;
      prog.push_back(s);
      pend = PixOps();
      epi_open = true;
    } else if (e.kind == E_FPM_HEX) {
      if (pend.n) prog.push_back(Step{Step::PIX, pend, PixOps(), nullptr});
      pend = PixOps();
      prog.push_back(Step{Step::FPM, PixOps(), PixOps(), &e});
      epi_open = false;
    } else if (e.kind == E_FPM_MASK) {
      if (pend.n) prog.push_back(Step{Step::PIX, pend, PixOps(), nullptr});
      pend = PixOps();
      Step s{Step::FPM, PixOps(), PixOps(), &e};
      s.calib = calib_mask;
      prog.push_back(s);
      epi_open = false;
    } else if (e.kind == E_FPM_HEX_DOUBLE) {
      prog.push_back(Step{Step::FPM_DOUBLE, pend, PixOps(), &e});  // ops ride in its split
      pend = PixOps();
      epi_open = false;
    } else if (e.kind == E_FFT_FPM) {
      prog.push_back(Step{Step::FFT_FPM, pend, PixOps(), &e});  // ops ride in the padding pass
      pend = PixOps();
      epi_open = false;
    } else if (e.kind == E_FRAUNHOFER) {
      prog.push_back(Step{Step::FINAL, pend, PixOps(), &e});
      pend = PixOps();
      epi_open = false;
    }
    sup0 = 0;  // after a transform every row can be nonzero
    sup1 = c->n;
  }
  if (pend.n) prog.push_back(Step{Step::PIX, pend, PixOps(), nullptr});
  // a Fresnel straight before a hex FPM hands over its result already split
  const char* env = getenv("CSG_FRESNEL_SPLIT");
  if (!(env && env[0] == '0'))
    for (size_t i = 0; i + 1 < prog.size(); ++i)
      if (prog[i].kind == Step::FRESNEL && prog[i + 1].kind == Step::FPM) {
        int ny = 0, nx = 0;
        mft_input_shape(prog[i + 1].e->mft1, &ny, &nx);
        if (ny == c->n && nx == c->n && !mft_is_high(prog[i + 1].e->mft1) &&
            !fft_is_dft_size(c->n)) {
          prog[i].split_to = prog[i + 1].e->mft1;
          prog[i + 1].presplit = true;
        }
      }
  return prog;
}

// One step of the walk over the chain's first F fields.
static int run_step(csg_chain* c, const Step& s, const FieldInfo& fi, int F) {
  csg_ctx* ctx = c->ctx;
  const int n = c->n;
  int rc = CSG_OK;
  {
    switch (s.kind) {
      case Step::PIX:
        rc = pixops_pass(ctx->stream, c->field, F, n, n, s.pro, fi);
        break;
      case Step::FRESNEL: {
        const bool high = c->precision == CSG_PREC_HIGH;
        FresnelArgs fa{c->lam_f, s.e->z, s.e->ap_rad, s.e->tab, c->slot, s.e->tab4};
        FftBand sup;  // rows a mask left nonzero, widened to the transform's row groups
        __nv_bfloat16* split = nullptr;
        if (s.split_to) {
          split = mft_split_buffer(s.split_to, F);
          CSG_CHECK(split, CSG_E_NOMEM, "Fresnel: FPM operand buffer allocation failed");
        }
        if (!fft_is_dft_size(n) &&
            fft_row_support(n, s.sup0, std::min(s.sup1, n), &sup.lo, &sup.n, high) && sup.n < n)
          rc = fft2d_fused(ctx, c->field, F, n, -1, &fa, s.pro, s.epi, fi, nullptr, &sup, split,
                           high);
        else
          rc = fft2d_fused(ctx, c->field, F, n, -1, &fa, s.pro, s.epi, fi, nullptr, nullptr,
                           split, high);
        break;
      }
      case Step::FPM: {
        const Elem& e = *s.e;
        if (e.kind == E_FPM_MASK) {
          rc = mft_execute_ops(ctx, e.mft1, c->field, c->fpm, F, c->slot, 0, nullptr, nullptr,
                               PixOps(), fi, nullptr, nullptr, nullptr, s.presplit);
          if (!rc)
            rc = mft_execute_ops(ctx, e.mft2, c->fpm, c->field, F, c->slot, e.bab,
                                 s.calib ? e.cmask : e.dmask, c->slot, PixOps(), fi, nullptr,
                                 &e.win);
          break;
        }
        CSG_CHECK(c->sags && c->sag_hex == e.n_hex, CSG_E_STATE,
                  "hex FPM: candidate sags not set (csg_chain_sags) or wrong hex count");
        // (fliplr(M) - 1) for each field's (candidate, wavelength) on the box
        rc = hex_mask_region(ctx, e.hex_id, e.count, e.S, e.r0, e.c0, e.RR, e.CC, e.n_sub,
                             c->sags, e.n_hex, F, c->cand, c->lam_f, e.phase_sign, 1, 1.0,
                             c->fpm_mask, c->phasors);
        if (!rc)
          rc = mft_execute_ops(ctx, e.mft1, c->field, c->fpm, F, c->slot, 0, nullptr, nullptr,
                               PixOps(), fi, nullptr, nullptr, nullptr, s.presplit);
        // E + MFT2[...] on the window of the stops that follow (accumulate)
        if (!rc) rc = mft_execute_ops(ctx, e.mft2, c->fpm, c->field, F, c->slot, 1, c->fpm_mask,
                                      c->ident, PixOps(), fi, nullptr, &e.win);
        break;
      }
      case Step::FINAL:
        rc = mft_execute_ops(ctx, s.e->mft, c->field, c->image, F, c->slot, 0, nullptr, nullptr,
                             s.pro, fi, &s.e->win, nullptr, nullptr, false,
                             c->precision == CSG_PREC_HIGH ? c->image_lo : nullptr);
        break;
      case Step::FPM_DOUBLE: {
        const Elem& e = *s.e;
        const bool hex = e.hex_id != nullptr;
        if (hex) {
          CSG_CHECK(c->sags && c->sag_hex == e.n_hex, CSG_E_STATE,
                    "hex FPM: candidate sags not set (csg_chain_sags) or wrong hex count");
          // M - 1 (no flip) for each field's (candidate, wavelength)
          rc = hex_mask_region(ctx, e.hex_id, e.count, e.S, 0, 0, e.S, e.S, e.n_sub, c->sags,
                               e.n_hex, F, c->cand, c->lam_f, e.phase_sign, 0, 1.0, c->fpm_mask,
                               c->phasors);
        }
        // Z = zoom grid field (the element ops ride in the split)
        if (!rc)
          rc = mft_execute_ops(ctx, e.mft1, c->field, c->padbuf, F, c->slot, 0, nullptr, nullptr,
                               s.pro, fi);
        // E = MFT_out[Z] + MFT_out[(M - 1) Z] over the mask block
        if (!rc)
          rc = mft_execute_ops(ctx, e.mft2, c->padbuf, c->field, F, c->slot, 0, nullptr, nullptr,
                               PixOps(), fi);
        const MftWindow blk{e.zr0, e.zc0, e.nz, e.nz};
        if (!rc)
          rc = mft_execute_ops(ctx, e.mft3, c->padbuf, c->field, F, c->slot, 1,
                               hex ? c->fpm_mask : e.dmask, hex ? c->ident : c->slot, PixOps(),
                               fi, &blk, nullptr);
        break;
      }
      case Step::FFT_FPM: {
        const Elem& e = *s.e;
        if (e.bab) {
          // the element's ops first (the Babinet term subtracts from E itself)
          if (s.pro.n) rc = pixops_pass(ctx->stream, c->field, F, n, n, s.pro, fi);
          if (!rc && e.bab == 1)
            rc = csg_mft_execute(ctx, e.mft1, c->field, c->fpm, F, c->slot, 0, nullptr, nullptr);
          if (!rc && e.bab == 1)
            rc = mft_execute_ops(ctx, e.mft2, c->fpm, c->field, F, c->slot, 1, e.dmask, c->slot,
                                 PixOps(), fi, nullptr, &e.win);
          break;
        }
        const bool high = c->precision == CSG_PREC_HIGH;
        FresnelArgs fa{c->lam_f, 0.0, 1.0, e.tab, c->slot, e.tab4};  // H = the mask table
        const int lo = (e.P - n) / 2;
        if (fft_band_supported(e.P, lo, n, high)) {
          // only the n rows that hold the field are transformed; the padding
          // is generated in registers and the crop is the last pass's store
          rc = pixops_pass(ctx->stream, c->field, F, n, n, s.pro, fi);
          FftBand band;
          band.lo = lo;
          band.n = n;
          band.src = c->field;
          band.dst = c->field;
          if (!rc)
            rc = fft2d_fused(ctx, c->padbuf, F, e.P, -1, &fa, PixOps(), PixOps(), fi, &band,
                             nullptr, nullptr, high);
        } else {
          rc = pad_center_pass(ctx->stream, c->field, c->padbuf, F, n, e.P, s.pro, fi);
          if (!rc)
            rc = fft2d_fused(ctx, c->padbuf, F, e.P, -1, &fa, PixOps(), PixOps(), fi, nullptr,
                             nullptr, nullptr, high);
          if (!rc) rc = crop_center_pass(ctx->stream, c->padbuf, c->field, F, n, e.P);
        }
        break;
      }
    }
  }
  return rc;
}

static int run_walk(csg_chain* c, int calibrating) {
  FieldInfo fi;
  fi.lam = c->lam_f;
  fi.amp = c->amp;
  fi.tip = c->tip;
  fi.tilt = c->tilt;
  fi.slot = c->slot;
  for (const Step& s : plan_walk(c, calibrating)) {
    int rc = run_step(c, s, fi, c->n_fields);
    if (rc) return rc;
  }
  return CSG_OK;
}

// Run the element walk on the current batch. calibrating != 0 skips every
// element added with disable_for_calibration (the reference's calibration
// propagation, regionContrast.cpp:124-143). use_graph != 0 captures the walk
// into a CUDA graph on first use and replays it afterwards.
int csg_chain_execute(csg_chain* c, int calibrating, int use_graph) {
  CSG_CHECK(c, CSG_E_ARG, "csg_chain_execute: null chain");
  CSG_CHECK(c->n_fields > 0, CSG_E_STATE, "csg_chain_execute: no batch (csg_chain_set_batch)");
  DeviceGuard g(c->ctx->device);
  int rc = prepare(c);
  if (rc) return rc;
  if (!use_graph) return run_walk(c, calibrating);
  CSG_CHECK(c->ctx->stream != nullptr, CSG_E_STATE,
            "csg_chain_execute: graph capture needs a non-default stream");
  if (c->exec && c->graph_calib != calibrating) drop_graph(c);
  if (!c->exec) {
    rc = run_walk(c, calibrating);  // warm-up: first-use allocations happen outside capture
    if (rc) return rc;
    CSG_CUDA(cudaStreamSynchronize(c->ctx->stream));
    CSG_CUDA(cudaStreamBeginCapture(c->ctx->stream, cudaStreamCaptureModeThreadLocal));
    rc = run_walk(c, calibrating);
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->ctx->stream, &gr);
    if (rc) {
      if (gr) cudaGraphDestroy(gr);
      return rc;
    }
    CSG_CHECK(e == cudaSuccess, CSG_E_CUDA,
              std::string("graph capture: ") + cudaGetErrorString(e));
    c->graph = gr;
    CSG_CUDA(cudaGraphInstantiate(&c->exec, gr, 0));
    c->graph_calib = calibrating;
  }
  CSG_CUDA(cudaGraphLaunch(c->exec, c->ctx->stream));
  return CSG_OK;
}

}  // extern "C"

// ------------------------------------------------------ response matrix
namespace csg {

// Mask of one response column on the transformed box (makeHexCFpmResponse
// with complexHexMaskFPM's useOnlyThisHex, complexHexMaskFPM.cpp:72-87, all
// sags zero): column h < n_hex keeps the sub-pixel counts of hex h only;
// column n_hex keeps the counts outside every hex and is the Babinet column
// (fliplr(M) - 1, fpmPupToLyot.cpp:444-450). Output [K][2][RR][CC] (real).
__global__ void k_hex_column_mask(const int16_t* __restrict__ hex_id,
                                  const uint16_t* __restrict__ count, int S, int r0, int c0,
                                  int RR, int CC, float inv_nsub2, int n_hex,
                                  const int* __restrict__ col, float* __restrict__ out) {
  const int j = blockIdx.y;
  const int h = col[j];
  const int plane = RR * CC;
  const size_t splane = (size_t)S * S;
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < plane; o += gridDim.x * blockDim.x) {
    const int r = r0 + o / CC, cc = c0 + o % CC;
    const size_t src = (size_t)r * S + (S - 1 - cc);  // fliplr
    float m = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int id = hex_id[k * splane + src];
      if (id == h || (h == n_hex && id < 0)) m += (float)count[k * splane + src];
    }
    float* base = out + (size_t)j * 2 * plane + o;
    base[0] = m * inv_nsub2 - (h == n_hex ? 1.f : 0.f);
    base[plane] = 0.f;
  }
}

// Chunk fields j: the Babinet column starts from the field E (the "+ E" of
// fpmPupToLyot.cpp:155-158), every other column from zero.
__global__ void k_response_init(const float* __restrict__ e0, float* __restrict__ out, int n,
                                const int* __restrict__ col, const int* __restrict__ base,
                                int n_hex) {
  const int j = blockIdx.y;
  const size_t fp = (size_t)2 * n * n;
  const bool bab = col[j] == n_hex;
  const float* src = e0 + (size_t)base[j] * fp;
  float* dst = out + (size_t)j * fp;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < fp;
       i += (size_t)gridDim.x * blockDim.x)
    dst[i] = bab ? src[i] : 0.f;
}

// M[base][pix][col] (complex FP64, interleaved) <- region pixels of the image.
__global__ void k_response_gather(const float* __restrict__ img, int no, const int* __restrict__ pix,
                                  int n_pix, const int* __restrict__ col,
                                  const int* __restrict__ base, int ncol,
                                  double* __restrict__ M) {
  const int j = blockIdx.y;
  const size_t plane = (size_t)no * no;
  const float* re = img + (size_t)j * 2 * plane;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n_pix; p += gridDim.x * blockDim.x) {
    const size_t o = ((size_t)base[j] * n_pix + p) * ncol + col[j];
    M[2 * o] = re[pix[p]];
    M[2 * o + 1] = re[plane + pix[p]];
  }
}

}  // namespace csg

extern "C" {

// makeHexCFpmResponse::compute_response (makeHexCFpmResponse.cpp:91-190) for
// the chain's current batch (each field one (wavelength, source) pair; the
// candidate index is ignored): column h of M for base field b is the final
// image at the region pixels with only hex h in the fpm_index-th hex FPM
// (Babinet off), and column n_hex the Babinet response of the area outside
// the hexes. The walk up to the FPM and its forward transform run once per
// base field; the columns are batched through the return transform and the
// rest of the walk in chunks. m_host: complex<double> interleaved, row-major
// [n_base][n_pix][n_hex + 1] (csg_respobj_create's layout); calib_max: the
// maximum of the calibration intensity summed over the batch
// (makeHexCFpmResponse.cpp:96-113).
int csg_chain_response(csg_chain* c, int fpm_index, const int* pix_idx, int n_pix,
                       double* m_host, double* calib_max) {
  CSG_CHECK(c && pix_idx && m_host && calib_max && n_pix > 0, CSG_E_ARG,
            "csg_chain_response: bad argument");
  CSG_CHECK(c->n_fields > 0, CSG_E_STATE, "csg_chain_response: no batch (csg_chain_set_batch)");
  DeviceGuard g(c->ctx->device);
  csg_ctx* ctx = c->ctx;
  cudaStream_t st = ctx->stream;
  int rc = prepare(c);
  if (rc) return rc;
  const int B = c->n_fields, n = c->n;
  std::vector<Step> prog = plan_walk(c, 0);
  int fi_step = -1, k = 0;
  for (size_t i = 0; i < prog.size(); ++i)
    if (prog[i].kind == Step::FPM && prog[i].e->kind == E_FPM_HEX && k++ == fpm_index)
      fi_step = (int)i;
  CSG_CHECK(fi_step >= 0, CSG_E_ARG, "csg_chain_response: no such hex FPM element");
  for (size_t i = fi_step + 1; i < prog.size(); ++i)
    CSG_CHECK(prog[i].kind == Step::PIX || prog[i].kind == Step::FINAL, CSG_E_STATE,
              "csg_chain_response: only element ops and the final image may follow the FPM");
  CSG_CHECK(prog.back().kind == Step::FINAL, CSG_E_STATE,
            "csg_chain_response: the walk must end in a fraunhoferFocal");
  const Elem& e = *prog[fi_step].e;
  const Elem& fin = *prog.back().e;
  const int no = fin.n_out, ncol = e.n_hex + 1;
  for (int p = 0; p < n_pix; ++p)
    CSG_CHECK(pix_idx[p] >= 0 && pix_idx[p] < no * no, CSG_E_ARG,
              "csg_chain_response: region pixel outside the image");

  // calibration normalisation: max over pixels of sum_fields |E|^2
  rc = run_walk(c, 1);
  if (rc) return rc;
  {
    double* isum = nullptr;
    double* imax = nullptr;
    CSG_CUDA(cudaMalloc(&isum, sizeof(double) * no * no));
    CSG_CUDA(cudaMalloc(&imax, sizeof(double)));
    rc = csg_intensity(ctx, c->image, no, no, B, isum, imax);
    if (!rc) CSG_CUDA(cudaMemcpyAsync(calib_max, imax, sizeof(double), cudaMemcpyDeviceToHost, st));
    CSG_CUDA(cudaStreamSynchronize(st));
    cudaFree(isum);
    cudaFree(imax);
    if (rc) return rc;
  }

  // the walk up to the FPM and its forward transform, once per base field
  FieldInfo fi{c->lam_f, c->amp, c->tip, c->tilt, c->slot};
  for (int i = 0; i < fi_step && !rc; ++i) rc = run_step(c, prog[i], fi, B);
  if (rc) return rc;
  rc = mft_execute_ops(ctx, e.mft1, c->field, c->fpm, B, c->slot, 0, nullptr, nullptr, PixOps(),
                       fi, nullptr, nullptr, nullptr, prog[fi_step].presplit);
  if (rc) return rc;

  // chunks of columns x base fields
  const long long total = (long long)ncol * B;
  const int K = (int)std::min<long long>(total, 128);
  const size_t fbytes = sizeof(float) * 2 * n * n;
  float *e0 = nullptr, *work = nullptr, *mask = nullptr, *img = nullptr;
  double* Md = nullptr;
  int *d_idx = nullptr, *d_pix = nullptr;
  auto cleanup = [&]() {
    for (void* p : {(void*)e0, (void*)work, (void*)mask, (void*)img, (void*)Md, (void*)d_idx,
                    (void*)d_pix})
      cudaFree(p);
  };
  const size_t box = (size_t)e.RR * e.CC;
  if (cudaMalloc(&e0, fbytes * B) != cudaSuccess || cudaMalloc(&work, fbytes * K) != cudaSuccess ||
      cudaMalloc(&mask, sizeof(float) * 2 * box * K) != cudaSuccess ||
      cudaMalloc(&img, sizeof(float) * 2 * no * no * K) != cudaSuccess ||
      cudaMalloc(&Md, sizeof(double) * 2 * (size_t)B * n_pix * ncol) != cudaSuccess ||
      cudaMalloc(&d_idx, sizeof(int) * 6 * K) != cudaSuccess ||
      cudaMalloc(&d_pix, sizeof(int) * n_pix) != cudaSuccess) {
    cudaGetLastError();
    cleanup();
    set_error("csg_chain_response: allocation failed");
    return CSG_E_NOMEM;
  }
  CSG_CUDA(cudaMemcpyAsync(e0, c->field, fbytes * B, cudaMemcpyDeviceToDevice, st));
  CSG_CUDA(cudaMemcpyAsync(d_pix, pix_idx, sizeof(int) * n_pix, cudaMemcpyHostToDevice, st));
  int* d_col = d_idx;
  int* d_base = d_idx + K;
  int* d_slot = d_idx + 2 * K;
  int* d_ident = d_idx + 3 * K;
  double* d_lam = reinterpret_cast<double*>(d_idx + 4 * K);  // 2K ints = K doubles
  std::vector<int> h_slot(B);
  std::vector<double> h_lam(B);
  CSG_CUDA(cudaMemcpyAsync(h_slot.data(), c->slot, sizeof(int) * B, cudaMemcpyDeviceToHost, st));
  CSG_CUDA(cudaMemcpyAsync(h_lam.data(), c->lam_f, sizeof(double) * B, cudaMemcpyDeviceToHost, st));
  CSG_CUDA(cudaStreamSynchronize(st));
  rc = csg_mft_reserve(e.mft2, K);
  if (!rc) rc = csg_mft_reserve(fin.mft, K);
  std::vector<int> hb(4 * K + 2 * K);
  for (long long j0 = 0; j0 < total && !rc; j0 += K) {
    const int nk = (int)std::min<long long>(K, total - j0);
    for (int j = 0; j < nk; ++j) {
      const long long jj = j0 + j;
      const int b = (int)(jj % B), h = (int)(jj / B);
      hb[j] = h;
      hb[K + j] = b;
      hb[2 * K + j] = h_slot[b];
      hb[3 * K + j] = j;
      memcpy(&hb[4 * K + 2 * j], &h_lam[b], sizeof(double));
    }
    CSG_CUDA(cudaMemcpyAsync(d_idx, hb.data(), sizeof(int) * 6 * K, cudaMemcpyHostToDevice, st));
    dim3 gm(grid_for((long long)box, 256, 256), nk);
    k_hex_column_mask<<<gm, 256, 0, st>>>(e.hex_id, e.count, e.S, e.r0, e.c0, e.RR, e.CC,
                                          1.f / (float)(e.n_sub * e.n_sub), e.n_hex, d_col, mask);
    CSG_LAUNCH_CHECK();
    dim3 gi(grid_for((long long)2 * n * n, 256, 512), nk);
    k_response_init<<<gi, 256, 0, st>>>(e0, work, n, d_col, d_base, e.n_hex);
    CSG_LAUNCH_CHECK();
    FieldInfo fk{d_lam, nullptr, nullptr, nullptr, d_slot};
    rc = mft_execute_ops(ctx, e.mft2, c->fpm, work, nk, d_slot, 1, mask, d_ident, PixOps(), fk,
                         nullptr, &e.win, d_base);
    for (size_t i = fi_step + 1; i < prog.size() && !rc; ++i) {
      const Step& s = prog[i];
      if (s.kind == Step::PIX)
        rc = pixops_pass(st, work, nk, n, n, s.pro, fk);
      else
        rc = mft_execute_ops(ctx, s.e->mft, work, img, nk, d_slot, 0, nullptr, nullptr, s.pro,
                             fk, &s.e->win, nullptr);
    }
    if (rc) break;
    dim3 gg(grid_for(n_pix, 256, 64), nk);
    k_response_gather<<<gg, 256, 0, st>>>(img, no, d_pix, n_pix, d_col, d_base, ncol, Md);
    CSG_LAUNCH_CHECK();
    CSG_CUDA(cudaStreamSynchronize(st));  // the host index staging is reused
  }
  if (!rc) {
    cudaError_t ce = cudaMemcpyAsync(m_host, Md, sizeof(double) * 2 * (size_t)B * n_pix * ncol,
                                     cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) {
      set_error(std::string("csg_chain_response: ") + cudaGetErrorString(ce));
      rc = CSG_E_CUDA;
    }
  }
  cudaStreamSynchronize(st);
  cleanup();
  return rc;
}

// Final-plane field of the batch: [F][2][n_out][n_out] fp32 on the device.
int csg_chain_image(csg_chain* c, float** dev_image, int* n_out) {
  CSG_CHECK(c && dev_image && n_out, CSG_E_ARG, "csg_chain_image: null argument");
  *dev_image = c->image;
  *n_out = 0;
  for (auto& e : c->elems)
    if (e.kind == E_FRAUNHOFER) *n_out = e.n_out;
  return CSG_OK;
}

// Fixed-mask FPMs added after this call reproduce the reference's
// calibration-hat behaviour (see the header).
int csg_chain_set_reference_calibration(csg_chain* c, int enable) {
  CSG_CHECK(c, CSG_E_ARG, "csg_chain_set_reference_calibration: null chain");
  c->ref_calibration = enable != 0;
  return CSG_OK;
}

// CSG_PREC_HIGH chains: the low-order words of the final image (the image
// is image + image_lo); null at other precisions.
int csg_chain_image_lo(csg_chain* c, float** dev_image_lo) {
  CSG_CHECK(c && dev_image_lo, CSG_E_ARG, "csg_chain_image_lo: null argument");
  *dev_image_lo = c->precision == CSG_PREC_HIGH ? c->image_lo : nullptr;
  return CSG_OK;
}

// Pupil-plane working field [F][2][n][n] (the field before the final MFT).
int csg_chain_field(csg_chain* c, float** dev_field) {
  CSG_CHECK(c && dev_field, CSG_E_ARG, "csg_chain_field: null argument");
  *dev_field = c->field;
  return CSG_OK;
}

}  // extern "C"
