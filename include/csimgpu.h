/*
 * csimgpu.h - C ABI of the GB300-native csim propagation hot path.
 *
 * Every entry point replaces one reference call on the propagation path; the
 * reference interface it stands in for is cited beside it (paths are relative
 * to the csim source tree). The ABI carries plain pointers and sizes only.
 *
 * Conventions
 *  - Device fields are planar fp32 ("c32p"): for a batch of F fields of
 *    R rows (y) x C cols (x) the layout is [F][2][R][C] (real plane, then
 *    imaginary plane), row-major, x fastest. Row r / column c is the
 *    reference's Armadillo element (r, c) (csim_geom.cpp:203-214: x runs
 *    along columns).
 *  - Host fields handed to the upload/download calls are complex<double>
 *    interleaved, either Armadillo column-major (CSG_LAYOUT_COLMAJOR, the
 *    layout of efield.E[s][p] cubes, efield.hpp:45-52) or row-major.
 *  - Wavelengths, coordinates and phases are passed in FP64.
 *  - Every call returns 0 or a negative CSG_E_* code; csg_last_error() gives
 *    the message of the last failure on the calling thread.
 *  - Calls are asynchronous on the context's stream; csg_sync() waits and
 *    reports device-side failures (bounded waits that ran out).
 */
#ifndef CSIMGPU_H
#define CSIMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define CSG_OK 0
#define CSG_E_ARG (-1)      /* bad pointer / size / enum */
#define CSG_E_SHAPE (-2)    /* unsupported or inconsistent shape */
#define CSG_E_CUDA (-3)     /* CUDA runtime/driver error */
#define CSG_E_TIMEOUT (-4)  /* a device-side bounded wait ran out */
#define CSG_E_NOMEM (-5)    /* device allocation failed */
#define CSG_E_NAN (-6)      /* non-finite host value where a finite one is required */
#define CSG_E_STATE (-7)    /* object used in the wrong state */

#define CSG_LAYOUT_COLMAJOR 0 /* Armadillo cube: (r,c,s) at r + c*R + s*R*C */
#define CSG_LAYOUT_ROWMAJOR 1 /* numpy C order [s][r][c] */

/* MFT precision: number of bf16 cross products kept of the 3-way split.
 * 6 keeps every product down to 2^-16 relative (fp32-class results), 3 keeps
 * x1y1 + x1y2 + x2y1 (about 2^-16 relative error per product). */
#define CSG_PREC_BF16X6 6
#define CSG_PREC_BF16X3 3
/* High precision: the six products of an exponent-aligned split (all values
 * of a 64-wide K group of an operand row share one power-of-two grid, so
 * every tensor-core sum of the leading products is exact) with compensated
 * two-float accumulation across K groups; in a chain, the Fresnel and
 * padded-FFT passes also run in double-float arithmetic, and the final
 * image carries a low-order plane (csg_chain_image_lo). Peak-normalised
 * field errors against FP64 at the 1e-8 level instead of the 1e-7 level. */
#define CSG_PREC_HIGH 16

typedef struct csg_ctx csg_ctx;
typedef struct csg_mft csg_mft;
typedef struct csg_chain csg_chain;
typedef struct csg_respobj csg_respobj;
typedef struct csg_de csg_de;
typedef struct csg_dm csg_dm;
typedef struct csg_mlp csg_mlp;

/* ------------------------------------------------------------ context */
/* One context per host thread: owns a CUDA stream on `device`. No global
 * state (the reference's globalTelescope / globalCoronagraph / initialEfield,
 * telescope.cpp:15, coronagraph.cpp:36, efield.cpp:20, become arguments). */
int csg_create(csg_ctx** ctx, int device);
int csg_destroy(csg_ctx* ctx);
const char* csg_last_error(void);
/* Wait for the context's stream and report CSG_E_TIMEOUT if a kernel gave up
 * on a bounded wait since the last call. */
int csg_sync(csg_ctx* ctx);
/* Cycles a tensor-core transform launched from this context lets one of its
 * roles (operand loads, products, drains) wait for another before it gives
 * up: it then stops, waits out its own operand loads and products, releases
 * its tensor memory and records the failure, which the next csg_sync reports
 * as CSG_E_TIMEOUT (the context stays usable). 0 (the default) is about one
 * second at the GPU's clock, far above any legitimate wait; a small value
 * makes the give-up path testable. Graphs captured before a change keep the
 * value they were captured with. */
int csg_set_wait_budget(csg_ctx* ctx, long long cycles);
/* Run subsequent work on an external stream (a cudaStream_t; NULL is CUDA's
 * default stream). A new context runs on its own non-blocking stream. */
int csg_set_stream(csg_ctx* ctx, void* stream);
void* csg_get_stream(csg_ctx* ctx);
/* Context-owned device memory (freed at csg_destroy if not freed before). */
int csg_alloc(csg_ctx* ctx, size_t bytes, void** dptr);
int csg_free(csg_ctx* ctx, void* dptr);
int csg_memcpy_h2d(csg_ctx* ctx, void* dst, const void* src, size_t bytes);
int csg_memcpy_d2h(csg_ctx* ctx, void* dst, const void* src, size_t bytes);
/* Pipelined readout of a result: src (device) is copied on the context's
 * stream into one of two context-owned staging buffers (a device-to-device
 * copy), and from there to dst (host, pinned for overlap) on a separate copy
 * stream, so the device-to-host transfer overlaps the work queued after this
 * call. dst holds the data after the next csg_sync, which also waits for the
 * copy stream. Not usable inside stream capture. */
int csg_readout_d2h(csg_ctx* ctx, void* dst, const void* src, size_t bytes);
int csg_memset(csg_ctx* ctx, void* dst, int value, size_t bytes);
/* Version string of the library build. */
const char* csg_version(void);
/* Number of kernels the library has launched from host code (all contexts);
 * graph replays launch kernels without host code and are not counted. */
unsigned long long csg_launch_count(void);
/* Per-kernel timing, the device-side counterpart of the reference's
 * per-element wall-clock timers (coronagraph.cpp:183-198, csim -t): when
 * enabled, CUDA events bracket every instrumented launch on the context's
 * stream (never inside graph capture). csg_profile_report writes
 * {"kernel": {"count", "ms", "flops", "bytes"}} JSON, flops/bytes being the
 * algorithmic work of those launches. */
int csg_profile(csg_ctx* ctx, int enable);
int csg_profile_report(csg_ctx* ctx, char* buf, size_t len);

/* ---------------------------------------------------- field transfer */
/* Upload n_fields complex<double> fields (host, interleaved) of rows x cols
 * into planar fp32 device fields. Replaces the implicit residency of
 * efield.E[s][p] cubes (efield.hpp:45-52); `layout` is CSG_LAYOUT_*.
 * `staging` is a device scratch of >= n_fields*rows*cols*16 bytes. */
int csg_field_upload(csg_ctx* ctx, const double* host, int layout, int rows, int cols,
                     int n_fields, void* staging, float* dev_field);
int csg_field_download(csg_ctx* ctx, const float* dev_field, int rows, int cols, int n_fields,
                       void* staging, double* host, int layout);

/* ------------------------------------------------------ field sources */
/* efield::init_point_sources (efield.cpp:179-206) with the pointSource
 * setter's sqrt(flux) and magnification scaling (efield.cpp:295-304):
 * E_f = amp_f * exp(2 pi i (2 x tip_f / Lx + 2 y tilt_f / Ly)) on the
 * pixel-centre grid x_c = -(C dx - dx)/2 + c dx (csim_geom.cpp:113-142).
 * amp/tip/tilt are per field (tip/tilt already multiplied by magnification). */
int csg_point_source(csg_ctx* ctx, float* field, int n_fields, int rows, int cols,
                     double dx, double dy, const double* amp, const double* tip,
                     const double* tilt);

/* ------------------------------------------------------ field elements */
/* mask::execute (mask.cpp:23-51): E *= m (real mask, fp32 [rows][cols]).
 * ref_quirk != 0 multiplies by (m + i m) as the reference does
 * (cxMaskMat.set_real(m); set_imag(m), mask.cpp:53-58). */
int csg_mask_real(csg_ctx* ctx, float* field, int n_fields, int rows, int cols,
                  const float* mask, int ref_quirk);
/* mirror::execute / deformableMirror::execute (mirror.cpp:23-49, :66-72;
 * deformableMirror.cpp:22-45): E *= exp(-sign 4 pi i sag / lambda_f).
 * sag is fp32 metres [rows][cols]; the phase is reduced in turns in FP64
 * per pixel before the fp32 sincos. lambda is per field. */
int csg_phase_screen(csg_ctx* ctx, float* field, int n_fields, int rows, int cols,
                     const float* sag, const double* lambda, double sign);
/* complexMask::execute (complexMask.cpp:24-55): centred sub-array
 * E[r0+r][c0+c] *= amp exp(-i ph), r0 = rows/2 - mrows/2. */
int csg_complex_mask(csg_ctx* ctx, float* field, int n_fields, int rows, int cols,
                     const float* amp, const float* ph, int mrows, int mcols);

/* ------------------------------------------------------ 2-D transforms */
/* fft::execute / ifft::execute on a square N x N slice (csim_fft.cpp:62-95,
 * :127, :192-193): forward exp(-i), inverse exp(+i) divided by N^2.
 * N a power of two in [64, 4096] (register-resident FFT passes), or any other
 * multiple of 8 up to 8192, which FFTW plans as well (csim_fft.cpp:111-115):
 * those run as an exact-phase DFT matrix product on the tensor cores (O(N^3);
 * the first call for a size builds and keeps its plans in the context).
 * direction: -1 forward, +1 inverse. */
int csg_fft2d(csg_ctx* ctx, float* field, int n_fields, int n, int direction);
/* csg_fft2d with a precision: CSG_PREC_HIGH runs the passes in two-float
 * arithmetic (about 48-bit intermediates; fields stay fp32 in memory). */
int csg_fft2d_prec(csg_ctx* ctx, float* field, int n_fields, int n, int direction,
                   int precision);
/* fresnelPropagateAS::execute (csim_fft.cpp:371-392): per field
 * E <- IFFT(FFT(E) exp(i 2 pi / lambda_f z sqrt(1 - (lambda_f/apRad)^2 H / 4))),
 * H = fftshifted integer frequency index squared. One fused pipeline:
 * row FFT, column FFT x transfer x column IFFT, row IFFT. */
int csg_fresnel(csg_ctx* ctx, float* field, int n_fields, int n, const double* lambda,
                double ap_rad, double z);
/* csg_fresnel with a precision: CSG_PREC_HIGH evaluates the transfer function
 * in FP64 and runs the three passes in two-float arithmetic (fields stay fp32
 * in memory); it allocates a per-call table of n_fields * n^2 * 16 bytes and
 * returns after the work is done. Other precisions are csg_fresnel. Sizes
 * that are not powers of two propagate E' = c (E + IDFT[DFT(E) (H/c - 1)]),
 * c = exp(2 pi i z / lambda_f), with the DFT products of csg_fft2d: about
 * 3e-7 of the field peak in every precision. */
int csg_fresnel_prec(csg_ctx* ctx, float* field, int n_fields, int n, const double* lambda,
                     double ap_rad, double z, int precision);

/* ------------------------------------------------------------------ MFT */
/* Matrix Fourier transform plan: the reference's zoomFft (csim_fft.cpp:
 * 670-708 init, 786-826 execute; Bluestein CZT 422-665) evaluated as
 *   out[v][u] = pref_s * sum_{y,x} in[y][x] exp(sgn 2 pi i (xin_x xout_u + yin_y yout_v) / lf_s)
 * with one (lf, pref) per operator slot s (one slot per wavelength).
 * zoomFft semantics: sgn = -1, pref = dxin dyin / (i lf).
 * The two contractions run on tcgen05 tensor cores with a three-way bf16
 * split of both operands and fp32 accumulation; `precision` is CSG_PREC_*.
 * Coordinates are FP64 vectors (xin: n_in_x, yin: n_in_y, xout: n_out_x,
 * yout: n_out_y); pref is interleaved (re, im) per slot. */
int csg_mft_create(csg_ctx* ctx, csg_mft** plan, int n_in_y, int n_in_x, int n_out_y,
                   int n_out_x, const double* yin, const double* xin, const double* yout,
                   const double* xout, int n_slots, const double* lf, const double* pref,
                   double sgn, int precision);
/* Ragged plan: per-wavelength focal grids of different sizes in one launch
 * (zoomFft output grows with lambda at fixed pixel scale). Slot s maps to an
 * n_out[s] x n_out[s] grid whose coordinates are yout/xout[s][0..n_out[s])
 * (arrays [n_slots][n_out_max]); the plan's outputs are n_out_max^2 planes
 * holding slot s's transform in the leading n_out[s] rows and columns and
 * zeros elsewhere. */
int csg_mft_create_ragged(csg_ctx* ctx, csg_mft** plan, int n_in_y, int n_in_x, int n_out_max,
                          const int* n_out, const double* yin, const double* xin,
                          const double* yout, const double* xout, int n_slots, const double* lf,
                          const double* pref, double sgn, int precision);
int csg_mft_destroy(csg_mft* plan);
/* Transform n_fields planar fields (in: [F][2][n_in_y][n_in_x]) into
 * out ([F][2][n_out_y][n_out_x]); slot[f] picks the operator slot of field f
 * (device int array). accumulate != 0 adds into out (the Babinet "+ E" of
 * fpmPupToLyot.cpp:155-158). `in_mul` (optional, planar complex
 * [n_mul][2][n_in_y][n_in_x], field f uses mul index mul_idx[f]) multiplies
 * the input first (the focal-plane mask of doubleFraunhoferFPM /
 * fpmPupToLyot). */
int csg_mft_execute(csg_ctx* ctx, csg_mft* plan, const float* in, float* out, int n_fields,
                    const int* slot, int accumulate, const float* in_mul, const int* mul_idx);
/* csg_mft_execute of a CSG_PREC_HIGH plan that also stores the low-order
 * words of its two-float results: the transform is out + out_lo (both
 * [F][2][n_out_y][n_out_x] fp32), about 2^-24 closer to exact than out
 * alone. No accumulation or input multiplier. */
int csg_mft_execute_lo(csg_ctx* ctx, csg_mft* plan, const float* in, float* out, float* out_lo,
                       int n_fields, const int* slot);
/* Bytes of device scratch the plan uses for n_fields (informational). */
size_t csg_mft_workspace_bytes(csg_mft* plan, int n_fields);

/* ---------------------------------------------------------- hex FPM */
/* complexHexMaskFPM::make_complex_intpolated_mask (complexHexMaskFPM.cpp:
 * 44-99) for a batch of (candidate, wavelength) masks:
 *   M = sum_{k<3} n[k] exp(i phaseSign 4 pi sag[id[k]] / lambda) / nSub^2
 * with sag 0 where id < 0. Tables: hex_id int16 [3][S][S], count uint16
 * [3][S][S] (the reference's interpHexNum / interpNSubPix cubes).
 * sags: [n_cand][n_hex] FP64. For output j: candidate cand[j], wavelength
 * lambda[j]; out is planar [n_out][2][S][S] holding fliplr(M) - subtract
 * (fpmIntHexCMCForPupToLyot::set_fpmMatAmp, fpmPupToLyot.cpp:441-451:
 * flip = 1, subtract = 1 for the Babinet form). use_only_hex selects one
 * hex as the reference's useOnlyThisHex (-1 = all; n_hex = outside only). */
int csg_hex_mask(csg_ctx* ctx, const int16_t* hex_id, const uint16_t* count, int S, int n_sub,
                 const double* sags, int n_hex, int n_out, const int* cand, const double* lambda,
                 double phase_sign, int flip, double subtract, int use_only_hex, float* out);
/* csg_hex_mask for callers that cannot let the library allocate device
 * memory (no counterpart in the reference, which computes masks on the
 * CPU). Same arguments and results as csg_hex_mask; its per-call scratch is a
 * fixed device array of CSG_HEX_NOALLOC_MAX_PHASORS complex values (2 MiB,
 * held by every GPU that loads the library until the process exits), so
 * n_out * (n_hex + 1) must not exceed that, else CSG_E_SHAPE. It calls no
 * cudaMalloc/cudaFree. The first call on a device looks up the array's
 * device address (a one-time set-up); make that first call before any stream
 * capture. All calls share the one array: calls whose work overlaps on the
 * GPU (different streams or contexts on one device) race and must be
 * ordered by the caller. The array's device address is looked up once per
 * device and kept for the process; after cudaDeviceReset it is no longer
 * valid, so a process that resets a device must not call this again on it. */
#define CSG_HEX_NOALLOC_MAX_PHASORS 262144
int csg_hex_mask_noalloc(csg_ctx* ctx, const int16_t* hex_id, const uint16_t* count, int S,
                         int n_sub, const double* sags, int n_hex, int n_out, const int* cand,
                         const double* lambda, double phase_sign, int flip, double subtract,
                         int use_only_hex, float* out);
/* Build the interpolation tables on the GPU (complexHexMaskFPM.cpp:317-469,
 * make_hex_array + make_interpolation_data). Hex centres (hex_x, hex_y,
 * device FP64) are in hex-step units; `pitch` is the centre distance of
 * neighbouring hexes in those units (sqrt(3) for the reference's own
 * layout, complexHexMaskFPM.cpp:236-315, which reproduces its hexRadius
 * formula exactly). Design array A x A, mask S x S at pixel_scale, n_sub^2
 * samples per mask pixel. Where hexes overlap the highest index wins; a
 * fourth distinct hex in one pixel is counted as outside and reported in
 * *n_overflow (the reference asserts). reference_single_thread != 0
 * reproduces the reference's tables as its loop produces them on one OpenMP
 * thread: the on-array check of each cell after a row's first passing cell
 * uses the row index left by the previous cell's last sub-sample
 * (complexHexMaskFPM.cpp:395-423), which drops the cells of the rows whose
 * last sub-samples fall off the design array (only where hexes reach the
 * array's edge does this change a table value); 0 checks every cell at its
 * midpoint. Synchronous. */
int csg_hex_tables(csg_ctx* ctx, const double* hex_x, const double* hex_y, int n_hex,
                   int n_rings, int design_size, double fpm_scale_factor, double hex_gap,
                   double pitch, int S, int n_sub, double pixel_scale, double fpm_radius,
                   int16_t* hex_id, uint16_t* count, int* n_overflow,
                   int reference_single_thread);

/* ------------------------------------------------- coronagraph chain */
/* Batched element walk: coronagraph::init (coronagraph.cpp:50-168) builds the
 * element list; coronagraph::execute (coronagraph.cpp:175-200) runs it. Here
 * the list is built with the csg_chain_add_* calls (in optical order) and one
 * csg_chain_execute runs every element once over a whole batch of fields,
 * each field one (wavelength, source, candidate) triple. The field is
 * N x N (N a multiple of 8 in [64, 4096]; a Fresnel element at a size that
 * is not a power of two runs as DFT products, see csg_fft2d) at pixel_scale
 * metres; lambda[n_lambda] are the
 * efield's wavelengths (efield.cpp:351-417). `precision` is CSG_PREC_*. */
int csg_chain_create(csg_ctx* ctx, csg_chain** chain, int n, double pixel_scale, int n_lambda,
                     const double* lambda, int precision);
int csg_chain_destroy(csg_chain* chain);
/* mask (mask.cpp:23-58): host fp32 N x N; ref_quirk as csg_mask_real.
 * disable_for_calibration as celem's flag (celem.cpp:63-130). */
int csg_chain_add_mask(csg_chain* chain, const float* mask, int ref_quirk,
                       int disable_for_calibration);
/* mirror (mirror.cpp:23-72): host fp32 sag N x N in metres, mirrorSign. */
int csg_chain_add_mirror(csg_chain* chain, const float* sag, double sign);
/* fresnelPropagator (fresnelPropagator.cpp:23-61, no padding): z =
 * propagationSign |next.position - prev.position|, ap_rad = the efield's
 * arrayRadiusPhysical (efield.cpp:419-430). */
int csg_chain_add_fresnel(csg_chain* chain, double z, double ap_rad);
/* fresnelPropagator with padFactor (fresnelPropagator.cpp:41-54): the field
 * is embedded at the centre of a 2N x 2N zero array, propagated with aperture
 * radius pad_factor ap_rad (the reference's padded array is 2N for any
 * padFactor other than 1) and cropped back; pad_factor 1 is
 * csg_chain_add_fresnel. 2N at most 4096. */
int csg_chain_add_fresnel_padded(csg_chain* chain, double z, double ap_rad, double pad_factor);
/* complexMask (complexMask.cpp:24-66): centred amp exp(-i ph), host fp32. */
int csg_chain_add_complex_mask(csg_chain* chain, const float* amp, const float* ph, int mrows,
                               int mcols, int disable_for_calibration);
/* doubleFraunhoferFPM (doubleFraunhoferFPM.cpp:23-110): as
 * csg_chain_add_fpm_hex_double with a fixed complex mask (host fp32,
 * rows x cols, multiples of 8; mask_im may be null) on the centred block and
 * a zoom-grid pixel per wavelength, zoom_pixel[l] (the reference's dxprime =
 * 2 (beamRadius / (pixelScale N zoomFactor)) lambda 80). */
int csg_chain_add_fpm_double_mask(csg_chain* chain, const float* mask_re, const float* mask_im,
                                  int rows, int cols, const double* zoom_pixel,
                                  double pad_factor, double lf_factor,
                                  int disable_for_calibration);
/* fpmPupToLyot with a fixed focal-plane mask: the fpmCMCForPupToLyot
 * (fpmPupToLyot.cpp:303-367) and fpmBinaryForPupToLyot (:521-557) adapters,
 * in the same matrix-Fourier form as csg_chain_add_fpm_hex:
 *   babinet != 0:  E <- E + c MFT2[(M - 1) MFT1[E]]   (CMC with doBabinet)
 *   babinet == 0:  E <- c MFT2[M MFT1[E]]             (binary, CMC without)
 * mask_re / mask_im (host, mask_im may be null): the reference's mask cube
 * [n_mask][rows][cols] (complexMaskCube), of which slice mask_index is
 * applied at every wavelength (maskIndex, fpmPupToLyot.cpp:355-360; -1, the
 * reference's default, takes slice 0); pixel mask_pixel (maskGeom.set_xy(mask,
 * pixel)), rows and cols multiples of 8; lf: the lambdaFocalLength of each
 * wavelength (fRatioSign lambda focalRatio 2 beamRadius for the CMC,
 * fRatioSign lambda primaryfLength for the binary mask); c = zoomFftSign
 * mask_pixel^2 dx^2 / (fRatioSign lf^2). calib_re / calib_im ([rows][cols],
 * may be null: a mask of ones, the CMC's fpmMatAmpCalib): the mask the
 * calibration walk applies when disable_for_calibration is set (the binary
 * adapter's calibMat), at every wavelength unless
 * csg_chain_set_reference_calibration is on. */
int csg_chain_add_fpm_mask(csg_chain* chain, const float* mask_re, const float* mask_im,
                           int n_mask, int mask_index, int rows, int cols, double mask_pixel,
                           const double* lf,
                           double f_ratio_sign, double zoom_fft_sign, int babinet,
                           const float* calib_re, const float* calib_im,
                           int disable_for_calibration);
/* doubleFraunhoferInterpFPM with complexHexMaskFPM
 * (doubleFraunhoferInterpFPM.cpp:24-65, init_geom :86-121;
 * complexHexMaskFPM.cpp:25-42): zoom FFT of the field to a zoom grid of
 * pad_factor N pixels of size fpm_scale at coordinates (i - n/2) fpm_scale
 * with lambda f = lf_factor lambda (3.52 in the reference), the S x S
 * interpolated hex mask M (candidate sags, no flip) multiplied onto the
 * centred block of that grid, and the zoom FFT back at -lf_factor lambda.
 * Computed as Z = MFT_in[E]; E <- MFT_out[Z] + MFT_out,box[(M - 1) Z_box]:
 * three split-bf16 transforms, the last accumulating. Tables as
 * csg_hex_mask; S a multiple of 8, pad_factor N a multiple of 8 and >= S. */
int csg_chain_add_fpm_hex_double(csg_chain* chain, const int16_t* hex_id, const uint16_t* count,
                                 int S, int n_sub, int n_hex, double fpm_scale, double pad_factor,
                                 double lf_factor, double phase_sign,
                                 int disable_for_calibration);
/* fpmPupToLyot + fpmIntHexCMCForPupToLyot + complexHexMaskFPM
 * (fpmPupToLyot.cpp:24-167, 419-455; complexHexMaskFPM.cpp:44-99) in
 * matrix-Fourier Babinet form, algebraically identical to the reference's
 * 2N circular convolution:
 *   E <- E + c MFT2[(fliplr(M_cand,lambda) - 1) MFT1[E]]
 * lf' = fRatioSign lambda focalRatio 2 beamRadius, mask pixel dm (the hex
 * mask's pixelScale), c = zoomFftSign dm^2 dx^2 / (fRatioSign lf'^2).
 * Tables (host) as csg_hex_mask; candidate sags come from csg_chain_sags. */
int csg_chain_add_fpm_hex(csg_chain* chain, const int16_t* hex_id, const uint16_t* count, int S,
                          int n_sub, int n_hex, double dm, double focal_ratio, double beam_radius,
                          double f_ratio_sign, double zoom_fft_sign, double phase_sign,
                          int disable_for_calibration);
/* The reference computes the calibration mask's transform once, for the
 * first wavelength its loop reaches, and leaves the other wavelengths' with
 * a zero transform (fftMaskHatCalibComputed, fpmPupToLyot.cpp:56, 86-92).
 * With a Babinet mask (hex, CMC with doBabinet) the calibration mask is
 * 1 - 1 = 0 at every wavelength, so nothing changes; without Babinet (the
 * binary adapter, CMC without doBabinet) the calibration field of every
 * wavelength but the first is zero there. This library calibrates every
 * wavelength with its own transform by default; enable != 0 makes fixed-mask
 * FPMs added after this call reproduce the reference (first wavelength
 * only, the result of its loop on one thread). Default 0. */
int csg_chain_set_reference_calibration(csg_chain* chain, int enable);
/* Hex FPMs added after this call transform only the bounding box of the
 * support of fliplr(M) - 1 (rounded out to multiples of 128): M = 1 wherever
 * no hex covers a mask pixel, for any sags, so the Babinet term is exactly
 * the full-grid one. enable = 0 transforms the whole S x S grid. Default 1. */
int csg_chain_set_support_crop(csg_chain* chain, int enable);
/* The box [r0, r0 + rows) x [c0, c0 + cols) of the idx-th hex FPM element. */
int csg_chain_fpm_region(csg_chain* chain, int idx, int* r0, int* c0, int* rows, int* cols);
/* Padded-FFT focal-plane mask, the plain Lyot coronagraph's occulter (the
 * fpmPupToLyot pattern of fpmPupToLyot.cpp:112-161 with an FFT-sampled mask,
 * without Babinet): E <- crop_n(ifft_pad(mask_lambda . fft_pad(embed_pad(E)))).
 * mask_re / mask_im (may be null): host fp32 [n_lambda][pad][pad] in centred
 * focal coordinates (index pad/2 is zero frequency); pad a power of two >= N. */
int csg_chain_add_fft_fpm(csg_chain* chain, int pad, const float* mask_re, const float* mask_im,
                          int disable_for_calibration);
/* Padded-FFT occulters added after this call run in Babinet form when
 * 1 - mask is nonzero only on a box of at most 1/16 of the pad x pad grid
 * (sides rounded up to multiples of 8): E - crop(ifft((1 - M) fft(embed(E))))
 * with both transforms evaluated as exact DFT sums over the box's
 * frequencies (two MFTs, the return one writing only the window of the stops
 * that follow, as for hex FPMs); a mask of ones is the identity. enable = 0
 * keeps the padded FFT. Default 1. */
int csg_chain_set_fft_fpm_babinet(csg_chain* chain, int enable);
/* fraunhoferFocal (fraunhoferFocal.cpp:23-72): zoomFft to n_out x n_out at
 * out_pixel (= loD / samplesPerflD), lambda f = lambda lf_scale with
 * lf_scale = 2 beamRadius primaryfRatio. Must be the last element. */
int csg_chain_add_fraunhofer(csg_chain* chain, int n_out, double out_pixel, double lf_scale);
/* fraunhoferFocal with a per-wavelength output size n_out[n_lambda] at the
 * same out_pixel (a ragged batch, one launch): images are n_max^2 planes
 * holding wavelength l's n_out[l]^2 image in their leading rows and columns. */
int csg_chain_add_fraunhofer_ragged(csg_chain* chain, const int* n_out, double out_pixel,
                                    double lf_scale);
/* The batch: per field the wavelength index, point-source amplitude
 * (sqrt(flux)), tip and tilt (times magnification), and candidate index. */
int csg_chain_set_batch(csg_chain* chain, int n_fields, const int* lambda_idx, const double* amp,
                        const double* tip, const double* tilt, const int* cand);
/* Device FP64 buffer [n_cand][n_hex] of candidate FPM sags, written in place
 * by the caller or the DE kernels (complexHexMaskFPM set_optimization_data,
 * complexHexMaskFPM.cpp:176-191). */
int csg_chain_sags(csg_chain* chain, int n_cand, int n_hex, double** dev_sags);
/* Device FP64 arrays [n_fields] of the batch's source amplitude, tip and tilt
 * (any pointer may be null); written in place between executions they change
 * the sources without a new batch or graph. */
int csg_chain_batch_buffers(csg_chain* chain, double** amp, double** tip, double** tilt);
/* Run the walk (calibrating != 0 skips disable_for_calibration elements, the
 * calibration propagation of regionContrast.cpp:124-143); use_graph != 0
 * captures a CUDA graph on first use and replays it on later calls. */
int csg_chain_execute(csg_chain* chain, int calibrating, int use_graph);
/* makeHexCFpmResponse::compute_response (makeHexCFpmResponse.cpp:91-190)
 * for the current batch (one base field per (wavelength, source); candidate
 * ignored): column h < n_hex of M is the final image at the n_pix region
 * pixels (row-major flat indices into the n_out^2 image) with only hex h in
 * the fpm_index-th hex FPM and no Babinet term; column n_hex is the Babinet
 * response of the area outside every hex. The walk up to the FPM runs once
 * per base field; the columns run batched. m_host: complex<double>
 * interleaved [n_base][n_pix][n_hex + 1] (csg_respobj_create's layout);
 * calib_max: max over pixels of the calibration intensity summed over the
 * batch. Synchronous. */
int csg_chain_response(csg_chain* chain, int fpm_index, const int* pix_idx, int n_pix,
                       double* m_host, double* calib_max);
/* Device pointers to the final image fields [F][2][n_out][n_out] and to the
 * working pupil-plane fields [F][2][N][N]. */
int csg_chain_image(csg_chain* chain, float** dev_image, int* n_out);
/* CSG_PREC_HIGH chains: the low-order words of the final image, same layout
 * (the image is image + image_lo to ~2^-33 of its values); NULL at other
 * precisions. */
int csg_chain_image_lo(csg_chain* chain, float** dev_image_lo);
int csg_chain_field(csg_chain* chain, float** dev_field);
/* Pre-size an MFT plan's scratch for n_fields (so graph capture allocates
 * nothing) and autotune its tensor-core tile width (128 or 64 output
 * columns per tile, and 256 where the output is at least 256 wide) by
 * timing each at that batch size. Set the environment variable
 * CSG_MFT_AUTOTUNE=0 to keep the default width (128). */
int csg_mft_reserve(csg_mft* plan, int n_fields);
/* Fix the plan's tile width (64, 128 or 256 output columns per tile, 256
 * only for outputs at least 256 wide; 0 returns to the default and lets
 * csg_mft_reserve autotune it again). */
int csg_mft_set_tile(csg_mft* plan, int bn);
/* The chosen tile width and the measured ms per transform of each width. */
int csg_mft_tuning(csg_mft* plan, int* bn, float* ms128, float* ms64);
/* Every autotuning decision of the process as a JSON list. */
int csg_mft_tuning_log(char* buf, size_t len);

/* ------------------------------------------------------ deformable mirror */
/* deformableMirror::compute_influence_function / compute_deformable_mirror_surface
 * (deformableMirror.cpp:205-270): Gaussian influence of width sigma actuator
 * pitches, n_act x n_act actuators as delta points on the upsampled grid,
 * half-cell shift, fft_truncate to N x N, times the influence spectrum,
 * inverse FFT, real part. The whole chain is separable, so the surface is
 * computed exactly as Re(M A M^T) with an N x n_act FP64 basis M built once
 * per geometry. */
int csg_dm_create(csg_ctx* ctx, csg_dm** dm, int n, int n_act, double sigma);
int csg_dm_destroy(csg_dm* dm);
/* Device FP64 strokes [n_act][n_act] (metres) -> device fp32 surface [N][N]
 * (metres), on the context's stream. Apply it with a mirror element
 * (deformableMirror::execute = mirror::execute with this surface). */
int csg_dm_surface(csg_dm* dm, const double* act, float* surface);

/* ------------------------------------------------------- surrogate MLP */
/* No reference counterpart: a fully connected network n_in -> hidden[] -> 1
 * (exact-erf GELU) that maps a hex-FPM sag vector and wavelength to log10
 * dark-hole contrast, used to pre-screen DE trial vectors. bf16 weights and
 * activations, fp32 accumulation (tcgen05 GEMMs), fp32 master weights, Adam.
 * Batches are multiples of 8 up to max_batch; hidden widths multiples of 8. */
int csg_mlp_create(csg_ctx* ctx, csg_mlp** mlp, int n_in, int n_hidden, const int* hidden,
                   int max_batch, unsigned long long seed);
int csg_mlp_destroy(csg_mlp* mlp);
/* Input batch from device FP64 sags [B][n_var] and wavelengths [B]: mode 0
 * x = sag / sag_scale; mode 1 the hex phasors cos, sin(4 pi sag_scale sag /
 * lambda) (2 n_var features; sag_scale = phaseSign); then (lambda - lam0) /
 * lam_scale. */
int csg_mlp_features(csg_mlp* mlp, const double* sags, int n_var, const double* lam,
                     double sag_scale, double lam0, double lam_scale, int batch, int mode);
/* Input batch from raw device fp32 features [B][n_in]. */
int csg_mlp_set_input(csg_mlp* mlp, const float* x, int batch);
/* Prediction of the current input batch into y (device fp32 [B], may be null). */
int csg_mlp_forward(csg_mlp* mlp, int batch, float* y);
/* Forward, MSE loss against t (device fp32 [B]; *loss device scalar, may be
 * null), backward and one Adam step (lr = 0: gradients only). */
int csg_mlp_train_step(csg_mlp* mlp, int batch, const float* t, float lr, float* loss);
/* Device pointers of layer l: fp32 weights [out][in], bias [out] and their
 * gradients from the last training step (any pointer may be null). */
int csg_mlp_param(csg_mlp* mlp, int layer, float** w, float** b, float** gw, float** gb);

/* ---------------------------------------------------- intensity / contrast */
/* regionContrast::compute_intensity (regionContrast.cpp:124-143) and the
 * contrast mean (:195) / optObjective mean-or-max (optObjective.cpp:56-67):
 * For each group g (n_groups groups of `per_group` consecutive fields),
 * I_g = sum_fields |E|^2 restricted to the n_pix region pixels pix_idx
 * (row-major flat indices); out[g] = reduce(I_g) * scale where reduce is
 * mean (mode 0) or max (mode 1). FP64 accumulation. */
int csg_region_reduce(csg_ctx* ctx, const float* field, int rows, int cols, int n_groups,
                      int per_group, const int* pix_idx, int n_pix, int mode, double scale,
                      double* out);
/* Full-image intensity sum over n_fields fields into out [rows][cols]
 * (FP64) and its maximum into out_max (the calibration max of
 * regionContrast.cpp:139-142). */
int csg_intensity(csg_ctx* ctx, const float* field, int rows, int cols, int n_fields,
                  double* out, double* out_max);

/* contrastCurve::make_contrast_curve (contrastCurve.cpp:127-146): the mean
 * of intensity[n][n] * scale (device FP64; scale = 1 / calibration max) over
 * overlapping annuli s[i-1] < R < s[i+1], i = 1 .. n_samples - 2, where R is
 * the distance of each pixel centre (-(pixel n - pixel) / 2 + k pixel) from
 * the axis divided by lod, and samples (device, n_samples) are the
 * reference's linspace(0, max(pixelX / loD), n_samples). out_mean (device,
 * n_samples - 2): bin means (NaN for an empty bin). work: device scratch of
 * 2 (n_samples - 2) doubles. */
int csg_contrast_curve(csg_ctx* ctx, const double* intensity, int n, double pixel, double lod,
                       double scale, const double* samples, int n_samples, double* work,
                       double* out_mean);
/* linearOptimizer::compute_jacobian (linearOptimizer.cpp:420-495) over one
 * batched walk: image (device, fp32 planar [(n_var + 1) * n_base][2][n_out][n_out])
 * holds candidate 0 (unperturbed) and candidates 1 .. n_var (variable i - 1
 * moved by dx), each as n_base consecutive fields (sources x wavelengths).
 * jac (device FP64, row-major [2 n_base n_pix][n_var]): column i is
 * (E_{i+1} - E_0) / dx at the region pixels pix_idx (flat row-major indices),
 * rows [Re; Im] per base field, base fields in order. */
int csg_fd_jacobian(csg_ctx* ctx, const float* image, int n_out, int n_base, int n_var,
                    const int* pix_idx, int n_pix, double dx, double* jac);

/* ---------------------------------------- response-matrix objective */
/* optHexRespObjective (optObjective.cpp:24-69): M cubes for every (s, p, l)
 * as complex<double> interleaved host row-major [n_mat][npix][ncol]
 * (ncol = nhex + 1), wavelength of each matrix, calibration intensity. */
int csg_respobj_create(csg_ctx* ctx, csg_respobj** obj, const double* m_host, int n_mat,
                       int npix, int ncol, const double* wavelength, double calib,
                       double phase_sign, int objective /*0 mean, 1 max*/);
int csg_respobj_destroy(csg_respobj* obj);
/* optHexRespObjective::execute(mat& optData, rowvec& objVal): x is device
 * FP64 [pop][nvar] (nvar = ncol - 1; candidate-major, i.e. the transpose of
 * the reference's nvar x pop matrix), out device FP64 [pop]. */
int csg_respobj_execute(csg_respobj* obj, const double* x, int pop, double* out);

/* ------------------------------------------------ differential evolution */
/* differentialEvolutionOptimizer (differentialEvolutionOptimizer.cpp:216-468;
 * deStrategy.cpp:23-158) with its state on the device. Populations are FP64
 * [pop][nvar] (candidate-major: the transpose of the reference's nvar x pop
 * matrix). A generation is csg_de_generate (permutations, mutation, binomial
 * crossover without a forced index, bounce-back into [mean + init bounds]
 * clipped to the global bounds) -> the objective on the trial population,
 * written to f_trial -> csg_de_select (greedy selection, best member,
 * population statistics, generation + 1). Random numbers come from a
 * counter-based generator keyed by (seed, generation, stream, index), so a
 * generation is reproducible and can be captured in a CUDA graph. */
int csg_de_create(csg_ctx* ctx, csg_de** de, int pop, int nvar, uint64_t seed);
int csg_de_destroy(csg_de* de);
/* globalBounds and initBounds per variable (host FP64 arrays of nvar). */
int csg_de_set_bounds(csg_de* de, const double* global_lo, const double* global_hi,
                      const double* init_lo, const double* init_hi);
/* init_population (:336-358): origin + spread (u - 1/2) (initUB - initLB)
 * (type 0) or origin + spread n (initUB - initLB) (type 1, normal). */
int csg_de_init(csg_de* de, const double* origin_host, double spread, int type);
/* Device buffers of the state: population, objective values, trial
 * population and trial objective values. */
int csg_de_buffers(csg_de* de, double** pop, double** f, double** trial, double** f_trial);
/* Write trial vectors into a caller buffer instead (e.g. a chain's sags). */
int csg_de_set_trial_buffer(csg_de* de, double* trial);
/* strategy 0 = DE/rand/1, 1 = DE/local-to-best/1, 2 = either-or. */
int csg_de_generate(csg_de* de, int strategy, double f_weight, double cr);
/* Another independent trial set of the same generation (draw > 0; draw 0 is
 * csg_de_generate), for screening several trials per member with a
 * surrogate before the full evaluation. */
int csg_de_generate_draw(csg_de* de, int strategy, double f_weight, double cr, int draw);
/* initial != 0 after evaluating a fresh population (no selection). */
int csg_de_select(csg_de* de, int initial);
/* bestVal = huge, as on a re-initialisation (:249-258). */
int csg_de_reset_best(csg_de* de);
int csg_de_stats(csg_de* de, double* best_val, double* mean_dist, double* max_dist,
                 unsigned long long* generation, double* best_vec);

#ifdef __cplusplus
}
#endif
#endif /* CSIMGPU_H */
