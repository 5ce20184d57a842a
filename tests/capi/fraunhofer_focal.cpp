// A C++ caller of the C ABI, without Python: the sequence a reference-side
// fraunhoferFocal element runs on the GPU (zoomFft::init / execute,
// csim_fft.cpp:670-826, behind fraunhoferFocal::execute,
// fraunhoferFocal.cpp:23-63). It builds an Armadillo-layout complex<double>
// cube (column-major, rows x cols x n_lambda), uploads it, transforms it
// with one plan of one operator slot per wavelength, downloads the result
// in the same layout and checks it against the transform summed here in
// double precision. Exit status 0 when the peak-normalised error is below
// the bound given as the first argument (default 1e-5).
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "csimgpu.h"

using cd = std::complex<double>;

static int check(int rc, const char* what) {
  if (rc != CSG_OK) {
    std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, csg_last_error());
    std::exit(2);
  }
  return rc;
}

int main(int argc, char** argv) {
  const double bound = argc > 1 ? std::atof(argv[1]) : 1e-5;
  const int precision = argc > 2 ? std::atoi(argv[2]) : CSG_PREC_BF16X6;
  const int rows = 96, cols = 128, nx = 40, nl = 2;  // input rows (y) x cols (x), output nx^2
  const double dx = 2e-5, dout = 3e-6;
  const double lam[nl] = {6.2e-7, 6.8e-7};
  // pixel centres -(n d - d) / 2 + i d (csim_geom.cpp:130-135)
  auto centres = [](int n, double d) {
    std::vector<double> v(n);
    for (int i = 0; i < n; ++i) v[i] = -(d * n - d) / 2.0 + i * d;
    return v;
  };
  const std::vector<double> xin = centres(cols, dx), yin = centres(rows, dx),
                            xo = centres(nx, dout);
  std::vector<double> lf(nl), pref(2 * nl);
  for (int l = 0; l < nl; ++l) {
    lf[l] = lam[l] * 2.0 * 0.05 * 15.0;  // lambda 2 beamRadius primaryfRatio
    pref[2 * l] = 0.0;                   // dx dy / (i lf)
    pref[2 * l + 1] = -dx * dx / lf[l];
  }
  // the efield cube: Armadillo (r, c, s) at r + c rows + s rows cols
  std::vector<cd> cube((size_t)rows * cols * nl);
  for (int s = 0; s < nl; ++s)
    for (int c = 0; c < cols; ++c)
      for (int r = 0; r < rows; ++r) {
        const double rr = std::hypot(yin[r], xin[c]);
        const double amp = rr < 0.45 * rows * dx ? 1.0 : 0.0;
        const double ph = 0.3 * std::sin(7.0 * xin[c] / (cols * dx) + 3.0 * s) +
                          0.2 * std::cos(5.0 * yin[r] / (rows * dx));
        cube[r + (size_t)c * rows + (size_t)s * rows * cols] = amp * std::polar(1.0, ph);
      }

  csg_ctx* ctx = nullptr;
  check(csg_create(&ctx, 0), "csg_create");
  csg_mft* plan = nullptr;
  check(csg_mft_create(ctx, &plan, rows, cols, nx, nx, yin.data(), xin.data(), xo.data(),
                       xo.data(), nl, lf.data(), pref.data(), -1.0, precision),
        "csg_mft_create");
  void *staging = nullptr, *din = nullptr, *dout_p = nullptr, *dslot = nullptr;
  check(csg_alloc(ctx, (size_t)rows * cols * nl * 16, &staging), "csg_alloc");
  check(csg_alloc(ctx, (size_t)rows * cols * nl * 8, &din), "csg_alloc");
  check(csg_alloc(ctx, (size_t)nx * nx * nl * 8, &dout_p), "csg_alloc");
  check(csg_alloc(ctx, nl * sizeof(int), &dslot), "csg_alloc");
  const int slots[nl] = {0, 1};
  check(csg_memcpy_h2d(ctx, dslot, slots, sizeof(slots)), "csg_memcpy_h2d");
  check(csg_field_upload(ctx, reinterpret_cast<const double*>(cube.data()), CSG_LAYOUT_COLMAJOR,
                         rows, cols, nl, staging, static_cast<float*>(din)),
        "csg_field_upload");
  check(csg_mft_execute(ctx, plan, static_cast<float*>(din), static_cast<float*>(dout_p), nl,
                        static_cast<int*>(dslot), 0, nullptr, nullptr),
        "csg_mft_execute");
  std::vector<cd> out((size_t)nx * nx * nl);
  check(csg_field_download(ctx, static_cast<float*>(dout_p), nx, nx, nl, staging,
                           reinterpret_cast<double*>(out.data()), CSG_LAYOUT_COLMAJOR),
        "csg_field_download");
  check(csg_sync(ctx), "csg_sync");

  // out[v][u] = pref sum_{y,x} in[y][x] exp(-2 pi i (x xo_u + y yo_v) / lf)
  const double pi = std::acos(-1.0);
  double err = 0.0, peak = 0.0;
  for (int s = 0; s < nl; ++s) {
    std::vector<cd> t((size_t)rows * nx);  // T[y][u]
    for (int r = 0; r < rows; ++r)
      for (int u = 0; u < nx; ++u) {
        cd acc = 0.0;
        for (int c = 0; c < cols; ++c)
          acc += cube[r + (size_t)c * rows + (size_t)s * rows * cols] *
                 std::polar(1.0, -2.0 * pi * xin[c] * xo[u] / lf[s]);
        t[(size_t)r * nx + u] = acc;
      }
    const cd pr(pref[2 * s], pref[2 * s + 1]);
    for (int v = 0; v < nx; ++v)
      for (int u = 0; u < nx; ++u) {
        cd acc = 0.0;
        for (int r = 0; r < rows; ++r)
          acc += t[(size_t)r * nx + u] * std::polar(1.0, -2.0 * pi * yin[r] * xo[v] / lf[s]);
        acc *= pr;
        const cd got = out[v + (size_t)u * nx + (size_t)s * nx * nx];  // column-major (v, u)
        err = std::max(err, std::abs(got - acc));
        peak = std::max(peak, std::abs(acc));
      }
  }
  std::printf("fraunhofer_focal: peak-normalised error %.3e (bound %.1e)\n", err / peak, bound);
  csg_mft_destroy(plan);
  csg_destroy(ctx);
  return err / peak < bound ? 0 : 1;
}
