/*
 * Plain-C restatement of the reference's hex focal-plane-mask table builder.
 * TEST INFRASTRUCTURE ONLY: the oracle for csg_hex_tables; the shipped
 * library never links it.
 *
 *  make_hex_array           complexHexMaskFPM.cpp:317-366
 *  make_interpolation_data  complexHexMaskFPM.cpp:372-469
 *
 * Compiled with -ffp-contract=off so every FP64 expression rounds exactly as
 * the reference's x86-64 build (no fused multiply-add).
 *
 * Differences that are stated, not hidden:
 *  - `pitch` is the centre-to-centre distance of neighbouring hexes in hex
 *    units; the reference formula hexRadius = hexStepPix (1-gap) sqrt(3)/2
 *    is pitch = sqrt(3) (its own layout); standard-ring layouts use pitch 1.
 *  - where hexes overlap (negative gap) the highest hex index wins; the
 *    reference writes them from an OpenMP loop in unspecified order.
 *  - a fourth distinct hex inside one mask pixel (the reference asserts) is
 *    counted as outside and reported through the return value.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

void make_hex_array(const double* hex_x, const double* hex_y, int n_hex, int n_rings, int A,
                    double fpm_scale_factor, double hex_gap, double pitch, int32_t* design) {
  const double vx = sqrt(3.0) / 2.0, vy = 0.5;
  const double step_pix = (0.5 * A) / n_rings * fpm_scale_factor;
  const double radius = step_pix * (1.0 - hex_gap) * (pitch / 2.0);
  const double outer = 2.0 * radius / sqrt(3.0);
  const double close_sq = outer * outer;
  for (int i = 0; i < A * A; ++i) design[i] = -1;
  for (int h = 0; h < n_hex; ++h) {
    const double cx = 0.5 * A + hex_x[h] * step_pix;
    const double cy = 0.5 * A + hex_y[h] * step_pix;
    int i0 = (int)floor(cy - outer) - 1, i1 = (int)ceil(cy + outer) + 1;
    int j0 = (int)floor(cx - outer) - 1, j1 = (int)ceil(cx + outer) + 1;
    if (i0 < 0) i0 = 0;
    if (j0 < 0) j0 = 0;
    if (i1 > A - 1) i1 = A - 1;
    if (j1 > A - 1) j1 = A - 1;
    for (int ii = i0; ii <= i1; ++ii) {
      for (int jj = j0; jj <= j1; ++jj) {
        const double dx = (double)jj - cx;
        const double dy = (double)ii - cy;
        const double r2 = dx * dx + dy * dy;
        if (r2 > close_sq) continue;
        const double dpx = dx * vx, dpy = dy * vy;
        if (fabs(dy) < radius && fabs(dpx + dpy) < radius && fabs(dpx - dpy) < radius) {
          if (h > design[ii * A + jj]) design[ii * A + jj] = h;
        }
      }
    }
  }
}

/* hex_id / count: [3][S][S]. Returns the number of pixels that met a fourth
 * distinct hex. stale != 0 reproduces the reference's loop as it runs on one
 * OpenMP thread: its on-array check of a cell uses the row index ii1 left by
 * the last sub-sample of the previous processed cell of the row (the variable
 * is shared by the check and the sub-sample loop, complexHexMaskFPM.cpp:
 * 395-423), the midpoint's only until the first cell of the row passes. */
int make_interpolation_data(const int32_t* design, int A, int S, int n_sub, double pixel_scale,
                            double fpm_radius, double fpm_scale_factor, int16_t* hex_id,
                            uint16_t* count, int stale) {
  const double ac1 = -S / 2.0 - 0.5;
  const double xc1 = (0.5 / fpm_radius) * fpm_scale_factor;
  const long plane = (long)S * S;
  int overflow = 0;
  for (long k = 0; k < 3 * plane; ++k) {
    hex_id[k] = -1;
    count[k] = 0;
  }
  for (int i = 0; i < S; ++i) {
    const int iii_c = (int)(n_sub / 2.0);
    const double xc = (i + ac1 + (0.5 + iii_c) / ((double)n_sub)) * pixel_scale;
    const int ii1c = (int)((0.5 + xc * xc1) * A + 0.5);
    int ii1_check = ii1c;
    for (int j = 0; j < S; ++j) {
      const int jjj_c = (int)(n_sub / 2.0);
      const double yc = (j + ac1 + (0.5 + jjj_c) / ((double)n_sub)) * pixel_scale;
      const int jj1c = (int)((0.5 + yc * xc1) * A + 0.5);
      if (ii1_check < 0 || ii1_check >= A || jj1c < 0 || jj1c >= A) continue;
      if (stale) {  /* the sub-sample loop leaves its last row index behind */
        const double xl = (i + ac1 + (0.5 + (n_sub - 1)) / ((double)n_sub)) * pixel_scale;
        ii1_check = (int)((0.5 + xl * xc1) * A + 0.5);
      }
      int list[3];
      int nl = 0;
      unsigned cnt[3] = {0, 0, 0};
      int over = 0;
      for (int iii = 0; iii < n_sub; ++iii) {
        for (int jjj = 0; jjj < n_sub; ++jjj) {
          const double x = (i + ac1 + (0.5 + iii) / ((double)n_sub)) * pixel_scale;
          const double y = (j + ac1 + (0.5 + jjj) / ((double)n_sub)) * pixel_scale;
          const int ii1 = (int)((0.5 + x * xc1) * A + 0.5);
          const int jj1 = (int)((0.5 + y * xc1) * A + 0.5);
          if (ii1 < 0 || ii1 >= A || jj1 < 0 || jj1 >= A) {
            cnt[0]++;
            continue;
          }
          const int h = design[ii1 * A + jj1];
          if (h < 0) {
            cnt[0]++;
            continue;
          }
          int k = 0;
          while (k < nl && list[k] != h) ++k;
          if (k == nl) {
            if (nl == 3) {
              over = 1;
              cnt[0]++;
              continue;
            }
            list[nl++] = h;
          }
          cnt[k]++;
        }
      }
      overflow += over;
      for (int k = 0; k < 3; ++k) {
        count[k * plane + (long)i * S + j] = (uint16_t)cnt[k];
        if (k < nl) hex_id[k * plane + (long)i * S + j] = (int16_t)list[k];
      }
    }
  }
  for (long p = 0; p < plane; ++p) {
    if (count[p] + count[plane + p] + count[2 * plane + p] == 0) count[p] = (uint16_t)(n_sub * n_sub);
  }
  return overflow;
}
