"""FP64 CPU restatement of the reference's transform layer (src/lib/csim_fft.cpp).

TEST INFRASTRUCTURE ONLY: this is the correctness oracle and the timed CPU
baseline. The shipped library never imports it.

Array convention: numpy [row][col] == Armadillo (row, col); rows are y and
columns are x (csim_geom.cpp:203-214 builds pixelXX from pixelX along columns).
Cubes are [slice][row][col] with slices = wavelengths.
The FFTs use scipy.fft (pocketfft, FP64), which agrees with FFTW to ~1e-15.
"""
from __future__ import annotations

import math
import os

import numpy as np
import scipy.fft as sfft

WORKERS = os.cpu_count() or 1


# --------------------------------------------------------------------- FFT --
def fft2(a: np.ndarray) -> np.ndarray:
    """Forward 2-D DFT, exp(-i...), unnormalised (csim_fft.cpp:62-65, :127)."""
    return sfft.fft2(a, axes=(-2, -1), workers=WORKERS)


def ifft2(a: np.ndarray) -> np.ndarray:
    """Inverse 2-D DFT divided by n_elem (csim_fft.cpp:91-95, :192-193)."""
    return sfft.ifft2(a, axes=(-2, -1), workers=WORKERS)


def fft_shift(a: np.ndarray) -> np.ndarray:
    """Circular shift by floor(n/2) on both axes (csim_fft.cpp:296-318)."""
    r, c = a.shape[-2:]
    return np.roll(np.roll(a, r // 2, axis=-2), c // 2, axis=-1)


def fft_truncate(a: np.ndarray, tr: int, tc: int) -> np.ndarray:
    """Spectral truncation with Nyquist averaging (csim_fft.cpp:322-367)."""
    nr, nc = a.shape
    cr, cc = -(-tr // 2), -(-tc // 2)      # ceil(t/2)
    fr, fc = tr // 2, tc // 2              # floor(t/2)
    rows = np.r_[0:cr, nr - fr:nr]
    cols = np.r_[0:cc, nc - fc:nc]
    out = a[np.ix_(rows, cols)].copy()
    if tr % 2 == 0:
        src = a[tr // 2, cols]
        out[tr // 2, :] = (src + out[tr // 2, :]) / 2.0
    if tc % 2 == 0:
        src = a[rows, tc // 2]
        out[:, tc // 2] = (src + out[:, tc // 2]) / 2.0
    if tr % 2 == 0 and tc % 2 == 0:
        out[tr // 2, tc // 2] = (a[tr // 2, tc // 2] + a[tr // 2, nc - fc]
                                 + a[nr - fr, tc // 2] + a[nr - fr, nc - fc]) / 4.0
    return out


# ------------------------------------------------------------- Fresnel AS --
def fresnel_freq2(nr: int, nc: int) -> np.ndarray:
    """fft_shift(H) with H[r,c] = vH[c]^2 + vH[r]^2, vH = regspace(-N/2, N/2-1)
    (csim_fft.cpp:377-381). H.each_row() = vH.t() and H + H.t() only make
    sense for a square array, so only N x N is accepted."""
    if nr != nc:
        raise ValueError("fresnelPropagateAS needs a square array")
    vh = np.arange(-(nr // 2), nr // 2, dtype=np.float64)
    return fft_shift(vh[None, :] ** 2 + vh[:, None] ** 2)


def fresnel_propagate_as(cube: np.ndarray, lambdas, ap_rad: float, z: float) -> np.ndarray:
    """Angular-spectrum Fresnel propagation per slice (csim_fft.cpp:371-392):
    E <- IFFT(FFT(E) * exp(i k z sqrt(1 - (lambda/apRad)^2 H / 4)))."""
    cube = np.asarray(cube, dtype=np.complex128)
    nr, nc = cube.shape[-2:]
    h = fresnel_freq2(nr, nc)
    out = np.empty_like(cube)
    for sl, lam in enumerate(lambdas):
        k = 2.0 * math.pi / lam
        ch = np.exp(1j * k * z * np.sqrt(1.0 - 0.25 * (lam / ap_rad) ** 2 * h))
        out[sl] = ifft2(fft2(cube[sl]) * ch)
    return out


# ------------------------------------------------------- chirp-Z (Bluestein) --
def czt1d(x: np.ndarray, k: int, w: float, a: float) -> np.ndarray:
    """Bluestein CZT along axis 0 of x (m x n), as csim_fft.cpp:442-665:
    out[q, c] = sum_n x[n, c] exp(i (w n q - a n)); nfft = 2^ceil(log2(m+k-1))."""
    m = x.shape[0]
    nfft = 1 << int(math.ceil(math.log2(m + k - 1)))
    mm = max(m, k)
    kk = np.arange(m + mm - 1, dtype=np.float64) - m + 1.0
    ww = w * (kk * kk / 2.0)
    nn = np.arange(m, dtype=np.float64)
    caa = np.exp(1j * (a * (-nn) + ww[m - 1:2 * m - 1]))
    iww = np.zeros(nfft, dtype=np.complex128)
    iww[:m - 1 + k] = np.exp(-1j * ww[:m - 1 + k])
    fv = sfft.fft(iww)
    y = np.zeros((nfft, x.shape[1]), dtype=np.complex128)
    y[:m] = x * caa[:, None]
    g = sfft.ifft(sfft.fft(y, axis=0, workers=WORKERS) * fv[:, None], axis=0, workers=WORKERS)
    expww = np.exp(1j * ww[m - 1:m - 1 + k])
    return g[m - 1:m + k - 1] * expww[:, None]


def czt2d(x: np.ndarray, k: int, wx: float, ax: float, wy: float, ay: float) -> np.ndarray:
    """Columns with (wy, ay), transpose, columns with (wx, ax), transpose
    (csim_fft.cpp:422-440)."""
    o1 = czt1d(x, k, wy, ay).T
    return czt1d(o1, k, wx, ax).T


# ------------------------------------------------------------ geometry --
class ArrayGeom:
    """Pixel-centre coordinates (csim_geom.cpp:113-142 set_xy, :144-170
    set_xy_offset_m1, :203-214 set_mesh). x runs along columns, y along rows."""

    def __init__(self, pixel_x, pixel_y, dx, dy):
        self.pixelX = np.asarray(pixel_x, dtype=np.float64)
        self.pixelY = np.asarray(pixel_y, dtype=np.float64)
        self.pixelSizeX = float(dx)
        self.pixelSizeY = float(dy)
        self.physicalSizeX = self.pixelSizeX * self.pixelX.size
        self.physicalSizeY = self.pixelSizeY * self.pixelY.size

    @classmethod
    def set_xy(cls, nx: int, ny: int, dx: float, dy: float | None = None,
               ox: float = 0.0, oy: float = 0.0) -> "ArrayGeom":
        dy = dx if dy is None else dy
        px = -(dx * nx - dx) / 2.0 + np.arange(nx) * dx - ox
        py = -(dy * ny - dy) / 2.0 + np.arange(ny) * dy - oy
        return cls(px, py, dx, dy)

    @classmethod
    def set_xy_offset_m1(cls, nx: int, ny: int, d: float) -> "ArrayGeom":
        return cls((np.arange(nx) - nx / 2.0) * d, (np.arange(ny) - ny / 2.0) * d, d, d)

    def mesh(self):
        xx = np.broadcast_to(self.pixelX[None, :], (self.pixelY.size, self.pixelX.size))
        yy = np.broadcast_to(self.pixelY[:, None], (self.pixelY.size, self.pixelX.size))
        return xx, yy, np.sqrt(xx ** 2 + yy ** 2), np.arctan2(yy, xx)


# ------------------------------------------------------------ zoom FFT --
class ZoomFft:
    """Physical-unit zoom FFT (csim_fft.cpp:670-708 init, :786-826 execute).

    execute() runs the reference algorithm (Bluestein CZT + post phase);
    mft() evaluates the identical sum directly as A @ E @ B.T:
      out[r, c] = dx dy / (i lf) * sum_{j,l} E[j, l]
                  exp(-2 pi i (xin_l xout_c + yin_j yout_r) / lf)
    The output is always Nx x Nx (csim_fft.cpp:414-420)."""

    def __init__(self, ag_in: ArrayGeom, ag_out: ArrayGeom, lfl):
        self.gin, self.gout = ag_in, ag_out
        self.lfl = np.atleast_1d(np.asarray(lfl, dtype=np.float64))
        self.Nx = ag_out.pixelX.size
        self.Ax = 2 * math.pi * ag_in.pixelSizeX * ag_out.pixelX[0] / self.lfl
        self.Wx = -2 * math.pi * ag_in.pixelSizeX * ag_out.pixelSizeX / self.lfl
        if (ag_in.pixelSizeX != ag_in.pixelSizeY or ag_out.pixelSizeX != ag_out.pixelSizeY
                or ag_out.pixelY[0] != ag_out.pixelX[0]):
            self.Ay = 2 * math.pi * ag_in.pixelSizeY * ag_out.pixelY[0] / self.lfl
            self.Wy = -2 * math.pi * ag_in.pixelSizeY * ag_out.pixelSizeY / self.lfl
        else:
            self.Ay, self.Wy = self.Ax.copy(), self.Wx.copy()
        self.mxPmy = (ag_in.pixelX[0] * ag_out.pixelX[None, :]
                      + ag_in.pixelY[0] * ag_out.pixelY[:, None])

    def execute(self, e: np.ndarray, sl: int) -> np.ndarray:
        out = czt2d(np.asarray(e, dtype=np.complex128), self.Nx, self.Wx[sl], self.Ax[sl],
                    self.Wy[sl], self.Ay[sl])
        f1 = -2 * math.pi * 1j / self.lfl[sl]
        f2 = self.gin.pixelSizeX * self.gin.pixelSizeY / (1j * self.lfl[sl])
        return out * (np.exp(f1 * self.mxPmy[:out.shape[0], :out.shape[1]]) * f2)

    def mft(self, e: np.ndarray, sl: int) -> np.ndarray:
        return mft(e, self.gin.pixelX, self.gin.pixelY, self.gout.pixelX[:self.Nx],
                   self.gout.pixelY[:self.Nx], self.lfl[sl],
                   self.gin.pixelSizeX * self.gin.pixelSizeY / (1j * self.lfl[sl]))


def mft_matrices(xin, yin, xout, yout, lf: float, sign: float = -1.0):
    """Row and column kernels of the matrix Fourier transform:
    A[r, j] = exp(sign 2 pi i yin_j yout_r / lf), B[c, l] = exp(sign 2 pi i xin_l xout_c / lf).
    Phases are reduced in turns in FP64 before the exponential."""
    ta = np.outer(np.asarray(yout, np.float64), np.asarray(yin, np.float64)) / lf
    tb = np.outer(np.asarray(xout, np.float64), np.asarray(xin, np.float64)) / lf
    ta -= np.rint(ta)
    tb -= np.rint(tb)
    return np.exp(sign * 2j * math.pi * ta), np.exp(sign * 2j * math.pi * tb)


def mft(e, xin, yin, xout, yout, lf: float, pref: complex, sign: float = -1.0) -> np.ndarray:
    """out = pref * A @ e @ B.T (see mft_matrices); e is [..., rows(y), cols(x)]."""
    a, b = mft_matrices(xin, yin, xout, yout, lf, sign)
    return pref * (a @ np.asarray(e, dtype=np.complex128) @ b.T)
