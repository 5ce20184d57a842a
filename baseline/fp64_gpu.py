"""The plain FP64 GPU path: the comparator the split-precision batched path is
measured against (field propagations/s), not part of the library and never
selected at run time.

It is what a direct GPU port of the reference's PIAACMC walk looks like:
complex128 throughout, one field at a time, cuFFT (Z2Z) for the Fresnel
propagation and cuBLAS (ZGEMM) for the matrix Fourier transforms, through
PyTorch. Per wavelength it precomputes what the reference caches (mirror
phases, mirror.cpp:66-72) plus the Fresnel transfer function and the MFT
operators; per field it builds the hex mask on the full S x S grid from the
interpolation tables (complexHexMaskFPM.cpp:44-99) and runs
  source x (1 + i) pupil x M1 -> IFFT(FFT(E) H) -> x M2
  -> E + c MFT2[(fliplr(M) - 1) MFT1[E]]   (fpmPupToLyot in its Babinet MFT form)
  -> x (1 + i) Lyot -> final MFT,
the sequence and formulas of the reference's elements (fresnelPropagator,
csim_fft.cpp:371-392; fpmPupToLyot.cpp:24-167; fraunhoferFocal.cpp:23-72).
"""
from __future__ import annotations

import math
import time

import numpy as np
import torch


def _grid(n: int, d: float, shift: float = 0.0) -> np.ndarray:
    """Pixel centres -(d n - d) / 2 + i d (csim_geom.cpp:130-135), shifted."""
    return -(d * n - d) / 2.0 + np.arange(n) * d + shift


def _mft_ops(xin, xout, lf: float, sign: float, dev) -> torch.Tensor:
    """exp(sign 2 pi i xout_r xin_k / lf), phases reduced in turns in FP64."""
    t = np.outer(xout, xin) / lf
    t -= np.rint(t)
    return torch.as_tensor(np.exp(sign * 2j * math.pi * t), device=dev)


class Fp64Piaacmc:
    """The PIAACMC chain of the bench on complex128, one field per call.
    dtype=torch.complex64 gives the same plain path in single precision
    (every table, field and product complex64): the precision comparator."""

    def __init__(self, inp: dict, spec, device: str = "cuda", dtype=torch.complex128,
                 fpm_box=None):
        """fpm_box (r0, c0, rows, cols): transform only that box of the mask
        grid (where fliplr(M) - 1 can be nonzero) and only the Lyot stop's
        bounding window of the pupil plane, the exact crops the GPU chain
        makes, so the comparison isolates precision and batching."""
        self.dev = torch.device(device)
        self.dtype = dtype
        ef, tel = inp["ef"], inp["tel"]
        n, dx = ef.n, inp["dx"]
        self.n = n
        S = inp["hex_id"].shape[-1]
        self.ids = torch.as_tensor(inp["hex_id"].astype(np.int64), device=self.dev)
        self.cnt = torch.as_tensor(inp["count"].astype(np.float64), device=self.dev)
        self.n_sub = spec.n_sub
        xe = _grid(n, dx)
        xm = _grid(S, inp["dm"])
        pupil = torch.as_tensor(inp["pupil"], device=self.dev, dtype=torch.float64)
        lyot = torch.as_tensor(inp["lyot"], device=self.dev, dtype=torch.float64)
        self.lyot = lyot * (1 + 1j)  # mask.cpp: (m + i m)
        n_out = int(math.ceil(spec.n_out_fov * spec.spl))
        xo = _grid(n_out, inp["lod_image"] / spec.spl)
        fr = np.fft.fftfreq(n, 1.0 / n)  # integer frequency index in FFT order
        f2 = fr[:, None] ** 2 + fr[None, :] ** 2
        ap_rad = ef.arrayRadiusPhysical
        self.box = fpm_box
        if fpm_box is not None:
            nz = np.nonzero(inp["lyot"])
            self.win = (int(nz[0].min()), int(nz[0].max()) + 1, int(nz[1].min()),
                        int(nz[1].max()) + 1)
        self.per_lam = []
        for lam in inp["lam"]:
            k = 2.0 * math.pi / lam
            h = np.exp(1j * k * spec.z * np.sqrt(1.0 - 0.25 * (lam / ap_rad) ** 2 * f2))
            sag1 = torch.as_tensor(inp["sag1"].astype(np.float64), device=self.dev)
            sag2 = torch.as_tensor(inp["sag2"].astype(np.float64), device=self.dev)
            m1 = torch.exp((-1.0 * 4.0 * math.pi / lam) * 1j * sag1)
            m2 = torch.exp((+1.0 * 4.0 * math.pi / lam) * 1j * sag2)  # mirror sign -1
            lf = -1.0 * lam * spec.fpm_focal_ratio * 2 * ef.beamRadiusPhysical  # fRatioSign -1
            c = -1.0 * inp["dm"] ** 2 / (1j * lf) * dx * dx / (-1j * -1.0 * lf)  # zoomFftSign -1
            lff = lam * 2 * ef.beamRadiusPhysical * tel.primaryfRatio
            self.per_lam.append(dict(
                pre=pupil * (1 + 1j) * m1, H=torch.as_tensor(h, device=self.dev), m2=m2,
                A1=_mft_ops(xe, xm, lf, +1.0, self.dev), A2=_mft_ops(xm, xe + dx / 2, lf, -1.0,
                                                                     self.dev), c=c,
                A3=_mft_ops(xe, xo, lff, -1.0, self.dev), pref3=dx * dx / (1j * lff), lam=lam))

    def mask(self, sags: torch.Tensor, lam: float) -> torch.Tensor:
        """fliplr(M) - 1 of the hex mask on the S x S grid."""
        ids = self.ids
        sag = torch.where(ids > -1, sags[ids.clamp(min=0)], torch.zeros((), dtype=sags.dtype,
                                                                         device=self.dev))
        m = (self.cnt * torch.exp(2 * math.pi * 1j * 2.0 * sag / lam)).sum(0) / float(
            self.n_sub * self.n_sub)
        return torch.flip(m, dims=[1]) - 1.0

    def field(self, li: int, amp: float, sags: torch.Tensor,
              calibrating: bool = False) -> torch.Tensor:
        """Final image field of an on-axis source of amplitude amp at
        wavelength index li with the candidate's sags (calibrating: without
        the focal-plane mask)."""
        p = self.per_lam[li]
        d = self.dtype
        c = (lambda t: t.to(d)) if d != torch.complex128 else (lambda t: t)
        e = amp * c(p["pre"])
        e = torch.fft.ifft2(torch.fft.fft2(e) * c(p["H"]))
        e = e * c(p["m2"])
        if self.box is not None:  # the support box and the Lyot window only
            r0, c0, R, C = self.box
            w0, w1, v0, v1 = self.win
            if not calibrating:
                A1, A2 = c(p["A1"]), c(p["A2"])
                f = A1[r0:r0 + R] @ e @ A1[c0:c0 + C].T
                m = c(self.mask(sags, p["lam"]))[r0:r0 + R, c0:c0 + C]
                g = complex(p["c"]) * (A2[w0:w1, r0:r0 + R] @ (m * f) @ A2[v0:v1, c0:c0 + C].T)
                ew = e[w0:w1, v0:v1] + g
            else:
                ew = e[w0:w1, v0:v1]
            ew = ew * c(self.lyot)[w0:w1, v0:v1]
            A3 = c(p["A3"])
            return complex(p["pref3"]) * (A3[:, w0:w1] @ ew @ A3[:, v0:v1].T)
        if not calibrating:
            A1, A2 = c(p["A1"]), c(p["A2"])
            f = A1 @ e @ A1.T  # square grids: the same operator on both axes
            g = complex(p["c"]) * (A2 @ (c(self.mask(sags, p["lam"])) * f) @ A2.T)
            e = e + g
        e = e * c(self.lyot)
        A3 = c(p["A3"])
        return complex(p["pref3"]) * (A3 @ e @ A3.T)


def throughput(model: Fp64Piaacmc, sags: np.ndarray, budget_s: float, n_max: int):
    """Fields/s of the plain path over candidates sags[c] (wavelength 0, on-axis),
    one field per call, timed end to end on the device."""
    dev = model.dev
    s = [torch.as_tensor(v, device=dev) for v in sags]
    model.field(0, 1.0, s[0])  # warm-up (cuFFT plans, cuBLAS handles)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n = 0
    while n < n_max and time.perf_counter() - t0 < budget_s:
        model.field(0, 1.0, s[n % len(s)])
        n += 1
        torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return n / dt, n, dt
