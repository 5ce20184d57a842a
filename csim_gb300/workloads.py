"""Seeded synthetic inputs with the shapes of the benchmark configurations.

The reference's own example data (pupils, PIAA sags, hex tables, response
matrices) are not available, so every workload here is generated from a
seed: apertures, Zernike aberrations, PIAA even-polynomial sags, standard hex
layouts and uniform hex sags. Hex interpolation tables are built on the GPU
by csg_hex_tables.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import coronagraph as cg
from ._lib import call
from .runtime import Context, dvec, ptr


def circle_mask(n: int, radius_px: float, obstruction: float = 0.0) -> np.ndarray:
    """Pixel-centred disk (optionally annular) on an n x n grid."""
    c = (n - 1) / 2.0
    yy, xx = np.mgrid[:n, :n]
    r = np.hypot(xx - c, yy - c)
    m = (r <= radius_px).astype(np.float64)
    if obstruction > 0:
        m[r < obstruction * radius_px] = 0.0
    return m


def piaa_sag(n: int, dx: float, radius: float, rng: np.random.Generator, pv: float = 2e-6,
             order: int = 10) -> np.ndarray:
    """Radially symmetric even polynomial sum_{k=1..order/2} c_k (r/R)^{2k},
    clamped at r = R, scaled to the given peak-to-valley inside the beam."""
    x = -(dx * n - dx) / 2.0 + np.arange(n) * dx
    rr = np.minimum(np.hypot(x[None, :], x[:, None]) / radius, 1.0)
    coef = rng.standard_normal(order // 2)
    sag = sum(c * rr ** (2 * (k + 1)) for k, c in enumerate(coef))
    inside = rr < 1.0
    span = sag[inside].max() - sag[inside].min()
    return sag * (pv / span)


def hex_layout_standard(n_rings: int):
    """Standard hexagonal rings (3 n (n+1) + 1 cells), unit neighbour pitch,
    numbered ring by ring (counter-clockwise from +x)."""
    pts = []
    for q in range(-n_rings, n_rings + 1):
        for r in range(max(-n_rings, -q - n_rings), min(n_rings, -q + n_rings) + 1):
            x = 1.5 * q / math.sqrt(3.0)
            y = (r + q / 2.0)
            ring = max(abs(q), abs(r), abs(-q - r))
            pts.append((ring, math.atan2(y, x) % (2 * math.pi), x, y))
    pts.sort(key=lambda p: (p[0], p[1]))
    return np.array([p[2] for p in pts]), np.array([p[3] for p in pts])


def hex_tables(ctx: Context, hex_x, hex_y, n_rings, design_size, fpm_scale_factor, hex_gap,
               pitch, S, n_sub, pixel_scale, fpm_radius):
    """Interpolation tables [3][S][S] (int16 ids, uint16 counts) built on the
    GPU; returned as host numpy arrays."""
    hx, hy = dvec(hex_x), dvec(hex_y)
    ids = torch.empty((3, S, S), dtype=torch.int16, device="cuda")
    cnt = torch.empty((3, S, S), dtype=torch.int16, device="cuda")
    over = C.c_int()
    call("csg_hex_tables", ctx.h, ptr(hx), ptr(hy), hx.numel(), n_rings, design_size,
         fpm_scale_factor, hex_gap, pitch, S, n_sub, pixel_scale, fpm_radius, ptr(ids), ptr(cnt),
         C.byref(over))
    return ids.cpu().numpy(), cnt.cpu().numpy().view(np.uint16), over.value


@dataclass
class PiaacmcSpec:
    """PIAACMC-style chain (the 1024^2 PIAA + hex-FPM benchmark): PIAA M1 and
    M2 even-polynomial sags (PV 2 um) separated by 1.0 m of Fresnel
    propagation, a hex-tiled phase FPM (standard rings) applied through the
    Babinet matrix-Fourier form on an S x S grid at 1/16 lambda/D, a 0.95
    Lyot stop and a final 256^2 MFT at 0.25 lambda/D."""
    n: int = 1024
    beam_px: int = 800
    beam_radius: float = 0.022
    wavelengths: tuple = (650e-9,)
    f_ratio: float = 15.1           # telescope primary f-ratio
    diameter: float = 2.4
    z: float = 1.0
    fpm_focal_ratio: float = 80.0
    S: int = 512
    fpm_sampling: float = 16.0      # mask pixels per lambda/D
    n_rings: int = 8
    n_sub: int = 64
    design_size: int = 2048
    fpm_scale_factor: float = 0.9
    hex_gap: float = 0.01
    fpm_radius_lod: float = 2.0
    sag_range: float = 0.5e-6
    lyot: float = 0.95
    n_out_fov: float = 64.0
    spl: float = 4.0
    seed: int = 2

    @property
    def n_hex(self) -> int:
        return 3 * self.n_rings * (self.n_rings + 1) + 1


def build_piaacmc(ctx: Context, spec: PiaacmcSpec, sources=None, precision: int = 6):
    """Returns (coronagraph, inputs dict with every array the oracle needs)."""
    rng = np.random.default_rng(spec.seed)
    dx = 2 * spec.beam_radius / spec.beam_px
    lam = np.asarray(spec.wavelengths, dtype=np.float64)
    tel = cg.Telescope(spec.diameter, spec.f_ratio)
    ef = cg.EField(spec.n, spec.beam_radius, dx, lam, sources or [cg.PointSource()])
    pupil = circle_mask(spec.n, spec.beam_px / 2.0)
    lyot = circle_mask(spec.n, spec.lyot * spec.beam_px / 2.0)
    sag1 = piaa_sag(spec.n, dx, spec.beam_radius, rng).astype(np.float32)
    sag2 = piaa_sag(spec.n, dx, spec.beam_radius, rng).astype(np.float32)
    lam_ref = float(lam.mean())
    lod_fpm = lam_ref * spec.fpm_focal_ratio           # lambda/D at the FPM (metres)
    dm = lod_fpm / spec.fpm_sampling
    hx, hy = hex_layout_standard(spec.n_rings)
    ids, cnt, over = hex_tables(ctx, hx, hy, spec.n_rings, spec.design_size,
                                spec.fpm_scale_factor, spec.hex_gap, 1.0, spec.S, spec.n_sub, dm,
                                spec.fpm_radius_lod * lod_fpm)
    elems = [
        cg.Mask(pupil),
        cg.Mirror(sag1, 1.0),
        cg.FresnelPropagator(spec.z),
        cg.Mirror(sag2, -1.0),
        cg.FpmPupToLyotHex(ids, cnt, spec.n_sub, len(hx), dm, spec.fpm_focal_ratio),
        cg.Mask(lyot),
        cg.FraunhoferFocal(lam_ref, spec.spl, spec.n_out_fov),
    ]
    cor = cg.Coronagraph(ctx, tel, ef, elems, precision)
    inputs = dict(pupil=pupil, lyot=lyot, sag1=sag1, sag2=sag2, hex_id=ids, count=cnt, dm=dm,
                  dx=dx, lam=lam, tel=tel, ef=ef, hex_x=hx, hex_y=hy, overflow=over,
                  lod_image=tel.compute_loD(lam_ref))
    return cor, inputs


def random_sags(rng: np.random.Generator, n_cand: int, n_hex: int, half_range: float):
    return rng.uniform(-half_range, half_range, (n_cand, n_hex))
