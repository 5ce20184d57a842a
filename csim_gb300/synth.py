"""Seeded synthetic inputs (pure numpy) with the shapes of the benchmark
configurations, and the plain descriptions of telescope, field and sources.

The reference's own example data (pupils, PIAA sags, hex tables, response
matrices) are not available, so every workload is generated from a seed:
apertures, PIAA even-polynomial sags, standard hex layouts and uniform hex
sags. This module has no GPU dependency; the hex interpolation tables are
built on the GPU by workloads.hex_tables.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Telescope:
    """telescope.cpp:21-60."""
    primaryDiameter: float
    primaryfRatio: float
    magnification: float = 1.0

    @property
    def primaryfLength(self) -> float:
        return self.primaryfRatio * self.primaryDiameter

    def compute_loD(self, lam: float) -> float:
        return self.magnification * self.primaryfLength * lam / self.primaryDiameter


@dataclass
class PointSource:
    """efield pointSource: flux (amplitude sqrt(flux)), tip/tilt in the
    reference's units (multiplied by the telescope magnification)."""
    flux: float = 1.0
    tip: float = 0.0
    tilt: float = 0.0


@dataclass
class EField:
    """efield.cpp: square N x N array, beam radius and pixel scale (metres)."""
    n: int
    beamRadiusPhysical: float
    pixelScale: float
    wavelengths: np.ndarray
    sources: list = field(default_factory=lambda: [PointSource()])

    @property
    def arrayRadiusPhysical(self) -> float:
        beam_px = math.ceil(2 * self.beamRadiusPhysical / self.pixelScale)
        return self.beamRadiusPhysical * self.n / beam_px

    def pixel_centres(self) -> np.ndarray:
        d = self.pixelScale
        return -(d * self.n - d) / 2.0 + np.arange(self.n) * d


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
    # "random": seeded PIAA sags (the benchmark's shapes, no dark hole);
    # "apodized": optics with a deep dark hole for the optimisers (see
    # prolate_apodizer): flat PIAA mirrors and a prolate-apodized pupil
    design: str = "random"

    @property
    def n_hex(self) -> int:
        return 3 * self.n_rings * (self.n_rings + 1) + 1


def designed_piaacmc_spec(**kw) -> PiaacmcSpec:
    """The PIAACMC chain with optics that admit a deep dark hole: the pupil
    apodized by the prolate spheroidal function of a focal-plane disk of
    radius alpha (about 0.53 lambda/D) whose eigenvalue is 1/2, and flat PIAA
    mirrors 1 mm apart. With the apodization psi, Pi psi = psi / 2 on the
    pupil (Pi: band-limit to the disk), so a focal mask that shifts the disk
    by pi gives E_Lyot = psi - 2 Pi psi = 0 (the phase-mask coronagraph
    limit, Guyon 2003-2010). The hex mask has to find that phase pattern,
    including its chromatic and pixelation compromises: with zero sags the
    2-8 lambda/D contrast is ~4e-4, the ideal pi disk gives ~2e-6 over a 10%
    band (1e-7 range at one wavelength), and per-hex phases can do better."""
    base = dict(design="apodized", z=1e-3)
    base.update(kw)
    return PiaacmcSpec(**base)


def prolate_radial(alpha: float, n: int = 160):
    """Fundamental eigenfunction of the band-limiting operator Pi on radial
    functions of a disk pupil of radius 1/2 (units of D) for a focal disk of
    radius alpha (lambda/D): (Pi f)(r) = int_0^{1/2} K(r, r') f(r') r' dr',
    K(r, r') = 4 pi^2 int_0^alpha J0(2 pi rho r) J0(2 pi rho r') rho d rho,
    discretised by Gauss-Legendre quadrature (Nystrom). Returns (eigenvalue,
    f evaluator)."""
    from scipy.special import j0
    x, w = np.polynomial.legendre.leggauss(n)
    r, wr = 0.25 * (x + 1), 0.25 * w
    y, v = np.polynomial.legendre.leggauss(n)
    rho, wp = 0.5 * alpha * (y + 1), 0.5 * alpha * v
    J = j0(2 * np.pi * np.outer(r, rho))
    K = (2 * np.pi) ** 2 * (J * (wp * rho)) @ J.T
    s = np.sqrt(wr * r)
    ev, V = np.linalg.eigh(s[:, None] * K * s[None, :])
    lam0, f = ev[-1], V[:, -1] / s
    f = f if f[0] > 0 else -f
    coef = wr * r * f / lam0

    def evaluate(rq):
        rq = np.asarray(rq, np.float64)
        Jq = j0(2 * np.pi * np.outer(rq.ravel(), rho))
        Kq = (2 * np.pi) ** 2 * (Jq * (wp * rho)) @ J.T
        return (Kq @ coef).reshape(rq.shape)
    return lam0, evaluate


def prolate_apodizer(n: int, radius_px: float, target: float = 0.5):
    """Pupil amplitude [n][n]: the prolate function whose eigenvalue is
    `target` (disk radius found by bisection), normalised to 1 at the centre,
    zero outside the pupil radius radius_px. Returns (apodizer, alpha)."""
    lo, hi = 0.2, 1.5
    for _ in range(40):
        mid = 0.5 * (lo + hi)
        if prolate_radial(mid)[0] < target:
            lo = mid
        else:
            hi = mid
    alpha = 0.5 * (lo + hi)
    _, f = prolate_radial(alpha)
    c = np.arange(n) - n / 2 + 0.5
    rr = np.hypot(c[:, None], c[None, :]) / (2.0 * radius_px)  # units of D
    a = np.zeros((n, n))
    m = rr <= 0.5
    a[m] = f(rr[m])
    return a / f(np.zeros(1))[0], alpha


def piaacmc_arrays(spec: PiaacmcSpec, sources=None) -> dict:
    """Every seeded host-side input of the PIAACMC chain except the hex
    interpolation tables (pupil, Lyot stop, PIAA sags, hex centres, mask
    geometry, telescope and efield descriptions)."""
    rng = np.random.default_rng(spec.seed)
    dx = 2 * spec.beam_radius / spec.beam_px
    lam = np.asarray(spec.wavelengths, dtype=np.float64)
    tel = Telescope(spec.diameter, spec.f_ratio)
    ef = EField(spec.n, spec.beam_radius, dx, lam, sources or [PointSource()])
    lam_ref = float(lam.mean())
    lod_fpm = lam_ref * spec.fpm_focal_ratio           # lambda/D at the FPM (metres)
    hx, hy = hex_layout_standard(spec.n_rings)
    if spec.design == "apodized":
        pupil, _ = prolate_apodizer(spec.n, spec.beam_px / 2.0)
        pupil = pupil.astype(np.float32)
        sag1 = np.zeros((spec.n, spec.n), np.float32)
        sag2 = np.zeros((spec.n, spec.n), np.float32)
    else:
        pupil = circle_mask(spec.n, spec.beam_px / 2.0)
        sag1 = piaa_sag(spec.n, dx, spec.beam_radius, rng).astype(np.float32)
        sag2 = piaa_sag(spec.n, dx, spec.beam_radius, rng).astype(np.float32)
    return dict(pupil=pupil,
                lyot=circle_mask(spec.n, spec.lyot * spec.beam_px / 2.0),
                sag1=sag1, sag2=sag2,
                dm=lod_fpm / spec.fpm_sampling, fpm_radius=spec.fpm_radius_lod * lod_fpm,
                dx=dx, lam=lam, tel=tel, ef=ef, hex_x=hx, hex_y=hy, lam_ref=lam_ref,
                lod_image=tel.compute_loD(lam_ref))




# ------------------------------------------------------------ plain Lyot
def noll_nm(j: int):
    """Noll index j >= 1 -> radial order n and azimuthal m (m > 0: cos,
    m < 0: sin, even j carries cos)."""
    n = 0
    while (n + 1) * (n + 2) // 2 < j:
        n += 1
    k = j - n * (n + 1) // 2 - 1
    m = 2 * ((k + 1) // 2) if n % 2 == 0 else 2 * (k // 2) + 1
    return n, (m if (j % 2 == 0 or m == 0) else -m)


def zernike(j: int, rho: np.ndarray, theta: np.ndarray) -> np.ndarray:
    """Orthonormal (over the unit disk) Zernike polynomial of Noll index j."""
    n, m = noll_nm(j)
    am = abs(m)
    rad = np.zeros_like(rho)
    for s in range((n - am) // 2 + 1):
        c = ((-1) ** s * math.factorial(n - s)
             / (math.factorial(s) * math.factorial((n + am) // 2 - s)
                * math.factorial((n - am) // 2 - s)))
        rad = rad + c * rho ** (n - 2 * s)
    if m == 0:
        return math.sqrt(n + 1) * rad
    ang = np.cos(am * theta) if m > 0 else np.sin(am * theta)
    return math.sqrt(2 * (n + 1)) * rad * ang


@dataclass
class PlainLyotSpec:
    """Plain Lyot coronagraph: 512^2 pupil, circular aperture of radius 200 px
    with a 0.3 central obstruction, Zernike 4-15 aberration (N(0,1)
    coefficients, seeded) scaled to 10 nm RMS wavefront, zero-padded 2048^2
    FFT to the focal plane, opaque occulting disk of radius 3 lambda/D,
    inverse FFT, Lyot stop at 0.9 of the pupil radius, final 128^2 MFT at
    0.25 lambda/D (+-16 lambda/D)."""
    n: int = 512
    pad: int = 2048
    radius_px: float = 200.0
    obstruction: float = 0.3
    beam_radius: float = 0.01
    wavelengths: tuple = (550e-9,)
    f_ratio: float = 15.0
    diameter: float = 2.4
    zernike_modes: tuple = tuple(range(4, 16))
    wfe_rms: float = 10e-9
    occulter_lod: float = 3.0
    lyot: float = 0.9
    n_out_fov: float = 32.0
    spl: float = 4.0
    seed: int = 5


def plain_lyot_arrays(spec: PlainLyotSpec, sources=None) -> dict:
    """Seeded host-side inputs of the plain Lyot chain: pupil, aberration
    (as a mirror sag: half the wavefront), FFT-sampled occulter per
    wavelength, Lyot stop, telescope and efield."""
    rng = np.random.default_rng(spec.seed)
    dx = spec.beam_radius / spec.radius_px
    lam = np.asarray(spec.wavelengths, dtype=np.float64)
    tel = Telescope(spec.diameter, spec.f_ratio)
    ef = EField(spec.n, spec.beam_radius, dx, lam, sources or [PointSource()])
    pupil = circle_mask(spec.n, spec.radius_px, spec.obstruction)
    c = (spec.n - 1) / 2.0
    yy, xx = np.mgrid[:spec.n, :spec.n]
    rho = np.hypot(xx - c, yy - c) / spec.radius_px
    theta = np.arctan2(yy - c, xx - c)
    coef = rng.standard_normal(len(spec.zernike_modes))
    w = sum(a * zernike(j, rho, theta) for a, j in zip(coef, spec.zernike_modes))
    inside = pupil > 0
    w = w - w[inside].mean()
    w *= spec.wfe_rms / np.sqrt(np.mean(w[inside] ** 2))
    w[~inside] = 0.0
    # FFT focal sampling: 2 R / pad lambda/D per pixel at every wavelength;
    # the occulter has a fixed size in lambda_ref / D
    lam_ref = float(lam.mean())
    P = spec.pad
    fy, fx = np.mgrid[:P, :P]
    fr = np.hypot(fx - P // 2, fy - P // 2) * (2 * spec.radius_px / P)  # lambda/D
    occ = np.stack([(fr > spec.occulter_lod * lam_ref / l).astype(np.float32) for l in lam])
    return dict(pupil=pupil, sag=(0.5 * w).astype(np.float32), occulter=occ,
                lyot=circle_mask(spec.n, spec.lyot * spec.radius_px), dx=dx, lam=lam, tel=tel,
                ef=ef, lam_ref=lam_ref, lod_image=tel.compute_loD(lam_ref))


# ------------------------------------------------------------- broadband
def segmented_hex_aperture(n: int, n_rings: int, radius_px: float, gap: float) -> np.ndarray:
    """Hex-segmented aperture: the 3 n (n+1) + 1 flat-topped hexagonal
    segments of the standard rings (neighbours along 90 and +-30 degrees),
    scaled so the outermost segment corners touch radius_px, each segment
    shrunk by gap of the segment pitch (1% gaps: gap = 0.01)."""
    # outermost corner distance in pitch units: ring n along 30 deg plus the
    # circumradius 1/sqrt(3)
    pitch = radius_px / (n_rings + 1.0 / math.sqrt(3.0))
    c = (n - 1) / 2.0
    yy, xx = np.mgrid[:n, :n]
    x = (xx - c) / pitch
    y = (yy - c) / pitch
    # axial coordinates of the lattice (e_q = (sqrt(3)/2, 1/2), e_r = (0, 1))
    q = x * 2.0 / math.sqrt(3.0)
    r = y - q / 2.0
    # cube rounding to the nearest lattice point
    cx, cz = q, r
    cy = -cx - cz
    rx, ry, rz = np.rint(cx), np.rint(cy), np.rint(cz)
    dxr, dyr, dzr = np.abs(rx - cx), np.abs(ry - cy), np.abs(rz - cz)
    fix_x = (dxr > dyr) & (dxr > dzr)
    fix_y = ~fix_x & (dyr > dzr)
    rx = np.where(fix_x, -ry - rz, rx)
    ry = np.where(fix_y, -rx - rz, ry)
    rz = np.where(~fix_x & ~fix_y, -rx - ry, rz)
    ring = np.maximum(np.maximum(np.abs(rx), np.abs(ry)), np.abs(rz))
    # position inside the segment, in pitch units
    px = x - rx * math.sqrt(3.0) / 2.0
    py = y - (rz + rx / 2.0)
    apo = 0.5 - gap / 2.0  # apothem of the shrunk segment
    inside = (np.abs(py) <= apo) & (math.sqrt(3.0) * np.abs(px) + np.abs(py) <= 2.0 * apo)
    return ((ring <= n_rings) & inside).astype(np.float64)


@dataclass
class BroadbandSpec:
    """Broadband batched propagation: 2048^2 pupil with a 6-ring segmented hex
    aperture (127 segments, 1% gaps), a 48 x 48 actuator deformable mirror
    (Gaussian influence, sigma = 1 actuator pitch, strokes N(0, 5 nm)),
    11 wavelengths uniform over a 10% band at 650 nm, 3 sources (on axis and
    +-0.01 lambda/D), and per-wavelength focal grids of 460^2 .. 540^2 at one
    pixel scale (the grid grows with lambda), all 33 fields in one launch."""
    n: int = 2048
    radius_px: float = 900.0
    n_rings: int = 6
    gap: float = 0.01
    beam_radius: float = 0.025
    center: float = 650e-9
    bandwidth: float = 0.10
    n_lambda: int = 11
    f_ratio: float = 15.0
    diameter: float = 2.4
    n_act: int = 48
    dm_sigma: float = 1.0
    dm_rms: float = 5e-9
    source_offsets_lod: tuple = (0.0, 0.01, -0.01)
    n_out_min: int = 460
    n_out_max: int = 540
    spl: float = 4.0
    seed: int = 11

    def n_out(self) -> list:
        return [int(round(v)) for v in np.linspace(self.n_out_min, self.n_out_max, self.n_lambda)]


def broadband_arrays(spec: BroadbandSpec) -> dict:
    """Seeded host-side inputs of the broadband chain (the DM surface itself is
    built from the strokes by the DM element)."""
    rng = np.random.default_rng(spec.seed)
    dx = spec.beam_radius / spec.radius_px
    # wavelengthBandwidth (efield.cpp:351-417): n points uniform over c (1 +- f/2)
    lam = np.linspace(spec.center * (1 - spec.bandwidth / 2), spec.center * (1 + spec.bandwidth / 2),
                      spec.n_lambda)
    tel = Telescope(spec.diameter, spec.f_ratio)
    # a tilt of t lambda/D: phase 2 pi (2 x tip / Lx) has gradient 2 pi / D_beam
    lx = spec.n * dx
    srcs = [PointSource(1.0, o * lx / (2.0 * 2.0 * spec.beam_radius), 0.0)
            for o in spec.source_offsets_lod]
    ef = EField(spec.n, spec.beam_radius, dx, lam, srcs)
    act = rng.normal(0.0, spec.dm_rms, (spec.n_act, spec.n_act))
    lam_ref = float(spec.center)
    return dict(pupil=segmented_hex_aperture(spec.n, spec.n_rings, spec.radius_px, spec.gap),
                act=act, dx=dx, lam=lam, tel=tel, ef=ef, lam_ref=lam_ref,
                lod_image=tel.compute_loD(lam_ref), n_out=spec.n_out())
