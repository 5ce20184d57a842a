"""FP64 CPU restatement of the reference's optical elements, region contrast and
response-matrix objective.

TEST INFRASTRUCTURE ONLY: this is the correctness oracle (and the timed CPU
baseline). The shipped library never imports it.

Every function names the reference lines it restates. Arrays are numpy
[row(y)][col(x)] (== Armadillo (row, col)); cubes are [slice][row][col].
"""
from __future__ import annotations

import math

import numpy as np

from .csim_fft import (ArrayGeom, ZoomFft, fft2, fft_shift, fft_truncate, ifft2,
                       fresnel_propagate_as, mft)


# ------------------------------------------------------------- telescope --
class Telescope:
    """telescope.cpp:21-30 (primaryfLength = fRatio * D), :58-60 compute_loD."""

    def __init__(self, primary_diameter: float, primary_f_ratio: float, magnification: float = 1.0):
        self.primaryDiameter = primary_diameter
        self.primaryfRatio = primary_f_ratio
        self.magnification = magnification
        self.primaryfLength = primary_f_ratio * primary_diameter

    def compute_loD(self, lam: float) -> float:
        return self.magnification * self.primaryfLength * lam / self.primaryDiameter


# ----------------------------------------------------------------- efield --
def optical_parameters(beam_radius: float, pixel_scale: float, array_size: int):
    """efield.cpp:419-430: beamSizePixels = ceil(2 R / dx); arrayRadiusPhysical
    = R * arraySizePixels / beamSizePixels."""
    beam_px = math.ceil(2 * beam_radius / pixel_scale)
    return beam_radius * array_size / beam_px


def wavelength_bandwidth(center: float, frac: float, n: int) -> np.ndarray:
    """efield.cpp:365-381 set_wavelength_bandwidth."""
    lo = center - center * frac / 2
    hi = center + center * frac / 2
    if n == 1:
        return np.array([lo])
    d = (hi - lo) / (n - 1.0)
    return lo + np.arange(n) * d


def point_source_field(geom: ArrayGeom, nlam: int, flux: float, tip: float, tilt: float,
                       magnification: float = 1.0) -> np.ndarray:
    """efield.cpp:295-304 (pointSource: amplitude sqrt(flux), tip/tilt scaled by
    magnification) and :179-206 init_point_sources:
    E = sqrt(flux) * exp(2 pi i (2 xx tip / Lx + 2 yy tilt / Ly)) on every slice."""
    xx, yy, _, _ = geom.mesh()
    amp = math.sqrt(flux)
    tip *= magnification
    tilt *= magnification
    ph = np.exp(1j * 2.0 * math.pi * (2 * xx * tip / geom.physicalSizeX
                                      + 2 * yy * tilt / geom.physicalSizeY))
    return np.broadcast_to(amp * ph, (nlam,) + xx.shape).astype(np.complex128)


# ----------------------------------------------------------- field masks --
def mask_apply(cube: np.ndarray, m: np.ndarray) -> np.ndarray:
    """mask.cpp:38-46 with cxMaskMat = m + i m (mask.cpp:53-58): the reference
    multiplies by (1+i) m, i.e. sqrt(2) e^{i pi/4} m."""
    return cube * (m + 1j * m)[None]


def mirror_apply(cube: np.ndarray, sag: np.ndarray, lambdas, sign: float = 1.0) -> np.ndarray:
    """mirror.cpp:35-44 with mirrorPhase = exp(-sign 4 pi i sag / lambda) (:66-72)."""
    out = np.empty_like(cube)
    for k, lam in enumerate(lambdas):
        out[k] = cube[k] * np.exp((-sign * 2 * 2 * math.pi / lam) * 1j * sag)
    return out


def complex_mask_apply(cube: np.ndarray, amp: np.ndarray, ph: np.ndarray) -> np.ndarray:
    """complexMask.cpp:24-55 and :57-66: centred sub-array * amp exp(-i ph)."""
    out = cube.copy()
    cm = amp * np.exp(-1j * ph)
    r0 = cube.shape[-2] // 2 - cm.shape[0] // 2
    c0 = cube.shape[-1] // 2 - cm.shape[1] // 2
    out[..., r0:r0 + cm.shape[0], c0:c0 + cm.shape[1]] *= cm
    return out


# ------------------------------------------------------- deformable mirror --
def dm_influence(geom: ArrayGeom, sigma: float, n_act: int) -> np.ndarray:
    """deformableMirror.cpp:205-214: exp(-4 ln2 r^2 / s^2), s = sigma L / nAct."""
    xx, yy, _, _ = geom.mesh()
    s = sigma * geom.physicalSizeX / float(n_act)
    return np.exp(-4 * math.log(2) * (xx ** 2 + yy ** 2) / (s * s))


def dm_surface(act: np.ndarray, influence: np.ndarray) -> np.ndarray:
    """deformableMirror.cpp:216-270: upsample actuators to delta points, FFT,
    half-cell shift phase, fft_truncate to the influence size, multiply by
    FFT(influence), IFFT, real part."""
    nar, nac = act.shape
    nr, nc = influence.shape
    ur = math.ceil((nr + 1) / float(nar))
    uc = math.ceil((nc + 1) / float(nac))
    up = np.zeros((ur * nar, uc * nac))
    up[::ur, ::uc] = act
    ft = fft2(up.astype(np.complex128))
    n_up_r, n_up_c = ft.shape
    hr, hc = n_up_r // 2, n_up_c // 2
    fx = np.concatenate([np.linspace(0.0, hr - 1, hr), np.linspace(-hr, -1.0, hr)]) / nr
    fy = np.concatenate([np.linspace(0.0, hc - 1, hc), np.linspace(-hc, -1.0, hc)]) / nc
    fxs = np.ones((n_up_r, 1)) * fx[None, :]
    fys = fy[:, None] * np.ones((1, n_up_c))
    phase = fxs * (nr * (1 - 1 / float(nar)) / 2) + fys * (nc * (1 - 1 / float(nac)) / 2)
    ft = ft * np.exp(2 * math.pi * 1j * phase)
    trunc = fft_truncate(ft, nr, nc)
    return np.real(ifft2(trunc * fft2(influence.astype(np.complex128))))


# --------------------------------------------------------------- Fresnel --
def fresnel_element(cube, lambdas, array_radius: float, z: float, pad: int = 1):
    """fresnelPropagator.cpp:23-61 (optional 2x zero pad, crop)."""
    if pad == 1:
        return fresnel_propagate_as(cube, lambdas, array_radius, z)
    nr, nc = cube.shape[-2:]
    p = np.zeros(cube.shape[:-2] + (2 * nr, 2 * nc), dtype=np.complex128)
    p[..., nr // 2:3 * nr // 2, nc // 2:3 * nc // 2] = cube
    p = fresnel_propagate_as(p, lambdas, pad * array_radius, z)
    return p[..., nr // 2:3 * nr // 2, nc // 2:3 * nc // 2].copy()


# --------------------------------------------------------- final image MFT --
def fraunhofer_focal_geometry(tel: Telescope, ref_lambda: float, fov_fld: float, spl: float) -> ArrayGeom:
    """fraunhoferFocal.cpp:65-72: ceil(FOV * spl)^2 pixels at loD / spl."""
    n = math.ceil(fov_fld * spl)
    return ArrayGeom.set_xy(n, n, tel.compute_loD(ref_lambda) / spl)


def fraunhofer_focal(cube, gin: ArrayGeom, gout: ArrayGeom, lambdas, beam_radius: float,
                     f_ratio: float, use_czt: bool = False):
    """fraunhoferFocal.cpp:23-63: lambda f = lambda 2 R fRatio, zoomFft to gout."""
    lfl = np.asarray(lambdas) * 2 * beam_radius * f_ratio
    z = ZoomFft(gin, gout, lfl)
    return np.stack([(z.execute if use_czt else z.mft)(cube[k], k) for k in range(len(lambdas))])


# --------------------------------------------------------------- hex FPM --
def hex_centers(n_rings: int, hex_step: float = 1.0):
    """complexHexMaskFPM.cpp:236-315 (radial cut (int)sqrt(hx^2+hy^2) < nRings,
    ring-by-ring numbering, sorted by number)."""
    i_max = int(n_rings / 3 + 2)
    j_max = int(n_rings / math.sqrt(3) + 2)
    bad = 1e8
    hx_l, hy_l, ring_l, num_l = [], [], [], []
    idx = 0
    for ii1 in range(-i_max, i_max):
        for jj1 in range(-j_max, j_max):
            hx = hex_step * ii1 * 3.0
            hy = hex_step * jj1 * math.sqrt(3.0)
            for _ in range(2):
                ring = int(math.sqrt(hx * hx + hy * hy))
                hx_l.append(hx); hy_l.append(hy); ring_l.append(ring)
                num_l.append(0.0 if ring < n_rings else bad + idx)
                idx += 1
                hx += hex_step * 1.5
                hy += hex_step * math.sqrt(3.0) / 2.0
    num = np.array(num_l)
    ring = np.array(ring_l)
    cnt = 0
    for r in range(n_rings + 1):
        for i in np.nonzero((ring == r) & (num == 0))[0]:
            num[i] = cnt
            cnt += 1
    order = np.argsort(num, kind="stable")
    num, hx, hy, ring = num[order], np.array(hx_l)[order], np.array(hy_l)[order], ring[order]
    good = num < bad
    return num[good].astype(np.int64), hx[good], hy[good], ring[good]


def hex_centers_standard(n_rings: int):
    """Standard hexagonal rings (3 n (n + 1) + 1 cells), used by the synthetic
    workloads that ask for "N rings (M hexes)"; same centre spacing as the
    reference layout (neighbour distance sqrt(3) hexStep)."""
    pts = []
    for q in range(-n_rings, n_rings + 1):
        for r in range(max(-n_rings, -q - n_rings), min(n_rings, -q + n_rings) + 1):
            x = 1.5 * q
            y = math.sqrt(3.0) * (r + q / 2.0)
            ring = max(abs(q), abs(r), abs(-q - r))
            pts.append((ring, math.atan2(y, x), x, y))
    pts.sort(key=lambda p: (p[0], p[1]))
    hx = np.array([p[2] for p in pts])
    hy = np.array([p[3] for p in pts])
    ring = np.array([p[0] for p in pts])
    return np.arange(len(pts)), hx, hy, ring


def complex_interpolated_mask(hexnum: np.ndarray, nsub: np.ndarray, sags: np.ndarray,
                              lam: float, n_sub_pix: int, phase_sign: float = 1.0,
                              use_only_this_hex: int = -1) -> np.ndarray:
    """complexHexMaskFPM.cpp:44-99: gather sags by hex id (0 outside the mask),
    optional useOnlyThisHex selection, then
    sum_k n[k] exp(phaseSign 2 pi i 2 sag / lambda) / nSubPix^2.
    hexnum/nsub are [3][S][S] (slices first)."""
    ids = hexnum.astype(np.int64)
    sag = np.where(ids > -1, sags[np.clip(ids, 0, None)], 0.0)
    n = nsub.astype(np.float64)
    if use_only_this_hex > -1:
        keep = (ids == use_only_this_hex)
        if use_only_this_hex == sags.size:
            keep |= (ids == -1)
        n = np.where(keep, n, 0.0)
    return (n * np.exp(phase_sign * 2 * math.pi * 1j * 2.0 * sag / lam)).sum(0) / float(n_sub_pix * n_sub_pix)


def double_fraunhofer_interp_fpm(cube, lambdas, egeom: ArrayGeom, fpm_scale: float,
                                 pad_factor: float, masks, lf_factor: float = 3.52):
    """doubleFraunhoferInterpFPM::execute (doubleFraunhoferInterpFPM.cpp:24-65)
    with its geometry (init_geom, :86-121) and complexHexMaskFPM::execute
    (complexHexMaskFPM.cpp:25-42), per wavelength slice: zoomFft of E to an
    nz x nz grid (nz = int(padFactor N), pixel centres (i - nz/2) fpmScale)
    at lambda f = 3.52 lambda; the S x S mask multiplies the block starting at
    (nz/2 - S/2, nz/2 - S/2), the rest of the grid is left as it is; zoomFft
    back to E's geometry at -3.52 lambda. masks[sl] is the complex
    interpolated mask of slice sl (complex_interpolated_mask, no flip);
    fpm_scale is one zoom pixel or one per slice."""
    cube = np.asarray(cube, dtype=np.complex128)
    n = cube.shape[-1]
    nz = int(pad_factor * n)
    scales = np.broadcast_to(np.asarray(fpm_scale, dtype=np.float64), (len(lambdas),))
    out = np.empty_like(cube)
    for sl, lam in enumerate(lambdas):
        zg = ArrayGeom.set_xy_offset_m1(nz, nz, float(scales[sl]))
        lf_in = lf_factor * lam
        z = ZoomFft(egeom, zg, [lf_in]).mft(cube[sl], 0)
        m = np.asarray(masks[sl])
        r0, c0 = nz // 2 - m.shape[0] // 2, nz // 2 - m.shape[1] // 2
        z[r0:r0 + m.shape[0], c0:c0 + m.shape[1]] *= m
        out[sl] = ZoomFft(zg, egeom, [-lf_in]).mft(z, 0)
    return out


def double_fraunhofer_fpm(cube, lambdas, egeom: ArrayGeom, beam_radius: float,
                          pixel_scale: float, zoom_factor: float, pad_factor: float, mask):
    """doubleFraunhoferFPM::execute (doubleFraunhoferFPM.cpp:23-110): the
    same walk as doubleFraunhoferInterpFPM with the zoom pixel
    dxprime = 2 (beamRadius / (pixelScale N zoomFactor)) lambda 80 of each
    slice and one fixed complex mask (slice maskIndex) on every slice."""
    n = np.asarray(cube).shape[-2]
    scales = [2 * (beam_radius / (pixel_scale * n * zoom_factor)) * lam * 80 for lam in lambdas]
    return double_fraunhofer_interp_fpm(cube, lambdas, egeom, scales, pad_factor,
                                        [mask] * len(lambdas))


def hex_mask_pixel_scale(beam_radius: float, pixel_scale: float, mask_size: int,
                         zoom_factor: float, lambda_ref: float, fpm_f_ratio: float) -> float:
    """complexHexMaskFPM.cpp:199-206 / :367-369 compute_fpmScale."""
    return 2 * (beam_radius / (pixel_scale * mask_size * zoom_factor)) * lambda_ref * fpm_f_ratio


# -------------------------------------------------- fpmPupToLyot (Babinet) --
def pup_to_lyot_conv(cube, lambdas, egeom: ArrayGeom, mask_geom: ArrayGeom, mask_m1,
                     lfl, f_ratio_sign: float, zoom_fft_sign: float, babinet: bool = True,
                     use_czt: bool = False):
    """fpmPupToLyot.cpp:24-167, reference algorithm: per lambda the mask hat
    FFT(fft_shift(zoomFftSign zoomFft(maskGeom -> paddedGeom)(M - 1))) is built
    (:76-99); per field: embed E at [N/2, 3N/2) in 2N x 2N, FFT, multiply by the
    mask hat, IFFT, times dx^2 / (-i fRatioSign lambda f), + padded E (Babinet),
    crop (:112-161). mask_m1 is [slice][S][S] = fliplr(M) - 1 for the hex adapter
    (:444-450); lfl already carries fRatioSign (:427-431)."""
    nr, nc = cube.shape[-2:]
    pgeom = ArrayGeom.set_xy(2 * nc, 2 * nr, egeom.pixelSizeX)
    out = np.empty_like(cube)
    for sl, lam in enumerate(lambdas):
        z = ZoomFft(mask_geom, pgeom, lfl)
        hat = zoom_fft_sign * (z.execute if use_czt else z.mft)(mask_m1[sl], sl)
        fhat = fft2(fft_shift(hat))
        scale = pgeom.pixelSizeX ** 2 / (-1j * f_ratio_sign * lfl[sl])
        p = np.zeros((2 * nr, 2 * nc), dtype=np.complex128)
        p[nr // 2:3 * nr // 2, nc // 2:3 * nc // 2] = cube[sl]
        r = ifft2(fhat * fft2(p)) * scale
        if babinet:
            r = r + p
        out[sl] = r[nr // 2:3 * nr // 2, nc // 2:3 * nc // 2]
    return out


def pup_to_lyot_mft(cube, lambdas, egeom: ArrayGeom, mask_geom: ArrayGeom, mask_m1,
                    lfl, f_ratio_sign: float, zoom_fft_sign: float):
    """The same linear operator as pup_to_lyot_conv in matrix-Fourier form.
    The 2N circular convolution never wraps (E is embedded in the central N),
    and fft_shift by N places the kernel origin on the padded pixel at +dx/2, so
    E_out(x) = E(x) + c * sum_m (M-1)(m) e^{-2 pi i m (x + dx/2) / lf}
                                  * sum_j E(j) e^{+2 pi i m x_j / lf}
    with c = zoomFftSign * dm^2 / (i lf) * dx^2 / (-i fRatioSign lf)."""
    out = np.empty_like(cube)
    dx = egeom.pixelSizeX
    dm = mask_geom.pixelSizeX
    for sl, lam in enumerate(lambdas):
        lf = lfl[sl]
        f = mft(cube[sl], egeom.pixelX, egeom.pixelY, mask_geom.pixelX, mask_geom.pixelY,
                lf, 1.0, sign=+1.0)
        c = zoom_fft_sign * dm * dm / (1j * lf) * dx * dx / (-1j * f_ratio_sign * lf)
        g = mft(mask_m1[sl] * f, mask_geom.pixelX, mask_geom.pixelY,
                egeom.pixelX + dx / 2, egeom.pixelY + dx / 2, lf, c, sign=-1.0)
        out[sl] = cube[sl] + g
    return out


def padded_fft_fpm(cube, pad: int, masks):
    """Plain Lyot occulter with an FFT-sampled mask: per slice embed E at the
    centre of a zeroed pad x pad array (the embedding of
    fpmPupToLyot.cpp:112-118), FFT, multiply by the mask given in centred
    focal coordinates (masks[sl], index pad // 2 = zero frequency), inverse
    FFT (/ pad^2) and crop the centre (:154-157)."""
    n = cube.shape[-1]
    o = (pad - n) // 2
    out = np.empty_like(cube)
    for sl in range(cube.shape[0]):
        p = np.zeros((pad, pad), dtype=np.complex128)
        p[o:o + n, o:o + n] = cube[sl]
        r = ifft2(fft2(p) * np.fft.ifftshift(masks[sl]))
        out[sl] = r[o:o + n, o:o + n]
    return out


# ------------------------------------------------------- region contrast --
def region_pixels(geom: ArrayGeom, loD: float, radius1, radius2, angle1=-180.0, angle2=180.0,
                  xlim1=-1e300, xlim2=1e300) -> np.ndarray:
    """regionContrast.cpp:89-101 (returns a boolean [row][col] mask).
    The defaults select a full annulus; the reference's strict angle bounds
    exclude theta == +-180 exactly as here."""
    xx, yy, rr, tt = geom.mesh()
    return ((xx / loD >= xlim1) & (xx / loD <= xlim2) & (rr / loD >= radius1) & (rr / loD <= radius2)
            & (tt > angle1 * math.pi / 180) & (tt < angle2 * math.pi / 180))


def intensity_sum(fields) -> np.ndarray:
    """regionContrast.cpp:132-141: I = sum over sources, polarizations and
    wavelengths of |E|^2. fields: iterable of [slice][row][col] cubes."""
    tot = None
    for f in fields:
        i = (np.abs(f) ** 2).sum(0)
        tot = i if tot is None else tot + i
    return tot


def region_contrast(full_i: np.ndarray, calib_i: np.ndarray, region: np.ndarray) -> float:
    """regionContrast.cpp:145-195: mean over the region of I / max(I_calib)."""
    return float(np.mean((full_i / calib_i.max())[region]))


# ------------------------------------------------ response-matrix objective --
def opt_hex_resp_objective(m_cubes, wavelengths, calib: float, x: np.ndarray,
                           phase_sign: float = 1.0, objective: str = "mean") -> np.ndarray:
    """optObjective.cpp:24-69: X~ = [X; 0]; per (s, p, lambda):
    P = exp(i phaseSign 4 pi / lambda X~), E = M P, pix += |E|^2;
    f = mean (or max) over pixels / calib. m_cubes: list over (s, p) of
    [slice][npix][nhex+1] complex arrays; x: [nvar][pop]."""
    xf = np.vstack([x, np.zeros((1, x.shape[1]))])
    pix = np.zeros((m_cubes[0].shape[1], x.shape[1]))
    for m in m_cubes:
        for sl, lam in enumerate(wavelengths):
            a = phase_sign * 4 * math.pi / lam
            e = m[sl] @ np.exp(1j * a * xf)
            pix += (e * e.conj()).real
    red = pix.mean(0) if objective == "mean" else pix.max(0)
    return red / calib


# ---------------------------------------------------- zoomFftPropagator --
def zoom_fft_propagator_geometry(n_rows: int, n_cols: int, beam_radius: float,
                                 pixel_scale: float, lambda0: float, zoom_factor: float,
                                 pad_factor: float, direction: int):
    """zoomFftPropagator::execute (zoomFftPropagator.cpp:23-91): the output
    grid and lambda f. dir +1: padFactor N pixels of dxprime =
    2 (beamRadius / (pixelScale N zoomFactor)) lambda0 80 at (i - n/2) dxprime,
    lambda f = 3.52 lambda0; dir -1: N / padFactor pixels of pixelScale at
    (i - n/2) pixelScale, lambda f = -3.52 lambda0 (lambda0: the first
    wavelength, for every slice)."""
    if direction == 1:
        d = 2 * (beam_radius / (pixel_scale * n_rows * zoom_factor)) * lambda0 * 80
        nr, nc, lf = int(pad_factor * n_rows), int(pad_factor * n_cols), lambda0 * 3.52
    else:
        d = pixel_scale
        nr, nc, lf = int(n_rows / pad_factor), int(n_cols / pad_factor), -lambda0 * 3.52
    return ArrayGeom((np.arange(nc) - nc / 2.0) * d, (np.arange(nr) - nr / 2.0) * d, d, d), lf


def zoom_fft_propagator(cube, gin: ArrayGeom, beam_radius: float, pixel_scale: float,
                        lambdas, zoom_factor: float, pad_factor: float, direction: int):
    """The element on every slice: zoomFft from gin to the element's grid."""
    n_rows, n_cols = cube.shape[-2:]
    gout, lf = zoom_fft_propagator_geometry(n_rows, n_cols, beam_radius, pixel_scale,
                                            float(lambdas[0]), zoom_factor, pad_factor, direction)
    z = ZoomFft(gin, gout, [lf] * len(lambdas))
    return np.stack([z.mft(cube[k], k) for k in range(len(lambdas))]), gout
