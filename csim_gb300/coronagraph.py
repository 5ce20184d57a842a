"""Host-side mirror of the reference's coronagraph API, driving the native
chain executor through the C ABI.

Names follow the reference: a ``Telescope`` (telescope.cpp), an ``EField``
description (efield.cpp), element classes named after the reference's
elements (mask, mirror, fresnelPropagator, complexMask, fpmPupToLyot with the
interpolated-hex adapter, fraunhoferFocal), a ``Coronagraph`` that walks them
(coronagraph.cpp:175-200) for a whole batch of (wavelength, source,
candidate) fields at once, and ``RegionContrast`` (regionContrast.cpp).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from ._lib import CSG_PREC_BF16X6, call
from .runtime import Context, dvec, ptr


from .synth import EField, PointSource, Telescope  # noqa: E402,F401


# ------------------------------------------------------------- elements
@dataclass
class Mask:
    """mask element (mask.cpp): real mask, multiplied as (m + i m) when
    ref_quirk is set, exactly as the reference does."""
    mask: np.ndarray
    ref_quirk: bool = True
    disableForCalibration: bool = False


@dataclass
class Mirror:
    """mirror element (mirror.cpp): sag in metres, phase -sign 4 pi sag / lambda."""
    sag: np.ndarray
    mirrorSign: float = 1.0


@dataclass
class FresnelPropagator:
    """fresnelPropagator (fresnelPropagator.cpp): signed distance z; padFactor
    other than 1 propagates in a 2N x 2N zero-padded array with padFactor
    times the aperture radius (fresnelPropagator.cpp:41-54)."""
    z: float
    padFactor: float = 1.0


@dataclass
class ComplexMask:
    """complexMask (complexMask.cpp): centred amp exp(-i ph)."""
    amp: np.ndarray
    ph: np.ndarray
    disableForCalibration: bool = False


@dataclass
class FpmPupToLyotMask:
    """fpmPupToLyot with a fixed mask (fpmCMCForPupToLyot, fpmBinaryForPupToLyot):
    complex mask cube [n_mask][rows][cols] (or 2-D) of pixel pixelScale
    (metres), of which slice maskIndex (-1: the first) is applied at every
    wavelength as the reference does; lambdaFocalLength per wavelength (with
    fRatioSign), doBabinet; calibMask [rows][cols] (None: ones) is what the
    calibration walk applies when disabled for it."""
    mask: np.ndarray
    pixelScale: float
    lambdaFocalLength: np.ndarray
    fRatioSign: float = -1.0
    zoomFftSign: float = -1.0
    doBabinet: bool = True
    calibMask: np.ndarray | None = None
    disableForCalibration: bool = True
    maskIndex: int = -1


@dataclass
class ZoomFftPropagator:
    """zoomFftPropagator (zoomFftPropagator.cpp:23-91): a zoom FFT of the
    field to a padFactor N grid of pixel dxprime = 2 (beamRadius / (pixelScale
    N zoomFactor)) lambda0 80 at lambda f = 3.52 lambda0 (dir +1), or back to
    N / padFactor pixels of pixelScale at -3.52 lambda0 (dir -1); lambda0 is
    the first wavelength, used for every wavelength as the reference does.
    The field changes size, so it runs on its own (``propagate``), not inside
    a Coronagraph walk: one csg_mft plan per geometry."""
    zoomFactor: float
    padFactor: float = 2.0
    dir: int = 1

    def geometry(self, ef: EField, n_rows: int, n_cols: int):
        """(output y, output x, pixel, lambda f)."""
        lam0 = float(np.asarray(ef.wavelengths)[0])
        if self.dir == 1:
            d = 2 * (ef.beamRadiusPhysical / (ef.pixelScale * n_rows * self.zoomFactor)) * lam0 * 80
            nr, nc, lf = int(self.padFactor * n_rows), int(self.padFactor * n_cols), lam0 * 3.52
        else:
            d = ef.pixelScale
            nr, nc = int(n_rows / self.padFactor), int(n_cols / self.padFactor)
            lf = -lam0 * 3.52
        return (np.arange(nr) - nr / 2.0) * d, (np.arange(nc) - nc / 2.0) * d, d, lf

    def propagate(self, ctx: Context, field, ef: EField, yin, xin, dxin: float,
                  precision: int = CSG_PREC_BF16X6):
        """field [F][2][rows][cols] on the grid (yin, xin) of pixel dxin ->
        (output field, (yout, xout, pixel))."""
        from .runtime import Mft
        n_rows, n_cols = field.shape[-2:]
        yout, xout, d, lf = self.geometry(ef, n_rows, n_cols)
        plan = Mft(ctx, yin, xin, yout, xout, [lf], dxin * dxin / (1j * lf), -1.0, precision)
        out = plan(field, dvec([0] * field.shape[0], torch.int32))
        ctx.sync()
        plan.close()
        return out, (yout, xout, d)


@dataclass
class DoubleFraunhoferFPM:
    """doubleFraunhoferFPM: zoom FFT to a padFactor N grid whose pixel is
    2 (beamRadius / (pixelScale N zoomFactor)) lambda 80 for each wavelength,
    the fixed complex mask on its centred block, zoom FFT back (lambda f =
    +-3.52 lambda). mask: [rows][cols] or the reference's cube
    [n_slices][rows][cols], of which slice maskIndex (-1: the first) is used
    (doubleFraunhoferFPM.cpp:86-95)."""
    mask: np.ndarray
    zoomFactor: float
    padFactor: float = 2.0
    disableForCalibration: bool = True
    lambdaFocalFactor: float = 3.52  # doubleFraunhoferFPM.cpp:44-45
    maskIndex: int = -1


@dataclass
class DoubleFraunhoferInterpFPM:
    """doubleFraunhoferInterpFPM with its complexHexMaskFPM: zoom FFT of the
    field to a padFactor N grid of pixel fpmScale (metres) at lambda f =
    3.52 lambda, the hex mask (tables [3][S][S], candidate sags, phaseSign)
    on the centred S x S block, zoom FFT back at -3.52 lambda."""
    hex_id: np.ndarray
    count: np.ndarray
    n_sub: int
    n_hex: int
    fpmScale: float
    padFactor: float = 2.0
    phaseSign: float = 1.0
    disableForCalibration: bool = True
    lambdaFocalFactor: float = 3.52  # doubleFraunhoferInterpFPM.cpp:99


@dataclass
class FpmPupToLyotHex:
    """fpmPupToLyot + fpmIntHexCMCForPupToLyot + complexHexMaskFPM: hex tables
    [3][S][S] (ids, counts), nSubPix, hex count, mask pixel scale (metres),
    focalRatio, fRatioSign, zoomFftSign, phaseSign."""
    hex_id: np.ndarray
    count: np.ndarray
    n_sub: int
    n_hex: int
    pixelScale: float
    focalRatio: float
    fRatioSign: float = -1.0
    zoomFftSign: float = -1.0
    phaseSign: float = 1.0
    disableForCalibration: bool = True


@dataclass
class PaddedFftFpm:
    """Plain Lyot occulter: embed the N x N field in a zeroed pad x pad grid,
    FFT, multiply by the focal-plane mask (centred focal coordinates, one
    [pad][pad] array per wavelength or one for all), inverse FFT, crop
    (the fpmPupToLyot embedding pattern with an FFT-sampled mask, no Babinet)."""
    pad: int
    mask: np.ndarray
    disableForCalibration: bool = True


@dataclass
class DeformableMirror:
    """deformableMirror (deformableMirror.cpp): actuator strokes [nA][nA]
    (metres), Gaussian influence width sigma (actuator pitches); the surface
    is computed on the GPU (csg_dm_surface) and applied like a mirror."""
    actuators: np.ndarray
    sigma: float = 1.0
    mirrorSign: float = 1.0


@dataclass
class FraunhoferFocalRagged:
    """fraunhoferFocal with a per-wavelength image size at one pixel scale
    (loD(referenceLambda) / samplesPerflD): a ragged batch in one launch."""
    referenceLambda: float
    samplesPerflD: float
    n_out: list


@dataclass
class FraunhoferFocal:
    """fraunhoferFocal (fraunhoferFocal.cpp:65-72): ceil(FOV spl)^2 pixels at
    loD(referenceLambda) / spl."""
    referenceLambda: float
    samplesPerflD: float
    FOVflD: float

    def n_out(self) -> int:
        return math.ceil(self.FOVflD * self.samplesPerflD)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Coronagraph:
    """Batched coronagraph (coronagraph.cpp). ``set_batch`` chooses the fields;
    ``execute`` runs every element once over the batch and returns the final
    image fields as a planar fp32 tensor [F, 2, n_out, n_out]."""

    def __init__(self, ctx: Context, tel: Telescope, ef: EField, elements: list,
                 precision: int = CSG_PREC_BF16X6, support_crop: bool = True,
                 fft_fpm_babinet: bool = True, reference_calibration: bool = False):
        self.ctx, self.tel, self.ef, self.elements = ctx, tel, ef, elements
        lam = np.ascontiguousarray(ef.wavelengths, dtype=np.float64)
        h = C.c_void_p()
        call("csg_chain_create", ctx.h, C.byref(h), ef.n, ef.pixelScale, lam.size,
             lam.ctypes.data_as(C.c_void_p), precision)
        self.h = h
        call("csg_chain_set_support_crop", self.h, int(support_crop))
        call("csg_chain_set_fft_fpm_babinet", self.h, int(fft_fpm_babinet))
        # fixed-mask FPMs without Babinet: calibrate only the first wavelength,
        # as the reference's compute-once calibration transform does
        call("csg_chain_set_reference_calibration", self.h, int(reference_calibration))
        self.n_hex = None
        self.n_out = None
        self.out_pixel = None
        for e in elements:
            self._add(e)

    def _add(self, e):
        if isinstance(e, Mask):
            m = _f32(e.mask)
            call("csg_chain_add_mask", self.h, m.ctypes.data_as(C.c_void_p), int(e.ref_quirk),
                 int(e.disableForCalibration))
        elif isinstance(e, Mirror):
            s = _f32(e.sag)
            call("csg_chain_add_mirror", self.h, s.ctypes.data_as(C.c_void_p), e.mirrorSign)
        elif isinstance(e, FresnelPropagator):
            if e.padFactor == 1:
                call("csg_chain_add_fresnel", self.h, e.z, self.ef.arrayRadiusPhysical)
            else:
                call("csg_chain_add_fresnel_padded", self.h, e.z, self.ef.arrayRadiusPhysical,
                     float(e.padFactor))
        elif isinstance(e, ComplexMask):
            a, p = _f32(e.amp), _f32(e.ph)
            call("csg_chain_add_complex_mask", self.h, a.ctypes.data_as(C.c_void_p),
                 p.ctypes.data_as(C.c_void_p), a.shape[0], a.shape[1],
                 int(e.disableForCalibration))
        elif isinstance(e, FpmPupToLyotHex):
            ids = np.ascontiguousarray(e.hex_id, np.int16)
            cnt = np.ascontiguousarray(e.count, np.uint16)
            call("csg_chain_add_fpm_hex", self.h, ids.ctypes.data_as(C.c_void_p),
                 cnt.ctypes.data_as(C.c_void_p), ids.shape[-1], e.n_sub, e.n_hex, e.pixelScale,
                 e.focalRatio, self.ef.beamRadiusPhysical, e.fRatioSign, e.zoomFftSign,
                 e.phaseSign, int(e.disableForCalibration))
            self.n_hex = e.n_hex
        elif isinstance(e, FpmPupToLyotMask):
            m = np.asarray(e.mask)
            m = m[None] if m.ndim == 2 else m
            re, im = _f32(m.real), _f32(m.imag)
            lf = np.ascontiguousarray(e.lambdaFocalLength, np.float64)
            cre = cim = None
            if e.calibMask is not None:
                cm = np.asarray(e.calibMask)
                if cm.shape != m.shape[1:]:
                    raise ValueError("calibMask must be [rows][cols] of the mask")
                cre, cim = _f32(cm.real), _f32(cm.imag)
            ptr = lambda a: a.ctypes.data_as(C.c_void_p) if a is not None else None  # noqa: E731
            call("csg_chain_add_fpm_mask", self.h, ptr(re), ptr(im), m.shape[0], int(e.maskIndex),
                 m.shape[1], m.shape[2], e.pixelScale, ptr(lf), e.fRatioSign, e.zoomFftSign,
                 int(e.doBabinet), ptr(cre), ptr(cim), int(e.disableForCalibration))
        elif isinstance(e, DoubleFraunhoferFPM):
            m = np.asarray(e.mask)
            if m.ndim == 3:
                m = m[max(int(e.maskIndex), 0)]
            if m.ndim != 2:
                raise ValueError("doubleFraunhoferFPM mask must be [rows][cols] or a cube")
            re, im = _f32(m.real), _f32(m.imag)
            ef = self.ef
            zpx = np.ascontiguousarray(
                [2 * (ef.beamRadiusPhysical / (ef.pixelScale * ef.n * e.zoomFactor)) * lam * 80
                 for lam in ef.wavelengths], np.float64)
            call("csg_chain_add_fpm_double_mask", self.h, re.ctypes.data_as(C.c_void_p),
                 im.ctypes.data_as(C.c_void_p), m.shape[0], m.shape[1],
                 zpx.ctypes.data_as(C.c_void_p), e.padFactor, e.lambdaFocalFactor,
                 int(e.disableForCalibration))
        elif isinstance(e, DoubleFraunhoferInterpFPM):
            ids = np.ascontiguousarray(e.hex_id, np.int16)
            cnt = np.ascontiguousarray(e.count, np.uint16)
            call("csg_chain_add_fpm_hex_double", self.h, ids.ctypes.data_as(C.c_void_p),
                 cnt.ctypes.data_as(C.c_void_p), ids.shape[-1], e.n_sub, e.n_hex, e.fpmScale,
                 e.padFactor, e.lambdaFocalFactor, e.phaseSign, int(e.disableForCalibration))
            self.n_hex = e.n_hex
        elif isinstance(e, PaddedFftFpm):
            L = len(self.ef.wavelengths)
            m = np.asarray(e.mask)
            if m.ndim == 2:
                m = np.broadcast_to(m, (L,) + m.shape)
            assert m.shape == (L, e.pad, e.pad), "mask must be [n_lambda][pad][pad]"
            re = _f32(m.real)
            im = _f32(m.imag) if np.iscomplexobj(m) else None
            call("csg_chain_add_fft_fpm", self.h, e.pad, re.ctypes.data_as(C.c_void_p),
                 im.ctypes.data_as(C.c_void_p) if im is not None else None,
                 int(e.disableForCalibration))
        elif isinstance(e, DeformableMirror):
            surf = dm_surface(self.ctx, np.asarray(e.actuators, np.float64), self.ef.n, e.sigma)
            self.dm_surface = surf
            s = _f32(surf)
            call("csg_chain_add_mirror", self.h, s.ctypes.data_as(C.c_void_p), e.mirrorSign)
        elif isinstance(e, FraunhoferFocalRagged):
            sizes = np.ascontiguousarray(e.n_out, np.int32)
            assert sizes.size == len(self.ef.wavelengths)
            self.n_out = int(sizes.max())
            self.n_out_l = sizes
            self.out_pixel = self.tel.compute_loD(e.referenceLambda) / e.samplesPerflD
            call("csg_chain_add_fraunhofer_ragged", self.h, sizes.ctypes.data_as(C.c_void_p),
                 self.out_pixel, 2 * self.ef.beamRadiusPhysical * self.tel.primaryfRatio)
        elif isinstance(e, FraunhoferFocal):
            self.n_out = e.n_out()
            self.out_pixel = self.tel.compute_loD(e.referenceLambda) / e.samplesPerflD
            call("csg_chain_add_fraunhofer", self.h, self.n_out, self.out_pixel,
                 2 * self.ef.beamRadiusPhysical * self.tel.primaryfRatio)
        else:
            raise TypeError(f"unsupported element {type(e).__name__}")

    def fpm_region(self, idx: int = 0):
        """(r0, c0, rows, cols) of the mask grid the idx-th hex FPM transforms."""
        v = [C.c_int() for _ in range(4)]
        call("csg_chain_fpm_region", self.h, idx, *[C.byref(x) for x in v])
        return tuple(x.value for x in v)

    def set_batch(self, lambda_idx, amp, tip, tilt, cand):
        arrs = [np.ascontiguousarray(lambda_idx, np.int32), np.ascontiguousarray(amp, np.float64),
                np.ascontiguousarray(tip, np.float64), np.ascontiguousarray(tilt, np.float64),
                np.ascontiguousarray(cand, np.int32)]
        self.n_fields = arrs[0].size
        self._batch = arrs
        call("csg_chain_set_batch", self.h, self.n_fields,
             *[a.ctypes.data_as(C.c_void_p) for a in arrs])

    def batch_all(self, n_cand: int = 1):
        """Every (candidate, source, wavelength) combination, candidate-major."""
        L = len(self.ef.wavelengths)
        li, amp, tip, tilt, cand = [], [], [], [], []
        for c in range(n_cand):
            for s in self.ef.sources:
                for l in range(L):
                    li.append(l)
                    amp.append(math.sqrt(s.flux))
                    tip.append(s.tip * self.tel.magnification)
                    tilt.append(s.tilt * self.tel.magnification)
                    cand.append(c)
        self.set_batch(li, amp, tip, tilt, cand)
        return len(li)

    def source_buffers(self):
        """Device FP64 views [n_fields] of the batch's amplitude, tip and tilt
        (written in place between executions)."""
        a, t, u = C.c_void_p(), C.c_void_p(), C.c_void_p()
        call("csg_chain_batch_buffers", self.h, C.byref(a), C.byref(t), C.byref(u))
        return tuple(_tensor_from_ptr(p.value, (self.n_fields,), torch.float64) for p in (a, t, u))

    def sags(self, n_cand: int) -> torch.Tensor:
        """The device sag buffer [n_cand, n_hex] (a torch view, written in place)."""
        p = C.c_void_p()
        call("csg_chain_sags", self.h, n_cand, self.n_hex, C.byref(p))
        self._sag_ptr = p.value
        return _tensor_from_ptr(p.value, (n_cand, self.n_hex), torch.float64)

    def response(self, pix_idx, fpm_index: int = 0):
        """makeHexCFpmResponse: (M [n_base][n_pix][n_hex + 1] complex128,
        calibration max) for the current batch's (wavelength, source) fields."""
        pix = np.ascontiguousarray(pix_idx, np.int32)
        m = np.zeros((self.n_fields, pix.size, self.n_hex + 1), np.complex128)
        cmax = C.c_double()
        call("csg_chain_response", self.h, fpm_index, pix.ctypes.data_as(C.c_void_p), pix.size,
             m.ctypes.data_as(C.c_void_p), C.byref(cmax))
        return m, cmax.value

    def execute(self, calibrating: bool = False, use_graph: bool = False) -> torch.Tensor:
        call("csg_chain_execute", self.h, int(calibrating), int(use_graph))
        p = C.c_void_p()
        n = C.c_int()
        call("csg_chain_image", self.h, C.byref(p), C.byref(n))
        return _tensor_from_ptr(p.value, (self.n_fields, 2, n.value, n.value), torch.float32)

    def image_lo(self):
        """CSG_PREC_HIGH chains: the low-order words of the last image (the
        image is execute() + image_lo()); None at other precisions."""
        p = C.c_void_p()
        n = C.c_int()
        call("csg_chain_image", self.h, C.byref(C.c_void_p()), C.byref(n))
        call("csg_chain_image_lo", self.h, C.byref(p))
        if not p.value:
            return None
        return _tensor_from_ptr(p.value, (self.n_fields, 2, n.value, n.value), torch.float32)

    def close(self):
        if self.h:
            call("csg_chain_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dm_surface(ctx: Context, act: np.ndarray, n: int, sigma: float) -> np.ndarray:
    """deformableMirror surface [n][n] (metres) from strokes [nA][nA] on the GPU."""
    h = C.c_void_p()
    call("csg_dm_create", ctx.h, C.byref(h), n, act.shape[0], sigma)
    try:
        a = torch.as_tensor(np.ascontiguousarray(act, np.float64), device="cuda")
        out = torch.empty((n, n), dtype=torch.float32, device="cuda")
        call("csg_dm_surface", h, ptr(a), ptr(out))
        ctx.sync()
        return out.cpu().numpy()
    finally:
        call("csg_dm_destroy", h)


def _tensor_from_ptr(addr: int, shape, dtype) -> torch.Tensor:
    """Zero-copy torch view of library-owned device memory (valid while the
    owning object lives)."""
    n = int(np.prod(shape))
    elem = torch.tensor([], dtype=dtype).element_size()

    class _Holder:
        __cuda_array_interface__ = {
            "shape": tuple(shape), "typestr": {torch.float32: "<f4", torch.float64: "<f8"}[dtype],
            "data": (addr, False), "version": 3, "strides": None,
        }
    del n, elem
    return torch.as_tensor(_Holder(), device="cuda")


class RegionContrast:
    """regionContrast (regionContrast.cpp:89-205): region pixels of the output
    geometry, mean (or max) of sum_{s,lambda} |E|^2 over the region divided by
    the calibration maximum."""

    def __init__(self, ctx: Context, n_out: int, out_pixel: float, loD: float, radius1: float,
                 radius2: float, angle1: float = -180.0, angle2: float = 180.0,
                 xlim1: float = -1e300, xlim2: float = 1e300):
        x = -(out_pixel * n_out - out_pixel) / 2.0 + np.arange(n_out) * out_pixel
        xx = np.broadcast_to(x[None, :], (n_out, n_out))
        yy = np.broadcast_to(x[:, None], (n_out, n_out))
        rr = np.sqrt(xx ** 2 + yy ** 2)
        tt = np.arctan2(yy, xx)
        sel = ((xx / loD >= xlim1) & (xx / loD <= xlim2) & (rr / loD >= radius1)
               & (rr / loD <= radius2) & (tt > angle1 * math.pi / 180) & (tt < angle2 * math.pi / 180))
        self.mask = sel
        self.pix = dvec(np.flatnonzero(sel.ravel()).astype(np.int32), torch.int32)
        self.ctx = ctx

    def calibration_max(self, image: torch.Tensor) -> float:
        _, mx = self.ctx.intensity(image)
        self.ctx.sync()
        return float(mx.item())

    def contrast(self, image: torch.Tensor, per_group: int, calib_max: float, mode: int = 0):
        return self.ctx.region_reduce(image, per_group, self.pix, mode=mode, scale=1.0 / calib_max)


def linspace_reference(start: float, end: float, n: int) -> np.ndarray:
    """arma::linspace: start + i (end - start) / (n - 1), the last value end."""
    if n < 2:
        return np.array([end], dtype=np.float64)[:n]
    d = (end - start) / (n - 1)
    out = start + np.arange(n, dtype=np.float64) * d
    out[-1] = end
    return out


class ContrastCurve:
    """contrastCurve (contrastCurve.cpp:68-158): the radial profile of the
    image intensity (summed over the batch's fields) normalised by the
    calibration maximum, averaged over overlapping annuli on the GPU. Sample
    points linspace(0, max(pixelX / loD), (n - 2) / pixelSampling); the
    reference writes bins 1 .. end as "%f %e" lines (`lines`)."""

    def __init__(self, ctx: Context, n_out: int, out_pixel: float, loD: float,
                 pixel_sampling: int = 1):
        self.ctx, self.n, self.pixel, self.loD = ctx, n_out, out_pixel, loD
        x_max = (-(out_pixel * n_out - out_pixel) / 2.0 + (n_out - 1) * out_pixel) / loD
        k = int((n_out - 2) / pixel_sampling)
        if k < 3:
            raise ValueError("contrast curve: too few sample points")
        self.samples = linspace_reference(0.0, x_max, k)
        self._s = dvec(self.samples)
        self._work = torch.empty(2 * (k - 2), dtype=torch.float64, device="cuda")
        self._mean = torch.empty(k - 2, dtype=torch.float64, device="cuda")
        self._inten = torch.empty((n_out, n_out), dtype=torch.float64, device="cuda")
        self._max = torch.empty(1, dtype=torch.float64, device="cuda")

    def compute(self, image: torch.Tensor, n_fields: int, calib_max: float):
        """(positions, means) of bins 1 .. K-2 for the image fields [F][2][n][n]."""
        call("csg_intensity", self.ctx.h, ptr(image), self.n, self.n, n_fields, ptr(self._inten),
             ptr(self._max))
        call("csg_contrast_curve", self.ctx.h, ptr(self._inten), self.n, self.pixel, self.loD,
             1.0 / calib_max, ptr(self._s), self.samples.size, ptr(self._work), ptr(self._mean))
        self.ctx.sync()
        return self.samples[1:-1].copy(), self._mean.cpu().numpy()

    @staticmethod
    def lines(pos: np.ndarray, mean: np.ndarray) -> str:
        """The reference's output file body (contrastCurve.cpp:148-151)."""
        return "".join(f"{p:f} {m:e}\n" for p, m in zip(pos[1:], mean[1:]))
