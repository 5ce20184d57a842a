"""FP64 oracle of the PIAACMC-style element walk (coronagraph.cpp:175-200)
built from the restated elements.

TEST INFRASTRUCTURE ONLY.
"""
from __future__ import annotations

import numpy as np

from . import csim_fft as of
from . import elements as oe


def host_inputs(spec, sources=None) -> dict:
    """The PIAACMC inputs built entirely on the CPU: the seeded arrays plus
    hex tables from the C restatement of the reference's table builder."""
    from csim_gb300.synth import piaacmc_arrays  # seeded input generators (numpy only)
    from . import native
    a = piaacmc_arrays(spec, sources)
    d = native.hex_design_array(a["hex_x"], a["hex_y"], spec.n_rings, spec.design_size,
                                spec.fpm_scale_factor, spec.hex_gap, 1.0)
    ids, cnt, over = native.interpolation_tables(d, spec.S, spec.n_sub, a["dm"], a["fpm_radius"],
                                                 spec.fpm_scale_factor)
    a.update(hex_id=ids, count=cnt, overflow=over)
    return a


def piaacmc_field(inp: dict, spec, lam: float, amp: float, tip: float, tilt: float,
                  sags: np.ndarray | None, calibrating: bool = False, conv_form: bool = False,
                  czt: bool = False):
    """One (wavelength, source, candidate) field through mask -> mirror ->
    fresnel -> mirror -> fpmPupToLyot(hex, Babinet) -> mask -> fraunhoferFocal.
    conv_form runs the reference's fpmPupToLyot algorithm (mask hat + 2N FFT
    convolution); czt evaluates every zoom FFT by the reference's Bluestein
    chirp-Z algorithm instead of the direct matrix product.
    Returns the final image field [n_out][n_out]."""
    ef, tel = inp["ef"], inp["tel"]
    n, dx = ef.n, inp["dx"]
    geom = of.ArrayGeom.set_xy(n, n, dx)
    e = oe.point_source_field(geom, 1, amp * amp, tip, tilt)
    e = oe.mask_apply(e, inp["pupil"])
    e = oe.mirror_apply(e, inp["sag1"].astype(np.float64), [lam], 1.0)
    e = oe.fresnel_element(e, [lam], ef.arrayRadiusPhysical, spec.z)
    e = oe.mirror_apply(e, inp["sag2"].astype(np.float64), [lam], -1.0)
    if not calibrating:
        S = inp["hex_id"].shape[-1]
        mgeom = of.ArrayGeom.set_xy(S, S, inp["dm"])
        m = oe.complex_interpolated_mask(inp["hex_id"], inp["count"], sags, lam, spec.n_sub, 1.0)
        m1 = (np.fliplr(m) - 1.0)[None]
        fr, zs = -1.0, -1.0
        lfl = np.array([fr * lam * spec.fpm_focal_ratio * 2 * ef.beamRadiusPhysical])
        if conv_form:
            e = oe.pup_to_lyot_conv(e, [lam], geom, mgeom, m1, lfl, fr, zs, use_czt=czt)
        else:
            e = oe.pup_to_lyot_mft(e, [lam], geom, mgeom, m1, lfl, fr, zs)
    e = oe.mask_apply(e, inp["lyot"])
    n_out = int(np.ceil(spec.n_out_fov * spec.spl))
    gout = of.ArrayGeom.set_xy(n_out, n_out, inp["lod_image"] / spec.spl)
    return oe.fraunhofer_focal(e, geom, gout, [lam], ef.beamRadiusPhysical, tel.primaryfRatio,
                               use_czt=czt)[0]


def plain_lyot_field(inp: dict, spec, lam_idx: int, amp: float, tip: float, tilt: float,
                     calibrating: bool = False, czt: bool = False):
    """One field of the plain Lyot coronagraph: point source -> pupil mask ->
    aberration (mirror) -> padded-FFT occulter -> Lyot mask ->
    fraunhoferFocal. Returns the final image field [n_out][n_out]."""
    ef, tel = inp["ef"], inp["tel"]
    lam = float(inp["lam"][lam_idx])
    n, dx = ef.n, inp["dx"]
    geom = of.ArrayGeom.set_xy(n, n, dx)
    e = oe.point_source_field(geom, 1, amp * amp, tip, tilt)
    e = oe.mask_apply(e, inp["pupil"])
    e = oe.mirror_apply(e, inp["sag"].astype(np.float64), [lam], 1.0)
    if not calibrating:
        e = oe.padded_fft_fpm(e, spec.pad, inp["occulter"][lam_idx:lam_idx + 1].astype(np.float64))
    e = oe.mask_apply(e, inp["lyot"])
    n_out = int(np.ceil(spec.n_out_fov * spec.spl))
    gout = of.ArrayGeom.set_xy(n_out, n_out, inp["lod_image"] / spec.spl)
    return oe.fraunhofer_focal(e, geom, gout, [lam], ef.beamRadiusPhysical, tel.primaryfRatio,
                               use_czt=czt)[0]


def broadband_field(inp: dict, spec, lam_idx: int, amp: float, tip: float, tilt: float,
                    surface=None):
    """One (wavelength, source) field of the broadband chain: point source ->
    segmented aperture (mask) -> deformable mirror -> fraunhoferFocal onto the
    wavelength's own n_out[l]^2 grid. surface: the DM surface (FP64 oracle
    surface from the strokes when None)."""
    ef, tel = inp["ef"], inp["tel"]
    lam = float(inp["lam"][lam_idx])
    n, dx = ef.n, inp["dx"]
    geom = of.ArrayGeom.set_xy(n, n, dx)
    if surface is None:
        surface = oe.dm_surface(inp["act"], oe.dm_influence(geom, spec.dm_sigma, spec.n_act))
    e = oe.point_source_field(geom, 1, amp * amp, tip, tilt)
    e = oe.mask_apply(e, inp["pupil"])
    e = oe.mirror_apply(e, surface, [lam], 1.0)
    n_out = inp["n_out"][lam_idx]
    gout = of.ArrayGeom.set_xy(n_out, n_out, inp["lod_image"] / spec.spl)
    return oe.fraunhofer_focal(e, geom, gout, [lam], ef.beamRadiusPhysical, tel.primaryfRatio)[0]
