"""FP64 oracle of the PIAACMC-style element walk (coronagraph.cpp:175-200)
built from the restated elements.

TEST INFRASTRUCTURE ONLY.
"""
from __future__ import annotations

import numpy as np

from . import csim_fft as of
from . import elements as oe


def piaacmc_field(inp: dict, spec, lam: float, amp: float, tip: float, tilt: float,
                  sags: np.ndarray | None, calibrating: bool = False, conv_form: bool = False):
    """One (wavelength, source, candidate) field through mask -> mirror ->
    fresnel -> mirror -> fpmPupToLyot(hex, Babinet) -> mask -> fraunhoferFocal.
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
        f = oe.pup_to_lyot_conv if conv_form else oe.pup_to_lyot_mft
        e = f(e, [lam], geom, mgeom, m1, lfl, fr, zs)
    e = oe.mask_apply(e, inp["lyot"])
    n_out = int(np.ceil(spec.n_out_fov * spec.spl))
    gout = of.ArrayGeom.set_xy(n_out, n_out, inp["lod_image"] / spec.spl)
    return oe.fraunhofer_focal(e, geom, gout, [lam], ef.beamRadiusPhysical, tel.primaryfRatio)[0]
