"""Broadband batch on the GPU against the FP64 oracle: deformable-mirror
surface (deformableMirror.cpp:205-270), ragged per-wavelength MFT plans, and
the segmented-aperture -> DM -> ragged fraunhoferFocal chain.

Bounds: DM surface to fp32 storage (1e-6 of its peak); fields 1e-6 of the
batch's image peak; the padding outside each wavelength's grid is zero.
"""
import numpy as np
import pytest
import torch

from oracle import chain as oc
from oracle import csim_fft as of
from oracle import elements as oe

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,n_act,sigma", [(256, 16, 1.0), (2048, 48, 1.0)])
def test_dm_surface_matches_oracle(ctx, n, n_act, sigma):
    from csim_gb300 import coronagraph as cg
    rng = np.random.default_rng(n_act)
    act = rng.normal(0.0, 5e-9, (n_act, n_act))
    got = cg.dm_surface(ctx, act, n, sigma)
    geom = of.ArrayGeom.set_xy(n, n, 1e-5)
    ref = oe.dm_surface(act, oe.dm_influence(geom, sigma, n_act))
    assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("sizes", [[40, 56, 48], [100, 300, 140]])
def test_ragged_mft_matches_oracle(ctx, sizes):
    """One launch for every wavelength's grid; with grids spanning several
    128-wide tiles the tiles wholly beyond a wavelength's grid are skipped and
    must still come out zero (the output buffer starts as NaN)."""
    from csim_gb300 import _lib
    from csim_gb300.runtime import dvec, from_planar, to_planar
    import ctypes as C
    rng = np.random.default_rng(5)
    n_in = 96
    n_max = max(sizes)
    L = len(sizes)
    gin = of.ArrayGeom.set_xy(n_in, n_in, 1e-5)
    lf = np.array([6e-7, 6.5e-7, 7e-7]) * 40
    pref = np.stack([gin.pixelSizeX ** 2 / (1j * v) for v in lf])
    pref_il = np.stack([pref.real, pref.imag], 1).ravel()
    pix = 2.1e-6
    xo = np.zeros((L, n_max))
    for s, m in enumerate(sizes):
        xo[s, :m] = of.ArrayGeom.set_xy(m, m, pix).pixelX
    h = C.c_void_p()
    sz = np.ascontiguousarray(sizes, np.int32)
    xin = np.ascontiguousarray(gin.pixelX)
    _lib.call("csg_mft_create_ragged", ctx.h, C.byref(h), n_in, n_in, n_max,
              sz.ctypes.data_as(C.c_void_p), xin.ctypes.data_as(C.c_void_p),
              xin.ctypes.data_as(C.c_void_p), xo.ctypes.data_as(C.c_void_p),
              xo.ctypes.data_as(C.c_void_p), L, lf.ctypes.data_as(C.c_void_p),
              pref_il.ctypes.data_as(C.c_void_p), -1.0, 6)
    try:
        F = 6
        slots = np.array([0, 1, 2, 2, 1, 0], np.int32)
        e = rng.standard_normal((F, n_in, n_in)) + 1j * rng.standard_normal((F, n_in, n_in))
        inp = to_planar(e)
        out = torch.full((F, 2, n_max, n_max), float("nan"), dtype=torch.float32, device="cuda")
        sl = dvec(slots, torch.int32)
        _lib.call("csg_mft_execute", ctx.h, h, C.c_void_p(inp.data_ptr()),
                  C.c_void_p(out.data_ptr()), F, C.c_void_p(sl.data_ptr()), 0, None, None)
        ctx.sync()
        got = from_planar(out)
        for f in range(F):
            s = slots[f]
            m = sizes[s]
            go = of.ArrayGeom.set_xy(m, m, pix)
            ref = of.mft(e[f], gin.pixelX, gin.pixelY, go.pixelX, go.pixelY, lf[s], pref[s])
            assert np.abs(got[f, :m, :m] - ref).max() / np.abs(ref).max() < 2e-6
            assert np.abs(got[f, m:, :]).max(initial=0) == 0
            assert np.abs(got[f, :, m:]).max(initial=0) == 0
    finally:
        _lib.call("csg_mft_destroy", h)


def test_broadband_chain_matches_oracle(ctx):
    from csim_gb300 import workloads as W
    spec = W.BroadbandSpec(n=256, radius_px=110.0, n_rings=3, n_lambda=3, n_act=16,
                           n_out_min=56, n_out_max=72, spl=4.0)
    cor, inp = W.build_broadband(ctx, spec)
    F = cor.batch_all(1)
    assert F == 9
    img = cor.execute().clone()
    ctx.sync()
    got = img[:, 0].double().cpu().numpy() + 1j * img[:, 1].double().cpu().numpy()
    li, amp, tip, tilt, _ = cor._batch
    refs = [oc.broadband_field(inp, spec, int(li[f]), amp[f], tip[f], tilt[f],
                               surface=inp["dm_surface"].astype(np.float64)) for f in range(F)]
    peak = max(np.abs(r).max() for r in refs)
    for f in range(F):
        m = inp["n_out"][li[f]]
        assert np.abs(got[f, :m, :m] - refs[f]).max() / peak < 1e-6
        assert np.abs(got[f, m:, :]).max(initial=0) == 0
        assert np.abs(got[f, :, m:]).max(initial=0) == 0
    # the GPU surface is the oracle's within fp32
    geom = of.ArrayGeom.set_xy(spec.n, spec.n, inp["dx"])
    ref_s = oe.dm_surface(inp["act"], oe.dm_influence(geom, spec.dm_sigma, spec.n_act))
    assert np.abs(inp["dm_surface"] - ref_s).max() <= 1e-6 * np.abs(ref_s).max()
    cor.close()
