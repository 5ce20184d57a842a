"""makeHexCFpmResponse on the GPU: the response matrix M (one column per hex
plus the Babinet column) must reproduce full propagation for any sags,
E_region(X) = M [exp(i phaseSign 4 pi X / lambda); 1] (optObjective.cpp:
24-69), and the response objective on M must give the propagated contrast.
Also checks the Babinet column against the FP64 oracle directly.
"""
import math

import numpy as np
import pytest
import torch

from oracle import chain as oc
from oracle import elements as oe

pytestmark = pytest.mark.gpu


def small_spec(**kw):
    from csim_gb300.workloads import PiaacmcSpec
    base = dict(n=256, beam_px=200, wavelengths=(640e-9, 660e-9), S=128, fpm_sampling=8.0,
                n_rings=3, n_sub=8, design_size=512, n_out_fov=32.0, spl=4.0)
    base.update(kw)
    return PiaacmcSpec(**base)


def test_response_matrix_reproduces_propagation(ctx):
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import optimize as opt
    from csim_gb300 import workloads as W
    spec = small_spec()
    cor, inp = W.build_piaacmc(ctx, spec)
    n_hex = inp["hex_x"].size
    B = cor.batch_all(1)  # base fields: one per wavelength
    reg = cg.RegionContrast(ctx, cor.n_out, cor.out_pixel, inp["lod_image"], 2.0, 8.0)
    pix = np.flatnonzero(reg.mask.ravel()).astype(np.int32)
    M, cmax = cor.response(pix)
    assert M.shape == (B, pix.size, n_hex + 1)
    # calibration max as the chain computes it
    cal = cor.execute(calibrating=True)
    assert abs(reg.calibration_max(cal) - cmax) / cmax < 1e-6
    # random candidates propagated in full vs the linear response
    rng = np.random.default_rng(12)
    P = 3
    X = W.random_sags(rng, P, n_hex, spec.sag_range)
    cor.sags(P).copy_(torch.as_tensor(X))
    cor.batch_all(P)
    img = cor.execute().clone()
    ctx.sync()
    e = (img[:, 0].double() + 1j * img[:, 1].double()).cpu().numpy().reshape(P, B, -1)[..., pix]
    lam = inp["lam"]
    peak = math.sqrt(cmax)
    for p in range(P):
        for b in range(B):
            ph = np.exp(1j * 4 * math.pi / lam[b] * np.append(X[p], 0.0))
            lin = M[b] @ ph
            assert np.abs(lin - e[p, b]).max() / peak < 2e-6
    # the response objective on M equals the propagated contrast
    obj = opt.RespObjective(ctx, M, lam, cmax)
    got = obj(torch.as_tensor(X, device="cuda")).cpu().numpy()
    con = reg.contrast(img, B, cmax).cpu().numpy()
    assert np.allclose(got, con, rtol=2e-5), (got, con)
    obj.close()
    # the Babinet column (all sags zero, nothing but the outside area) against
    # the FP64 oracle: M[:, :, -1] + sum_h M[:, :, h] = the zero-sag field
    zero = np.zeros(n_hex)
    for b in range(B):
        ref = oc.piaacmc_field(inp, spec, lam[b], 1.0, 0.0, 0.0, zero).ravel()[pix]
        assert np.abs(M[b].sum(1) - ref).max() / peak < 2e-6
    cor.close()
