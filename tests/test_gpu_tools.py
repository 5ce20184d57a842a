"""The callers around the propagation on the GPU: the contrast curve and
the finite-difference Jacobian against the oracle's restatements, and a
reference-format script building the same chain as the direct API.

Bounds: contrast-curve bins to 1e-12 relative (FP64 sums in another order);
Jacobian columns to 2% of their norm (fp32 fields differenced at dx = 1e-7 m
against FP64 ones); the script-built chain bit-identical to the direct one.
"""
import math
import os

import numpy as np
import pytest
import torch

from oracle import chain as oc
from oracle import tools as ot

pytestmark = pytest.mark.gpu


def small_spec(**kw):
    from csim_gb300.workloads import PiaacmcSpec
    base = dict(n=256, beam_px=200, wavelengths=(640e-9, 660e-9), S=128, fpm_sampling=8.0,
                n_rings=3, n_sub=8, design_size=512, n_out_fov=32.0, spl=4.0)
    base.update(kw)
    return PiaacmcSpec(**base)


def test_contrast_curve_matches_oracle(ctx):
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    spec = small_spec()
    cor, inp = W.build_piaacmc(ctx, spec)
    rng = np.random.default_rng(7)
    cor.sags(1).copy_(torch.as_tensor(W.random_sags(rng, 1, inp["hex_x"].size, spec.sag_range)))
    F = cor.batch_all(1)
    cal = cor.execute(calibrating=True).clone()
    full = cor.execute().clone()
    _, mx = ctx.intensity(cal)
    inten, _ = ctx.intensity(full)
    ctx.sync()
    n_out = full.shape[-1]
    lod = inp["lod_image"]
    for sampling in (1, 2):
        cc = cg.ContrastCurve(ctx, n_out, cor.out_pixel, lod, sampling)
        pos, mean = cc.compute(full, F, float(mx.item()))
        px = (-(cor.out_pixel * n_out - cor.out_pixel) / 2.0 + np.arange(n_out) * cor.out_pixel)
        rpos, rmean = ot.contrast_curve(inten.cpu().numpy() / float(mx.item()), px / lod,
                                        px / lod, sampling)
        assert np.array_equal(pos, rpos)
        ok = ~np.isnan(rmean)
        assert np.array_equal(np.isnan(mean), ~ok)
        assert np.allclose(mean[ok], rmean[ok], rtol=1e-12, atol=0)
    cor.close()


def test_fd_jacobian_matches_oracle(ctx):
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import optimize as O
    from csim_gb300 import workloads as W
    spec = small_spec()
    cor, inp = W.build_piaacmc(ctx, spec)
    rng = np.random.default_rng(8)
    n_hex = inp["hex_x"].size
    x0 = W.random_sags(rng, 1, n_hex, spec.sag_range)[0]
    dx = 1e-7
    n_out = int(math.ceil(spec.n_out_fov * spec.spl))
    reg = cg.RegionContrast(ctx, n_out, cor.out_pixel, inp["lod_image"], 2.0, 8.0)
    pix = np.flatnonzero(reg.mask.ravel())
    jac = O.fd_jacobian(cor, x0, dx, pix).cpu().numpy()
    n_base = len(inp["lam"])  # one on-axis source x wavelengths
    assert jac.shape == (2 * n_base * pix.size, n_hex)
    lam = inp["lam"]

    def field(x, b):
        return oc.piaacmc_field(inp, spec, lam[b], 1.0, 0.0, 0.0, x)

    cols = [0, 7, n_hex - 1]
    ref = ot.fd_jacobian(field, x0, dx, cols, pix, n_base)
    for j, c in enumerate(cols):
        err = np.linalg.norm(jac[:, c] - ref[:, j]) / np.linalg.norm(ref[:, j])
        assert err < 2e-2, (c, err)
    cor.close()


SCRIPT = """# small PIAACMC-style chain in the reference's script format
start
  telescope
  primaryDiameter:{D}
  primaryFRatio:{fr}
end
start
  efield
  setSize:{n}, {n}, {nl}
  pointSource:1.0, 0.0, 0.0
  pointSource:0.5, 0.02, -0.01
  wavelengthList:{lams}
  beamRadiusPhysical:{br}
  pixelScale:{dx}
end
start
  coronagraph
  start
    mask
    filename:pupil.fits
    position:0
    name:entrance pupil
  end
  start
    mirror
    filename:sag1.fits
    position:0
    name:PIAA M1
  end
  start
    fresnelPropagator
    propagationSign:1
  end
  start
    mirror
    filename:sag2.fits
    position:{z}
    sign:-1
    name:PIAA M2
  end
  start
    fpmPupToLyot
    name:FPM
    position:{z}
    focalRatio: {ffr}
    fRatioSign: -1
    zoomFftSign: -1
    disableForCalibration:on
    start
      fpmIntHexCMCForPupToLyot
      zoomFactor: 16
      start
        complexHexMaskFPM
        maskNRings: {rings}
        fpmMaskSize: {S}
        hexStep: 1
        fpmArraySize: {A}
        fpmScaleFactor: {sf}
        hexGap: {gap}
        nSubPix: {nsub}
        fpmRadius: {frad}
        pixelScale: {pix}
        sagFilename:sags.fits
      end
    end
  end
  start
    mask
    filename:lyot.fits
    position:{z}
    name:Lyot stop
  end
  start
    fraunhoferFocal
    position:{z}
    referenceLambda:{lref}
    samplesPerflD:{spl}
    FOVflD:{fov}
  end
end
start
  regionContrast
  referenceLambda:{lref}
  radii:2,8
  anglesInDegrees:-90,90
  filename:regionContrast.txt
end
start
  makeContrastCurve
  filename:contrastCurve.txt
end
"""


def test_script_builds_the_direct_chain(ctx, tmp_path):
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import fits
    from csim_gb300 import script as S
    from csim_gb300 import workloads as W
    from csim_gb300.synth import EField
    spec = small_spec()
    a = W.piaacmc_arrays(spec)
    rings = 3
    hx, hy = S.hex_centers_reference(rings)
    rng = np.random.default_rng(9)
    sags = rng.uniform(-spec.sag_range, spec.sag_range, hx.size)
    for name, arr in (("pupil", a["pupil"]), ("sag1", a["sag1"]), ("sag2", a["sag2"]),
                      ("lyot", a["lyot"])):
        fits.write(str(tmp_path / f"{name}.fits"), arr)
    fits.write(str(tmp_path / "sags.fits"), sags)
    txt = SCRIPT.format(D=spec.diameter, fr=spec.f_ratio, n=spec.n, nl=len(a["lam"]),
                        lams=" ".join(repr(float(v)) for v in a["lam"]), br=spec.beam_radius,
                        dx=repr(a["dx"]), z=spec.z, ffr=spec.fpm_focal_ratio, rings=rings,
                        S=spec.S, A=spec.design_size, sf=spec.fpm_scale_factor,
                        gap=spec.hex_gap, nsub=spec.n_sub, frad=repr(a["fpm_radius"]),
                        pix=repr(a["dm"]), lref=repr(a["lam_ref"]), spl=spec.spl,
                        fov=spec.n_out_fov)
    (tmp_path / "chain.txt").write_text(txt)
    sc = S.load(str(tmp_path / "chain.txt"), ctx)
    assert sc.names[:2] == ["entrance pupil", "PIAA M1"]
    assert sc.elements[2].z == spec.z  # sign |next.position - prev.position|
    # the same chain through the direct API
    ids, cnt, over = W.hex_tables(ctx, hx, hy, rings, spec.design_size, spec.fpm_scale_factor,
                                  spec.hex_gap, math.sqrt(3.0), spec.S, spec.n_sub, a["dm"],
                                  a["fpm_radius"])
    ef = EField(spec.n, spec.beam_radius, a["dx"], a["lam"],
                [cg.PointSource(1.0, 0.0, 0.0), cg.PointSource(0.5, 0.02, -0.01)])
    elems = [cg.Mask(a["pupil"]), cg.Mirror(a["sag1"], 1.0), cg.FresnelPropagator(spec.z),
             cg.Mirror(a["sag2"], -1.0),
             cg.FpmPupToLyotHex(ids, cnt, spec.n_sub, hx.size, a["dm"], spec.fpm_focal_ratio),
             cg.Mask(a["lyot"]),
             cg.FraunhoferFocal(a["lam_ref"], spec.spl, spec.n_out_fov)]
    direct = cg.Coronagraph(ctx, a["tel"], ef, elems)
    direct.sags(1).copy_(torch.as_tensor(sags))
    outs = []
    for cor in (sc.coronagraph, direct):
        cor.batch_all(1)
        outs.append((cor.execute().clone(), cor.execute(calibrating=True).clone()))
    ctx.sync()
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])
    # the script's tool blocks, written in the reference's formats
    res = S.run_tools(sc, str(tmp_path))
    lines = (tmp_path / "regionContrast.txt").read_text().splitlines()
    assert lines[0] == "-90.000000, 90.000000" and lines[1] == "2.000000, 8.000000"
    assert float(lines[3]) == pytest.approx(res["regionContrast"][0], rel=1e-6)
    cc = (tmp_path / "contrastCurve.txt").read_text().splitlines()
    pos, mean = res["contrastCurve"][0]
    assert len(cc) == pos.size - 1
    assert float(cc[0].split()[1]) == pytest.approx(mean[1], rel=1e-6)
    sc.coronagraph.close()
    direct.close()
