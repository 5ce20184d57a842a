"""Full-chain parity: the batched PIAACMC-style walk on the GPU against the
FP64 oracle, including the reference's own 2N-convolution fpmPupToLyot.

Errors are peak-normalised to the calibration (FPM-free) image peak, the
normalisation the dark-hole contrast uses (regionContrast.cpp:145-195).
Bounds: field error < 1e-6 of the calibration peak (the fp32-storage floor
of the full-size chain is 0.7e-7; this path measures 3.7e-7 to 5.0e-7, a
plain complex64 evaluation 1.3e-6 to 1.9e-6); contrast (mean normalised
intensity over a 2-8 lambda/D annulus) within 1%.
"""
import math

import numpy as np
import pytest
import torch

from oracle import chain as oc
from oracle import csim_fft as of
from oracle import elements as oe
from oracle import native

pytestmark = pytest.mark.gpu


def small_spec(**kw):
    from csim_gb300.workloads import PiaacmcSpec
    base = dict(n=256, beam_px=200, wavelengths=(640e-9, 660e-9), S=128, fpm_sampling=8.0,
                n_rings=3, n_sub=8, design_size=512, n_out_fov=32.0, spl=4.0)
    base.update(kw)
    return PiaacmcSpec(**base)


def test_hex_tables_match_oracle(ctx):
    from csim_gb300 import workloads as W
    hx, hy = W.hex_layout_standard(4)
    for S, n_sub, A in [(64, 8, 256), (96, 16, 512)]:
        pix = 2e-6
        ids, cnt, over = W.hex_tables(ctx, hx, hy, 4, A, 0.9, 0.01, 1.0, S, n_sub, pix,
                                      S * pix * 0.45)
        d = native.hex_design_array(hx, hy, 4, A, 0.9, 0.01, 1.0)
        rid, rcnt, rover = native.interpolation_tables(d, S, n_sub, pix, S * pix * 0.45, 0.9)
        assert over == rover
        assert np.array_equal(ids, rid)
        assert np.array_equal(cnt, rcnt)


def test_hex_tables_single_thread_quirk_matches_oracle(ctx):
    """The GPU tables with reference_single_thread equal the C oracle's
    restatement of the reference's one-thread loop, bit for bit, on a
    geometry where the quirk changes a row (hexes reaching the array edge)."""
    from csim_gb300 import workloads as W
    hx, hy = W.hex_layout_standard(4)
    A, S, n_sub, pix = 256, 64, 8, 2e-6
    d = native.hex_design_array(hx, hy, 4, A, 1.0, 0.01, 1.0)
    for stale in (False, True):
        ids, cnt, _ = W.hex_tables(ctx, hx, hy, 4, A, 1.0, 0.01, 1.0, S, n_sub, pix,
                                   S * pix * 0.49, reference_single_thread=stale)
        rid, rcnt, _ = native.interpolation_tables(d, S, n_sub, pix, S * pix * 0.49, 1.0,
                                                   stale=stale)
        assert np.array_equal(ids, rid) and np.array_equal(cnt, rcnt), stale


@pytest.mark.parametrize("conv_form", [False, True])
def test_piaacmc_chain_matches_oracle(ctx, conv_form):
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    spec = small_spec()
    sources = [cg.PointSource(1.0, 0.0, 0.0), cg.PointSource(0.5, 0.02, -0.01)]
    cor, inp = W.build_piaacmc(ctx, spec, sources)
    rng = np.random.default_rng(4)
    n_cand = 2
    sags = W.random_sags(rng, n_cand, inp["hex_x"].size, spec.sag_range)
    cor.sags(n_cand).copy_(torch.as_tensor(sags))
    F = cor.batch_all(n_cand)
    img = cor.execute(calibrating=False).clone()
    cal = cor.execute(calibrating=True).clone()
    ctx.sync()
    got = img[:, 0].double().cpu().numpy() + 1j * img[:, 1].double().cpu().numpy()
    gcal = cal[:, 0].double().cpu().numpy() + 1j * cal[:, 1].double().cpu().numpy()
    li, amp, tip, tilt, cand = cor._batch
    lam = inp["lam"]
    peak = 0.0
    refs, rcal = [], []
    for f in range(F):
        if conv_form and f >= 2:
            break
        args = (inp, spec, lam[li[f]], amp[f], tip[f], tilt[f], sags[cand[f]])
        refs.append(oc.piaacmc_field(*args, conv_form=conv_form))
        rcal.append(oc.piaacmc_field(*args, calibrating=True))
        peak = max(peak, np.abs(rcal[-1]).max())
    e_cal = max(np.abs(gcal[f] - rcal[f]).max() for f in range(len(refs))) / peak
    e_img = max(np.abs(got[f] - refs[f]).max() for f in range(len(refs))) / peak
    print(f"\npiaacmc n={spec.n} conv_form={conv_form}: calibration field {e_cal:.3e}, final "
          f"field {e_img:.3e} (of the calibration peak)")
    assert e_cal < 1e-6 and e_img < 1e-6, (e_cal, e_img)
    if conv_form:
        return
    # dark-hole contrast per candidate, 2-8 lambda/D
    n_out = img.shape[-1]
    reg = cg.RegionContrast(ctx, n_out, cor.out_pixel, inp["lod_image"], 2.0, 8.0)
    per = F // n_cand
    ical = (np.abs(gcal[:per]) ** 2).sum(0)
    cmax = ical.max()
    con = reg.contrast(img, per, cmax).cpu().numpy()
    rcmax = (np.abs(np.array(rcal[:per])) ** 2).sum(0).max()
    for c in range(n_cand):
        full = (np.abs(np.array(refs[c * per:(c + 1) * per])) ** 2).sum(0)
        ref_con = oe.region_contrast(full, np.full_like(full, rcmax), reg.mask)
        assert abs(con[c] - ref_con) / ref_con < 0.01, (con[c], ref_con)


@pytest.mark.parametrize("precision", [6, 16])
def test_piaacmc_full_size_field_and_contrast(ctx, precision):
    """The 1024^2 PIAACMC configuration itself (512^2 mask grid, 217 hexes,
    64 x 64 sub-pixel tables, 256^2 image, the mask's support crop), three
    candidates and an on-axis plus an off-axis source, against the FP64
    oracle: final and calibration fields within 1e-6 of the calibration peak
    (measured 3.7e-7 and 5.0e-7; storing the fields and tables in fp32 alone,
    with exact arithmetic, already costs 0.7e-7, and single-precision FFTs
    1.1e-7: tests/test_precision_floor.py), closer to the oracle than
    the same chain evaluated plainly in complex64 (cuFFT, complex64 matmuls:
    1.9e-6), and dark-hole contrast (2-8 lambda/D) within 1%.
    precision 16 (CSG_PREC_HIGH: aligned-split transforms with exact
    tensor sums, two-float Fresnel passes, image + its low-order plane):
    both fields within 1e-7 of the calibration peak."""
    from baseline.fp64_gpu import Fp64Piaacmc
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    spec = W.PiaacmcSpec()
    sources = [cg.PointSource(1.0, 0.0, 0.0), cg.PointSource(0.3, 0.015, -0.01)]
    cor, inp = W.build_piaacmc(ctx, spec, sources, precision=precision)
    n_cand = 3
    sags = W.random_sags(np.random.default_rng(21), n_cand, spec.n_hex, spec.sag_range)
    cor.sags(n_cand).copy_(torch.as_tensor(sags))
    F = cor.batch_all(n_cand)
    high = precision == 16

    def run(calibrating):
        im = cor.execute(calibrating=calibrating).clone()
        full = im.double()
        if high:
            full = full + cor.image_lo().double()
        return im, full[:, 0].cpu().numpy() + 1j * full[:, 1].cpu().numpy()

    img, got = run(False)
    cal, gcal = run(True)
    ctx.sync()
    li, amp, tip, tilt, cand = cor._batch
    lam = inp["lam"]
    refs, rcal = [], []
    for f in range(F):
        args = (inp, spec, lam[li[f]], amp[f], tip[f], tilt[f], sags[cand[f]])
        refs.append(oc.piaacmc_field(*args))
        rcal.append(oc.piaacmc_field(*args, calibrating=True))
    peak = max(np.abs(r).max() for r in rcal)
    e_cal = max(np.abs(gcal[f] - rcal[f]).max() for f in range(F)) / peak
    e_img = max(np.abs(got[f] - refs[f]).max() for f in range(F)) / peak
    reg = cg.RegionContrast(ctx, img.shape[-1], cor.out_pixel, inp["lod_image"], 2.0, 8.0)
    per = F // n_cand
    cmax = (np.abs(gcal[:per]) ** 2).sum(0).max()
    con = reg.contrast(img, per, cmax).cpu().numpy()
    rcmax = (np.abs(np.array(rcal[:per])) ** 2).sum(0).max()
    e_con = 0.0
    for c in range(n_cand):
        full = (np.abs(np.array(refs[c * per:(c + 1) * per])) ** 2).sum(0)
        ref_con = oe.region_contrast(full, np.full_like(full, rcmax), reg.mask)
        e_con = max(e_con, abs(con[c] - ref_con) / ref_con)
    # the plain complex64 path on the on-axis fields (source 0 of each candidate)
    plain = Fp64Piaacmc(inp, spec, dtype=torch.complex64)
    e_plain = e_ours = 0.0
    for c in range(n_cand):
        f = c * per
        g = plain.field(int(li[f]), float(amp[f]), torch.as_tensor(sags[c], device="cuda"))
        g = g.to(torch.complex128).cpu().numpy()
        e_plain = max(e_plain, np.abs(g - refs[f]).max() / peak)
        e_ours = max(e_ours, np.abs(got[f] - refs[f]).max() / peak)
    print(f"\nfull-size piaacmc precision {precision}: calibration field {e_cal:.3e}, final "
          f"field {e_img:.3e} (of the calibration peak; on-axis {e_ours:.3e}, plain complex64 "
          f"path {e_plain:.3e}), contrast {e_con:.3e} relative")
    bound = 1e-7 if high else 1e-6
    assert e_cal < bound and e_img < bound, (e_cal, e_img)
    assert e_ours < e_plain, (e_ours, e_plain)
    assert e_con < 0.01, e_con


def test_fresnel_split_handoff_is_exact(ctx, monkeypatch):
    """The Fresnel's last row pass writing the hex FPM's operand split (the
    default) gives bit-identical images to the separate split pass
    (CSG_FRESNEL_SPLIT=0): the parts come from the same fp32 values."""
    from csim_gb300 import _lib
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    spec = small_spec()
    cor, inp = W.build_piaacmc(ctx, spec, [cg.PointSource(1.0, 0.0, 0.0),
                                           cg.PointSource(0.5, 0.02, -0.01)])
    cor.sags(3).copy_(torch.as_tensor(W.random_sags(np.random.default_rng(8), 3,
                                                    inp["hex_x"].size, 5e-7)))
    cor.batch_all(3)
    cor.execute(use_graph=False)  # plans, buffers and tile tuning first
    outs, launches = [], []
    for flag in ("1", "0"):
        monkeypatch.setenv("CSG_FRESNEL_SPLIT", flag)
        n0 = _lib.api["csg_launch_count"]()
        outs.append(cor.execute(use_graph=False).clone())
        launches.append(_lib.api["csg_launch_count"]() - n0)
    ctx.sync()
    assert launches[1] - launches[0] == 1  # one split pass fewer
    assert torch.equal(outs[0], outs[1])
    cor.close()


def test_fpm_support_crop_is_exact(ctx):
    """Transforming only the support of fliplr(M) - 1 gives the full-grid
    result (to fp32 rounding), and the box really is smaller than the grid."""
    from csim_gb300 import workloads as W
    spec = small_spec(S=256, fpm_sampling=16.0, n_rings=3)
    rng = np.random.default_rng(6)
    outs = []
    for crop in (True, False):
        cor, inp = W.build_piaacmc(ctx, spec, support_crop=crop)
        sags = W.random_sags(rng if not outs else np.random.default_rng(6), 2, inp["hex_x"].size,
                             5e-7)
        cor.sags(2).copy_(torch.as_tensor(sags))
        cor.batch_all(2)
        outs.append(cor.execute().clone())
        region = cor.fpm_region()
        ctx.sync()
        if crop:
            assert region[2] < spec.S and region[3] < spec.S, region
        else:
            assert region == (0, 0, spec.S, spec.S)
        cor.close()
    a, b = outs
    peak = b.abs().max().item()
    assert (a - b).abs().max().item() / peak < 1e-6


def test_chain_graph_replay_is_identical(ctx):
    from csim_gb300 import workloads as W
    spec = small_spec(wavelengths=(650e-9,))
    cor, inp = W.build_piaacmc(ctx, spec)
    rng = np.random.default_rng(5)
    cor.sags(3).copy_(torch.as_tensor(W.random_sags(rng, 3, inp["hex_x"].size, 5e-7)))
    cor.batch_all(3)
    s = torch.cuda.Stream()
    ctx.bind_stream(s)
    try:
        with torch.cuda.stream(s):
            a = cor.execute(use_graph=False).clone()
            b = cor.execute(use_graph=True).clone()
            c = cor.execute(use_graph=True).clone()
        ctx.sync()
    finally:
        ctx.bind_stream(torch.cuda.current_stream())
    assert torch.equal(a, b) and torch.equal(b, c)


def test_double_fraunhofer_hex_fpm_matches_oracle(ctx):
    """doubleFraunhoferInterpFPM (zoom FFT in, hex mask on the centred block
    of a 2N zoom grid, zoom FFT out) in a pupil -> PIAA M1 -> FPM -> Lyot ->
    image chain, two candidates and an off-axis source, against the oracle:
    fields within 1e-6 of the calibration peak."""
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    from oracle import csim_fft as of
    spec = small_spec()
    sources = [cg.PointSource(1.0, 0.0, 0.0), cg.PointSource(0.5, 0.02, -0.01)]
    a = W.piaacmc_arrays(spec, sources)
    ids, cnt, _ = W.hex_tables(ctx, a["hex_x"], a["hex_y"], spec.n_rings, spec.design_size,
                               spec.fpm_scale_factor, spec.hex_gap, 1.0, spec.S, spec.n_sub,
                               a["dm"], a["fpm_radius"])
    n, dx, lam_ref = spec.n, a["dx"], float(a["lam_ref"])
    fpm_scale = 3.52 * lam_ref / (n * dx) / 2.0  # zoom grid at twice the FFT sampling
    n_hex = len(a["hex_x"])
    elems = [cg.Mask(a["pupil"]), cg.Mirror(a["sag1"], 1.0),
             cg.DoubleFraunhoferInterpFPM(ids, cnt, spec.n_sub, n_hex, fpm_scale, 2.0),
             cg.Mask(a["lyot"]), cg.FraunhoferFocal(a["lam_ref"], spec.spl, spec.n_out_fov)]
    cor = cg.Coronagraph(ctx, a["tel"], a["ef"], elems, 6, True)
    n_cand = 2
    sags = W.random_sags(np.random.default_rng(13), n_cand, n_hex, spec.sag_range)
    cor.sags(n_cand).copy_(torch.as_tensor(sags))
    F = cor.batch_all(n_cand)
    img = cor.execute(calibrating=False).clone()
    cal = cor.execute(calibrating=True).clone()
    ctx.sync()
    got = img[:, 0].double().cpu().numpy() + 1j * img[:, 1].double().cpu().numpy()
    gcal = cal[:, 0].double().cpu().numpy() + 1j * cal[:, 1].double().cpu().numpy()
    li, amp, tip, tilt, cand = cor._batch
    ef, tel = a["ef"], a["tel"]
    geom = of.ArrayGeom.set_xy(n, n, dx)
    n_out = int(np.ceil(spec.n_out_fov * spec.spl))
    gout = of.ArrayGeom.set_xy(n_out, n_out, a["lod_image"] / spec.spl)
    peak, errs = 0.0, []
    for f in range(F):
        lam = float(a["lam"][li[f]])
        e = oe.point_source_field(geom, 1, amp[f] * amp[f], tip[f], tilt[f])
        e = oe.mask_apply(e, a["pupil"])
        e = oe.mirror_apply(e, a["sag1"].astype(np.float64), [lam], 1.0)
        e_cal = e
        m = oe.complex_interpolated_mask(ids, cnt, sags[cand[f]], lam, spec.n_sub, 1.0)
        e = oe.double_fraunhofer_interp_fpm(e, [lam], geom, fpm_scale, 2.0, [m])
        out = []
        for x in (e, e_cal):
            x = oe.mask_apply(x, a["lyot"])
            out.append(oe.fraunhofer_focal(x, geom, gout, [lam], ef.beamRadiusPhysical,
                                           tel.primaryfRatio)[0])
        peak = max(peak, np.abs(out[1]).max())
        errs.append((np.abs(got[f] - out[0]).max(), np.abs(gcal[f] - out[1]).max()))
    e_img = max(x[0] for x in errs) / peak
    e_cal = max(x[1] for x in errs) / peak
    print(f"\ndouble Fraunhofer hex FPM: calibration field {e_cal:.3e}, final field {e_img:.3e} "
          f"(of the calibration peak)")
    assert e_cal < 1e-6 and e_img < 1e-6, (e_cal, e_img)
    cor.close()


@pytest.mark.parametrize("babinet", [True, False])
def test_fixed_mask_fpm_matches_reference_algorithm(ctx, babinet):
    """fpmPupToLyot with a fixed mask (the CMC adapter with doBabinet, the
    binary adapter without, with its calibration mask) on a rectangular
    mask grid, against the oracle running the reference's own 2N FFT
    convolution: fields within 1e-6 of the calibration peak."""
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    from oracle import csim_fft as of
    spec = small_spec(wavelengths=(640e-9, 660e-9))
    sources = [cg.PointSource(1.0, 0.0, 0.0), cg.PointSource(0.5, 0.02, -0.01)]
    a = W.piaacmc_arrays(spec, sources)
    rows, cols, dm = 64, 48, a["dm"]
    rng = np.random.default_rng(17)
    yy, xx = np.mgrid[0:rows, 0:cols]
    r = np.hypot(yy - rows / 2 + 0.5, xx - cols / 2 + 0.5)
    if babinet:  # complex mask amp exp(-i ph)
        mask = (0.6 + 0.4 * rng.random((rows, cols))) * np.exp(-1j * rng.uniform(-2, 2, (rows, cols)))
        calib = None
    else:  # binary occulter and its calibration mask
        mask = (r > 8.0).astype(np.complex128)
        calib = np.ones((rows, cols), np.complex128)
    ef, tel = a["ef"], a["tel"]
    lfl = np.array([-1.0 * lam * spec.fpm_focal_ratio * 2 * ef.beamRadiusPhysical
                    for lam in a["lam"]])
    elems = [cg.Mask(a["pupil"]), cg.Mirror(a["sag1"], 1.0),
             cg.FpmPupToLyotMask(mask, dm, lfl, -1.0, -1.0, babinet, calib),
             cg.Mask(a["lyot"]), cg.FraunhoferFocal(a["lam_ref"], spec.spl, spec.n_out_fov)]
    cor = cg.Coronagraph(ctx, tel, ef, elems, 6, True)
    F = cor.batch_all(1)
    img = cor.execute(calibrating=False).clone()
    cal = cor.execute(calibrating=True).clone()
    ctx.sync()
    got = img[:, 0].double().cpu().numpy() + 1j * img[:, 1].double().cpu().numpy()
    gcal = cal[:, 0].double().cpu().numpy() + 1j * cal[:, 1].double().cpu().numpy()
    li, amp, tip, tilt, _ = cor._batch
    n, dx = spec.n, a["dx"]
    geom = of.ArrayGeom.set_xy(n, n, dx)
    mgeom = of.ArrayGeom.set_xy(cols, rows, dm)
    n_out = int(np.ceil(spec.n_out_fov * spec.spl))
    gout = of.ArrayGeom.set_xy(n_out, n_out, a["lod_image"] / spec.spl)
    peak, e_img, e_cal = 0.0, 0.0, 0.0
    for f in range(F):
        lam = float(a["lam"][li[f]])
        e = oe.point_source_field(geom, 1, amp[f] * amp[f], tip[f], tilt[f])
        e = oe.mask_apply(e, a["pupil"])
        e = oe.mirror_apply(e, a["sag1"].astype(np.float64), [lam], 1.0)
        outs = []
        for m in (mask, calib):
            if m is None:
                x = e
            else:
                mm = (m - 1.0) if babinet else m
                x = oe.pup_to_lyot_conv(e, [lam], geom, mgeom, mm[None], lfl[li[f]:li[f] + 1],
                                        -1.0, -1.0, babinet=babinet)
            x = oe.mask_apply(x, a["lyot"])
            outs.append(oe.fraunhofer_focal(x, geom, gout, [lam], ef.beamRadiusPhysical,
                                            tel.primaryfRatio)[0])
        peak = max(peak, np.abs(outs[1]).max())
        e_img = max(e_img, np.abs(got[f] - outs[0]).max())
        e_cal = max(e_cal, np.abs(gcal[f] - outs[1]).max())
    e_img, e_cal = e_img / peak, e_cal / peak
    print(f"\nfixed-mask fpmPupToLyot babinet={babinet}: calibration field {e_cal:.3e}, final "
          f"field {e_img:.3e} (of the calibration peak)")
    assert e_cal < 1e-6 and e_img < 1e-6, (e_cal, e_img)
    cor.close()


def test_double_fraunhofer_fixed_mask_matches_oracle(ctx):
    """doubleFraunhoferFPM: a fixed rectangular complex mask on the centred
    block of a zoom grid whose pixel scales with each wavelength, two
    wavelengths, against the oracle: fields within 1e-6 of the calibration
    peak."""
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    from oracle import csim_fft as of
    spec = small_spec(wavelengths=(620e-9, 680e-9))
    a = W.piaacmc_arrays(spec, [cg.PointSource(1.0, 0.0, 0.0), cg.PointSource(0.5, 0.02, 0.0)])
    ef, tel = a["ef"], a["tel"]
    n, dx = spec.n, a["dx"]
    rows, cols = 64, 48
    rng = np.random.default_rng(19)
    mask = (0.5 + 0.5 * rng.random((rows, cols))) * np.exp(1j * rng.uniform(-2, 2, (rows, cols)))
    # zoom pixel about half the FFT sampling at 650 nm
    zf = 2 * ef.beamRadiusPhysical / (ef.pixelScale * n) * 80 * n * dx / (3.52 * 0.5)
    elems = [cg.Mask(a["pupil"]), cg.Mirror(a["sag1"], 1.0), cg.DoubleFraunhoferFPM(mask, zf, 2.0),
             cg.Mask(a["lyot"]), cg.FraunhoferFocal(a["lam_ref"], spec.spl, spec.n_out_fov)]
    cor = cg.Coronagraph(ctx, tel, ef, elems, 6, True)
    F = cor.batch_all(1)
    img = cor.execute(calibrating=False).clone()
    cal = cor.execute(calibrating=True).clone()
    ctx.sync()
    got = img[:, 0].double().cpu().numpy() + 1j * img[:, 1].double().cpu().numpy()
    gcal = cal[:, 0].double().cpu().numpy() + 1j * cal[:, 1].double().cpu().numpy()
    li, amp, tip, tilt, _ = cor._batch
    geom = of.ArrayGeom.set_xy(n, n, dx)
    n_out = int(np.ceil(spec.n_out_fov * spec.spl))
    gout = of.ArrayGeom.set_xy(n_out, n_out, a["lod_image"] / spec.spl)
    peak, e_img, e_cal = 0.0, 0.0, 0.0
    for f in range(F):
        lam = float(a["lam"][li[f]])
        e = oe.point_source_field(geom, 1, amp[f] * amp[f], tip[f], tilt[f])
        e = oe.mask_apply(e, a["pupil"])
        e = oe.mirror_apply(e, a["sag1"].astype(np.float64), [lam], 1.0)
        outs = []
        for x in (oe.double_fraunhofer_fpm(e, [lam], geom, ef.beamRadiusPhysical, ef.pixelScale,
                                           zf, 2.0, mask), e):
            x = oe.mask_apply(x, a["lyot"])
            outs.append(oe.fraunhofer_focal(x, geom, gout, [lam], ef.beamRadiusPhysical,
                                            tel.primaryfRatio)[0])
        peak = max(peak, np.abs(outs[1]).max())
        e_img = max(e_img, np.abs(got[f] - outs[0]).max())
        e_cal = max(e_cal, np.abs(gcal[f] - outs[1]).max())
    e_img, e_cal = e_img / peak, e_cal / peak
    print(f"\ndoubleFraunhoferFPM fixed mask: calibration field {e_cal:.3e}, final field "
          f"{e_img:.3e} (of the calibration peak)")
    assert e_cal < 1e-6 and e_img < 1e-6, (e_cal, e_img)
    cor.close()


def _fixed_mask_chain(ctx, mask, calib, babinet, mask_index=-1, reference_calibration=False):
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    spec = small_spec(wavelengths=(640e-9, 660e-9))
    a = W.piaacmc_arrays(spec, [cg.PointSource(1.0, 0.0, 0.0)])
    ef, tel = a["ef"], a["tel"]
    lfl = np.array([-1.0 * lam * spec.fpm_focal_ratio * 2 * ef.beamRadiusPhysical
                    for lam in a["lam"]])
    elems = [cg.Mask(a["pupil"]), cg.Mirror(a["sag1"], 1.0),
             cg.FpmPupToLyotMask(mask, a["dm"], lfl, -1.0, -1.0, babinet, calib,
                                 maskIndex=mask_index),
             cg.Mask(a["lyot"]), cg.FraunhoferFocal(a["lam_ref"], spec.spl, spec.n_out_fov)]
    cor = cg.Coronagraph(ctx, tel, ef, elems, 6, True,
                         reference_calibration=reference_calibration)
    cor.batch_all(1)
    img = cor.execute(calibrating=False).clone()
    cal = cor.execute(calibrating=True).clone()
    ctx.sync()
    li = np.asarray(cor._batch[0])
    cor.close()
    return img, cal, li


def test_fixed_mask_fpm_uses_one_mask_slice(ctx):
    """The reference applies one slice of the mask cube, maskIndex (the first
    slice when it is -1), at every wavelength (fpmPupToLyot.cpp:355-360): a
    three-slice cube with maskIndex 2 gives the images of slice 2 alone, and
    maskIndex -1 those of slice 0."""
    rng = np.random.default_rng(23)
    cube = (0.6 + 0.4 * rng.random((3, 32, 24))) * np.exp(-1j * rng.uniform(-2, 2, (3, 32, 24)))
    for idx, sl in ((2, 2), (-1, 0)):
        img_c, cal_c, _ = _fixed_mask_chain(ctx, cube, None, True, mask_index=idx)
        img_s, cal_s, _ = _fixed_mask_chain(ctx, cube[sl], None, True)
        assert torch.equal(img_c, img_s) and torch.equal(cal_c, cal_s), idx


def test_reference_calibration_first_wavelength_only(ctx):
    """Binary mask (no Babinet) with its calibration mask at two wavelengths:
    by default every wavelength's calibration field is its own transform;
    with reference_calibration, as the reference's compute-once calibration
    transform leaves it (fpmPupToLyot.cpp:56, 86-92), the first wavelength's
    field is unchanged and the second's is zero."""
    yy, xx = np.mgrid[0:32, 0:32]
    mask = (np.hypot(yy - 15.5, xx - 15.5) > 6.0).astype(np.complex128)
    calib = np.ones((32, 32), np.complex128)
    img0, cal0, li = _fixed_mask_chain(ctx, mask, calib, False)
    img1, cal1, _ = _fixed_mask_chain(ctx, mask, calib, False, reference_calibration=True)
    first, second = li == 0, li == 1
    assert torch.equal(img0, img1)
    assert torch.equal(cal1[first], cal0[first])
    assert cal0[second].abs().max().item() > 0
    assert cal1[second].abs().max().item() == 0.0


@pytest.mark.parametrize("precision", [6, 16])
def test_padded_fresnel_matches_oracle(ctx, precision):
    """fresnelPropagator with padFactor 2 (fresnelPropagator.cpp:41-54): the
    field propagated in a 2N zero-padded array with twice the aperture
    radius, cropped; the chain's band-limited padded passes against the FP64
    oracle's explicit pad / propagate / crop."""
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    spec = small_spec(wavelengths=(640e-9, 660e-9), z=0.4)
    a = W.piaacmc_arrays(spec, [cg.PointSource(1.0, 0.0, 0.0), cg.PointSource(0.7, 0.03, 0.0)])
    ef, tel = a["ef"], a["tel"]
    elems = [cg.Mask(a["pupil"]), cg.Mirror(a["sag1"], 1.0), cg.FresnelPropagator(spec.z, 2.0),
             cg.Mirror(a["sag2"], -1.0), cg.Mask(a["lyot"]),
             cg.FraunhoferFocal(a["lam_ref"], spec.spl, spec.n_out_fov)]
    cor = cg.Coronagraph(ctx, tel, ef, elems, precision, True)
    F = cor.batch_all(1)
    im = cor.execute().clone()
    full = im.double() + (cor.image_lo().double() if precision == 16 else 0.0)
    ctx.sync()
    got = full[:, 0].cpu().numpy() + 1j * full[:, 1].cpu().numpy()
    li, amp, tip, tilt, _ = cor._batch
    n, dx = spec.n, a["dx"]
    geom = of.ArrayGeom.set_xy(n, n, dx)
    n_out = int(np.ceil(spec.n_out_fov * spec.spl))
    gout = of.ArrayGeom.set_xy(n_out, n_out, a["lod_image"] / spec.spl)
    err, peak = 0.0, 0.0
    for f in range(F):
        lam = float(a["lam"][li[f]])
        e = oe.point_source_field(geom, 1, amp[f] * amp[f], tip[f], tilt[f])
        e = oe.mask_apply(e, a["pupil"])
        e = oe.mirror_apply(e, a["sag1"].astype(np.float64), [lam], 1.0)
        e = oe.fresnel_element(e, [lam], ef.arrayRadiusPhysical, spec.z, pad=2)
        e = oe.mirror_apply(e, a["sag2"].astype(np.float64), [lam], -1.0)
        e = oe.mask_apply(e, a["lyot"])
        ref = oe.fraunhofer_focal(e, geom, gout, [lam], ef.beamRadiusPhysical,
                                  tel.primaryfRatio)[0]
        peak = max(peak, np.abs(ref).max())
        err = max(err, np.abs(got[f] - ref).max())
    err /= peak
    print(f"\npadded Fresnel (padFactor 2) precision {precision}: field error {err:.3e} of the "
          "image peak")
    assert err < (1e-7 if precision == 16 else 1e-6), err
    cor.close()


def test_zoom_fft_propagator_pair_matches_oracle(ctx):
    """zoomFftPropagator (zoomFftPropagator.cpp:23-91) out to the padded zoom
    grid and back, one wavelength (the element takes the first wavelength's
    lambda f for every slice), against the oracle's restatement."""
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import runtime as R
    from csim_gb300.synth import EField, PointSource, circle_mask
    n, br = 128, 0.01
    dx = 2 * br / 100
    lam = np.array([6.5e-7])
    ef = EField(n, br, dx, lam, [PointSource()])
    geom = of.ArrayGeom.set_xy(n, n, dx)
    e = oe.mask_apply(oe.point_source_field(geom, 1, 1.0, 0.1, 0.0), circle_mask(n, 50.0))
    out_ref, g1 = oe.zoom_fft_propagator(e, geom, br, dx, lam, 4.0, 2.0, 1)
    back_ref, g2 = oe.zoom_fft_propagator(out_ref, g1, br, dx, lam, 4.0, 2.0, -1)
    fwd = cg.ZoomFftPropagator(4.0, 2.0, 1)
    out, (y1, x1, d1) = fwd.propagate(ctx, R.to_planar(e), ef, geom.pixelY, geom.pixelX, dx)
    assert np.allclose(x1, g1.pixelX) and d1 == g1.pixelSizeX
    inv = cg.ZoomFftPropagator(4.0, 2.0, -1)
    back, (y2, x2, d2) = inv.propagate(ctx, out, ef, y1, x1, d1)
    got1, got2 = R.from_planar(out)[0], R.from_planar(back)[0]
    e1 = np.abs(got1 - out_ref[0]).max() / np.abs(out_ref[0]).max()
    e2 = np.abs(got2 - back_ref[0]).max() / np.abs(back_ref[0]).max()
    print(f"\nzoomFftPropagator pair: {e1:.3e}, {e2:.3e}")
    assert got1.shape == (256, 256) and got2.shape == (128, 128)
    assert e1 < 1e-6 and e2 < 1e-6
