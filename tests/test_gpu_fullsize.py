"""The broadband and differential-evolution configurations at their own
sizes against the FP64 oracle.

Broadband: the 2048^2 segmented pupil with the 48^2 deformable mirror,
11 wavelengths x 3 sources = 33 fields in one launch onto ragged 460^2..540^2
images (fraunhoferFocal, fraunhoferFocal.cpp:23-72); one field per
wavelength is checked, normalised to the largest image peak. DE: the
1024^2 PIAACMC chain with the 1261-hex (20-ring) mask at 5 wavelengths over a
10% band (complexHexMaskFPM.cpp:44-99), two candidates, normalised to the
calibration peak. Both in the default mode (field error below 1e-6) and the
high-precision mode (below 1e-7); contrast within 1% for DE.
"""
import numpy as np
import pytest
import torch

from oracle import chain as oc
from oracle import elements as oe

pytestmark = pytest.mark.gpu


def _images(cor, high, calibrating=False):
    im = cor.execute(calibrating=calibrating).clone()
    full = im.double()
    if high:
        full = full + cor.image_lo().double()
    return im, full[:, 0].cpu().numpy() + 1j * full[:, 1].cpu().numpy()


@pytest.mark.parametrize("precision", [6, 16])
def test_broadband_full_size(ctx, precision):
    from csim_gb300 import workloads as W
    spec = W.BroadbandSpec()
    cor, inp = W.build_broadband(ctx, spec, precision=precision)
    F = cor.batch_all(1)
    assert F == 33
    _, got = _images(cor, precision == 16)
    ctx.sync()
    li, amp, tip, tilt, _ = cor._batch
    surface = inp["dm_surface"].astype(np.float64)
    n_src = len(spec.source_offsets_lod)
    # one field per wavelength, cycling through the sources
    fields = [s * spec.n_lambda + l for l, s in zip(range(spec.n_lambda),
                                                     [l % n_src for l in range(spec.n_lambda)])]
    refs = {f: oc.broadband_field(inp, spec, int(li[f]), amp[f], tip[f], tilt[f], surface=surface)
            for f in fields}
    peak = max(np.abs(r).max() for r in refs.values())
    err = 0.0
    for f, r in refs.items():
        m = inp["n_out"][li[f]]
        assert r.shape == (m, m)
        err = max(err, np.abs(got[f, :m, :m] - r).max() / peak)
        assert np.abs(got[f, m:, :]).max(initial=0) == 0
        assert np.abs(got[f, :, m:]).max(initial=0) == 0
    print(f"\nbroadband 2048^2, 33 fields, precision {precision}: field error {err:.3e} "
          f"of the image peak ({len(fields)} fields checked)")
    assert err < (1e-7 if precision == 16 else 1e-6), err
    cor.close()


@pytest.mark.parametrize("precision", [6, 16])
def test_de_configuration_full_size(ctx, precision):
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    lam = tuple(np.linspace(650e-9 * 0.95, 650e-9 * 1.05, 5))
    spec = W.PiaacmcSpec(n_rings=20, wavelengths=lam, sag_range=0.6e-6)
    assert spec.n_hex == 1261
    cor, inp = W.build_piaacmc(ctx, spec, precision=precision)
    n_cand = 2
    sags = W.random_sags(np.random.default_rng(31), n_cand, spec.n_hex, spec.sag_range)
    cor.sags(n_cand).copy_(torch.as_tensor(sags))
    F = cor.batch_all(n_cand)
    assert F == 10
    high = precision == 16
    img, got = _images(cor, high)
    _, gcal = _images(cor, high, calibrating=True)
    ctx.sync()
    li, amp, tip, tilt, cand = cor._batch
    refs, rcal = [], []
    for f in range(F):
        args = (inp, spec, lam[li[f]], amp[f], tip[f], tilt[f], sags[cand[f]])
        refs.append(oc.piaacmc_field(*args))
        if f < len(lam):  # the calibration walk does not depend on the candidate
            rcal.append(oc.piaacmc_field(*args, calibrating=True))
    peak = max(np.abs(r).max() for r in rcal)
    e_img = max(np.abs(got[f] - refs[f]).max() for f in range(F)) / peak
    e_cal = max(np.abs(gcal[f] - rcal[f]).max() for f in range(len(lam))) / peak
    reg = cg.RegionContrast(ctx, img.shape[-1], cor.out_pixel, inp["lod_image"], 2.0, 8.0)
    per = F // n_cand
    cmax = (np.abs(gcal[:per]) ** 2).sum(0).max()
    con = reg.contrast(img, per, cmax).cpu().numpy()
    rcmax = (np.abs(np.array(rcal)) ** 2).sum(0).max()
    e_con = 0.0
    for c in range(n_cand):
        full = (np.abs(np.array(refs[c * per:(c + 1) * per])) ** 2).sum(0)
        ref_con = oe.region_contrast(full, np.full_like(full, rcmax), reg.mask)
        e_con = max(e_con, abs(con[c] - ref_con) / ref_con)
    print(f"\nDE configuration (1261 hexes, 5 lambda, 1024^2) precision {precision}: calibration "
          f"field {e_cal:.3e}, final field {e_img:.3e} (of the calibration peak), contrast "
          f"{e_con:.3e} relative")
    bound = 1e-7 if high else 1e-6
    assert e_cal < bound and e_img < bound, (e_cal, e_img)
    assert e_con < 0.01, e_con
    cor.close()
