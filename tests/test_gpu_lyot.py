"""Plain Lyot coronagraph (512^2 pupil, 2048^2 padded-FFT occulter, Lyot
stop, 128^2 final MFT) on the GPU against the FP64 oracle.

Errors are peak-normalised to the calibration (occulter-free) image peak;
bounds: field error <= 1e-6 of that peak, dark-hole contrast within 1%.
"""
import numpy as np
import pytest
import torch

from oracle import chain as oc
from oracle import elements as oe

pytestmark = pytest.mark.gpu


def _cplx(t):
    return t[:, 0].double().cpu().numpy() + 1j * t[:, 1].double().cpu().numpy()


@pytest.mark.parametrize("full,babinet,precision",
                         [(False, True, 6), (False, False, 6), (True, True, 6), (True, False, 6),
                          (False, False, 16), (True, True, 16), (True, False, 16)])
def test_plain_lyot_matches_oracle(ctx, full, babinet, precision):
    """Both forms of the occulter: the Babinet pair of MFTs over the support
    of 1 - M (the default for a compact occulter) and the padded FFT.
    precision 16 (CSG_PREC_HIGH, image + its low-order plane): fields within
    1e-7 of the calibration peak."""
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    if full:
        spec = W.PlainLyotSpec()  # the 512^2 / 2048^2 / 128^2 configuration
        sources = [cg.PointSource(1.0, 0.0, 0.0)]
    else:
        spec = W.PlainLyotSpec(n=128, pad=512, radius_px=50.0, wavelengths=(530e-9, 570e-9),
                               n_out_fov=16.0)
        sources = [cg.PointSource(1.0, 0.0, 0.0), cg.PointSource(0.5, 0.3, -0.2)]
    cor, inp = W.build_plain_lyot(ctx, spec, sources, precision=precision,
                                  fft_fpm_babinet=babinet)
    F = cor.batch_all(1)
    high = precision == 16

    def run(calibrating):
        t = cor.execute(calibrating=calibrating).clone()
        full = t.double() + (cor.image_lo().double() if high else 0.0)
        return t, full[:, 0].cpu().numpy() + 1j * full[:, 1].cpu().numpy()

    img_t, img = run(False)
    _, cal = run(True)
    ctx.sync()
    li, amp, tip, tilt, _ = cor._batch
    refs, rcal = [], []
    for f in range(F):
        refs.append(oc.plain_lyot_field(inp, spec, int(li[f]), amp[f], tip[f], tilt[f]))
        rcal.append(oc.plain_lyot_field(inp, spec, int(li[f]), amp[f], tip[f], tilt[f],
                                        calibrating=True))
    peak = max(np.abs(r).max() for r in rcal)
    e_cal = max(np.abs(cal[f] - rcal[f]).max() for f in range(F)) / peak
    e_img = max(np.abs(img[f] - refs[f]).max() for f in range(F)) / peak
    # contrast over 3-12 lambda/D (outside the 3 lambda/D occulter)
    n_out = img.shape[-1]
    reg = cg.RegionContrast(ctx, n_out, cor.out_pixel, inp["lod_image"], 3.0,
                            min(12.0, spec.n_out_fov / 2 - 1))
    ical = (np.abs(cal) ** 2).sum(0)
    con = reg.contrast(img_t, F, ical.max()).cpu().numpy()[0]
    rfull = (np.abs(np.array(refs)) ** 2).sum(0)
    rmax = (np.abs(np.array(rcal)) ** 2).sum(0).max()
    ref_con = oe.region_contrast(rfull, np.full_like(rfull, rmax), reg.mask)
    print(f"\nplain Lyot n={spec.n} babinet={babinet} precision {precision}: calibration field "
          f"{e_cal:.3e}, final field {e_img:.3e} (of the calibration peak), contrast "
          f"{abs(con - ref_con) / ref_con:.3e} relative")
    bound = 1e-7 if high else 1e-6
    assert e_cal < bound and e_img < bound, (e_cal, e_img)
    assert abs(con - ref_con) / ref_con < 0.01, (con, ref_con)
    assert ref_con < 1e-2  # the occulter and stop do suppress the star
    cor.close()


def test_padded_fft_fpm_identity_mask(ctx):
    """A mask of ones makes the padded-FFT element the identity (pad, FFT,
    IFFT, crop), to fp32 FFT rounding."""
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    spec = W.PlainLyotSpec(n=128, pad=256, radius_px=50.0, n_out_fov=16.0)
    a = W.plain_lyot_arrays(spec)
    ones = np.ones((spec.pad, spec.pad), np.float32)
    e1 = [cg.Mask(a["pupil"]), cg.Mirror(a["sag"], 1.0), cg.PaddedFftFpm(spec.pad, ones, False),
          cg.FraunhoferFocal(a["lam_ref"], spec.spl, spec.n_out_fov)]
    e0 = [cg.Mask(a["pupil"]), cg.Mirror(a["sag"], 1.0),
          cg.FraunhoferFocal(a["lam_ref"], spec.spl, spec.n_out_fov)]
    outs = []
    for el in (e1, e0):
        cor = cg.Coronagraph(ctx, a["tel"], a["ef"], el)
        cor.batch_all(1)
        outs.append(cor.execute().clone())
        ctx.sync()
        cor.close()
    peak = outs[1].abs().max().item()
    assert (outs[0] - outs[1]).abs().max().item() / peak < 1e-6
