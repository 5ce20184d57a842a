"""Transform sizes that are not powers of two. The reference plans FFTW for
any array size (csim_fft.cpp:111-115; its own spc_input.txt uses
arraySizePixels 1000); here such sizes run the 2-D DFT as an exact-phase
matrix product on the tensor cores. Against numpy's FFT and the FP64
oracle's Fresnel and chain."""
import numpy as np
import pytest
import torch

from oracle import csim_fft as of
from oracle import elements as oe

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,precision", [(200, 6), (1000, 6), (1000, 16)])
def test_fft2d_any_multiple_of_8(ctx, n, precision):
    from csim_gb300 import runtime as R
    rng = np.random.default_rng(n)
    x = rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))
    t = R.to_planar(x)
    ctx.fft2d(t, -1, precision=precision)
    ctx.sync()
    got = R.from_planar(t)
    ref = np.fft.fft2(x)
    e_f = np.abs(got - ref).max() / np.abs(ref).max()
    ctx.fft2d(t, +1, precision=precision)
    ctx.sync()
    back = R.from_planar(t)
    e_b = np.abs(back - x).max() / np.abs(x).max()
    print(f"\nDFT {n}^2 precision {precision}: forward {e_f:.3e}, round trip {e_b:.3e}")
    assert e_f < (1e-6 if precision == 6 else 2e-7) and e_b < 2e-6


@pytest.mark.parametrize("precision", [6, 16])
def test_fresnel_size_1000_matches_oracle(ctx, precision):
    from csim_gb300 import runtime as R
    n, dx = 1000, 4e-5
    geom = of.ArrayGeom.set_xy(n, n, dx)
    lam = np.array([6.0e-7, 7.0e-7])
    yy, xx = np.mgrid[:n, :n]
    ap = (np.hypot(xx - n / 2 + 0.5, yy - n / 2 + 0.5) < 0.4 * n).astype(np.float64)
    e = oe.mask_apply(oe.point_source_field(geom, 2, 1.0, 0.05, -0.02), ap)
    t = R.to_planar(e)
    e32 = R.from_planar(t)  # the input as uploaded (fp32), the oracle's input too
    ctx.fresnel(t, R.dvec(lam), dx * n / 2, 0.3, precision=precision)
    ctx.sync()
    got = R.from_planar(t)
    ref = oe.fresnel_element(e32, lam, dx * n / 2, 0.3)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    print(f"\nFresnel 1000^2 precision {precision}: {err:.3e} of the field peak")
    # the DFT product propagates E + IDFT[DFT(E) (H' - 1)] (H' = H without
    # its zero-frequency phase): measured 3.1e-7 / 3.3e-7, set by the
    # three-part split of the transforms in both modes
    assert err < 5e-7, err


def test_chain_at_size_1000_matches_oracle(ctx):
    """A chain at the reference example's 1000 x 1000 array: pupil mask ->
    mirror -> Fresnel -> Lyot mask -> final MFT."""
    from csim_gb300 import coronagraph as cg
    from csim_gb300.synth import EField, PointSource, Telescope, circle_mask
    n, br = 1000, 0.02
    dx = 2 * br / 800
    lam = np.array([6.4e-7, 6.6e-7])
    ef = EField(n, br, dx, lam, [PointSource(1.0, 0.0, 0.0), PointSource(0.5, 0.02, 0.01)])
    tel = Telescope(2.4, 15.0)
    rng = np.random.default_rng(3)
    pupil = circle_mask(n, 400.0)
    lyot = circle_mask(n, 380.0)
    yy, xx = np.mgrid[:n, :n]
    sag = (3e-8 * np.sin(xx / 37.0) * np.cos(yy / 53.0)).astype(np.float32)
    elems = [cg.Mask(pupil), cg.Mirror(sag, 1.0), cg.FresnelPropagator(0.5), cg.Mask(lyot),
             cg.FraunhoferFocal(float(lam.mean()), 4.0, 16.0)]
    cor = cg.Coronagraph(ctx, tel, ef, elems)
    F = cor.batch_all(1)
    img = cor.execute().clone()
    ctx.sync()
    got = img[:, 0].double().cpu().numpy() + 1j * img[:, 1].double().cpu().numpy()
    li, amp, tip, tilt, _ = cor._batch
    geom = of.ArrayGeom.set_xy(n, n, dx)
    n_out = int(np.ceil(16.0 * 4.0))
    gout = of.ArrayGeom.set_xy(n_out, n_out, tel.compute_loD(float(lam.mean())) / 4.0)
    err = peak = 0.0
    for f in range(F):
        lm = float(lam[li[f]])
        e = oe.point_source_field(geom, 1, amp[f] ** 2, tip[f], tilt[f])
        e = oe.mask_apply(e, pupil)
        e = oe.mirror_apply(e, sag.astype(np.float64), [lm], 1.0)
        e = oe.fresnel_element(e, [lm], ef.arrayRadiusPhysical, 0.5)
        e = oe.mask_apply(e, lyot)
        ref = oe.fraunhofer_focal(e, geom, gout, [lm], br, tel.primaryfRatio)[0]
        peak = max(peak, np.abs(ref).max())
        err = max(err, np.abs(got[f] - ref).max())
    print(f"\nchain at 1000^2: field error {err / peak:.3e} of the image peak")
    assert err / peak < 1e-6
    cor.close()
