"""GPU parity of the individual C-ABI operations against the FP64 oracle.

Tolerances: the fields run in fp32 with bf16x6-split tensor-core MFTs, so
errors are stated relative to the peak |E| of the oracle result
("peak-normalised"), the metric the path is specified against (<= 1e-7 for
the full chain's final field); per-operation bounds are given per test.
"""
import math

import numpy as np
import pytest
import torch

from oracle import csim_fft as of
from oracle import elements as oe

pytestmark = pytest.mark.gpu


def rt():
    from csim_gb300 import runtime
    return runtime


def peak_err(got, ref):
    return float(np.abs(got - ref).max() / np.abs(ref).max())


def rms_err(got, ref):
    return float(np.linalg.norm(got - ref) / np.linalg.norm(ref))


# Random (white) test fields have no dominant peak, so an fp32-class result
# is bounded by its relative rms error (cuBLAS complex64 gives 3e-7 on the
# same inputs) and a loose peak bound; physical fields get the peak bound.
RMS_TOL = 1e-6
RANDOM_PEAK_TOL = 1e-5


def c64_rms(gin, gout, lf, pref, e, ref):
    """Relative rms error of the same MFT evaluated in complex64 (fp32) on the
    CPU: the conditioning of the product sets what an fp32-class result can
    reach (some random inputs cancel heavily)."""
    a, b = of.mft_matrices(gin.pixelX, gin.pixelY, gout.pixelX, gout.pixelY, lf)
    out = (np.complex64(pref) * a.astype(np.complex64)) @ e.astype(np.complex64) @ b.T.astype(np.complex64)
    return rms_err(out.astype(np.complex128), ref)


def rand_field(rng, f, r, c):
    return rng.standard_normal((f, r, c)) + 1j * rng.standard_normal((f, r, c))


# ---------------------------------------------------------------- MFT
@pytest.mark.parametrize("n_in,n_out", [(256, 128), (512, 256), (256, 384)])
def test_mft_zoomfft_semantics(ctx, n_in, n_out):
    R = rt()
    rng = np.random.default_rng(10)
    lam = np.array([6.5e-7, 7.1e-7])
    gin = of.ArrayGeom.set_xy(n_in, n_in, 1e-5)
    gout = of.ArrayGeom.set_xy(n_out, n_out, 2.1e-6)
    lf = lam * 40.0
    pref = gin.pixelSizeX * gin.pixelSizeY / (1j * lf)
    e = rand_field(rng, 3, n_in, n_in)
    slots = np.array([0, 1, 1], dtype=np.int32)
    plan = R.Mft(ctx, gin.pixelY, gin.pixelX, gout.pixelY, gout.pixelX, lf, pref, -1.0)
    out = plan(R.to_planar(e), R.dvec(slots, torch.int32))
    ctx.sync()
    got = R.from_planar(out)
    for f in range(3):
        z = of.ZoomFft(gin, gout, lf)
        ref = z.mft(e[f], int(slots[f]))
        assert rms_err(got[f], ref) < max(RMS_TOL, 1.5 * c64_rms(gin, gout, lf[slots[f]],
                                                                 pref[slots[f]], e[f], ref))
        assert peak_err(got[f], ref) < RANDOM_PEAK_TOL


def test_mft_bf16x3_and_unaligned_output(ctx):
    """bf16x3 (the three largest split products: ~2^-16 relative) with an
    odd output width, whose rows break the TMA store alignment and take the
    per-thread epilogue; bf16x6 on the same plan shape stays fp32-class."""
    from csim_gb300._lib import CSG_PREC_BF16X3
    R = rt()
    rng = np.random.default_rng(13)
    n_in, n_out = 256, 127
    gin = of.ArrayGeom.set_xy(n_in, n_in, 1e-5)
    gout = of.ArrayGeom.set_xy(n_out, n_out, 2.1e-6)
    lf = np.array([6.5e-7 * 40.0])
    pref = gin.pixelSizeX * gin.pixelSizeY / (1j * lf)
    e = rand_field(rng, 2, n_in, n_in)
    ref = [of.mft(e[f], gin.pixelX, gin.pixelY, gout.pixelX, gout.pixelY, lf[0], pref[0])
           for f in range(2)]
    errs = {}
    for prec in (CSG_PREC_BF16X3, R.CSG_PREC_BF16X6):
        plan = R.Mft(ctx, gin.pixelY, gin.pixelX, gout.pixelY, gout.pixelX, lf, pref, -1.0,
                     precision=prec)
        out = plan(R.to_planar(e), R.dvec([0, 0], torch.int32))
        ctx.sync()
        got = R.from_planar(out)
        plan.close()
        errs[prec] = max(rms_err(got[f], ref[f]) for f in range(2))
    assert errs[R.CSG_PREC_BF16X6] < RMS_TOL
    assert 1e-7 < errs[CSG_PREC_BF16X3] < 1e-4


def test_mft_accumulate_and_input_multiplier(ctx):
    R = rt()
    rng = np.random.default_rng(11)
    n, s = 256, 128
    gin = of.ArrayGeom.set_xy(n, n, 1e-5)
    gm = of.ArrayGeom.set_xy(s, s, 3e-6)
    lf = np.array([3e-5])
    e = rand_field(rng, 2, n, n)
    mul = rand_field(rng, 2, n, n)
    base = rand_field(rng, 2, s, s)
    plan = R.Mft(ctx, gin.pixelY, gin.pixelX, gm.pixelY, gm.pixelX, lf, [0.3 - 0.2j], +1.0)
    out = R.to_planar(base)
    plan(R.to_planar(e), R.dvec([0, 0], torch.int32), out=out, accumulate=True,
         in_mul=R.to_planar(mul), mul_idx=R.dvec([1, 0], torch.int32))
    ctx.sync()
    got = R.from_planar(out)
    for f, mi in [(0, 1), (1, 0)]:
        ref = base[f] + of.mft(e[f] * mul[mi], gin.pixelX, gin.pixelY, gm.pixelX, gm.pixelY,
                               lf[0], 0.3 - 0.2j, sign=+1.0)
        assert rms_err(got[f], ref) < RMS_TOL
        assert peak_err(got[f], ref) < RANDOM_PEAK_TOL


def test_mft_pupil_to_fpm_size(ctx):
    """The PIAACMC focal-plane-mask transform size: 1024^2 -> 512^2."""
    R = rt()
    rng = np.random.default_rng(12)
    n, s = 1024, 512
    gin = of.ArrayGeom.set_xy(n, n, 1e-5)
    gm = of.ArrayGeom.set_xy(s, s, 1.3e-6)
    lf = np.array([6.5e-7 * 3.52])
    yy, xx = np.mgrid[:n, :n]
    pupil = ((xx - n / 2 + .5) ** 2 + (yy - n / 2 + .5) ** 2 < (0.45 * n) ** 2).astype(float)
    e = pupil * np.exp(1j * rng.standard_normal((n, n)) * 0.1)
    plan = R.Mft(ctx, gin.pixelY, gin.pixelX, gm.pixelY, gm.pixelX, lf,
                 gin.pixelSizeX ** 2 / (1j * lf), -1.0)
    out = plan(R.to_planar(e[None]), R.dvec([0], torch.int32))
    ctx.sync()
    got = R.from_planar(out)[0]
    ref = of.mft(e, gin.pixelX, gin.pixelY, gm.pixelX, gm.pixelY, lf[0],
                 gin.pixelSizeX ** 2 / (1j * lf[0]))
    assert peak_err(got, ref) < 3e-6
    assert rms_err(got, ref) < RMS_TOL


# ---------------------------------------------------------------- FFT
@pytest.mark.parametrize("n", [64, 128, 256, 512, 1024, 2048])
def test_fft2d_forward_inverse(ctx, n):
    R = rt()
    rng = np.random.default_rng(n)
    e = rand_field(rng, 2, n, n)
    t = R.to_planar(e)
    ctx.fft2d(t, -1)
    ctx.sync()
    got = R.from_planar(t)
    ref = np.fft.fft2(e)
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert rel < 2e-6, rel
    ctx.fft2d(t, +1)
    ctx.sync()
    back = R.from_planar(t)
    assert np.linalg.norm(back - e) / np.linalg.norm(e) < 4e-6


@pytest.mark.parametrize("n", [256, 1024])
def test_fresnel_matches_oracle(ctx, n):
    R = rt()
    rng = np.random.default_rng(5)
    yy, xx = np.mgrid[:n, :n]
    ap = ((xx - n / 2 + .5) ** 2 + (yy - n / 2 + .5) ** 2 < (0.4 * n) ** 2).astype(float)
    e = ap * np.exp(1j * 0.3 * rng.standard_normal((n, n)))
    lam = np.array([6.5e-7, 6.0e-7])
    ap_rad, z = 0.012, 1.0
    t = R.to_planar(np.stack([e, e]))
    ctx.fresnel(t, R.dvec(lam), ap_rad, z)
    ctx.sync()
    got = R.from_planar(t)
    ref = of.fresnel_propagate_as(np.stack([e, e]), lam, ap_rad, z)
    for k in range(2):
        assert peak_err(got[k], ref[k]) < 3e-6


# ------------------------------------------------------------ elements
def test_point_source_mask_phase(ctx):
    R = rt()
    n = 128
    geom = of.ArrayGeom.set_xy(n, n, 1e-4)
    tips = np.array([0.0, 0.37, -1.25])
    tilts = np.array([0.0, -0.2, 3.5])
    t = torch.empty((3, 2, n, n), dtype=torch.float32, device="cuda")
    ctx.point_source(t, geom.pixelSizeX, geom.pixelSizeY, R.dvec([1.0, 0.5, 2.0]), R.dvec(tips),
                     R.dvec(tilts))
    ctx.sync()
    got = R.from_planar(t)
    for f, (a, tp, tl) in enumerate(zip([1.0, 0.5, 2.0], tips, tilts)):
        ref = oe.point_source_field(geom, 1, a * a, tp, tl)[0]
        assert peak_err(got[f], ref) < 2e-6
    rng = np.random.default_rng(6)
    m = rng.uniform(0, 1, (n, n))
    e = rand_field(rng, 2, n, n)
    t = R.to_planar(e)
    ctx.mask_real(t, R.dvec(m, torch.float32), ref_quirk=True)
    ctx.sync()
    assert peak_err(R.from_planar(t), oe.mask_apply(e, m)) < 1e-6
    sag = rng.uniform(-1e-6, 1e-6, (n, n)).astype(np.float32)
    lam = np.array([6.5e-7, 5.5e-7])
    t = R.to_planar(e)
    ctx.phase_screen(t, R.dvec(sag, torch.float32), R.dvec(lam), 1.0)
    ctx.sync()
    got = R.from_planar(t)
    for k in range(2):
        ref = oe.mirror_apply(e[k:k + 1], sag.astype(np.float64), [lam[k]], 1.0)[0]
        assert peak_err(got[k], ref) < 2e-6


def test_complex_mask(ctx):
    R = rt()
    rng = np.random.default_rng(7)
    e = rand_field(rng, 2, 64, 64)
    amp = rng.uniform(0, 1, (20, 20))
    ph = rng.uniform(-3, 3, (20, 20))
    t = R.to_planar(e)
    ctx.complex_mask(t, R.dvec(amp, torch.float32), R.dvec(ph, torch.float32))
    ctx.sync()
    assert peak_err(R.from_planar(t), oe.complex_mask_apply(e, amp, ph)) < 2e-6


def _random_tables(rng, S, nhex, nsub):
    ids = np.full((3, S, S), -1, np.int16)
    cnt = np.zeros((3, S, S), np.uint16)
    tot = nsub * nsub
    for r in range(S):
        for c in range(S):
            k = rng.integers(0, 4)
            parts = np.sort(rng.integers(0, tot + 1, size=max(k - 1, 0)))
            sizes = np.diff(np.concatenate([[0], parts, [tot]])) if k else np.array([tot])
            for j, sz in enumerate(sizes[:3]):
                cnt[j, r, c] = sz
                ids[j, r, c] = rng.integers(0, nhex) if k else -1
    return ids, cnt


@pytest.mark.parametrize("only", [-1, 5, 40])
def test_hex_mask(ctx, only):
    R = rt()
    rng = np.random.default_rng(8)
    S, nhex, nsub = 48, 40, 8
    ids, cnt = _random_tables(rng, S, nhex, nsub)
    sags = rng.uniform(-5e-7, 5e-7, (3, nhex))
    cand = np.array([2, 0, 1, 2], np.int32)
    lam = np.array([6.5e-7, 6.5e-7, 7e-7, 6e-7])
    out = ctx.hex_mask(R.dvec(ids, torch.int16), R.dvec(cnt.astype(np.int16), torch.int16), nsub,
                       R.dvec(sags), R.dvec(cand, torch.int32), R.dvec(lam), 1.0, True, 1.0,
                       only)
    ctx.sync()
    got = R.from_planar(out)
    for j in range(4):
        m = oe.complex_interpolated_mask(ids, cnt, sags[cand[j]], lam[j], nsub, 1.0, only)
        ref = np.fliplr(m) - 1.0
        assert np.abs(got[j] - ref).max() < 3e-6


def test_intensity_and_region(ctx):
    R = rt()
    rng = np.random.default_rng(9)
    e = rand_field(rng, 6, 32, 32)
    t = R.to_planar(e)
    inten, mx = ctx.intensity(t)
    ctx.sync()
    ref = (np.abs(R.from_planar(t)) ** 2).sum(0)
    assert np.allclose(inten.cpu().numpy(), ref, rtol=1e-12)
    assert abs(mx.item() - ref.max()) < 1e-12 * ref.max()
    pix = np.array([0, 5, 77, 1000, 1023], np.int32)
    for mode in (0, 1):
        out = ctx.region_reduce(t, 3, R.dvec(pix, torch.int32), mode=mode, scale=0.5)
        ctx.sync()
        ee = R.from_planar(t)
        for g in range(2):
            ig = (np.abs(ee[3 * g:3 * g + 3]) ** 2).sum(0).ravel()[pix]
            red = ig.mean() if mode == 0 else ig.max()
            assert abs(out[g].item() - 0.5 * red) < 1e-12 * red


def test_pipelined_readout(ctx):
    """csg_readout_d2h: results copied out through the two staging buffers
    while later work overwrites the source are the values at call time."""
    import ctypes as C
    from csim_gb300._lib import call
    n = 1 << 20
    src = torch.empty(n, dtype=torch.float32, device="cuda")
    hosts = [torch.empty(n, dtype=torch.float32).pin_memory() for _ in range(3)]
    stream = torch.cuda.Stream()
    ctx.bind_stream(stream)
    try:
        with torch.cuda.stream(stream):
            for i, h in enumerate(hosts):
                src.fill_(float(i + 1))
                call("csg_readout_d2h", ctx.h, C.c_void_p(h.data_ptr()),
                     C.c_void_p(src.data_ptr()), n * 4)
            src.fill_(-1.0)  # later work on the source does not reach the host copies
        ctx.sync()
    finally:
        ctx.bind_stream(torch.cuda.current_stream())
    for i, h in enumerate(hosts):
        assert bool((h == float(i + 1)).all())


@pytest.mark.parametrize("bn", [64, 128, 256])
def test_mft_tile_widths(ctx, bn):
    """Every tensor-core tile width (64 and 128 with 64-wide K blocks, 256
    with 32-wide K blocks and 256-wide products) gives the same fp32-class
    transform, for a plain and an accumulating launch."""
    R = rt()
    rng = np.random.default_rng(14)
    n_in, n_out = 256, 320
    gin = of.ArrayGeom.set_xy(n_in, n_in, 1e-5)
    gout = of.ArrayGeom.set_xy(n_out, n_out, 2.1e-6)
    lf = np.array([6.5e-7 * 40.0, 6.9e-7 * 40.0])
    pref = gin.pixelSizeX * gin.pixelSizeY / (1j * lf)
    e = rand_field(rng, 3, n_in, n_in)
    slots = np.array([0, 1, 1], dtype=np.int32)
    plan = R.Mft(ctx, gin.pixelY, gin.pixelX, gout.pixelY, gout.pixelX, lf, pref, -1.0)
    plan.set_tile(bn)
    refs = [of.mft(e[f], gin.pixelX, gin.pixelY, gout.pixelX, gout.pixelY, lf[slots[f]],
                   pref[slots[f]]) for f in range(3)]
    got = R.from_planar(plan(R.to_planar(e), R.dvec(slots, torch.int32)))
    # accumulating onto a base of the result's own magnitude (fp32 sums of
    # very different magnitudes would hide the transform's error)
    scale = float(np.sqrt(np.mean(np.abs(refs[0]) ** 2)))
    base = scale * rand_field(rng, 3, n_out, n_out)
    out = R.to_planar(base)
    plan(R.to_planar(e), R.dvec(slots, torch.int32), out=out, accumulate=True)
    ctx.sync()
    acc = R.from_planar(out)
    for f in range(3):
        assert rms_err(got[f], refs[f]) < RMS_TOL
        assert peak_err(got[f], refs[f]) < RANDOM_PEAK_TOL
        assert rms_err(acc[f], base[f] + refs[f]) < 2 * RMS_TOL
    plan.close()
