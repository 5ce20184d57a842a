"""CPU tests of the oracle against the reference's own fixtures and identities."""
import math
import os

import numpy as np
import pytest

from oracle import csim_fft as of
from oracle import elements as oe

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_response_objective_known_answer():
    """optHexRespObjective(mono M, bestOptVector) reproduces the recorded DE
    best value (optObjective.cpp:24-69; optBestVal.txt last line, %g)."""
    g = np.load(os.path.join(GOLD, "mono_response.npz"))
    for x, rec in zip(g["best_x"], g["best_val"]):
        f = oe.opt_hex_resp_objective([g["M"]], g["wavelengths"], float(g["calib"]), x[:, None])
        assert abs(f[0] - 1.3501189541e-10) / 1.35e-10 < 1e-8
        assert abs(f[0] - rec) / rec < 5e-6  # recorded with 6 significant digits


def test_response_objective_max_and_batch():
    g = np.load(os.path.join(GOLD, "mono_response.npz"))
    rng = np.random.default_rng(3)
    x = np.hstack([g["best_x"][0][:, None], rng.uniform(-5e-8, 5e-8, (499, 3))])
    f = oe.opt_hex_resp_objective([g["M"]], g["wavelengths"], float(g["calib"]), x)
    fm = oe.opt_hex_resp_objective([g["M"]], g["wavelengths"], float(g["calib"]), x, objective="max")
    assert f.shape == (4,) and np.all(fm >= f)
    assert abs(f[0] - 1.3501189541e-10) / 1.35e-10 < 1e-8


def test_bluestein_equals_mft():
    rng = np.random.default_rng(0)
    for n, k in [(64, 48), (50, 64), (128, 37)]:
        e = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        z = of.ZoomFft(of.ArrayGeom.set_xy(n, n, 1e-4), of.ArrayGeom.set_xy(k, k, 3e-6), [2.3e-6])
        a, b = z.execute(e, 0), z.mft(e, 0)
        assert np.abs(a - b).max() / np.abs(b).max() < 1e-12


def test_pup_to_lyot_conv_equals_mft_form():
    rng = np.random.default_rng(1)
    n, s = 32, 24
    e = rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))
    m1 = rng.standard_normal((2, s, s)) + 1j * rng.standard_normal((2, s, s))
    eg, mg = of.ArrayGeom.set_xy(n, n, 1e-4), of.ArrayGeom.set_xy(s, s, 2.3e-6)
    lam = [6.5e-7, 7e-7]
    lfl = -np.array(lam) * 3.0 * 2 * n * 1e-4 / 2
    a = oe.pup_to_lyot_conv(e, lam, eg, mg, m1, lfl, -1.0, 1.0)
    b = oe.pup_to_lyot_mft(e, lam, eg, mg, m1, lfl, -1.0, 1.0)
    assert np.abs(a - b).max() / np.abs(a).max() < 1e-12


def test_hex_counts_match_reference_layouts():
    assert len(oe.hex_centers(20)[0]) == 499      # fixture width - 1
    g = np.load(os.path.join(GOLD, "hex_counts.npz"))
    assert len(oe.hex_centers(32)[0]) == int(g["wfirst_sags_len"])
    assert len(oe.hex_centers_standard(8)[0]) == 217
    assert len(oe.hex_centers_standard(20)[0]) == 1261


def test_fresnel_is_unitary_and_reversible():
    rng = np.random.default_rng(2)
    e = rng.standard_normal((1, 64, 64)) + 1j * rng.standard_normal((1, 64, 64))
    p = of.fresnel_propagate_as(e, [6.5e-7], 0.01, 1.0)
    assert abs(np.linalg.norm(p) / np.linalg.norm(e) - 1) < 1e-12
    back = of.fresnel_propagate_as(p, [6.5e-7], 0.01, -1.0)
    assert np.abs(back - e).max() < 1e-10


def test_fresnel_unit_phase_form():
    """The form the DFT-product Fresnel (sizes that are not powers of two)
    evaluates: E' = c (E + IDFT[DFT(E) (H / c - 1)]), c = exp(2 pi i z / lambda)
    the transfer function at zero frequency, equals fresnelPropagateAS."""
    rng = np.random.default_rng(4)
    n, lam, ap, z = 96, 6.5e-7, 0.01, 0.7
    e = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    ref = of.fresnel_propagate_as(e[None], [lam], ap, z)[0]
    f = np.fft.fftfreq(n, 1.0 / n)
    f2 = f[:, None] ** 2 + f[None, :] ** 2
    zl = z / lam
    tau = -zl * (0.25 * (lam / ap) ** 2 * f2) / (1 + np.sqrt(1 - 0.25 * (lam / ap) ** 2 * f2))
    c = np.exp(2j * np.pi * (zl - np.rint(zl)))
    hm1 = np.exp(2j * np.pi * tau) - 1.0  # H / c - 1
    got = c * (e + np.fft.ifft2(np.fft.fft2(e) * hm1))
    assert np.abs(got - ref).max() < 1e-9 * np.abs(ref).max()


def test_fft_shift_floor_and_truncate():
    a = np.arange(25.0).reshape(5, 5)
    assert np.array_equal(of.fft_shift(a), np.fft.fftshift(a))  # floor(5/2)=2 == numpy for odd
    b = np.arange(36.0).reshape(6, 6) + 0j
    t = of.fft_truncate(b, 4, 4)
    assert t.shape == (4, 4)
    assert t[0, 0] == b[0, 0]
    assert t[2, 0] == (b[2, 0] + b[4, 0]) / 2


def test_mask_quirk_and_mirror():
    e = np.ones((1, 4, 4), complex)
    m = np.full((4, 4), 0.5)
    assert np.allclose(oe.mask_apply(e, m), 0.5 + 0.5j)
    s = np.full((4, 4), 1e-7)
    out = oe.mirror_apply(e, s, [6.5e-7], 1.0)
    assert np.allclose(out, np.exp(-4j * math.pi * 1e-7 / 6.5e-7))


def test_padded_fft_fpm_is_centred_convolution():
    """The plain-Lyot occulter restatement: a mask of ones is the identity,
    and a general mask equals the circular convolution of the padded field
    with the inverse FFT of the (ifftshifted) mask, cropped."""
    rng = np.random.default_rng(3)
    n, pad = 16, 64
    e = rng.standard_normal((1, n, n)) + 1j * rng.standard_normal((1, n, n))
    assert np.allclose(oe.padded_fft_fpm(e, pad, np.ones((1, pad, pad))), e, atol=1e-13)
    m = rng.uniform(0, 1, (1, pad, pad))
    got = oe.padded_fft_fpm(e, pad, m)
    k = np.fft.ifft2(np.fft.ifftshift(m[0]))
    p = np.zeros((pad, pad), complex)
    o = (pad - n) // 2
    p[o:o + n, o:o + n] = e[0]
    conv = np.zeros((pad, pad), complex)
    for dy in range(pad):
        for dx in range(pad):
            if k[dy, dx] != 0:
                conv += k[dy, dx] * np.roll(np.roll(p, dy, 0), dx, 1)
    assert np.allclose(got[0], conv[o:o + n, o:o + n], atol=1e-12)


def _dm_separable(act, n, sigma):
    """Separable restatement of the DM surface used by the GPU (Re(M A M^T))."""
    nA = act.shape[0]
    ur = -(-(n + 1) // nA)
    U = ur * nA
    s = sigma * n / nA
    y = -(n - 1) / 2.0 + np.arange(n)
    ghat = np.fft.fft(np.exp(-4 * math.log(2) * y * y / (s * s)))
    h = n * (1 - 1 / nA) / 2

    def Y(k):
        f = np.where(k < U // 2, k, k - U) / n
        return np.exp(2j * math.pi * (f[:, None] * h - np.outer(k, np.arange(nA)) / nA))
    kp = np.arange(n)
    src = np.where(kp < n // 2, kp, U - n + kp)
    X = Y(src)
    X[n // 2] = 0.5 * (Y(np.array([n // 2]))[0] + Y(np.array([U - n // 2]))[0])
    X = X * ghat[:, None]
    M = np.fft.ifft(X, axis=0)
    return np.real(M @ act @ M.T)


@pytest.mark.parametrize("n,nA,sigma", [(64, 8, 1.0), (128, 12, 1.3), (256, 48, 1.0)])
def test_dm_surface_separable_form(n, nA, sigma):
    """deformableMirror.cpp:216-270 (upsample, FFT, shift, fft_truncate,
    x FFT(influence), IFFT, real) equals Re(M A M^T) with the N x nA basis
    the GPU builds."""
    rng = np.random.default_rng(n)
    act = rng.normal(0, 5e-9, (nA, nA))
    geom = of.ArrayGeom.set_xy(n, n, 1e-4)
    ref = oe.dm_surface(act, oe.dm_influence(geom, sigma, nA))
    got = _dm_separable(act, n, sigma)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_double_fraunhofer_restatement():
    """doubleFraunhoferInterpFPM: the restatement's direct matrix transforms
    equal the reference's Bluestein zoom FFTs on the same geometry, and the
    form the GPU computes, MFT_out[Z] + MFT_out[(M - 1) Z] over the centred
    S x S block only, equals masking that block of Z in place."""
    rng = np.random.default_rng(12)
    n, pad, S, lam = 32, 2.0, 16, 6.5e-7
    dx = 1e-4
    geom = of.ArrayGeom.set_xy(n, n, dx)
    fpm_scale = 3.52 * lam / (n * dx) / 2.0
    e = rng.normal(size=(1, n, n)) + 1j * rng.normal(size=(1, n, n))
    m = np.exp(1j * rng.uniform(-3, 3, (S, S))) * rng.uniform(0.5, 1.0, (S, S))
    out = oe.double_fraunhofer_interp_fpm(e, [lam], geom, fpm_scale, pad, [m])
    nz = int(pad * n)
    zg = of.ArrayGeom.set_xy_offset_m1(nz, nz, fpm_scale)
    zin, zout = of.ZoomFft(geom, zg, [3.52 * lam]), of.ZoomFft(zg, geom, [-3.52 * lam])
    z = zin.execute(e[0], 0)  # the reference's chirp-Z path
    r0 = nz // 2 - S // 2
    z[r0:r0 + S, r0:r0 + S] *= m
    ref = zout.execute(z, 0)
    peak = np.abs(ref).max()
    assert np.abs(out[0] - ref).max() / peak < 1e-11
    # decomposed form
    z = zin.mft(e[0], 0)
    blk = np.zeros_like(z)
    blk[r0:r0 + S, r0:r0 + S] = (m - 1.0) * z[r0:r0 + S, r0:r0 + S]
    dec = zout.mft(z, 0) + zout.mft(blk, 0)
    assert np.abs(out[0] - dec).max() / peak < 1e-12


def test_single_thread_row_check_quirk():
    """make_interpolation_data on one OpenMP thread checks each cell after a
    row's first passing cell with the row index left by the previous cell's
    last sub-sample (complexHexMaskFPM.cpp:395-423). Where that index falls
    off the design array and hexes reach the array's edge (scale factor 1,
    mask grid a little wider than the array), the reference leaves the rest
    of that mask row unfilled; the midpoint check fills it. Elsewhere the
    two agree."""
    from oracle import native
    from csim_gb300.synth import hex_layout_standard
    hx, hy = hex_layout_standard(4)
    A, S, n_sub, pix = 256, 64, 8, 2e-6
    d = native.hex_design_array(hx, hy, 4, A, 1.0, 0.01, 1.0)
    mid = native.interpolation_tables(d, S, n_sub, pix, S * pix * 0.49, 1.0)
    ref = native.interpolation_tables(d, S, n_sub, pix, S * pix * 0.49, 1.0, stale=True)
    diff = (mid[0] != ref[0]).any(0) | (mid[1] != ref[1]).any(0)
    rows = sorted(set(np.argwhere(diff)[:, 0].tolist()))
    assert rows == [S - 1] and diff.sum() > 10
    # the reference's unfilled cells read as outside every hex
    r = S - 1
    cols = np.argwhere(diff[r])[:, 0]
    assert (ref[0][:, r, cols] == -1).all()
    assert (ref[1][0, r, cols] == n_sub * n_sub).all()
    # with the standard 0.9 scale factor no hex reaches the edge: identical
    d9 = native.hex_design_array(hx, hy, 4, A, 0.9, 0.01, 1.0)
    a = native.interpolation_tables(d9, S, n_sub, pix, S * pix * 0.45, 0.9)
    b = native.interpolation_tables(d9, S, n_sub, pix, S * pix * 0.45, 0.9, stale=True)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_prolate_apodizer_has_eigenvalue_one_half():
    """The designed optics' apodization: the fundamental radial prolate of a
    focal disk whose band-limiting eigenvalue is 1/2 (a pi-phase disk then
    cancels it in the Lyot plane), monotone from 1 at the centre to ~0.71 at
    the pupil edge, zero outside."""
    from csim_gb300.synth import prolate_apodizer, prolate_radial
    a, alpha = prolate_apodizer(128, 50.0)
    assert abs(prolate_radial(alpha)[0] - 0.5) < 1e-6
    assert 0.52 < alpha < 0.54
    row = a[64, 64:]
    assert abs(row[0] - 1.0) < 1e-3 and np.all(np.diff(row[:49]) <= 1e-12)
    assert 0.69 < row[49] < 0.73 and row[60] == 0.0
