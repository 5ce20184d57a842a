"""The C ABI's boundary: the Armadillo-layout field transfer the reference's
elements would use (csg_field_upload / csg_field_download, efield.hpp:45-52),
and the status codes of rejected calls (bad shapes, non-finite inputs, bad
enums), after which the context keeps working."""
import ctypes as C

import numpy as np
import pytest
import torch

from csim_gb300 import _lib
from oracle import csim_fft as of

pytestmark = pytest.mark.gpu
P = C.c_void_p


def _dev(n_bytes):
    return torch.empty(n_bytes, dtype=torch.uint8, device="cuda")


@pytest.mark.parametrize("layout", [0, 1])
def test_field_upload_download_round_trip(ctx, layout):
    """complex<double> fields in Armadillo column-major (layout 0: (r, c, s)
    at r + c R + s R C) or row-major order: upload to planar fp32, download
    back, equal to the input rounded to fp32; the planar field holds element
    (r, c) at row r, column c."""
    rng = np.random.default_rng(2)
    R, Cc, F = 48, 40, 3
    cube = rng.standard_normal((F, R, Cc)) + 1j * rng.standard_normal((F, R, Cc))  # [s][r][c]
    host = np.ascontiguousarray(np.transpose(cube, (0, 2, 1)) if layout == 0 else cube)
    staging = _dev(F * R * Cc * 16)
    dev = torch.empty((F, 2, R, Cc), dtype=torch.float32, device="cuda")
    _lib.call("csg_field_upload", ctx.h, host.ctypes.data_as(P), layout, R, Cc, F,
              P(staging.data_ptr()), P(dev.data_ptr()))
    back = np.empty_like(host)
    _lib.call("csg_field_download", ctx.h, P(dev.data_ptr()), R, Cc, F, P(staging.data_ptr()),
              back.ctypes.data_as(P), layout)
    ctx.sync()
    planar = dev.double().cpu().numpy()
    r32 = cube.astype(np.complex64).astype(np.complex128)
    assert np.array_equal(planar[:, 0] + 1j * planar[:, 1], r32)
    assert np.array_equal(back, np.transpose(r32, (0, 2, 1)) if layout == 0 else r32)


def test_column_major_upload_mft_download_matches_oracle(ctx):
    """An Armadillo cube through upload, an MFT plan and download, compared
    with the FP64 oracle's zoom transform of the same cube."""
    from csim_gb300 import runtime as R
    rng = np.random.default_rng(4)
    ny, nx, no, F = 64, 80, 32, 2
    cube = rng.standard_normal((F, ny, nx)) + 1j * rng.standard_normal((F, ny, nx))
    host = np.ascontiguousarray(np.transpose(cube, (0, 2, 1)))
    yin = (np.arange(ny) - ny / 2 + 0.5) * 1e-5
    xin = (np.arange(nx) - nx / 2 + 0.5) * 1e-5
    xo = (np.arange(no) - no / 2 + 0.5) * 2e-6
    lf = 1.3e-6 * 1.5
    pref = 1e-10 / (1j * lf)
    plan = R.Mft(ctx, yin, xin, xo, xo, [lf], pref, -1.0)
    staging = _dev(F * ny * nx * 16)
    din = torch.empty((F, 2, ny, nx), dtype=torch.float32, device="cuda")
    _lib.call("csg_field_upload", ctx.h, host.ctypes.data_as(P), 0, ny, nx, F,
              P(staging.data_ptr()), P(din.data_ptr()))
    out = plan(din, R.dvec([0] * F, torch.int32))
    back = np.empty((F, no, no), np.complex128)
    _lib.call("csg_field_download", ctx.h, P(out.data_ptr()), no, no, F, P(staging.data_ptr()),
              back.ctypes.data_as(P), 0)
    ctx.sync()
    got = np.transpose(back, (0, 2, 1))
    for f in range(F):
        ref = of.mft(cube[f], xin, yin, xo, xo, lf, pref)
        assert np.abs(got[f] - ref).max() / np.abs(ref).max() < 1e-6
    plan.close()


def _code(fn, *args):
    try:
        _lib.call(fn, *args)
    except _lib.CsgError as e:
        return e.code, str(e)
    return 0, ""


def test_rejected_calls_return_status_codes(ctx):
    from csim_gb300 import runtime as R
    f = torch.zeros((1, 2, 96, 96), dtype=torch.float32, device="cuda")
    # sizes that are neither powers of two nor multiples of 8 are refused
    # with CSG_E_SHAPE before the field is touched (96 runs as a DFT product)
    assert _code("csg_fft2d", ctx.h, P(f.data_ptr()), 1, 100, -1)[0] == -2
    assert _code("csg_fft2d", ctx.h, P(f.data_ptr()), 1, 96, -1)[0] == 0
    # bad enums: direction, precision, layout
    g = torch.zeros((1, 2, 64, 64), dtype=torch.float32, device="cuda")
    assert _code("csg_fft2d", ctx.h, P(g.data_ptr()), 1, 64, 0)[0] == -1
    assert _code("csg_fft2d_prec", ctx.h, P(g.data_ptr()), 1, 64, -1, 7)[0] == -1
    host = np.zeros((4, 4), np.complex128)
    assert _code("csg_field_upload", ctx.h, host.ctypes.data_as(P), 5, 4, 4, 1,
                 P(g.data_ptr()), P(g.data_ptr()))[0] == -1
    # MFT inputs must be multiples of 8; non-finite coordinates are CSG_E_NAN
    v = np.arange(12, dtype=np.float64)
    lf = np.array([1.0])
    h = P()
    dp = lambda a: a.ctypes.data_as(P)  # noqa: E731
    assert _code("csg_mft_create", ctx.h, C.byref(h), 12, 12, 8, 8, dp(v), dp(v), dp(v[:8]),
                 dp(v[:8]), 1, dp(lf), None, -1.0, 6)[0] == -2
    w = np.arange(16, dtype=np.float64)
    w[3] = np.nan
    code, msg = _code("csg_mft_create", ctx.h, C.byref(h), 16, 16, 8, 8, dp(w), dp(w), dp(w[:8]),
                      dp(w[:8]), 1, dp(lf), None, -1.0, 6)
    assert code == -6 and "non-finite" in msg
    assert _code("csg_mft_create", ctx.h, C.byref(h), 16, 16, 8, 8, dp(v), dp(v), dp(v[:8]),
                 dp(v[:8]), 1, dp(lf), None, -1.0, 5)[0] == -1
    lam = R.dvec([6.5e-7])
    assert _code("csg_fresnel", ctx.h, P(g.data_ptr()), 1, 64, P(lam.data_ptr()),
                 float("nan"), 1.0)[0] == -6
    assert _code("csg_fresnel", ctx.h, P(g.data_ptr()), 1, 64, P(lam.data_ptr()), -1.0,
                 1.0)[0] == -1
    ch = P()
    bad = np.array([6.5e-7, np.inf])
    assert _code("csg_chain_create", ctx.h, C.byref(ch), 64, 1e-5, 2, dp(bad), 6)[0] == -6
    # the context still works after the refusals
    ctx.fft2d(g, -1)
    ctx.sync()
