"""Bounded waits in the tensor-core transforms (celem.hpp:34 elements have no
failure reporting; here a device-side wait that runs out becomes a status).
With a wait budget of a few cycles the transform's roles give up on each
other: the kernel stops, waits out its own operand loads and products,
releases its tensor memory and returns, and csg_sync reports CSG_E_TIMEOUT.
The same context then runs the transform again with the default budget and
gets the right answer. No fault, trap or hang is involved."""
import numpy as np
import pytest
import torch

from csim_gb300 import _lib
from oracle import csim_fft as of

pytestmark = pytest.mark.gpu


def test_wait_budget_timeout_then_recovery():
    from csim_gb300 import runtime as R
    ctx = R.Context(0)
    try:
        rng = np.random.default_rng(9)
        n, no, F = 512, 128, 16
        x = rng.standard_normal((F, n, n)) + 1j * rng.standard_normal((F, n, n))
        xi = np.arange(n) - n / 2 + 0.5
        xo = (np.arange(no) - no / 2 + 0.5) * 0.37
        plan = R.Mft(ctx, xi, xi, xo, xo, [1.0 * n], 1.0, -1.0)
        plan.set_tile(128)
        inp = R.to_planar(x)
        slot = R.dvec([0] * F, torch.int32)
        out = plan(inp, slot)
        ctx.sync()
        _lib.call("csg_set_wait_budget", ctx.h, 2)
        plan(inp, slot, out=out)
        with pytest.raises(_lib.CsgError) as e:
            ctx.sync()
        assert e.value.code == -4, e.value
        _lib.call("csg_set_wait_budget", ctx.h, 0)
        out = plan(inp, slot)
        ctx.sync()  # the status was cleared by the failing sync
        got = R.from_planar(out)
        ref = of.mft(x[3], xi, xi, xo, xo, 1.0 * n, 1.0)
        assert np.abs(got[3] - ref).max() / np.abs(ref).max() < 1e-6
        plan.close()
    finally:
        ctx.close()
