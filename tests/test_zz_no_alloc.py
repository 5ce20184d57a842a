"""csg_hex_mask_noalloc: the hex focal-plane mask for callers that cannot let
the library allocate device memory (for example an application that reserves
its whole memory budget at start-up). Its results must equal csg_hex_mask's,
call after call, while the shared scratch array keeps the previous call's
contents. This file is collected last so a failure here never hides another
test; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 3e-6  # the tolerance the hex-mask parity tests use


def _tables(rng, S, n_hex, n_sub):
    ids = np.full((3, S, S), -1, np.int16)
    cnt = np.zeros((3, S, S), np.uint16)
    tot = n_sub * n_sub
    for r in range(S):
        for c in range(S):
            k = int(rng.integers(0, 4))
            cuts = np.sort(rng.integers(0, tot + 1, size=max(k - 1, 0)))
            sizes = np.diff(np.concatenate([[0], cuts, [tot]])) if k else np.array([tot])
            for j, sz in enumerate(sizes[:3]):
                cnt[j, r, c] = sz
                ids[j, r, c] = rng.integers(0, n_hex) if k else -1
    return ids, cnt


def _call(name, ctx, ids, cnt, n_sub, sags, cand, lam, only, out):
    from csim_gb300._lib import call
    from csim_gb300.runtime import ptr
    call(name, ctx.h, ptr(ids), ptr(cnt), ids.shape[-1], n_sub, ptr(sags), sags.shape[1],
         cand.numel(), ptr(cand), ptr(lam), 1.0, 1, 1.0, only, ptr(out))


def test_noalloc_matches_allocating_entry_point_twice():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from csim_gb300.runtime import Context, dvec
    ctx = Context(0)
    rng = np.random.default_rng(21)
    S, n_hex, n_sub = 40, 37, 8
    ids_h, cnt_h = _tables(rng, S, n_hex, n_sub)
    ids = dvec(ids_h, torch.int16)
    cnt = dvec(cnt_h.view(np.int16), torch.int16)
    for call_no, only in enumerate([-1, 7]):  # two calls in a row, different inputs
        sags = dvec(rng.uniform(-5e-7, 5e-7, (3, n_hex)))
        cand = dvec(rng.integers(0, 3, 5).astype(np.int32), torch.int32)
        lam = dvec(rng.uniform(6e-7, 7e-7, 5))
        ref = torch.empty((5, 2, S, S), dtype=torch.float32, device="cuda")
        got = torch.full((5, 2, S, S), float("nan"), dtype=torch.float32, device="cuda")
        _call("csg_hex_mask", ctx, ids, cnt, n_sub, sags, cand, lam, only, ref)
        _call("csg_hex_mask_noalloc", ctx, ids, cnt, n_sub, sags, cand, lam, only, got)
        ctx.sync()
        a, b = ref.cpu().numpy(), got.cpu().numpy()
        assert np.isfinite(b).all(), f"call {call_no}: unwritten output"
        assert np.abs(a - b).max() < TOL, f"call {call_no}"
    ctx.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from csim_gb300._lib import CsgError
    from csim_gb300.runtime import Context, dvec
    ctx = Context(0)
    S, n_hex, n_sub = 8, 4095, 4
    ids = torch.zeros((3, S, S), dtype=torch.int16, device="cuda")
    cnt = torch.zeros((3, S, S), dtype=torch.int16, device="cuda")
    n_out = 262144 // (n_hex + 1) + 1          # one output past the fixed scratch
    sags = dvec(np.zeros((1, n_hex)))
    cand = dvec(np.zeros(n_out, np.int32), torch.int32)
    lam = dvec(np.full(n_out, 6.5e-7))
    out = torch.empty((n_out, 2, S, S), dtype=torch.float32, device="cuda")
    with pytest.raises(CsgError) as ei:
        _call("csg_hex_mask_noalloc", ctx, ids, cnt, n_sub, sags, cand, lam, -1, out)
    assert "exceeds the fixed scratch" in str(ei.value)
    ctx.close()
