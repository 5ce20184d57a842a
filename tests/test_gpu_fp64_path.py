"""The plain FP64 GPU path (the bench's comparator, baseline/fp64_gpu.py)
against the FP64 oracle: it must be the same computation, so the error is
FP64 rounding (<= 1e-10 of the image peak)."""
import numpy as np
import pytest
import torch

from oracle import chain as oc

pytestmark = pytest.mark.gpu


def test_fp64_gpu_path_matches_oracle(ctx):
    from baseline.fp64_gpu import Fp64Piaacmc, throughput
    from csim_gb300 import workloads as W
    spec = W.PiaacmcSpec(n=256, beam_px=200, wavelengths=(640e-9, 660e-9), S=128,
                         fpm_sampling=8.0, n_rings=3, n_sub=8, design_size=512, n_out_fov=32.0,
                         spl=4.0)
    cor, inp = W.build_piaacmc(ctx, spec)
    box = tuple(cor.fpm_region())
    cor.close()
    rng = np.random.default_rng(11)
    sags = W.random_sags(rng, 2, inp["hex_x"].size, spec.sag_range)
    model = Fp64Piaacmc(inp, spec)
    for li in range(len(inp["lam"])):
        got = model.field(li, 0.8, torch.as_tensor(sags[li], device="cuda")).cpu().numpy()
        ref = oc.piaacmc_field(inp, spec, inp["lam"][li], 0.8, 0.0, 0.0, sags[li])
        assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-10
    v, n, dt = throughput(model, sags, 1.0, 3)
    assert n == 3 and v > 0
    # the support-cropped comparator is the same computation (exact crops)
    cropped = Fp64Piaacmc(inp, spec, fpm_box=box)
    for li in range(len(inp["lam"])):
        s = torch.as_tensor(sags[li], device="cuda")
        for cal in (False, True):
            a = cropped.field(li, 0.8, s, calibrating=cal).cpu().numpy()
            b = model.field(li, 0.8, s, calibrating=cal).cpu().numpy()
            assert np.abs(a - b).max() / np.abs(b).max() < 1e-10
