"""Surrogate MLP: GPU forward/backward against the FP64 oracle (same bf16
rounding points), training convergence, and what surrogate screening gains
over plain DE on the response-matrix objective (the exact linear equivalent
of full propagation).
"""
import math

import numpy as np
import pytest
import torch

from oracle import mlp as om

pytestmark = pytest.mark.gpu


def test_mlp_gradients_match_oracle(ctx):
    from csim_gb300.surrogate import Surrogate
    rng = np.random.default_rng(0)
    B, n_in, hidden = 64, 40, (64, 32, 16)
    net = Surrogate(ctx, n_in, hidden, max_batch=B, seed=3)
    x = rng.standard_normal((B, n_in)).astype(np.float32)
    t = rng.standard_normal(B).astype(np.float32)
    net.set_input(torch.as_tensor(x, device="cuda"))
    loss = net.train_step(B, torch.as_tensor(t, device="cuda"), 0.0)
    ctx.sync()
    ws, bs, gws, gbs = [], [], [], []
    for l in range(net.n_layers):
        w, b, gw, gb = net.param(l)
        ws.append(w.double().cpu().numpy())
        bs.append(b.double().cpu().numpy())
        gws.append(gw.double().cpu().numpy())
        gbs.append(gb.double().cpu().numpy())
    ref_loss, rgw, rgb = om.loss_and_grads(x.astype(np.float64), t.astype(np.float64), ws, bs)
    assert abs(float(loss.item()) - ref_loss) / ref_loss < 1e-4
    for l in range(net.n_layers):
        ew = np.linalg.norm(gws[l] - rgw[l]) / np.linalg.norm(rgw[l])
        eb = np.linalg.norm(gbs[l] - rgb[l]) / np.linalg.norm(rgb[l])
        assert ew < 2e-3 and eb < 2e-3, (l, ew, eb)
    # forward prediction
    y = net.forward(B).double().cpu().numpy()
    ry, _, _ = om.forward(x.astype(np.float64), ws, bs)
    assert np.abs(y - ry).max() / np.abs(ry).max() < 1e-4
    net.close()


def test_mlp_training_reduces_loss(ctx):
    from csim_gb300.surrogate import Surrogate
    rng = np.random.default_rng(1)
    B, n_in = 256, 64
    net = Surrogate(ctx, n_in, (128, 64), max_batch=B, seed=5)
    a = rng.standard_normal(n_in) / math.sqrt(n_in)
    losses = []
    for step in range(300):
        x = rng.standard_normal((B, n_in)).astype(np.float32)
        t = np.sin(2.0 * (x @ a)).astype(np.float32)
        net.set_input(torch.as_tensor(x, device="cuda"))
        losses.append(float(net.train_step(B, torch.as_tensor(t, device="cuda"), 3e-3).item()))
    assert np.mean(losses[-20:]) < 0.2 * np.mean(losses[:20]), (losses[:3], losses[-3:])
    net.close()


def test_screened_de_beats_plain_de(ctx):
    """What surrogate screening gains: a response-matrix problem
    (optHexRespObjective, optObjective.cpp:24-69) with 37 hexes, 2
    wavelengths and a known exact null (the Babinet column cancels the hex
    columns at a hidden sag vector). With equal numbers of full evaluations,
    DE that screens 8 trials per member with the trained surrogate reaches a
    lower contrast than plain DE, for each of two seeds."""
    from csim_gb300 import optimize as opt
    from csim_gb300 import surrogate as su
    rng = np.random.default_rng(7)
    nvar, npix = 37, 128
    lam = np.array([640e-9, 660e-9])
    half = 80e-9
    xstar = rng.uniform(-half, half, nvar)
    M = np.empty((2, npix, nvar + 1), complex)
    for l in range(2):
        M[l, :, :nvar] = rng.standard_normal((npix, nvar)) + 1j * rng.standard_normal((npix, nvar))
        M[l, :, nvar] = -M[l, :, :nvar] @ np.exp(1j * 4 * math.pi / lam[l] * xstar)
    full = opt.RespObjective(ctx, M, lam, 1.0)
    per_lam = [opt.RespObjective(ctx, M[l:l + 1], lam[l:l + 1], 1.0) for l in range(2)]
    assert float(full(torch.as_tensor(xstar[None], device="cuda")).item()) < 1e-10
    # training samples: random sag vectors, per-wavelength log10 contrast
    n = 16384
    X = torch.as_tensor(rng.uniform(-half, half, (n, nvar)), device="cuda")
    xs, ls, ys = [], [], []
    for l, obj in enumerate(per_lam):
        xs.append(X)
        ls.append(torch.full((n,), lam[l], dtype=torch.float64, device="cuda"))
        ys.append(torch.log10(obj(X)).float())
    model = su.ContrastModel(ctx, nvar, lam, 1.0, hidden=(256, 128, 64), max_batch=1024, seed=1)
    hist = model.train(torch.cat(xs), torch.cat(ls), torch.cat(ys), epochs=12, batch=256,
                       lr=1e-3)
    assert hist[-1] < 0.3 * hist[0], hist
    # ranking quality on fresh candidates
    Xt = torch.as_tensor(rng.uniform(-half, half, (512, nvar)), device="cuda")
    true = full(Xt).cpu().numpy()
    pred = model.predict_cost(Xt).cpu().numpy()
    rank = lambda v: np.argsort(np.argsort(v))
    rho = np.corrcoef(rank(true), rank(pred))[0, 1]
    assert rho > 0.6, rho

    def run(screened, seed):
        cfg = opt.DEConfig(populationSize=32, maxIterations=40, globalBounds=(-half, half),
                           initBounds=(-half, half), initSpread=1.0, seed=seed,
                           startStrategy="deRand1", baseStrategy="deRand1",
                           endStrategy="deRand1", outputInterval=1000, crossoverProb=0.9,
                           fWeight=0.7)
        de = (su.ScreenedDE(ctx, nvar, cfg, model, draws=8) if screened
              else opt.DifferentialEvolution(ctx, nvar, cfg))
        best, _, _ = de.optimize(lambda x, out: full(x, out))
        de.close()
        return best

    for seed in (3, 4):
        plain, screened = run(False, seed), run(True, seed)
        assert screened < plain, (seed, screened, plain)
    model.close()
