"""GPU parity of the optimisation path: the response-matrix objective against
the reference's recorded known answer and the FP64 oracle, and the device DE
generation bit for bit against its restatement."""
import os

import numpy as np
import pytest
import torch

from oracle import de as ode
from oracle import elements as oe

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_response_objective_known_answer(ctx):
    """optHexRespObjective on the reference's mono response matrix at its
    recorded best vector: 1.35012e-10 (optBestVal.txt; oracle 1.3501189541e-10)."""
    from csim_gb300.optimize import RespObjective
    g = np.load(os.path.join(GOLD, "mono_response.npz"))
    obj = RespObjective(ctx, g["M"], g["wavelengths"], float(g["calib"]))
    x = torch.as_tensor(np.ascontiguousarray(g["best_x"]), device="cuda")
    f = obj(x)
    ctx.sync()
    f = f.cpu().numpy()
    for v, rec in zip(f, g["best_val"]):
        assert abs(v - 1.3501189541e-10) / 1.35e-10 < 1e-3, v
        assert abs(v - rec) / rec < 1e-3


@pytest.mark.parametrize("mode", ["mean", "max"])
def test_response_objective_population(ctx, mode):
    from csim_gb300.optimize import RespObjective
    g = np.load(os.path.join(GOLD, "mono_response.npz"))
    rng = np.random.default_rng(5)
    pop = 40
    x = g["best_x"][0][None, :] + rng.uniform(-2e-8, 2e-8, (pop, 499))
    # three (s, lambda) matrices at two wavelengths: exercises the slot map
    m = np.concatenate([g["M"], 0.7 * g["M"], g["M"] * np.exp(0.3j)])
    lam = [6.5e-7, 6.5e-7, 6.6e-7]
    obj = RespObjective(ctx, m, lam, float(g["calib"]), objective=mode)
    f = obj(torch.as_tensor(np.ascontiguousarray(x), device="cuda"))
    ctx.sync()
    # each matrix with its own wavelength (optObjective.cpp:36-50)
    pix = np.zeros((636, pop))
    xf = np.vstack([x.T, np.zeros((1, pop))])
    for i in range(3):
        e = m[i] @ np.exp(1j * 4 * np.pi / lam[i] * xf)
        pix += (e * e.conj()).real
    ref = (pix.mean(0) if mode == "mean" else pix.max(0)) / float(g["calib"])
    np.testing.assert_allclose(f.cpu().numpy(), ref, rtol=2e-3)


def _de_setup(ctx, P=12, nv=9, seed=11):
    from csim_gb300.optimize import DEConfig, DifferentialEvolution
    cfg = DEConfig(populationSize=P, seed=seed, initBounds=(-1e-7, 1e-7), globalBounds=(-3e-7, 3e-7))
    d = DifferentialEvolution(ctx, nv, cfg)
    return d, cfg


def test_de_generation_bit_exact(ctx):
    from csim_gb300._lib import call
    P, nv, seed = 12, 9, 11
    d, cfg = _de_setup(ctx, P, nv, seed)
    ilo, ihi = np.full(nv, -1e-7), np.full(nv, 1e-7)
    glo, ghi = np.full(nv, -3e-7), np.full(nv, 3e-7)
    origin = np.linspace(-2e-8, 2e-8, nv)
    # fresh population: objective = sum of squares (any deterministic function)
    def objective(x, out):
        out.copy_((x * x).sum(1) * 1e12)
    d.initialise(origin, 1.0, objective)
    ctx.sync()
    pop0 = d.pop.cpu().numpy()
    np.testing.assert_array_equal(pop0, ode.init_uniform(P, origin, ilo, ihi, 1.0, seed))
    f = d.f.cpu().numpy()
    best_val, best = 1e300, np.zeros(nv)
    pop, fv, best_val, best, mean, _ = ode.select(pop0, f, pop0, f + 1, best_val, best)
    for gen, strategy in enumerate([0, 1, 2, 2, 1]):
        call("csg_de_generate", d.h, strategy, 0.7, 0.9)
        ctx.sync()
        tri = d.trial.cpu().numpy()
        ref_tri, _ = ode.trial(pop, best, mean, glo, ghi, ilo, ihi, strategy, 0.7, 0.9, seed, gen)
        np.testing.assert_array_equal(tri, ref_tri)
        objective(d.trial, d.f_trial)
        call("csg_de_select", d.h, 0)
        ctx.sync()
        ft = d.f_trial.cpu().numpy()
        pop, fv, best_val, best, mean, _ = ode.select(pop, fv, ref_tri, ft, best_val, best)
        np.testing.assert_array_equal(d.pop.cpu().numpy(), pop)
        bv, _, _, g, vec = d.stats(True)
        assert g == gen + 1 and bv == best_val and np.array_equal(vec, best)
    d.close()


def test_de_minimises_response_objective(ctx):
    """A short DE run on the mono response problem lowers the contrast well
    below its starting population."""
    from csim_gb300.optimize import DEConfig, DifferentialEvolution, RespObjective
    g = np.load(os.path.join(GOLD, "mono_response.npz"))
    obj = RespObjective(ctx, g["M"], g["wavelengths"], float(g["calib"]))
    cfg = DEConfig(populationSize=64, maxIterations=150, outputInterval=50, fWeight=0.5,
                   crossoverProb=1.0, initBounds=(-5e-8, 5e-8), seed=3)
    d = DifferentialEvolution(ctx, 499, cfg, mean=np.zeros(499))
    best, vec, hist = d.optimize(obj)
    ctx.sync()
    f0 = oe.opt_hex_resp_objective([g["M"]], g["wavelengths"], float(g["calib"]),
                                   np.zeros((499, 1)))[0]
    ref = oe.opt_hex_resp_objective([g["M"]], g["wavelengths"], float(g["calib"]), vec[:, None])[0]
    assert abs(ref - best) / best < 1e-3      # the device value is the true objective
    assert best < 0.5 * f0                    # and it improved on the flat mask
    d.close()


def test_graphed_generation_matches_eager(ctx):
    """DE by full propagation: generations replayed from one captured CUDA
    graph (trial generation, the chain walk, contrast reduction, selection)
    give exactly the populations and values of eagerly launched generations."""
    import torch
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import optimize as opt
    from csim_gb300.workloads import PiaacmcSpec, build_piaacmc
    spec = PiaacmcSpec(n=256, beam_px=200, wavelengths=(640e-9, 660e-9), S=128,
                       fpm_sampling=8.0, n_rings=3, n_sub=8, design_size=512, n_out_fov=32.0,
                       spl=4.0)
    stream = torch.cuda.Stream()
    ctx.bind_stream(stream)
    results = []
    try:
        _run_graph_vs_eager(ctx, spec, stream, results, cg, opt, build_piaacmc)
    finally:  # the session context goes back to torch's current stream
        ctx.bind_stream(torch.cuda.current_stream())
    (p0, f0, g0), (p1, f1, g1) = results
    assert g0 == g1
    assert torch.equal(p0, p1) and torch.equal(f0, f1)


def _run_graph_vs_eager(ctx, spec, stream, results, cg, opt, build_piaacmc):
    import torch
    with torch.cuda.stream(stream):
        for graphed in (False, True):
            cor, inp = build_piaacmc(ctx, spec)
            reg = cg.RegionContrast(ctx, cor.n_out, cor.out_pixel, inp["lod_image"], 2.0, 8.0)
            P = 16
            obj = opt.PropagatedObjective(cor, reg, P, use_graph=False)
            cfg = opt.DEConfig(populationSize=P, globalBounds=(-5e-7, 5e-7),
                               initBounds=(-5e-7, 5e-7), fWeight=0.7, crossoverProb=0.9, seed=9)
            de = opt.DifferentialEvolution(ctx, inp["hex_x"].size, cfg)
            de.set_trial_buffer(obj.sags)
            de.initialise(np.zeros(inp["hex_x"].size), 1.0, obj)
            if graphed:
                g = opt.GraphedGeneration(de, "deRand1", obj, stream)  # runs one generation
                for _ in range(3):
                    g.replay()
            else:
                for _ in range(4):
                    de.generation("deRand1", obj)
            stream.synchronize()
            results.append((de.pop.clone(), de.f.clone(), de.stats()[3]))
            de.close()
            cor.close()
