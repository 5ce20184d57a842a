"""Field-propagation throughput of the PIAACMC-style 1024^2 chain on GB300.

One step = one batch of B fields (default 64 FPM candidates, lambda = 650 nm,
on-axis source), each propagated through the full element walk
(pupil mask -> PIAA M1 -> Fresnel 1 m -> PIAA M2 -> 217-hex FPM via
512^2 MFT at 1/16 lambda/D (Babinet) -> Lyot 0.95 -> 256^2 MFT at
0.25 lambda/D) and reduced to the 2-8 lambda/D dark-hole contrast of every
candidate. Metric: field propagations per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--workload piaacmc|plain_lyot|broadband|de]

The other workloads measure the plain Lyot coronagraph (512^2 pupil,
2048^2 padded-FFT occulter, 128^2 image; a batch of off-axis sources) and
the broadband batch (2048^2 segmented pupil + DM, 11 wavelengths x 3
sources onto ragged 460^2..540^2 images in one launch) and differential
evolution by full propagation (1261 hexes, 5 wavelengths, population 64:
one generation = 320 fields, replayed as one CUDA graph).

Under torchrun each rank runs its own batch (candidates are independent:
weak scaling, no data-path collective); timing is the max over ranks.
`--impl reference` times the reference-semantics CPU restatement of the same
path (the reference itself needs FFTW/Armadillo/cfitsio, absent here).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = ("piaacmc-1024: pupil + PIAA M1/M2 (even poly, PV 2um) + Fresnel 1.0 m + "
            "217-hex FPM (8 rings, U(+-0.5um)) via 512^2 MFT at 1/16 lambda/D, Babinet + "
            "Lyot 0.95 + 256^2 MFT at 0.25 lambda/D + 2-8 lambda/D contrast")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        # the dominant GEMM is timed within a ~5 ms step: the burst figure applies
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [l.strip().split(", ") for l in open(self.path) if l.strip()]
        os.unlink(self.path)
        if not rows:
            return None
        def mhz(v):
            try:
                return float(v.split()[0])
            except Exception:
                return float("nan")
        sm = [mhz(r[1]) for r in rows if len(r) > 8]
        mx = [mhz(r[2]) for r in rows if len(r) > 8]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip() == "Active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ------------------------------------------------------------------ CPU
def cpu_fields_per_s(spec, inp, sags, budget_s: float, max_fields: int):
    """Reference-semantics CPU restatement (FP64, scipy/pocketfft + BLAS, all
    host threads) of the same per-field path: the reference's own
    fpmPupToLyot algorithm (mask hat by chirp-Z zoom + 2N x 2N FFT
    convolution, recomputed for every candidate's mask)."""
    from oracle import chain as oc
    t0 = time.perf_counter()
    n = 0
    while n < max_fields and (time.perf_counter() - t0) < budget_s:
        oc.piaacmc_field(inp, spec, float(inp["lam"][0]), 1.0, 0.0, 0.0, sags[n % len(sags)],
                         conv_form=True, czt=True)
        n += 1
    dt = time.perf_counter() - t0
    return n / dt, n, dt


def reference_arm(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    from csim_gb300.synth import PiaacmcSpec
    from oracle.chain import host_inputs
    spec = PiaacmcSpec()
    inp = host_inputs(spec)
    rng = np.random.default_rng(7)
    sags = rng.uniform(-spec.sag_range, spec.sag_range, (8, spec.n_hex))
    per_step = 1 if args.steps > 20 else 2  # bounded: the whole run stays within minutes
    for _ in range(args.warmup):
        cpu_fields_per_s(spec, inp, sags, 1e9, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_fields_per_s(spec, inp, sags, 1e9, per_step)
    dt = time.perf_counter() - t0
    v = per_step * args.steps / dt
    cores = os.cpu_count()
    line = {"metric": "field propagations/s", "value": v, "unit": "fields/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": WORKLOAD, "fields_per_step": per_step},
            "cpu_baseline": {"value": v, "unit": "fields/s", "cores": cores, "kind": "port",
                             "sample": f"{per_step} fields per step x {args.steps} steps"},
            "e2e": {"value": v, "unit": "fields/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ GPU
class Workload:
    """One benchmark configuration: the chain, its batch, the per-step
    device work (graph replay + contrast reduction) and the host input a
    user uploads every step for the end-to-end number."""


def setup_piaacmc(args, ctx, W, cg, rank):
    import torch
    wl = Workload()
    spec = W.PiaacmcSpec()
    B = args.fields
    cor, inp = W.build_piaacmc(ctx, spec, precision=args.precision, support_crop=not args.no_crop)
    rng = np.random.default_rng(100 + rank)
    sags_h = W.random_sags(rng, B, spec.n_hex, spec.sag_range)
    sags_d = cor.sags(B)
    sags_d.copy_(torch.as_tensor(sags_h))
    cor.batch_all(1)
    cal = cor.execute(calibrating=True)
    reg = cg.RegionContrast(ctx, cor.n_out, cor.out_pixel, inp["lod_image"], 2.0, 8.0)
    wl.cmax = reg.calibration_max(cal)
    cor.batch_all(B)
    wl.per_group = 1
    wl.cor, wl.inp, wl.reg, wl.B, wl.spec = cor, inp, reg, B, spec
    # every step the candidates' sags come from the host
    wl.host_in, wl.dev_in = torch.as_tensor(sags_h), sags_d
    wl.cpu = lambda budget, nmax: cpu_fields_per_s(spec, inp, sags_h, budget, nmax)

    def fp64(budget, nmax, crop=False):  # the plain FP64 GPU path on the same inputs
        from baseline.fp64_gpu import Fp64Piaacmc, throughput
        box = tuple(cor.fpm_region()) if crop else None
        return throughput(Fp64Piaacmc(inp, spec, fpm_box=box), sags_h[:8], budget, nmax)
    wl.fp64 = fp64
    wl.cpu_sample = ("FP64, reference algorithm: chirp-Z mask hat + 2048^2 FFT convolution")
    wl.bound = "tensor"
    wl.config = {"workload": WORKLOAD, "fields_per_step": B, "n": spec.n, "fpm_grid": spec.S,
                 "n_hex": spec.n_hex, "image": cor.n_out,
                 "precision": f"bf16x{args.precision}", "fpm_support_crop": not args.no_crop,
                 "fpm_transformed_box": list(cor.fpm_region()),
                 "l2": f"working set > L2 (fields + MFT operands ~{0.024 * B:.1f} GB per step)"}
    return wl


def setup_plain_lyot(args, ctx, W, cg, rank):
    """Plain Lyot coronagraph (512^2 pupil, 2048^2 padded-FFT occulter, 0.9
    Lyot stop, 128^2 final MFT): a batch of point sources at random offsets
    within 4 lambda/D, uploaded every step. The occulter runs in its Babinet
    form (an MFT pair over the support of 1 - mask) unless --fft-occulter."""
    import torch
    wl = Workload()
    spec = W.PlainLyotSpec()
    B = args.fields
    cor, inp = W.build_plain_lyot(ctx, spec, precision=args.precision,
                                  fft_fpm_babinet=not args.fft_occulter)
    cor.batch_all(1)
    cal = cor.execute(calibrating=True)
    reg = cg.RegionContrast(ctx, cor.n_out, cor.out_pixel, inp["lod_image"], 3.0, 12.0)
    wl.cmax = reg.calibration_max(cal)
    rng = np.random.default_rng(200 + rank)
    lx = spec.n * inp["dx"]
    per_lod = lx / (2.0 * 2.0 * spec.beam_radius)  # tip of one lambda/D
    tips = rng.uniform(-4, 4, (2, B)) * per_lod
    cor.set_batch(np.zeros(B, np.int32), np.ones(B), tips[0], tips[1], np.zeros(B, np.int32))
    _, tip_d, tilt_d = cor.source_buffers()
    wl.per_group = 1
    wl.cor, wl.inp, wl.reg, wl.B, wl.spec = cor, inp, reg, B, spec
    wl.host_in = torch.as_tensor(np.concatenate([tips[0], tips[1]]))
    wl.dev_in = torch.empty(2 * B, dtype=torch.float64, device="cuda")
    wl.dev_split = (tip_d, tilt_d)

    def cpu(budget, nmax):
        from oracle import chain as oc
        t0 = time.perf_counter()
        n = 0
        while n < nmax and time.perf_counter() - t0 < budget:
            oc.plain_lyot_field(inp, spec, 0, 1.0, tips[0][n % B], tips[1][n % B])
            n += 1
        dt = time.perf_counter() - t0
        return n / dt, n, dt
    wl.cpu = cpu
    wl.cpu_sample = "FP64 numpy/scipy: 2048^2 FFT occulter + direct MFT"
    # the occulter's Babinet form runs on the MFT GEMMs; its padded FFT on the FFT passes
    wl.bound = "hbm" if args.fft_occulter else "tensor"
    wl.config = {"workload": "plain-lyot-512: 512^2 pupil (r = 200 px, 0.3 obstruction), "
                             "Zernike 4-15 at 10 nm RMS, 2048^2 FFT, 3 lambda/D occulter, "
                             "Lyot 0.9, 128^2 MFT at 0.25 lambda/D",
                 "fields_per_step": B, "n": spec.n, "pad": spec.pad, "image": cor.n_out,
                 "occulter": ("padded 2048^2 FFT" if args.fft_occulter else
                              "Babinet form: MFT pair over the support box of 1 - mask"),
                 "l2": "working set > L2 (fields 134 MB at 64 fields; padded 2 GB with the "
                       "FFT occulter)"}
    return wl


def setup_broadband(args, ctx, W, cg, rank):
    """Broadband batch: 2048^2 segmented pupil with a 48^2 DM, 11 wavelengths
    x 3 sources = 33 fields in one launch onto ragged 460^2..540^2 grids; the
    sources' offsets are uploaded every step."""
    import torch
    wl = Workload()
    spec = W.BroadbandSpec()
    cor, inp = W.build_broadband(ctx, spec, precision=args.precision)
    B = cor.batch_all(1)
    _, tip_d, tilt_d = cor.source_buffers()
    tips = np.stack([tip_d.cpu().numpy(), tilt_d.cpu().numpy()])
    wl.per_group = B
    wl.cor, wl.inp, wl.reg, wl.B, wl.spec = cor, inp, None, B, spec
    wl.cmax = 1.0
    wl.host_in = torch.as_tensor(np.concatenate([tips[0], tips[1]]))
    wl.dev_in = torch.empty(2 * B, dtype=torch.float64, device="cuda")
    wl.dev_split = (tip_d, tilt_d)
    li, amp, tip, tilt, _ = cor._batch

    def cpu(budget, nmax):
        from oracle import chain as oc
        t0 = time.perf_counter()
        n = 0
        surf = inp["dm_surface"].astype(np.float64)
        while n < nmax and time.perf_counter() - t0 < budget:
            f = n % B
            oc.broadband_field(inp, spec, int(li[f]), amp[f], tip[f], tilt[f], surface=surf)
            n += 1
        dt = time.perf_counter() - t0
        return n / dt, n, dt
    wl.cpu = cpu
    wl.cpu_sample = "FP64 numpy: direct 2048^2 -> n_lambda^2 MFT per field"
    wl.bound = "tensor"
    wl.config = {"workload": "broadband-2048: 6-ring segmented aperture, 48^2 DM, 11 lambda "
                             "(10% at 650 nm) x 3 sources, ragged 460^2..540^2 MFTs in one launch",
                 "fields_per_step": B, "n": spec.n, "image_sizes": inp["n_out"],
                 "precision": f"bf16x{args.precision}",
                 "l2": "working set > L2 (33 x 32 MB fields + MFT operands)"}
    return wl


def setup_de(args, ctx, W, cg, rank):
    """Differential evolution by full propagation: 1261 hexes (20 rings), 5
    wavelengths over a 10% band at 650 nm, population 64, the PIAACMC chain at
    1024^2; one step is one generation (trial generation, 320 propagated
    fields, contrast per candidate, greedy selection) replayed as one CUDA
    graph."""
    import torch
    from csim_gb300 import optimize as opt
    wl = Workload()
    lam = tuple(np.linspace(650e-9 * 0.95, 650e-9 * 1.05, 5))
    spec = W.PiaacmcSpec(n_rings=20, wavelengths=lam, sag_range=0.6e-6)
    P = 64
    cor, inp = W.build_piaacmc(ctx, spec, precision=args.precision, support_crop=not args.no_crop)
    reg = cg.RegionContrast(ctx, cor.n_out, cor.out_pixel, inp["lod_image"], 2.0, 8.0)
    obj = opt.PropagatedObjective(cor, reg, P, use_graph=False)
    cfg = opt.DEConfig(populationSize=P, globalBounds=(-0.6e-6, 0.6e-6),
                       initBounds=(-0.6e-6, 0.6e-6), fWeight=0.7, crossoverProb=0.9,
                       seed=11 + rank)
    de = opt.DifferentialEvolution(ctx, spec.n_hex, cfg)
    de.set_trial_buffer(obj.sags)
    de.initialise(np.zeros(spec.n_hex), 1.0, obj)
    stream = torch.cuda.current_stream()
    wl.gen = opt.GraphedGeneration(de, "deRand1", obj, stream)
    wl.de, wl.obj = de, obj
    wl.cor, wl.inp, wl.reg, wl.B, wl.spec = cor, inp, None, obj.per * P, spec
    wl.per_group = obj.per
    wl.cmax = obj.cmax
    # end to end: the population comes from the host every generation and
    # the objective values go back
    wl.host_in, wl.dev_in = de.pop.cpu(), de.pop
    wl.cpu = None  # the CPU restatement of propagation is the piaacmc workload's baseline
    wl.bound = "tensor"
    wl.config = {"workload": "de-piaacmc-1024: DE/rand/1 (F 0.7, CR 0.9), population 64, "
                             "1261 hexes (20 rings, U(+-0.6um)), 5 lambda (10% at 650 nm), one "
                             "generation = 320 propagated fields + selection, CUDA graph",
                 "fields_per_step": wl.B, "n": spec.n, "n_hex": spec.n_hex, "population": P,
                 "precision": f"bf16x{args.precision}",
                 "l2": "working set > L2 (320 fields x 8 MB)"}
    return wl


def surrogate_experiment(args):
    """Surrogate-screened DE against plain GPU DE on the DE configuration
    (1261 hexes, 5 wavelengths over 10% at 650 nm, the 1024^2 chain,
    population 64, DE/local-to-best/1 with F 0.7, CR 0.9, initial sags within
    +-10 nm of zero as the reference's scripts start, bounds +-0.6 um), on
    optics that admit a deep dark hole (synth.designed_piaacmc_spec). Both
    arms start from the same population and run for the same wall time;
    the screened arm's clock includes its training samples (DE trajectory
    plus random perturbations, all propagated) and training. Reports the
    wall time to each contrast decade of both arms, the surrogate's RMS
    log10 error, and the FP64 oracle's contrast for each arm's best vector."""
    import torch
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import optimize as opt
    from csim_gb300 import surrogate as sg
    from csim_gb300 import workloads as W
    from csim_gb300.runtime import Context
    from csim_gb300.synth import designed_piaacmc_spec
    from oracle import chain as oc
    from oracle import elements as oe
    ctx = Context(0)
    stream = torch.cuda.Stream(0)  # graph capture needs a stream of its own
    ctx.bind_stream(stream)
    with torch.cuda.stream(stream):
        return _surrogate_experiment(args, ctx, torch, cg, opt, sg, W, designed_piaacmc_spec, oc,
                                     oe)


def _surrogate_experiment(args, ctx, torch, cg, opt, sg, W, designed_piaacmc_spec, oc, oe):
    lam = tuple(np.linspace(650e-9 * 0.95, 650e-9 * 1.05, 5))
    spec = designed_piaacmc_spec(n_rings=20, wavelengths=lam, sag_range=0.6e-6)
    cor, inp = W.build_piaacmc(ctx, spec, precision=args.precision)
    reg = cg.RegionContrast(ctx, cor.n_out, cor.out_pixel, inp["lod_image"], 2.0, 8.0)
    P = 64
    obj = sg.PerLambdaObjective(cor, reg, P)
    cfg = opt.DEConfig(populationSize=P, globalBounds=(-0.6e-6, 0.6e-6),
                       initBounds=(-1e-8, 1e-8), fWeight=0.7, crossoverProb=0.9, seed=7)
    strategy = "deLocalToBest1"
    zeros = np.zeros(spec.n_hex)

    plain = opt.DifferentialEvolution(ctx, spec.n_hex, cfg)
    plain.set_trial_buffer(obj.sags)
    plain.initialise(zeros, 1.0, obj)
    f0 = plain.stats()[0]
    h_plain, g_plain = sg.run_plain_de(plain, obj, strategy, args.seconds, 10 ** 9)
    best_plain = plain.stats(True)

    model = sg.ContrastModel(ctx, spec.n_hex, lam, hidden=(1024, 512, 256),
                             features=args.features, seed=3)
    scr = sg.ScreenedDE(ctx, spec.n_hex, cfg, model, draws=args.draws)
    scr.set_trial_buffer(obj.sags)
    scr.initialise(zeros, 1.0, obj)
    assert abs(scr.stats()[0] - f0) <= 1e-12 * abs(f0)  # the same start
    buf = sg.SampleBuffer(max(args.train_samples, 400000), spec.n_hex, lam)
    h_scr, g_scr, info = sg.run_screened_de(
        scr, obj, strategy, args.seconds, 10 ** 9, args.warm_gens, args.train_samples,
        args.epochs, buf, np.random.default_rng(5), cfg.globalBounds, batch=args.train_batch)
    best_scr = scr.stats(True)

    def oracle_cost(vec):
        """FP64 oracle contrast of one sag vector (every wavelength)."""
        fields = [oc.piaacmc_field(inp, spec, lm, 1.0, 0.0, 0.0, vec) for lm in lam]
        cal = [oc.piaacmc_field(inp, spec, lm, 1.0, 0.0, 0.0, vec, calibrating=True)
               for lm in lam]
        full = (np.abs(np.array(fields)) ** 2).sum(0)
        cmax = (np.abs(np.array(cal)) ** 2).sum(0).max()
        return oe.region_contrast(full, np.full_like(full, cmax), reg.mask)

    checks = {}
    for name, (bv, _, _, _, vec) in (("plain", best_plain), ("screened", best_scr)):
        ref = oracle_cost(vec)
        checks[name] = {"gpu": bv, "fp64_oracle": ref, "relative": abs(bv - ref) / ref}
    d_plain, d_scr = sg.decade_times(h_plain), sg.decade_times(h_scr)
    speedup = {k: d_plain[k] / d_scr[k] for k in d_scr if k in d_plain and d_scr[k] > 0}
    line = {
        "metric": "wall time to each dark-hole contrast decade (2-8 lambda/D), plain vs "
                  "surrogate-screened GPU DE",
        "unit": "s", "higher_is_better": False, "n_gpus": 1, "data": "synthetic (seeded)",
        "config": {"workload": "surrogate-de: DE configuration (1261 hexes, 20 rings, 5 lambda "
                               "over 10% at 650 nm, 1024^2 chain, population 64, "
                               "DE/local-to-best/1 F 0.7 CR 0.9, sags start within +-10 nm, "
                               "bounds +-0.6 um) on prolate-apodized optics; MLP "
                               f"{model.n_in}-1024-512-256-1 ({args.features} inputs), "
                               f"{args.draws} draws x 64 screened per generation, top 64 "
                               "propagated",
                   "seconds_per_arm": args.seconds, "precision": args.precision},
        "start_contrast": f0,
        "plain": {"generations": g_plain, "best": best_plain[0], "decades_s": d_plain},
        "screened": {"generations": g_scr, "best": best_scr[0], "decades_s": d_scr, **info},
        "speedup_per_decade": speedup,
        "time_to_1e-10": {"plain": d_plain.get("1e-10"), "screened": d_scr.get("1e-10")},
        "oracle_check": checks,
    }
    print(json.dumps(line))
    return 0


SETUP = {"piaacmc": setup_piaacmc, "plain_lyot": setup_plain_lyot, "broadband": setup_broadband,
         "de": setup_de}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    # 152 fields (candidates) per step: with 152 SMs every MFT GEMM launch is a
    # whole number of persistent-CTA rounds (16, 2, 12, 72, 24 and 8 tiles per
    # field) and every FFT grid a whole number of waves
    ap.add_argument("--fields", type=int, default=152)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="piaacmc", choices=sorted(SETUP) + ["surrogate"],
                    help="piaacmc (headline), plain_lyot, broadband, de, surrogate")
    ap.add_argument("--seconds", type=float, default=60.0,
                    help="surrogate: wall time of each DE arm")
    ap.add_argument("--draws", type=int, default=16, help="surrogate: trial sets per generation")
    ap.add_argument("--warm-gens", type=int, default=300,
                    help="surrogate: plain generations collecting training samples")
    ap.add_argument("--train-samples", type=int, default=200000)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--train-batch", type=int, default=512)
    ap.add_argument("--features", default="sag", choices=["sag", "phasor"])
    ap.add_argument("--precision", type=int, default=6)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--fft-occulter", action="store_true",
                    help="plain_lyot: keep the occulter as a padded 2048^2 FFT instead of its "
                         "Babinet form (the MFT pair over the support of 1 - mask)")
    ap.add_argument("--no-crop", action="store_true",
                    help="transform the whole 512^2 FPM grid instead of the mask's support")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "surrogate":
        return surrogate_experiment(args)

    import torch
    import ctypes as C
    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from csim_gb300 import _lib
    from csim_gb300 import coronagraph as cg
    from csim_gb300 import workloads as W
    from csim_gb300.runtime import Context
    from csim_gb300.sharding import max_over_ranks

    ctx = Context(local)
    stream = torch.cuda.Stream(local)
    ctx.bind_stream(stream)
    with torch.cuda.stream(stream):
        wl = SETUP[args.workload](args, ctx, W, cg, rank)
        cor, B = wl.cor, wl.B
        n_groups = B // wl.per_group
        contrast = torch.zeros(n_groups, dtype=torch.float64, device="cuda")

        def step():
            if hasattr(wl, "gen"):  # one DE generation, replayed as one graph
                wl.gen.replay()
                return wl.de.f
            img = cor.execute(calibrating=False, use_graph=True)
            if wl.reg is not None:
                ctx.region_reduce(img, wl.per_group, wl.reg.pix, mode=0, scale=1.0 / wl.cmax,
                                  out=contrast)
            return img

        for _ in range(args.warmup):
            step()
        ctx.sync()
        # kernels per step, counted on an eager (non-graph) step after the
        # warm-up; graph replays launch exactly these kernels
        n0 = _lib.api["csg_launch_count"]()
        if hasattr(wl, "gen"):
            wl.de.generation("deRand1", wl.obj)
        else:
            img = cor.execute(use_graph=False)
            if wl.reg is not None:
                ctx.region_reduce(img, wl.per_group, wl.reg.pix, mode=0, scale=1.0 / wl.cmax,
                                  out=contrast)
        launches_per_step = _lib.api["csg_launch_count"]() - n0
        ctx.sync()

    hbm_peak, tc_peak, peak_kind = peaks()
    clocks = ClockSampler(local)
    clocks.start()
    # keep the GPU busy while nvidia-smi starts, so its first samples fall
    # under load rather than on an idle GPU
    with torch.cuda.stream(stream):
        t_spin = time.perf_counter()
        while time.perf_counter() - t_spin < 0.5:
            step()
            stream.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms = max_over_ranks(ev0.elapsed_time(ev1), "cuda")
    ctx.sync()
    value = B * args.steps * ws / (ms / 1e3)

    # ---- e2e through the C ABI with host buffers (pinned), every step: H2D
    # of the step's input (the candidates' sags, or the sources' offsets), the
    # walk, the contrast, D2H of the final image fields and the contrasts.
    img0 = step()
    host_in = wl.host_in.pin_memory()
    host_img = torch.empty(img0.shape, dtype=img0.dtype).pin_memory()
    host_con = torch.empty(n_groups, dtype=torch.float64).pin_memory()
    h2d = host_in.numel() * host_in.element_size()
    d2h = host_img.numel() * host_img.element_size() + (n_groups * 8 if wl.reg is not None else 0)
    with torch.cuda.stream(stream):
        def e2e_step():
            _lib.call("csg_memcpy_h2d", ctx.h, C.c_void_p(wl.dev_in.data_ptr()),
                      C.c_void_p(host_in.data_ptr()), h2d)
            if hasattr(wl, "dev_split"):  # tip / tilt halves into the chain's batch
                half = wl.dev_in.numel() // 2
                wl.dev_split[0].copy_(wl.dev_in[:half])
                wl.dev_split[1].copy_(wl.dev_in[half:])
            img = step()
            # pipelined readout: the device-to-host copies run on the
            # context's copy stream while the next step computes
            _lib.call("csg_readout_d2h", ctx.h, C.c_void_p(host_img.data_ptr()),
                      C.c_void_p(img.data_ptr()), host_img.numel() * host_img.element_size())
            if wl.reg is not None:
                _lib.call("csg_readout_d2h", ctx.h, C.c_void_p(host_con.data_ptr()),
                          C.c_void_p(contrast.data_ptr()), n_groups * 8)
        for _ in range(3):
            e2e_step()
        ctx.sync()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        ctx.sync()
        e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, "cuda")
    e2e_value = B * args.steps * ws / e2e_s

    # ---- dominant kernel, timed live with CUDA events on its stream
    with torch.cuda.stream(stream):
        _lib.call("csg_profile", ctx.h, 1)
        for _ in range(3):
            cor.execute(use_graph=False)
        buf = C.create_string_buffer(1 << 16)
        _lib.call("csg_profile_report", ctx.h, buf, len(buf))
        _lib.call("csg_profile", ctx.h, 0)
    prof = json.loads(buf.value.decode())
    tbuf = C.create_string_buffer(1 << 16)
    _lib.call("csg_mft_tuning_log", tbuf, len(tbuf))
    tuning = json.loads(tbuf.value.decode())
    # per-launch kernels only (the fresnel / fft aggregates repeat their passes)
    total_ms = sum(v["ms"] for k, v in prof.items() if k not in ("fresnel_3pass", "fft2d_2pass"))
    kernels = {k: {"count": v["count"], "ms": round(v["ms"], 4),
                   **({"gbs": round(v["bytes"] / v["ms"] / 1e6, 1)} if v["bytes"] else {})}
               for k, v in prof.items()}
    g = prof.get("mft_gemm", {"count": 1, "ms": float("nan"), "flops": 0.0, "bytes": 0.0})
    if wl.bound == "tensor":
        gemm_tflops = g["flops"] / (g["ms"] / 1e3) / 1e12
        roofline = {"bound": "tensor", "kernel": "k_split_gemm (tcgen05 split-bf16 MFT)",
                    "achieved": gemm_tflops, "peak": tc_peak, "unit": "TFLOP/s",
                    "frac": gemm_tflops / tc_peak, "peak_kind": f"{peak_kind} bf16 burst",
                    "traffic": TRAFFIC_PER_FIELD * B if args.workload == "piaacmc" else None,
                    "algorithmic_flops_per_launch": g["flops"] / g["count"],
                    "avg_launch_ms": g["ms"] / g["count"],
                    "executed_bf16_tflops": gemm_tflops * (3 if args.precision == 3 else 6),
                    "share_of_step": g["ms"] / total_ms if total_ms else None}
    else:  # the padded-FFT occulter passes dominate
        fz = prof.get("fresnel_3pass", {"count": 1, "ms": float("nan"), "bytes": 0.0})
        gbs = fz["bytes"] / (fz["ms"] / 1e3) / 1e9
        passes = sum(prof[k]["ms"] for k in prof if k.startswith("fft_"))
        roofline = {"bound": "hbm", "kernel": "k_fft_rows / k_fft_cols (padded-FFT occulter)",
                    "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                    "peak_kind": f"{peak_kind} copy bandwidth", "traffic": None,
                    "algorithmic_bytes_per_launch": fz["bytes"] / fz["count"],
                    "avg_launch_ms": fz["ms"] / fz["count"],
                    "share_of_step": passes / total_ms if total_ms else None}
    roofline["kernels"] = kernels
    roofline["mft_tile_autotune"] = tuning
    if "fresnel_3pass" in prof and wl.bound == "tensor":
        fz = prof["fresnel_3pass"]
        roofline["fresnel_gbs"] = fz["bytes"] / (fz["ms"] / 1e3) / 1e9
        roofline["fresnel_frac_hbm"] = roofline["fresnel_gbs"] / hbm_peak

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu and wl.cpu is not None:
        v, n, dt = wl.cpu(15.0, 32)
        cpu = {"value": v, "unit": "fields/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{n} fields of the same workload in {dt:.1f} s ({wl.cpu_sample})"}

    # the comparator: the plain FP64 GPU path (complex128, one field per call,
    # cuFFT + cuBLAS ZGEMM), a bounded sample on the same inputs
    fp64 = None
    if rank == 0 and ws == 1 and not args.no_cpu and getattr(wl, "fp64", None) is not None:
        v, n, dt = wl.fp64(10.0, 400)
        fp64 = {"value": v, "unit": "fields/s", "sample": f"{n} fields in {dt:.1f} s",
                "speedup": value / v, "e2e_speedup": e2e_value / v,
                "note": "full 512^2 mask grid and 1024^2 pupil transforms"}
        if args.workload == "piaacmc" and not args.no_crop:
            vc, nc, dtc = wl.fp64(10.0, 400, crop=True)
            fp64["with_support_crop"] = {
                "value": vc, "sample": f"{nc} fields in {dtc:.1f} s",
                "speedup": value / vc, "e2e_speedup": e2e_value / vc,
                "note": "the same exact crops as the GPU chain: mask support box and Lyot "
                        "window, so the ratio is precision and batching alone"}

    wl.config["parallelism"] = f"fields sharded over {ws} rank(s)"
    line = {"metric": "field propagations/s", "value": value, "unit": "fields/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": PREC_DTYPE.get(args.precision, str(args.precision)),
            "data": "synthetic (seeded)",
            "config": wl.config,
            "e2e": {"value": e2e_value, "unit": "fields/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches_per_step * args.steps,
            "roofline": roofline, "clocks": clk, "cpu_baseline": cpu}
    if fp64 is not None:
        line["fp64_gpu_path"] = fp64
    if rank == 0 and ws == 1 and args.workload == "piaacmc" and args.precision != 16 \
            and not args.no_cpu:
        line["high_precision"] = high_precision_leg(args, ctx, stream, W, cg, wl, value)
    if wl.reg is not None:
        line["contrast_sample"] = float(contrast[0].item())
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


PREC_DTYPE = {
    6: "f32 fields, bf16x6-split tensor-core MFT, f64 phases",
    3: "f32 fields, bf16x3-split tensor-core MFT, f64 phases",
    16: "f32 fields, exponent-aligned bf16x6 MFT (exact tensor sums, two-float accumulation), "
        "two-float FFT/Fresnel passes, f64 phases, two-float image",
}


def high_precision_leg(args, ctx, stream, W, cg, wl, fast_value):
    """The same PIAACMC workload at CSG_PREC_HIGH: device-timed fields/s over
    the same number of steps, and the final-field error of the first field
    (on-axis, candidate 0) of both modes against the plain FP64 GPU path
    (complex128 cuFFT / ZGEMM, equal to the FP64 oracle to 1e-10),
    peak-normalised to that path's calibration image peak."""
    import copy
    import torch
    from baseline.fp64_gpu import Fp64Piaacmc
    a2 = copy.copy(args)
    a2.precision = 16
    with torch.cuda.stream(stream):
        hw = SETUP["piaacmc"](a2, ctx, W, cg, 0)
        for _ in range(args.warmup):
            hw.cor.execute(calibrating=False, use_graph=True)
        ctx.sync()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            hw.cor.execute(calibrating=False, use_graph=True)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        # field 0 of each mode against the FP64 GPU path
        img_f = wl.cor.execute(calibrating=False, use_graph=False)[0].double()
        img_h = hw.cor.execute(calibrating=False, use_graph=False)[0].double() + \
            hw.cor.image_lo()[0].double()
        ctx.sync()
    ref = Fp64Piaacmc(hw.inp, hw.spec)
    sags0 = hw.host_in[0].to("cuda")
    e_ref = ref.field(0, 1.0, sags0)
    peak = ref.field(0, 1.0, sags0, calibrating=True).abs().max().item()
    err = lambda t: ((torch.complex(t[0], t[1]) - e_ref).abs().max() / peak).item()  # noqa: E731
    value = hw.B * args.steps / (ms / 1e3)
    out = {"value": value, "unit": "fields/s", "ms_per_step": ms / args.steps,
           "relative_to_default": value / fast_value, "dtype": PREC_DTYPE[16],
           "field_error_vs_fp64": {"default": err(img_f), "high": err(img_h),
                                   "normalisation": "calibration image peak, field 0"}}
    hw.cor.close()
    return out


# dram__bytes_read.sum + dram__bytes_write.sum per k_split_gemm launch,
# averaged over the six GEMM launches of one step, per field of the step: an
# ncu capture at 32 fields (1149.1 MB per step), which scales with the field
# count (the 64-field step moved 2 x its traffic).
TRAFFIC_PER_FIELD = 1149.1e6 / 32 / 6

if __name__ == "__main__":
    sys.exit(main())
