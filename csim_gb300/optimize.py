"""Optimisation on the GPU: the response-matrix objective (optHexRespObjective),
a fully propagated dark-hole objective, and the differential-evolution driver
(differentialEvolutionOptimizer::optimize) built on the device-resident DE
state of the C ABI.

Populations are candidate-major [pop][nvar] device tensors (the transpose of
the reference's nvar x pop matrices).
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from ._lib import call
from .runtime import Context, ptr


def _view(addr: int, shape, dtype=torch.float64) -> torch.Tensor:
    from .coronagraph import _tensor_from_ptr
    return _tensor_from_ptr(addr, shape, dtype)


class RespObjective:
    """optHexRespObjective (optObjective.cpp:24-69): M matrices for every
    (source, polarization, wavelength) as complex [n_mat][npix][nhex+1]."""

    def __init__(self, ctx: Context, m: np.ndarray, wavelengths, calib: float,
                 phase_sign: float = 1.0, objective: str = "mean"):
        self.ctx = ctx
        m = np.ascontiguousarray(m, dtype=np.complex128)
        if m.ndim == 2:
            m = m[None]
        lam = np.ascontiguousarray(np.broadcast_to(np.asarray(wavelengths, np.float64), (m.shape[0],)))
        h = C.c_void_p()
        call("csg_respobj_create", ctx.h, C.byref(h), m.ctypes.data_as(C.c_void_p), m.shape[0],
             m.shape[1], m.shape[2], lam.ctypes.data_as(C.c_void_p), float(calib),
             float(phase_sign), 0 if objective == "mean" else 1)
        self.h = h
        self.nvar = m.shape[2] - 1

    def __call__(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        pop = x.shape[0]
        if out is None:
            out = torch.empty(pop, dtype=torch.float64, device=x.device)
        call("csg_respobj_execute", self.h, ptr(x), pop, ptr(out))
        return out

    def close(self):
        if self.h:
            call("csg_respobj_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PropagatedObjective:
    """Dark-hole contrast of every candidate by full propagation: the chain
    walks every (candidate, source, wavelength) field and the region mean of
    sum |E|^2 over each candidate's fields is divided by the calibration
    maximum (regionContrast.cpp:124-205). The candidates' sags are the
    chain's sag buffer (`sags`), which the DE state writes its trial vectors
    into."""

    def __init__(self, cor, region, pop: int, use_graph: bool = True):
        self.cor, self.region, self.pop = cor, region, pop
        self.sags = cor.sags(pop)
        self.per = cor.batch_all(pop) // pop
        cal = cor.execute(calibrating=True)
        # calibration normaliser: one candidate's fields carry every (s, lambda)
        self.cmax = region.calibration_max(cal[: self.per].contiguous())
        self.use_graph = use_graph

    def __call__(self, x: torch.Tensor, out: torch.Tensor) -> torch.Tensor:
        if x.data_ptr() != self.sags.data_ptr():
            self.sags.copy_(x)
        img = self.cor.execute(calibrating=False, use_graph=self.use_graph)
        return self.region.ctx.region_reduce(img, self.per, self.region.pix, 0, 1.0 / self.cmax,
                                             out=out)


STRATEGIES = {"deRand1": 0, "deLocalToBest1": 1, "eitherOr": 2}


class GraphedGeneration:
    """One DE generation (trial generation, the objective's launches, greedy
    selection) captured once as a CUDA graph on `stream` and replayed: the
    generation counter and the random streams live on the device, so every
    replay is the next generation. The objective must launch only (no host
    synchronisation or allocation), e.g. PropagatedObjective(use_graph=False)
    writing the trials in place through DifferentialEvolution.set_trial_buffer."""

    def __init__(self, de: "DifferentialEvolution", strategy: str, objective,
                 stream: torch.cuda.Stream):
        from .sharding import ShardedObjective
        if isinstance(objective, ShardedObjective):
            # the per-generation all-gather stays outside captured graphs: a
            # sharded generation runs eager, the chain's own graph replayed
            raise ValueError("a sharded objective runs the eager generation, not a captured one")
        self.de, self.graph = de, torch.cuda.CUDAGraph()
        code = STRATEGIES[strategy]
        cfg = de.cfg

        def body():
            call("csg_de_generate", de.h, code, cfg.fWeight, cfg.crossoverProb)
            objective(de.trial, de.f_trial)
            call("csg_de_select", de.h, 0)
        with torch.cuda.stream(stream):
            body()  # eager warm-up: first-use set-up happens outside the capture
            stream.synchronize()
        with torch.cuda.graph(self.graph, stream=stream):
            body()

    def replay(self):
        self.graph.replay()


@dataclass
class DEConfig:
    """differentialEvolutionOptimizer settings (differentialEvolutionOptimizer.cpp:66-197)."""
    populationSize: int = 64
    startStrategy: str = "deLocalToBest1"
    baseStrategy: str = "eitherOr"
    endStrategy: str = "deLocalToBest1"
    reinitStrategy: str | None = None
    initSpread: float = 1.0
    reinitCompression: float = 0.1
    reinitSpread: float = 1e-12
    globalBounds: tuple = (-5e-7, 5e-7)
    initBounds: tuple = (-1e-8, 1e-8)
    initType: str = "uniformRandom"
    maxIterations: int = 200
    stopObjectiveValue: float = 1e-12
    stopPopulationSpread: float = 0.0
    reinitChangefracThreshold: float = 1e-3
    maxSmallChange: int = 5
    maxRetries: int = 5000000
    fWeight: float = 0.5
    crossoverProb: float = 1.0
    baseStrategySpreadSwitch: float = 1e-7
    endStrategySpreadSwitch: float = 0.0
    outputInterval: int = 100
    seed: int = 1


class DifferentialEvolution:
    """differentialEvolutionOptimizer::optimize (:216-330) driving the device
    DE state. `objective(x, out)` evaluates a [pop][nvar] device population
    into out[pop]. Returns the history of (generation, best value, seconds)."""

    def __init__(self, ctx: Context, nvar: int, cfg: DEConfig, mean: np.ndarray | None = None):
        self.ctx, self.cfg, self.nvar = ctx, cfg, nvar
        h = C.c_void_p()
        call("csg_de_create", ctx.h, C.byref(h), cfg.populationSize, nvar, cfg.seed)
        self.h = h
        ones = np.ones(nvar)
        gl, gh = cfg.globalBounds
        il, ih = cfg.initBounds
        arrs = [np.ascontiguousarray(v * ones) for v in (gl, gh, il, ih)]
        call("csg_de_set_bounds", self.h, *[a.ctypes.data_as(C.c_void_p) for a in arrs])
        self.mean = np.zeros(nvar) if mean is None else np.asarray(mean, np.float64)
        pp, fp, tp, ftp = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        call("csg_de_buffers", self.h, C.byref(pp), C.byref(fp), C.byref(tp), C.byref(ftp))
        P = cfg.populationSize
        self.pop = _view(pp.value, (P, nvar))
        self.f = _view(fp.value, (P,))
        self.trial = _view(tp.value, (P, nvar))
        self.f_trial = _view(ftp.value, (P,))

    def set_trial_buffer(self, buf: torch.Tensor):
        call("csg_de_set_trial_buffer", self.h, ptr(buf))
        self.trial = buf

    def stats(self, with_best=False):
        bv, md, mx = C.c_double(), C.c_double(), C.c_double()
        gen = C.c_ulonglong()
        best = np.empty(self.nvar) if with_best else None
        call("csg_de_stats", self.h, C.byref(bv), C.byref(md), C.byref(mx), C.byref(gen),
             best.ctypes.data_as(C.c_void_p) if with_best else None)
        return bv.value, md.value, mx.value, gen.value, best

    def initialise(self, origin, spread, objective, typ=None):
        typ = (0 if self.cfg.initType == "uniformRandom" else 1) if typ is None else typ
        o = np.ascontiguousarray(origin, np.float64)
        call("csg_de_init", self.h, o.ctypes.data_as(C.c_void_p), float(spread), typ)
        # evaluate the fresh population through the objective's input buffer
        self.trial.copy_(self.pop)
        objective(self.trial, self.f)
        call("csg_de_select", self.h, 1)

    def generation(self, strategy: str, objective):
        call("csg_de_generate", self.h, STRATEGIES[strategy], self.cfg.fWeight,
             self.cfg.crossoverProb)
        objective(self.trial, self.f_trial)
        call("csg_de_select", self.h, 0)

    def optimize(self, objective, max_seconds: float = 1e30, log=None):
        cfg = self.cfg
        strategy = cfg.startStrategy or cfg.baseStrategy or cfg.endStrategy
        reinit = cfg.reinitStrategy or cfg.baseStrategy
        self.initialise(self.mean, cfg.initSpread, objective)
        global_best = math.inf
        global_vec = None
        t0 = time.perf_counter()
        history = []
        it = 0
        retry = 0
        small = 0
        prev_best = 0.0
        sel_base = sel_end = False
        do_reinit = False
        spread_mean = math.inf
        while True:
            bv, spread_mean, spread_max, _, _ = self.stats()
            if bv < global_best:
                global_best, global_vec = bv, self.stats(True)[4]
            if it > 0 and ((it > cfg.maxIterations or bv < cfg.stopObjectiveValue
                            or spread_max < cfg.stopPopulationSpread) or retry > cfg.maxRetries):
                break
            if small >= cfg.maxSmallChange or do_reinit or spread_mean < cfg.reinitSpread:
                strategy = reinit
                call("csg_de_reset_best", self.h)
                self.initialise(global_vec, cfg.reinitCompression * cfg.initSpread, objective,
                                typ=0)
                small, do_reinit = 0, False
                retry += 1
            self.generation(strategy, objective)
            if it % cfg.outputInterval == 0:
                bv, spread_mean, _, _, _ = self.stats()
                if spread_mean < cfg.baseStrategySpreadSwitch and not sel_base:
                    strategy, sel_base, do_reinit = cfg.baseStrategy, True, True
                if spread_mean < cfg.endStrategySpreadSwitch and not sel_end:
                    strategy, sel_end, do_reinit = cfg.endStrategy, True, True
                small = small + 1 if abs((bv - prev_best) / bv) < cfg.reinitChangefracThreshold else 0
                prev_best = bv
                history.append((it, min(bv, global_best), time.perf_counter() - t0))
                if log:
                    log(it, bv, spread_mean)
            it += 1
            if time.perf_counter() - t0 > max_seconds:
                break
        bv, _, _, _, vec = self.stats(True)
        if bv < global_best:
            global_best, global_vec = bv, vec
        history.append((it, global_best, time.perf_counter() - t0))
        return global_best, global_vec, history

    def close(self):
        if self.h:
            call("csg_de_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fd_jacobian(cor, sags0: np.ndarray, dx: float, pix_idx: np.ndarray) -> torch.Tensor:
    """linearOptimizer::compute_jacobian (linearOptimizer.cpp:420-495) with
    the N + 1 propagations batched into one walk: candidate 0 carries sags0,
    candidate i + 1 sags0 with variable i moved by dx. Returns the device
    Jacobian [2 n_base n_pix][N] (FP64): column i = (E_{i+1} - E_0) / dx at the
    region pixels, rows [Re; Im] per base field (sources x wavelengths)."""
    sags0 = np.asarray(sags0, dtype=np.float64)
    n_var = sags0.size
    cand = np.repeat(sags0[None, :], n_var + 1, axis=0)
    cand[np.arange(1, n_var + 1), np.arange(n_var)] += dx
    cor.sags(n_var + 1).copy_(torch.as_tensor(cand))
    cor.batch_all(n_var + 1)
    img = cor.execute()
    n_base = cor.n_fields // (n_var + 1)
    pix = torch.as_tensor(np.ascontiguousarray(pix_idx, np.int32), device="cuda")
    jac = torch.empty((2 * n_base * pix.numel(), n_var), dtype=torch.float64, device="cuda")
    call("csg_fd_jacobian", cor.ctx.h, ptr(img), img.shape[-1], n_base, n_var, ptr(pix),
         pix.numel(), float(dx), ptr(jac))
    return jac
