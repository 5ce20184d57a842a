"""Surrogate-screened differential evolution (no reference counterpart).

A small MLP (``csg_mlp_*``: tcgen05 bf16 GEMMs with fused GELU epilogues,
fp32 Adam) maps a hex-FPM sag vector and a wavelength to the log10
dark-hole contrast at that wavelength. It is trained on samples the GPU
propagator itself produces (random and DE-trajectory sag vectors), and in
``ScreenedDE`` it ranks several DE trial vectors per population member each
generation; only the best-ranked trial of each member is propagated in full
and judged by the true objective (plain DE is the fallback: with one draw
per member it is exactly the reference's DE).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from ._lib import call
from .optimize import STRATEGIES, DifferentialEvolution, _view
from .runtime import Context, ptr


class Surrogate:
    """MLP n_in -> hidden -> 1 on the GPU."""

    def __init__(self, ctx: Context, n_in: int, hidden=(1024, 512, 256), max_batch: int = 1024,
                 seed: int = 0):
        self.ctx, self.n_in, self.max_batch = ctx, n_in, max_batch
        hid = np.ascontiguousarray(hidden, np.int32)
        h = C.c_void_p()
        call("csg_mlp_create", ctx.h, C.byref(h), n_in, hid.size, hid.ctypes.data_as(C.c_void_p),
             max_batch, seed)
        self.h = h
        self.n_layers = hid.size + 1
        self.dims = [n_in] + list(hidden) + [1]
        self._loss = torch.zeros(1, dtype=torch.float32, device="cuda")

    def set_input(self, x: torch.Tensor):
        call("csg_mlp_set_input", self.h, ptr(x), x.shape[0])

    def features(self, sags: torch.Tensor, lam: torch.Tensor, sag_scale: float, lam0: float,
                 lam_scale: float, mode: int = 1):
        call("csg_mlp_features", self.h, ptr(sags), sags.shape[1], ptr(lam), sag_scale, lam0,
             lam_scale, sags.shape[0], mode)

    def forward(self, batch: int, out: torch.Tensor | None = None) -> torch.Tensor:
        if out is None:
            out = torch.empty(batch, dtype=torch.float32, device="cuda")
        call("csg_mlp_forward", self.h, batch, ptr(out))
        return out

    def train_step(self, batch: int, target: torch.Tensor, lr: float) -> torch.Tensor:
        call("csg_mlp_train_step", self.h, batch, ptr(target), float(lr), ptr(self._loss))
        return self._loss

    def param(self, layer: int):
        """(W, b, gW, gb) fp32 device views of one layer."""
        w, b, gw, gb = (C.c_void_p() for _ in range(4))
        call("csg_mlp_param", self.h, layer, C.byref(w), C.byref(b), C.byref(gw), C.byref(gb))
        o, i = self.dims[layer + 1], self.dims[layer]
        f32 = torch.float32
        return (_view(w.value, (o, i), f32), _view(b.value, (o,), f32),
                _view(gw.value, (o, i), f32), _view(gb.value, (o,), f32))

    def close(self):
        if self.h:
            call("csg_mlp_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ContrastModel:
    """Surrogate of the per-wavelength log10 contrast of a sag vector. Its
    inputs are the hex phasors cos, sin(phaseSign 4 pi sag / lambda) of every
    hex and the normalised wavelength: the contrast is a quadratic form in
    those phasors (optObjective.cpp:39-49), which the network learns far more
    easily than from raw sags."""

    def __init__(self, ctx: Context, n_var: int, wavelengths, phase_sign: float = 1.0,
                 hidden=(1024, 512, 256), max_batch: int = 1024, seed: int = 0):
        self.n_var = n_var
        self.lam = np.asarray(wavelengths, np.float64)
        self.lam0 = float(self.lam.mean())
        self.lam_scale = float(max(self.lam.max() - self.lam.min(), 1e-30) / 2)
        self.sag_scale = phase_sign
        n_in = (2 * n_var + 1 + 7) // 8 * 8
        self.net = Surrogate(ctx, n_in, hidden, max_batch, seed)
        self.max_batch = max_batch
        self.mu, self.sigma = 0.0, 1.0  # target standardisation (set by train)

    def _load(self, sags: torch.Tensor, lam: torch.Tensor):
        self.net.features(sags, lam, self.sag_scale, self.lam0, self.lam_scale, mode=1)

    def train(self, sags: torch.Tensor, lam: torch.Tensor, log10c: torch.Tensor, epochs: int,
              batch: int = 256, lr: float = 1e-3, seed: int = 0):
        """sags [n][n_var] fp64, lam [n] fp64, log10c [n] fp32 (device).
        Targets are standardised (mean, std of this training set) so that
        small contrast differences are not lost to bf16 activations. Returns
        the per-epoch mean training loss (in standardised units)."""
        n = sags.shape[0]
        self.mu = float(log10c.double().mean().item())
        self.sigma = float(max(log10c.double().std().item(), 1e-12))
        log10c = ((log10c.double() - self.mu) / self.sigma).float()
        g = torch.Generator(device="cuda")
        g.manual_seed(seed)
        hist = []
        for _ in range(epochs):
            perm = torch.randperm(n, device="cuda", generator=g)
            tot, cnt = 0.0, 0
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                self._load(sags[idx].contiguous(), lam[idx].contiguous())
                loss = self.net.train_step(batch, log10c[idx].contiguous(), lr)
                tot += float(loss.item())
                cnt += 1
            hist.append(tot / max(cnt, 1))
        return hist

    def predict(self, sags: torch.Tensor, lam: torch.Tensor) -> torch.Tensor:
        n = sags.shape[0]
        out = torch.empty(n, dtype=torch.float32, device="cuda")
        for s in range(0, n, self.max_batch):
            e = min(n, s + self.max_batch)
            b = (e - s + 7) // 8 * 8
            sg = torch.zeros((b, self.n_var), dtype=torch.float64, device="cuda")
            lm = torch.full((b,), self.lam0, dtype=torch.float64, device="cuda")
            sg[:e - s] = sags[s:e]
            lm[:e - s] = lam[s:e]
            self._load(sg, lm)
            out[s:e] = self.net.forward(b)[:e - s]
        return out * self.sigma + self.mu

    def predict_cost(self, sags: torch.Tensor) -> torch.Tensor:
        """Predicted broadband cost of each candidate: the sum over the
        wavelengths of 10^(predicted log10 contrast)."""
        P, L = sags.shape[0], self.lam.size
        rep = sags.repeat_interleave(L, 0)
        lam = torch.as_tensor(np.tile(self.lam, P), device="cuda")
        return torch.pow(10.0, self.predict(rep, lam).double()).view(P, L).sum(1)

    def close(self):
        self.net.close()


class ScreenedDE(DifferentialEvolution):
    """DE whose generation draws `draws` independent trial sets (draws x pop
    trial vectors), ranks them with the surrogate and propagates only each
    member's best-ranked trial."""

    def __init__(self, ctx: Context, nvar: int, cfg, model: ContrastModel, draws: int = 16,
                 mean=None):
        super().__init__(ctx, nvar, cfg, mean)
        self.model, self.draws = model, draws
        P = cfg.populationSize
        self._cand = torch.empty((draws, P, nvar), dtype=torch.float64, device="cuda")

    def generation(self, strategy: str, objective):
        for d in range(self.draws):
            call("csg_de_generate_draw", self.h, STRATEGIES[strategy], self.cfg.fWeight,
                 self.cfg.crossoverProb, d)
            self._cand[d].copy_(self.trial)
        P = self.cfg.populationSize
        cost = self.model.predict_cost(self._cand.view(-1, self.nvar)).view(self.draws, P)
        pick = cost.argmin(0)
        self.trial.copy_(self._cand[pick, torch.arange(P, device="cuda")])
        objective(self.trial, self.f_trial)
        call("csg_de_select", self.h, 0)
