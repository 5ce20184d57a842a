"""Surrogate-screened differential evolution (no reference counterpart).

A small MLP (``csg_mlp_*``: tcgen05 bf16 GEMMs with fused GELU epilogues,
fp32 Adam) maps a hex-FPM sag vector and a wavelength to the log10
dark-hole contrast at that wavelength. It is trained on samples the GPU
propagator itself produces (random and DE-trajectory sag vectors), and in
``ScreenedDE`` it ranks several DE trial vectors per population member each
generation; only the best-ranked trial of each member is propagated in full
and evaluated by the true objective (plain DE is the fallback: with one draw
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
                 hidden=(1024, 512, 256), max_batch: int = 1024, seed: int = 0,
                 features: str = "phasor", sag_unit: float = 1e-7):
        """features "phasor": cos and sin of every hex phase (2 n_var + 1
        inputs); "sag": the sags themselves in units of sag_unit and the
        wavelength (n_var + 1 inputs). Input widths are padded to 8."""
        self.n_var = n_var
        self.lam = np.asarray(wavelengths, np.float64)
        self.lam0 = float(self.lam.mean())
        self.lam_scale = float(max(self.lam.max() - self.lam.min(), 1e-30) / 2)
        self.mode = 1 if features == "phasor" else 0
        self.sag_scale = phase_sign if self.mode == 1 else sag_unit
        n_in = ((2 * n_var if self.mode == 1 else n_var) + 1 + 7) // 8 * 8
        self.n_in = n_in
        self.net = Surrogate(ctx, n_in, hidden, max_batch, seed)
        self.max_batch = max_batch
        self.mu, self.sigma = 0.0, 1.0  # target standardisation (set by train)

    def _load(self, sags: torch.Tensor, lam: torch.Tensor):
        self.net.features(sags, lam, self.sag_scale, self.lam0, self.lam_scale, mode=self.mode)

    def train(self, sags: torch.Tensor, lam: torch.Tensor, log10c: torch.Tensor, epochs: int,
              batch: int = 256, lr: float = 1e-3, seed: int = 0, restandardise: bool = True):
        """sags [n][n_var] fp64, lam [n] fp64, log10c [n] fp32 (device).
        Targets are standardised (mean, std of this training set, kept when
        restandardise is False, for fine-tuning) so that small contrast
        differences are not lost to bf16 activations. Returns the per-epoch
        mean training loss (in standardised units)."""
        n = sags.shape[0]
        if restandardise:
            self.mu = float(log10c.double().mean().item())
            self.sigma = float(max(log10c.double().std().item(), 1e-12))
        log10c = ((log10c.double() - self.mu) / self.sigma).float()
        g = torch.Generator(device="cuda")
        g.manual_seed(seed)
        hist = []
        for _ in range(epochs):
            perm = torch.randperm(n, device="cuda", generator=g)
            tot = torch.zeros((), dtype=torch.float64, device="cuda")
            cnt = 0
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                self._load(sags[idx].contiguous(), lam[idx].contiguous())
                tot += self.net.train_step(batch, log10c[idx].contiguous(), lr)[0]
                cnt += 1
            hist.append(float(tot.item()) / max(cnt, 1))  # one host sync per epoch
        return hist

    def predict(self, sags: torch.Tensor, lam: torch.Tensor) -> torch.Tensor:
        n = sags.shape[0]
        out = torch.empty(n, dtype=torch.float32, device="cuda")
        for s in range(0, n, self.max_batch):
            e = min(n, s + self.max_batch)
            b = (e - s + 7) // 8 * 8
            if b == e - s:  # whole batch: the inputs as they are
                self._load(sags[s:e].contiguous(), lam[s:e].contiguous())
            else:
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


class PerLambdaObjective:
    """The propagated dark-hole objective (regionContrast.cpp:124-205 over
    every (candidate, source, wavelength) field of the chain) that also keeps
    each field's own contrast: field_c[candidate * per + k] is the region
    mean of that field's |E|^2 over the calibration maximum, and a
    candidate's cost is the sum over its fields (so the cost is the mean over
    the region of sum_fields |E|^2 / calibration max, the PropagatedObjective
    value)."""

    def __init__(self, cor, region, pop: int):
        self.cor, self.region, self.pop = cor, region, pop
        self.sags = cor.sags(pop)
        self.per = cor.batch_all(pop) // pop
        cal = cor.execute(calibrating=True)
        self.cmax = region.calibration_max(cal[: self.per].contiguous())
        self.field_c = torch.empty(pop * self.per, dtype=torch.float64, device="cuda")

    def __call__(self, x: torch.Tensor, out: torch.Tensor) -> torch.Tensor:
        if x.data_ptr() != self.sags.data_ptr():
            self.sags.copy_(x)
        img = self.cor.execute(calibrating=False, use_graph=True)
        self.region.ctx.region_reduce(img, 1, self.region.pix, 0, 1.0 / self.cmax,
                                      out=self.field_c)
        out.copy_(self.field_c.view(self.pop, self.per).sum(1))
        return out


class SampleBuffer:
    """Device ring of (sag vector, wavelength, log10 contrast) samples."""

    def __init__(self, cap: int, n_var: int, wavelengths):
        self.cap, self.n = cap, 0
        self.lam_set = torch.as_tensor(np.asarray(wavelengths, np.float64), device="cuda")
        self.sags = torch.empty((cap, n_var), dtype=torch.float64, device="cuda")
        self.lam = torch.empty(cap, dtype=torch.float64, device="cuda")
        self.logc = torch.empty(cap, dtype=torch.float32, device="cuda")
        self.head = 0

    def add(self, x: torch.Tensor, field_c: torch.Tensor):
        """x [P][n_var]; field_c [P * L] (candidate-major, wavelength fastest)."""
        L = self.lam_set.numel()
        k = field_c.numel()
        rows = torch.arange(k, device="cuda")
        idx = (self.head + rows) % self.cap
        self.sags[idx] = x.repeat_interleave(L, 0)
        self.lam[idx] = self.lam_set.repeat(k // L)
        self.logc[idx] = torch.log10(field_c.clamp_min(1e-30)).float()
        self.head = (self.head + k) % self.cap
        self.n = min(self.cap, self.n + k)

    def recent(self, m: int):
        m = min(m, self.n)
        idx = (self.head - 1 - torch.arange(m, device="cuda")) % self.cap
        return self.sags[idx], self.lam[idx], self.logc[idx]


def decade_times(history, floor: int = -14):
    """{"1e-k": seconds to the first best value <= 10^-k} from (t, best) pairs."""
    out = {}
    for k in range(1, -floor + 1):
        th = 10.0 ** (-k)
        hit = next((t for t, b in history if b <= th), None)
        if hit is not None:
            out[f"1e-{k}"] = hit
    return out


def run_plain_de(de, objective, strategy: str, seconds: float, max_gens: int):
    """Plain GPU DE from de's initial state: (t, best) after every generation."""
    import time
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = [(0.0, de.stats()[0])]
    g = 0
    while g < max_gens and time.perf_counter() - t0 < seconds:
        de.generation(strategy, objective)
        g += 1
        hist.append((time.perf_counter() - t0, de.stats()[0]))
    return hist, g


def run_screened_de(de: "ScreenedDE", objective: PerLambdaObjective, strategy: str,
                    seconds: float, max_gens: int, warm_gens: int, n_train: int, epochs: int,
                    buf: SampleBuffer, rng: np.random.Generator, bounds, retrain_every: int = 100,
                    log=None, batch: int = 512):
    """Surrogate-screened DE, every step on the clock: warm_gens plain
    generations whose trials (all their fields) become training samples,
    random perturbations of the population (log-uniform scales) until
    n_train samples, training, then screened generations (each draws
    de.draws trial sets, ranks every trial with the surrogate and
    propagates each member's best-ranked one) whose propagated trials keep
    feeding the sample buffer, with a one-epoch fine-tune every
    retrain_every generations. Returns the (t, best) history, the number
    of generations, the phase boundaries and the online log10 errors of the
    surrogate on the trials it chose (predicted against propagated)."""
    import time
    P, nvar = de.cfg.populationSize, de.nvar
    model = de.model
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = [(0.0, de.stats()[0])]
    g = 0
    while g < warm_gens and time.perf_counter() - t0 < seconds:
        DifferentialEvolution.generation(de, strategy, objective)
        buf.add(objective.sags, objective.field_c)
        g += 1
        hist.append((time.perf_counter() - t0, de.stats()[0]))
    lo, hi = bounds
    out = torch.empty(P, dtype=torch.float64, device="cuda")
    while buf.n < n_train and time.perf_counter() - t0 < seconds:
        scale = 10.0 ** rng.uniform(-9.5, -7.0, (P, 1))
        x = de.pop + torch.as_tensor(scale, device="cuda") * torch.randn(
            (P, nvar), dtype=torch.float64, device="cuda")
        objective(x.clamp(lo, hi), out)
        buf.add(objective.sags, objective.field_c)
    t_samples = time.perf_counter() - t0
    # 10% of the samples held out to validate the surrogate
    perm = torch.randperm(buf.n, device="cuda")
    n_hold = buf.n // 10
    hold, tr = perm[:n_hold], perm[n_hold:]
    t_gather = time.perf_counter() - t0
    model.train(buf.sags[tr], buf.lam[tr], buf.logc[tr], epochs, batch=batch)
    pred = model.predict(buf.sags[hold], buf.lam[hold])
    rms_hold = float(torch.sqrt(((pred - buf.logc[hold]) ** 2).mean()).item())
    t_train = time.perf_counter() - t0
    hist.append((t_train, de.stats()[0]))
    L = objective.per
    lam_rep = torch.as_tensor(np.tile(model.lam, P), device="cuda")
    online = []
    g2 = 0
    while g < max_gens and time.perf_counter() - t0 < seconds:
        de.generation(strategy, objective)
        buf.add(objective.sags, objective.field_c)
        if g2 % 10 == 0:  # the surrogate's error on the trials it picked
            p = model.predict(objective.sags.repeat_interleave(L, 0), lam_rep)
            online.append(float(torch.sqrt(((p.double() - torch.log10(
                objective.field_c.clamp_min(1e-30))) ** 2).mean()).item()))
        g += 1
        g2 += 1
        if retrain_every and g2 % retrain_every == 0:
            xs, ls, cs = buf.recent(min(buf.n, 20 * retrain_every * P * L))
            model.train(xs, ls, cs, 1, batch=batch, restandardise=False)
        hist.append((time.perf_counter() - t0, de.stats()[0]))
        if log and g2 % 200 == 0:
            log(g, hist[-1])
    return hist, g, {"warm_generations": warm_gens, "samples_s": t_samples,
                     "trained_s": t_train, "n_samples": int(buf.n),
                     "rms_log10_holdout": rms_hold,
                     "rms_log10_online": float(np.mean(online)) if online else None}
