"""Learned warm start of the Jacobi solve: sample recording, training and evaluation.

The reference solves every substep from lambda = 0 (source/incompressibility.cpp:24
recomputes lambda from scratch in each of the solverIterations passes), so a
compressed region needs many Jacobi passes to reach a density-error target.  Here
a small network predicts, from features of a substep's first density pass, the
lambda that the first position update uses:

    features  f0 neighbour count, f1 rho/rho0 - 1, f2 kernel width / radius,
              f3 the plain Jacobi lambda of that pass, f4 velocity divergence /
              density, f5 sum of the lambdas applied to the particle in the
              previous substep (carried through the sort and split/merge),
              f6 the mean of f5 over the particle's neighbours
    target    sum of min(0, lambda) over the first K plain passes of the substep
    network   7 -> 64 -> 64 -> 1 ReLU, BF16 weights, FP32 accumulation (inference
              on tcgen05.mma in the substep, training on mma.sync)

Only the first update changes; the following passes are the plain solve, which
keeps measuring the mean compression error and stops at density_error_target.
The network therefore decides how many passes a substep needs, never the error
the substep ends with.  Two guards bound what the solver takes from it (an
over-relaxation bound and a neighbour minimum); select_warm_start picks the
network and the bound by the pass count on validation scenes, among those that
leave the fluid no more energetic than the plain solve.

Everything runs on the GPU through the C ABI: the substep appends samples to
device buffers (apbf_record_samples), training calls the project's forward /
backward / Adam kernels (apbf_mlp_train_step), inference is fused into the
substep (apbf_set_warm_start).  torch only holds device memory.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path
from typing import Callable

import numpy as np
import torch

from . import _native as N

PARAMS = N.MLP_PARAMS
P_MU, P_IS, P_W1, P_B1, P_W2, P_B2, P_W3, P_B3, P_YS, P_YM, P_OMEGA, P_NMIN = (0, 8, 16, 528, 592, 4688, 4752, 4816,
                                                                             4817, 4818, 4819, 4820)
HIDDEN, FEATURE_SLOTS, FEATURES_USED = 64, 8, 7
FEATURE_NAMES = ("neighbour_count", "density_ratio_minus_1", "kernel_width_over_radius", "plain_lambda",
                 "velocity_divergence", "previous_substep_lambda", "neighbours_previous_substep_lambda")


def _ptr(t: torch.Tensor | None) -> C.c_void_p:
    return C.c_void_p(t.data_ptr() if t is not None else 0)


def _stream() -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class WarmStartNet:
    """FP32 master parameters, Adam moments and the training / inference calls."""

    def __init__(self, device: int = 0, seed: int = 0):
        self.lib = N.load()
        self.device = torch.device(f"cuda:{device}")
        n = C.c_uint32()
        N.check(self.lib.apbf_mlp_param_count(C.byref(n)), "apbf_mlp_param_count")
        if n.value != PARAMS:
            raise RuntimeError(f"library has {n.value} parameters, expected {PARAMS}")
        rng = np.random.default_rng(seed)
        p = np.zeros(PARAMS, np.float32)
        p[P_IS:P_IS + FEATURES_USED] = 1.0
        # He initialisation of the ReLU layers; a small output layer
        p[P_W1:P_B1] = (rng.standard_normal((HIDDEN, FEATURE_SLOTS)) * np.sqrt(2.0 / FEATURES_USED)).ravel()
        p[P_W1:P_B1].reshape(HIDDEN, FEATURE_SLOTS)[:, FEATURES_USED:] = 0.0
        p[P_W2:P_B2] = (rng.standard_normal((HIDDEN, HIDDEN)) * np.sqrt(2.0 / HIDDEN)).ravel()
        p[P_W3:P_B3] = rng.standard_normal(HIDDEN) * np.sqrt(1.0 / HIDDEN) * 0.1
        p[P_YS] = 1.0
        self.params = torch.from_numpy(p).to(self.device)
        self.m = torch.zeros(PARAMS, dtype=torch.float32, device=self.device)
        self.v = torch.zeros_like(self.m)
        self.step = 0
        self._partials = torch.empty(0, dtype=torch.float32, device=self.device)
        self.loss = torch.zeros(1, dtype=torch.float32, device=self.device)

    # ---- normalisation ----
    def set_normalization(self, X: torch.Tensor, T: torch.Tensor) -> None:
        """Feature means / inverse deviations and the target scale from a sample set."""
        Xu = X[:, :FEATURES_USED].double()
        mu = Xu.mean(0)
        sd = Xu.std(0)
        inv = torch.where(sd > 1e-12, 1.0 / sd.clamp_min(1e-12), torch.zeros_like(sd))
        p = self.params
        p[P_MU:P_MU + FEATURE_SLOTS] = 0.0
        p[P_IS:P_IS + FEATURE_SLOTS] = 0.0
        p[P_MU:P_MU + FEATURES_USED] = mu.float()
        p[P_IS:P_IS + FEATURES_USED] = inv.float()
        ys = float(T.double().std())
        p[P_YS] = ys if ys > 0 else 1.0
        p[P_YM] = float(T.double().mean())

    @property
    def omega_max(self) -> float:
        return float(self.params[P_OMEGA].item())

    @omega_max.setter
    def omega_max(self, v: float) -> None:
        """> 0: the solver clamps the learned lambda to [v * lambda, lambda] where the
        plain lambda of the pass is negative (a bounded per-particle over-relaxation)
        and uses 0 elsewhere; 0: the network's lambda as it is."""
        self.params[P_OMEGA] = float(v)

    @property
    def min_neighbors(self) -> float:
        return float(self.params[P_NMIN].item())

    @min_neighbors.setter
    def min_neighbors(self, v: float) -> None:
        """Particles with fewer neighbours keep the plain lambda in the learned update."""
        self.params[P_NMIN] = float(v)

    def normalise_targets(self, T: torch.Tensor) -> torch.Tensor:
        return ((T - self.params[P_YM]) / self.params[P_YS]).contiguous()

    # ---- kernels ----
    def forward(self, X: torch.Tensor) -> torch.Tensor:
        """lambda (physical units) for n feature rows of 8 floats."""
        X = X.contiguous()
        n = X.shape[0]
        out = torch.empty(n, dtype=torch.float32, device=self.device)
        N.check(self.lib.apbf_mlp_forward(_ptr(self.params), _ptr(X), n, _ptr(out), _stream()), "apbf_mlp_forward")
        return out

    def _scratch(self, n: int) -> torch.Tensor:
        f = C.c_uint32()
        N.check(self.lib.apbf_mlp_partials_size(n, C.byref(f)), "apbf_mlp_partials_size")
        if self._partials.numel() < f.value:
            self._partials = torch.empty(f.value, dtype=torch.float32, device=self.device)
        return self._partials

    def train_step(self, X: torch.Tensor, Tn: torch.Tensor, lr: float, over_weight: float = 1.0) -> None:
        """One Adam step on normalised targets; the batch loss lands in self.loss."""
        n = X.shape[0]
        N.check(self.lib.apbf_mlp_train_step(_ptr(self.params), _ptr(self.m), _ptr(self.v), _ptr(self._scratch(n)),
                                             _ptr(X), _ptr(Tn), n, C.c_float(lr), C.c_float(over_weight), self.step,
                                             None, _ptr(self.loss), _stream()), "apbf_mlp_train_step")
        self.step += 1

    def gradient(self, X: torch.Tensor, Tn: torch.Tensor, over_weight: float = 1.0) -> tuple[float, torch.Tensor]:
        """Loss and gradient of the batch, parameters unchanged (lr = 0)."""
        n = X.shape[0]
        g = torch.zeros(PARAMS, dtype=torch.float32, device=self.device)
        m = torch.zeros_like(g)
        v = torch.zeros_like(g)
        N.check(self.lib.apbf_mlp_train_step(_ptr(self.params), _ptr(m), _ptr(v), _ptr(self._scratch(n)),
                                             _ptr(X.contiguous()), _ptr(Tn.contiguous()), n, C.c_float(0.0),
                                             C.c_float(over_weight), 0, _ptr(g), _ptr(self.loss), _stream()),
                "apbf_mlp_train_step")
        return float(self.loss.item()), g

    def fit(self, X: torch.Tensor, T: torch.Tensor, epochs: int = 4, batch: int = 32768, lr: float = 2e-3,
            seed: int = 0, lr_final: float = 2e-4, over_weight: float = 1.0) -> list[float]:
        """Minibatch Adam over (X, T); targets in physical units.  Returns the mean loss of
        each epoch (normalised space).  The learning rate decays geometrically to lr_final.
        over_weight > 1 weighs predictions that push harder than the target by that
        factor (expectile regression), so the learned first update errs on the side of
        the plain solve, which the following passes complete."""
        Tn = self.normalise_targets(T)
        n = X.shape[0]
        gen = torch.Generator(device=self.device)
        gen.manual_seed(seed)
        steps = max(1, epochs * ((n + batch - 1) // batch))
        decay = (lr_final / lr) ** (1.0 / steps) if lr_final > 0 else 1.0
        history = []
        k = 0
        for _ in range(epochs):
            perm = torch.randperm(n, device=self.device, generator=gen)
            acc = torch.zeros(1, dtype=torch.float64, device=self.device)
            nb = 0
            for b0 in range(0, n, batch):
                idx = perm[b0:b0 + batch]
                self.train_step(X[idx].contiguous(), Tn[idx].contiguous(), lr * decay ** k, over_weight)
                acc += self.loss.double()
                nb += 1
                k += 1
            history.append(float(acc.item()) / nb)
        return history

    # ---- persistence ----
    def state(self) -> np.ndarray:
        return self.params.detach().cpu().numpy().copy()

    def load_state(self, p: np.ndarray) -> None:
        p = np.asarray(p, np.float32).ravel()
        if p.size != PARAMS:
            raise ValueError(f"expected {PARAMS} parameters, got {p.size}")
        self.params.copy_(torch.from_numpy(p))

    def save(self, path: str | Path) -> None:
        np.save(Path(path), self.state())

    def load(self, path: str | Path) -> None:
        self.load_state(np.load(Path(path)))


@dataclass
class SampleBuffer:
    """Device buffers that substeps append training samples to."""

    features: torch.Tensor   # (capacity, 8) float32
    targets: torch.Tensor    # (capacity,) float32
    count: torch.Tensor      # (1,) int32, advanced on the device

    @classmethod
    def allocate(cls, capacity: int, device: int = 0) -> "SampleBuffer":
        d = torch.device(f"cuda:{device}")
        return cls(torch.zeros((capacity, FEATURE_SLOTS), dtype=torch.float32, device=d),
                   torch.zeros(capacity, dtype=torch.float32, device=d),
                   torch.zeros(1, dtype=torch.int32, device=d))

    def size(self) -> int:
        return int(self.count.item())

    def view(self) -> tuple[torch.Tensor, torch.Tensor]:
        n = self.size()
        return self.features[:n], self.targets[:n]


def record_rollout(ctx, dt: float, substeps: int, buf: SampleBuffer, iterations: int, every: int = 1,
                   start: int = 0) -> None:
    """Runs `substeps` plain substeps; from substep `start` on, every `every`-th one
    appends one sample per particle to `buf` (target over `iterations` passes)."""
    for s in range(substeps):
        if s >= start and (s - start) % every == 0:
            ctx.record_samples(iterations, buf.features, buf.targets, buf.count)
        ctx.substep(dt)


def density_passes(ctx, dt: float, substeps: int) -> float:
    """Mean density passes per substep over `substeps` substeps (status counter)."""
    ctx.check_status()  # clears the counter
    for _ in range(substeps):
        ctx.substep(dt)
    return ctx.check_status().density_passes / max(substeps, 1)


@dataclass
class ValidationCase:
    """A validation scene for select_warm_start: `make(mode, params)` returns a new
    context at the scene's start with warm-start `mode` (params: a network's
    parameter vector, or None); `before` substeps run uncounted, then `counted`
    substeps are measured."""

    make: Callable
    dt: float
    before: int
    counted: int


def run_case(case: ValidationCase, mode: int, params: torch.Tensor | None = None) -> dict:
    """Runs a validation scene from its start: density passes per counted substep,
    substeps that reached the error target, and at the end the mean squared particle
    speed (twice the kinetic energy per unit mass) and the 99th percentile of the
    particle heights (y, length units: the splash)."""
    ctx = case.make(mode, params)
    for _ in range(case.before):
        ctx.substep(case.dt)
    ctx.check_status()
    for _ in range(case.counted):
        ctx.substep(case.dt)
    info = ctx.check_status()
    n, _ = ctx.lengths()
    view = ctx.fluid_view()
    v = view["velocity"][:n, :3].double()
    e = float((v * v).sum(1).mean().item()) if n else 0.0
    y = view["position"][:n, 1].double() / 262144.0
    h = float(torch.sort(y).values[min(n - 1, int(0.99 * n))].item()) if n else 0.0
    ctx.close()
    return {"passes": info.density_passes / max(case.counted, 1), "converged": int(info.converged_substeps),
            "mean_v2": e, "y_p99": h, "particles": int(n)}


# over-relaxation bounds that select_warm_start compares for every network
OMEGA_CANDIDATES = (1.5, 2.0, 3.0, 4.0, 6.0)


def select_warm_start(nets: dict, cases: list, omegas=OMEGA_CANDIDATES, min_neighbors: float = 16.0,
                      energy_slack: float = 1.05, height_slack: float = 1.25) -> tuple[dict | None, dict]:
    """Chooses a trained network and its over-relaxation bound by validation.

    A learned first update that pushes too hard still meets the density-error
    target (the following passes only correct compression) but leaves the fluid
    with extra kinetic energy: particles move apart faster than the plain solve
    would move them, and thrown-off particles have no neighbours and no error.
    So every candidate (each network of `nets` x each bound of `omegas`) runs each
    validation scene from its start, and is admissible only if all its counted
    substeps reach the target, its final mean squared speed is at most
    `energy_slack` times, and its final 99th-percentile particle height at most
    `height_slack` times, the largest of the plain rules that reached the target in
    every counted substep (the reference Jacobi rule and the projected rule, run
    on the same scenes; with neither, the larger of the two).  Of the admissible
    candidates the one with the fewest density passes per substep, weighted by the
    scenes' particle counts, wins (ties: the smaller bound).  A slack <= 0 drops
    its condition.

    Returns ({"net": key, "omega_max", "min_neighbors", "params": tensor} or None
    when no candidate is admissible — the networks then keep the guards they came
    with — and a table of every run)."""
    guards = {k: (net.omega_max, net.min_neighbors) for k, net in nets.items()}
    plain = []
    for c in cases:
        plain.append({"reference_rule": run_case(c, 0), "projected_rule": run_case(c, N.WARM_PROJECTED)})
    def bound(key, slack):
        out = []
        for c, p in zip(cases, plain):
            conv = [r[key] for r in p.values() if r["converged"] == c.counted]
            ref = max(conv) if conv else max(r[key] for r in p.values())
            out.append(slack * ref if slack > 0 else float("inf"))
        return out

    bounds, hbounds = bound("mean_v2", energy_slack), bound("y_p99", height_slack)
    weights = [max(p["reference_rule"]["particles"], 1) for p in plain]
    table: dict = {"plain": plain, "energy_bound": bounds, "height_bound": hbounds, "candidates": {}}
    best = None
    for key, net in nets.items():
        for om in omegas:
            net.omega_max, net.min_neighbors = om, min_neighbors
            params = net.params.clone()
            runs = [run_case(c, N.WARM_LEARNED | N.WARM_PROJECTED, params) for c in cases]
            ok = all(r["converged"] == c.counted and r["mean_v2"] <= b and r["y_p99"] <= hb
                     for r, c, b, hb in zip(runs, cases, bounds, hbounds))
            score = sum(w * r["passes"] for w, r in zip(weights, runs)) / sum(weights)
            table["candidates"][f"{key} / omega {om:g}"] = {
                "passes": round(score, 3), "admissible": ok,
                "energy_ratio": [round(r["mean_v2"] / max(p["reference_rule"]["mean_v2"], 1e-30), 3)
                                 for r, p in zip(runs, plain)],
                "height_ratio": [round(r["y_p99"] / max(p["reference_rule"]["y_p99"], 1e-30), 3)
                                 for r, p in zip(runs, plain)]}
            if ok and (best is None or (score, om) < (best[0], best[2])):
                best = (score, key, om, params)
    if best is None:
        for k, net in nets.items():
            net.omega_max, net.min_neighbors = guards[k]
        return None, table
    _, key, om, params = best
    nets[key].omega_max, nets[key].min_neighbors = om, min_neighbors
    return {"net": key, "omega_max": om, "min_neighbors": min_neighbors, "params": params}, table
