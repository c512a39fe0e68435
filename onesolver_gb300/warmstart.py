"""Learned warm start for simulated annealing: data, training, gate, evaluation.

Workflow (all annealing and all network arithmetic run on the GPU through
the C ABI):

1. ``sk_qubo(n, seed)`` -- Sherrington-Kirkpatrick instances, J_ij ~ N(0, 1/n),
   h = 0, as QUBOs (x = (s + 1) / 2, offset dropped).
2. ``label_states(instances)`` -- the best state plain SA finds on each
   training instance (one batched anneal).
3. ``WarmStartNet.train`` -- Adam on the oriented labels.
4. ``probe_gate`` -- short probe anneals from the predicted probabilities
   and from fair coins; the warm start is used only when it ends lower.
5. ``time_to_target`` -- the sweep budget (and wall time) each method needs to
   come within a relative gap of a target energy.

``load_shipped`` returns the network the library ships for SK n = 1024
(trained by ``python -m onesolver_gb300.train_warmstart`` on 4,096 instances)
with its held-out seeds and their 10^5-sweep plain-SA targets.

Plain random-init SA is both the fallback and the yardstick: targets come from
long plain runs and every comparison uses the same number of trajectories.
"""
from __future__ import annotations

import json
import math
import time
from dataclasses import dataclass, field
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from . import (ACCEPT_PHYSICAL, AnnealPlan, BatchedAnnealPlan, Context, WarmStartNet, anneal, default_context,
               geometric_schedule)


SHIPPED = Path(__file__).resolve().parent / "data" / "warmstart_sk1024.npz"


@dataclass
class Shipped:
    """The network the library ships for SK n = 1024 (train_warmstart.py) and
    its held-out seeds with their 10^5-sweep plain-SA target energies."""
    net: "WarmStartNet"
    meta: dict
    eval_seeds: np.ndarray
    targets: np.ndarray


def load_shipped(ctx: Optional[Context] = None) -> Shipped:
    d = np.load(SHIPPED)
    meta = json.loads(str(d["meta"]))
    net = WarmStartNet(hidden=meta["hidden"], layers=meta["layers"], orient=meta["orient"], ctx=ctx)
    net.set_params(d["params"])
    return Shipped(net, meta, d["eval_seeds"].copy(), d["targets"].copy())


def sk_qubo(n: int, seed: int) -> np.ndarray:
    """SK instance as a QUBO: Q_ij = 4 J_ij (i != j), Q_ii = -2 sum_j J_ij."""
    rng = np.random.default_rng(seed)
    J = np.triu(rng.normal(0.0, 1.0 / math.sqrt(n), size=(n, n)), 1)
    Js = J + J.T
    f = 4.0 * Js
    np.fill_diagonal(f, -2.0 * Js.sum(axis=1))
    return f


def label_states(instances: Sequence[np.ndarray], *, num_tries: int = 64, sweeps: int = 500,
                 beta_min: float = 0.1, beta_max: float = 5.0, seed: int = 11,
                 ctx: Optional[Context] = None, chunk: int = 64) -> list[np.ndarray]:
    """Best state found by plain SA on each instance (batched, `chunk` at a time)."""
    ctx = ctx or default_context()
    beta = geometric_schedule(beta_min, beta_max, sweeps)
    out = []
    for i in range(0, len(instances), chunk):
        part = list(instances[i:i + chunk])
        plan = BatchedAnnealPlan(part, beta, num_tries=num_tries, resync_every=max(1, sweeps // 2), seed=seed + i,
                                 ctx=ctx)
        plan.execute()
        out.extend(r.state.copy() for r in plan.result())
        plan.close()
    return out


def train_net(instances, labels, *, epochs: int = 20, lr: float = 2e-3, seed: int = 1, orient: bool = True,
              ctx: Optional[Context] = None) -> tuple[WarmStartNet, np.ndarray]:
    net = WarmStartNet(seed=seed, orient=orient, ctx=ctx)
    for f, y in zip(instances, labels):
        net.add(f, y)
    hist = net.train(epochs, lr=lr, seed=seed)
    net.clear()
    return net, hist


def sharpen(prob: np.ndarray, temperature: float) -> np.ndarray:
    """sigmoid(logit(p) / temperature): the same per-spin preferences, more
    (temperature < 1) or less decided."""
    p = np.clip(np.asarray(prob, dtype=np.float64), 1e-6, 1 - 1e-6)
    return (1.0 / (1.0 + np.exp(-np.log(p / (1 - p)) / temperature))).astype(np.float32)


@dataclass
class GateResult:
    use_warm: bool
    warm_energy: float             # mean probe energy of the chosen temperature
    cold_energy: float
    temperature: float = 1.0       # sharpening of the kept warm start
    prob: Optional[np.ndarray] = None  # the warm start to use (None: fair coins)


def probe_gate(f: np.ndarray, prob: np.ndarray, *, sweeps: int = 50, num_tries: int = 128, seed: int = 5,
               beta_min: float = 2.0, beta_max: float = 5.0, temperatures: Sequence[float] = (1.0,),
               ctx: Optional[Context] = None) -> GateResult:
    """Short probe anneals with the same schedule, from the predicted
    probabilities (sharpened by each temperature) and from fair coins; the
    warm start with the lowest mean probe energy is kept only if it ends
    lower than fair coins. The default keeps the network's calibrated
    probabilities: sharper starts end the probe lower on average but, with
    less spread between trajectories, take longer to the best-of-T target
    (SK n = 1024: median 85 sweeps at temperature 0.25 against 60 at 1)."""
    beta = geometric_schedule(beta_min, beta_max, sweeps)
    cold = anneal(f, beta, num_tries=num_tries, site_order=1, acceptance=ACCEPT_PHYSICAL, seed=seed + 1, ctx=ctx)
    best = None
    for tau in temperatures:
        p = sharpen(prob, tau)
        warm = anneal(f, beta, num_tries=num_tries, site_order=1, acceptance=ACCEPT_PHYSICAL, init_prob=p,
                      seed=seed, ctx=ctx)
        e = float(warm.traj_energies.mean())
        if best is None or e < best[0]:
            best = (e, tau, p)
    e_cold = float(cold.traj_energies.mean())
    use = best[0] < e_cold
    return GateResult(use, best[0], e_cold, best[1], best[2] if use else None)


@dataclass
class TTT:
    sweeps: Optional[int]          # smallest budget that reached the target (None: never)
    seconds: Optional[float]       # wall time of that run
    energies: dict = field(default_factory=dict)


def time_to_target(f: np.ndarray, target: float, *, rel_gap: float = 0.005, init_prob=None, net=None,
                   budgets: Sequence[int] = (25, 35, 50, 70, 100, 140, 200, 280, 400, 800, 1600),
                   num_tries: int = 512,
                   beta_min: float = 0.1, beta_max: float = 5.0, seed: int = 21,
                   ctx: Optional[Context] = None) -> TTT:
    """Smallest sweep budget whose best energy is within rel_gap of target.
    Each try is one whole anneal through the C ABI (upload, kernels, answer);
    with `net`, the try also predicts the warm start on the device from the
    plan's own matrix (AnnealPlan.warm_start), inside the timed region."""
    thr = target + rel_gap * abs(target)
    res = TTT(None, None)
    for s in budgets:
        beta = geometric_schedule(beta_min, beta_max, s)
        t0 = time.perf_counter()
        if net is not None:
            plan = AnnealPlan(f, beta, num_tries=num_tries, site_order=1, acceptance=ACCEPT_PHYSICAL,
                              resync_every=-1, seed=seed, ctx=ctx)
            plan.warm_start(net)
            plan.execute()
            r = plan.result()
            plan.close()
        else:
            r = anneal(f, beta, num_tries=num_tries, site_order=1, acceptance=ACCEPT_PHYSICAL, init_prob=init_prob,
                       resync_every=-1, seed=seed, ctx=ctx)  # no drift check: every arm only wants its best energy
        dt = time.perf_counter() - t0
        res.energies[s] = r.energy
        if r.energy <= thr:
            res.sweeps, res.seconds = s, dt
            break
    return res
