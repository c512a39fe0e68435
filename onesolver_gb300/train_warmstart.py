"""Train the shipped learned warm start and compute its evaluation targets.

Produces onesolver_gb300/data/warmstart_sk1024.npz, the network the library
ships for SK instances with n = 1024 (J_ij ~ N(0, 1/n), the learned-warm-start
configuration), and the yardsticks it is measured against:

1. 4,096 seeded training instances (seeds 0 .. 4095), each labelled with the
   best state that plain batched SA finds on it (64 trajectories x 500
   sweeps, geometric beta 0.1 -> 5.0), 64 instances at a time so that the
   host holds at most 64 matrices;
2. Adam on the oriented labels, by the library's own forward, backward and
   Adam kernels (os_mpnn_train), all 4,096 instances staged on the GPU;
3. for the 256 held-out seeds 10000 .. 10255, the target energy: the best
   energy of plain SA with 10^5 sweeps (geometric beta 0.1 -> 5.0, 64
   trajectories), run as batched anneals of 128 instances.

Everything runs on the GPU through the C ABI; it takes a few minutes on one
GB300. Usage: python -m onesolver_gb300.train_warmstart [--out PATH]
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from . import BatchedAnnealPlan, Context, WarmStartNet, geometric_schedule
from .warmstart import label_states, sk_qubo

DATA = Path(__file__).resolve().parent / "data" / "warmstart_sk1024.npz"
N = 1024
TRAIN_SEEDS = range(0, 4096)
EVAL_SEEDS = range(10000, 10256)


def plain_targets(seeds, *, sweeps: int = 100_000, num_tries: int = 64, chunk: int = 128, seed: int = 97,
                  ctx=None) -> np.ndarray:
    """Best energy of plain SA (sweeps geometric 0.1 -> 5.0) per seed."""
    beta = geometric_schedule(0.1, 5.0, sweeps)
    seeds = list(seeds)
    out = []
    for i in range(0, len(seeds), chunk):
        fs = [sk_qubo(N, s) for s in seeds[i:i + chunk]]
        plan = BatchedAnnealPlan(fs, beta, num_tries=num_tries, resync_every=1000, seed=seed + i, ctx=ctx)
        plan.execute()
        out.extend(r.energy for r in plan.result())
        plan.close()
    return np.asarray(out, dtype=np.float64)


def main(out: Path, epochs: int, lr: float, quick: bool = False) -> None:
    ctx = Context(0)
    train_seeds = range(0, 64) if quick else TRAIN_SEEDS
    eval_seeds = range(10000, 10004) if quick else EVAL_SEEDS
    t0 = time.perf_counter()
    net = WarmStartNet(seed=1, orient=True, ctx=ctx)
    seeds = list(train_seeds)
    for i in range(0, len(seeds), 64):
        fs = [sk_qubo(N, s) for s in seeds[i:i + 64]]
        labels = label_states(fs, num_tries=64, sweeps=500, ctx=ctx)
        for f, y in zip(fs, labels):
            net.add(f, y)
    t_label = time.perf_counter() - t0
    t0 = time.perf_counter()
    hist = net.train(epochs, lr=lr, seed=1)
    t_train = time.perf_counter() - t0
    params = net.params()
    net.close()
    t0 = time.perf_counter()
    targets = plain_targets(eval_seeds, sweeps=1000 if quick else 100_000, ctx=ctx)
    t_target = time.perf_counter() - t0
    meta = {"n": N, "train_seeds": [train_seeds.start, train_seeds.stop], "labels": "plain batched SA, 64 "
            "trajectories x 500 sweeps, geometric beta 0.1 -> 5.0", "epochs": epochs, "lr": lr,
            "hidden": 64, "layers": 3, "orient": True, "eval_seeds": [eval_seeds.start, eval_seeds.stop],
            "targets": "best of plain SA, 64 trajectories x 100,000 sweeps, geometric beta 0.1 -> 5.0",
            "loss_first_last": [float(hist[0]), float(hist[-1])],
            "seconds": {"label": t_label, "train": t_train, "targets": t_target}}
    out.parent.mkdir(parents=True, exist_ok=True)
    np.savez(out, params=params, loss=hist, eval_seeds=np.arange(eval_seeds.start, eval_seeds.stop),
             targets=targets, meta=json.dumps(meta))
    print(json.dumps(meta))
    ctx.close()


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", type=Path, default=DATA)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--quick", action="store_true", help="64 training instances, 4 held-out seeds (smoke run)")
    a = ap.parse_args()
    main(a.out, a.epochs, a.lr, a.quick)
