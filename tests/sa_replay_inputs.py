"""Randoms for the annealing replay tests.

The kernels test an attempt as dE < threshold (FP32); the reference tests
new_energy < current_energy || exp((current_energy - new_energy) / beta) > u
(annealing.hpp:106-108), or exp(-beta dE) > u under the physical rule. With
threshold = -beta ln u (reference rule) or -ln(u) / beta (physical rule) the
two agree for every integer dE as long as the threshold is not within
rounding of an integer, so uniforms whose threshold lies within 1e-3 of one
are drawn again. Thresholds stay below 2^13 in magnitude, where FP32 rounds
by less than 5e-4, so the FP32 threshold sits on the same side of every
integer as the exact one.
"""
from __future__ import annotations

import numpy as np


def thresholds(u: np.ndarray, beta_per_step: np.ndarray, acceptance: int) -> np.ndarray:
    """FP64 thresholds of uniforms u ([T, S] or [T, S, n]) at the step's beta."""
    b = beta_per_step.reshape((1, -1) + (1,) * (u.ndim - 2))
    lu = np.log(u)
    return -b * lu if acceptance == 0 else -lu / b


def replay_randoms(rng: np.random.Generator, beta: np.ndarray, sweeps_per_beta: int, T: int, n: int,
                   acceptance: int, sequential: bool = True):
    """(u, thr32): uniforms in (0, 1) for every attempt and the FP32
    thresholds the kernels use, shape [T, S, n] for sequential sweeps and
    [T, S] for random sites (S = len(beta) * sweeps_per_beta)."""
    bs = np.repeat(np.asarray(beta, dtype=np.float64), sweeps_per_beta)
    S = len(bs)
    shape = (T, S, n) if sequential else (T, S)
    u = rng.random(shape)
    for _ in range(1000):
        u = np.where(u <= 0.0, 0.5, u)
        thr = thresholds(u, bs, acceptance)
        bad = (np.abs(thr - np.round(thr)) < 1e-3) | (np.abs(thr) >= 8192.0)
        if not bad.any():
            return u, thr.astype(np.float32)
        u[bad] = rng.random(int(bad.sum()))
    raise RuntimeError("could not draw tie-free thresholds")


def random_sites(rng: np.random.Generator, T: int, S: int, n: int) -> np.ndarray:
    return rng.integers(0, n, size=(T, S)).astype(np.int32)
