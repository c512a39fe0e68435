"""The packed exhaustive variant's arithmetic, modelled on the CPU.

The enumeration kernel's packed form (exhaustive_kernels.cuh,
process_item_packed) walks two blocks of 2^G states at once in one 32-bit
register, (E_b + 16384) * 65536 + (E_a + 16384), with plain 32-bit adds of
packed step constants and packed coupling sums, and between block pairs flips
one walked bit with a delta split into per-item sums. The library takes this
form only when the upper-triangle coefficient magnitudes sum to at most
8,000 (choose_variant in exhaustive.cu), so that every state energy stays in
a 16-bit half. This model re-runs those exact steps in numpy (mod 2^32) for
every item of an n = 18 instance and checks every block pair's per-half
minima against a brute-force scan of all 2^18 states, including instances at
the 8,000 limit with all-negative, all-positive and mixed signs.
"""
from __future__ import annotations

import numpy as np
import pytest

G = 10          # inner (unrolled) bits
L = 6           # loop bits per item (LOOP_BITS)
BIAS = 16384
PACK_MAX_ABS = 8000
M32 = 1 << 32


def ctz(t: int) -> int:
    k = 0
    while not (t >> k) & 1:
        k += 1
    return k


def gray(t: int) -> int:
    return t ^ (t >> 1)


def pack2(v: int) -> int:
    return (v * 65537) % M32


def all_energies(q: np.ndarray) -> np.ndarray:
    """E(x) = sum_{i set} q_ii + sum_{i < j, both set} q_ij for every x < 2^n."""
    n = q.shape[0]
    x = ((np.arange(1 << n)[:, None] >> np.arange(n)[None, :]) & 1).astype(np.int64)
    up = np.triu(q, 1)
    return x @ np.diag(q) + ((x @ up) * x).sum(axis=1)


def inner_steps(q: np.ndarray):
    """Bit k, direction and packed constant pack2(kf[t]) of inner steps t = 1 .. 2^G - 1."""
    ks, ups, kp = [], [], []
    for t in range(1, 1 << G):
        k = ctz(t)
        prev = gray(t - 1)
        up = (gray(t) >> k) & 1
        base = int(q[k, k]) + sum(int(q[k, j]) for j in range(G) if j != k and (prev >> j) & 1)
        ks.append(k)
        ups.append(up)
        kp.append(pack2(base if up else -base))
    return np.array(ks), np.array(ups, dtype=bool), np.array(kp, dtype=np.int64)


def packed_item_minima(q: np.ndarray, item: int, steps) -> list[tuple[int, int]]:
    """Per-half minima of every block pair of `item`, by the kernel's packed steps."""
    n = q.shape[0]
    ks, ups, kp = steps
    top = G + L - 1
    W = L - 1
    xa = item << (G + L)
    set_bits = [j for j in range(n) if (xa >> j) & 1]
    Ea = sum(int(q[i, i]) for i in set_bits) + sum(int(q[i, j]) for i in set_bits for j in set_bits if i < j)
    ca = [sum(int(q[j, i]) for j in set_bits) for i in range(G)]
    bw = [int(q[G + w, G + w]) + sum(int(q[j, G + w]) for j in set_bits) for w in range(W)]
    sumt = int(q[top, top]) + sum(int(q[top, j]) for j in set_bits)
    c2 = [((ca[i] + int(q[top, i])) * 65536 + ca[i]) % M32 for i in range(G)]
    E2s = ((Ea + sumt + BIAS) * 65536 + (Ea + BIAS)) % M32
    out = []
    for B in range(1 << W):
        c2a = np.array(c2, dtype=np.int64)
        d = (kp + np.where(ups, c2a[ks], -c2a[ks])) % M32
        E = np.concatenate(([E2s], (E2s + np.cumsum(d)) % M32))
        lo, hi = E & 0xFFFF, E >> 16
        assert lo.min() >= 0 and lo.max() < 32768 and hi.max() < 32768, "a half left its range"
        out.append((int(lo.min()) - BIAS, int(hi.min()) - BIAS))
        if B + 1 < (1 << W):
            w = ctz(B + 1)
            mbit = G + w
            was = (xa >> mbit) & 1
            row = q[mbit]
            walked = ((xa >> G) & ((1 << W) - 1)) & ~(1 << w)
            s = bw[w] + sum(int(row[G + v]) for v in range(W) if (walked >> v) & 1)
            sum2 = (s * 65537 + int(row[top]) * 65536) % M32
            E2s = (E2s - sum2) % M32 if was else (E2s + sum2) % M32
            xa ^= 1 << mbit
            sgn = -65537 if was else 65537
            c2 = [(c2[i] + int(row[i]) * sgn) % M32 for i in range(G)]
    return out


def brute_item_minima(E: np.ndarray, item: int) -> list[tuple[int, int]]:
    top = G + L - 1
    W = L - 1
    out = []
    inner = np.arange(1 << G)
    for B in range(1 << W):
        base = (item << (G + L)) | (gray(B) << G)
        out.append((int(E[base | inner].min()), int(E[base | (1 << top) | inner].min())))
    return out


def symmetric(upper: np.ndarray) -> np.ndarray:
    u = np.triu(upper)
    return u + np.triu(u, 1).T


def at_limit(n: int, sign: int, seed: int) -> np.ndarray:
    """Integer coefficients whose upper-triangle magnitudes sum to exactly
    PACK_MAX_ABS; sign +1 / -1 all alike, 0 random signs."""
    rng = np.random.default_rng(seed)
    iu = np.triu_indices(n)
    m = len(iu[0])
    mags = np.full(m, PACK_MAX_ABS // m, dtype=np.int64)
    mags[rng.permutation(m)[:PACK_MAX_ABS - mags.sum()]] += 1
    signs = np.full(m, sign) if sign else rng.choice([-1, 1], size=m)
    up = np.zeros((n, n), dtype=np.int64)
    up[iu] = mags * signs
    assert np.abs(up[iu]).sum() == PACK_MAX_ABS
    return symmetric(up)


CASES = {
    "uniform8": lambda: symmetric(np.random.default_rng(3).integers(-8, 9, size=(18, 18))),
    "limit_negative": lambda: at_limit(18, -1, 1),
    "limit_positive": lambda: at_limit(18, +1, 2),
    "limit_mixed": lambda: at_limit(18, 0, 3),
}


@pytest.mark.parametrize("case", list(CASES))
def test_packed_walk_minima_match_brute_force(case):
    q = CASES[case]()
    n = q.shape[0]
    E = all_energies(q)
    steps = inner_steps(q)
    for item in range(1 << (n - G - L)):
        assert packed_item_minima(q, item, steps) == brute_item_minima(E, item), (case, item)
