"""Test helpers: a minimal reader for well-formed .qubo text and seeded
instance generators. Independent of the product parser, so the oracle can be
pinned on its own."""
from __future__ import annotations

import numpy as np


def read_maps(text: str):
    """(n, linear, quadratic) of a well-formed .qubo text; first key wins."""
    lin, quad, used = {}, {}, set()
    for line in text.splitlines():
        s = line.strip()
        if not s or s[0] in "cp":
            continue
        i, j, v = s.split()
        i, j, v = int(i), int(j), float(v)
        if i == j:
            lin.setdefault(i, v)
        else:
            quad.setdefault((i, j), v)
        used.update((i, j))
    return max(used) + 1, lin, quad


def dense_from_text(text: str) -> np.ndarray:
    n, lin, quad = read_maps(text)
    f = np.zeros((n, n))
    for i, v in lin.items():
        f[i, i] = v
    for (i, j), v in quad.items():
        f[i, j] = f[j, i] = v
    return f


def random_int_qubo(n: int, seed: int, lo: int = -8, hi: int = 8) -> np.ndarray:
    """Dense upper-triangular integer QUBO (symmetrised), entries U{lo..hi}."""
    rng = np.random.default_rng(seed)
    u = np.triu(rng.integers(lo, hi + 1, size=(n, n)).astype(np.float64))
    return u + np.triu(u, 1).T


def random_normal_qubo(n: int, seed: int, scale: float = 1.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    u = np.triu(rng.normal(0.0, scale, size=(n, n)))
    return u + np.triu(u, 1).T
