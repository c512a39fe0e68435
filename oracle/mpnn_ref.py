"""FP64 CPU restatement of the warm-start network (test infrastructure only).

Same parameter layout, features and loss as the GPU implementation
(onesolver_gb300/csrc/mpnn.cu); optionally rounds the coupling matrix and the
message operands to BF16 at the points where the GPU does, so that GPU
gradients can be compared with it closely. With ``bf16=False`` it is the exact
FP64 network, whose analytic gradient the tests check by finite differences.
"""
from __future__ import annotations

import numpy as np

FEAT = 5
SPEC_RHO_ITERS = 16
SPEC_ITERS = 96


def bf16(a):
    """Round to bfloat16 (round to nearest even), returned as float64."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def layout(H: int, L: int):
    off = {"w_in": 0, "b_in": FEAT * H}
    p = FEAT * H + H
    for l in range(L):
        off[f"ws{l}"] = p
        off[f"wm{l}"] = p + H * H
        off[f"b{l}"] = p + 2 * H * H
        p += 2 * H * H + H
    off["w_out"] = p
    off["b_out"] = p + H
    return off, p + H + 1


def spectral(c: np.ndarray) -> np.ndarray:
    """Feature u of the GPU's spectral feature (onesolver_gb300/csrc/mpnn.cu):
    power iterations on C^ for its spectral radius rho, then on
    (1.05 rho I - C^) from the same start vector; u = sqrt(n) v sign(v_0).
    Here in FP64; the GPU forms the matrix-vector products in FP32 (FP64
    norms), which the tests' tolerances on features and predictions cover."""
    n = c.shape[0]
    i = np.arange(n, dtype=np.uint64)
    v0 = 1.0 + 0.25 * (((i * np.uint64(2654435761)) & np.uint64(0xFFFFFFFF)) >> np.uint64(24)).astype(np.float64) / 255.0
    v = v0 / np.sqrt(np.sum(v0 * v0))
    nrm = 0.0
    for _ in range(SPEC_RHO_ITERS):
        w = c @ v
        nrm = np.sqrt(np.sum(w * w))
        v = w / nrm if nrm > 0 else w * 0.0
    if not nrm > 0:
        return np.zeros(n)
    sigma = 1.05 * nrm
    v = v0 / np.sqrt(np.sum(v0 * v0))
    for _ in range(SPEC_ITERS):
        w = sigma * v - c @ v
        v = w / np.sqrt(np.sum(w * w))
    return np.sqrt(n) * v * (-1.0 if v[0] < 0 else 1.0)


def stage(f: np.ndarray, use_bf16: bool = True):
    """Scaled couplings C^ and node features X, as the GPU stages them."""
    n = f.shape[0]
    up = np.triu(f, 1)
    iu = np.triu_indices(n, 1)
    rms = np.sqrt(np.mean(up[iu] ** 2)) if n > 1 else 0.0
    scale = rms * np.sqrt(n) if rms > 0 else 1.0
    c = (up + up.T) / scale
    c32 = c.astype(np.float32).astype(np.float64)
    c_hat = bf16(c32) if use_bf16 else c
    rowsum = (up + up.T).sum(axis=1)
    x = np.zeros((n, FEAT))
    x[:, 0] = 1.0
    x[:, 1] = np.diag(f) / scale
    x[:, 2] = rowsum / scale
    x[0, 3] = 1.0
    x[:, 4] = spectral(c)
    x = x.astype(np.float32).astype(np.float64)
    return c_hat, x


def orient_label(label, orient: bool = True, u=None):
    """Labels in the orientation that agrees with the spectral feature u
    (sum_i (2 y_i - 1) u_i >= 0), as the GPU orients them; y_0 = 1 decides
    an exact tie or a missing u."""
    y = np.asarray(label, dtype=np.float64)
    if not orient:
        return y
    a = 0.0 if u is None else float(np.sum((2.0 * y - 1.0) * np.asarray(u, dtype=np.float64)))
    if a != 0.0:
        return 1.0 - y if a < 0.0 else y
    return 1.0 - y if y[0] == 0 else y


def loss_grad(params: np.ndarray, f: np.ndarray, label, H: int = 64, L: int = 3, use_bf16: bool = True,
              orient: bool = True):
    """(loss, gradient, probabilities) of the network on one instance."""
    P = np.asarray(params, dtype=np.float64)
    off, total = layout(H, L)
    n = f.shape[0]
    c, x = stage(f, use_bf16)
    y = orient_label(label, orient, x[:, 4])
    q = (lambda a: bf16(a)) if use_bf16 else (lambda a: a)
    W_in = P[off["w_in"]:off["w_in"] + FEAT * H].reshape(FEAT, H)
    b_in = P[off["b_in"]:off["b_in"] + H]
    Zs, Hs, Ms = [], [], []
    Z0 = x @ W_in + b_in
    Hs.append(np.maximum(Z0, 0.0))
    Zs.append(Z0)
    for l in range(L):
        Ws = P[off[f"ws{l}"]:off[f"ws{l}"] + H * H].reshape(H, H)
        Wm = P[off[f"wm{l}"]:off[f"wm{l}"] + H * H].reshape(H, H)
        b = P[off[f"b{l}"]:off[f"b{l}"] + H]
        M = c @ q(Hs[-1])
        Z = Hs[-1] @ Ws + M @ Wm + b
        Ms.append(M)
        Zs.append(Z)
        Hs.append(np.maximum(Z, 0.0))
    w_out = P[off["w_out"]:off["w_out"] + H]
    b_out = P[off["b_out"]]
    z = Hs[-1] @ w_out + b_out
    p = 1.0 / (1.0 + np.exp(-z))
    loss = np.mean(np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))
    G = np.zeros(total)
    dz = (p - y) / n
    G[off["w_out"]:off["w_out"] + H] = Hs[-1].T @ dz
    G[off["b_out"]] = dz.sum()
    dH = np.outer(dz, w_out)
    for l in reversed(range(L)):
        Ws = P[off[f"ws{l}"]:off[f"ws{l}"] + H * H].reshape(H, H)
        Wm = P[off[f"wm{l}"]:off[f"wm{l}"] + H * H].reshape(H, H)
        dZ = dH * (Zs[l + 1] > 0)
        G[off[f"ws{l}"]:off[f"ws{l}"] + H * H] = (Hs[l].T @ dZ).ravel()
        G[off[f"wm{l}"]:off[f"wm{l}"] + H * H] = (Ms[l].T @ dZ).ravel()
        G[off[f"b{l}"]:off[f"b{l}"] + H] = dZ.sum(axis=0)
        dM = dZ @ Wm.T
        dH = dZ @ Ws.T + c @ q(dM)
    dZ0 = dH * (Zs[0] > 0)
    G[off["w_in"]:off["w_in"] + FEAT * H] = (x.T @ dZ0).ravel()
    G[off["b_in"]:off["b_in"] + H] = dZ0.sum(axis=0)
    return float(loss), G, p
