"""The learned warm start: oracle self-check (CPU), GPU gradients against
the FP64 oracle, training, and the gain of a trained warm start over random
initial spins."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import mpnn_ref
from tests.qubo_text import random_normal_qubo


def _params(H, L, seed):
    off, total = mpnn_ref.layout(H, L)
    rng = np.random.default_rng(seed)
    return rng.normal(0.0, 0.3, size=total)


def test_oracle_gradient_matches_finite_differences():
    H, L, n = 8, 2, 7
    f = random_normal_qubo(n, 3)
    label = np.random.default_rng(1).integers(0, 2, size=n)
    P = _params(H, L, 2)
    loss, g, _ = mpnn_ref.loss_grad(P, f, label, H, L, use_bf16=False)
    rng = np.random.default_rng(4)
    for k in rng.choice(P.size, size=40, replace=False):
        e = np.zeros_like(P)
        e[k] = 1e-6
        lp, _, _ = mpnn_ref.loss_grad(P + e, f, label, H, L, use_bf16=False)
        lm, _, _ = mpnn_ref.loss_grad(P - e, f, label, H, L, use_bf16=False)
        num = (lp - lm) / 2e-6
        assert abs(num - g[k]) <= 1e-6 + 1e-4 * abs(num), (k, num, g[k])


def test_orientation_makes_label_flip_invariant():
    f = random_normal_qubo(10, 0)
    P = _params(64, 3, 0)
    lab = np.random.default_rng(0).integers(0, 2, size=10)
    a = mpnn_ref.loss_grad(P, f, lab)
    b = mpnn_ref.loss_grad(P, f, 1 - lab)
    assert a[0] == b[0]


@pytest.mark.gpu
@pytest.mark.parametrize("n", [64, 96, 200])
def test_gpu_loss_and_gradients_match_oracle(native, ctx, n):
    net = native.WarmStartNet(ctx=ctx, seed=3)
    f = random_normal_qubo(n, n)
    label = np.random.default_rng(n).integers(0, 2, size=n)
    idx = net.add(f, label)
    P = net.params().astype(np.float64)
    loss, g = net.loss_grad(idx)
    loss_ref, g_ref, _ = mpnn_ref.loss_grad(P, f, label)
    assert abs(loss - loss_ref) <= 1e-4 * abs(loss_ref)
    off, total = mpnn_ref.layout(64, 3)
    names = ["w_in", "b_in"] + [f"{k}{l}" for l in range(3) for k in ("ws", "wm", "b")] + ["w_out", "b_out"]
    sizes = {"w_in": 4 * 64, "b_in": 64, "w_out": 64, "b_out": 1}
    for name in names:
        size = sizes.get(name, 64 * 64 if name[:2] in ("ws", "wm") else 64)
        a = g[off[name]:off[name] + size].astype(np.float64)
        b = g_ref[off[name]:off[name] + size]
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        assert err < 2e-3, (name, err)
    net.close()


def _field_dominated(n, seed):
    """Instances whose ground state follows the sign of the linear terms:
    strong linear terms, weak couplings."""
    rng = np.random.default_rng(seed)
    u = np.triu(rng.normal(0.0, 0.05, size=(n, n)), 1)
    f = u + u.T
    d = rng.choice([-1.0, 1.0], size=n) * rng.uniform(0.5, 1.5, size=n)
    np.fill_diagonal(f, d)
    label = (d < 0).astype(np.uint8)
    return f, label


@pytest.mark.gpu
def test_shipped_network_beats_fair_coins_on_sk(native, ctx):
    """The shipped network (trained on 4,096 SK n = 1024 instances by
    train_warmstart.py) on held-out SK seeds: short anneals started from its
    predictions end lower than the same anneals from fair coins (same
    schedule, trajectories and Philox seed), and reach the seed's 10^5-sweep
    plain-SA target within 0.5% in 50 sweeps more often."""
    from onesolver_gb300 import warmstart as ws
    sh = ws.load_shipped(ctx)
    beta = native.geometric_schedule(2.0, 5.0, 50)
    warm_hits = cold_hits = 0
    for k in range(6):
        f = ws.sk_qubo(1024, int(sh.eval_seeds[k]))
        thr = sh.targets[k] + 0.005 * abs(sh.targets[k])
        prob = sh.net.predict(f)
        assert np.all((prob > 0) & (prob < 1))
        warm = native.anneal(f, beta, num_tries=512, site_order=1, acceptance=1, init_prob=prob, seed=9,
                             resync_every=-1, ctx=ctx)
        cold = native.anneal(f, beta, num_tries=512, site_order=1, acceptance=1, seed=9, resync_every=-1, ctx=ctx)
        assert warm.traj_energies.mean() < cold.traj_energies.mean(), k
        warm_hits += warm.energy <= thr
        cold_hits += cold.energy <= thr
    assert warm_hits > cold_hits, (warm_hits, cold_hits)
    sh.net.close()


@pytest.mark.gpu
def test_plan_warm_start_equals_host_prediction(native, ctx):
    """os_sa_plan_warm_start (the network on the plan's device-resident
    matrix, probabilities straight into the plan) starts the same trajectories
    as passing the host-path prediction as init_prob."""
    from onesolver_gb300 import warmstart as ws
    sh = ws.load_shipped(ctx)
    f = ws.sk_qubo(1024, int(sh.eval_seeds[0]))
    beta = native.geometric_schedule(2.0, 5.0, 30)
    prob = sh.net.predict(f)
    a = native.AnnealPlan(f, beta, num_tries=256, acceptance=1, init_prob=prob, seed=4, ctx=ctx)
    b = native.AnnealPlan(f, beta, num_tries=256, acceptance=1, seed=4, ctx=ctx)
    b.warm_start(sh.net)
    for p in (a, b):
        p.execute()
    ra, rb = a.result(traj_states=True), b.result(traj_states=True)
    assert np.array_equal(ra.traj_energies, rb.traj_energies)
    assert np.array_equal(ra.traj_states, rb.traj_states)
    a.close(), b.close()
    g = random_normal_qubo(64, 1)
    sp = native.AnnealPlan(native.Csr.from_dense(g), beta, num_tries=8, ctx=ctx)
    with pytest.raises(native.OneSolverError):
        sp.warm_start(sh.net)   # dense plans only
    sp.close()
    sh.net.close()


@pytest.mark.gpu
def test_training_learns_and_warm_start_gains(native, orc, ctx):
    net = native.WarmStartNet(ctx=ctx, seed=7, orient=False)
    for s in range(24):
        f, lab = _field_dominated(128, s)
        net.add(f, lab)
    hist = net.train(epochs=30, lr=3e-3, seed=1)
    assert hist[-1] < 0.5 * hist[0], hist
    # Held-out instance: the predicted probabilities recover the optimum, and
    # a short anneal warm-started from them ends lower than one started from
    # fair coins (same schedule, same seed).
    f, lab = _field_dominated(128, 1000)
    prob = net.predict(f)
    pred = (prob > 0.5).astype(np.uint8)
    assert (pred == lab).mean() > 0.9
    beta = native.geometric_schedule(5.0, 10.0, 2)
    warm = native.anneal(f, beta, num_tries=64, site_order=1, acceptance=1, init_prob=prob, seed=5, ctx=ctx)
    cold = native.anneal(f, beta, num_tries=64, site_order=1, acceptance=1, seed=5, ctx=ctx)
    assert warm.traj_energies.mean() < cold.traj_energies.mean()
    net.close()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1024, 1100])
def test_prediction_at_and_past_the_register_row_matches_oracle(native, ctx, n):
    """The FP32 power iteration (rows of 1,024 and of 1,152 padded
    couplings, past the 1,024 the staged row loads cover in registers) and
    the whole forward pass match the oracle's FP64 restatement."""
    net = native.WarmStartNet(seed=5, ctx=ctx)
    f = random_normal_qubo(n, 11)
    p = net.predict(f)
    _, _, p_ref = mpnn_ref.loss_grad(net.params().astype(np.float64), f, np.zeros(n))
    np.testing.assert_allclose(p, p_ref, atol=5e-3)
    net.close()


@pytest.mark.gpu
def test_predict_graph_matches_oracle_and_follows_parameters(native, ctx):
    """predict() replays one captured graph per size: its probabilities match
    the oracle's forward pass, repeat exactly, follow a size change and read
    the current parameters."""
    net = native.WarmStartNet(seed=3, ctx=ctx)
    fa, fb = random_normal_qubo(96, 5), random_normal_qubo(160, 6)
    for f in (fa, fb, fa):
        p = net.predict(f)
        _, _, p_ref = mpnn_ref.loss_grad(net.params().astype(np.float64), f, np.zeros(f.shape[0]))
        np.testing.assert_allclose(p, p_ref, atol=5e-3)
        assert np.array_equal(net.predict(f), p)
    p1 = net.predict(fa).astype(np.float64)
    P = net.params()
    P[-1] += 1.0  # output bias: every logit moves by +1
    net.set_params(P)
    p2 = net.predict(fa).astype(np.float64)
    logit = lambda q: np.log(q / (1 - q))
    np.testing.assert_allclose(logit(p2) - logit(p1), 1.0, atol=2e-3)
    net.close()
