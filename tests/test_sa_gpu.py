"""Simulated annealing on the GPU against the oracle.

* Philox: the device generator against the published algorithm (oracle).
* Verification mode: with the same precomputed (init, site, u) arrays, the
  GPU and the oracle's transcription of annealing.hpp:87-125 must produce
  bit-identical spin trajectories (integer coefficients).
* Free-running mode: every returned state is re-scored in FP64 and must match
  the reference's energy function within 1e-9 relative; energy distributions
  are compared with the oracle's free-running reference algorithm by a
  two-sample Kolmogorov-Smirnov test.
"""
from __future__ import annotations

import numpy as np
import pytest
from scipy import stats

from tests.qubo_text import dense_from_text, random_int_qubo, random_normal_qubo

pytestmark = pytest.mark.gpu

REL = 1e-9


def test_philox_matches_published_algorithm(native, orc, ctx):
    ctr, key = [7, 11, 13, 0x20000001], [0xDEADBEEF, 12345]
    dev = native.philox_sample(ctr, key, 64, ctx=ctx)
    for i in range(64):
        assert dev[i].tolist() == orc.philox([ctr[0] + i, ctr[1], ctr[2], ctr[3]], key)


def _verify_inputs(n, T, steps, seed):
    rng = np.random.default_rng(seed)
    init = rng.integers(0, 2, size=(T, n)).astype(np.uint8)
    site = rng.integers(0, n, size=(T, steps)).astype(np.int32)
    u = rng.random(size=(T, steps))
    return init, site, u


@pytest.mark.parametrize("n,spb,acceptance", [(5, 1, 0), (17, 3, 0), (40, 1, 1), (64, 2, 0), (100, 1, 1)])
def test_verification_mode_bit_identical(native, orc, ctx, n, spb, acceptance):
    T, iters = 24, 300
    f = random_int_qubo(n, n + spb, -4, 4)
    beta = orc.schedule_geometric(0.1, 3.0, iters)
    init, site, u = _verify_inputs(n, T, iters * spb, n)
    g = native.sa_verify(f, beta, init, site, u, sweeps_per_beta=spb, acceptance=acceptance, ctx=ctx)
    bs, be, fs, fe, ac = orc.anneal_verify(f, beta, init, site, u, spb, acceptance)
    assert np.array_equal(g.final_states, fs)
    assert np.array_equal(g.best_states, bs)
    assert np.array_equal(g.final_energies, fe)
    assert np.array_equal(g.best_energies, be)
    assert np.array_equal(g.accept_count, ac)
    assert ac.sum() > 0


def test_verification_mode_reference_schedule_shapes(native, orc, ctx):
    # The CLI's linear schedule rises to beta_min + beta_max and the
    # reference rule divides by beta (it heats up): the transcription must
    # follow it anyway.
    n, T, iters = 12, 8, 200
    f = random_int_qubo(n, 3)
    beta = orc.schedule_linear(0.1, 1.0, iters)
    init, site, u = _verify_inputs(n, T, iters, 1)
    g = native.sa_verify(f, beta, init, site, u, ctx=ctx)
    bs, be, fs, fe, ac = orc.anneal_verify(f, beta, init, site, u, 1, 0)
    assert np.array_equal(g.final_states, fs) and np.array_equal(g.best_energies, be)


def test_energy_batch_is_reference_bit_exact(native, orc, ctx):
    f = random_normal_qubo(70, 2)
    states = np.random.default_rng(0).integers(0, 2, size=(200, 70)).astype(np.uint8)
    assert np.array_equal(native.energy_batch(f, states, ctx=ctx), orc.energy_batch(f, states))


def _ks(a, b):
    """Two-sample KS test on energies compared at the re-score tolerance:
    values of `a` within REL of a value of `b` take that value, so ground
    states found by both sides count as the same energy."""
    a = np.asarray(a, dtype=np.float64).copy()
    ub = np.unique(np.asarray(b, dtype=np.float64))
    idx = np.clip(np.searchsorted(ub, a), 1, len(ub) - 1) if len(ub) > 1 else np.zeros(len(a), dtype=int)
    for cand in (idx - 1, idx):
        c = ub[np.clip(cand, 0, len(ub) - 1)]
        close = np.abs(a - c) <= REL * np.abs(c)
        a[close] = c[close]
    return stats.ks_2samp(a, b)


def _rescore_ok(orc, f, res):
    e = orc.energy_batch(f, res.traj_states)
    np.testing.assert_allclose(res.traj_energies, e, rtol=REL, atol=0)
    assert res.energy == res.traj_energies.min()
    assert orc.energy(f, res.state) == pytest.approx(res.energy, rel=REL, abs=0)


@pytest.mark.parametrize("site_order,acceptance", [(0, 0), (0, 1), (1, 0), (1, 1)])
@pytest.mark.parametrize("n", [7, 33, 64, 200])
def test_returned_states_rescore(native, orc, ctx, n, site_order, acceptance):
    f = random_normal_qubo(n, n)
    beta = native.geometric_schedule(0.1, 3.0, 60)
    res = native.anneal(f, beta, num_tries=50, site_order=site_order, acceptance=acceptance, seed=3,
                        resync_every=20, ctx=ctx, traj_states=True)
    _rescore_ok(orc, f, res)
    assert res.max_field_drift < 1e-3
    steps = 60 * (n if site_order == 1 else 1)
    assert res.attempts == 50 * steps


@pytest.mark.parametrize("n,T", [(100, 300), (200, 37), (1024, 130)])
def test_integer_instance_has_zero_field_drift(native, orc, ctx, n, T):
    """Integer couplings: the tensor-core initial fields (three BF16 terms,
    FP32 accumulation) and every FP32 field update are exact, so the FP64
    resyncs find no drift at all; the states re-score like any other."""
    f = random_int_qubo(n, 7)
    beta = native.geometric_schedule(0.2, 3.0, 24)
    res = native.anneal(f, beta, num_tries=T, site_order=1, acceptance=1, resync_every=6, seed=4, ctx=ctx,
                        traj_states=True)
    assert res.max_field_drift == 0.0
    _rescore_ok(orc, f, res)


def test_reference_config_n64(native, orc, ctx):
    """N=64 dense FP64 QUBO, N(0,1) entries from seed 0, num-tries=100,
    num-iter=100, geometric beta 0.1 -> 1.0, the reference's semantics
    (random sites, exp((E - E') / beta) > u)."""
    f = random_normal_qubo(64, 0)
    beta = native.geometric_schedule(0.1, 1.0, 100)
    res = native.anneal(f, beta, num_tries=100, ctx=ctx, traj_states=True)
    _rescore_ok(orc, f, res)
    assert res.attempts == 100 * 100


@pytest.mark.parametrize("site_order,acceptance", [(0, 0), (1, 1)])
def test_energy_distribution_matches_oracle(native, orc, ctx, site_order, acceptance):
    n, T = 24, 600
    f = random_normal_qubo(n, 42)
    iters = 40
    beta = native.geometric_schedule(0.2, 4.0, iters)
    spb = 3
    res = native.anneal(f, beta, num_tries=T, sweeps_per_beta=spb, site_order=site_order,
                        acceptance=acceptance, seed=11, ctx=ctx)
    _, e_ref, _ = orc.anneal_free(f, beta, T, spb, seed=99, acceptance=acceptance, site_order=site_order)
    ks = _ks(res.traj_energies, e_ref)
    assert ks.pvalue > 1e-3, (ks, res.traj_energies.mean(), e_ref.mean())


def test_warm_start_bias(native, orc, ctx):
    # With init_prob = the ground state and zero temperature steps the anneal
    # stays there.
    f = random_int_qubo(16, 5)
    e_min, s_min = orc.exhaustive(f)
    prob = np.array([(s_min >> i) & 1 for i in range(16)], dtype=np.float32)
    beta = np.full(5, 1e9)
    res = native.anneal(f, beta, num_tries=8, site_order=1, acceptance=1, init_prob=prob, ctx=ctx)
    assert res.energy == e_min


def test_no_resync_mode(native, orc, ctx):
    """resync_every = -1: no FP64 resync at all (drift reported as -1), the
    same trajectories as with a final resync, states still re-scored."""
    f = random_normal_qubo(96, 4)
    beta = native.geometric_schedule(0.2, 3.0, 30)
    a = native.anneal(f, beta, num_tries=40, site_order=1, acceptance=1, resync_every=-1, seed=9, ctx=ctx,
                      traj_states=True)
    b = native.anneal(f, beta, num_tries=40, site_order=1, acceptance=1, resync_every=0, seed=9, ctx=ctx,
                      traj_states=True)
    assert a.max_field_drift == -1.0 and b.max_field_drift >= 0.0
    assert np.array_equal(a.traj_energies, b.traj_energies)
    _rescore_ok(orc, f, a)
    with pytest.raises(native.OneSolverError):
        native.anneal(f, beta, resync_every=-2, ctx=ctx)


def test_plan_api_and_launch_count(native, orc, ctx):
    f = random_normal_qubo(96, 1)
    beta = native.linear_schedule(0.1, 2.9, 50)
    plan = native.AnnealPlan(f, beta, num_tries=64, resync_every=10, ctx=ctx)
    plan.execute()
    r1 = plan.result(traj_states=True)
    plan.execute()
    r2 = plan.result(traj_states=True)
    assert np.array_equal(r1.traj_energies, r2.traj_energies)  # same seed: deterministic
    # initial spins, fields (tensor cores) and energies; 5 x (sweeps, resync); unpack, re-score
    assert plan.launches == 3 + 2 * 5 + 2
    _rescore_ok(orc, f, r1)
    plan.close()


def test_invalid_parameters(native, ctx):
    f = random_normal_qubo(8, 0)
    with pytest.raises(native.OneSolverError):
        native.anneal(f, [], ctx=ctx)
    with pytest.raises(native.OneSolverError):
        native.anneal(f, [1.0], num_tries=0, ctx=ctx)
    with pytest.raises(native.OneSolverError):
        native.anneal(np.zeros((2049, 2049)), [1.0], ctx=ctx)
    for i, j in ((2, 5), (3, 3)):
        g = f.copy()
        g[i, j] = np.nan
        with pytest.raises(native.OneSolverError, match="non-finite"):
            native.anneal(g, [1.0], ctx=ctx)
    g = f.copy()
    g[6, 1] = np.inf  # below the diagonal: the reference reads the upper triangle only
    native.anneal(g, [1.0], ctx=ctx)
    with pytest.raises(native.OneSolverError):
        native.sa_verify(f, [1.0], np.zeros((1, 8), np.uint8), np.full((1, 1), 8, np.int32), np.zeros((1, 1)),
                         ctx=ctx)


# ---------------------------------------------------------------------------
# Sparse (Chimera) path
# ---------------------------------------------------------------------------

def chimera_ising(L: int, seed: int):
    """L x L Chimera of K4,4 cells (8 L^2 spins) with J in {-1, +1}, h = 0,
    converted to QUBO: Q_ij = 4 J_ij, Q_ii = -2 sum_j J_ij (offset dropped),
    the mapping of benchmarks/annealing/scripts/convert_qbsolv_to_coo.py."""
    rng = np.random.default_rng(seed)
    n = 8 * L * L
    edges = []

    def idx(r, c, side, k):
        return ((r * L + c) * 8) + side * 4 + k

    for r in range(L):
        for c in range(L):
            for a in range(4):
                for b in range(4):
                    edges.append((idx(r, c, 0, a), idx(r, c, 1, b)))
            if r + 1 < L:
                for k in range(4):
                    edges.append((idx(r, c, 0, k), idx(r + 1, c, 0, k)))
            if c + 1 < L:
                for k in range(4):
                    edges.append((idx(r, c, 1, k), idx(r, c + 1, 1, k)))
    J = rng.choice([-1.0, 1.0], size=len(edges))
    f = np.zeros((n, n))
    for (i, j), v in zip(edges, J):
        a, b = min(i, j), max(i, j)
        f[a, b] += 4 * v
        f[b, a] += 4 * v
        f[a, a] -= 2 * v
        f[b, b] -= 2 * v
    return f


def test_sparse_matches_rescore_and_dense_statistics(native, orc, ctx):
    f = chimera_ising(3, 0)  # 72 spins
    csr = native.Csr.from_dense(f)
    beta = native.linear_schedule(0.1, 2.9, 30)
    rs = native.anneal_sparse(csr, beta, num_tries=400, sweeps_per_beta=2, resync_every=16, seed=5,
                              ctx=ctx, traj_states=True)
    _rescore_ok(orc, f, rs)
    assert rs.max_field_drift < 1e-4
    assert rs.attempts == 400 * 60 * 72
    rd = native.anneal(f, beta, num_tries=400, sweeps_per_beta=2, site_order=1, acceptance=1, seed=6, ctx=ctx)
    # Same Markov chain family (sequential sweeps in different site orders):
    # final best-energy distributions agree.
    ks = _ks(rs.traj_energies, rd.traj_energies)
    assert ks.pvalue > 1e-3, ks


def test_sparse_energy_distribution_matches_oracle(native, orc, ctx):
    f = chimera_ising(2, 3)  # 32 spins
    csr = native.Csr.from_dense(f)
    beta = native.geometric_schedule(0.2, 3.0, 25)
    plan = native.AnnealPlan(csr, beta, num_tries=500, acceptance=1, seed=2, ctx=ctx)
    try:
        plan.execute()
        rs = plan.result()
        order = plan.sweep_order()
    finally:
        plan.close()
    # The oracle's chain in the kernel's colour-sorted sweep order, with the
    # kernel's sweep-end best-state bookkeeping: the same Markov chain.
    _, e_ref, _ = orc.anneal_free_fields(f, beta, 500, 1, seed=8, acceptance=1, site_order=1, order=order,
                                         best_at_sweep_end=True)
    ks = _ks(rs.traj_energies, e_ref)
    assert ks.pvalue > 1e-3, ks


def test_chimera_droplet_fixture_beats_published_sa(native, orc, ctx, golden_chimera):
    """benchmarks/annealing: the published best SA energy on droplet 128/001
    (best of 1,200 reference runs) is -221.573; the tensor-network ground
    state is -235.867."""
    g = golden_chimera["128"]
    from tests.conftest import GOLDEN
    m = native.Model.load(GOLDEN / g["file"])
    f = m.flatten()
    csr = native.Csr.from_dense(f)
    beta = native.geometric_schedule(0.1, 10.0, 200)
    res = native.anneal_sparse(csr, beta, num_tries=256, sweeps_per_beta=5, resync_every=256, acceptance=1,
                               seed=1, ctx=ctx, traj_states=True)
    _rescore_ok(orc, f, res)
    assert res.energy <= g["published_best_sa"]
    assert res.energy >= g["tn_ground_qubo"] - 1e-6


def test_sparse_rejects_bad_csr(native, ctx):
    csr = native.Csr.from_dense(chimera_ising(1, 0))
    bad = native.Csr(csr.n, csr.row_ptr.copy(), csr.col.copy(), csr.val.copy(), csr.diag.copy())
    bad.val[0] += 1.0  # breaks symmetry
    with pytest.raises(native.OneSolverError):
        native.anneal_sparse(bad, [1.0], ctx=ctx)


# ---------------------------------------------------------------------------
# Batched (many instances, one persistent launch per chunk, CUDA graph)
# ---------------------------------------------------------------------------

def _batch_instances():
    sizes = (40, 64, 100, 130, 33, 257)
    return [random_normal_qubo(n, 100 + n, scale=1.0 / np.sqrt(n)) for n in sizes]


def test_batched_rescore_and_statistics(native, orc, ctx):
    fs = _batch_instances()
    beta = native.geometric_schedule(0.1, 5.0, 40)
    rs = native.anneal_batched(fs, beta, num_tries=160, resync_every=16, ctx=ctx, traj_states=True)
    assert len(rs) == len(fs)
    for f, r in zip(fs, rs):
        _rescore_ok(orc, f, r)
        assert r.attempts == 160 * 40 * f.shape[0]
        assert r.max_field_drift < 1e-4
        single = native.anneal(f, beta, num_tries=160, site_order=1, acceptance=1, resync_every=16, seed=77,
                               ctx=ctx)
        ks = _ks(r.traj_energies, single.traj_energies)
        assert ks.pvalue > 1e-3, (f.shape[0], ks)


def test_batched_plan_graph_replay_and_autotune(native, orc, ctx):
    fs = _batch_instances()[:4]
    beta = native.geometric_schedule(0.1, 3.0, 24)
    plan = native.BatchedAnnealPlan(fs, beta, num_tries=64, resync_every=8, ctx=ctx)
    assert plan.warps in (4, 8, 16)
    plan.execute()
    r1 = plan.result(traj_states=True)
    plan.execute()  # replays the captured graph
    r2 = plan.result(traj_states=True)
    for a, b, f in zip(r1, r2, fs):
        assert np.array_equal(a.traj_energies, b.traj_energies)
        assert np.array_equal(a.traj_states, b.traj_states)
        _rescore_ok(orc, f, a)
    assert plan.kernel_ms() > 0
    plan.close()


def test_batched_rejects_random_order(native, ctx):
    with pytest.raises(native.OneSolverError):
        arr, fs = native._batch_inputs(_batch_instances()[:2])
        b = np.ascontiguousarray([1.0])
        prm = native._sa_params(b, 1, 8, 1, 1, native.SITES_RANDOM, 0, None)
        res, keeps = native._batch_results(fs, 8, False)
        native._check(native.lib().os_sa_run_batched(ctx.handle, len(fs), arr, native.C.byref(prm), res))
