"""Bit-exact replay of the production annealing kernels (GPU).

Every dense, sparse and batched plan can run in replay mode
(os_sa_plan_set_replay): the caller's initial spins and per-attempt
thresholds replace the Philox draws, and everything else is the production
path -- the staged-tile, read-only-row, random-site, colour-parallel and
batched persistent sweep kernels, their ballot rounds, field updates, energy
and best-state bookkeeping, the tensor-core field initialisation and the FP64
resyncs. On integer coefficients the FP32 fields and energies are exact, so
the final spins, best spins, tracked energies and accepted-flip counts must
equal the oracle's transcription of the reference's Metropolis loop
(annealing.hpp:97-123, orc_sa_replay) run in the kernel's site order, bit for
bit, under both acceptance rules.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests.qubo_text import random_int_qubo
from tests.sa_replay_inputs import random_sites, replay_randoms

pytestmark = pytest.mark.gpu


def schedule(acceptance: int, num_iter: int) -> np.ndarray:
    # Hot to cold under each rule (the reference rule's beta acts as a
    # temperature): a mix of accepted uphill, accepted downhill and rejected
    # attempts at these coefficient scales.
    return np.geomspace(40.0, 1.0, num_iter) if acceptance == 0 else np.geomspace(0.02, 1.0, num_iter)


def check_same(got, ref):
    fs, bs, fe, be, ac = ref
    assert np.array_equal(got.accepted.astype(np.int64), ac), "accepted flips"
    assert np.array_equal(got.final_states, fs), "final spins"
    assert np.array_equal(got.energies, fe), "tracked energies"
    assert np.array_equal(got.best_states, bs), "best spins"
    assert np.array_equal(got.best_energies, be), "best energies"
    assert ac.sum() > 0


def dense_replay(native, orc, ctx, f, *, T, num_iter, spb, acceptance, sequential=True, resync_every=0,
                 full_energy=False, seed=0):
    rng = np.random.default_rng(seed)
    n = f.shape[0]
    beta = schedule(acceptance, num_iter)
    init = rng.integers(0, 2, size=(T, n)).astype(np.uint8)
    u, thr = replay_randoms(rng, beta, spb, T, n, acceptance, sequential=sequential)
    site = None if sequential else random_sites(rng, T, num_iter * spb, n)
    plan = native.AnnealPlan(f, beta, num_tries=T, sweeps_per_beta=spb, acceptance=acceptance,
                             site_order=native.SITES_SEQUENTIAL if sequential else native.SITES_RANDOM,
                             resync_every=resync_every, ctx=ctx)
    try:
        plan.set_replay(init, thr, site)
        plan.execute()
        got = plan.trajectories()
        order = plan.sweep_order() if sequential else None
        # the same plan back on Philox draws still runs
        plan.clear_replay()
        plan.execute()
        plan.result()
    finally:
        plan.close()
    ref = orc.sa_replay(f, beta, init, u, sweeps_per_beta=spb, acceptance=acceptance, mode=1 if sequential else 0,
                        order=order, site=site, full_energy=full_energy)
    check_same(got, ref)
    return order


@pytest.mark.parametrize("acceptance", [0, 1])
def test_dense_tile_kernel_n64_reference_loop(native, orc, ctx, acceptance):
    """Staged-tile kernel, against the reference's full energy per attempt."""
    f = random_int_qubo(64, 1, -4, 4)
    order = dense_replay(native, orc, ctx, f, T=40, num_iter=10, spb=2, acceptance=acceptance, resync_every=7,
                         full_energy=True, seed=acceptance)
    # the documented visit order: slot by slot, lanes in order
    expect = [128 * (s // 4) + 4 * l + s % 4 for s in range(4) for l in range(32)]
    assert order.tolist() == [k for k in expect if k < 64]


@pytest.mark.parametrize("n,T", [(1024, 64), (700, 48), (100, 24)])
@pytest.mark.parametrize("acceptance", [0, 1])
def test_dense_tile_kernel(native, orc, ctx, n, T, acceptance):
    """n = 1024 fills its slot class (the variant without padding tests),
    700 and 100 do not."""
    f = random_int_qubo(n, n, -3, 3)
    dense_replay(native, orc, ctx, f, T=T, num_iter=3, spb=1, acceptance=acceptance, resync_every=2,
                 seed=10 + acceptance)


@pytest.mark.parametrize("acceptance", [0, 1])
def test_dense_readonly_row_kernel_n2048(native, orc, ctx, acceptance):
    """n = 2048 is above the staged-tile limit: rows come through the read-only path."""
    f = random_int_qubo(2048, 5, -2, 2)
    dense_replay(native, orc, ctx, f, T=32, num_iter=3, spb=1, acceptance=acceptance, seed=20 + acceptance)


@pytest.mark.parametrize("n", [64, 1024])
@pytest.mark.parametrize("acceptance", [0, 1])
def test_dense_random_site_kernel(native, orc, ctx, n, acceptance):
    """The reference's one random site per step."""
    f = random_int_qubo(n, 7, -3, 3)
    dense_replay(native, orc, ctx, f, T=48, num_iter=50, spb=40, acceptance=acceptance, sequential=False,
                 resync_every=700, full_energy=n <= 64, seed=30 + acceptance)


def sparse_replay(native, orc, ctx, csr, *, T, num_iter, acceptance, resync_every=0, full_energy=False, seed=0):
    rng = np.random.default_rng(seed)
    n = csr.n
    beta = schedule(acceptance, num_iter)
    init = rng.integers(0, 2, size=(T, n)).astype(np.uint8)
    u, thr = replay_randoms(rng, beta, 1, T, n, acceptance)
    plan = native.AnnealPlan(csr, beta, num_tries=T, acceptance=acceptance, resync_every=resync_every, ctx=ctx)
    try:
        plan.set_replay(init, thr)
        plan.execute()
        got = plan.trajectories()
        order = plan.sweep_order()
    finally:
        plan.close()
    assert sorted(order.tolist()) == list(range(n))
    ref = orc.sa_replay(csr.to_dense(), beta, init, u, acceptance=acceptance, mode=2, order=order,
                        full_energy=full_energy)
    check_same(got, ref)
    return order


@pytest.mark.parametrize("acceptance", [0, 1])
def test_sparse_kernel_chimera2048(native, orc, ctx, acceptance):
    """Colour-parallel sweeps on the 2,048-spin Chimera graph (16 x 16 K4,4
    cells, J = +-1): a sweep is the sequential sweep in colour-sorted order,
    the best state is checked at the end of every sweep."""
    import bench
    csr = bench.chimera_csr(16, 3)
    order = sparse_replay(native, orc, ctx, csr, T=64, num_iter=4, acceptance=acceptance, resync_every=3,
                          seed=40 + acceptance)
    # two colour classes of 1,024 sites, no coupler inside a class
    f = csr.to_dense()
    np.fill_diagonal(f, 0.0)
    first, second = order[:1024], order[1024:]
    assert not f[np.ix_(first, first)].any() and not f[np.ix_(second, second)].any()


def test_sparse_kernel_small_chimera_reference_loop(native, orc, ctx):
    import bench
    sparse_replay(native, orc, ctx, bench.chimera_csr(4, 1), T=24, num_iter=12, acceptance=1, full_energy=True,
                  seed=50)


@pytest.mark.parametrize("acceptance", [0, 1])
def test_batched_kernel(native, orc, ctx, acceptance):
    """The persistent batched launch over 16 instances of uneven n in
    [64, 1024]: every instance's trajectories equal the oracle's."""
    rng = np.random.default_rng(60 + acceptance)
    sizes = [64, 1024, 129, 700, 96, 512, 300, 1000, 77, 256, 640, 200, 999, 128, 450, 65]
    fs = [random_int_qubo(n, 100 + k, -3, 3) for k, n in enumerate(sizes)]
    T, num_iter = 8, 3
    beta = schedule(acceptance, num_iter)
    inits, us, thrs = [], [], []
    for n in sizes:
        inits.append(rng.integers(0, 2, size=(T, n)).astype(np.uint8))
        u, thr = replay_randoms(rng, beta, 1, T, n, acceptance)
        us.append(u)
        thrs.append(thr)
    plan = native.BatchedAnnealPlan(fs, beta, num_tries=T, acceptance=acceptance, resync_every=2, ctx=ctx)
    try:
        plan.set_replay(inits, thrs)
        plan.execute()
        got = plan.trajectories()
        orders = plan.sweep_order()
        plan.execute()  # a second replay (graph replayed) gives the same trajectories
        again = plan.trajectories()
    finally:
        plan.close()
    for k, n in enumerate(sizes):
        ref = orc.sa_replay(fs[k], beta, inits[k], us[k], acceptance=acceptance, mode=1, order=orders[k])
        check_same(got[k], ref)
        assert np.array_equal(again[k].final_states, got[k].final_states)


def test_replay_argument_checks(native, ctx):
    f = random_int_qubo(32, 0)
    plan = native.AnnealPlan(f, [1.0, 0.5], num_tries=4, site_order=native.SITES_RANDOM, ctx=ctx)
    try:
        init = np.zeros((4, 32), np.uint8)
        thr = np.zeros((4, 2), np.float32)
        with pytest.raises(native.OneSolverError):
            plan.set_replay(init, thr)            # random sites need the sites
        with pytest.raises(native.OneSolverError):
            plan.set_replay(init, thr, np.full((4, 2), 32, np.int32))   # site out of range
        with pytest.raises(native.OneSolverError):
            plan.sweep_order()                    # no fixed sweep order
    finally:
        plan.close()
