"""Free-running statistical parity at the benchmark configurations' sizes (GPU).

The GPU kernels draw Philox randoms; the reference draws from oneMKL's
philox4x32x10 (annealing.hpp:87), whose stream cannot be reproduced, so
free-running runs are compared in law: the GPU's best-energy distribution
over trajectories against that of the oracle's free-running chain
(orc_anneal_free_fields: the reference's Metropolis loop, annealing.hpp:
97-123, with FP64 local fields and its own host RNG, pinned bit for bit
against the reference-algorithm anneal in test_replay_oracle.py), run in the
kernel's own sweep order and with the kernel's best-state bookkeeping, i.e.
the same Markov chain. Two-sample KS tests, p > 1e-3 per instance (batched:
Bonferroni over the instances), on the configurations' instance sizes with
truncated sweep counts:

* SK n = 1,024, J ~ N(0, 1/n), 512 trajectories (the learned warm start's
  family, dense staged-tile kernel);
* Chimera 16 x 16 (2,048 spins, J = +-1), 1,024 trajectories, linear beta
  (the sparse colour-parallel kernel);
* 32 instances of the batched configuration, n ~ U[64, 1024], N(0, 1/n)
  entries, 256 trajectories each (the persistent batched kernel).
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from tests.test_sa_gpu import _ks

pytestmark = pytest.mark.gpu


def test_sk1024_matches_the_reference_chain(native, orc, ctx):
    import bench
    f = bench.sk_qubo(1024, 11)
    beta = native.geometric_schedule(0.1, 5.0, 150)
    T = 512
    plan = native.AnnealPlan(f, beta, num_tries=T, acceptance=native.ACCEPT_PHYSICAL,
                             site_order=native.SITES_SEQUENTIAL, resync_every=50, seed=21, ctx=ctx)
    try:
        plan.execute()
        res = plan.result()
        order = plan.sweep_order()
    finally:
        plan.close()
    _, e_ref, _ = orc.anneal_free_fields(f, beta, T, 1, seed=5, acceptance=1, site_order=1, order=order)
    ks = _ks(res.traj_energies, e_ref)
    assert ks.pvalue > 1e-3, (ks, res.traj_energies.mean(), e_ref.mean())


def test_chimera2048_matches_the_reference_chain(native, orc, ctx):
    import bench
    csr = bench.chimera_csr(16, 7)
    beta = native.linear_schedule(0.1, 2.9, 100)
    T = 1024
    plan = native.AnnealPlan(csr, beta, num_tries=T, acceptance=native.ACCEPT_PHYSICAL, resync_every=40, seed=3,
                             ctx=ctx)
    try:
        plan.execute()
        res = plan.result()
        order = plan.sweep_order()
    finally:
        plan.close()
    _, e_ref, _ = orc.anneal_free_fields(csr.to_dense(), beta, T, 1, seed=9, acceptance=1, site_order=1,
                                         order=order, best_at_sweep_end=True)
    ks = _ks(res.traj_energies, e_ref)
    assert ks.pvalue > 1e-3, (ks, res.traj_energies.mean(), e_ref.mean())


def test_batched_configuration_matches_the_reference_chain(native, orc, ctx):
    import bench
    rng = np.random.default_rng(4)
    sizes = rng.integers(64, 1025, size=32)
    fs = [bench.normal_qubo(int(m), 500 + k, scale=1.0 / math.sqrt(m)) for k, m in enumerate(sizes)]
    beta = native.geometric_schedule(0.1, 5.0, 60)
    T = 256
    plan = native.BatchedAnnealPlan(fs, beta, num_tries=T, resync_every=20, seed=8, ctx=ctx)
    try:
        plan.execute()
        res = plan.result()
        orders = plan.sweep_order()
    finally:
        plan.close()
    pvals = []
    for k, f in enumerate(fs):
        _, e_ref, _ = orc.anneal_free_fields(f, beta, T, 1, seed=100 + k, acceptance=1, site_order=1,
                                             order=orders[k])
        pvals.append(_ks(res[k].traj_energies, e_ref).pvalue)
    assert min(pvals) > 1e-3 / len(fs), sorted(pvals)[:4]
