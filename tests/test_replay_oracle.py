"""The replay oracle (orc_sa_replay) against the reference transcriptions (CPU).

orc_sa_replay restates the Metropolis loop of annealing.hpp:97-123 in a given
site order; the GPU replay tests compare the sweep kernels with it. Here it is
pinned against orc_anneal_verify (the reference's kernel body with given
(site, u) pairs, itself checked against a pure-Python transcription in
test_oracle_golden.py), and its O(n)-per-flip local-field form against its
reference-faithful form that recomputes the full energy every attempt.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests.qubo_text import random_int_qubo
from tests.sa_replay_inputs import random_sites, replay_randoms


@pytest.mark.parametrize("acceptance", [0, 1])
def test_random_sites_equal_the_reference_body(orc, acceptance):
    rng = np.random.default_rng(3 + acceptance)
    n, T, spb = 24, 6, 3
    f = random_int_qubo(n, 11, -4, 4)
    beta = np.geomspace(8.0, 0.5, 20) if acceptance == 0 else np.geomspace(0.05, 1.5, 20)
    init = rng.integers(0, 2, size=(T, n)).astype(np.uint8)
    u, _ = replay_randoms(rng, beta, spb, T, n, acceptance, sequential=False)
    site = random_sites(rng, T, len(beta) * spb, n)
    bs, be, fs, fe, ac = orc.anneal_verify(f, beta, init, site, u, sweeps_per_beta=spb, acceptance=acceptance)
    for full in (True, False):
        rf, rb, rfe, rbe, rac = orc.sa_replay(f, beta, init, u, sweeps_per_beta=spb, acceptance=acceptance,
                                              mode=0, site=site, full_energy=full)
        assert np.array_equal(rf, fs) and np.array_equal(rb, bs)
        assert np.array_equal(rfe, fe) and np.array_equal(rbe, be) and np.array_equal(rac, ac)


@pytest.mark.parametrize("acceptance", [0, 1])
def test_sequential_sweeps_equal_the_reference_body(orc, acceptance):
    """A sequential sweep in a given order is the reference's loop with the
    sites listed in that order, n attempts per step (best state checked after
    every attempt)."""
    rng = np.random.default_rng(7 + acceptance)
    n, T, spb = 20, 5, 2
    f = random_int_qubo(n, 12, -4, 4)
    beta = np.geomspace(8.0, 0.5, 6) if acceptance == 0 else np.geomspace(0.05, 1.5, 6)
    init = rng.integers(0, 2, size=(T, n)).astype(np.uint8)
    u, _ = replay_randoms(rng, beta, spb, T, n, acceptance)
    order = rng.permutation(n).astype(np.int32)
    S = len(beta) * spb
    site = np.tile(order, (T, S))
    u_flat = u[:, :, order].reshape(T, S * n)
    bs, be, fs, fe, ac = orc.anneal_verify(f, np.repeat(beta, spb), init, site, u_flat, sweeps_per_beta=n,
                                           acceptance=acceptance)
    for full in (True, False):
        rf, rb, rfe, rbe, rac = orc.sa_replay(f, beta, init, u, sweeps_per_beta=spb, acceptance=acceptance,
                                              mode=1, order=order, full_energy=full)
        assert np.array_equal(rf, fs) and np.array_equal(rb, bs)
        assert np.array_equal(rfe, fe) and np.array_equal(rbe, be) and np.array_equal(rac, ac)


def test_sweep_end_bookkeeping(orc):
    """Mode 2 (best state checked at sweep ends) keeps the same chain as
    mode 1 and a best energy that is the minimum over sweep-end energies."""
    rng = np.random.default_rng(5)
    n, T = 18, 8
    f = random_int_qubo(n, 2, -4, 4)
    beta = np.geomspace(0.05, 2.0, 12)
    init = rng.integers(0, 2, size=(T, n)).astype(np.uint8)
    u, _ = replay_randoms(rng, beta, 1, T, n, 1)
    m1 = orc.sa_replay(f, beta, init, u, acceptance=1, mode=1)
    m2 = orc.sa_replay(f, beta, init, u, acceptance=1, mode=2)
    m2f = orc.sa_replay(f, beta, init, u, acceptance=1, mode=2, full_energy=True)
    assert all(np.array_equal(a, b) for a, b in zip(m2, m2f))
    assert np.array_equal(m1[0], m2[0]) and np.array_equal(m1[2], m2[2]) and np.array_equal(m1[4], m2[4])
    assert np.all(m2[3] >= m1[3])
    # the best of mode 2 is a sweep-end state: its energy is its FP64 energy
    assert np.array_equal(orc.energy_batch(f, m2[1]), m2[3])


def test_thresholds_agree_with_the_exp_rule():
    """Every integer dE gets the same decision from dE < thr32 and from the
    reference's exp test on u."""
    rng = np.random.default_rng(1)
    beta = np.geomspace(0.02, 3.0, 7)
    for acceptance in (0, 1):
        b = beta if acceptance == 1 else beta * 30
        u, thr = replay_randoms(rng, b, 1, 4, 50, acceptance)
        bs = b.reshape(1, -1, 1)
        for de in range(-40, 41):
            ref = (de < 0) | (np.exp(-de / bs) > u if acceptance == 0 else np.exp(-bs * de) > u)
            assert np.array_equal(de < thr, ref)


@pytest.mark.parametrize("site_order,acceptance", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_local_field_chain_equals_the_reference_chain(orc, site_order, acceptance):
    """orc_anneal_free_fields draws the same randoms in the same order as the
    reference-algorithm anneal (full FP64 energy per attempt): on an integer
    instance the two give the same best states and energies, bit for bit."""
    n, T = 22, 12
    f = random_int_qubo(n, 31, -4, 4)
    beta = np.geomspace(8.0, 0.5, 15) if acceptance == 0 else np.geomspace(0.05, 1.5, 15)
    a = orc.anneal_free(f, beta, T, 3, seed=17, acceptance=acceptance, site_order=site_order)
    b = orc.anneal_free_fields(f, beta, T, 3, seed=17, acceptance=acceptance, site_order=site_order)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]


def test_local_field_chain_sweep_order_and_bookkeeping(orc):
    """A given sweep order and sweep-end bookkeeping: best energies are the
    energies of the best states, never below the per-attempt bookkeeping's."""
    n, T = 40, 16
    f = random_int_qubo(n, 8, -3, 3)
    beta = np.geomspace(0.05, 2.0, 20)
    order = np.random.default_rng(0).permutation(n)
    a = orc.anneal_free_fields(f, beta, T, 1, seed=3, acceptance=1, site_order=1, order=order)
    b = orc.anneal_free_fields(f, beta, T, 1, seed=3, acceptance=1, site_order=1, order=order,
                               best_at_sweep_end=True)
    assert np.array_equal(orc.energy_batch(f, a[0]), a[1])
    assert np.array_equal(orc.energy_batch(f, b[0]), b[1])
    assert np.all(b[1] >= a[1])
