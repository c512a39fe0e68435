"""Parallel tempering (replica exchange) on the sparse sweep kernel.

No reference counterpart: the reference's annealing benchmark recommends
parallel tempering as the next solver (benchmarks/annealing/performance.md:
52-59) after its SA runs missed every tensor-network ground state of the
Chimera droplet instances (benchmarks/annealing/README:20-21).

CPU tests pin the oracle's exchange rule (tests of the rule itself and a
second, pure-Python transcription). GPU tests check:
  * the device exchange step against the oracle, bit for bit, on fixed
    energies (os_pt_exchange_replay);
  * one temperature and no exchanges reproduces the sparse anneal at that
    constant beta exactly (same kernel, same Philox counters);
  * the per-temperature energy distributions of many independent chains
    match the exact Boltzmann averages of a small instance (enumerated);
  * every returned state re-scores to the reported FP64 energy;
  * the droplet 128/001 tensor-network ground state is reached.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from tests.test_sa_gpu import chimera_ising


def _py_exchange(beta, e, seed, round0, rounds, temps, philox):
    """Independent transcription of the exchange rule over Python ints/floats."""
    chains, nt = temps.shape
    temps = temps.copy()
    at = np.zeros_like(temps)
    for c in range(chains):
        for r in range(nt):
            at[c, temps[c, r]] = r
    swaps = [0] * max(nt - 1, 0)
    key = [seed & 0xFFFFFFFF, seed >> 32]
    for c in range(chains):
        for rnd in range(round0, round0 + rounds):
            for k in range(rnd % 2, nt - 1, 2):
                hot, cold = at[c, k], at[c, k + 1]
                d = (beta[k + 1] - beta[k]) * (e[c, cold] - e[c, hot])
                ok = d >= 0.0
                if not ok:
                    w = philox([k, rnd, c, 4 << 28], key)[0]
                    ok = math.log((w + 0.5) * 2.0 ** -32) < d
                if ok:
                    at[c, k], at[c, k + 1] = cold, hot
                    temps[c, cold], temps[c, hot] = k, k + 1
                    swaps[k] += 1
    return temps, np.array(swaps, dtype=np.uint64)


def _exchange_case(chains, nt, seed):
    rng = np.random.default_rng(seed)
    beta = np.geomspace(0.1, 4.0, nt)
    e = np.round(rng.normal(0.0, 3.0, size=(chains, nt)), 3)
    temps = np.array([rng.permutation(nt) for _ in range(chains)], dtype=np.int32)
    return beta, e, temps


def test_oracle_exchange_matches_python_transcription(orc):
    beta, e, temps = _exchange_case(7, 9, 0)
    for round0, rounds in [(0, 1), (1, 1), (0, 25), (13, 8)]:
        t1, s1 = orc.pt_exchange(beta, e, 99, round0, rounds, temps)
        t2, s2 = _py_exchange(beta, e, 99, round0, rounds, temps, orc.philox)
        assert np.array_equal(t1, t2) and np.array_equal(s1, s2)


def test_oracle_exchange_rule(orc):
    # Temperature labels stay a permutation of every chain.
    beta, e, temps = _exchange_case(50, 12, 1)
    t, sw = orc.pt_exchange(beta, e, 3, 0, 200, temps)
    assert all(sorted(row) == list(range(12)) for row in t.tolist())
    # Equal inverse temperatures: d = 0, every tried pair swaps.
    t, sw = orc.pt_exchange(np.ones(5), e[:, :5], 3, 0, 1, np.tile(np.arange(5), (50, 1)))
    assert sw.tolist() == [50, 0, 50, 0]
    assert t[0].tolist() == [1, 0, 3, 2, 4]
    # Two replicas with d = -0.7 every round: the acceptance rate is exp(-0.7)
    # (each swap exchanges the energies' roles, so d stays -0.7 only while the
    # labels are back in place; use fresh identity labels every round).
    chains = 40000
    b = np.array([1.0, 1.7])
    en = np.tile([0.0, -1.0], (chains, 1))  # E_cold - E_hot = -1 at the start
    t, sw = orc.pt_exchange(b, en, 11, 0, 1, np.tile([0, 1], (chains, 1)))
    rate = sw[0] / chains
    p = math.exp(-0.7)
    assert abs(rate - p) < 5 * math.sqrt(p * (1 - p) / chains), (rate, p)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("chains,nt,round0,rounds", [(1, 2, 0, 1), (300, 12, 0, 40), (129, 7, 5, 33)])
def test_exchange_replay_bit_exact(native, orc, ctx, chains, nt, round0, rounds):
    beta, e, temps = _exchange_case(chains, nt, chains + nt)
    tg, sg = native.pt_exchange_replay(beta, e, temps, seed=77, round0=round0, num_rounds=rounds, ctx=ctx)
    to, so = orc.pt_exchange(beta, e, 77, round0, rounds, temps)
    assert np.array_equal(tg, to)
    assert np.array_equal(sg, so)


@pytest.mark.gpu
def test_one_temperature_is_the_constant_beta_anneal(native, ctx):
    # Integer couplings: FP32 fields and tracked energies are exact, so the
    # launch and resync split cannot change a decision.
    f = chimera_ising(3, 4)  # 72 spins
    csr = native.Csr.from_dense(f)
    pt = native.temper_sparse(csr, [1.3], num_chains=64, num_rounds=20, sweeps_per_round=5, resync_every=2,
                              seed=21, ctx=ctx)
    sa = native.anneal_sparse(csr, [1.3], num_tries=64, sweeps_per_beta=100, resync_every=10, acceptance=1,
                              seed=21, ctx=ctx, traj_states=True)
    assert np.array_equal(pt.chain_energies, sa.traj_energies)
    assert pt.energy == sa.energy and np.array_equal(pt.state, sa.state)
    assert pt.attempts == sa.attempts and pt.accepted == sa.accepted
    assert pt.max_field_drift == 0.0
    assert pt.swaps_accepted.size == 0


def _random_sparse_ising(n, deg, seed):
    """Random graph (about deg couplings per spin), J in {-1, +1}, h in {-1, 0, 1},
    as an integer QUBO (x = (s+1)/2, offset dropped)."""
    rng = np.random.default_rng(seed)
    f = np.zeros((n, n))
    edges = set()
    while len(edges) < n * deg // 2:
        i, j = rng.integers(0, n, 2)
        if i != j:
            edges.add((min(i, j), max(i, j)))
    for i, j in sorted(edges):
        v = rng.choice([-1.0, 1.0])
        f[i, j] += 4 * v
        f[j, i] += 4 * v
        f[i, i] -= 2 * v
        f[j, j] -= 2 * v
    f[np.arange(n), np.arange(n)] += 2 * rng.integers(-1, 2, n)
    return f


def _all_energies(f):
    n = f.shape[0]
    x = ((np.arange(1 << n)[:, None] >> np.arange(n)) & 1).astype(np.float64)
    return np.einsum("si,ij,sj->s", x, np.triu(f, 1), x) + x @ np.diag(f)


@pytest.mark.gpu
def test_temperature_marginals_are_boltzmann(native, orc, ctx):
    f = _random_sparse_ising(14, 3, 5)
    allE = _all_energies(f)
    beta = np.geomspace(0.05, 1.2, 8)
    chains = 3000
    res = native.temper_sparse(native.Csr.from_dense(f), beta, num_chains=chains, num_rounds=150,
                               sweeps_per_round=2, seed=8, ctx=ctx, final_states=True)
    # Final states re-score to the reported energies, and every temperature
    # is held by exactly one replica of each chain.
    fe = orc.energy_batch(f, res.final_states.reshape(-1, f.shape[0]))
    assert np.array_equal(fe, res.final_energies.reshape(-1))
    assert (np.sort(res.final_temps, axis=1) == np.arange(len(beta))).all()
    emin = allE.min()
    for k, b in enumerate(beta):
        w = np.exp(-b * (allE - emin))
        w /= w.sum()
        mean = float(w @ allE)
        sd = math.sqrt(float(w @ (allE - mean) ** 2))
        got = res.final_energies[res.final_temps == k]
        assert got.size == chains
        assert abs(got.mean() - mean) < 5 * sd / math.sqrt(chains) + 1e-9, (k, b, got.mean(), mean)
    assert (res.swaps_accepted > 0).all()
    assert (res.swaps_accepted <= res.swaps_attempted).all()


@pytest.mark.gpu
def test_droplet_128_reaches_tensor_network_ground_state(native, orc, ctx, golden_chimera):
    """Droplet 128/001: the reference's best SA energy over 1,200 runs is
    -221.573 and the tensor-network ground state is -235.867."""
    from tests.conftest import GOLDEN
    g = golden_chimera["128"]
    f = native.Model.load(GOLDEN / g["file"]).flatten()
    res = native.temper_sparse(native.Csr.from_dense(f), np.geomspace(0.05, 3.0, 24), num_chains=64,
                               num_rounds=800, sweeps_per_round=5, resync_every=100, seed=3, ctx=ctx)
    assert res.energy == pytest.approx(orc.energy(f, res.state), rel=1e-9, abs=0)
    assert abs(res.energy - g["tn_ground_qubo"]) < 1e-6, res.energy
    assert res.max_field_drift < 1e-3


@pytest.mark.gpu
def test_tempering_rejects_bad_arguments(native, ctx):
    csr = native.Csr.from_dense(chimera_ising(1, 0))
    with pytest.raises(native.OneSolverError, match="non-decreasing"):
        native.temper_sparse(csr, [1.0, 0.5], ctx=ctx)
    with pytest.raises(native.OneSolverError, match="finite"):
        native.temper_sparse(csr, [-1.0, 0.5], ctx=ctx)
    with pytest.raises(native.OneSolverError, match="65535"):
        native.temper_sparse(csr, np.linspace(0.1, 1, 64), num_chains=1025, ctx=ctx)
    with pytest.raises(native.OneSolverError, match="positive"):
        native.temper_sparse(csr, [1.0], num_rounds=0, ctx=ctx)
    with pytest.raises(native.OneSolverError, match="permutation"):
        native.pt_exchange_replay([0.1, 1.0], np.zeros((2, 2)), np.zeros((2, 2), np.int32), ctx=ctx)


@pytest.mark.gpu
def test_droplet_512_reaches_tensor_network_ground_state(native, orc, ctx, golden_chimera):
    """Droplet 512/001: the reference's best SA energy is -674.96 and the
    tensor-network ground state is -928.747; 10^5 sweeps of 128 chains x 32
    temperatures (about 3 s on one GB300) reach it."""
    from tests.conftest import GOLDEN
    g = golden_chimera["512"]
    f = native.Model.load(GOLDEN / g["file"]).flatten()
    res = native.temper_sparse(native.Csr.from_dense(f), np.geomspace(0.05, 3.0, 32), num_chains=128,
                               num_rounds=20000, sweeps_per_round=5, resync_every=200, seed=7, ctx=ctx)
    assert res.energy == pytest.approx(orc.energy(f, res.state), rel=1e-9, abs=0)
    assert abs(res.energy - g["tn_ground_qubo"]) < 1e-6, res.energy


def test_tempering_arguments_are_checked_on_the_host(native):
    """The parameter checks run before the device is touched, so they are
    exercised here without a GPU (a null context): bad parameters are
    INVALID_ARG with the reason, good ones reach the context check."""
    import ctypes as C
    L = native.lib()
    q = native.Csr.from_dense(chimera_ising(1, 0))._c()

    def run(beta, chains=2, rounds=1, spr=1, resync=0):
        b = np.ascontiguousarray(beta, dtype=np.float64)
        prm = native._PtParams(native._dptr(b), len(b), chains, rounds, spr, 1, resync)
        res = native._PtResult()
        st = L.os_pt_run_sparse(None, C.byref(q), C.byref(prm), C.byref(res))
        return st, L.os_last_error().decode()

    for args, msg in [(([1.0, 0.5],), "non-decreasing"), (([np.nan],), "finite"), (([-0.1],), "finite"),
                      ((np.linspace(0.1, 1, 64), 1025), "65535"), (([1.0], 2, 0), "positive"),
                      (([1.0], 2, 1, 0), "positive"), (([1.0], 0), "num_chains"), (([1.0], 2, 1, 1, -1), "resync")]:
        st, err = run(*args)
        assert st == native.INVALID_ARG and msg in err, (args, err)
    st, err = run([0.5, 1.0])
    assert st == native.INVALID_ARG and "null context" in err

    def replay(temps, beta=(0.1, 1.0)):
        b = np.ascontiguousarray(beta, dtype=np.float64)
        t = np.ascontiguousarray(temps, dtype=np.int32)
        e = np.zeros(t.size)
        st = L.os_pt_exchange_replay(None, t.shape[0], t.shape[1], native._dptr(b), native._dptr(e), 1, 0, 1,
                                     t.ctypes.data_as(C.POINTER(C.c_int32)), None)
        return st, L.os_last_error().decode()

    st, err = replay([[0, 0], [0, 1]])
    assert st == native.INVALID_ARG and "chain 0 is not a permutation" in err
    st, err = replay([[1, 0], [0, 1]])
    assert st == native.INVALID_ARG and "null context" in err
