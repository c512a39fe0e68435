"""Population annealing on the sparse sweep kernel.

No reference counterpart: the reference's annealing benchmark names
population annealing beside parallel tempering as the next solver
(benchmarks/annealing/performance.md:52-59).

CPU tests pin the oracle's resampling step (a second, pure-Python
transcription; the systematic-resampling count bound). GPU tests check:
  * the device resampling step against the oracle, bit for bit, through
    os_pa_resample_replay;
  * the free-energy estimates ln Z(beta_k) against exact enumeration of a
    small instance;
  * the final population's mean energy against the exact Boltzmann mean;
  * every returned state re-scores to the reported FP64 energy.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from tests.test_pt import _all_energies, _random_sparse_ising


def _py_resample(e, dbeta, seed, step, philox):
    """Independent transcription of the resampling rule over Python floats."""
    R, B = len(e), 1024
    L = (R + B - 1) // B
    emin = min(e)
    cum = [0.0] * R
    tot = []
    for b in range(B):
        run = 0.0
        for i in range(b * L, min(R, (b + 1) * L)):
            run += math.exp(-dbeta * (e[i] - emin))
            cum[i] = run
        tot.append(run)
    pre, gsum = [], []
    for g in range(32):
        run = 0.0
        for k in range(32):
            pre.append(run)
            run += tot[32 * g + k]
        gsum.append(run)
    goff, acc = [], 0.0
    for g in range(32):
        goff.append(acc)
        acc += gsum[g]
    for b in range(B):
        for i in range(b * L, min(R, (b + 1) * L)):
            cum[i] = (goff[b // 32] + pre[b]) + cum[i]
    w = philox([step, 0, 0, 5 << 28], [seed & 0xFFFFFFFF, seed >> 32])[0]
    u = (w + 0.5) * 2.0 ** -32
    stride = acc / R
    par = []
    for j in range(R):
        t = (u + j) * stride
        lo, hi = 0, R - 1
        while lo < hi:
            mid = (lo + hi) // 2
            if cum[mid] > t:
                hi = mid
            else:
                lo = mid + 1
        par.append(lo)
    return np.array(par, dtype=np.int32), (-dbeta * emin) + math.log(acc / R)


def test_oracle_resample_matches_python_transcription(orc):
    rng = np.random.default_rng(0)
    for R, dbeta in [(1, 0.3), (7, 0.0), (1500, 0.4), (3000, 2.5)]:
        e = np.round(rng.normal(0, 4, R), 3)
        p1, l1 = orc.pa_resample(e, dbeta, 17, 3)
        p2, l2 = _py_resample(e.tolist(), dbeta, 17, 3, orc.philox)
        assert np.array_equal(p1, p2) and l1 == l2


def test_oracle_resample_rule(orc):
    # Equal weights: every slot keeps its own replica, ln Q = 0.
    p, lq = orc.pa_resample(np.arange(50, dtype=np.float64), 0.0, 1, 0)
    assert p.tolist() == list(range(50)) and lq == 0.0
    # Systematic resampling: replica i gets floor or ceil of R w_i / W copies.
    rng = np.random.default_rng(3)
    e = rng.normal(0, 3, 4000)
    p, lq = orc.pa_resample(e, 0.7, 9, 2)
    w = np.exp(-0.7 * (e - e.min()))
    expect = len(e) * w / w.sum()
    counts = np.bincount(p, minlength=len(e))
    assert (np.abs(counts - expect) < 1 + 1e-9).all()
    assert (np.diff(p) >= 0).all()
    assert lq == pytest.approx(-0.7 * e.min() + math.log(w.mean()), rel=1e-12)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("R,dbeta,step", [(1, 0.5, 0), (1000, 0.0, 4), (4097, 0.8, 11), (70000, 3.0, 2)])
def test_resample_replay_bit_exact(native, orc, ctx, R, dbeta, step):
    e = np.round(np.random.default_rng(R).normal(0, 5, R), 4)
    pg, lg = native.pa_resample_replay(e, dbeta, seed=23, step=step, ctx=ctx)
    po, lo = orc.pa_resample(e, dbeta, 23, step)
    assert np.array_equal(pg, po)
    assert lg == pytest.approx(lo, rel=1e-13, abs=1e-13)


@pytest.mark.gpu
def test_free_energy_and_final_population_match_enumeration(native, orc, ctx):
    f = _random_sparse_ising(14, 3, 2)
    allE = _all_energies(f)
    beta = np.linspace(0.02, 1.0, 50)
    R = 20000
    res = native.population_anneal_sparse(native.Csr.from_dense(f), beta, population=R, sweeps_per_beta=2,
                                          seed=4, ctx=ctx, final_states=True)
    emin = allE.min()
    exact = np.array([-b * emin + math.log(np.exp(-b * (allE - emin)).sum()) for b in beta])
    assert np.abs(res.log_z - exact).max() < 0.05, np.abs(res.log_z - exact).max()
    fe = orc.energy_batch(f, res.final_states)
    assert np.array_equal(fe, res.final_energies)
    w = np.exp(-beta[-1] * (allE - emin))
    w /= w.sum()
    mean = float(w @ allE)
    sd = math.sqrt(float(w @ (allE - mean) ** 2))
    assert 1 <= res.families <= R
    assert abs(res.final_energies.mean() - mean) < 5 * sd / math.sqrt(res.families) + 1e-9
    assert res.energy == pytest.approx(orc.energy(f, res.state), rel=1e-9, abs=0)
    assert res.energy >= emin and res.attempts == R * 50 * 2 * 14


@pytest.mark.gpu
def test_population_annealing_rejects_bad_arguments(native, ctx):
    from tests.test_sa_gpu import chimera_ising
    csr = native.Csr.from_dense(chimera_ising(1, 0))
    with pytest.raises(native.OneSolverError, match="population"):
        native.population_anneal_sparse(csr, [1.0], population=0, ctx=ctx)
    with pytest.raises(native.OneSolverError, match="population"):
        native.population_anneal_sparse(csr, [1.0], population=70000, ctx=ctx)
    with pytest.raises(native.OneSolverError, match="finite"):
        native.population_anneal_sparse(csr, [1.0, float("nan")], ctx=ctx)
    with pytest.raises(native.OneSolverError, match="finite"):
        native.pa_resample_replay(np.array([0.0, np.inf]), 0.5, ctx=ctx)


@pytest.mark.gpu
def test_droplet_128_reaches_tensor_network_ground_state(native, orc, ctx, golden_chimera):
    """Droplet 128/001 (reference best SA -221.573, tensor-network ground
    state -235.867): 8,192 replicas, 300 steps of linear beta 0.05 -> 3.0 with
    5 sweeps each."""
    from tests.conftest import GOLDEN
    g = golden_chimera["128"]
    f = native.Model.load(GOLDEN / g["file"]).flatten()
    res = native.population_anneal_sparse(native.Csr.from_dense(f), np.linspace(0.05, 3.0, 300), population=8192,
                                          sweeps_per_beta=5, resync_every=50, seed=5, ctx=ctx)
    assert res.energy == pytest.approx(orc.energy(f, res.state), rel=1e-9, abs=0)
    assert abs(res.energy - g["tn_ground_qubo"]) < 1e-6, res.energy
    assert res.max_field_drift < 1e-3


def _slot_ranges(e, dbeta, seed, step, philox):
    """The device's assignment method (pa_assign_kernel) over Python floats:
    each replica writes itself into [slots_below(C_{i-1}), slots_below(C_i)),
    starting every block from its predecessor's last sum (offset + total)."""
    R, B = len(e), 1024
    L = (R + B - 1) // B
    emin = min(e)
    loc, tot = [0.0] * R, [0.0] * B
    for b in range(B):
        run = 0.0
        for i in range(b * L, min(R, (b + 1) * L)):
            run += math.exp(-dbeta * (e[i] - emin))
            loc[i] = run
        tot[b] = run
    pre, goff = [0.0] * B, [0.0] * 32
    for g in range(32):
        run = 0.0
        for k in range(32):
            pre[32 * g + k] = run
            run += tot[32 * g + k]
        goff[g] = run
    W = 0.0
    for g in range(32):
        v = goff[g]
        goff[g] = W
        W += v
    w = philox([step, 0, 0, 5 << 28], [seed & 0xFFFFFFFF, seed >> 32])[0]
    u = (w + 0.5) * 2.0 ** -32
    stride, inv = W / R, R / W

    def below(c):
        q = c * inv - u
        j = 0 if q <= 0.0 else (R if q >= R else math.ceil(q))
        while j > 0 and (u + (j - 1)) * stride >= c:
            j -= 1
        while j < R and (u + j) * stride < c:
            j += 1
        return j

    par = [-1] * R
    for b in range(B):
        b0, b1 = b * L, min(R, (b + 1) * L)
        if b0 >= b1:
            continue
        off = goff[b // 32] + pre[b]
        j = 0 if b == 0 else below(goff[(b - 1) // 32] + pre[b - 1] + tot[b - 1])
        for i in range(b0, b1):
            j1 = R if i == R - 1 else below(off + loc[i])
            while j < j1:
                par[j] = i
                j += 1
    return np.array(par, dtype=np.int32)


@pytest.mark.parametrize("R,dbeta,scale", [(1, 0.5, 1.0), (2, 3.0, 1.0), (5, 40.0, 10.0), (1023, 0.2, 3.0),
                                           (1025, 9.0, 5.0), (2049, 0.0, 1.0), (3000, 60.0, 20.0)])
def test_device_slot_range_method_equals_first_exceeding_rule(orc, R, dbeta, scale):
    # The kernel assigns slots by ranges; the definition (and the oracle) is
    # a search for the first cumulative sum above each target. They must give
    # the same parents everywhere, including weights that underflow to zero
    # (large dbeta) and ties between equal energies.
    rng = np.random.default_rng(R)
    e = np.round(rng.normal(0, scale, R), 1)
    for step in (0, 7):
        par = _slot_ranges(e.tolist(), dbeta, 31, step, orc.philox)
        ref, _ = orc.pa_resample(e, dbeta, 31, step)
        assert (par >= 0).all()
        assert np.array_equal(par, ref)


def test_population_arguments_are_checked_on_the_host(native):
    """Parameter checks run before the device is touched (null context here)."""
    import ctypes as C
    from tests.test_sa_gpu import chimera_ising
    L = native.lib()
    q = native.Csr.from_dense(chimera_ising(1, 0))._c()

    def run(beta, population=16, spb=1, resync=0):
        b = np.ascontiguousarray(beta, dtype=np.float64)
        prm = native._PaParams(native._dptr(b), len(b), spb, population, 1, resync)
        res = native._PaResult()
        st = L.os_pa_run_sparse(None, C.byref(q), C.byref(prm), C.byref(res))
        return st, L.os_last_error().decode()

    for args, msg in [(([1.0], 0), "population"), (([1.0], 70000), "population"), (([np.inf],), "finite"),
                      (([1.0], 16, 0), "sweeps_per_beta"), (([1.0], 16, 1, -2), "resync")]:
        st, err = run(*args)
        assert st == native.INVALID_ARG and msg in err, (args, err)
    st, err = run([0.2, 0.4])
    assert st == native.INVALID_ARG and "null context" in err

    par = np.zeros(2, dtype=np.int32)
    lq = C.c_double()
    e = np.array([0.0, np.nan])
    st = L.os_pa_resample_replay(None, 2, native._dptr(e), 0.5, 1, 0, par.ctypes.data_as(C.POINTER(C.c_int32)),
                                 C.byref(lq))
    assert st == native.INVALID_ARG and "not finite" in L.os_last_error().decode()
