"""Pin the oracle against the reference's own known-answer tests (CPU)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from tests.qubo_text import dense_from_text, random_int_qubo, read_maps


def test_exhaustive_golden_energies(orc, golden_exhaustive):
    # tests/exhaustive_test.cpp:144-158: |E - expected| < 1e-13 for five files.
    assert len(golden_exhaustive["cases"]) == 5
    for case in golden_exhaustive["cases"]:
        f = dense_from_text(case["text"])
        e, s = orc.exhaustive(f)
        assert abs(e - case["energy"]) < 1e-13
        assert orc.energy_bits(f, s) == e


def test_exhaustive_examples_match_cases(orc, golden_exhaustive):
    # The example files are the same instances as the test strings.
    by_energy = {case["energy"] for case in golden_exhaustive["cases"]}
    for name in ("test1.qubo", "test2.qubo", "csp5.qubo", "csp7.qubo", "csp13.qubo"):
        e, _ = orc.exhaustive(dense_from_text(golden_exhaustive["examples"][name]))
        assert any(abs(e - v) < 1e-13 for v in by_energy), name


def test_flatten_layout(orc, golden_io):
    # tests/qubo_helpers_test.cpp:12-30.
    g = golden_io["flatten"]
    lin = {i: v for i, v in g["linear"]}
    quad = {(i, j): v for i, j, v in g["quadratic"]}
    out = orc.flatten(g["n"], lin, quad)
    assert out.ravel().tolist() == g["expected"]


def test_solution_csv_bytes(orc, golden_io):
    # tests/io_test.cpp:108-118.
    g = golden_io["csv"]
    assert orc.solution_csv(g["state"], g["energy"]) == g["expected"]


def test_energy_matches_bits_form(orc):
    f = random_int_qubo(9, 3)
    rng = np.random.default_rng(0)
    for _ in range(50):
        s = int(rng.integers(0, 1 << 9))
        bits = [(s >> i) & 1 for i in range(9)]
        assert orc.energy(f, bits) == orc.energy_bits(f, s)


def test_schedules_reference_semantics(orc):
    # app/one-solver-anneal.cpp:23-39: linear ends at beta_min + beta_max.
    lin = orc.schedule_linear(0.1, 3.0, 11)
    assert lin[0] == 0.1 and lin[-1] == pytest.approx(3.1)
    geo = orc.schedule_geometric(0.1, 1.0, 100)
    alpha = math.pow(1.0 / 0.1, 1.0 / 99)
    x = 0.1
    for i in range(1, 100):
        x = x * alpha
        assert geo[i] == x
    assert math.isnan(orc.schedule_linear(0.1, 1.0, 1)[0])


def test_schedules_python_mirror(native, orc):
    for n in (2, 3, 100, 1000):
        assert np.array_equal(native.linear_schedule(0.1, 3.0, n), orc.schedule_linear(0.1, 3.0, n))
        assert np.array_equal(native.geometric_schedule(0.1, 5.0, n), orc.schedule_geometric(0.1, 5.0, n))


def test_philox_known_answers(orc):
    # Philox4x32-10 known-answer vectors of the Random123 distribution.
    assert orc.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert orc.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert orc.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def _py_anneal(f, beta, init, site, u, spb, acceptance):
    """Pure-Python transcription of annealing.hpp:87-125 (tiny sizes)."""
    n = f.shape[0]

    def energy(x):
        r = 0.0
        for i in range(n):
            for j in range(i, n):
                r += f[i, j] * x[i] * x[j]
        return r

    out = []
    for t in range(init.shape[0]):
        cur = [int(v) for v in init[t]]
        best = list(cur)
        be = energy(cur)
        ce = be
        for it, b in enumerate(beta):
            for sw in range(spb):
                a = it * spb + sw
                k = int(site[t, a])
                cur[k] = 1 - cur[k]
                ne = energy(cur)
                if ne < ce:
                    acc = True
                elif acceptance == 0:
                    acc = math.exp((ce - ne) / b) > u[t, a]
                else:
                    acc = math.exp(-b * (ne - ce)) > u[t, a]
                if acc:
                    ce = ne
                else:
                    cur[k] = 1 - cur[k]
                if ce < be:
                    be = ce
                    best = list(cur)
        out.append((best, be, cur, ce))
    return out


@pytest.mark.parametrize("acceptance", [0, 1])
def test_anneal_verify_matches_python(orc, acceptance):
    n, T, iters, spb = 7, 3, 40, 2
    f = random_int_qubo(n, 11, -3, 3)
    rng = np.random.default_rng(5)
    beta = orc.schedule_geometric(0.1, 2.0, iters)
    init = rng.integers(0, 2, size=(T, n)).astype(np.uint8)
    site = rng.integers(0, n, size=(T, iters * spb)).astype(np.int32)
    u = rng.random(size=(T, iters * spb))
    bs, be, fs, fe, ac = orc.anneal_verify(f, beta, init, site, u, spb, acceptance)
    ref = _py_anneal(f, beta, init, site, u, spb, acceptance)
    for t in range(T):
        assert bs[t].tolist() == ref[t][0]
        assert be[t] == ref[t][1]
        assert fs[t].tolist() == ref[t][2]
        assert fe[t] == ref[t][3]


def test_exhaustive_all_counts_ties(orc):
    f = np.zeros((6, 6))
    e, count, states = orc.exhaustive_all(f)
    assert e == 0.0 and count == 64 and states.tolist() == list(range(64))


def test_read_maps_first_key_wins():
    n, lin, quad = read_maps("p qubo 0 3 1 1\n0 0 1\n0 0 5\n0 2 3\n")
    assert n == 3 and lin == {0: 1.0} and quad == {(0, 2): 3.0}


@pytest.mark.parametrize("n,seed,lo,hi", [(1, 0, -8, 8), (9, 5, 0, 0), (12, 1, -8, 8), (16, 4, -1, 1),
                                          (18, 2, -8, 8), (20, 3, -2, 2)])
def test_integer_table_scan_matches_reference_loop(orc, n, seed, lo, hi):
    """The byte-table scan that makes the n = 36 fixtures equals the
    reference's O(n^2)-per-state FP64 loop (energy, count, every minimiser)."""
    f = random_int_qubo(n, seed, lo, hi)
    e, count, states = orc.exhaustive_all(f)
    ei, ci, si = orc.exhaustive_int_all(f)
    assert (ei, ci) == (e, count)
    assert si.tolist() == states.tolist()
    # a sub-range, as shards use it
    if n >= 12:
        lo_s, hi_s = 3 << (n - 4), 7 << (n - 4)
        e2, c2, s2 = orc.exhaustive_all(f, lo_s, hi_s)
        assert orc.exhaustive_int_all(f, lo_s, hi_s)[:2] == (e2, c2)


def test_integer_table_scan_rejects_fractions(orc):
    f = random_int_qubo(8, 0)
    f[2, 5] = f[5, 2] = 0.5
    with pytest.raises(ValueError):
        orc.exhaustive_int_all(f)


def test_exhaustive36_fixture_is_consistent(orc):
    """The committed n = 36 answers: each listed minimiser has the listed
    energy under the reference's FP64 energy function, the list is sorted,
    and its first entry is the reference's answer."""
    import json
    from pathlib import Path
    data = json.loads((Path(__file__).parent / "golden" / "exhaustive36_golden.json").read_text())
    assert sorted(data) == ["0", "1", "2"]
    for seed, d in data.items():
        f = random_int_qubo(36, int(seed))
        assert d["count"] == len(d["states"]) >= 1
        assert d["states"] == sorted(d["states"]) and d["state"] == d["states"][0]
        for s in d["states"]:
            assert orc.energy_bits(f, s) == d["energy"]
