"""Exhaustive search on the GPU against the oracle (bit-exact).

The reference's contract (include/exhaustive/exhaustive.hpp:29-167): the
minimum of the FP64 energy over all 2^n states, and the smallest state integer
reaching it. The GPU path additionally returns the whole degenerate set, which
is compared with the oracle's exact-equality set.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from tests.qubo_text import dense_from_text, random_int_qubo, random_normal_qubo

pytestmark = pytest.mark.gpu


def check_against_oracle(native, orc, ctx, f, **kw):
    res = native.exhaustive(f, ctx=ctx, max_minimisers=1 << 16, **kw)
    e, count, states = orc.exhaustive_all(f)
    e_ref, s_ref = orc.exhaustive(f)
    assert res.energy == e == e_ref
    assert res.state == s_ref
    assert res.count == count
    assert res.states.tolist() == states.tolist()
    return res


def test_golden_instances(native, orc, ctx, golden_exhaustive):
    # tests/exhaustive_test.cpp:144-158 (tolerance 1e-13), plus exact parity.
    for case in golden_exhaustive["cases"]:
        f = native.Model.parse(case["text"]).flatten()
        res = check_against_oracle(native, orc, ctx, f)
        assert abs(res.energy - case["energy"]) < 1e-13


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 13, 14, 15, 16, 19, 22])
def test_random_integer_instances(native, orc, ctx, n):
    for seed in range(3):
        res = check_against_oracle(native, orc, ctx, random_int_qubo(n, seed))
        assert res.coef_kind == native.COEF_INT32


@pytest.mark.parametrize("n", [4, 12, 16, 20])
def test_small_range_has_many_ties(native, orc, ctx, n):
    # Coefficients in {-1, 0, 1} give large degenerate sets.
    for seed in range(3):
        check_against_oracle(native, orc, ctx, random_int_qubo(n, 100 + seed, -1, 1))


@pytest.mark.parametrize("n", [3, 9, 14, 18])
def test_fixed_point_path_non_integer(native, orc, ctx, n):
    for seed in range(3):
        res = check_against_oracle(native, orc, ctx, random_normal_qubo(n, seed))
        assert res.coef_kind == native.COEF_FIXED64


def test_fixed_point_decimal_ties(native, orc, ctx):
    # Decimal coefficients whose FP64 sums round: ties are decided by the
    # reference's summation order, which the re-score reproduces.
    rng = np.random.default_rng(7)
    n = 16
    u = np.triu(rng.integers(-20, 21, size=(n, n)) * 0.1)
    f = u + np.triu(u, 1).T
    check_against_oracle(native, orc, ctx, f)


def test_int64_path(native, orc, ctx):
    f = random_int_qubo(16, 4, -(10 ** 8), 10 ** 8)
    res = check_against_oracle(native, orc, ctx, f)
    assert res.coef_kind == native.COEF_INT64


def test_forced_kinds_agree(native, orc, ctx):
    f = random_int_qubo(17, 9)
    a = native.exhaustive(f, ctx=ctx, coef_kind=native.COEF_INT32)
    b = native.exhaustive(f, ctx=ctx, coef_kind=native.COEF_INT64)
    c = native.exhaustive(f, ctx=ctx, coef_kind=native.COEF_FIXED64)
    for r in (b, c):
        assert (r.energy, r.state, r.count, r.states.tolist()) == (a.energy, a.state, a.count, a.states.tolist())
    with pytest.raises(native.OneSolverError):
        native.exhaustive(random_normal_qubo(10, 0), ctx=ctx, coef_kind=native.COEF_INT32)


def test_all_zero_degenerate_collect_pass(native, ctx):
    # Every state is a minimiser: per-thread lists overflow, the collection
    # pass counts them exactly; the buffer holds only max_minimisers.
    n = 20
    res = native.exhaustive(np.zeros((n, n)), ctx=ctx, max_minimisers=100, allow_overflow=True)
    assert res.status == native.OVERFLOW_MINIMISERS
    assert res.energy == 0.0 and res.state == 0 and res.count == 1 << n
    assert res.collect_passes == 2
    assert len(res.states) == 100
    with pytest.raises(native.OneSolverError):
        native.exhaustive(np.zeros((n, n)), ctx=ctx, max_minimisers=100)
    # Asking for no states is not an overflow.
    res0 = native.exhaustive(np.zeros((n, n)), ctx=ctx, max_minimisers=0)
    assert res0.count == 1 << n


def test_shards_cover_the_space(native, orc, ctx):
    f = random_int_qubo(20, 21)
    full = native.exhaustive(f, ctx=ctx)
    parts = [native.exhaustive(f, ctx=ctx, fixed_high_bits=3, prefix=p) for p in range(8)]
    best = min(p.energy for p in parts)
    assert best == full.energy
    assert sum(p.count for p in parts if p.energy == best) == full.count
    assert min(p.state for p in parts if p.energy == best) == full.state
    for p in (0, 5):
        e, s = orc.exhaustive(f, p << 17, (p + 1) << 17)
        assert parts[p].energy == e and parts[p].state == s


def test_plan_reexecute_is_stable(native, ctx):
    f = random_int_qubo(24, 2)
    plan = native.ExhaustivePlan(f, ctx=ctx)
    plan.execute()
    a = plan.result()
    plan.execute()
    b = plan.result()
    assert (a.energy, a.state, a.count) == (b.energy, b.state, b.count)
    assert plan.launches >= 2
    plan.close()


def test_invalid_arguments(native, ctx):
    with pytest.raises(native.OneSolverError):
        native.exhaustive(np.zeros((51, 51)), ctx=ctx)
    with pytest.raises(native.OneSolverError):
        native.exhaustive(random_int_qubo(8, 0), ctx=ctx, fixed_high_bits=8)
    with pytest.raises(native.OneSolverError):
        native.exhaustive(random_int_qubo(8, 0), ctx=ctx, fixed_high_bits=2, prefix=4)
    f = random_int_qubo(8, 0)
    f[1, 2] = np.nan
    with pytest.raises(native.OneSolverError):
        native.exhaustive(f, ctx=ctx)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_n36_config(native, orc, ctx, seed):
    """Dense N=36, integer coefficients in [-8, 8] (2^36 states): the ground
    energy, the reference's answer, the number of minimisers and every
    minimiser equal the oracle's own full scan of all 2^36 states, committed
    as tests/golden/exhaustive36_golden.json (made by
    tests/golden/make_exhaustive36.py)."""
    import json
    gold = json.loads((Path(__file__).parent / "golden" / "exhaustive36_golden.json").read_text())[str(seed)]
    f = random_int_qubo(36, seed)
    res = native.exhaustive(f, ctx=ctx, max_minimisers=1 << 16)
    assert res.states_enumerated == 1 << 36
    assert res.energy == gold["energy"]
    assert res.state == gold["state"]
    assert res.count == gold["count"]
    assert res.states.tolist() == gold["states"]
    # The fused variant reaches the same answer.
    r2 = native.exhaustive(f, ctx=ctx, max_minimisers=1 << 16, variant=2)
    assert (r2.energy, r2.state, r2.count, r2.states.tolist()) == (res.energy, res.state, res.count,
                                                                  gold["states"])
    # Shards of 2^22 states agree with the oracle's scan of the same range,
    # and no shard goes below the global minimum.
    for p in (0, (1 << 14) - 1, 5461, int(res.state >> 22)):
        part = native.exhaustive(f, ctx=ctx, fixed_high_bits=14, prefix=p)
        e, s = orc.exhaustive(f, p << 22, (p + 1) << 22)
        assert part.energy == e and part.state == s
        assert part.energy >= res.energy


@pytest.mark.parametrize("n", [14, 21, 27, 30])
def test_inner_widths_agree(native, orc, ctx, n):
    f = random_int_qubo(n, 40 + n, -2, 2)
    res = [native.exhaustive(f, ctx=ctx, inner_bits=g, variant=v, max_minimisers=1 << 16)
           for g in (9, 10) for v in (1, 2, 3)]
    for r in res[1:]:
        assert (r.energy, r.state, r.count, r.states.tolist()) == \
            (res[0].energy, res[0].state, res[0].count, res[0].states.tolist())
    # Every width and variant against the oracle's full scan.
    e, count, states = orc.exhaustive_all(f) if n <= 21 else orc.exhaustive_int_all(f)
    assert (res[0].energy, res[0].count) == (e, count)
    assert res[0].state == int(states[0])
    assert res[0].states.tolist() == states.tolist()


@pytest.mark.parametrize("fill", ["neg", "pos", "alternating"])
def test_packed_variant_at_its_range_limit(native, orc, ctx, fill):
    """The packed variant holds energies in 16-bit halves; it is exact up to
    coefficient magnitudes summing to 8,000 (here 7,980, all of one sign, so
    the extreme energies and coupling sums reach the limit)."""
    n = 20
    v = {"neg": -38.0, "pos": 38.0}.get(fill)
    if v is None:
        f = np.where((np.arange(n)[:, None] + np.arange(n)[None, :]) % 2 == 0, 38.0, -38.0)
    else:
        f = np.full((n, n), v)
    assert np.abs(np.triu(f)).sum() == 7980
    plan = native.ExhaustivePlan(f, ctx=ctx, max_minimisers=1 << 16)
    assert plan.variant == 3
    plan.close()
    for variant in (0, 2, 3):
        check_against_oracle(native, orc, ctx, f, variant=variant)


def test_packed_variant_only_where_exact(native, ctx):
    f = np.full((20, 20), 40.0)   # magnitudes sum to 8,400
    plan = native.ExhaustivePlan(f, ctx=ctx)
    assert plan.variant == 2      # the default falls back to the 32-bit pair
    plan.close()
    with pytest.raises(native.OneSolverError, match="packed"):
        native.exhaustive(f, ctx=ctx, variant=3)
    with pytest.raises(native.OneSolverError):
        native.exhaustive(random_int_qubo(20, 0), ctx=ctx, variant=4)
