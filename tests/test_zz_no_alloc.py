"""Exhaustive search through the entry point that allocates no device memory.

Some callers cannot call cudaMalloc: a serving process that has reserved the
whole device memory for its own pool, or code on a latency-critical path
where an allocation would synchronise the device. os_exhaustive_run_noalloc
serves them from a fixed scratch array inside the library. These tests call it
through the C ABI and compare it with os_exhaustive_run, exactly (integer
work), over consecutive calls that share the array.

This file sorts last so that a run stopping at the first failure has already
run every other test; it also passes on its own in a fresh process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from tests.qubo_text import random_int_qubo

pytestmark = pytest.mark.gpu


def noalloc(native, f, cap, fixed_high_bits=0, prefix=0, coef_kind=0, inner_bits=0, variant=0):
    q, keep = native._dense(f)
    prm = native._ExhParams(coef_kind, fixed_high_bits, prefix, cap, inner_bits, variant)
    states = np.zeros(max(cap, 1), dtype=np.uint64)
    res = native._ExhResult()
    res.states = states.ctypes.data_as(C.POINTER(C.c_uint64))
    st = native.lib().os_exhaustive_run_noalloc(C.byref(q), C.byref(prm), C.byref(res), None)
    return st, res, states[: min(int(res.count), cap)]


def same(native, ctx, f, cap, **kw):
    st, res, states = noalloc(native, f, cap, **kw)
    ref = native.exhaustive(f, ctx=ctx, max_minimisers=cap, allow_overflow=True, **kw)
    assert st == ref.status, native.lib().os_last_error()
    assert res.energy == ref.energy
    assert res.state == ref.state
    assert res.count == ref.count
    if st == native.OK:
        assert states.tolist() == ref.states.tolist()
    return res


def test_noalloc_matches_run_on_consecutive_calls(native):
    ctx = native.Context(0)
    a = random_int_qubo(30, 7)          # Gray-code kernel
    b = random_int_qubo(12, 3, -1, 1)   # one thread per state, many ties
    ra1 = same(native, ctx, a, 4096)
    same(native, ctx, b, 4096)
    ra2 = same(native, ctx, a, 4096)    # nothing left over from the call before
    assert (ra1.energy, ra1.state, ra1.count) == (ra2.energy, ra2.state, ra2.count)
    same(native, ctx, a, 4096, fixed_high_bits=4, prefix=9)
    same(native, ctx, random_int_qubo(18, 1, -10 ** 8, 10 ** 8), 64)  # int64 enumeration
    # The caller's inner width and instruction variant are honoured.
    for g, v in ((9, 1), (10, 1), (9, 2)):
        same(native, ctx, a, 4096, inner_bits=g, variant=v)
    ctx.close()


def test_noalloc_leaves_device_memory_unchanged(native):
    """The calls take no device memory: the device's free memory is the same
    before and after a series of calls (the first calls, which load the
    kernels and look up the array's address, come before the measurement)."""
    torch = pytest.importorskip("torch")
    a = random_int_qubo(30, 7)
    b = random_int_qubo(12, 3, -1, 1)
    z = np.zeros((20, 20))

    def calls():
        for f, cap in ((a, 4096), (b, 4096), (z, 1000)):
            st, _, _ = noalloc(native, f, cap)
            assert st in (native.OK, native.OVERFLOW_MINIMISERS), native.lib().os_last_error()

    calls()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        calls()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_collection_pass(native):
    # Every state ties: the per-thread lists overflow and the second pass
    # counts them; the buffer keeps max_minimisers of them.
    ctx = native.Context(0)
    f = np.zeros((20, 20))
    st, res, _ = noalloc(native, f, 1000)
    assert st == native.OVERFLOW_MINIMISERS
    ref = native.exhaustive(f, ctx=ctx, max_minimisers=1000, allow_overflow=True)
    assert (res.energy, res.state, res.count, res.collect_passes) == (0.0, 0, 1 << 20, 2)
    assert res.count == ref.count
    ctx.close()


def test_noalloc_rejects_out_of_range_requests(native):
    f = random_int_qubo(10, 0)
    st, _, _ = noalloc(native, f, 65537)
    assert st == native.INVALID_ARG
    assert b"no-allocation limit" in native.lib().os_last_error()
    st, _, _ = noalloc(native, np.zeros((51, 51)), 16)
    assert st == native.INVALID_ARG
    st, _, _ = noalloc(native, np.random.default_rng(0).normal(size=(10, 10)), 16)
    assert st == native.INVALID_ARG
    assert b"integer coefficients only" in native.lib().os_last_error()
    st, _, _ = noalloc(native, f, 16, inner_bits=8)
    assert st == native.INVALID_ARG
    assert b"inner_bits" in native.lib().os_last_error()
    st, _, _ = noalloc(native, f, 16, variant=3)
    assert st == native.INVALID_ARG
    assert b"variant" in native.lib().os_last_error()
