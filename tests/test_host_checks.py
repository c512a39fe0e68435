"""Parameter checks of the annealing and exhaustive-search entry points, on
the CPU.

The C ABI validates a call's parameters before it touches the device, so the
checks run here with a null context: a bad parameter is INVALID_ARG with its
reason in os_last_error(), and a good set of parameters gets as far as the
context check ("null context"). The reference rejects the same schedules in
its CLI (app/one-solver-anneal.cpp:83-115) or fails inside the kernel.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest


def _params(native, beta, **kw):
    b = np.ascontiguousarray(beta, dtype=np.float64)
    prm = native._sa_params(b, kw.get("spb", 1), kw.get("tries", 4), 1, kw.get("acc", 1), kw.get("order", 1),
                            kw.get("resync", 0), None)
    return prm, b


def _dense_plan(native, f, beta, **kw):
    q, keep = native._dense(f)
    prm, b = _params(native, beta, **kw)
    h = C.c_void_p()
    st = native.lib().os_sa_plan_create_dense(None, C.byref(q), C.byref(prm), C.byref(h))
    return st, native.lib().os_last_error().decode()


@pytest.mark.parametrize("beta,kw,msg", [
    ([], {}, "empty beta schedule"),
    ([1.0, np.nan], {}, "beta[1] is NaN"),
    ([1.0], {"tries": 0}, "num_tries must be positive"),
    ([1.0], {"spb": 0}, "sweeps_per_beta must be positive"),
    ([1.0], {"acc": 7}, "unknown acceptance rule 7"),
    ([1.0], {"order": 3}, "unknown site order 3"),
    ([1.0], {"resync": -2}, "resync_every must be >= -1"),
])
def test_dense_plan_rejects_bad_schedules(native, beta, kw, msg):
    st, err = _dense_plan(native, np.eye(4), beta, **kw)
    assert st == native.INVALID_ARG and msg in err, err


def test_dense_plan_with_good_parameters_reaches_the_context(native):
    st, err = _dense_plan(native, np.eye(4), [0.5, 1.0], resync=-1)
    assert st == native.INVALID_ARG and "null context" in err


def test_sparse_plan_checks(native):
    csr = native.Csr.from_dense(np.array([[1.0, -2.0], [-2.0, 0.5]]))
    q = csr._c()
    L = native.lib()
    h = C.c_void_p()
    for kw, msg in [({"resync": -1}, "dense plans only"), ({"order": 0}, "site_order must be SEQUENTIAL"),
                    ({"tries": 0}, "num_tries")]:
        prm, b = _params(native, [1.0], **kw)
        st = L.os_sa_plan_create_sparse(None, C.byref(q), C.byref(prm), C.byref(h))
        assert st == native.INVALID_ARG and msg in L.os_last_error().decode()
    prm, b = _params(native, [1.0])
    st = L.os_sa_plan_create_sparse(None, C.byref(q), C.byref(prm), C.byref(h))
    assert st == native.INVALID_ARG and "null context" in L.os_last_error().decode()


def test_batched_plan_checks(native):
    L = native.lib()
    arr, fs = native._batch_inputs([np.eye(3), np.eye(5)])
    h = C.c_void_p()
    prm, b = _params(native, [1.0])
    st = L.os_sa_plan_create_batched(None, 0, arr, C.byref(prm), C.byref(h))
    assert st == native.INVALID_ARG and "empty batch" in L.os_last_error().decode()
    prm, b = _params(native, [1.0], resync=-1)
    st = L.os_sa_plan_create_batched(None, 2, arr, C.byref(prm), C.byref(h))
    assert st == native.INVALID_ARG and "dense plans only" in L.os_last_error().decode()
    prm, b = _params(native, [1.0])
    st = L.os_sa_plan_create_batched(None, 2, arr, C.byref(prm), C.byref(h))
    assert st == native.INVALID_ARG and "null context" in L.os_last_error().decode()


def _exh(native, f, **kw):
    q, keep = native._dense(f)
    prm = native._ExhParams(kw.get("kind", 0), kw.get("fixed", 0), kw.get("prefix", 0), kw.get("cap", 16),
                            kw.get("inner", 0), kw.get("variant", 0))
    h = C.c_void_p()
    st = native.lib().os_exhaustive_plan_create(None, C.byref(q), C.byref(prm), C.byref(h))
    return st, native.lib().os_last_error().decode()


@pytest.mark.parametrize("f,kw,msg", [
    (np.zeros((51, 51)), {}, "supports 1..50 variables"),
    (np.array([[1.0, np.inf], [np.inf, 0.0]]), {}, "coefficient (0,1) is not finite"),
    (np.eye(6), {"fixed": 6}, "fixed_high_bits must be in [0, n)"),
    (np.eye(6), {"fixed": 2, "prefix": 4}, "prefix does not fit"),
    (np.eye(6), {"prefix": 1}, "prefix given without fixed_high_bits"),
    (np.eye(6), {"inner": 8}, "inner_bits must be 0"),
    (np.eye(6), {"variant": 9}, "unknown variant 9"),
    (np.eye(6) * 0.5, {"kind": 1}, "not int32-exact"),
    (np.eye(6), {"kind": 9}, "unknown coef_kind 9"),
])
def test_exhaustive_plan_checks(native, f, kw, msg):
    st, err = _exh(native, f, **kw)
    assert st == native.INVALID_ARG and msg in err, err


def test_exhaustive_plan_with_good_parameters_reaches_the_context(native):
    st, err = _exh(native, np.eye(6), fixed=2, prefix=3)
    assert st == native.INVALID_ARG and "null context" in err
