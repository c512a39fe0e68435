"""Oracle: CPU restatement of oneSolver's hot paths (test infrastructure only).

Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs, as the checker and as the timed reference algorithm. The
product library never imports or links it. The functions wrap
oracle/_build/liboracle.so (built from oracle/oracle.cpp by oracle/Makefile);
each C function cites the reference code it restates.

Parity pin: the reference cannot be compiled here (SYCL, Boost and oneMKL are
absent), so this restatement is pinned against the reference's own
known-answer tests (tests/exhaustive_test.cpp golden energies,
tests/qubo_helpers_test.cpp flatten layout, tests/io_test.cpp CSV bytes);
see tests/test_oracle_golden.py.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path
from typing import Optional

import numpy as np

_DIR = Path(__file__).resolve().parent
SO = _DIR / "_build" / "liboracle.so"
_lib: Optional[C.CDLL] = None

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_U64 = C.POINTER(C.c_uint64)


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(_DIR)], check=True)
    return SO


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not SO.exists():
            build()
        L = C.CDLL(str(SO))
        L.orc_flatten.argtypes = [C.c_int, C.c_int, _I, _D, C.c_int, _I, _I, _D, _D]
        L.orc_flatten.restype = None
        L.orc_energy.argtypes = [_D, C.c_char_p, C.c_int]
        L.orc_energy.restype = C.c_double
        L.orc_energy_batch.argtypes = [_D, C.c_char_p, C.c_int, C.c_int, _D]
        L.orc_energy_batch.restype = None
        L.orc_energy_bits.argtypes = [_D, C.c_int, C.c_uint64]
        L.orc_energy_bits.restype = C.c_double
        L.orc_schedule_linear.argtypes = [_D, C.c_double, C.c_double, C.c_uint]
        L.orc_schedule_linear.restype = None
        L.orc_schedule_geometric.argtypes = [_D, C.c_double, C.c_double, C.c_uint]
        L.orc_schedule_geometric.restype = None
        L.orc_exhaustive.argtypes = [_D, C.c_int, C.c_uint64, C.c_uint64, C.c_int, _D, _U64]
        L.orc_exhaustive.restype = None
        L.orc_exhaustive_all.argtypes = [_D, C.c_int, C.c_uint64, C.c_uint64, C.c_int, _D, _U64, C.c_uint64]
        L.orc_exhaustive_all.restype = C.c_uint64
        L.orc_exhaustive_int_all.argtypes = [_D, C.c_int, C.c_uint64, C.c_uint64, C.c_int,
                                             C.POINTER(C.c_int64), _U64, C.c_uint64]
        L.orc_exhaustive_int_all.restype = C.c_int64
        L.orc_anneal_verify.argtypes = [_D, C.c_int, _D, C.c_int, C.c_int, C.c_int, C.c_char_p, _I, _D, C.c_int,
                                        C.c_char_p, _D, C.c_char_p, _D, C.POINTER(C.c_int64)]
        L.orc_anneal_verify.restype = None
        L.orc_anneal_free.argtypes = [_D, C.c_int, _D, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_int, C.c_int,
                                      C.c_int, C.c_char_p, _D]
        L.orc_anneal_free.restype = C.c_int64
        L.orc_sa_replay.argtypes = [_D, C.c_int, _D, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _I,
                                    C.c_char_p, _I, _D, C.c_int, C.c_int, C.c_char_p, C.c_char_p, _D, _D,
                                    C.POINTER(C.c_int64)]
        L.orc_sa_replay.restype = None
        L.orc_anneal_free_fields.argtypes = [_D, C.c_int, _D, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_int,
                                             C.c_int, _I, C.c_int, C.c_int, C.c_char_p, _D]
        L.orc_anneal_free_fields.restype = C.c_int64
        L.orc_argmin.argtypes = [_D, C.c_int]
        L.orc_argmin.restype = C.c_int
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_philox4x32_10.restype = None
        L.orc_pt_exchange.argtypes = [C.c_int, C.c_int, _D, _D, C.c_uint64, C.c_int, C.c_int, _I, _U64]
        L.orc_pt_exchange.restype = None
        L.orc_pa_resample.argtypes = [C.c_int, _D, C.c_double, C.c_uint64, C.c_int, _I, _D]
        L.orc_pa_resample.restype = None
        L.orc_solution_csv.argtypes = [C.c_char_p, C.c_int, C.c_double, C.c_char_p, C.c_int]
        L.orc_solution_csv.restype = C.c_int
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_D)


def flatten(n: int, linear: dict, quadratic: dict) -> np.ndarray:
    """helpers::flatten_qubo from the model's coefficient maps."""
    li = np.array(list(linear.keys()), dtype=np.int32)
    lv = np.array(list(linear.values()), dtype=np.float64)
    qi = np.array([k[0] for k in quadratic], dtype=np.int32)
    qj = np.array([k[1] for k in quadratic], dtype=np.int32)
    qv = np.array(list(quadratic.values()), dtype=np.float64)
    out = np.zeros(n * n)
    lib().orc_flatten(n, len(li), li.ctypes.data_as(_I), _d(lv), len(qi), qi.ctypes.data_as(_I),
                      qj.ctypes.data_as(_I), _d(qv), _d(out))
    return out.reshape(n, n)


def energy(f: np.ndarray, state) -> float:
    f = np.ascontiguousarray(f, dtype=np.float64)
    s = bytes(bytearray(int(v) for v in state))
    return lib().orc_energy(_d(f), s, f.shape[0])


def energy_batch(f: np.ndarray, states: np.ndarray) -> np.ndarray:
    f = np.ascontiguousarray(f, dtype=np.float64)
    s = np.ascontiguousarray(states, dtype=np.uint8)
    out = np.zeros(s.shape[0])
    lib().orc_energy_batch(_d(f), s.ctypes.data_as(C.c_char_p), f.shape[0], s.shape[0], _d(out))
    return out


def energy_bits(f: np.ndarray, state: int) -> float:
    f = np.ascontiguousarray(f, dtype=np.float64)
    return lib().orc_energy_bits(_d(f), f.shape[0], int(state))


def schedule_linear(beta_min: float, beta_max: float, num_iter: int) -> np.ndarray:
    out = np.zeros(num_iter)
    lib().orc_schedule_linear(_d(out), beta_min, beta_max, num_iter)
    return out


def schedule_geometric(beta_min: float, beta_max: float, num_iter: int) -> np.ndarray:
    out = np.zeros(num_iter)
    lib().orc_schedule_geometric(_d(out), beta_min, beta_max, num_iter)
    return out


def exhaustive(f: np.ndarray, begin: int = 0, end: Optional[int] = None, threads: int = 0):
    """The reference's exhaustive scan over [begin, end): (energy, first minimising state)."""
    f = np.ascontiguousarray(f, dtype=np.float64)
    n = f.shape[0]
    end = (1 << n) if end is None else end
    threads = threads or min(16, os.cpu_count() or 1)
    e = C.c_double()
    s = C.c_uint64()
    lib().orc_exhaustive(_d(f), n, begin, end, threads, C.byref(e), C.byref(s))
    return e.value, s.value


def exhaustive_all(f: np.ndarray, begin: int = 0, end: Optional[int] = None, threads: int = 0, cap: int = 1 << 16):
    """(energy, count, ascending minimisers) under the reference's FP64 energy."""
    f = np.ascontiguousarray(f, dtype=np.float64)
    n = f.shape[0]
    end = (1 << n) if end is None else end
    threads = threads or min(16, os.cpu_count() or 1)
    e = C.c_double()
    states = np.zeros(cap, dtype=np.uint64)
    count = lib().orc_exhaustive_all(_d(f), n, begin, end, threads, C.byref(e), states.ctypes.data_as(_U64), cap)
    return e.value, int(count), np.sort(states[: min(count, cap)])


def exhaustive_int_all(f: np.ndarray, begin: int = 0, end: Optional[int] = None, threads: int = 0,
                       cap: int = 1 << 16):
    """(energy, count, ascending minimisers) of an integer-coefficient QUBO, every
    state's energy evaluated on its own from per-row byte tables (exact in int64)."""
    f = np.ascontiguousarray(f, dtype=np.float64)
    n = f.shape[0]
    end = (1 << n) if end is None else end
    threads = threads or (os.cpu_count() or 1)
    e = C.c_int64()
    states = np.zeros(max(cap, 1), dtype=np.uint64)
    count = lib().orc_exhaustive_int_all(_d(f), n, begin, end, threads, C.byref(e),
                                         states.ctypes.data_as(_U64), cap)
    if count < 0:
        raise ValueError("exhaustive_int_all needs integer coefficients (|q| < 2^40) and 1 <= n <= 63")
    return float(e.value), int(count), states[: min(count, cap)].copy()


def anneal_verify(f, beta, init, site, u, sweeps_per_beta=1, acceptance=0):
    f = np.ascontiguousarray(f, dtype=np.float64)
    n = f.shape[0]
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    init = np.ascontiguousarray(init, dtype=np.uint8)
    T = init.shape[0]
    site = np.ascontiguousarray(site, dtype=np.int32)
    u = np.ascontiguousarray(u, dtype=np.float64)
    bs = C.create_string_buffer(T * n)
    fs = C.create_string_buffer(T * n)
    be = np.zeros(T)
    fe = np.zeros(T)
    ac = np.zeros(T, dtype=np.int64)
    lib().orc_anneal_verify(_d(f), n, _d(beta), len(beta), T, sweeps_per_beta, init.ctypes.data_as(C.c_char_p),
                            site.ctypes.data_as(_I), _d(u), acceptance, C.cast(bs, C.c_char_p), _d(be),
                            C.cast(fs, C.c_char_p), _d(fe), ac.ctypes.data_as(C.POINTER(C.c_int64)))
    return (np.frombuffer(bs.raw[: T * n], np.uint8).reshape(T, n).copy(), be,
            np.frombuffer(fs.raw[: T * n], np.uint8).reshape(T, n).copy(), fe, ac)


def anneal_free(f, beta, num_tries, sweeps_per_beta=1, seed=1, acceptance=0, site_order=0, threads=0):
    """Free-running reference-algorithm anneal on host cores: (best states, best energies, attempts)."""
    f = np.ascontiguousarray(f, dtype=np.float64)
    n = f.shape[0]
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    threads = threads or min(16, os.cpu_count() or 1)
    bs = C.create_string_buffer(num_tries * n)
    be = np.zeros(num_tries)
    att = lib().orc_anneal_free(_d(f), n, _d(beta), len(beta), num_tries, sweeps_per_beta, seed, acceptance,
                                site_order, threads, C.cast(bs, C.c_char_p), _d(be))
    return np.frombuffer(bs.raw[: num_tries * n], np.uint8).reshape(num_tries, n).copy(), be, int(att)


def anneal_free_fields(f, beta, num_tries, sweeps_per_beta=1, seed=1, acceptance=0, site_order=0, order=None,
                       best_at_sweep_end=False, threads=0):
    """The free-running reference chain with FP64 local fields and a given
    sweep order (orc_anneal_free_fields): (best states, best energies, attempts)."""
    f = np.ascontiguousarray(f, dtype=np.float64)
    n = f.shape[0]
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    threads = threads or (os.cpu_count() or 1)
    order_a = None if order is None else np.ascontiguousarray(order, dtype=np.int32)
    bs = C.create_string_buffer(num_tries * n)
    be = np.zeros(num_tries)
    att = lib().orc_anneal_free_fields(_d(f), n, _d(beta), len(beta), sweeps_per_beta, num_tries, seed, acceptance,
                                       site_order, None if order_a is None else order_a.ctypes.data_as(_I),
                                       1 if best_at_sweep_end else 0, threads, C.cast(bs, C.c_char_p), _d(be))
    return np.frombuffer(bs.raw[: num_tries * n], np.uint8).reshape(num_tries, n).copy(), be, int(att)


def sa_replay(f, beta, init, u, *, sweeps_per_beta=1, acceptance=0, mode=1, order=None, site=None,
              full_energy=False, threads=0):
    """The reference's Metropolis loop (annealing.hpp:97-123) on given randoms in a
    given site order (orc_sa_replay): mode 0 random sites (site [T, S], u [T, S]),
    1 sequential sweeps in `order` with the best state checked after every
    attempt, 2 the same with the best state checked at the end of every sweep
    (u [T, S, n] by site). Returns (final_states, best_states, final_energies,
    best_energies, accepted)."""
    f = np.ascontiguousarray(f, dtype=np.float64)
    n = f.shape[0]
    beta = np.ascontiguousarray(beta, dtype=np.float64)
    init = np.ascontiguousarray(init, dtype=np.uint8)
    T = init.shape[0]
    u = np.ascontiguousarray(u, dtype=np.float64)
    order_a = np.ascontiguousarray(np.arange(n) if order is None else order, dtype=np.int32)
    site_a = np.ascontiguousarray(np.zeros(1) if site is None else site, dtype=np.int32)
    threads = threads or min(16, os.cpu_count() or 1)
    fs = C.create_string_buffer(T * n)
    bs = C.create_string_buffer(T * n)
    fe = np.zeros(T)
    be = np.zeros(T)
    ac = np.zeros(T, dtype=np.int64)
    lib().orc_sa_replay(_d(f), n, _d(beta), len(beta), sweeps_per_beta, T, acceptance, mode,
                        order_a.ctypes.data_as(_I), init.ctypes.data_as(C.c_char_p), site_a.ctypes.data_as(_I),
                        _d(u), 1 if full_energy else 0, threads, C.cast(fs, C.c_char_p), C.cast(bs, C.c_char_p),
                        _d(fe), _d(be), ac.ctypes.data_as(C.POINTER(C.c_int64)))
    return (np.frombuffer(fs.raw[: T * n], np.uint8).reshape(T, n).copy(),
            np.frombuffer(bs.raw[: T * n], np.uint8).reshape(T, n).copy(), fe, be, ac)


def philox(ctr, key) -> list[int]:
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


def pt_exchange(beta, energies, seed: int, round0: int, rounds: int, temps):
    """Replica-exchange rounds with fixed energies (energies, temps: chains x nt);
    returns (temps after the rounds, accepted exchanges per adjacent pair)."""
    b = np.ascontiguousarray(beta, dtype=np.float64)
    e = np.ascontiguousarray(energies, dtype=np.float64)
    t = np.ascontiguousarray(temps, dtype=np.int32).copy()
    chains, nt = t.shape
    sw = np.zeros(max(nt - 1, 1), dtype=np.uint64)
    lib().orc_pt_exchange(chains, nt, _d(b), _d(e), seed, round0, rounds,
                          t.ctypes.data_as(_I), sw.ctypes.data_as(_U64))
    return t, sw[: nt - 1]


def pa_resample(energies, dbeta: float, seed: int, step: int):
    """One systematic resampling step; returns (parent of each slot, ln Q)."""
    e = np.ascontiguousarray(energies, dtype=np.float64)
    par = np.zeros(len(e), dtype=np.int32)
    lq = C.c_double()
    lib().orc_pa_resample(len(e), _d(e), dbeta, seed, step, par.ctypes.data_as(_I), C.byref(lq))
    return par, lq.value


def solution_csv(state, energy_value: float) -> str:
    s = bytes(bytearray(int(v) for v in state))
    buf = C.create_string_buffer(1 << 16)
    k = lib().orc_solution_csv(s, len(s), energy_value, buf, 1 << 16)
    return buf.raw[:k].decode()
