"""onesolver_gb300: Python host API over the GB300 oneSolver C ABI.

The product is the native library ``lib/libonesolver.so`` (CUDA kernels for
sm_103a behind the C ABI declared in ``include/onesolver.h``). This module is
a thin ctypes mirror of that ABI and of the reference's user-facing calls:

* :class:`Model` -- ``qubo::QUBOModel::load`` and friends (the reference's
  ``include/model/qubo.hpp``), parsed by the library's C++ reader;
* :func:`exhaustive` -- ``exhaustive::solve`` (``include/exhaustive/exhaustive.hpp``);
* :func:`anneal` / :func:`anneal_sparse` -- ``sa::anneal``
  (``include/simulated_annealing/annealing.hpp``);
* :func:`linear_schedule` / :func:`geometric_schedule` -- the CLI's beta
  schedules (``app/one-solver-anneal.cpp:23-39``);
* :func:`temper_sparse` / :func:`population_anneal_sparse` -- parallel
  tempering and population annealing on the sparse sweep kernel (no reference
  counterpart; ``benchmarks/annealing/performance.md:52-59`` names them as the
  next solvers).

There is no CPU fallback: every solver call runs on the GPU through the native
library, and importing the library fails loudly when it has not been built.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import weakref
from dataclasses import dataclass, field
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "lib" / "libonesolver.so"

# os_status
OK, INVALID_ARG, CUDA_ERROR, TIMEOUT, OVERFLOW_MINIMISERS, NO_DEVICE, PARSE_ERROR, UNSUPPORTED = range(8)
# os_coef_kind
COEF_AUTO, COEF_INT32, COEF_INT64, COEF_FIXED64 = range(4)
# os_acceptance
ACCEPT_REFERENCE, ACCEPT_PHYSICAL = 0, 1
# os_site_order
SITES_RANDOM, SITES_SEQUENTIAL = 0, 1


class OneSolverError(RuntimeError):
    """A C ABI call returned a non-OK status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{_STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.message = message


class ParseError(OneSolverError, ValueError):
    """The .qubo text was rejected (the reference throws std::invalid_argument)."""


_STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "CUDA_ERROR", 3: "TIMEOUT", 4: "OVERFLOW_MINIMISERS",
                 5: "NO_DEVICE", 6: "PARSE_ERROR", 7: "UNSUPPORTED"}


class _QuboDense(C.Structure):
    _fields_ = [("n", C.c_int32), ("f", C.POINTER(C.c_double))]


class _QuboCsr(C.Structure):
    _fields_ = [("n", C.c_int32), ("row_ptr", C.POINTER(C.c_int32)), ("col", C.POINTER(C.c_int32)),
                ("val", C.POINTER(C.c_double)), ("diag", C.POINTER(C.c_double))]


class _ExhParams(C.Structure):
    _fields_ = [("coef_kind", C.c_int32), ("fixed_high_bits", C.c_int32), ("prefix", C.c_uint64),
                ("max_minimisers", C.c_uint64), ("inner_bits", C.c_int32), ("variant", C.c_int32)]


class _ExhResult(C.Structure):
    _fields_ = [("energy", C.c_double), ("state", C.c_uint64), ("count", C.c_uint64),
                ("states", C.POINTER(C.c_uint64)), ("states_enumerated", C.c_uint64),
                ("coef_kind_used", C.c_int32), ("collect_passes", C.c_int32)]


class _SaParams(C.Structure):
    _fields_ = [("beta", C.POINTER(C.c_double)), ("num_iter", C.c_int32), ("sweeps_per_beta", C.c_int32),
                ("num_tries", C.c_uint32), ("seed", C.c_uint64), ("acceptance", C.c_int32),
                ("site_order", C.c_int32), ("resync_every", C.c_int32), ("init_prob", C.POINTER(C.c_float))]


class _SaResult(C.Structure):
    _fields_ = [("state", C.c_char_p), ("energy", C.c_double), ("traj_energies", C.POINTER(C.c_double)),
                ("traj_states", C.c_char_p), ("max_field_drift", C.c_double), ("attempts", C.c_uint64),
                ("accepted", C.c_uint64)]


class _PtParams(C.Structure):
    _fields_ = [("beta", C.POINTER(C.c_double)), ("num_temps", C.c_int32), ("num_chains", C.c_uint32),
                ("num_rounds", C.c_int32), ("sweeps_per_round", C.c_int32), ("seed", C.c_uint64),
                ("resync_every", C.c_int32)]


class _PtResult(C.Structure):
    _fields_ = [("state", C.c_char_p), ("energy", C.c_double), ("chain_energies", C.POINTER(C.c_double)),
                ("final_temps", C.POINTER(C.c_int32)), ("final_energies", C.POINTER(C.c_double)),
                ("final_states", C.c_char_p), ("swaps_accepted", C.POINTER(C.c_uint64)),
                ("swaps_attempted", C.POINTER(C.c_uint64)), ("max_field_drift", C.c_double),
                ("attempts", C.c_uint64), ("accepted", C.c_uint64), ("device_ms", C.c_double)]


class _PaParams(C.Structure):
    _fields_ = [("beta", C.POINTER(C.c_double)), ("num_steps", C.c_int32), ("sweeps_per_beta", C.c_int32),
                ("population", C.c_uint32), ("seed", C.c_uint64), ("resync_every", C.c_int32)]


class _PaResult(C.Structure):
    _fields_ = [("state", C.c_char_p), ("energy", C.c_double), ("log_z", C.POINTER(C.c_double)),
                ("final_energies", C.POINTER(C.c_double)), ("final_states", C.c_char_p),
                ("families", C.c_uint32), ("max_field_drift", C.c_double), ("attempts", C.c_uint64),
                ("accepted", C.c_uint64), ("device_ms", C.c_double)]


_lib: Optional[C.CDLL] = None

# Every symbol of include/onesolver.h with (restype, argtypes).
_P = C.c_void_p
SIGNATURES = {
    "os_abi_version": (C.c_int32, []),
    "os_last_error": (C.c_char_p, []),
    "os_status_string": (C.c_char_p, [C.c_int]),
    "os_select_device": (C.c_int, [C.c_char_p, C.POINTER(C.c_int32)]),
    "os_device_name": (C.c_int, [C.c_int32, C.c_char_p, C.c_size_t]),
    "os_ctx_create": (C.c_int, [C.c_int32, C.POINTER(_P)]),
    "os_ctx_destroy": (C.c_int, [_P]),
    "os_ctx_set_stream": (C.c_int, [_P, _P]),
    "os_model_parse": (C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(_P)]),
    "os_model_load_file": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "os_model_free": (None, [_P]),
    "os_model_nodes": (C.c_int64, [_P]),
    "os_model_num_linear": (C.c_int64, [_P]),
    "os_model_num_quadratic": (C.c_int64, [_P]),
    "os_model_get_variable": (C.c_double, [_P, C.c_int32]),
    "os_model_get_connection": (C.c_double, [_P, C.c_int32, C.c_int32]),
    "os_model_flatten": (C.c_int, [_P, C.POINTER(C.c_double), C.c_size_t]),
    "os_model_str": (C.c_int, [_P, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "os_solution_csv": (C.c_int, [C.c_char_p, C.c_int32, C.c_double, C.c_char_p, C.c_size_t,
                                  C.POINTER(C.c_size_t)]),
    "os_ising_to_qubo_text": (C.c_int, [C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t),
                                        C.POINTER(C.c_double)]),
    "os_exhaustive_run": (C.c_int, [_P, C.POINTER(_QuboDense), C.POINTER(_ExhParams), C.POINTER(_ExhResult)]),
    "os_exhaustive_plan_create": (C.c_int, [_P, C.POINTER(_QuboDense), C.POINTER(_ExhParams), C.POINTER(_P)]),
    "os_exhaustive_plan_execute": (C.c_int, [_P]),
    "os_exhaustive_plan_result": (C.c_int, [_P, C.POINTER(_ExhResult)]),
    "os_exhaustive_plan_launches": (C.c_int32, [_P]),
    "os_exhaustive_plan_variant": (C.c_int32, [_P]),
    "os_exhaustive_plan_destroy": (None, [_P]),
    "os_exhaustive_plan_kernel_ms": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "os_exhaustive_run_noalloc": (C.c_int, [C.POINTER(_QuboDense), C.POINTER(_ExhParams), C.POINTER(_ExhResult),
                                            _P]),
    "os_sa_run": (C.c_int, [_P, C.POINTER(_QuboDense), C.POINTER(_SaParams), C.POINTER(_SaResult)]),
    "os_sa_run_sparse": (C.c_int, [_P, C.POINTER(_QuboCsr), C.POINTER(_SaParams), C.POINTER(_SaResult)]),
    "os_sa_verify": (C.c_int, [_P, C.POINTER(_QuboDense), C.POINTER(C.c_double), C.c_int32, C.c_int32,
                               C.c_uint32, C.c_int32, C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_double),
                               C.c_char_p, C.POINTER(C.c_double), C.c_char_p, C.POINTER(C.c_double),
                               C.POINTER(C.c_int64)]),
    "os_energy_batch": (C.c_int, [_P, C.POINTER(_QuboDense), C.c_char_p, C.c_int32, C.POINTER(C.c_double)]),
    "os_sa_plan_create_dense": (C.c_int, [_P, C.POINTER(_QuboDense), C.POINTER(_SaParams), C.POINTER(_P)]),
    "os_sa_plan_create_sparse": (C.c_int, [_P, C.POINTER(_QuboCsr), C.POINTER(_SaParams), C.POINTER(_P)]),
    "os_sa_plan_execute": (C.c_int, [_P]),
    "os_sa_plan_result": (C.c_int, [_P, C.POINTER(_SaResult)]),
    "os_sa_plan_launches": (C.c_int32, [_P]),
    "os_sa_plan_destroy": (None, [_P]),
    "os_sa_run_batched": (C.c_int, [_P, C.c_int32, C.POINTER(_QuboDense), C.POINTER(_SaParams),
                                    C.POINTER(_SaResult)]),
    "os_sa_plan_create_batched": (C.c_int, [_P, C.c_int32, C.POINTER(_QuboDense), C.POINTER(_SaParams),
                                            C.POINTER(_P)]),
    "os_sa_plan_result_batched": (C.c_int, [_P, C.POINTER(_SaResult)]),
    "os_sa_plan_tuned_warps": (C.c_int32, [_P]),
    "os_sa_plan_kernel_ms": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "os_sa_plan_set_replay": (C.c_int, [_P, _P]),
    "os_sa_plan_trajectories": (C.c_int, [_P, C.c_char_p, C.c_char_p, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double), C.POINTER(C.c_uint64)]),
    "os_sa_plan_sweep_order": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "os_pt_run_sparse": (C.c_int, [_P, C.POINTER(_QuboCsr), C.POINTER(_PtParams), C.POINTER(_PtResult)]),
    "os_pt_exchange_replay": (C.c_int, [_P, C.c_uint32, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.c_uint64, C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                        C.POINTER(C.c_uint64)]),
    "os_pa_run_sparse": (C.c_int, [_P, C.POINTER(_QuboCsr), C.POINTER(_PaParams), C.POINTER(_PaResult)]),
    "os_pa_resample_replay": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_double), C.c_double, C.c_uint64, C.c_int32,
                                        C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "os_philox_sample": (C.c_int, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_int32,
                                   C.POINTER(C.c_uint32)]),
    "os_mpnn_create": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(_P)]),
    "os_mpnn_destroy": (None, [_P]),
    "os_mpnn_num_params": (C.c_int64, [_P]),
    "os_mpnn_get_params": (C.c_int, [_P, C.POINTER(C.c_float), C.c_size_t]),
    "os_mpnn_set_params": (C.c_int, [_P, C.POINTER(C.c_float), C.c_size_t]),
    "os_mpnn_add_instance": (C.c_int, [_P, C.POINTER(_QuboDense), C.c_char_p, C.POINTER(C.c_int32)]),
    "os_mpnn_clear_instances": (C.c_int, [_P]),
    "os_mpnn_loss_grad": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_size_t]),
    "os_mpnn_train": (C.c_int, [_P, C.c_int32, C.c_float, C.c_uint64, C.POINTER(C.c_float)]),
    "os_mpnn_predict": (C.c_int, [_P, C.POINTER(_QuboDense), C.POINTER(C.c_float)]),
    "os_sa_plan_warm_start": (C.c_int, [_P, _P]),
    "os_probe_int32_peak": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "os_probe_exhaustive_pair": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_double)]),
    "os_probe_fp32_fma_peak": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "os_probe_smem_row_peak": (C.c_int, [_P, C.POINTER(C.c_double)]),
}


def lib() -> C.CDLL:
    """The loaded native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"`")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(status: int, cls=OneSolverError) -> None:
    if status != OK:
        msg = lib().os_last_error()
        raise cls(status, msg.decode() if msg else "")


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _dense(f: np.ndarray) -> tuple[_QuboDense, np.ndarray]:
    f = np.ascontiguousarray(f, dtype=np.float64)
    if f.ndim != 2 or f.shape[0] != f.shape[1]:
        raise ValueError("QUBO matrix must be square")
    return _QuboDense(f.shape[0], _dptr(f)), f


# --------------------------------------------------------------------------
# Devices and contexts
# --------------------------------------------------------------------------

def select_device(device_type: str) -> int:
    """devices::construct_device_selector (include/helpers/devices.hpp:27-42)."""
    out = C.c_int32(-1)
    st = lib().os_select_device(device_type.encode(), C.byref(out))
    _check(st)
    return out.value


def device_name(device: int = 0) -> str:
    buf = C.create_string_buffer(256)
    _check(lib().os_device_name(device, buf, 256))
    return buf.value.decode()


class Context:
    """One CUDA device and stream (the reference's sycl::queue)."""

    def __init__(self, device: int = 0):
        self._h = _P()
        self._children = weakref.WeakSet()
        _check(lib().os_ctx_create(device, C.byref(self._h)))
        self.device = device

    def _adopt(self, obj) -> None:
        """Plans and networks made on this context: close() closes them
        first (their device buffers are freed in order on its stream)."""
        self._children.add(obj)

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: Optional[int]) -> None:
        _check(lib().os_ctx_set_stream(self._h, _P(stream_ptr) if stream_ptr else None))

    def close(self) -> None:
        if self._h:
            for child in list(self._children):
                try:
                    child.close()
                except Exception:
                    pass
            lib().os_ctx_destroy(self._h)
            self._h = _P()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Optional[Context] = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


# --------------------------------------------------------------------------
# Model and IO
# --------------------------------------------------------------------------

class Model:
    """qubo::QUBOModel<int, double> as loaded by QUBOModel::load."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def parse(cls, text: str | bytes) -> "Model":
        data = text.encode() if isinstance(text, str) else bytes(text)
        h = _P()
        _check(lib().os_model_parse(data, len(data), C.byref(h)), ParseError)
        return cls(h)

    @classmethod
    def load(cls, path: str | os.PathLike) -> "Model":
        h = _P()
        st = lib().os_model_load_file(str(path).encode(), C.byref(h))
        _check(st, ParseError if st == PARSE_ERROR else OneSolverError)
        return cls(h)

    @property
    def nodes(self) -> int:
        return int(lib().os_model_nodes(self._h))

    @property
    def num_linear(self) -> int:
        return int(lib().os_model_num_linear(self._h))

    @property
    def num_quadratic(self) -> int:
        return int(lib().os_model_num_quadratic(self._h))

    def get_variable(self, i: int) -> float:
        return float(lib().os_model_get_variable(self._h, i))

    def get_connection(self, i: int, j: int) -> float:
        return float(lib().os_model_get_connection(self._h, i, j))

    def flatten(self) -> np.ndarray:
        """helpers::flatten_qubo: n x n symmetric matrix, diagonal = linear terms."""
        n = self.nodes
        out = np.zeros((n, n), dtype=np.float64)
        _check(lib().os_model_flatten(self._h, _dptr(out), out.size))
        return out

    def str(self) -> str:
        need = C.c_size_t(0)
        lib().os_model_str(self._h, None, 0, C.byref(need))
        buf = C.create_string_buffer(need.value + 1)
        _check(lib().os_model_str(self._h, buf, need.value + 1, C.byref(need)))
        return buf.value.decode()

    def __del__(self):
        try:
            if self._h:
                lib().os_model_free(self._h)
                self._h = None
        except Exception:
            pass


def ising_to_qubo_text(text: str) -> tuple[str, float]:
    """Ising COO text ("i j bias", 1-based) -> (QUBO text in the reference
    converter's format, offset) with E_ising(s) = E_qubo(x) + offset."""
    data = text.encode()
    need = C.c_size_t(0)
    off = C.c_double(0.0)
    _check(lib().os_ising_to_qubo_text(data, len(data), None, 0, C.byref(need), C.byref(off)))
    buf = C.create_string_buffer(need.value + 1)
    _check(lib().os_ising_to_qubo_text(data, len(data), buf, need.value + 1, C.byref(need), C.byref(off)))
    return buf.value.decode(), off.value


def solution_csv(state: Sequence[int], energy: float) -> str:
    """qubo::Solution::save: two-line CSV, energy at 6 significant digits."""
    s = bytes(bytearray(int(v) for v in state))
    need = C.c_size_t(0)
    lib().os_solution_csv(s, len(s), energy, None, 0, C.byref(need))
    buf = C.create_string_buffer(need.value + 1)
    _check(lib().os_solution_csv(s, len(s), energy, buf, need.value + 1, C.byref(need)))
    return buf.value.decode()


# --------------------------------------------------------------------------
# Schedules (app/one-solver-anneal.cpp:23-39, reproduced exactly)
# --------------------------------------------------------------------------

def linear_schedule(beta_min: float, beta_max: float, num_iter: int) -> np.ndarray:
    """beta_i = beta_min + beta_max * i / (num_iter - 1): ends at beta_min + beta_max."""
    out = np.empty(num_iter, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        for i in range(num_iter):
            den = float(num_iter - 1)
            out[i] = beta_min + (beta_max * i / den if den != 0.0 else (math.nan if i == 0 else math.inf))
    return out


def geometric_schedule(beta_min: float, beta_max: float, num_iter: int) -> np.ndarray:
    """Running FP64 product with alpha = (beta_max / beta_min) ** (1 / (num_iter - 1))."""
    out = np.empty(num_iter, dtype=np.float64)
    out[0] = beta_min
    if num_iter > 1:
        alpha = math.pow(beta_max / beta_min, 1.0 / (num_iter - 1))
        for i in range(1, num_iter):
            out[i] = out[i - 1] * alpha
    return out


# --------------------------------------------------------------------------
# Exhaustive search
# --------------------------------------------------------------------------

@dataclass
class ExhaustiveResult:
    energy: float
    state: int                  # smallest minimising state (the reference's answer)
    count: int                  # number of degenerate minimisers
    states: np.ndarray          # uint64, ascending (up to max_minimisers)
    states_enumerated: int
    coef_kind: int
    collect_passes: int
    status: int = OK

    def state_bits(self, n: int) -> list[int]:
        """helpers::ulong_to_vec: bit i = variable i."""
        return [(self.state >> i) & 1 for i in range(n)]


def _exh_params(coef_kind, fixed_high_bits, prefix, max_minimisers, inner_bits=0, variant=0) -> _ExhParams:
    return _ExhParams(coef_kind, fixed_high_bits, prefix, max_minimisers, inner_bits, variant)


def _exh_result(res: _ExhResult, states: np.ndarray, cap: int, status: int) -> ExhaustiveResult:
    k = min(int(res.count), cap)
    return ExhaustiveResult(res.energy, int(res.state), int(res.count), states[:k].copy(),
                            int(res.states_enumerated), int(res.coef_kind_used), int(res.collect_passes), status)


def exhaustive(f: np.ndarray, *, ctx: Optional[Context] = None, coef_kind: int = COEF_AUTO,
               fixed_high_bits: int = 0, prefix: int = 0, max_minimisers: int = 4096,
               allow_overflow: bool = False, inner_bits: int = 0, variant: int = 0) -> ExhaustiveResult:
    """exhaustive::solve on the GPU: ground energy, reference minimiser, degenerate set."""
    ctx = ctx or default_context()
    q, keep = _dense(f)
    states = np.zeros(max(max_minimisers, 1), dtype=np.uint64)
    res = _ExhResult()
    res.states = states.ctypes.data_as(C.POINTER(C.c_uint64))
    prm = _exh_params(coef_kind, fixed_high_bits, prefix, max_minimisers, inner_bits, variant)
    st = lib().os_exhaustive_run(ctx.handle, C.byref(q), C.byref(prm), C.byref(res))
    if st == OVERFLOW_MINIMISERS and allow_overflow:
        return _exh_result(res, states, max_minimisers, st)
    _check(st)
    return _exh_result(res, states, max_minimisers, st)


class ExhaustivePlan:
    """Device-resident exhaustive search (create / execute / result)."""

    def __init__(self, f: np.ndarray, *, ctx: Optional[Context] = None, coef_kind: int = COEF_AUTO,
                 fixed_high_bits: int = 0, prefix: int = 0, max_minimisers: int = 4096, inner_bits: int = 0,
                 variant: int = 0):
        self.ctx = ctx or default_context()
        self.ctx._adopt(self)
        q, self._keep = _dense(f)
        self.cap = max_minimisers
        self._h = _P()
        prm = _exh_params(coef_kind, fixed_high_bits, prefix, max_minimisers, inner_bits, variant)
        _check(lib().os_exhaustive_plan_create(self.ctx.handle, C.byref(q), C.byref(prm), C.byref(self._h)))

    def execute(self) -> None:
        _check(lib().os_exhaustive_plan_execute(self._h))

    @property
    def launches(self) -> int:
        return int(lib().os_exhaustive_plan_launches(self._h))

    @property
    def variant(self) -> int:
        """Instruction variant of the enumeration (0: one thread per state)."""
        return int(lib().os_exhaustive_plan_variant(self._h))

    def kernel_ms(self) -> float:
        """Device time of the last execute's enumeration kernel (CUDA events)."""
        v = C.c_float()
        _check(lib().os_exhaustive_plan_kernel_ms(self._h, C.byref(v)))
        return float(v.value)

    def result(self) -> ExhaustiveResult:
        states = np.zeros(max(self.cap, 1), dtype=np.uint64)
        res = _ExhResult()
        res.states = states.ctypes.data_as(C.POINTER(C.c_uint64))
        st = lib().os_exhaustive_plan_result(self._h, C.byref(res))
        if st not in (OK, OVERFLOW_MINIMISERS):
            _check(st)
        return _exh_result(res, states, self.cap, st)

    def close(self) -> None:
        if self._h:
            lib().os_exhaustive_plan_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------------------
# Simulated annealing
# --------------------------------------------------------------------------

@dataclass
class AnnealResult:
    state: np.ndarray           # uint8[n], best state over all trajectories
    energy: float               # its FP64 energy (reference energy function)
    traj_energies: np.ndarray   # float64[num_tries]
    traj_states: Optional[np.ndarray]
    max_field_drift: float
    attempts: int
    accepted: int


def _sa_params(beta: np.ndarray, sweeps_per_beta: int, num_tries: int, seed: int, acceptance: int,
               site_order: int, resync_every: int, init_prob: Optional[np.ndarray]) -> _SaParams:
    prm = _SaParams()
    prm.beta = _dptr(beta)
    prm.num_iter = len(beta)
    prm.sweeps_per_beta = sweeps_per_beta
    prm.num_tries = num_tries
    prm.seed = seed
    prm.acceptance = acceptance
    prm.site_order = site_order
    prm.resync_every = resync_every
    prm.init_prob = init_prob.ctypes.data_as(C.POINTER(C.c_float)) if init_prob is not None else None
    return prm


def _sa_result(n: int, T: int, traj_states: bool) -> tuple[_SaResult, dict]:
    keep = {"state": C.create_string_buffer(n), "e": np.zeros(T, dtype=np.float64)}
    res = _SaResult()
    res.state = C.cast(keep["state"], C.c_char_p)
    res.traj_energies = _dptr(keep["e"])
    if traj_states:
        keep["ts"] = C.create_string_buffer(n * T)
        res.traj_states = C.cast(keep["ts"], C.c_char_p)
    return res, keep


def _finish_sa(res: _SaResult, keep: dict, n: int, T: int) -> AnnealResult:
    state = np.frombuffer(keep["state"].raw[:n], dtype=np.uint8).copy()
    ts = np.frombuffer(keep["ts"].raw[: n * T], dtype=np.uint8).reshape(T, n).copy() if "ts" in keep else None
    return AnnealResult(state, res.energy, keep["e"].copy(), ts, res.max_field_drift, int(res.attempts),
                        int(res.accepted))


def anneal(f: np.ndarray, beta: Sequence[float], *, num_tries: int = 100, sweeps_per_beta: int = 1,
           seed: int = 1234, acceptance: int = ACCEPT_REFERENCE, site_order: int = SITES_RANDOM,
           resync_every: int = 0, init_prob: Optional[np.ndarray] = None, ctx: Optional[Context] = None,
           traj_states: bool = False) -> AnnealResult:
    """sa::anneal on the GPU (dense QUBO). Defaults follow the reference CLI."""
    ctx = ctx or default_context()
    q, keepf = _dense(f)
    n = q.n
    b = np.ascontiguousarray(beta, dtype=np.float64)
    ip = None if init_prob is None else np.ascontiguousarray(init_prob, dtype=np.float32)
    prm = _sa_params(b, sweeps_per_beta, num_tries, seed, acceptance, site_order, resync_every, ip)
    res, keep = _sa_result(n, num_tries, traj_states)
    _check(lib().os_sa_run(ctx.handle, C.byref(q), C.byref(prm), C.byref(res)))
    return _finish_sa(res, keep, n, num_tries)


@dataclass
class Csr:
    """Symmetric sparse QUBO: off-diagonal CSR (both triangles) + diagonal."""
    n: int
    row_ptr: np.ndarray
    col: np.ndarray
    val: np.ndarray
    diag: np.ndarray

    @classmethod
    def from_dense(cls, f: np.ndarray) -> "Csr":
        f = np.asarray(f, dtype=np.float64)
        n = f.shape[0]
        up = np.triu(f, 1)
        sym = up + up.T
        rows, cols = np.nonzero(sym)
        order = np.lexsort((cols, rows))
        rows, cols = rows[order], cols[order]
        rp = np.zeros(n + 1, dtype=np.int32)
        np.add.at(rp, rows + 1, 1)
        rp = np.cumsum(rp).astype(np.int32)
        return cls(n, rp, cols.astype(np.int32), sym[rows, cols].astype(np.float64), np.diag(f).copy())

    def to_dense(self) -> np.ndarray:
        f = np.zeros((self.n, self.n), dtype=np.float64)
        for i in range(self.n):
            for k in range(self.row_ptr[i], self.row_ptr[i + 1]):
                f[i, self.col[k]] = self.val[k]
        f[np.arange(self.n), np.arange(self.n)] = self.diag
        return f

    def _c(self) -> _QuboCsr:
        self.row_ptr = np.ascontiguousarray(self.row_ptr, dtype=np.int32)
        self.col = np.ascontiguousarray(self.col, dtype=np.int32)
        self.val = np.ascontiguousarray(self.val, dtype=np.float64)
        self.diag = np.ascontiguousarray(self.diag, dtype=np.float64)
        return _QuboCsr(self.n, self.row_ptr.ctypes.data_as(C.POINTER(C.c_int32)),
                        self.col.ctypes.data_as(C.POINTER(C.c_int32)), _dptr(self.val), _dptr(self.diag))


def anneal_sparse(csr: Csr, beta: Sequence[float], *, num_tries: int = 100, sweeps_per_beta: int = 1,
                  seed: int = 1234, acceptance: int = ACCEPT_PHYSICAL, resync_every: int = 0,
                  init_prob: Optional[np.ndarray] = None, ctx: Optional[Context] = None,
                  traj_states: bool = False) -> AnnealResult:
    """sa::anneal on a sparse QUBO with colour-parallel sweeps (sequential order)."""
    ctx = ctx or default_context()
    q = csr._c()
    b = np.ascontiguousarray(beta, dtype=np.float64)
    ip = None if init_prob is None else np.ascontiguousarray(init_prob, dtype=np.float32)
    prm = _sa_params(b, sweeps_per_beta, num_tries, seed, acceptance, SITES_SEQUENTIAL, resync_every, ip)
    res, keep = _sa_result(csr.n, num_tries, traj_states)
    _check(lib().os_sa_run_sparse(ctx.handle, C.byref(q), C.byref(prm), C.byref(res)))
    return _finish_sa(res, keep, csr.n, num_tries)


class _SaReplay(C.Structure):
    _fields_ = [("init", C.c_char_p), ("threshold", C.POINTER(C.c_float)), ("site", C.POINTER(C.c_int32))]


@dataclass
class Trajectories:
    """Per-trajectory state of a plan after its last execute (one instance)."""
    final_states: np.ndarray    # uint8[T, n]
    best_states: np.ndarray     # uint8[T, n]
    energies: np.ndarray        # float64[T], tracked energy of the final state
    best_energies: np.ndarray   # float64[T], best tracked energy
    accepted: np.ndarray        # uint64[T], accepted flips


class _PlanReplay:
    """Replay (verification) mode shared by the dense, sparse and batched plans:
    caller-given initial spins and per-attempt thresholds (random sites: and
    sites) in place of the Philox draws, the rest of the plan unchanged."""

    def _sizes(self) -> list:
        raise NotImplementedError

    def set_replay(self, init, threshold, site=None) -> None:
        """init: [T, n] 0/1 (batched: one array per instance); threshold:
        [T, steps, n] for sequential sweeps (batched: one per instance) or
        [T, steps] for random sites, float32 (the attempt accepts when
        dE < threshold); site: [T, steps] for random sites."""
        if isinstance(init, np.ndarray):
            init, threshold = [init], [threshold]
        self._rp_init = np.ascontiguousarray(np.concatenate([np.asarray(a, np.uint8).reshape(-1) for a in init]))
        self._rp_thr = np.ascontiguousarray(
            np.concatenate([np.asarray(a, np.float32).reshape(-1) for a in threshold]))
        self._rp_site = None if site is None else np.ascontiguousarray(site, dtype=np.int32)
        rp = _SaReplay(self._rp_init.ctypes.data_as(C.c_char_p),
                       self._rp_thr.ctypes.data_as(C.POINTER(C.c_float)),
                       None if self._rp_site is None else self._rp_site.ctypes.data_as(C.POINTER(C.c_int32)))
        _check(lib().os_sa_plan_set_replay(self._h, C.byref(rp)))

    def clear_replay(self) -> None:
        _check(lib().os_sa_plan_set_replay(self._h, None))

    def trajectories(self):
        """Trajectories of the last execute (a list, one per instance, for batched plans)."""
        sizes = self._sizes()
        T = self.T
        nv = T * sum(sizes)
        G = T * len(sizes)
        fs = C.create_string_buffer(max(nv, 1))
        bs = C.create_string_buffer(max(nv, 1))
        e = np.zeros(G)
        eb = np.zeros(G)
        acc = np.zeros(G, dtype=np.uint64)
        _check(lib().os_sa_plan_trajectories(self._h, C.cast(fs, C.c_char_p), C.cast(bs, C.c_char_p), _dptr(e),
                                             _dptr(eb), acc.ctypes.data_as(C.POINTER(C.c_uint64))))
        f_all = np.frombuffer(fs.raw[:nv], np.uint8)
        b_all = np.frombuffer(bs.raw[:nv], np.uint8)
        out, off = [], 0
        for k, n in enumerate(sizes):
            sl = slice(off, off + T * n)
            g = slice(k * T, (k + 1) * T)
            out.append(Trajectories(f_all[sl].reshape(T, n).copy(), b_all[sl].reshape(T, n).copy(), e[g].copy(),
                                    eb[g].copy(), acc[g].copy()))
            off += T * n
        return out if len(sizes) > 1 or isinstance(self, BatchedAnnealPlan) else out[0]

    def sweep_order(self):
        """Site order of one sequential sweep (a list per instance for batched plans)."""
        sizes = self._sizes()
        order = np.zeros(sum(sizes), dtype=np.int32)
        _check(lib().os_sa_plan_sweep_order(self._h, order.ctypes.data_as(C.POINTER(C.c_int32))))
        parts = np.split(order, np.cumsum(sizes)[:-1])
        return parts if isinstance(self, BatchedAnnealPlan) else parts[0]


class AnnealPlan(_PlanReplay):
    """Device-resident anneal (dense or sparse): create / execute / result."""

    def __init__(self, qubo, beta: Sequence[float], *, num_tries: int = 100, sweeps_per_beta: int = 1,
                 seed: int = 1234, acceptance: int = ACCEPT_PHYSICAL, site_order: int = SITES_SEQUENTIAL,
                 resync_every: int = 0, init_prob: Optional[np.ndarray] = None, ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()
        self.ctx._adopt(self)
        self.T = num_tries
        self._b = np.ascontiguousarray(beta, dtype=np.float64)
        self._ip = None if init_prob is None else np.ascontiguousarray(init_prob, dtype=np.float32)
        prm = _sa_params(self._b, sweeps_per_beta, num_tries, seed, acceptance, site_order, resync_every, self._ip)
        self._h = _P()
        if isinstance(qubo, Csr):
            self.n = qubo.n
            self._q = qubo
            _check(lib().os_sa_plan_create_sparse(self.ctx.handle, C.byref(qubo._c()), C.byref(prm),
                                                  C.byref(self._h)))
        else:
            q, self._f = _dense(qubo)
            self.n = q.n
            _check(lib().os_sa_plan_create_dense(self.ctx.handle, C.byref(q), C.byref(prm), C.byref(self._h)))

    def execute(self) -> None:
        _check(lib().os_sa_plan_execute(self._h))

    @property
    def launches(self) -> int:
        return int(lib().os_sa_plan_launches(self._h))

    @property
    def warps(self) -> int:
        """Trajectories per CTA of the sweep launches (autotuned for staged tiles)."""
        return int(lib().os_sa_plan_tuned_warps(self._h))

    def kernel_ms(self) -> float:
        """Device time of the last execute's sweep kernels (CUDA events)."""
        v = C.c_float()
        _check(lib().os_sa_plan_kernel_ms(self._h, C.byref(v)))
        return float(v.value)

    def result(self, traj_states: bool = False) -> AnnealResult:
        res, keep = _sa_result(self.n, self.T, traj_states)
        _check(lib().os_sa_plan_result(self._h, C.byref(res)))
        return _finish_sa(res, keep, self.n, self.T)

    def _sizes(self) -> list:
        return [self.n]

    def warm_start(self, net: "WarmStartNet") -> None:
        """Initial spins from the network's prediction on this plan's own
        (device-resident) matrix, for the next executes (dense plans)."""
        _check(lib().os_sa_plan_warm_start(self._h, net._h))

    def close(self) -> None:
        if self._h:
            lib().os_sa_plan_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class TemperResult:
    state: np.ndarray            # uint8[n], best state any replica visited
    energy: float                # its FP64 energy (reference energy function)
    chain_energies: np.ndarray   # float64[num_chains], best per chain
    final_temps: np.ndarray      # int32[num_chains, num_temps], temperature index of each replica
    final_energies: np.ndarray   # float64[num_chains, num_temps], FP64 energy of each final state
    final_states: Optional[np.ndarray]
    swaps_accepted: np.ndarray   # uint64[num_temps - 1]
    swaps_attempted: np.ndarray  # uint64[num_temps - 1]
    max_field_drift: float
    attempts: int
    accepted: int
    device_ms: float


def temper_sparse(csr: Csr, beta: Sequence[float], *, num_chains: int = 32, num_rounds: int = 100,
                  sweeps_per_round: int = 10, seed: int = 1234, resync_every: int = 0,
                  ctx: Optional[Context] = None, final_states: bool = False) -> TemperResult:
    """Parallel tempering on a sparse QUBO: num_chains chains of len(beta)
    replicas, sweeps_per_round colour-parallel sweeps per round at each
    replica's inverse temperature, then one even/odd round of adjacent
    exchanges. No reference counterpart (its annealing benchmark names
    parallel tempering as the next solver, benchmarks/annealing/performance.md:52-59)."""
    ctx = ctx or default_context()
    q = csr._c()
    b = np.ascontiguousarray(beta, dtype=np.float64)
    nt, n = len(b), csr.n
    prm = _PtParams(_dptr(b), nt, num_chains, num_rounds, sweeps_per_round, seed, resync_every)
    T = num_chains * nt
    state = C.create_string_buffer(n)
    ce = np.zeros(num_chains, dtype=np.float64)
    ft = np.zeros(T, dtype=np.int32)
    fe = np.zeros(T, dtype=np.float64)
    sa = np.zeros(max(nt - 1, 1), dtype=np.uint64)
    st = np.zeros(max(nt - 1, 1), dtype=np.uint64)
    fs = C.create_string_buffer(n * T) if final_states else None
    res = _PtResult()
    res.state = C.cast(state, C.c_char_p)
    res.chain_energies = _dptr(ce)
    res.final_temps = ft.ctypes.data_as(C.POINTER(C.c_int32))
    res.final_energies = _dptr(fe)
    res.final_states = C.cast(fs, C.c_char_p) if fs is not None else None
    res.swaps_accepted = sa.ctypes.data_as(C.POINTER(C.c_uint64))
    res.swaps_attempted = st.ctypes.data_as(C.POINTER(C.c_uint64))
    _check(lib().os_pt_run_sparse(ctx.handle, C.byref(q), C.byref(prm), C.byref(res)))
    return TemperResult(np.frombuffer(state.raw[:n], dtype=np.uint8).copy(), res.energy, ce,
                        ft.reshape(num_chains, nt), fe.reshape(num_chains, nt),
                        np.frombuffer(fs.raw[: n * T], dtype=np.uint8).reshape(num_chains, nt, n).copy()
                        if fs is not None else None,
                        sa[: nt - 1], st[: nt - 1], res.max_field_drift, int(res.attempts), int(res.accepted),
                        res.device_ms)


def pt_exchange_replay(beta: Sequence[float], energies: np.ndarray, temps: np.ndarray, *, seed: int = 1234,
                       round0: int = 0, num_rounds: int = 1, ctx: Optional[Context] = None):
    """The exchange step of temper_sparse alone, on the GPU, with fixed
    energies (chains x temps); returns (temps after the rounds, accepted
    exchanges per adjacent pair)."""
    ctx = ctx or default_context()
    b = np.ascontiguousarray(beta, dtype=np.float64)
    e = np.ascontiguousarray(energies, dtype=np.float64)
    t = np.ascontiguousarray(temps, dtype=np.int32).copy()
    chains, nt = t.shape
    sw = np.zeros(max(nt - 1, 1), dtype=np.uint64)
    _check(lib().os_pt_exchange_replay(ctx.handle, chains, nt, _dptr(b), _dptr(e), seed, round0, num_rounds,
                                       t.ctypes.data_as(C.POINTER(C.c_int32)),
                                       sw.ctypes.data_as(C.POINTER(C.c_uint64))))
    return t, sw[: nt - 1]


@dataclass
class PopulationResult:
    state: np.ndarray            # uint8[n], best state any replica visited
    energy: float                # its FP64 energy (reference energy function)
    log_z: np.ndarray            # float64[num_steps], ln Z(beta[k]) estimates
    final_energies: np.ndarray   # float64[population]
    final_states: Optional[np.ndarray]
    families: int                # initial replicas with descendants at the end
    max_field_drift: float
    attempts: int
    accepted: int
    device_ms: float


def population_anneal_sparse(csr: Csr, beta: Sequence[float], *, population: int = 4096, sweeps_per_beta: int = 5,
                             seed: int = 1234, resync_every: int = 0, ctx: Optional[Context] = None,
                             final_states: bool = False) -> PopulationResult:
    """Population annealing on a sparse QUBO: systematic resampling between
    consecutive inverse temperatures (from beta = 0), then sweeps_per_beta
    colour-parallel sweeps of every replica. No reference counterpart
    (benchmarks/annealing/performance.md:52-59 names it as a next solver)."""
    ctx = ctx or default_context()
    q = csr._c()
    b = np.ascontiguousarray(beta, dtype=np.float64)
    n = csr.n
    prm = _PaParams(_dptr(b), len(b), sweeps_per_beta, population, seed, resync_every)
    state = C.create_string_buffer(n)
    lz = np.zeros(len(b), dtype=np.float64)
    fe = np.zeros(population, dtype=np.float64)
    fs = C.create_string_buffer(n * population) if final_states else None
    res = _PaResult()
    res.state = C.cast(state, C.c_char_p)
    res.log_z = _dptr(lz)
    res.final_energies = _dptr(fe)
    res.final_states = C.cast(fs, C.c_char_p) if fs is not None else None
    _check(lib().os_pa_run_sparse(ctx.handle, C.byref(q), C.byref(prm), C.byref(res)))
    return PopulationResult(np.frombuffer(state.raw[:n], dtype=np.uint8).copy(), res.energy, lz, fe,
                            np.frombuffer(fs.raw[: n * population], dtype=np.uint8).reshape(population, n).copy()
                            if fs is not None else None,
                            int(res.families), res.max_field_drift, int(res.attempts), int(res.accepted),
                            res.device_ms)


def pa_resample_replay(energies: np.ndarray, dbeta: float, *, seed: int = 1234, step: int = 0,
                       ctx: Optional[Context] = None):
    """The resampling step of population_anneal_sparse alone, on the GPU;
    returns (parent of each slot, ln Q)."""
    ctx = ctx or default_context()
    e = np.ascontiguousarray(energies, dtype=np.float64)
    par = np.zeros(len(e), dtype=np.int32)
    lq = C.c_double()
    _check(lib().os_pa_resample_replay(ctx.handle, len(e), _dptr(e), dbeta, seed, step,
                                       par.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(lq)))
    return par, lq.value


def _batch_inputs(instances):
    fs = [np.ascontiguousarray(f, dtype=np.float64) for f in instances]
    arr = (_QuboDense * len(fs))()
    for k, f in enumerate(fs):
        if f.ndim != 2 or f.shape[0] != f.shape[1]:
            raise ValueError("QUBO matrices must be square")
        arr[k] = _QuboDense(f.shape[0], _dptr(f))
    return arr, fs


def _batch_results(fs, T, traj_states):
    res = (_SaResult * len(fs))()
    keeps = []
    for k, f in enumerate(fs):
        r, keep = _sa_result(f.shape[0], T, traj_states)
        res[k] = r
        keeps.append(keep)
    return res, keeps


def anneal_batched(instances, beta: Sequence[float], *, num_tries: int = 256, sweeps_per_beta: int = 1,
                   seed: int = 1234, acceptance: int = ACCEPT_PHYSICAL, resync_every: int = 0,
                   ctx: Optional[Context] = None, traj_states: bool = False) -> list:
    """Many dense instances (uneven n), one shared schedule, one persistent launch per chunk."""
    ctx = ctx or default_context()
    arr, fs = _batch_inputs(instances)
    b = np.ascontiguousarray(beta, dtype=np.float64)
    prm = _sa_params(b, sweeps_per_beta, num_tries, seed, acceptance, SITES_SEQUENTIAL, resync_every, None)
    res, keeps = _batch_results(fs, num_tries, traj_states)
    _check(lib().os_sa_run_batched(ctx.handle, len(fs), arr, C.byref(prm), res))
    return [_finish_sa(res[k], keeps[k], fs[k].shape[0], num_tries) for k in range(len(fs))]


class BatchedAnnealPlan(_PlanReplay):
    """Device-resident batched anneal: create (autotunes) / execute (graph replay) / result."""

    def __init__(self, instances, beta: Sequence[float], *, num_tries: int = 256, sweeps_per_beta: int = 1,
                 seed: int = 1234, acceptance: int = ACCEPT_PHYSICAL, resync_every: int = 0,
                 ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()
        self.ctx._adopt(self)
        self.T = num_tries
        self._arr, self._fs = _batch_inputs(instances)
        self._b = np.ascontiguousarray(beta, dtype=np.float64)
        prm = _sa_params(self._b, sweeps_per_beta, num_tries, seed, acceptance, SITES_SEQUENTIAL, resync_every,
                         None)
        self._h = _P()
        _check(lib().os_sa_plan_create_batched(self.ctx.handle, len(self._fs), self._arr, C.byref(prm),
                                               C.byref(self._h)))

    def execute(self) -> None:
        _check(lib().os_sa_plan_execute(self._h))

    @property
    def launches(self) -> int:
        return int(lib().os_sa_plan_launches(self._h))

    @property
    def warps(self) -> int:
        return int(lib().os_sa_plan_tuned_warps(self._h))

    def kernel_ms(self) -> float:
        v = C.c_float()
        _check(lib().os_sa_plan_kernel_ms(self._h, C.byref(v)))
        return float(v.value)

    def result(self, traj_states: bool = False) -> list:
        res, keeps = _batch_results(self._fs, self.T, traj_states)
        _check(lib().os_sa_plan_result_batched(self._h, res))
        return [_finish_sa(res[k], keeps[k], self._fs[k].shape[0], self.T) for k in range(len(self._fs))]

    def _sizes(self) -> list:
        return [f.shape[0] for f in self._fs]

    def close(self) -> None:
        if self._h:
            lib().os_sa_plan_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class VerifyResult:
    best_states: np.ndarray
    best_energies: np.ndarray
    final_states: np.ndarray
    final_energies: np.ndarray
    accept_count: np.ndarray


def sa_verify(f: np.ndarray, beta: Sequence[float], init: np.ndarray, site: np.ndarray, u: np.ndarray, *,
              sweeps_per_beta: int = 1, acceptance: int = ACCEPT_REFERENCE,
              ctx: Optional[Context] = None) -> VerifyResult:
    """Deterministic verification mode: the reference's Metropolis rule with given randoms."""
    ctx = ctx or default_context()
    q, keepf = _dense(f)
    n = q.n
    b = np.ascontiguousarray(beta, dtype=np.float64)
    init = np.ascontiguousarray(init, dtype=np.uint8)
    T = init.shape[0]
    site = np.ascontiguousarray(site, dtype=np.int32)
    u = np.ascontiguousarray(u, dtype=np.float64)
    bs = C.create_string_buffer(T * n)
    fs = C.create_string_buffer(T * n)
    be = np.zeros(T)
    fe = np.zeros(T)
    ac = np.zeros(T, dtype=np.int64)
    st = lib().os_sa_verify(ctx.handle, C.byref(q), _dptr(b), len(b), sweeps_per_beta, T, acceptance,
                            init.ctypes.data_as(C.c_char_p), site.ctypes.data_as(C.POINTER(C.c_int32)), _dptr(u),
                            C.cast(bs, C.c_char_p), _dptr(be), C.cast(fs, C.c_char_p), _dptr(fe),
                            ac.ctypes.data_as(C.POINTER(C.c_int64)))
    _check(st)
    return VerifyResult(np.frombuffer(bs.raw[: T * n], np.uint8).reshape(T, n).copy(), be,
                        np.frombuffer(fs.raw[: T * n], np.uint8).reshape(T, n).copy(), fe, ac)


def energy_batch(f: np.ndarray, states: np.ndarray, *, ctx: Optional[Context] = None) -> np.ndarray:
    """FP64 energies under the reference's energy function, computed on the GPU."""
    ctx = ctx or default_context()
    q, keepf = _dense(f)
    s = np.ascontiguousarray(states, dtype=np.uint8)
    m = s.shape[0]
    out = np.zeros(m)
    _check(lib().os_energy_batch(ctx.handle, C.byref(q), s.ctypes.data_as(C.c_char_p), m, _dptr(out)))
    return out


class WarmStartNet:
    """The learned warm start: message-passing network trained on the GPU.

    ``add(f, label)`` stages a training instance (label: the best state found,
    n 0/1 values), ``train(epochs, lr)`` runs Adam, ``predict(f)`` returns
    per-spin P(x_i = 1) for ``anneal(..., init_prob=...)``.
    """

    def __init__(self, *, hidden: int = 64, layers: int = 3, orient: bool = True, seed: int = 1,
                 ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()
        self.ctx._adopt(self)
        self._h = _P()
        self.orient = orient
        _check(lib().os_mpnn_create(self.ctx.handle, hidden, layers, int(orient), seed, C.byref(self._h)))
        self.num_params = int(lib().os_mpnn_num_params(self._h))
        self._keep = []

    def params(self) -> np.ndarray:
        out = np.zeros(self.num_params, dtype=np.float32)
        _check(lib().os_mpnn_get_params(self._h, out.ctypes.data_as(C.POINTER(C.c_float)), out.size))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().os_mpnn_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float)), p.size))

    def add(self, f: np.ndarray, label=None) -> int:
        q, keep = _dense(f)
        lab = None if label is None else bytes(bytearray(int(v) for v in label))
        idx = C.c_int32(-1)
        _check(lib().os_mpnn_add_instance(self._h, C.byref(q), lab, C.byref(idx)))
        return idx.value

    def clear(self) -> None:
        _check(lib().os_mpnn_clear_instances(self._h))

    def loss_grad(self, index: int):
        loss = C.c_float()
        g = np.zeros(self.num_params, dtype=np.float32)
        _check(lib().os_mpnn_loss_grad(self._h, index, C.byref(loss), g.ctypes.data_as(C.POINTER(C.c_float)), g.size))
        return float(loss.value), g

    def train(self, epochs: int, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        out = np.zeros(max(epochs, 1), dtype=np.float32)
        _check(lib().os_mpnn_train(self._h, epochs, lr, seed, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out[:epochs]

    def predict(self, f: np.ndarray) -> np.ndarray:
        q, keep = _dense(f)
        out = np.zeros(q.n, dtype=np.float32)
        _check(lib().os_mpnn_predict(self._h, C.byref(q), out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def close(self) -> None:
        if self._h:
            lib().os_mpnn_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def probe_int32_peak(ctx: Optional[Context] = None) -> float:
    """Measured INT32 (add + min) issue rate of this GPU, Gop/s."""
    ctx = ctx or default_context()
    v = C.c_double()
    _check(lib().os_probe_int32_peak(ctx.handle, C.byref(v)))
    return v.value


def probe_exhaustive_pair(variant: int, ctx: Optional[Context] = None) -> float:
    """States/s of exhaustive variant `variant`'s own inner block walk (1, 2
    or 3; 3 = packed, two states per add): the enumeration's instruction
    sequence without its per-item bookkeeping."""
    ctx = ctx or default_context()
    v = C.c_double()
    _check(lib().os_probe_exhaustive_pair(ctx.handle, variant, C.byref(v)))
    return float(v.value)


def probe_fp32_fma_peak(ctx: Optional[Context] = None) -> float:
    """Measured FP32 FMA rate of this GPU, GFLOP/s."""
    ctx = ctx or default_context()
    v = C.c_double()
    _check(lib().os_probe_fp32_fma_peak(ctx.handle, C.byref(v)))
    return v.value


def probe_smem_row_peak(ctx: Optional[Context] = None) -> float:
    """Measured shared-memory read rate of the dense field update (128-bit
    shared loads feeding paired FP32 FMAs), GB/s."""
    ctx = ctx or default_context()
    v = C.c_double()
    _check(lib().os_probe_smem_row_peak(ctx.handle, C.byref(v)))
    return v.value


def philox_sample(ctr: Sequence[int], key: Sequence[int], count: int, *, ctx: Optional[Context] = None) -> np.ndarray:
    """Device Philox4x32-10 words for `count` consecutive counters (ctr[0] += i)."""
    ctx = ctx or default_context()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    out = np.zeros(4 * count, dtype=np.uint32)
    _check(lib().os_philox_sample(ctx.handle, c, k, count, out.ctypes.data_as(C.POINTER(C.c_uint32))))
    return out.reshape(count, 4)
