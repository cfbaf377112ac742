"""ctypes binding of the C ABI in include/pgx.h (libpgx.so, built in-tree).

There is deliberately no fallback: if the library is missing or no GB300 can
be opened, every call raises. Status codes map onto Python exceptions the way
pagmo's C++ exceptions map in pygmo: PGX_ERR_INVALID -> ValueError (pagmo's
std::invalid_argument), PGX_ERR_CAPACITY -> OverflowError, PGX_ERR_TIMEOUT ->
TimeoutError, CUDA / no device -> RuntimeError.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libpgx.so"

OK, ERR_INVALID, ERR_CUDA, ERR_TIMEOUT, ERR_CAPACITY, ERR_NODEVICE, ERR_NOTIMPL = 0, 1, 2, 3, 4, 5, 6
RASTRIGIN, ROSENBROCK, LENNARD_JONES, ACKLEY, GRIEWANK, SCHWEFEL = 1, 2, 3, 4, 5, 6
ZDT, DTLZ = 7, 8
HS71 = 9
UNCONSTRAIN_METHODS = {"death penalty": 0, "kuri": 1, "weighted": 2, "ignore_c": 3, "ignore_o": 4}

# Exported symbols and their signatures (kept in step with include/pgx.h).
_vp, _u64, _i32, _d = C.c_void_p, C.c_uint64, C.c_int32, C.c_double
SIGNATURES = {
    "pgx_abi_version": (C.c_int, []),
    "pgx_build_id": (C.c_char_p, []),
    "pgx_last_error": (C.c_char_p, []),
    "pgx_context_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "pgx_context_destroy": (None, [_vp]),
    "pgx_context_launch_count": (_u64, [_vp]),
    "pgx_problem_nx": (C.c_int, [C.c_int, _u64, C.POINTER(_u64)]),
    "pgx_problem_bounds": (C.c_int, [C.c_int, _u64, _vp, _vp]),
    "pgx_batch_fitness": (C.c_int, [_vp, C.c_int, _u64, _vp, _u64, _vp]),
    "pgx_batch_gradient": (C.c_int, [_vp, C.c_int, _u64, _vp, _u64, _vp, _vp]),
    "pgx_batch_eval_device": (C.c_int, [_vp, C.c_int, _u64, _vp, _u64, _vp, _vp, _vp]),
    "pgx_fnds": (C.c_int, [_vp, _vp, _u64, _u64, _vp, _vp, _vp, _vp, _vp]),
    "pgx_fnds_dom_list": (C.c_int, [_vp, _vp, _u64, _u64, _vp, _vp, _u64, C.POINTER(_u64)]),
    "pgx_crowding_distance": (C.c_int, [_vp, _vp, _u64, _u64, _vp]),
    "pgx_select_best_n_mo": (C.c_int, [_vp, _vp, _u64, _u64, _u64, _vp, C.POINTER(_u64)]),
    "pgx_sort_population_mo": (C.c_int, [_vp, _vp, _u64, _u64, _vp]),
    "pgx_select_best_n_mo_device": (C.c_int, [_vp, _vp, _u64, _u64, _u64, _vp, _vp, _vp]),
    "pgx_sort_population_mo_device": (C.c_int, [_vp, _vp, _u64, _u64, _vp, _vp, _vp]),
    "pgx_std_sort_i64": (C.c_int, [_vp, _vp, _vp, _u64]),
    "pgx_nsga2_survival": (C.c_int, [_vp, _vp, _u64, _u64, _vp, _vp, _vp, _vp, _vp, _vp]),
    "pgx_nsga2_survival_device": (C.c_int, [_vp, _vp, _u64, _u64, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "pgx_measure_fp64_peak": (C.c_int, [_vp, C.POINTER(C.c_double)]),
    "pgx_refine_batch": (C.c_int, [_vp, C.c_int, _u64, _vp, _vp, _u64, _vp, _vp]),
    "pgx_refine_batch_device": (C.c_int, [_vp, C.c_int, _u64, _vp, _vp, _u64, _vp, _vp, _vp]),
    "pgx_nsga2_survival_device_noalloc": (C.c_int, [_vp, _u64, _u64, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "pgx_epoch_create": (C.c_int, [_vp, _vp, C.c_int, C.POINTER(_vp)]),
    "pgx_epoch_run": (C.c_int, [_vp, _vp]),
    "pgx_epoch_submit": (C.c_int, [_vp, _vp]),
    "pgx_epoch_collect": (C.c_int, [_vp]),
    "pgx_epoch_launch_device": (C.c_int, [_vp, _vp]),
    "pgx_epoch_info": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), C.POINTER(_u64)]),
    "pgx_epoch_destroy": (None, [_vp]),
    "pgx_requests_run_plain": (C.c_int, [_vp, _vp, C.c_int]),
    "pgx_mo_problem_dims": (C.c_int, [_vp, C.POINTER(_u64), C.POINTER(_u64), C.POINTER(_u64)]),
    "pgx_mo_problem_bounds": (C.c_int, [_vp, _vp, _vp]),
    "pgx_mo_batch_fitness": (C.c_int, [_vp, _vp, _vp, _u64, _vp]),
    "pgx_mo_batch_fitness_device": (C.c_int, [_vp, _vp, _vp, _u64, _vp, _vp]),
    "pgx_mo_p_distance": (C.c_int, [_vp, _vp, _vp, _u64, _vp]),
    "pgx_selftest_barrier_timeout": (C.c_int, [_vp, _u64, C.POINTER(C.c_int32)]),
    "pgx_selftest_lj_reciprocal": (C.c_int, [_vp, _vp, _u64, _vp, _vp]),
    "pgx_hypervolume": (C.c_int, [_vp, _vp, _u64, _u64, _vp, C.POINTER(C.c_double)]),
    "pgx_hypervolume_device": (C.c_int, [_vp, _vp, _u64, _u64, _vp, _vp, _vp]),
    "pgx_constrained_dims": (C.c_int, [C.c_int, _u64, _vp, _vp, _vp, _vp]),
    "pgx_constrained_bounds": (C.c_int, [C.c_int, _u64, _vp, _vp]),
    "pgx_constrained_batch_fitness": (C.c_int, [_vp, C.c_int, _u64, _vp, _u64, _vp]),
    "pgx_unconstrain_batch_fitness": (C.c_int, [_vp, C.c_int, _u64, _vp, _vp, _u64, _vp]),
    "pgx_hypervolume_exclusive": (C.c_int, [_vp, _vp, _u64, _u64, _vp, _u64, C.POINTER(C.c_double)]),
    "pgx_hypervolume_contributions": (C.c_int, [_vp, _vp, _u64, _u64, _vp, _vp]),
    "pgx_hypervolume_contributions_device": (C.c_int, [_vp, _vp, _u64, _u64, _vp, _vp, _vp]),
    "pgx_hypervolume_extreme_contributor": (C.c_int, [_vp, _vp, _u64, _u64, _vp, C.c_int, C.POINTER(_u64)]),
}


class pgx_request(C.Structure):
    """struct pgx_request of include/pgx.h."""
    _fields_ = [("kind", C.c_int), ("param", C.c_uint64), ("n_dvs", C.c_uint64), ("dvs", C.c_void_p),
                ("fvs", C.c_void_p), ("grads", C.c_void_p)]


class pgx_mo_problem(C.Structure):
    """struct pgx_mo_problem of include/pgx.h: zdt(prob_id, param) or dtlz(prob_id, dim=param, fdim, alpha)."""
    _fields_ = [("kind", C.c_int), ("prob_id", C.c_uint32), ("param", C.c_uint64), ("fdim", C.c_uint64),
                ("alpha", C.c_uint32)]


class pgx_unconstrain(C.Structure):
    """struct pgx_unconstrain of include/pgx.h: unconstrain's method code, weights and the inner tolerances."""
    _fields_ = [("method", C.c_int), ("weights", C.c_void_p), ("n_weights", C.c_uint64), ("c_tol", C.c_void_p)]


class pgx_refine_params(C.Structure):
    """struct pgx_refine_params of include/pgx.h."""
    _fields_ = [("hops", C.c_uint32), ("stop", C.c_uint32), ("steps", C.c_uint32), ("perturb", C.c_double),
                ("step0", C.c_double), ("step_min", C.c_double), ("seed", C.c_uint64)]


_lib = None
_lib_lock = threading.Lock()


def lib() -> C.CDLL:
    """The loaded libpgx.so (raises if it has not been built)."""
    global _lib
    with _lib_lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"libpgx.so not found at {LIB_PATH}; build it with `python -m pagmo2_gb300.build` "
                    "(there is no CPU fallback)")
            h = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(h, name)
                fn.restype = res
                fn.argtypes = args
            _lib = h
        return _lib


def last_error() -> str:
    m = lib().pgx_last_error()
    return m.decode() if m else ""


def check(status: int) -> None:
    if status == OK:
        return
    msg = last_error()
    if status == ERR_INVALID:
        raise ValueError(msg)
    if status == ERR_CAPACITY:
        raise OverflowError(msg)
    if status == ERR_TIMEOUT:
        raise TimeoutError(msg)
    if status == ERR_NOTIMPL:
        raise NotImplementedError(msg)
    raise RuntimeError(msg or f"pgx status {status}")


def ptr(a: np.ndarray | None) -> int | None:
    if a is None:
        return None
    return a.ctypes.data


class Context:
    """A pgx context on one CUDA device (streams, staging buffers)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().pgx_context_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def close(self) -> None:
        if self.handle:
            lib().pgx_context_destroy(self.handle)
            self.handle = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        return int(lib().pgx_context_launch_count(self.handle))


_default: dict[int, Context] = {}
_default_lock = threading.Lock()


def default_context(device: int = 0) -> Context:
    """One shared context per device, created on first use."""
    with _default_lock:
        ctx = _default.get(device)
        if ctx is None:
            ctx = Context(device)
            _default[device] = ctx
        return ctx


def problem_nx(kind: int, param: int) -> int:
    nx = C.c_uint64()
    check(lib().pgx_problem_nx(kind, param, C.byref(nx)))
    return int(nx.value)


def problem_bounds(kind: int, param: int) -> tuple[np.ndarray, np.ndarray]:
    nx = problem_nx(kind, param)
    lb = np.empty(nx)
    ub = np.empty(nx)
    check(lib().pgx_problem_bounds(kind, param, ptr(lb), ptr(ub)))
    return lb, ub


def mo_problem(kind: int, prob_id: int, param: int, fdim: int = 0, alpha: int = 0) -> pgx_mo_problem:
    if min(prob_id, param, fdim, alpha) < 0:
        raise OverflowError("can't convert negative value to unsigned int")
    return pgx_mo_problem(kind, prob_id, param, fdim, alpha)


def mo_problem_dims(p: pgx_mo_problem) -> tuple[int, int, int]:
    """(nx, nobj, nix) of a ZDT / DTLZ problem; ValueError with the reference's message if it is invalid."""
    nx, nobj, nix = C.c_uint64(), C.c_uint64(), C.c_uint64()
    check(lib().pgx_mo_problem_dims(C.byref(p), C.byref(nx), C.byref(nobj), C.byref(nix)))
    return int(nx.value), int(nobj.value), int(nix.value)


def mo_problem_bounds(p: pgx_mo_problem) -> tuple[np.ndarray, np.ndarray]:
    nx = mo_problem_dims(p)[0]
    lb, ub = np.empty(nx), np.empty(nx)
    check(lib().pgx_mo_problem_bounds(C.byref(p), ptr(lb), ptr(ub)))
    return lb, ub
