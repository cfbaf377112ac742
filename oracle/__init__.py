"""CPU oracle for the batch-evaluation path -- TEST INFRASTRUCTURE ONLY.

Loads oracle/_ref/liboracle.so (the C++ restatement in oracle.cpp) and, when
it has been built from the reference sources in this container,
oracle/_ref/libpagmo_ref.so (the unmodified reference compiled by
oracle/Makefile). Only tests/, __graft_entry__.smoke() and the CPU leg of
bench.py use this module, as the checker; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
ORACLE_SO = OUT / "liboracle.so"
REF_SO = OUT / "libpagmo_ref.so"
# The reference's sources: a pagmo 2.19.1 tree named by PGX_REFERENCE_ROOT, or
# the copy `make -C oracle stage` leaves in baseline/_ref/pagmo2 (git-ignored;
# it travels with the working tree). Neither present: the reference-pinned
# tests skip.
STAGED_ROOT = HERE.parent / "baseline" / "_ref" / "pagmo2"


def _reference_root() -> Path | None:
    env = os.environ.get("PGX_REFERENCE_ROOT")
    if env:
        return Path(env)
    return STAGED_ROOT if (STAGED_ROOT / "src" / "problem.cpp").exists() else None


REF_ROOT = _reference_root()

_vp, _u64 = C.c_void_p, C.c_uint64


def build(reference: bool | None = None) -> None:
    """Compile the oracle (always) and the reference library (when its sources exist).

    With PGX_REFERENCE_ROOT set, the tree is first staged into baseline/_ref/pagmo2
    so that later builds (also on machines without the tree) find it there."""
    r = subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    env = os.environ.get("PGX_REFERENCE_ROOT")
    if env and Path(env).resolve() != STAGED_ROOT.resolve() and (Path(env) / "src" / "problem.cpp").exists():
        r = subprocess.run(["make", "-s", "-C", str(HERE), "stage", f"PAGMO_SOURCE={env}"], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"staging the reference failed:\n{r.stdout}\n{r.stderr}")
    root = STAGED_ROOT if (STAGED_ROOT / "src" / "problem.cpp").exists() else _reference_root()
    if reference is None:
        reference = root is not None and (root / "src" / "problem.cpp").exists()
    if reference:
        if root is None:
            raise RuntimeError("the reference's sources are not present (set PGX_REFERENCE_ROOT)")
        jobs = str(max(2, os.cpu_count() or 2))
        r = subprocess.run(["make", "-s", f"-j{jobs}", "-C", str(HERE), "ref", f"REF_ROOT={root}"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")


def _p(a):
    return None if a is None else a.ctypes.data


def _pts2d(pts):
    """n x m float64 C array from an n x m array or a list of n equal-length lists."""
    p = np.ascontiguousarray(pts, dtype=np.float64)
    if p.ndim != 2:
        p = p.reshape(len(pts), -1) if p.size else np.zeros((len(pts), 0))
    return p


def _mo_spec(spec):
    """(family, prob_id, param, fdim, alpha) with defaults for the missing tail."""
    t = tuple(spec) + (0, 0, 0, 0, 0)[len(spec):]
    return int(t[0]), int(t[1]), int(t[2]), int(t[3]), int(t[4])


class _Oracle:
    def __init__(self, path: Path):
        self.h = C.CDLL(str(path))
        h = self.h
        for name in ("orc_rastrigin_fitness", "orc_rosenbrock_fitness"):
            getattr(h, name).restype = C.c_double
            getattr(h, name).argtypes = [_vp, _u64]
        h.orc_lj_fitness.restype = C.c_double
        h.orc_lj_fitness.argtypes = [_vp, _u64]
        for name in ("orc_rastrigin_fitness_ld", "orc_rosenbrock_fitness_ld", "orc_lj_fitness_ld"):
            getattr(h, name).restype = C.c_double
            getattr(h, name).argtypes = [_vp, _u64, _vp]
        h.orc_last_error.restype = C.c_char_p
        for name in ("orc_batch_fitness", "orc_batch_gradient"):
            getattr(h, name).argtypes = [C.c_int, _u64, _vp, _u64, _u64, _vp, C.c_int]
        for name in ("orc_batch_fitness_ld", "orc_batch_gradient_ld"):
            getattr(h, name).argtypes = [C.c_int, _u64, _vp, _u64, _u64, _vp, _vp, C.c_int]
        h.orc_pareto_dominance.argtypes = [_vp, _vp, _u64]
        h.orc_fnds.argtypes = [_vp, _u64, _u64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _u64]
        h.orc_crowding.argtypes = [_vp, _u64, _u64, _vp]
        h.orc_nsga2_crowding.argtypes = [_vp, _u64, _u64, _vp, _vp, _u64, _vp]
        h.orc_crowding_ex.argtypes = [_vp, _u64, _u64, C.c_int, _vp]
        h.orc_nsga2_crowding_ex.argtypes = [_vp, _u64, _u64, _vp, _vp, _u64, C.c_int, _vp]
        h.orc_sort_last_error.restype = C.c_char_p
        for name in ("orc_std_sort_keys", "orc_introsort_keys", "orc_introsort_chunked_keys",
                     "orc_introsort_lists_keys", "orc_heap_sort_keys", "orc_std_partial_sort_full"):
            getattr(h, name).argtypes = [_vp, _vp, _u64]
            getattr(h, name).restype = None
        h.orc_quicksort_adversary.argtypes = [_u64, _vp]
        h.orc_depth_limit_hits.restype = _u64
        h.orc_depth_limit_hits.argtypes = []
        h.orc_quicksort_adversary.restype = None
        h.orc_select_best_n_mo.argtypes = [_vp, _u64, _u64, _u64, _vp, _vp]
        h.orc_sort_population_mo.argtypes = [_vp, _u64, _u64, _vp]
        h.orc_mo_last_error.restype = C.c_char_p
        h.orc_zdt_p_distance.restype = C.c_double
        h.orc_zdt_p_distance.argtypes = [C.c_uint, _vp, _u64]
        h.orc_hypervolume_ld.argtypes = [_vp, _u64, _u64, _vp, _vp]
        h.orc_hvwfg.argtypes = [_vp, _u64, _u64, _vp, _vp]
        h.orc_hvwfg_contributions.argtypes = [_vp, _u64, _u64, _vp, _vp]
        h.orc_hs71_fitness.argtypes = [_vp, _u64, _vp]
        h.orc_hs71_fitness.restype = None
        h.orc_unconstrain_penalize.argtypes = [_vp, _u64, _u64, _u64, _u64, C.c_int, _vp, _vp, _vp]
        h.orc_mo_dims.argtypes = [C.c_int, C.c_uint, _u64, _u64, _vp, _vp]
        h.orc_mo_batch_fitness.argtypes = [C.c_int, C.c_uint, _u64, _u64, C.c_uint, _vp, _u64, _u64, _vp, C.c_int]
        h.orc_mo_batch_fitness_ld.argtypes = [C.c_int, C.c_uint, _u64, _u64, C.c_uint, _vp, _u64, _u64, _vp, _vp,
                                              C.c_int]
        h.orc_mo_batch_p_distance.argtypes = [C.c_int, C.c_uint, _u64, _u64, _vp, _u64, _u64, _vp, _vp, C.c_int]

    def _chk(self, st):
        if st != 0:
            raise ValueError(self.h.orc_last_error().decode())

    def _chk_sort(self, st):
        if st != 0:
            raise ValueError(self.h.orc_sort_last_error().decode())

    # batch evaluation -------------------------------------------------------
    def batch_fitness(self, kind, param, dvs, threads=0):
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        n, nx = x.shape
        f = np.empty(n)
        self._chk(self.h.orc_batch_fitness(kind, param, _p(x), n, nx, _p(f), threads))
        return f

    def batch_gradient(self, kind, param, dvs, threads=0):
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        n, nx = x.shape
        g = np.empty((n, nx))
        self._chk(self.h.orc_batch_gradient(kind, param, _p(x), n, nx, _p(g), threads))
        return g

    def batch_fitness_ld(self, kind, param, dvs, threads=0):
        """(value, condition scale) per row, long double."""
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        n, nx = x.shape
        f = np.empty(n)
        s = np.empty(n)
        self._chk(self.h.orc_batch_fitness_ld(kind, param, _p(x), n, nx, _p(f), _p(s), threads))
        return f, s

    def batch_gradient_ld(self, kind, param, dvs, threads=0):
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        n, nx = x.shape
        g = np.empty((n, nx))
        s = np.empty((n, nx))
        self._chk(self.h.orc_batch_gradient_ld(kind, param, _p(x), n, nx, _p(g), _p(s), threads))
        return g, s

    # multi-objective ---------------------------------------------------------
    def pareto_dominance(self, a, b):
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        return bool(self.h.orc_pareto_dominance(_p(a), _p(b), a.size))

    def fnds(self, pts, dom_list=True):
        p = np.ascontiguousarray(pts, dtype=np.float64)
        n, m = p.shape
        rank = np.empty(n, np.uint64)
        dc = np.empty(n, np.uint64)
        off = np.empty(n + 1, np.uint64)
        idx = np.empty(n, np.uint64)
        nf = C.c_uint64()
        cap = n * (n - 1) // 2 if dom_list else 0
        dlo = np.empty(n + 1, np.uint64) if dom_list else None
        dli = np.empty(max(cap, 1), np.uint64) if dom_list else None
        self._chk(self.h.orc_fnds(_p(p), n, m, _p(rank), _p(dc), _p(off), _p(idx), C.addressof(nf), _p(dlo),
                                  _p(dli), cap))
        k = nf.value
        out = {"rank": rank.astype(np.int64), "dom_count": dc.astype(np.int64),
               "front_offsets": off[:k + 1].astype(np.int64), "front_indices": idx.astype(np.int64)}
        if dom_list:
            out["dl_offsets"] = dlo.astype(np.int64)
            out["dl_indices"] = dli[:int(dlo[n])].astype(np.int64)
        return out

    def crowding(self, pts, stable=False):
        """crowding_distance; stable=True keeps tied values in input order."""
        p = np.ascontiguousarray(pts, dtype=np.float64)
        n, m = p.shape
        out = np.empty(n)
        self._chk(self.h.orc_crowding_ex(_p(p), n, m, int(stable), _p(out)))
        return out

    def nsga2_crowding(self, pts, front_offsets, front_indices, stable=False):
        p = np.ascontiguousarray(pts, dtype=np.float64)
        n, m = p.shape
        off = np.ascontiguousarray(front_offsets, dtype=np.uint64)
        idx = np.ascontiguousarray(front_indices, dtype=np.uint64)
        out = np.empty(n)
        self._chk(self.h.orc_nsga2_crowding_ex(_p(p), n, m, _p(off), _p(idx), off.size - 1, int(stable), _p(out)))
        return out

    # orderings -----------------------------------------------------------------
    def sort_keys(self, keys, values=None, method="std"):
        """(keys, values) sorted by key: method "std" (std::sort), "intro" (the
        restated introsort), "chunked" / "lists" (its two GPU partitions), "heap"
        (restated heapsort) or "std_heap" (std::partial_sort over the whole range)."""
        k = np.array(keys, dtype=np.int64)
        v = np.arange(k.size, dtype=np.int32) if values is None else np.array(values, dtype=np.int32)
        fn = {"std": self.h.orc_std_sort_keys, "intro": self.h.orc_introsort_keys,
              "chunked": self.h.orc_introsort_chunked_keys, "lists": self.h.orc_introsort_lists_keys,
              "heap": self.h.orc_heap_sort_keys,
              "std_heap": self.h.orc_std_partial_sort_full}[method]
        fn(_p(k), _p(v), k.size)
        return k, v

    def depth_limit_hits(self):
        """Ranges handed to heapsort so far by the restated introsorts (this thread)."""
        return int(self.h.orc_depth_limit_hits())

    def quicksort_adversary(self, n):
        out = np.empty(n, np.int64)
        self.h.orc_quicksort_adversary(n, _p(out))
        return out

    def select_best_n_mo(self, pts, N):
        p = _pts2d(pts)
        n, m = p.shape
        out = np.empty(max(n, 1), np.uint64)
        cnt = C.c_uint64()
        self._chk_sort(self.h.orc_select_best_n_mo(_p(p), n, m, N, _p(out), C.addressof(cnt)))
        return out[:cnt.value].astype(np.int64)

    def sort_population_mo(self, pts):
        p = _pts2d(pts)
        n, m = p.shape
        out = np.empty(max(n, 1), np.uint64)
        self._chk_sort(self.h.orc_sort_population_mo(_p(p), n, m, _p(out)))
        return out[:n].astype(np.int64)

    # hypervolume -------------------------------------------------------------------
    def hypervolume(self, pts, ref):
        """Long-double hypervolume of 2 or 3 objectives."""
        p = _pts2d(pts)
        r = np.ascontiguousarray(ref, dtype=np.float64)
        out = C.c_double()
        if self.h.orc_hypervolume_ld(_p(p), p.shape[0], p.shape[1], _p(r), C.byref(out)) != 0:
            raise ValueError("hypervolume oracle: 2 or 3 objectives and at least one point")
        return out.value

    def hvwfg(self, pts, ref):
        """WFG hypervolume in double, the reference's operation order (any m >= 2)."""
        p = _pts2d(pts)
        r = np.ascontiguousarray(ref, dtype=np.float64)
        out = C.c_double()
        if self.h.orc_hvwfg(_p(p), p.shape[0], p.shape[1], _p(r), C.byref(out)) != 0:
            raise ValueError("hvwfg oracle: at least one point of 2 or more objectives")
        return out.value

    def hs71_fitness(self, dvs):
        """hock_schittkowski_71 rows [f, ceq, cineq], the reference's double arithmetic."""
        x = np.ascontiguousarray(dvs, dtype=np.float64).reshape(-1, 4)
        out = np.empty((x.shape[0], 3))
        self.h.orc_hs71_fitness(_p(x), x.shape[0], _p(out))
        return out

    def unconstrain_hs71(self, method, dvs, weights=(), c_tol=None):
        """unconstrain{hock_schittkowski_71, method, weights} rows, the reference's double arithmetic."""
        codes = {"death penalty": 0, "kuri": 1, "weighted": 2, "ignore_c": 3, "ignore_o": 4}
        f = self.hs71_fitness(dvs)
        w = np.ascontiguousarray(weights if len(weights) else np.zeros(2), dtype=np.float64)
        tol = np.zeros(2) if c_tol is None else np.ascontiguousarray(c_tol, dtype=np.float64)
        out = np.empty(f.shape[0])
        if self.h.orc_unconstrain_penalize(_p(f), f.shape[0], 1, 1, 1, codes[method], _p(w), _p(tol), _p(out)):
            raise ValueError(method)
        return out

    def hvwfg_contributions(self, pts, ref):
        """Every point's exclusive contribution, WFG in double (any m >= 2)."""
        p = _pts2d(pts)
        r = np.ascontiguousarray(ref, dtype=np.float64)
        out = np.empty(p.shape[0])
        if self.h.orc_hvwfg_contributions(_p(p), p.shape[0], p.shape[1], _p(r), _p(out)) != 0:
            raise ValueError("hvwfg oracle: at least one point of 2 or more objectives")
        return out

    # ZDT / DTLZ ------------------------------------------------------------------
    # spec = (family, prob_id, param, fdim, alpha): family 7 = zdt{prob_id, param},
    # family 8 = dtlz{prob_id, dim=param, fdim, alpha} (the GPU library's kinds).
    def _chk_mo(self, st):
        if st != 0:
            raise ValueError(self.h.orc_mo_last_error().decode())

    def mo_dims(self, spec):
        fam, pid, param, fdim, _ = _mo_spec(spec)
        nx, nobj = C.c_uint64(), C.c_uint64()
        self._chk_mo(self.h.orc_mo_dims(fam, pid, param, fdim, C.byref(nx), C.byref(nobj)))
        return nx.value, nobj.value

    def mo_fitness(self, spec, dvs, threads=0):
        """Mirror of the reference's fitness over the rows: n x nobj."""
        fam, pid, param, fdim, alpha = _mo_spec(spec)
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        n, nx = x.shape
        f = np.empty((n, self.mo_dims(spec)[1]))
        self._chk_mo(self.h.orc_mo_batch_fitness(fam, pid, param, fdim, alpha, _p(x), n, nx, _p(f), threads))
        return f

    def mo_fitness_ld(self, spec, dvs, threads=0):
        """(values, error scales), long double, n x nobj each."""
        fam, pid, param, fdim, alpha = _mo_spec(spec)
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        n, nx = x.shape
        nobj = self.mo_dims(spec)[1]
        f, sc = np.empty((n, nobj)), np.empty((n, nobj))
        self._chk_mo(self.h.orc_mo_batch_fitness_ld(fam, pid, param, fdim, alpha, _p(x), n, nx, _p(f), _p(sc),
                                                    threads))
        return f, sc

    def mo_p_distance(self, spec, dvs, ld=False, threads=0):
        """p_distance of every row (mirror), or (values, scales) in long double."""
        fam, pid, param, fdim, _ = _mo_spec(spec)
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        n, nx = x.shape
        out = np.empty(n)
        sc = np.empty(n) if ld else None
        self._chk_mo(self.h.orc_mo_batch_p_distance(fam, pid, param, fdim, _p(x), n, nx, _p(out), _p(sc), threads))
        return (out, sc) if ld else out


class _Reference:
    """The reference's own compiled sources (only where they were built)."""

    def __init__(self, path: Path):
        self.h = C.CDLL(str(path))
        h = self.h
        h.ref_last_error.restype = C.c_char_p
        h.ref_thread_bfe.argtypes = [C.c_int, _u64, _vp, _u64, _u64, _vp, _vp]
        h.ref_load_dvs.argtypes = [_vp, _u64]
        h.ref_thread_bfe_loaded.argtypes = [C.c_int, _u64, _vp]
        h.ref_gradient_loaded.argtypes = [C.c_int, _u64, _vp, C.c_int]
        h.ref_fitness_rows.argtypes = [C.c_int, _u64, _vp, _u64, _u64, _vp]
        h.ref_gradient_rows.argtypes = [C.c_int, _u64, _vp, _u64, _u64, _vp]
        h.ref_bounds.argtypes = [C.c_int, _u64, _vp, _vp]
        h.ref_fnds.argtypes = [_vp, _u64, _u64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _u64]
        h.ref_crowding.argtypes = [_vp, _u64, _u64, _vp]
        h.ref_pareto_dominance.argtypes = [_vp, _vp, _u64, _vp]
        h.ref_select_best_n_mo.argtypes = [_vp, _u64, _u64, _u64, _vp, _vp]
        h.ref_sort_population_mo.argtypes = [_vp, _u64, _u64, _vp]
        mo = [C.c_int, C.c_uint, _u64, _u64, C.c_uint]
        h.ref_hypervolume.argtypes = [_vp, _u64, _u64, _vp, _vp]
        h.ref_hv_exclusive.argtypes = [_vp, _u64, _u64, _vp, _u64, _vp]
        h.ref_hv_contributions.argtypes = [_vp, _u64, _u64, _vp, C.c_int, _vp]
        h.ref_hv_extreme.argtypes = [_vp, _u64, _u64, _vp, C.c_int, _vp]
        h.ref_hvwfg_compute.argtypes = [_vp, _u64, _u64, _vp, _vp]
        h.ref_hs71_fitness.argtypes = [_vp, _u64, _vp]
        h.ref_unconstrain_hs71.argtypes = [C.c_char_p, _vp, _u64, _vp, _vp, _u64, _vp]
        h.ref_mo_dims.argtypes = mo + [_vp, _vp, _vp]
        h.ref_mo_bounds.argtypes = mo + [_vp, _vp]
        h.ref_mo_thread_bfe.argtypes = mo + [_vp, _u64, _u64, _vp]
        h.ref_mo_p_distance.argtypes = mo + [_vp, _u64, _u64, _vp]

    def _chk(self, st):
        if st == 1:
            raise ValueError(self.h.ref_last_error().decode())
        if st != 0:
            raise RuntimeError(self.h.ref_last_error().decode())

    def thread_bfe(self, kind, param, dvs):
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        n, nx = x.shape
        f = np.empty(n)
        fe = C.c_uint64()
        self._chk(self.h.ref_thread_bfe(kind, param, _p(x), n, nx, _p(f), C.byref(fe)))
        return f, fe.value

    def load(self, dvs):
        """Holds dvs as one vector_double inside the reference library (the form a
        pagmo algorithm hands its bfe); returns (n, nx) for the *_loaded calls."""
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        self._chk(self.h.ref_load_dvs(_p(x), x.size))
        return x.shape

    def thread_bfe_loaded(self, kind, param, out):
        """bfe{thread_bfe{}} over the loaded rows into out (n fitness values)."""
        self._chk(self.h.ref_thread_bfe_loaded(kind, param, _p(out)))
        return out

    def gradient_loaded(self, kind, param, out, threads):
        """problem::gradient over the loaded rows on `threads` threads into out (n, nx)."""
        self._chk(self.h.ref_gradient_loaded(kind, param, _p(out), int(threads)))
        return out

    def fitness_rows(self, kind, param, dvs):
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        n, nx = x.shape
        f = np.empty(n)
        self._chk(self.h.ref_fitness_rows(kind, param, _p(x), n, nx, _p(f)))
        return f

    def gradient_rows(self, kind, param, dvs):
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        n, nx = x.shape
        g = np.empty((n, nx))
        self._chk(self.h.ref_gradient_rows(kind, param, _p(x), n, nx, _p(g)))
        return g

    def bounds(self, kind, param, nx):
        lb = np.empty(nx)
        ub = np.empty(nx)
        self._chk(self.h.ref_bounds(kind, param, _p(lb), _p(ub)))
        return lb, ub

    def fnds(self, pts):
        p = np.ascontiguousarray(pts, dtype=np.float64)
        n, m = p.shape
        rank = np.empty(n, np.uint64)
        dc = np.empty(n, np.uint64)
        off = np.empty(n + 1, np.uint64)
        idx = np.empty(n, np.uint64)
        nf = C.c_uint64()
        cap = n * (n - 1) // 2
        dlo = np.empty(n + 1, np.uint64)
        dli = np.empty(max(cap, 1), np.uint64)
        self._chk(self.h.ref_fnds(_p(p), n, m, _p(rank), _p(dc), _p(off), _p(idx), C.addressof(nf), _p(dlo),
                                  _p(dli), cap))
        k = nf.value
        return {"rank": rank.astype(np.int64), "dom_count": dc.astype(np.int64),
                "front_offsets": off[:k + 1].astype(np.int64), "front_indices": idx.astype(np.int64),
                "dl_offsets": dlo.astype(np.int64), "dl_indices": dli[:int(dlo[n])].astype(np.int64)}

    def crowding(self, pts):
        p = np.ascontiguousarray(pts, dtype=np.float64)
        n, m = p.shape
        out = np.empty(n)
        self._chk(self.h.ref_crowding(_p(p), n, m, _p(out)))
        return out

    def select_best_n_mo(self, pts, N):
        p = _pts2d(pts)
        n, m = p.shape
        out = np.empty(max(n, 1), np.uint64)
        cnt = C.c_uint64()
        self._chk(self.h.ref_select_best_n_mo(_p(p), n, m, N, _p(out), C.addressof(cnt)))
        return out[:cnt.value].astype(np.int64)

    def sort_population_mo(self, pts):
        p = _pts2d(pts)
        n, m = p.shape
        out = np.empty(max(n, 1), np.uint64)
        self._chk(self.h.ref_sort_population_mo(_p(p), n, m, _p(out)))
        return out[:n].astype(np.int64)

    def pareto_dominance(self, a, b):
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        r = C.c_int()
        self._chk(self.h.ref_pareto_dominance(_p(a), _p(b), a.size, C.byref(r)))
        return bool(r.value)

    def hypervolume(self, pts, ref):
        """hypervolume(points, true).compute(ref) of the reference."""
        p = _pts2d(pts)
        r = np.ascontiguousarray(ref, dtype=np.float64)
        out = C.c_double()
        self._chk(self.h.ref_hypervolume(_p(p), p.shape[0], p.shape[1], _p(r), C.byref(out)))
        return out.value

    def hv_exclusive(self, pts, ref, p_idx):
        """hypervolume(points, true).exclusive(p_idx, ref) of the reference."""
        p = _pts2d(pts)
        r = np.ascontiguousarray(ref, dtype=np.float64)
        out = C.c_double()
        self._chk(self.h.ref_hv_exclusive(_p(p), p.shape[0], p.shape[1], _p(r), int(p_idx), C.byref(out)))
        return out.value

    def hv_contributions(self, pts, ref, wfg=False):
        """hypervolume(points, true).contributions(ref) of the reference (hvwfg() given explicitly with wfg)."""
        p = _pts2d(pts)
        r = np.ascontiguousarray(ref, dtype=np.float64)
        out = np.empty(p.shape[0])
        self._chk(self.h.ref_hv_contributions(_p(p), p.shape[0], p.shape[1], _p(r), int(bool(wfg)), _p(out)))
        return out

    def hv_extreme(self, pts, ref, greatest):
        """least_contributor(ref) / greatest_contributor(ref) of the reference."""
        p = _pts2d(pts)
        r = np.ascontiguousarray(ref, dtype=np.float64)
        out = C.c_uint64()
        self._chk(self.h.ref_hv_extreme(_p(p), p.shape[0], p.shape[1], _p(r), int(bool(greatest)), C.byref(out)))
        return out.value

    def hs71_fitness(self, dvs):
        """problem{hock_schittkowski_71{}}.fitness per row of the reference."""
        x = np.ascontiguousarray(dvs, dtype=np.float64).reshape(-1, 4)
        out = np.empty((x.shape[0], 3))
        self._chk(self.h.ref_hs71_fitness(_p(x), x.shape[0], _p(out)))
        return out

    def unconstrain_hs71(self, method, dvs, weights=(), c_tol=None):
        """problem{unconstrain{hock_schittkowski_71 (with c_tol), method, weights}}.fitness per row."""
        x = np.ascontiguousarray(dvs, dtype=np.float64).reshape(-1, 4)
        w = np.ascontiguousarray(weights, dtype=np.float64).reshape(-1)
        tol = None if c_tol is None else np.ascontiguousarray(c_tol, dtype=np.float64)
        out = np.empty(x.shape[0])
        self._chk(self.h.ref_unconstrain_hs71(method.encode(), _p(w) if w.size else None, w.size, _p(tol), _p(x),
                                              x.shape[0], _p(out)))
        return out

    def hvwfg(self, pts, ref):
        """hypervolume(points, true).compute(ref, hvwfg()) of the reference."""
        p = _pts2d(pts)
        r = np.ascontiguousarray(ref, dtype=np.float64)
        out = C.c_double()
        self._chk(self.h.ref_hvwfg_compute(_p(p), p.shape[0], p.shape[1], _p(r), C.byref(out)))
        return out.value

    # ZDT / DTLZ (spec as in the oracle) ---------------------------------------------
    def mo_dims(self, spec):
        """(nx, nobj, nix) of the constructed reference problem."""
        nx, nobj, nix = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._chk(self.h.ref_mo_dims(*_mo_spec(spec), C.byref(nx), C.byref(nobj), C.byref(nix)))
        return nx.value, nobj.value, nix.value

    def mo_bounds(self, spec):
        nx = self.mo_dims(spec)[0]
        lb, ub = np.empty(nx), np.empty(nx)
        self._chk(self.h.ref_mo_bounds(*_mo_spec(spec), _p(lb), _p(ub)))
        return lb, ub

    def mo_thread_bfe(self, spec, dvs):
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        n, nx = x.shape
        f = np.empty((n, self.mo_dims(spec)[1]))
        self._chk(self.h.ref_mo_thread_bfe(*_mo_spec(spec), _p(x), n, nx, _p(f)))
        return f

    def mo_p_distance(self, spec, dvs):
        x = np.ascontiguousarray(dvs, dtype=np.float64)
        n, nx = x.shape
        out = np.empty(n)
        self._chk(self.h.ref_mo_p_distance(*_mo_spec(spec), _p(x), n, nx, _p(out)))
        return out


_oracle = None
_reference = None


def oracle() -> _Oracle:
    global _oracle
    if _oracle is None:
        if not ORACLE_SO.exists():
            build(reference=False)
        _oracle = _Oracle(ORACLE_SO)
    return _oracle


def reference() -> _Reference | None:
    """The compiled reference, or None where it was not built (e.g. a machine without its sources)."""
    global _reference
    if _reference is None and REF_SO.exists():
        try:
            _reference = _Reference(REF_SO)
        except OSError:
            return None
    return _reference
