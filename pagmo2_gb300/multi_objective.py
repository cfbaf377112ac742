"""GPU NSGA-II survival with the reference's signatures
(src/utils/multi_objective.cpp:200-257, :280-315, :344-396, :425-465;
src/algorithms/nsga2.cpp:183-206).

``fast_non_dominated_sorting(points)`` returns the same 4-tuple as the
reference's ``fnds_return_type`` (fronts, dom_list, dom_count, rank), with the
fronts in the reference's order. ``crowding_distance(front)`` returns the
crowding distances of one front. ``nsga2_survival(points)`` runs the survival
block of one NSGA-II generation (fronts + per-front crowding) in one call.
``select_best_N_mo(points, N)`` and ``sort_population_mo(points)`` return the
reference's index lists. Wherever the reference sorts with std::sort, ties are
left in the order std::sort (GNU libstdc++) leaves them, so every output is
bit-exact with the reference.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from . import _native as _nat


def _points(points) -> tuple[np.ndarray, int, int]:
    if isinstance(points, np.ndarray) and points.ndim == 2:
        a = np.ascontiguousarray(points, dtype=np.float64)
        return a, a.shape[0], a.shape[1]
    rows = [np.asarray(p, dtype=np.float64).reshape(-1) for p in points]
    n = len(rows)
    m = rows[0].size if n else 0
    if any(r.size != m for r in rows):
        raise ValueError("Different number of objectives found in input fitnesses. I cannot define dominance")
    a = np.ascontiguousarray(np.stack(rows) if n else np.empty((0, 0)), dtype=np.float64).reshape(n, m)
    return a, n, m


def _fronts(off: np.ndarray, idx: np.ndarray, nf: int) -> list[list[int]]:
    return [idx[off[f]:off[f + 1]].tolist() for f in range(nf)]


def fnds_arrays(points, ctx: N.Context | None = None):
    """Flat outputs: (rank[n] int32, dom_count[n] int32, front_offsets[nf+1], front_indices[n])."""
    a, n, m = _points(points)
    if n < 2:
        raise ValueError(f"At least two points are needed for fast_non_dominated_sorting: {n} detected.")
    ctx = ctx or N.default_context()
    rank = np.empty(n, np.int32)
    dc = np.empty(n, np.int32)
    off = np.empty(n + 1, np.int32)
    idx = np.empty(n, np.int32)
    nf = C.c_int32()
    N.check(N.lib().pgx_fnds(ctx.handle, N.ptr(a), n, m, N.ptr(rank), N.ptr(dc), N.ptr(off), N.ptr(idx),
                             C.addressof(nf)))
    return rank, dc, off[:nf.value + 1].copy(), idx


def dom_list_arrays(points, ctx: N.Context | None = None):
    """(offsets[n+1] int64, indices[total] int32) of the reference's dom_list."""
    a, n, m = _points(points)
    if n < 2:
        raise ValueError(f"At least two points are needed for fast_non_dominated_sorting: {n} detected.")
    ctx = ctx or N.default_context()
    off = np.empty(n + 1, np.int64)
    total = C.c_uint64()
    st = N.lib().pgx_fnds_dom_list(ctx.handle, N.ptr(a), n, m, N.ptr(off), None, 0, C.byref(total))
    if st not in (N.OK, N.ERR_CAPACITY):
        N.check(st)
    idx = np.empty(max(int(total.value), 1), np.int32)
    N.check(N.lib().pgx_fnds_dom_list(ctx.handle, N.ptr(a), n, m, N.ptr(off), N.ptr(idx), idx.size,
                                      C.byref(total)))
    return off, idx[:int(total.value)]


def fast_non_dominated_sorting(points, ctx: N.Context | None = None, with_dom_list: bool = True):
    """(fronts, dom_list, dom_count, rank) as the reference returns them."""
    rank, dc, off, idx = fnds_arrays(points, ctx)
    fronts = _fronts(off, idx, off.size - 1)
    dom_list = None
    if with_dom_list:
        doff, didx = dom_list_arrays(points, ctx)
        dom_list = [didx[doff[i]:doff[i + 1]].tolist() for i in range(rank.size)]
    return fronts, dom_list, dc.tolist(), rank.tolist()


def crowding_distance(front, ctx: N.Context | None = None) -> np.ndarray:
    a, n, m = _points(front)
    if n < 2:
        raise ValueError(f"A non dominated front must contain at least two points: {n} detected.")
    if m < 2:
        raise ValueError(f"Points in the non dominated front must contain at least two objectives: {m} detected.")
    ctx = ctx or N.default_context()
    out = np.empty(n)
    N.check(N.lib().pgx_crowding_distance(ctx.handle, N.ptr(a), n, m, N.ptr(out)))
    return out


def nsga2_survival(points, ctx: N.Context | None = None):
    """(rank, dom_count, front_offsets, front_indices, crowding) for one population."""
    a, n, m = _points(points)
    if n < 2:
        raise ValueError(f"At least two points are needed for fast_non_dominated_sorting: {n} detected.")
    ctx = ctx or N.default_context()
    rank = np.empty(n, np.int32)
    dc = np.empty(n, np.int32)
    off = np.empty(n + 1, np.int32)
    idx = np.empty(n, np.int32)
    cd = np.empty(n)
    nf = C.c_int32()
    N.check(N.lib().pgx_nsga2_survival(ctx.handle, N.ptr(a), n, m, N.ptr(rank), N.ptr(dc), N.ptr(off), N.ptr(idx),
                                       C.addressof(nf), N.ptr(cd)))
    return rank, dc, off[:nf.value + 1].copy(), idx, cd



def select_best_N_mo(points, N: int, ctx: _nat.Context | None = None) -> list[int]:  # noqa: N802,N803
    """Indices of the best N points -- whole fronts while they fit, then the
    critical front by descending crowding distance -- as the reference's
    select_best_N_mo returns them."""
    a, n, m = _points(points)
    if N < 0:
        raise OverflowError("N must be non-negative")
    ctx = ctx or _nat.default_context()
    out = np.empty(max(min(N, n), 1), np.int32)
    cnt = C.c_uint64()
    _nat.check(_nat.lib().pgx_select_best_n_mo(ctx.handle, _nat.ptr(a) if a.size else None, n, m, N, _nat.ptr(out),
                                                C.byref(cnt)))
    return out[:cnt.value].tolist()


def sort_population_mo(points, ctx: _nat.Context | None = None) -> list[int]:
    """The points ordered by (non-domination rank, descending crowding
    distance), as the reference's sort_population_mo returns them."""
    a, n, m = _points(points)
    ctx = ctx or _nat.default_context()
    out = np.empty(max(n, 1), np.int32)
    _nat.check(_nat.lib().pgx_sort_population_mo(ctx.handle, _nat.ptr(a) if a.size else None, n, m, _nat.ptr(out)))
    return out[:n].tolist()


def std_sort_keys(keys, values=None, ctx: _nat.Context | None = None):
    """(keys, values) sorted by key on the GPU, equal keys left in the order
    std::sort (GNU libstdc++) leaves them; values default to 0..n-1."""
    k = np.array(keys, dtype=np.int64).reshape(-1)
    v = np.arange(k.size, dtype=np.int32) if values is None else np.array(values, dtype=np.int32).reshape(-1)
    if v.size != k.size:
        raise ValueError("keys and values differ in length")
    ctx = ctx or _nat.default_context()
    _nat.check(_nat.lib().pgx_std_sort_i64(ctx.handle, _nat.ptr(k), _nat.ptr(v), k.size))
    return k, v


class hypervolume:
    """pagmo's hypervolume indicator (src/utils/hypervolume.cpp) on the GPU, 2 to 16 objectives:
    compute(ref) is the measure of the region the points dominate, bounded by the reference point (hv2d /
    hv3d's result for 2 and 3 objectives, hvwfg's bit for bit for 4 and more); exclusive(p_idx, ref),
    contributions(ref), least_contributor(ref) and greatest_contributor(ref) are the reference's queries
    (hypervolume.cpp:249-401), the contributions by hvwfg's limit sets. Construction checks the points as the
    reference does (hypervolume.cpp:406-432); every query checks the reference point
    (hv_algorithm.cpp:226-258)."""

    def __init__(self, points, verify: bool = True, context: N.Context | None = None):
        rows = points.get_f() if hasattr(points, "get_f") else points
        if len(rows) == 0:
            raise ValueError("Point set cannot be empty.")
        if isinstance(rows, np.ndarray) and rows.ndim == 2:
            a = np.ascontiguousarray(rows, dtype=np.float64)
        else:
            vs = [np.asarray(r, dtype=np.float64).reshape(-1) for r in rows]
            if vs[0].size <= 1:
                raise ValueError("Points of dimension > 1 required.")
            if any(v.size != vs[0].size for v in vs):
                raise ValueError("All point set dimensions must be equal.")
            a = np.ascontiguousarray(np.stack(vs))
        if a.shape[1] <= 1:
            raise ValueError("Points of dimension > 1 required.")
        if verify and np.isnan(a).any():
            raise ValueError("A nan value has been encountered in the hypervolume points. Cannot construct the "
                             "hypervolume object")
        self._points = a
        self._ctx = context

    def get_points(self) -> np.ndarray:
        return self._points.copy()

    def compute(self, ref) -> float:
        r = np.ascontiguousarray(np.asarray(ref, dtype=np.float64).reshape(-1))
        n, m = self._points.shape
        if r.size != m:
            raise ValueError("Point set dimensions and reference point dimension must be equal.")
        ctx = self._ctx if self._ctx is not None else N.default_context()
        out = C.c_double()
        N.check(N.lib().pgx_hypervolume(ctx.handle, N.ptr(self._points), n, m, N.ptr(r), C.byref(out)))
        return out.value

    def _ref(self, ref):
        r = np.ascontiguousarray(np.asarray(ref, dtype=np.float64).reshape(-1))
        if r.size != self._points.shape[1]:
            raise ValueError("Point set dimensions and reference point dimension must be equal.")
        return r, (self._ctx if self._ctx is not None else N.default_context())

    def refpoint(self, offset: float = 0.0) -> np.ndarray:
        """The componentwise maximum of the points plus offset (hypervolume.cpp:160-180)."""
        return self._points.max(axis=0) + float(offset)

    def exclusive(self, p_idx: int, ref) -> float:
        """The volume only point p_idx dominates: compute(ref) minus the volume without it."""
        r, ctx = self._ref(ref)
        n, m = self._points.shape
        if int(p_idx) < 0:
            raise ValueError("Index of the individual is out of bounds.")
        out = C.c_double()
        N.check(N.lib().pgx_hypervolume_exclusive(ctx.handle, N.ptr(self._points), n, m, N.ptr(r), int(p_idx),
                                                  C.byref(out)))
        return out.value

    def contributions(self, ref) -> np.ndarray:
        """Every point's exclusive contribution."""
        r, ctx = self._ref(ref)
        n, m = self._points.shape
        out = np.empty(n)
        N.check(N.lib().pgx_hypervolume_contributions(ctx.handle, N.ptr(self._points), n, m, N.ptr(r), N.ptr(out)))
        return out

    def _extreme(self, ref, greatest: bool) -> int:
        r, ctx = self._ref(ref)
        n, m = self._points.shape
        out = C.c_uint64()
        N.check(N.lib().pgx_hypervolume_extreme_contributor(ctx.handle, N.ptr(self._points), n, m, N.ptr(r),
                                                            int(greatest), C.byref(out)))
        return out.value

    def least_contributor(self, ref) -> int:
        """The first index of the smallest contribution."""
        return self._extreme(ref, False)

    def greatest_contributor(self, ref) -> int:
        """The first index of the largest contribution."""
        return self._extreme(ref, True)
