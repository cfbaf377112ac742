"""Seeded synthetic inputs for the batch-evaluation workloads.

No public dataset is involved: every input is drawn from numpy's RandomState,
whose integer seeding is the classic mt19937 init_genrand and whose
random_sample() is genrand_res53 ((a >> 5) * 2^26 + (b >> 6)) / 2^53, so a C++
std::mt19937(seed) reproduces the same uniform stream.

Workloads (sizes as benchmarked):
  rastrigin   4096 x 50,    uniform in [-5.12, 5.12],          seed 1
  rosenbrock  65536 x 1000, uniform in [-5, 10],               seed 2
  lj          16384 clusters of 150 atoms (444 coordinates),
              uniform in lennard_jones::get_bounds,            seed 3
  lj_lattice  perturbed fcc clusters near equilibrium (sigma 0.05), for
              cancellation-sensitive checks
  nsga2       20000 points x 3 objectives: 30 nested simplex layers of radius
              1 + 0.1 k with N(0, 1e-3) jitter, plus 5 % exact duplicates,
              shuffled,                                        seed 4
  sphere      points on the positive orthant of the unit sphere (hypervolume
              of 4+ objectives),                               seed 6
  archipelago 64 islands, population log-uniform in [32, 4096], dimension
              uniform in [10, 500], problems round-robin over the three
              (lennard_jones gets N = round((dim + 6) / 3) atoms), seed 5
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _native as N


def bounds(kind: int, param: int) -> tuple[np.ndarray, np.ndarray]:
    """Box bounds of the reference UDPs (computed host-side, no device needed)."""
    if kind == N.RASTRIGIN:
        return np.full(param, -5.12), np.full(param, 5.12)
    if kind == N.ROSENBROCK:
        return np.full(param, -5.0), np.full(param, 10.0)
    if kind in (N.ACKLEY, N.GRIEWANK, N.SCHWEFEL):
        lo, hi = {N.ACKLEY: (-15.0, 30.0), N.GRIEWANK: (-600.0, 600.0), N.SCHWEFEL: (-500.0, 500.0)}[kind]
        return np.full(param, lo), np.full(param, hi)
    nx = 3 * param - 6
    lb = np.full(nx, -3.0)
    ub = np.full(nx, 3.0)
    z = np.arange(nx)
    sel = (z != 0) & (z % 3 == 0)
    lb[sel] = 0.0
    ub[sel] = 6.0
    return lb, ub


def nx_of(kind: int, param: int) -> int:
    return 3 * param - 6 if kind == N.LENNARD_JONES else param


def uniform_batch(kind: int, param: int, n: int, seed: int) -> np.ndarray:
    """n decision vectors, each coordinate uniform within the problem's bounds."""
    lb, ub = bounds(kind, param)
    rs = np.random.RandomState(seed)
    u = rs.random_sample((n, lb.size))
    return lb + (ub - lb) * u


def mo_bounds(kind: int, prob_id: int, param: int, fdim: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """Box bounds of zdt{prob_id, param} / dtlz{prob_id, param, fdim} (host-side,
    src/problems/zdt.cpp:108-133, src/problems/dtlz.cpp:116-119)."""
    if kind == N.ZDT:
        nx = 30 + 5 * (param - 1) if prob_id == 5 else param
        lb, ub = np.zeros(nx), np.ones(nx)
        if prob_id == 4:
            lb[1:], ub[1:] = -5.0, 5.0
        return lb, ub
    return np.zeros(param), np.ones(param)


def mo_uniform_batch(kind: int, prob_id: int, param: int, n: int, seed: int, fdim: int = 0) -> np.ndarray:
    """n ZDT / DTLZ decision vectors, uniform within the bounds."""
    lb, ub = mo_bounds(kind, prob_id, param, fdim)
    rs = np.random.RandomState(seed)
    return lb + (ub - lb) * rs.random_sample((n, lb.size))


def rastrigin_batch(n: int = 4096, dim: int = 50, seed: int = 1) -> np.ndarray:
    return uniform_batch(N.RASTRIGIN, dim, n, seed)


def rosenbrock_batch(n: int = 65536, dim: int = 1000, seed: int = 2) -> np.ndarray:
    return uniform_batch(N.ROSENBROCK, dim, n, seed)


def lj_batch(n: int = 16384, atoms: int = 150, seed: int = 3) -> np.ndarray:
    return uniform_batch(N.LENNARD_JONES, atoms, n, seed)


def lj_encode(pos: np.ndarray) -> np.ndarray:
    """Decision vector of an N x 3 cluster in the pinned-atom convention of
    lennard_jones::_r (src/problems/lennard_jones.cpp:132-151): translate atom 0
    to the origin, rotate atom 1 onto +z and atom 2 into the y-z plane."""
    p = pos - pos[0]
    ez = p[1] / np.linalg.norm(p[1])
    v = p[2] - (p[2] @ ez) * ez
    ey = v / np.linalg.norm(v)
    ex = np.cross(ey, ez)
    q = p @ np.stack([ex, ey, ez]).T
    return np.concatenate([[q[1, 2], q[2, 1], q[2, 2]], q[3:].reshape(-1)])


def lj_lattice_batch(n: int, atoms: int = 150, sigma: float = 0.05, seed: int = 13) -> np.ndarray:
    """Clusters cut from an fcc lattice at the LJ pair-minimum spacing, jittered."""
    rs = np.random.RandomState(seed)
    a = 2.0 ** (1.0 / 6.0) * np.sqrt(2.0)  # nearest-neighbour distance 2^(1/6)
    k = int(np.ceil((atoms / 4.0) ** (1.0 / 3.0))) + 1
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    cells = np.array([[i, j, l] for i in range(k) for j in range(k) for l in range(k)], dtype=float)
    lat = (cells[:, None, :] + base[None, :, :]).reshape(-1, 3) * a
    lat = lat[np.argsort(np.linalg.norm(lat - lat.mean(0), axis=1), kind="stable")][:atoms]
    out = np.empty((n, 3 * atoms - 6))
    for r in range(n):
        out[r] = lj_encode(lat + rs.normal(0.0, sigma, lat.shape))
    return out


def nsga2_points(n: int = 20000, m: int = 3, layers: int = 30, dup_frac: float = 0.05, seed: int = 4) -> np.ndarray:
    """Nested fronts: layer k holds points (1 + 0.1 k) * w, w uniform on the unit
    simplex (normalised exponentials), jittered by N(0, 1e-3); dup_frac of the
    rows are exact copies of earlier rows; the rows are shuffled."""
    rs = np.random.RandomState(seed)
    n_dup = int(round(n * dup_frac))
    n_uni = n - n_dup
    sizes = np.full(layers, n_uni // layers)
    sizes[: n_uni % layers] += 1
    rows = []
    for k, sz in enumerate(sizes):
        e = -np.log(1.0 - rs.random_sample((sz, m)))
        w = e / e.sum(axis=1, keepdims=True)
        rows.append((1.0 + 0.1 * k) * w + rs.normal(0.0, 1e-3, (sz, m)))
    pts = np.concatenate(rows)
    if n_dup:
        pts = np.concatenate([pts, pts[rs.randint(0, n_uni, n_dup)]])
    return np.ascontiguousarray(pts[rs.permutation(n)])


@dataclass
class island_request:
    kind: int
    param: int
    n: int
    dvs: np.ndarray

    @property
    def nx(self) -> int:
        return nx_of(self.kind, self.param)


def sphere_front(n: int = 2000, m: int = 5, seed: int = 6) -> np.ndarray:
    """n points of m objectives on the positive orthant of the unit sphere (squared uniform directions,
    normalised): a front on which most points are non-dominated, the hard case of the WFG hypervolume."""
    w = np.random.default_rng(seed).random((n, m)) ** 2
    return np.ascontiguousarray(w / np.linalg.norm(w, axis=1, keepdims=True))


def archipelago(islands: int = 64, seed: int = 5, pop_lo: int = 32, pop_hi: int = 4096, dim_lo: int = 10,
                dim_hi: int = 500) -> list[island_request]:
    """One migration epoch of a mixed archipelago."""
    rs = np.random.RandomState(seed)
    kinds = (N.RASTRIGIN, N.ROSENBROCK, N.LENNARD_JONES)
    out = []
    for i in range(islands):
        pop = int(round(np.exp(rs.uniform(np.log(pop_lo), np.log(pop_hi)))))
        dim = int(rs.randint(dim_lo, dim_hi + 1))
        kind = kinds[i % 3]
        param = max(3, int(round((dim + 6) / 3))) if kind == N.LENNARD_JONES else dim
        lb, ub = bounds(kind, param)
        dvs = lb + (ub - lb) * rs.random_sample((pop, lb.size))
        out.append(island_request(kind, param, pop, np.ascontiguousarray(dvs)))
    return out
