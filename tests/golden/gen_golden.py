"""Generates the golden fixtures in this directory from the reference itself.

The reference's hot-path sources are compiled unmodified by oracle/Makefile
into oracle/_ref/libpagmo_ref.so (this needs the reference tree, so run it
where that exists):

    make -C oracle ref REF_ROOT=<pagmo2 source tree>
    python tests/golden/gen_golden.py

Outputs (numpy .npz, small):
  fitness.npz  per case: the decision vectors, bfe{thread_bfe{}} fitness, and
               problem::gradient rows (rastrigin, rosenbrock); ackley,
               griewank and schwefel (fitness only)
  mo_problems.npz  per ZDT / DTLZ case: the problem (kind, prob_id, param,
               fdim, alpha), the decision vectors, bfe{thread_bfe{}} fitness
               (n x nobj) and p_distance of every row
  hv.npz       per case: points, reference point and hypervolume(points).compute(ref)
  mo.npz       per case: the objective vectors, fast_non_dominated_sorting
               (rank, dom_count, fronts, dom_list), crowding_distance of
               every front of three or more points, sort_population_mo and
               select_best_N_mo for a few N
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

import oracle  # noqa: E402
from pagmo2_gb300 import workloads as W  # noqa: E402

RAS, ROS, LJ, ACK, GRI, SCH = 1, 2, 3, 4, 5, 6


def fitness_cases():
    cases = []
    for dim, n, seed in ((1, 16, 101), (5, 32, 102), (50, 64, 103), (173, 8, 104)):
        cases.append((f"rastrigin_{dim}", RAS, dim, W.uniform_batch(RAS, dim, n, seed)))
    for dim, n, seed in ((2, 32, 201), (5, 16, 202), (37, 16, 203), (1000, 4, 204)):
        cases.append((f"rosenbrock_{dim}", ROS, dim, W.uniform_batch(ROS, dim, n, seed)))
    for atoms, n, seed in ((3, 16, 301), (4, 8, 302), (7, 8, 303), (33, 4, 304), (150, 2, 305)):
        cases.append((f"lj_{atoms}", LJ, atoms, W.uniform_batch(LJ, atoms, n, seed)))
    for atoms, n, seed in ((13, 4, 311), (38, 2, 312), (150, 2, 313)):
        cases.append((f"ljlat_{atoms}", LJ, atoms, W.lj_lattice_batch(n, atoms, seed=seed)))
    # near the optimum (cancellation in the gradients)
    cases.append(("rosenbrock_near_opt", ROS, 64, 1.0 + 1e-3 * np.random.RandomState(205).standard_normal((8, 64))))
    cases.append(("rastrigin_near_opt", RAS, 64, 1e-3 * np.random.RandomState(105).standard_normal((8, 64))))
    # integer points: exact values in the reference
    cases.append(("rastrigin_ints", RAS, 7, np.random.RandomState(106).randint(-5, 6, (8, 7)).astype(float)))
    # fitness-only problems (no reference gradient)
    for kind, name in ((ACK, "ackley"), (GRI, "griewank"), (SCH, "schwefel")):
        for dim, n, seed in ((1, 16, 501), (3, 16, 502), (50, 32, 503), (173, 8, 504), (1000, 4, 505)):
            cases.append((f"{name}_{dim}", kind, dim, W.uniform_batch(kind, dim, n, seed + 10 * kind)))
        cases.append((f"{name}_near_opt", kind, 64,
                      W.bounds(kind, 64)[0] * 0 + (420.9687 if kind == SCH else 0.0)
                      + 1e-3 * np.random.RandomState(506 + kind).standard_normal((8, 64))))
    return cases


ZDT, DTLZ = 7, 8


def mo_problem_cases():
    """(name, (kind, prob_id, param, fdim, alpha), dvs) for ZDT and DTLZ."""
    cases = []
    for pid, params in ((1, (2, 30, 173)), (2, (2, 30)), (3, (2, 30)), (4, (2, 10)), (5, (2, 11, 30)),
                        (6, (2, 10, 64))):
        for param in params:
            x = W.mo_uniform_batch(ZDT, pid, param, 16, 600 + 10 * pid + param)
            x[0, :] = W.mo_bounds(ZDT, pid, param)[0]  # lower corner
            x[1, :] = W.mo_bounds(ZDT, pid, param)[1]  # upper corner
            cases.append((f"zdt{pid}_{param}", (ZDT, pid, param, 0, 0), x))
    for pid in range(1, 8):
        for dim, fdim, alpha in ((5, 3, 100), (12, 3, 100), (10, 2, 100), (30, 10, 100), (50, 40, 3)):
            if pid != 4 and alpha != 100:
                alpha = 100
            x = W.mo_uniform_batch(DTLZ, pid, dim, 16, 700 + 10 * pid + dim)
            x[0, :] = 0.0
            x[1, :] = 1.0
            x[2, :] = 0.5
            cases.append((f"dtlz{pid}_{dim}_{fdim}_{alpha}", (DTLZ, pid, dim, fdim, alpha), x))
    return cases


def hv_cases():
    """(name, points, reference point) for hypervolume of 2 and 3 objectives."""
    rs = np.random.RandomState(900)
    cases = []
    for n, m in ((1, 2), (3, 2), (128, 2), (1000, 2), (2, 3), (128, 3), (700, 3), (3000, 3)):
        cases.append((f"uniform_{n}x{m}", rs.random_sample((n, m)), np.full(m, 1.1)))
    for n, m in ((200, 2), (400, 3)):
        pts = np.floor(rs.random_sample((n, m)) * 8) / 8  # ties and duplicates
        pts[:5, 0] = 1.0  # on the border of the reference point in one coordinate
        cases.append((f"grid_{n}x{m}", pts, np.full(m, 1.0)))
    w = -np.log(rs.random_sample((600, 3)))
    w /= w.sum(axis=1, keepdims=True)
    cases.append(("simplex_layers_1800x3", np.concatenate([w, 1.5 * w, 2.0 * w]), np.full(3, 2.5)))
    return cases


def mo_cases():
    cases = []
    # tests/multi_objective.cpp fnds examples
    cases.append(("ex11", np.array([[0, 7], [1, 5], [2, 3], [4, 2], [7, 1], [10, 0], [2, 6], [4, 4], [10, 2], [6, 6],
                                    [9, 5]], float)))
    cases.append(("ex4", np.array([[1, 2, 3], [-2, 3, 7], [-1, -2, -3], [0, 0, 0]], float)))
    rs = np.random.RandomState(401)
    cases.append(("rand2", rs.random_sample((200, 2))))
    cases.append(("rand3", rs.random_sample((300, 3))))
    cases.append(("rand5", rs.random_sample((150, 5))))
    cases.append(("grid3", rs.randint(0, 4, (120, 3)).astype(float)))  # many ties and duplicates
    cases.append(("nested", W.nsga2_points(600, 3, layers=10, seed=402)))
    cases.append(("nested_nodup", W.nsga2_points(500, 3, layers=8, dup_frac=0.0, seed=403)))
    p = rs.random_sample((60, 3))
    p[3, 1] = np.nan
    p[17, 0] = np.nan
    p[17, 2] = np.nan
    p[25] = np.nan
    p[40, 2] = -0.0
    p[41, 2] = 0.0
    p[50, 0] = -np.inf
    p[51, 1] = np.inf
    cases.append(("special", p))
    cases.append(("single_front", np.stack([np.linspace(0, 1, 64), 1 - np.linspace(0, 1, 64)], 1)))
    return cases


def main():
    ref = oracle.reference()
    if ref is None:
        raise SystemExit("oracle/_ref/libpagmo_ref.so is missing: build it with `make -C oracle ref` first")
    fit = {}
    for name, kind, param, x in fitness_cases():
        x = np.ascontiguousarray(x)
        f, fe = ref.thread_bfe(kind, param, x)
        assert fe == x.shape[0]
        fit[f"{name}/kind"] = np.array([kind, param])
        fit[f"{name}/x"] = x
        fit[f"{name}/f"] = f
        if kind in (RAS, ROS):
            fit[f"{name}/g"] = ref.gradient_rows(kind, param, x)
    np.savez_compressed(HERE / "fitness.npz", **fit)

    mop = {}
    for name, spec, x in mo_problem_cases():
        x = np.ascontiguousarray(x)
        mop[f"{name}/spec"] = np.array(spec, dtype=np.int64)
        mop[f"{name}/x"] = x
        mop[f"{name}/f"] = ref.mo_thread_bfe(spec, x)
        mop[f"{name}/p_distance"] = ref.mo_p_distance(spec, x)
    np.savez_compressed(HERE / "mo_problems.npz", **mop)

    hv = {}
    for name, pts, r in hv_cases():
        hv[f"{name}/points"] = pts
        hv[f"{name}/ref"] = r
        hv[f"{name}/hv"] = np.array([ref.hypervolume(pts, r)])
    np.savez_compressed(HERE / "hv.npz", **hv)

    mo = {}
    for name, p in mo_cases():
        r = ref.fnds(p)
        mo[f"{name}/points"] = p
        for k, v in r.items():
            mo[f"{name}/{k}"] = v
        off, idx = r["front_offsets"], r["front_indices"]
        cd = np.full(p.shape[0], np.nan)
        for fi in range(off.size - 1):
            members = idx[off[fi]:off[fi + 1]]
            if members.size >= 3 and p.shape[1] >= 2:
                cd[members] = ref.crowding(p[members])
            elif members.size in (1, 2):
                cd[members] = np.inf
        mo[f"{name}/crowding"] = cd
        # select_best_N_mo and sort_population_mo of the same points (ties in std::sort's order)
        n = p.shape[0]
        mo[f"{name}/sort_population"] = ref.sort_population_mo(p)
        for nb in sorted({1, n // 3, n // 2, n - 1}):
            mo[f"{name}/select_best_{nb}"] = ref.select_best_n_mo(p, nb)
    np.savez_compressed(HERE / "mo.npz", **mo)
    print("wrote", HERE / "fitness.npz", HERE / "mo_problems.npz", HERE / "hv.npz", HERE / "mo.npz")


if __name__ == "__main__":
    main()
