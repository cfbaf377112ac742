"""Pins the CPU oracle (oracle/oracle.cpp) to the reference.

1. The reference's own known answers (tests/lennard_jones.cpp:59-60,
   tests/rastrigin.cpp:56-62, tests/rosenbrock.cpp:70-79,
   tests/multi_objective.cpp:81-182).
2. The golden fixtures generated from the reference's compiled sources
   (tests/golden/gen_golden.py): the "mirror" functions must reproduce them
   exactly on x86-64 (same libm), the long-double functions within 1e-13 of
   the condition scale.
3. Where the reference library is built here, a fresh cross-check.
"""
import math
import platform

import numpy as np
import pytest

from pathlib import Path

GOLD = Path(__file__).resolve().parent / "golden"
EXACT = platform.machine() in ("x86_64", "AMD64")


def cases(npz):
    names = sorted({k.split("/")[0] for k in npz.files})
    return names


@pytest.fixture(scope="module")
def fit():
    return np.load(GOLD / "fitness.npz")


@pytest.fixture(scope="module")
def mo():
    return np.load(GOLD / "mo.npz")


# ---------------------------------------------------------------- known answers

def test_lj_known_answers(orc):
    f = orc.batch_fitness(3, 3, np.array([[1.12, -0.33, 2.34], [1.23, -1.23, 0.33]]))
    assert math.isclose(f[0], -1.7633355813175688, rel_tol=1e-15)
    assert math.isclose(f[1], -1.833100934753864, rel_tol=1e-15)
    fl, _ = orc.batch_fitness_ld(3, 3, np.array([[1.12, -0.33, 2.34], [1.23, -1.23, 0.33]]))
    assert math.isclose(fl[0], -1.7633355813175688, rel_tol=1e-15)
    assert math.isclose(fl[1], -1.833100934753864, rel_tol=1e-15)


def test_rastrigin_known_answers(orc):
    assert orc.batch_fitness(1, 1, np.array([[1.0]]))[0] == 1.0
    assert orc.batch_fitness(1, 5, np.ones((1, 5)))[0] == 5.0
    g = orc.batch_gradient(1, 5, np.ones((1, 5)))
    assert np.allclose(g, 2.0, rtol=1e-14, atol=0)


def test_rosenbrock_known_answers(orc):
    assert orc.batch_fitness(2, 2, np.array([[1.0, 1.0]]))[0] == 0.0
    assert orc.batch_fitness(2, 5, np.ones((1, 5)))[0] == 0.0
    g2 = orc.batch_gradient(2, 2, np.array([[0.1, 0.2]]))[0]
    assert abs(g2[0] + 9.4) < 1e-8 and abs(g2[1] - 38.0) < 1e-8
    g5 = orc.batch_gradient(2, 5, np.array([[0.1, 0.2, 0.3, 0.4, 0.5]]))[0]
    for got, want in zip(g5, (-9.4, 15.6, 13.4, 6.4, 68.0)):
        assert abs(got - want) < 1e-8


def test_fnds_reference_examples(orc):
    r = orc.fnds(np.array([[0, 7], [1, 5], [2, 3], [4, 2], [7, 1], [10, 0], [2, 6], [4, 4], [10, 2], [6, 6],
                           [9, 5]], float))
    fronts = [r["front_indices"][a:b].tolist() for a, b in zip(r["front_offsets"][:-1], r["front_offsets"][1:])]
    assert fronts == [[0, 1, 2, 3, 4, 5], [6, 7, 8], [9, 10]]
    assert r["dom_count"].tolist() == [0, 0, 0, 0, 0, 0, 2, 2, 3, 5, 5]
    dl = [r["dl_indices"][a:b].tolist() for a, b in zip(r["dl_offsets"][:-1], r["dl_offsets"][1:])]
    assert dl == [[], [6, 9, 10], [6, 7, 9, 10], [7, 8, 9, 10], [8, 10], [8], [9], [9, 10], [], [], []]
    assert r["rank"].tolist() == [0, 0, 0, 0, 0, 0, 1, 1, 1, 2, 2]

    r = orc.fnds(np.array([[1, 2, 3], [-2, 3, 7], [-1, -2, -3], [0, 0, 0]], float))
    fronts = [r["front_indices"][a:b].tolist() for a, b in zip(r["front_offsets"][:-1], r["front_offsets"][1:])]
    assert fronts == [[1, 2], [3], [0]]
    assert r["dom_count"].tolist() == [2, 0, 0, 1]
    assert r["rank"].tolist() == [2, 0, 0, 1]

    r = orc.fnds(np.zeros((4, 0)))
    assert r["front_offsets"].tolist() == [0, 4] and r["rank"].tolist() == [0, 0, 0, 0]
    for bad in (np.zeros((1, 3)), np.zeros((1, 0)), np.zeros((0, 0))):
        with pytest.raises(ValueError):
            orc.fnds(bad)


def test_crowding_reference_examples(orc):
    inf = math.inf
    assert orc.crowding(np.array([[0, 0], [-1, 1], [2, -2]], float)).tolist() == [2, inf, inf]
    assert orc.crowding(np.array([[0.25, 0.25], [-1, 1], [2, -2]], float)).tolist() == [2, inf, inf]
    assert orc.crowding(np.array([[0, 0, 0], [-1, 1, 2], [2, -2, -2]], float)).tolist() == [3, inf, inf]
    assert orc.crowding(np.array([[0, 0], [1, -1], [2, -2], [4, -4]], float)).tolist() == [inf, 1.0, 1.5, inf]
    assert orc.crowding(np.array([[0, 0], [0, 0]], float)).tolist() == [inf, inf]
    for bad in (np.zeros((0, 2)), np.zeros((2, 0)), np.zeros((1, 2)), np.zeros((2, 1))):
        with pytest.raises(ValueError):
            orc.crowding(bad)


def test_pareto_dominance_examples(orc):
    assert orc.pareto_dominance([1, 2, 3], [4, 5, 6])
    assert not orc.pareto_dominance([4, 5, 6], [4, 5, 6])
    assert orc.pareto_dominance([4, 5, 5], [4, 5, 6])
    assert not orc.pareto_dominance([1, 2, 3], [2, 1, 5])
    assert orc.pareto_dominance([2], [3])
    assert not orc.pareto_dominance(np.array([]), np.array([]))
    # NaN orders after every number (custom_comparisons.hpp:54-89)
    assert orc.pareto_dominance([1.0, 1.0], [1.0, math.nan])
    assert not orc.pareto_dominance([math.nan, 1.0], [1.0, 1.0])


# ------------------------------------------------------------------ golden vectors

def test_fitness_golden(orc, fit):
    for name in cases(fit):
        kind, param = fit[f"{name}/kind"]
        x, f = fit[f"{name}/x"], fit[f"{name}/f"]
        mine = orc.batch_fitness(int(kind), int(param), x, threads=2)
        fl, sc = orc.batch_fitness_ld(int(kind), int(param), x)
        if EXACT:
            assert np.array_equal(mine, f), name
        else:
            assert np.all(np.abs(mine - f) <= 1e-15 * sc), name
        assert np.all(np.abs(fl - f) <= 1e-13 * sc), (name, np.max(np.abs(fl - f) / sc))


def test_gradient_golden(orc, fit):
    for name in cases(fit):
        if f"{name}/g" not in fit.files:
            continue
        kind, param = fit[f"{name}/kind"]
        x, g = fit[f"{name}/x"], fit[f"{name}/g"]
        mine = orc.batch_gradient(int(kind), int(param), x)
        gl, gs = orc.batch_gradient_ld(int(kind), int(param), x)
        if EXACT:
            assert np.array_equal(mine, g), name
        assert np.all(np.abs(gl - g) <= 1e-13 * gs), (name, np.max(np.abs(gl - g) / gs))


def _fronts(off, idx):
    return [idx[a:b].tolist() for a, b in zip(off[:-1], off[1:])]


def test_fnds_golden(orc, mo):
    for name in cases(mo):
        p = mo[f"{name}/points"]
        r = orc.fnds(p)
        for key in ("rank", "dom_count", "dl_offsets", "dl_indices"):
            assert np.array_equal(r[key], mo[f"{name}/{key}"]), (name, key)
        assert _fronts(r["front_offsets"], r["front_indices"]) == _fronts(mo[f"{name}/front_offsets"],
                                                                          mo[f"{name}/front_indices"]), name


def test_crowding_golden(orc, mo):
    for name in cases(mo):
        p = mo[f"{name}/points"]
        if p.shape[1] < 2:
            continue
        cd = orc.nsga2_crowding(p, mo[f"{name}/front_offsets"], mo[f"{name}/front_indices"])
        want = mo[f"{name}/crowding"]
        # same std::sort implementation -> identical including tie order
        assert np.array_equal(cd, want, equal_nan=True), name


# ------------------------------------------------------------ fresh cross-check

def test_oracle_vs_reference_fresh(orc, ref):
    from pagmo2_gb300 import workloads as W

    for kind, param, n in ((1, 50, 256), (2, 1000, 32), (3, 150, 4), (3, 10, 64)):
        x = W.uniform_batch(kind, param, n, seed=999 + kind)
        f, fe = ref.thread_bfe(kind, param, x)
        assert fe == n
        assert np.array_equal(orc.batch_fitness(kind, param, x), f)
        if kind != 3:
            assert np.array_equal(orc.batch_gradient(kind, param, x), ref.gradient_rows(kind, param, x))
    p = W.nsga2_points(400, 3, layers=6, seed=77)
    a, b = orc.fnds(p), ref.fnds(p)
    for key in a:
        assert np.array_equal(a[key], b[key]), key


def test_select_and_sort_population_golden(orc, mo):
    for name in cases(mo):
        p = mo[f"{name}/points"]
        assert np.array_equal(orc.sort_population_mo(p), mo[f"{name}/sort_population"]), name
        for key in mo.files:
            if key.startswith(f"{name}/select_best_"):
                nb = int(key.rsplit("_", 1)[1])
                assert np.array_equal(orc.select_best_n_mo(p, nb), mo[key]), key


def test_ackley_griewank_schwefel_known_answers(orc):
    # tests/ackley.cpp:53-57, tests/griewank.cpp:52-56, tests/schwefel.cpp:52-56
    x1, x3 = np.array([[1.12]]), np.array([[-23.45, 12.34, 111.12]])
    for kind, k1, k3 in ((4, 4.659037611351948, 21.941495638130885), (5, 0.5646311537232878, 4.241511427781268),
                         (6, 418.0067810680098, 1338.0260195323838)):
        assert math.isclose(orc.batch_fitness(kind, 1, x1)[0], k1, rel_tol=1e-15)
        assert math.isclose(orc.batch_fitness(kind, 3, x3)[0], k3, rel_tol=1e-15)
        f1, _ = orc.batch_fitness_ld(kind, 1, x1)
        f3, _ = orc.batch_fitness_ld(kind, 3, x3)
        assert math.isclose(f1[0], k1, rel_tol=1e-14) and math.isclose(f3[0], k3, rel_tol=1e-14)
        with pytest.raises(ValueError, match="gradient"):
            orc.batch_gradient(kind, 3, x3)
