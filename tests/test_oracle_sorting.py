"""Pins the oracle's orderings (oracle/sorting.cpp) to the reference.

pagmo's crowding distance, select_best_N_mo and sort_population_mo sort with
std::sort, whose order of tied elements is the standard library's (libstdc++
introsort). The oracle restates that introsort three times -- sequentially and
with the two partition formulations the GPU uses (32-wide chunks; complete
stopper lists) -- and each must leave exactly the
permutation std::sort leaves, on random, tie-heavy, patterned and adversarial
inputs (McIlroy's adversary drives the introsort into its heapsort fallback).
select_best_N_mo / sort_population_mo are pinned to the reference's known
answers (tests/multi_objective.cpp:183-262) and, where the reference library
is built, to the reference itself on tie-heavy populations.
"""
import numpy as np
import pytest

SIZES = list(range(0, 70)) + [100, 257, 667, 1000, 4096]


def key_cases(orc, rng):
    for n in SIZES:
        for distinct in (1, 2, 3, 7, 1 << 40):
            yield f"random n={n} distinct={distinct}", rng.integers(0, distinct, n)
        if n > 1:
            yield f"sorted {n}", np.arange(n)
            yield f"reversed {n}", np.arange(n)[::-1].copy()
            yield f"organ pipe {n}", np.concatenate([np.arange(n // 2), np.arange(n - n // 2)[::-1]])
            yield f"sawtooth {n}", np.arange(n) % 5
            adv = orc.quicksort_adversary(n)
            yield f"adversary {n}", adv
            yield f"adversary with ties {n}", adv // 3


@pytest.mark.parametrize("method", ["intro", "chunked", "lists"])
def test_restated_introsort_matches_std_sort(orc, method):
    rng = np.random.default_rng(11)
    for label, k in key_cases(orc, rng):
        ks, vs = orc.sort_keys(k, method="std")
        k2, v2 = orc.sort_keys(k, method=method)
        assert np.array_equal(ks, k2) and np.array_equal(vs, v2), label


def test_adversary_reaches_heapsort(orc):
    for n in (100, 1000, 4096):
        h0 = orc.depth_limit_hits()
        orc.sort_keys(orc.quicksort_adversary(n), method="chunked")
        assert orc.depth_limit_hits() > h0


def test_restated_heapsort_matches_std_partial_sort(orc):
    rng = np.random.default_rng(12)
    for n in (0, 1, 2, 3, 4, 5, 16, 17, 64, 101, 1000):
        for distinct in (1, 3, 1 << 40):
            k = rng.integers(0, distinct, n)
            a = orc.sort_keys(k, method="heap")
            b = orc.sort_keys(k, method="std_heap")
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (n, distinct)


# ------------------------------------------------ select_best_N_mo / sort_population_mo

def test_sort_population_mo_known_answers(orc):
    assert list(orc.sort_population_mo(np.zeros((0, 2)))) == []
    assert list(orc.sort_population_mo([[1, 5, 2, 3]])) == [0]
    assert list(orc.sort_population_mo([[0.25, 0.25], [-1, 1], [2, -2]])) == [1, 2, 0]
    ex = [[0, 7], [1, 5], [2, 3], [4, 2], [7, 1], [10, 0], [2, 6], [4, 4], [10, 2], [6, 6], [9, 5]]
    assert list(orc.sort_population_mo(ex)) == [0, 5, 4, 3, 1, 2, 6, 8, 7, 9, 10]
    assert list(orc.sort_population_mo([[v] for v in range(11)])) == list(range(11))
    with pytest.raises(ValueError):
        orc.sort_population_mo(np.zeros((2, 0)))


def test_select_best_n_mo_known_answers(orc):
    assert list(orc.select_best_n_mo(np.zeros((0, 2)), 10)) == []
    assert list(orc.select_best_n_mo([[1, 2]], 10)) == [0]
    ex = [[1, 2], [2, 4], [-3, 2], [-3, -3]]
    assert list(orc.select_best_n_mo(ex, 10)) == [0, 1, 2, 3]
    assert list(orc.select_best_n_mo(ex, 4)) == [0, 1, 2, 3]
    for ex in ([[0, 7], [1, 5], [2, 3], [4, 2], [7, 1], [10, 0], [2, 6], [4, 4], [10, 2], [6, 6], [9, 5]],
               [[0, 7, -2], [1, 5, -4], [2, 3, 1], [4, 2, 2], [7, 1, -10], [10, 0, 43]],
               [[1, 1], [2, 2], [-1, -1], [1, -1], [-1, 1], [0, 0], [2, 2], [0, 0], [-2, 2], [3, -2], [-10, 2],
                [-8, 4], [4, -8]]):
        full = list(orc.sort_population_mo(ex))
        for N in range(1, len(ex) + 3):
            sel = list(orc.select_best_n_mo(ex, N))
            assert sorted(sel) == sorted(full[:min(N, len(ex))])
    with pytest.raises(ValueError):
        orc.select_best_n_mo(np.zeros((6, 0)), 2)
    assert list(orc.select_best_n_mo([[1, 2], [3, 4], [0, 1], [1, 0], [2, 2], [2, 4]], 0)) == []


def tie_heavy_population(rng, n, m, levels):
    """Points on a coarse grid: many equal objective values and duplicates."""
    return rng.integers(0, levels, (n, m)).astype(np.float64)


def test_select_and_sort_population_against_reference(orc, ref):
    rng = np.random.default_rng(13)
    for n, m, levels in ((12, 2, 3), (40, 2, 5), (64, 3, 4), (200, 2, 50), (300, 3, 6), (150, 4, 3)):
        for rep in range(3):
            p = tie_heavy_population(rng, n, m, levels)
            assert np.array_equal(orc.sort_population_mo(p), ref.sort_population_mo(p)), (n, m, levels, rep)
            for N in sorted({1, 2, n // 3, n // 2, n - 1, n}):
                assert np.array_equal(orc.select_best_n_mo(p, N), ref.select_best_n_mo(p, N)), (n, m, N)


def test_crowding_ties_against_reference(orc, ref):
    rng = np.random.default_rng(14)
    for n, m, levels in ((5, 2, 2), (33, 3, 3), (200, 2, 7), (700, 3, 10)):
        p = tie_heavy_population(rng, n, m, levels)
        a, b = orc.crowding(p), ref.crowding(p)
        assert np.array_equal(np.isnan(a), np.isnan(b))
        assert np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])
