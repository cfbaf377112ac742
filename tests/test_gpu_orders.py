"""GPU parity of the orderings behind crowding distance, select_best_N_mo and
sort_population_mo (through the C ABI): the device sort leaves exactly the
permutation std::sort leaves -- on random, tie-heavy, patterned and McIlroy
adversary inputs (which drive the introsort into its heapsort fallback), in
shared memory (up to 4096 pairs) and in global memory (larger) -- and the
index lists equal the oracle's (std::sort itself; the oracle is pinned to the
reference by tests/test_oracle_sorting.py) and the reference's known answers
(tests/multi_objective.cpp:183-262).
"""
import math

import numpy as np
import pytest

from pagmo2_gb300 import _native as N
from pagmo2_gb300 import multi_objective as MO
from pagmo2_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def key_cases(orc, rng):
    for n in (0, 1, 2, 3, 16, 17, 18, 31, 33, 64, 100, 257, 667, 1000, 4096, 4097, 10000, 50000):
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
    yield "extremes", np.array([np.iinfo(np.int64).max, np.iinfo(np.int64).min, 0, -1, 1] * 40)


def test_std_sort_permutation(ctx, orc):
    rng = np.random.default_rng(21)
    for label, k in key_cases(orc, rng):
        v = rng.permutation(k.size).astype(np.int32)
        want_k, want_v = orc.sort_keys(k, v, method="std")
        got_k, got_v = MO.std_sort_keys(k, v, ctx)
        assert np.array_equal(got_k, want_k), label
        assert np.array_equal(got_v, want_v), label


def tie_heavy(rng, n, m, levels):
    return rng.integers(0, levels, (n, m)).astype(np.float64)


def test_crowding_ties_bit_exact(ctx, orc):
    rng = np.random.default_rng(22)
    for n, m, levels in ((2, 2, 1), (3, 2, 1), (17, 2, 2), (40, 3, 3), (500, 2, 9), (5000, 3, 20), (9000, 2, 4)):
        p = tie_heavy(rng, n, m, levels)
        assert np.array_equal(MO.crowding_distance(p, ctx), orc.crowding(p), equal_nan=True), (n, m, levels)


def test_survival_crowding_tie_heavy(ctx, orc):
    rng = np.random.default_rng(23)
    for n, m, levels in ((64, 2, 3), (1000, 3, 6), (3000, 2, 40), (6000, 3, 5)):
        p = tie_heavy(rng, n, m, levels)
        rank, dc, off, idx, cd = MO.nsga2_survival(p, ctx)
        want = orc.fnds(p, dom_list=False)
        assert np.array_equal(off, want["front_offsets"]) and np.array_equal(idx, want["front_indices"])
        assert np.array_equal(cd, orc.nsga2_crowding(p, want["front_offsets"], want["front_indices"]),
                              equal_nan=True), (n, m, levels)


def test_one_front_larger_than_shared_memory(ctx, orc):
    # 2 objectives on an anti-diagonal: all 12000 points in one front, sorted in global memory
    rng = np.random.default_rng(24)
    t = np.round(rng.random(12000) * 3000) / 3000
    p = np.stack([t, 1.0 - t], axis=1)
    rank, dc, off, idx, cd = MO.nsga2_survival(p, ctx)
    assert off.size == 2
    assert np.array_equal(cd, orc.nsga2_crowding(p, off, idx), equal_nan=True)
    assert MO.sort_population_mo(p, ctx) == orc.sort_population_mo(p).tolist()
    assert MO.select_best_N_mo(p, 5000, ctx) == orc.select_best_n_mo(p, 5000).tolist()


def test_sort_population_mo_known_answers(ctx):
    assert MO.sort_population_mo(np.zeros((0, 2)), ctx) == []
    assert MO.sort_population_mo([[1, 5, 2, 3]], ctx) == [0]
    assert MO.sort_population_mo([[0.25, 0.25], [-1, 1], [2, -2]], ctx) == [1, 2, 0]
    ex = [[0, 7], [1, 5], [2, 3], [4, 2], [7, 1], [10, 0], [2, 6], [4, 4], [10, 2], [6, 6], [9, 5]]
    assert MO.sort_population_mo(ex, ctx) == [0, 5, 4, 3, 1, 2, 6, 8, 7, 9, 10]
    assert MO.sort_population_mo([[v] for v in range(11)], ctx) == list(range(11))
    with pytest.raises(ValueError, match="at least two objectives"):
        MO.sort_population_mo(np.zeros((2, 0)), ctx)


def test_select_best_n_mo_known_answers(ctx):
    assert MO.select_best_N_mo(np.zeros((0, 2)), 10, ctx) == []
    assert MO.select_best_N_mo([[1, 2]], 10, ctx) == [0]
    ex = [[1, 2], [2, 4], [-3, 2], [-3, -3]]
    assert MO.select_best_N_mo(ex, 10, ctx) == [0, 1, 2, 3]
    assert MO.select_best_N_mo(ex, 4, ctx) == [0, 1, 2, 3]
    for ex in ([[0, 7], [1, 5], [2, 3], [4, 2], [7, 1], [10, 0], [2, 6], [4, 4], [10, 2], [6, 6], [9, 5]],
               [[0, 7, -2], [1, 5, -4], [2, 3, 1], [4, 2, 2], [7, 1, -10], [10, 0, 43]],
               [[1, 1], [2, 2], [-1, -1], [1, -1], [-1, 1], [0, 0], [2, 2], [0, 0], [-2, 2], [3, -2], [-10, 2],
                [-8, 4], [4, -8]]):
        full = MO.sort_population_mo(ex, ctx)
        for n_best in range(1, len(ex) + 3):
            sel = MO.select_best_N_mo(ex, n_best, ctx)
            assert sorted(sel) == sorted(full[:min(n_best, len(ex))])
    with pytest.raises(ValueError, match="at least two objectives"):
        MO.select_best_N_mo(np.zeros((6, 0)), 2, ctx)
    assert MO.select_best_N_mo([[1, 2], [3, 4], [0, 1], [1, 0], [2, 2], [2, 4]], 0, ctx) == []


@pytest.mark.parametrize("n,m,levels", [(12, 2, 3), (64, 3, 4), (300, 2, 50), (1000, 3, 6), (2000, 4, 3)])
def test_select_and_sort_population_tie_heavy(ctx, orc, n, m, levels):
    rng = np.random.default_rng(n + m)
    p = tie_heavy(rng, n, m, levels)
    assert MO.sort_population_mo(p, ctx) == orc.sort_population_mo(p).tolist()
    for n_best in sorted({1, 2, n // 7, n // 3, n // 2, n - 1, n, n + 5}):
        assert MO.select_best_N_mo(p, n_best, ctx) == orc.select_best_n_mo(p, n_best).tolist(), n_best


def test_select_best_nested_fronts_workload(ctx, orc):
    p = W.nsga2_points(4000, 3, layers=30)
    for n_best in (1, 1000, 2000, 3999):
        assert MO.select_best_N_mo(p, n_best, ctx) == orc.select_best_n_mo(p, n_best).tolist()
    assert MO.sort_population_mo(p, ctx) == orc.sort_population_mo(p).tolist()


def test_single_objective_critical_front_raises(ctx):
    # a critical front needs crowding_distance, which needs two objectives
    with pytest.raises(ValueError, match="at least two objectives"):
        MO.select_best_N_mo([[1.0], [1.0], [2.0]], 1, ctx)
    assert MO.select_best_N_mo([[3.0], [1.0], [2.0]], 2, ctx) == [1, 2]
    assert MO.sort_population_mo([[3.0], [1.0], [2.0]], ctx) == [1, 2, 0]


def test_device_entry_points_status(ctx, orc):
    import torch

    L = N.lib()
    p = tie_heavy(np.random.default_rng(25), 500, 3, 5)
    dp = torch.from_numpy(p).cuda()
    out = torch.empty(500, dtype=torch.int32, device="cuda")
    st = torch.full((1,), 7, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    N.check(L.pgx_select_best_n_mo_device(ctx.handle, dp.data_ptr(), 500, 3, 123, out.data_ptr(), st.data_ptr(), s))
    torch.cuda.synchronize()
    assert st.item() == 0
    assert out[:123].cpu().tolist() == orc.select_best_n_mo(p, 123).tolist()
    N.check(L.pgx_sort_population_mo_device(ctx.handle, dp.data_ptr(), 500, 3, out.data_ptr(), st.data_ptr(), s))
    torch.cuda.synchronize()
    assert st.item() == 0
    assert out.cpu().tolist() == orc.sort_population_mo(p).tolist()
    # the reference would throw: status 1
    d1 = torch.tensor([[1.0], [1.0], [2.0]], dtype=torch.float64, device="cuda")
    N.check(L.pgx_select_best_n_mo_device(ctx.handle, d1.data_ptr(), 3, 1, 1, out.data_ptr(), st.data_ptr(), s))
    torch.cuda.synchronize()
    assert st.item() == 1


def test_nan_and_infinite_objectives(ctx, orc):
    rng = np.random.default_rng(26)
    p = tie_heavy(rng, 300, 3, 6)
    p[rng.integers(0, 300, 20), rng.integers(0, 3, 20)] = math.nan
    p[rng.integers(0, 300, 10), rng.integers(0, 3, 10)] = math.inf
    p[rng.integers(0, 300, 10), rng.integers(0, 3, 10)] = -math.inf
    p[rng.integers(0, 300, 10), 0] = -0.0
    assert MO.sort_population_mo(p, ctx) == orc.sort_population_mo(p).tolist()
    for n_best in (10, 150, 299):
        assert MO.select_best_N_mo(p, n_best, ctx) == orc.select_best_n_mo(p, n_best).tolist()
    rank, dc, off, idx, cd = MO.nsga2_survival(p, ctx)
    want = orc.fnds(p, dom_list=False)
    assert np.array_equal(cd, orc.nsga2_crowding(p, want["front_offsets"], want["front_indices"]), equal_nan=True)


def test_select_and_sort_population_golden(ctx):
    """The reference's own index lists (tests/golden/gen_golden.py), ties and NaN cases included."""
    from pathlib import Path

    gold = np.load(Path(__file__).resolve().parent / "golden" / "mo.npz")
    for name in sorted({k.split("/")[0] for k in gold.files}):
        p = gold[f"{name}/points"]
        assert MO.sort_population_mo(p, ctx) == gold[f"{name}/sort_population"].tolist(), name
        for key in gold.files:
            if key.startswith(f"{name}/select_best_"):
                nb = int(key.rsplit("_", 1)[1])
                assert MO.select_best_N_mo(p, nb, ctx) == gold[key].tolist(), key
