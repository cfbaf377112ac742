"""GPU parity of NSGA-II survival (through the C ABI): fast non-dominated
sorting bit-exact with the reference (ranks, domination counts, fronts in the
reference's order, dom_list) and crowding distance bit-exact with the
reference on every point, tied objective values included: the device sorts
leave ties in the order the reference's std::sort (GNU libstdc++ introsort)
leaves them.
"""
import math
from pathlib import Path

import numpy as np
import pytest

from pagmo2_gb300 import _native as N
from pagmo2_gb300 import multi_objective as MO
from pagmo2_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def fronts_of(off, idx):
    return [list(map(int, idx[a:b])) for a, b in zip(off[:-1], off[1:])]


def check_crowding(got, want):
    """Bit-exact, NaN where the reference has NaN."""
    assert np.array_equal(got, want, equal_nan=True), "crowding differs from the reference"


def test_golden_fnds_and_crowding(ctx, orc):
    gold = np.load(GOLD / "mo.npz")
    for name in sorted({k.split("/")[0] for k in gold.files}):
        p = gold[f"{name}/points"]
        rank, dc, off, idx, cd = MO.nsga2_survival(p, ctx)
        assert np.array_equal(rank, gold[f"{name}/rank"]), name
        assert np.array_equal(dc, gold[f"{name}/dom_count"]), name
        assert fronts_of(off, idx) == fronts_of(gold[f"{name}/front_offsets"], gold[f"{name}/front_indices"]), name
        doff, didx = MO.dom_list_arrays(p, ctx)
        assert np.array_equal(doff, gold[f"{name}/dl_offsets"]), name
        assert np.array_equal(didx, gold[f"{name}/dl_indices"]), name
        check_crowding(cd, gold[f"{name}/crowding"])


def test_reference_fnds_examples(ctx):
    # tests/multi_objective.cpp:81-145
    ex = [[0, 7], [1, 5], [2, 3], [4, 2], [7, 1], [10, 0], [2, 6], [4, 4], [10, 2], [6, 6], [9, 5]]
    fronts, dom_list, dom_count, rank = MO.fast_non_dominated_sorting(ex, ctx)
    assert fronts == [[0, 1, 2, 3, 4, 5], [6, 7, 8], [9, 10]]
    assert dom_list == [[], [6, 9, 10], [6, 7, 9, 10], [7, 8, 9, 10], [8, 10], [8], [9], [9, 10], [], [], []]
    assert dom_count == [0, 0, 0, 0, 0, 0, 2, 2, 3, 5, 5]
    assert rank == [0, 0, 0, 0, 0, 0, 1, 1, 1, 2, 2]
    fronts, dom_list, dom_count, rank = MO.fast_non_dominated_sorting([[1, 2, 3], [-2, 3, 7], [-1, -2, -3],
                                                                       [0, 0, 0]], ctx)
    assert (fronts, dom_list, dom_count, rank) == ([[1, 2], [3], [0]], [[], [], [0, 3], [0]], [2, 0, 0, 1],
                                                   [2, 0, 0, 1])
    fronts, dom_list, dom_count, rank = MO.fast_non_dominated_sorting(np.zeros((4, 0)), ctx)
    assert (fronts, dom_list, dom_count, rank) == ([[0, 1, 2, 3]], [[], [], [], []], [0, 0, 0, 0], [0, 0, 0, 0])
    for bad in ([[0, 0, 0]], [[]], []):
        with pytest.raises(ValueError):
            MO.fast_non_dominated_sorting(bad, ctx)
    for bad in ([[1, 3], [3, 42, 3], []], [[3, 4, 5], []]):
        with pytest.raises(ValueError):
            MO.fast_non_dominated_sorting(bad, ctx)


def test_reference_crowding_examples(ctx):
    # tests/multi_objective.cpp:147-182
    inf = math.inf
    assert MO.crowding_distance([[0, 0], [-1, 1], [2, -2]], ctx).tolist() == [2, inf, inf]
    assert MO.crowding_distance([[0.25, 0.25], [-1, 1], [2, -2]], ctx).tolist() == [2, inf, inf]
    assert MO.crowding_distance([[0, 0, 0], [-1, 1, 2], [2, -2, -2]], ctx).tolist() == [3, inf, inf]
    assert MO.crowding_distance([[0.25, 0.25, 0.25], [-1, 1, 2], [2, -2, -2]], ctx).tolist() == [3, inf, inf]
    assert MO.crowding_distance([[0, 0], [1, -1], [2, -2], [4, -4]], ctx).tolist() == [inf, 1.0, 1.5, inf]
    assert MO.crowding_distance([[0, 0], [0, 0]], ctx).tolist() == [inf, inf]
    for bad in ([], [[], []], [[1, 2]], [[1], [2]], [[2, 3], [3, 4], [2, 4, 5]]):
        with pytest.raises(ValueError):
            MO.crowding_distance(bad, ctx)


def test_crowding_degenerate_objective_is_nan(ctx, orc):
    # df == 0 with interior points: 0/0 as in the reference
    p = np.array([[1.0, 0.0], [1.0, 0.5], [1.0, 1.0], [1.0, 2.0]])
    got = MO.crowding_distance(p, ctx)
    want = orc.crowding(p)
    assert np.array_equal(got, want, equal_nan=True)


def test_config4_nested_fronts_full(ctx, orc):
    p = W.nsga2_points()  # 20000 x 3, 30 layers, 5 % duplicates
    rank, dc, off, idx, cd = MO.nsga2_survival(p, ctx)
    want = orc.fnds(p, dom_list=False)
    assert np.array_equal(rank, want["rank"])
    assert np.array_equal(dc, want["dom_count"])
    assert np.array_equal(off, want["front_offsets"])
    assert np.array_equal(idx, want["front_indices"])
    check_crowding(cd, orc.nsga2_crowding(p, want["front_offsets"], want["front_indices"]))


def layered_points(sizes, m, seed, dup_frac=0.02):
    """Fronts of exactly the given sizes: layer k lies on the plane where the objectives sum to 2 k, with
    non-negative offsets summing to at most 1 and the corner (0, ..., 0, 2 k), which dominates every point of
    layer k + 1; a layer's points are mutually non-dominated, and about dup_frac of them are copies of others of
    the same layer. The rows are shuffled."""
    rs = np.random.RandomState(seed)
    rows = []
    for k, sz in enumerate(sizes):
        e = -np.log(1.0 - rs.random_sample((sz, m)))
        pts = e / e.sum(axis=1, keepdims=True) * rs.random_sample((sz, 1))  # offsets: sum <= 1
        pts[:, -1] = 2.0 * k - pts[:, :-1].sum(axis=1)
        pts[0, :-1], pts[0, -1] = 0.0, 2.0 * k
        nd = int(sz * dup_frac)
        if nd and sz > 1:
            pts[sz - nd:] = pts[rs.randint(0, sz - nd, nd)]
        rows.append(pts)
    p = np.concatenate(rows)
    return np.ascontiguousarray(p[rs.permutation(len(p))])


@pytest.mark.parametrize("sizes,m", [
    # up to 32768 points: fronts of up to 2048 members (and keys) sorted while the next front is scanned, larger
    # ones across the grid, a small front after a large one, single points
    ([3000, 40, 2049, 2048, 700, 5000, 10, 1, 2100, 300, 1, 1, 2047], 3),
    # beyond 32768 points (no per-point maps in shared memory)
    ([6000, 100, 2048, 2049, 5000, 30, 9000, 7000, 1, 4500, 3000, 200], 2),
])
def test_front_size_transitions(ctx, orc, sizes, m):
    p = layered_points(sizes, m, seed=len(sizes) + m)
    rank, dc, off, idx, cd = MO.nsga2_survival(p, ctx)
    want = orc.fnds(p, dom_list=False)
    assert np.array_equal(rank, want["rank"])
    assert np.array_equal(dc, want["dom_count"])
    assert np.array_equal(off, want["front_offsets"])
    assert np.array_equal(idx, want["front_indices"])
    assert len(off) - 1 == len(sizes)
    check_crowding(cd, orc.nsga2_crowding(p, want["front_offsets"], want["front_indices"]))


@pytest.mark.parametrize("n,m,seed", [(2, 2, 1), (3, 1, 2), (33, 2, 3), (257, 4, 4), (1000, 3, 5), (700, 7, 6)])
def test_random_sets(ctx, orc, n, m, seed):
    rs = np.random.RandomState(seed)
    p = rs.random_sample((n, m))
    p[rs.randint(0, n, n // 10)] = p[rs.randint(0, n, n // 10)]  # duplicates
    rank, dc, off, idx = MO.fnds_arrays(p, ctx)
    want = orc.fnds(p)
    assert np.array_equal(rank, want["rank"]) and np.array_equal(dc, want["dom_count"])
    assert fronts_of(off, idx) == fronts_of(want["front_offsets"], want["front_indices"])
    doff, didx = MO.dom_list_arrays(p, ctx)
    assert np.array_equal(doff, want["dl_offsets"]) and np.array_equal(didx, want["dl_indices"])


def test_single_objective_front_of_three_raises_in_survival(ctx):
    # crowding_distance needs two objectives (multi_objective.cpp:290-294)
    with pytest.raises(ValueError):
        MO.nsga2_survival(np.array([[1.0], [1.0], [1.0]]), ctx)
    rank, dc, off, idx, cd = MO.nsga2_survival(np.array([[1.0], [2.0], [3.0]]), ctx)
    assert rank.tolist() == [0, 1, 2] and cd.tolist() == [math.inf] * 3


def test_grid_barrier_wait_is_bounded(ctx, orc):
    """Failure detection without a fault: a cooperative kernel whose second block never arrives at the grid
    barrier; the first block's wait gives up after a bounded number of polls, the kernel returns, the host reads
    the flag, and the same context then runs a full survival pass."""
    import ctypes as C
    import time

    flag = C.c_int32(-1)
    t = time.perf_counter()
    N.check(N.lib().pgx_selftest_barrier_timeout(ctx.handle, 1 << 14, C.byref(flag)))
    assert flag.value == 1
    assert time.perf_counter() - t < 30.0
    p = W.nsga2_points(1000, 3, layers=8)
    rank, dc, off, idx, cd = MO.nsga2_survival(p, ctx)
    want = orc.fnds(p, dom_list=False)
    assert np.array_equal(off, want["front_offsets"]) and np.array_equal(idx, want["front_indices"])
