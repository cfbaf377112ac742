"""GPU hypervolume of 2 and 3 objectives (pgx_hypervolume) against the long-double oracle, within 1e-13
relative (all slabs are non-negative, so the bound is relative to the volume itself), against the reference's
own values (tests/golden/hv.npz, within 1e-12 relative: the reference's hv3d sweep subtracts), the known answers
of tests/hypervolume.cpp:229-297, and the reference's checks and messages."""
from pathlib import Path

import numpy as np
import pytest

from pagmo2_gb300 import _native as N
from pagmo2_gb300 import multi_objective as MO
from pagmo2_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden" / "hv.npz"


def hv(points, ref, ctx):
    return MO.hypervolume(points, context=ctx).compute(ref)


def test_known_answers(ctx):
    assert hv([[1, 2], [2, 1]], [3, 3], ctx) == 3.0
    assert hv([[1, 2], [2, 1]], [2, 2], ctx) == 0.0
    assert hv([[1, 1, 1], [2, 2, 2]], [3, 3, 3], ctx) == 8.0
    assert hv([[1, 2, 1], [2, 1, 1]], [2, 2, 2], ctx) == 0.0
    assert abs(hv([[2.3, 4.5], [3.4, 3.4], [6.0, 1.2]], [7, 7], ctx) - 17.91) <= 1e-14
    assert abs(hv([[2.3, 4.5, 3.2], [3.4, 3.4, 3.4], [6.0, 1.2, 3.6]], [7, 7, 7], ctx) - 66.386) <= 1e-13


def test_golden_and_long_double(ctx, orc):
    gold = np.load(GOLD)
    for name in sorted({k.split("/")[0] for k in gold.files}):
        p, r, want = gold[f"{name}/points"], gold[f"{name}/ref"], float(gold[f"{name}/hv"][0])
        got = hv(p, r, ctx)
        exact = orc.hypervolume(p, r)
        assert abs(got - exact) <= 1e-13 * exact, (name, got, exact)
        assert abs(got - want) <= 1e-12 * max(want, 1e-300), (name, got, want)


def test_workload_sizes(ctx, orc):
    p = W.nsga2_points(20000, 3, layers=30)
    r = p.max(axis=0) + 0.5
    got = hv(p, r, ctx)
    q = p[:4000]  # the oracle is O(n^2 log n): checked on the first 4000 points
    exact = orc.hypervolume(q, r)
    assert abs(hv(q, r, ctx) - exact) <= 1e-13 * exact
    # adding points can only grow the volume; duplicating every point changes nothing
    assert hv(np.concatenate([p, p]), r, ctx) == pytest.approx(got, rel=1e-14, abs=0)
    assert got >= hv(p[:10000], r, ctx)


def test_checks(ctx):
    with pytest.raises(ValueError, match="Point set cannot be empty."):
        MO.hypervolume(np.zeros((0, 2)), context=ctx)
    with pytest.raises(ValueError, match="All point set dimensions must be equal."):
        MO.hypervolume([[2.3, 3.4, 5.6], [1.0, 2.0, 3.0, 4.0]], context=ctx)
    with pytest.raises(ValueError, match="nan value"):
        MO.hypervolume([[1.0, np.nan]], context=ctx)
    h = MO.hypervolume([[1, 3], [2, 2], [3, 1]], context=ctx)
    for bad in ([3, 1], [1.5, 1.5], [0, 0]):
        with pytest.raises(ValueError, match="Reference point is invalid"):
            h.compute(bad)
    with pytest.raises(ValueError, match="Point set dimensions and reference point dimension must be equal."):
        h.compute([3, 3, 3])
    with pytest.raises(NotImplementedError, match="2 or 3 objectives"):
        MO.hypervolume([[1, 1, 1, 1], [2, 2, 2, 2]], context=ctx).compute([3, 3, 3, 3])
