"""GPU hypervolume (pgx_hypervolume and the queries).

2 and 3 objectives: against the long-double oracle within 1e-13 relative (all slabs are non-negative, so the
bound is relative to the volume itself), against the reference's own values (tests/golden/hv.npz, within 1e-12
relative: the reference's hv3d sweep subtracts), the known answers of tests/hypervolume.cpp:229-297, and the
reference's checks and messages.

4 to 16 objectives (hvwfg) and every point's contribution (hvwfg's limit sets): bit for bit against the WFG
oracle (itself pinned bit for bit to the compiled reference) and, where it is built, the reference; the known
contributions of tests/hypervolume.cpp:322-460; the reference's test cases (hypervolume_test_data). For 2 and
3 objectives the reference's contributions come from hv3d's HyCon3D box sums unless a point is dominated: the
GPU's values equal the oracle's hvwfg restatement bit for bit and the reference's within 1e-12 of the point's
own box volume."""
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
    with pytest.raises(NotImplementedError, match="at most 16 objectives"):
        MO.hypervolume(np.zeros((2, 17)), context=ctx).compute(np.ones(17))
    with pytest.raises(ValueError, match="Index of the individual is out of bounds."):
        h.exclusive(3, [4, 4])
    with pytest.raises(ValueError, match="Reference point is invalid"):
        h.contributions([3, 1])
    with pytest.raises(ValueError, match="Reference point is invalid"):
        h.least_contributor([1.5, 1.5])


from test_oracle_hypervolume import KNOWN_CONTRIBUTIONS, lift2, read_typed, test_data_path, wfg_sets  # noqa: E402


def test_wfg_volume_bit_exact(ctx, orc):
    rng = np.random.default_rng(29)
    for label, p, r in wfg_sets(rng):
        if p.shape[1] < 4:
            continue
        assert hv(p, r, ctx) == orc.hvwfg(p, r), label


def test_wfg_volume_against_reference(ctx, ref):
    rng = np.random.default_rng(31)
    for label, p, r in wfg_sets(rng):
        if p.shape[1] >= 4:
            assert hv(p, r, ctx) == ref.hypervolume(p, r), label


def test_wfg_known_volumes(ctx):
    # tests/hypervolume.cpp:245-309
    assert hv([[1, 1, 1, 1], [2, 2, 2, 2]], [3, 3, 3, 3], ctx) == 16.0
    assert hv([[1, 1, 1, 3], [2, 2, 2, 3]], [3, 3, 3, 3], ctx) == 0.0
    assert hv([[1, 1, 1, 1], [1, 1, 1, 1]], [2, 2, 2, 2], ctx) == 1.0
    assert hv([[1, 1, 1, 1], [1, 1, 1, 1], [0, 0, 0, 0]], [2, 2, 2, 2], ctx) == 16.0
    assert hv([[2.3, 4.5, 3.2, 1.9, 6.0], [3.4, 3.4, 3.4, 2.1, 5.8], [6.0, 1.2, 3.6, 3.0, 6.0]],
              [7, 7, 7, 7, 7], ctx) == 373.21228


def oracle_contributions(orc, p, r):
    if len(p) == 1:
        return np.array([abs(np.prod(p[0] - r))])
    if p.shape[1] == 2:
        return orc.hvwfg_contributions(*lift2(p, r))
    return orc.hvwfg_contributions(p, r)


def test_contributions_bit_exact(ctx, orc):
    rng = np.random.default_rng(37)
    for label, p, r in wfg_sets(rng):
        h = MO.hypervolume(p, context=ctx)
        c = h.contributions(r)
        assert np.array_equal(c, oracle_contributions(orc, p, r)), label
        assert h.least_contributor(r) == int(np.argmin(c)), label
        assert h.greatest_contributor(r) == int(np.argmax(c)), label


def test_contributions_against_reference(ctx, ref):
    rng = np.random.default_rng(41)
    worst = 0.0
    for label, p, r in wfg_sets(rng):
        c = MO.hypervolume(p, context=ctx).contributions(r)
        want = ref.hv_contributions(p, r)
        if p.shape[1] >= 4 or len(p) == 1:
            assert np.array_equal(c, want), label
        else:  # hv3d's box sums: within 1e-12 of the point's own box volume
            box = np.abs(np.prod(r - p, axis=1))
            dev = np.abs(c - want) / np.maximum(box, 1e-300)
            worst = max(worst, float(dev.max()))
            assert np.all(dev <= 1e-12), (label, dev.max())
    print(f"\nCONTRIBUTIONS 2/3 objectives vs hv3d: max |c - c_ref| / box volume = {worst:.2e}")


def test_known_contributions_and_exclusive(ctx):
    for p, r, want in KNOWN_CONTRIBUTIONS:
        h = MO.hypervolume(p, context=ctx)
        want = [float(x) for x in want]
        assert list(h.contributions(r)) == want, p
        for i in range(len(p)):
            assert h.exclusive(i, r) == want[i], (p, i)


def test_reference_test_cases(ctx, orc):
    for name in ("c_max_t1_d5_n1024", "c_max_t1_d7_n64"):
        for p, r, want in read_typed(test_data_path(name), "compute"):
            got = hv(p, r, ctx)
            assert got == orc.hvwfg(p, r), name
            if name == "c_max_t1_d5_n1024":
                assert abs(got - want) < 1e-3  # testcases_list.txt's tolerance
    for name in ("e_max_d2", "e_max_d3", "e_max_d5"):
        for p, r, (i, want) in read_typed(test_data_path(name), "exclusive"):
            assert abs(MO.hypervolume(p, context=ctx).exclusive(i, r) - want) < 1e-8, name
    for name in ("lc_max_d2", "lc_max_d3"):
        for p, r, want in read_typed(test_data_path(name), "least"):
            assert MO.hypervolume(p, context=ctx).least_contributor(r) == want, name


def test_exclusive_against_reference(ctx, ref):
    rng = np.random.default_rng(43)
    for label, p, r in wfg_sets(rng):
        if len(p) > 5:
            continue
        h = MO.hypervolume(p, context=ctx)
        for i in range(len(p)):
            got, want = h.exclusive(i, r), ref.hv_exclusive(p, r, i)
            if p.shape[1] >= 4:
                assert got == want, (label, i)
            else:
                assert abs(got - want) <= 1e-12 * ref.hypervolume(p, r), (label, i)


@pytest.mark.parametrize("n,m", [(3000, 4), (2000, 5), (300, 7), (32, 12), (24, 16)])
def test_wfg_larger_fronts(ctx, orc, n, m):
    rng = np.random.default_rng(n + m)
    w = rng.random((n, m)) ** 2
    p = w / np.linalg.norm(w, axis=1, keepdims=True)  # a spherical front: most points non-dominated
    r = np.full(m, 1.1)
    assert hv(p, r, ctx) == orc.hvwfg(p, r)
    if n <= 2000:
        c = MO.hypervolume(p, context=ctx).contributions(r)
        assert np.array_equal(c, orc.hvwfg_contributions(p, r))


def test_contributions_device_entry(ctx, orc):
    import torch
    p = np.random.default_rng(5).random((50, 4))
    r = np.full(4, 1.1)
    dp = torch.from_numpy(p).cuda()
    dout = torch.empty(50, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    N.check(N.lib().pgx_hypervolume_contributions_device(ctx.handle, dp.data_ptr(), 50, 4, N.ptr(r),
                                                         dout.data_ptr(), torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert np.array_equal(dout.cpu().numpy(), orc.hvwfg_contributions(p, r))
