"""GPU parity of the ZDT and DTLZ batch fitness and p_distance (through the C ABI).

Tolerance: |gpu - x| <= 1e-13 * scale + 1e-300 per value, where x and scale
are the long-double oracle's value and first-order error scale
(oracle/mo_problems.cpp; the oracle is pinned to the reference by
tests/test_oracle_mo_problems.py). The 1e-300 absolute floor covers results
that underflow into the subnormal range (DTLZ4's x^100). ZDT5 counts bits:
its values are compared bit for bit. Known answers: tests/zdt.cpp and
tests/dtlz.cpp with the tolerances stated there.
"""
import math
from pathlib import Path

import numpy as np
import pytest

from pagmo2_gb300 import _native as N
from pagmo2_gb300 import problems as P
from pagmo2_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ZDT, DTLZ = N.ZDT, N.DTLZ
TOL, ATOL = 1e-13, 1e-300
GOLD = Path(__file__).resolve().parent / "golden" / "mo_problems.npz"


def udp_of(spec, ctx):
    kind, pid, param = spec[:3]
    if kind == ZDT:
        return P.zdt(pid, param, context=ctx)
    return P.dtlz(pid, param, spec[3], spec[4], context=ctx)


def check_against_oracle(orc, spec, x, got, label=""):
    want, sc = orc.mo_fitness_ld(spec, x)
    got = got.reshape(want.shape)
    if spec[0] == ZDT and spec[1] == 5:
        assert np.array_equal(got, orc.mo_fitness(spec, x)), (spec, label)
        return
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan), (spec, label)
    err = np.abs(got - want)[~nan]
    lim = (TOL * sc + ATOL)[~nan]
    bad = err > lim
    assert not bad.any(), (spec, label, err[bad][:4], lim[bad][:4])


def test_golden_fixtures(ctx, orc):
    gold = np.load(GOLD)
    names = sorted({k.split("/")[0] for k in gold.files})
    for name in names:
        spec = tuple(int(v) for v in gold[f"{name}/spec"])
        x = gold[f"{name}/x"]
        udp = udp_of(spec, ctx)
        f = udp.batch_fitness(x).reshape(x.shape[0], -1)
        check_against_oracle(orc, spec, x, f, name)
        # and against the reference's own values, with the same scale
        _, sc = orc.mo_fitness_ld(spec, x)
        ref_f = gold[f"{name}/f"]
        assert np.all(np.abs(f - ref_f) <= TOL * sc + ATOL), name
        pd = udp.batch_p_distance(x)
        pl, ps = orc.mo_p_distance(spec, x, ld=True)
        assert np.all(np.abs(pd - pl) <= TOL * ps + ATOL), name
        assert np.all(np.abs(pd - gold[f"{name}/p_distance"]) <= TOL * ps + ATOL), name


def close(a, b, rel):
    d = abs(a - b)
    return d == 0 or (d <= rel * abs(a) and d <= rel * abs(b))


def test_known_answers(ctx):
    # tests/zdt.cpp:68-178
    cases = [((1, 30), 0.25, (0.25, 2.3486121811340026)), ((1, 13), 0.33, (0.33, 2.825404001404863)),
             ((2, 30), 0.25, (0.25, 3.230769230769231)), ((2, 13), 0.33, (0.33, 3.9425692695214107)),
             ((3, 30), 0.25, (0.25, 2.0986121811340026)), ((3, 13), 0.33, (0.33, 3.092379609548596)),
             ((4, 30), 0.25, (0.25, 570.7417450526075)), ((4, 13), 0.33, (0.33, 178.75872382132619)),
             ((6, 30), 0.25, (0.6321205588285577, 7.309699961231513)),
             ((6, 13), 0.33, (0.999999983628226, 7.693505388431892))]
    for (pid, param), v, want in cases:
        got = P.zdt(pid, param, ctx).fitness(np.full(param, v))
        assert all(close(a, b, 1e-15) for a, b in zip(got, want)), (pid, param, got)
    x = np.ones(175)
    x[100:] = 0.0
    assert P.zdt(5, 30, ctx).fitness(x).tolist() == [31.0, 1.4193548387096775]
    x = np.full(90, 1.34677824)
    x[45:] = 0.345345
    assert P.zdt(5, 13, ctx).fitness(x).tolist() == [31.0, 0.6774193548387096]
    # tests/dtlz.cpp:60-196 (1e-12 %)
    dv1, dv2 = [0.5] * 5, [0.1, 0.2, 0.3, 0.4, 0.5]
    kats = {2: ([0.5000000000000001, 0.5, 0.7071067811865475], [0.9863148040113404, 0.3204731065093832,
                                                               0.16425618829224242]),
            4: ([1.0, 1.2391398122732624e-30, 1.2391398122732624e-30],
                [1.05, 2.090781951822753e-70, 1.6493361431346507e-100]),
            7: ([0.5, 0.5, 19.5], [0.1, 0.2, 16.228886997303473])}
    for pid, (f1, f2) in kats.items():
        udp = P.dtlz(pid, 5, 3, context=ctx)
        for dv, want in ((dv1, f1), (dv2, f2)):
            got = udp.fitness(dv)
            assert all(close(a, b, 1e-14) for a, b in zip(got, want)), (pid, got, want)
    # p_distance (tests/zdt.cpp:180-197, tests/dtlz.cpp:198-212)
    x = np.full(30, 0.143)
    xi = np.ones(175)
    xi[100:] = 0.0
    for (pid, param), v, want in (((1, 30), x, 1.2869999999999997), ((3, 30), x, 1.2869999999999997),
                                  ((4, 10), x, 355.63154167532053), ((6, 10), x, 5.534476131480399),
                                  ((5, 11), xi, 15.0)):
        assert close(P.zdt(pid, param, ctx).p_distance(v), want, 1e-15), (pid, param)
    res = [288.09711053693565, 0.14472200000000002, 288.09711053693565, 0.14472200000000002, 0.14472200000000002,
           1.7273931523406256, 2.0790000000000002]
    for pid in range(1, 8):
        assert close(P.dtlz(pid, 4, context=ctx).p_distance(np.full(4, 0.231)), res[pid - 1], 1e-14), pid
    with pytest.raises(ValueError, match="The size of the decision vector should be 4 while 3 was detected"):
        P.dtlz(3, 4, context=ctx).p_distance(np.full(3, 0.231))


def sweep_specs():
    for pid in (1, 2, 3, 4, 6):
        for param in (2, 3, 30, 100, 1000):
            yield (ZDT, pid, param, 0, 0)
    for param in (2, 11, 30, 200):
        yield (ZDT, 5, param, 0, 0)
    for pid in range(1, 8):
        for dim, fdim in ((3, 2), (5, 3), (12, 3), (50, 40), (293, 70), (100, 3), (1000, 5)):
            yield (DTLZ, pid, dim, fdim, 100 if pid != 4 else (3 if dim > 100 else 100))


@pytest.mark.parametrize("spec", list(sweep_specs()), ids=lambda s: "_".join(map(str, s)))
def test_shapes_against_long_double(ctx, orc, spec):
    lb, ub = W.mo_bounds(spec[0], spec[1], spec[2], spec[3])
    n = 257 if lb.size <= 300 else 33
    x = W.mo_uniform_batch(spec[0], spec[1], spec[2], n, seed=spec[1] * 1000 + spec[2], fdim=spec[3])
    x[0] = lb
    x[1] = ub
    udp = udp_of(spec, ctx)
    check_against_oracle(orc, spec, x, udp.batch_fitness(x))
    pd = udp.batch_p_distance(x)
    pl, ps = orc.mo_p_distance(spec, x, ld=True)
    if spec[0] == ZDT and spec[1] == 5:
        assert np.array_equal(pd, orc.mo_p_distance(spec, x))
    else:
        assert np.all(np.abs(pd - pl) <= TOL * ps + ATOL), spec


def test_large_batch_properties(ctx, orc):
    """1 M rows of ZDT1 30 (the NSGA-II benchmark shape): a sampled slice against
    the oracle, and the front property f1 = g (1 - sqrt(f0 / g)) exactly where g = 1."""
    udp = P.zdt(1, 30, ctx)
    x = W.mo_uniform_batch(ZDT, 1, 30, 1 << 20, seed=77)
    x[::1000, 1:] = 0.0  # on the Pareto front: g = 1
    f = udp.batch_fitness(x).reshape(-1, 2)
    idx = np.random.RandomState(5).choice(x.shape[0], 4096, replace=False)
    check_against_oracle(orc, (ZDT, 1, 30, 0, 0), x[idx], f[idx])
    front = f[::1000]
    assert np.array_equal(front[:, 0], x[::1000, 0])
    assert np.array_equal(front[:, 1], 1.0 - np.sqrt(x[::1000, 0]))


def test_nonfinite_inputs(ctx, orc):
    rng = np.random.RandomState(31)
    for spec in ((ZDT, 1, 30, 0, 0), (ZDT, 3, 30, 0, 0), (ZDT, 4, 10, 0, 0), (ZDT, 5, 11, 0, 0), (ZDT, 6, 10, 0, 0),
                 (DTLZ, 1, 12, 3, 100), (DTLZ, 2, 12, 3, 100), (DTLZ, 4, 12, 3, 100), (DTLZ, 6, 12, 3, 100),
                 (DTLZ, 7, 12, 3, 100)):
        lb, ub = W.mo_bounds(spec[0], spec[1], spec[2], spec[3])
        x = W.mo_uniform_batch(spec[0], spec[1], spec[2], 64, seed=3, fdim=spec[3])
        for v in (math.nan, math.inf, -math.inf, -0.0, 1e300, -1e-310):
            x[rng.randint(0, 64, 4), rng.randint(0, lb.size, 4)] = v
        got = udp_of(spec, ctx).batch_fitness(x).reshape(64, -1)
        want = orc.mo_fitness(spec, x)
        assert np.array_equal(np.isnan(got), np.isnan(want)), spec
        inf = np.isinf(want)
        assert np.array_equal(got[inf], want[inf]), spec
        fin = np.isfinite(want)
        _, sc = orc.mo_fitness_ld(spec, x)
        ok = np.abs(got[fin] - want[fin]) <= TOL * np.nan_to_num(sc[fin], nan=np.inf) + ATOL
        assert ok.all(), spec


def test_empty_and_invalid(ctx):
    udp = P.zdt(1, 30, ctx)
    assert udp.batch_fitness(np.zeros(0)).size == 0
    with pytest.raises(ValueError, match="not an exact multiple"):
        udp.batch_fitness(np.zeros(31))
    with pytest.raises(ValueError, match="prob_id=7 was detected"):
        P.zdt(7, 23, ctx)
    with pytest.raises(ValueError, match="has to be larger than the number of objectives"):
        P.dtlz(1, 3, 3, context=ctx)
    assert P.zdt(5, 11, ctx).get_nix() == 80 and P.zdt(1, 30, ctx).get_nix() == 0


def test_device_entry_point_and_survival_chain(ctx, orc):
    """pgx_mo_batch_fitness_device writes n x nobj objective rows that
    pgx_nsga2_survival_device consumes directly (NSGA-II's evaluate-then-survive
    step without a host round trip)."""
    import ctypes as C

    import torch

    from pagmo2_gb300 import multi_objective as MO

    L = N.lib()
    spec = N.mo_problem(DTLZ, 2, 12, 3, 100)
    x = W.mo_uniform_batch(DTLZ, 2, 12, 3000, seed=9, fdim=3)
    dx = torch.from_numpy(x).cuda()
    df = torch.empty((3000, 3), dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    N.check(L.pgx_mo_batch_fitness_device(ctx.handle, C.byref(spec), dx.data_ptr(), 3000, df.data_ptr(), s))
    torch.cuda.synchronize()
    host = P.dtlz(2, 12, 3, context=ctx).batch_fitness(x).reshape(3000, 3)
    f = df.cpu().numpy()
    assert np.array_equal(f, host)
    rank, dc, off, idx, cd = MO.nsga2_survival(f, ctx)
    want = orc.fnds(f, dom_list=False)
    assert np.array_equal(off, want["front_offsets"]) and np.array_equal(idx, want["front_indices"])


def test_gpu_bfe_and_population_p_distance(ctx):
    from pagmo2_gb300 import batch_evaluators as B

    udp = P.zdt(2, 30, ctx)
    prob = B.problem(udp)
    x = W.mo_uniform_batch(ZDT, 2, 30, 100, seed=4)
    f = B.bfe()(prob, x.ravel())
    assert prob.get_fevals() == 100 and f.size == 200
    assert np.array_equal(f, udp.batch_fitness(x))

    class pop:
        def get_x(self):
            return x

    per_row = udp.batch_p_distance(x)
    c = 0.0
    for v in per_row:
        c += v
    assert udp.p_distance(pop()) == c / 100
