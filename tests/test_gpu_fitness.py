"""GPU parity of batch fitness and gradient (through the C ABI) against the
reference's golden vectors and the long-double oracle.

Tolerance: |gpu - x| <= 1e-13 * scale per value, where scale is the
first-order error bound of the reference's own evaluation (the sum of the
absolute values of the summed terms, plus the rounded squares inside
rosenbrock's t = x_i^2 - x_{i+1}); computed by the oracle in long double.
"""
import math

import numpy as np
import pytest

from pathlib import Path

from pagmo2_gb300 import _native as N
from pagmo2_gb300 import batch_evaluators as B
from pagmo2_gb300 import problems as P
from pagmo2_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
TOL = 1e-13


def eval_gpu(ctx, kind, param, x, grad=True):
    udp = P.from_kind(kind, param, ctx)
    if grad:
        return udp.batch_gradient(x)
    return udp.batch_fitness(x), None


def rel_err(got, want, scale):
    return np.max(np.abs(got - want) / np.maximum(scale, np.finfo(float).tiny)) if got.size else 0.0


def check_against_oracle(orc, ctx, kind, param, x, grad=True):
    f, g = eval_gpu(ctx, kind, param, x, grad)
    fl, fs = orc.batch_fitness_ld(kind, param, x)
    assert rel_err(f, fl, fs) <= TOL, (kind, param, rel_err(f, fl, fs))
    if grad:
        gl, gs = orc.batch_gradient_ld(kind, param, x)
        assert rel_err(g, gl, gs) <= TOL, (kind, param, rel_err(g, gl, gs))
    return f, g


# ------------------------------------------------------------ reference pins

def test_golden_fitness_and_gradient(ctx, orc):
    gold = np.load(GOLD / "fitness.npz")
    names = sorted({k.split("/")[0] for k in gold.files})
    for name in names:
        kind, param = (int(v) for v in gold[f"{name}/kind"])
        x = gold[f"{name}/x"]
        if kind >= N.ACKLEY:  # fitness only, as in the reference
            f, _ = eval_gpu(ctx, kind, param, x, grad=False)
            fl, fs = orc.batch_fitness_ld(kind, param, x)
            assert rel_err(f, gold[f"{name}/f"], fs) <= TOL, (name, rel_err(f, gold[f"{name}/f"], fs))
            continue
        f, g = eval_gpu(ctx, kind, param, x)
        fl, fs = orc.batch_fitness_ld(kind, param, x)
        assert rel_err(f, gold[f"{name}/f"], fs) <= TOL, (name, rel_err(f, gold[f"{name}/f"], fs))
        # the fitness-only kernel agrees with the fused one
        f_only = P.from_kind(kind, param, ctx).batch_fitness(x)
        assert rel_err(f_only, f, fs) <= TOL, name
        if f"{name}/g" in gold.files:
            gl, gs = orc.batch_gradient_ld(kind, param, x)
            assert rel_err(g, gold[f"{name}/g"], gs) <= TOL, (name, rel_err(g, gold[f"{name}/g"], gs))
        else:
            gl, gs = orc.batch_gradient_ld(kind, param, x)
            assert rel_err(g, gl, gs) <= TOL, (name, rel_err(g, gl, gs))


def test_reference_known_answers(ctx):
    # tests/rastrigin.cpp:56-62 (exact), tests/rosenbrock.cpp:70-79, tests/lennard_jones.cpp:59-60
    assert P.rastrigin(1, ctx).fitness([1.0]).tolist() == [1.0]
    assert P.rastrigin(5, ctx).fitness([1.0] * 5).tolist() == [5.0]
    for g in (P.rastrigin(1, ctx).gradient([1.0]), P.rastrigin(5, ctx).gradient([1.0] * 5)):
        assert np.allclose(g, 2.0, rtol=1e-14, atol=0)
    assert P.rosenbrock(2, ctx).fitness([1.0, 1.0]).tolist() == [0.0]
    assert P.rosenbrock(5, ctx).fitness([1.0] * 5).tolist() == [0.0]
    g2 = P.rosenbrock(2, ctx).gradient([0.1, 0.2])
    assert abs(g2[0] + 9.4) < 1e-8 and abs(g2[1] - 38.0) < 1e-8
    g5 = P.rosenbrock(5, ctx).gradient([0.1, 0.2, 0.3, 0.4, 0.5])
    assert np.all(np.abs(g5 - np.array([-9.4, 15.6, 13.4, 6.4, 68.0])) < 1e-8)
    lj = P.lennard_jones(3, ctx)
    assert math.isclose(lj.fitness([1.12, -0.33, 2.34])[0], -1.7633355813175688, rel_tol=1e-15)
    assert math.isclose(lj.fitness([1.23, -1.23, 0.33])[0], -1.833100934753864, rel_tol=1e-15)


# ------------------------------------------------------------ seeded parity

@pytest.mark.parametrize("dim", [1, 2, 3, 7, 8, 9, 16, 17, 31, 33, 48, 49, 50, 64, 255, 257, 1000])
def test_rastrigin_dims(ctx, orc, dim):
    check_against_oracle(orc, ctx, N.RASTRIGIN, dim, W.uniform_batch(N.RASTRIGIN, dim, 97, seed=dim))


@pytest.mark.parametrize("dim", [2, 3, 5, 8, 9, 16, 17, 31, 32, 33, 47, 48, 49, 255, 256, 257, 1000, 1001])
def test_rosenbrock_dims(ctx, orc, dim):
    check_against_oracle(orc, ctx, N.ROSENBROCK, dim, W.uniform_batch(N.ROSENBROCK, dim, 67, seed=dim))


@pytest.mark.parametrize("atoms", [3, 4, 5, 6, 7, 32, 33, 34, 64, 65, 150])
def test_lennard_jones_atoms(ctx, orc, atoms):
    n = 24 if atoms <= 64 else 6
    check_against_oracle(orc, ctx, N.LENNARD_JONES, atoms, W.uniform_batch(N.LENNARD_JONES, atoms, n, seed=atoms))
    check_against_oracle(orc, ctx, N.LENNARD_JONES, atoms, W.lj_lattice_batch(n // 2 + 1, atoms, seed=atoms))


@pytest.mark.parametrize("dim", [3, 7, 20, 33, 50, 1000])
def test_rastrigin_rows_do_not_depend_on_the_batch(ctx, dim):
    """A rastrigin row gives bit-identical fitness and gradient whatever batch
    it is evaluated in: for these dimensions (but 1000) batches of up to 4864
    rows take 8 lanes per row and larger ones 4 (rows of 1 to 262144 here),
    and both sum a row in the same order. The fitness-only kernel gives the
    same fitness too."""
    x = W.uniform_batch(N.RASTRIGIN, dim, 262144 if dim < 1000 else 16384, seed=100 + dim)
    udp = P.rastrigin(dim, ctx)
    f_all, g_all = udp.batch_gradient(x)
    assert np.array_equal(udp.batch_fitness(x), f_all)
    for n in (1, 100, 4096, 4865, 10000, 65536):
        if n > x.shape[0]:
            continue
        f, g = udp.batch_gradient(x[:n])
        assert np.array_equal(f, f_all[:n]), (dim, n)
        assert np.array_equal(g, g_all[:n]), (dim, n)
        assert np.array_equal(udp.batch_fitness(x[:n]), f_all[:n]), (dim, n)


def test_config1_rastrigin_full(ctx, orc):
    x = W.rastrigin_batch()  # 4096 x 50, the reference's CPU-runnable case
    f, g = check_against_oracle(orc, ctx, N.RASTRIGIN, 50, x)
    fr = orc.batch_fitness(N.RASTRIGIN, 50, x)
    assert np.max(np.abs(f - fr) / np.abs(fr)) <= TOL


def test_config2_rosenbrock_sampled_and_properties(ctx, orc):
    x = W.rosenbrock_batch()  # 65536 x 1000
    udp = P.rosenbrock(1000, ctx)
    f, g = udp.batch_gradient(x)
    f_only = udp.batch_fitness(x)
    # size-independent: the fused and fitness-only kernels agree everywhere
    assert np.max(np.abs(f - f_only) / f) <= 1e-14
    assert np.all(np.isfinite(g))
    rows = np.random.RandomState(0).choice(x.shape[0], 96, replace=False)
    fl, fs = orc.batch_fitness_ld(N.ROSENBROCK, 1000, x[rows])
    gl, gs = orc.batch_gradient_ld(N.ROSENBROCK, 1000, x[rows])
    assert rel_err(f[rows], fl, fs) <= TOL and rel_err(g[rows], gl, gs) <= TOL
    # the plain relative error on these inputs is within the bar too
    assert np.max(np.abs(f[rows] - fl) / np.abs(fl)) <= TOL


def test_config3_lj_sampled(ctx, orc):
    x = W.lj_batch(2048, 150)
    udp = P.lennard_jones(150, ctx)
    f, g = udp.batch_gradient(x)
    assert np.max(np.abs(f - udp.batch_fitness(x)) / np.abs(f)) <= 1e-13
    rows = np.arange(0, 2048, 128)
    fl, fs = orc.batch_fitness_ld(N.LENNARD_JONES, 150, x[rows])
    gl, gs = orc.batch_gradient_ld(N.LENNARD_JONES, 150, x[rows])
    assert rel_err(f[rows], fl, fs) <= TOL and rel_err(g[rows], gl, gs) <= TOL


# --------------------------------------------------------- finite differences

def estimate_gradient_h(fun, x, dx=1e-2):
    """6th-order central differences (include/pagmo/utils/gradients_and_hessians.hpp:199-244)."""
    g = np.empty_like(x)
    for j in range(x.size):
        h = max(abs(x[j]), 1.0) * dx
        def at(k):
            y = x.copy()
            y[j] += k * h
            return fun(y)
        m1 = (at(1) - at(-1)) / 2.0
        m2 = (at(2) - at(-2)) / 4.0
        m3 = (at(3) - at(-3)) / 6.0
        g[j] = ((15.0 * m1 - 6.0 * m2) + m3) / (10.0 * h)
    return g


def estimate_gradient(fun, x, dx=1e-8):
    """Central differences (include/pagmo/utils/gradients_and_hessians.hpp:131-155)."""
    g = np.empty_like(x)
    for j in range(x.size):
        h = max(abs(x[j]), 1.0) * dx
        y1 = x.copy()
        y2 = x.copy()
        y1[j] += h
        y2[j] -= h
        g[j] = (fun(y1) - fun(y2)) / (2.0 * h)
    return g


def test_gradients_against_central_differences(ctx, orc):
    # dx = 1e-8: the rounding error of f(x +- h) is ~eps |f| / h, so this is a loose sanity bound
    for kind, param, x in ((N.RASTRIGIN, 6, W.uniform_batch(1, 6, 1, 5)[0]),
                           (N.ROSENBROCK, 6, W.uniform_batch(2, 6, 1, 6)[0]),
                           (N.LENNARD_JONES, 8, W.lj_lattice_batch(1, 8, seed=7)[0])):
        udp = P.from_kind(kind, param, ctx)
        g = udp.gradient(x)
        fd = estimate_gradient(lambda y: orc.batch_fitness_ld(kind, param, y[None, :])[0][0], x)
        f0 = abs(orc.batch_fitness_ld(kind, param, x[None, :])[0][0])
        tol = 1e-5 * max(1.0, np.max(np.abs(g))) + 1e-16 * f0 / 1e-8
        assert np.max(np.abs(g - fd)) <= tol, (kind, np.max(np.abs(g - fd)), tol)


def test_gradients_against_finite_differences(ctx, orc):
    for kind, param, x, dx, tol in ((N.RASTRIGIN, 6, W.uniform_batch(1, 6, 1, 5)[0], 1e-3, 1e-6),
                                    (N.ROSENBROCK, 6, W.uniform_batch(2, 6, 1, 6)[0], 1e-3, 1e-6),
                                    (N.LENNARD_JONES, 8, W.lj_lattice_batch(1, 8, seed=7)[0], 1e-3, 1e-6)):
        udp = P.from_kind(kind, param, ctx)
        g = udp.gradient(x)
        fd = estimate_gradient_h(lambda y: orc.batch_fitness_ld(kind, param, y[None, :])[0][0], x, dx)
        assert np.max(np.abs(g - fd)) <= tol * max(1.0, np.max(np.abs(g))), (kind, np.max(np.abs(g - fd)))


# ------------------------------------------------------------------ edge cases

def test_empty_batch_and_single_row(ctx):
    udp = P.rosenbrock(10, ctx)
    assert udp.batch_fitness(np.empty(0)).shape == (0,)
    f, g = udp.batch_gradient(np.empty((0, 10)))
    assert f.shape == (0,) and g.shape == (0, 10)
    assert udp.batch_fitness(np.ones(10)).tolist() == [0.0]


def test_wrong_sizes_raise(ctx):
    with pytest.raises(ValueError, match="is not an exact multiple of the dimension of the problem, 10"):
        P.rosenbrock(10, ctx).batch_fitness(np.zeros(15))
    with pytest.raises(ValueError):
        P.rastrigin(3, ctx).fitness([1.0, 2.0])


def test_lj_coinciding_atoms_give_inf(ctx, orc):
    x = W.lj_lattice_batch(3, 6, seed=2)
    x[1, 3:6] = 0.0  # atom 3 on top of atom 0
    x[2, 0] = 0.0    # atom 1 on top of atom 0
    f, g = P.lennard_jones(6, ctx).batch_gradient(x)
    assert np.isfinite(f[0]) and f[1] == math.inf and f[2] == math.inf
    assert orc.batch_fitness(N.LENNARD_JONES, 6, x)[1:].tolist() == [math.inf, math.inf]
    assert np.all(np.isnan(g[1, 3:6]))


def test_lj_reciprocal_on_device(ctx):
    """The pair loops' 1/d and 1/d^3 against the exact values (rational
    arithmetic where 1/d differs from the correctly rounded 1.0 / d): in
    2^-100 .. 2^100, the integer fixed-point path, 1/d within 0.5 + 2^-10
    units of the last place (correctly rounded but within 2^-10 units of a
    midpoint) and 1/d^3 within 0.5 + 2^-5 units; outside, the FP64 Newton
    step from the FP64 approximate reciprocal, 1/d within one unit."""
    from fractions import Fraction

    rs = np.random.RandomState(11)
    d = np.ldexp(1.0 + rs.random_sample(1_000_000), rs.randint(-100, 101, 1_000_000))
    edges = np.array([0, 1, 2, (1 << 52) - 1, (1 << 52) - 2, 1 << 51, (1 << 29) - 1, 1 << 29], dtype=np.uint64)
    ex = np.arange(-1021, 1022, dtype=np.int64)  # every binade with a normal reciprocal
    e_bits = ((ex + 1023).astype(np.uint64) << np.uint64(52))[:, None] | edges[None, :]
    d = np.concatenate([d, e_bits.ravel().view(np.float64), np.ldexp(1.0 + rs.random_sample(20000),
                                                                      rs.randint(-1021, 1022, 20000))])
    inv = np.empty_like(d)
    cube = np.empty_like(d)
    N.check(N.lib().pgx_selftest_lj_reciprocal(ctx.handle, d.ctypes.data, d.size, inv.ctypes.data,
                                               cube.ctypes.data))
    fast = (d >= 2.0 ** -100) & (d < 2.0 ** 101)
    bad = np.nonzero(inv != 1.0 / d)[0]
    assert np.count_nonzero(fast[bad]) <= np.count_nonzero(fast) // 10_000
    for i in bad:
        exact = 1 / Fraction(float(d[i]))
        ulp = Fraction(2) ** (math.frexp(float(exact))[1] - 53)
        bound = Fraction(1, 2) + Fraction(1, 1024) if fast[i] else Fraction(1)
        assert abs(Fraction(float(inv[i])) - exact) <= bound * ulp, float(d[i]).hex()
    # the cubes: exactly on a sample of the fast range, and every edge mantissa
    idx = np.concatenate([np.arange(0, 1_000_000, 97), np.nonzero(fast)[0][1_000_000:]])
    for i in idx:
        exact = 1 / Fraction(float(d[i])) ** 3
        ulp = Fraction(2) ** (math.frexp(float(exact))[1] - 53)
        assert abs(Fraction(float(cube[i])) - exact) <= (Fraction(1, 2) + Fraction(1, 32)) * ulp, float(d[i]).hex()


def test_integer_paths_at_their_range_edges(ctx, orc):
    """Inputs on both sides of the ranges the integer fixed-point paths take
    (rastrigin/ackley trig for 2^-60 <= |x| < 2^40, the Lennard-Jones pair for
    2^-100 <= r^2 < 2^101, the sums of squares over the whole double range),
    against the long-double oracle: the fallbacks and the fixed-point code
    agree with it alike."""
    rs = np.random.RandomState(21)
    # rastrigin / ackley: tiny, huge, exact multiples of 1/4 and 1/2 near 2^40, zeros
    vals = np.array([1e-70, -3e-25, 1e-17, 2.0 ** -60, -(2.0 ** -61), 0.0, -0.0, 0.25, -0.75, 1.5,
                     2.0 ** 40 - 0.5, -(2.0 ** 40) + 0.25, 2.0 ** 40, 1e13, -7.3e12, 123456.125])
    x = rs.choice(vals, size=(64, 9))
    x[:8] = rs.uniform(-5.12, 5.12, (8, 9))
    check_against_oracle(orc, ctx, N.RASTRIGIN, 9, x)
    check_against_oracle(orc, ctx, N.ACKLEY, 9, x, grad=False)
    # rosenbrock: squares far above and below 1 (no overflow to inf)
    x = rs.uniform(-5.0, 10.0, (32, 12))
    x[::2, ::3] *= 1e60
    x[1::2, 1::3] *= 1e-150
    check_against_oracle(orc, ctx, N.ROSENBROCK, 12, x)
    # lennard_jones, 6 atoms: clusters scaled so that some or all r^2 leave [2^-100, 2^101)
    base = W.lj_lattice_batch(8, 6, seed=4)
    rows = []
    for scale in (1e-20, 1e-14, 1.0, 1e14, 1e16, 1e30):
        rows.append(base * scale)
    mixed = base.copy()
    mixed[:, 3:6] *= 1e17  # atom 3 far out: its pairs on the slow path, the others not
    rows.append(mixed)
    x = np.concatenate(rows)
    check_against_oracle(orc, ctx, N.LENNARD_JONES, 6, x)


def test_nonfinite_inputs_propagate(ctx, orc):
    for kind, param in ((N.RASTRIGIN, 9), (N.ROSENBROCK, 9), (N.LENNARD_JONES, 5)):
        nx = N.problem_nx(kind, param)
        x = W.uniform_batch(kind, param, 3, seed=1)
        x[0, 2] = math.nan
        x[1, 1] = math.inf
        f = P.from_kind(kind, param, ctx).batch_fitness(x)
        fr = orc.batch_fitness(kind, param, x)
        for a, b in zip(f, fr):
            assert (math.isnan(a) and math.isnan(b)) or a == b or abs(a - b) <= 1e-13 * abs(b), (kind, a, b)


def test_device_entry_point_matches_host(ctx):
    torch = pytest.importorskip("torch")
    x = W.rosenbrock_batch(512, 300)
    udp = P.rosenbrock(300, ctx)
    f, g = udp.batch_gradient(x)
    dx = torch.from_numpy(x).cuda()
    df = torch.empty(512, dtype=torch.float64, device="cuda")
    dg = torch.empty((512, 300), dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    N.check(N.lib().pgx_batch_eval_device(ctx.handle, N.ROSENBROCK, 300, dx.data_ptr(), 512, df.data_ptr(),
                                          dg.data_ptr(), s))
    torch.cuda.synchronize()
    assert np.array_equal(df.cpu().numpy(), f) and np.array_equal(dg.cpu().numpy(), g)


# ------------------------------------------------------- bfe contract / fevals

def test_bfe_fevals_and_equality_with_per_call(ctx):
    # tests/thread_bfe.cpp:57-95: bfe output equals per-call fitness; fevals counted once
    prob = B.problem(P.rosenbrock(2, ctx))
    dvs = np.random.RandomState(5).uniform(-1, 1, 10000)
    fvs = B.bfe()(prob, dvs)
    assert prob.get_fevals() == 5000
    for i in range(0, 10000, 997 * 2):
        assert fvs[i // 2] == P.rosenbrock(2, ctx).fitness(dvs[i:i + 2])[0]


def test_gpu_bfe_rejects_unknown_problems(ctx):
    class other:
        def get_name(self):
            return "other"

    with pytest.raises(ValueError, match="Cannot use a gpu_bfe on the problem 'other'"):
        B.gpu_bfe()(other(), np.zeros(4))


# ------------------------------ opt-in: rosenbrock on the FP32 pipe (double-float)

def mixed_range_rows(rng, n, nx):
    """Rows where some 128-element chunks hold values outside the double-float
    range (|x| >= 2^20, 0 < |x| < 2^-60), zeros, signed zeros and the optimum."""
    x = rng.uniform(-5, 10, (n, nx))
    x[0] = 1.0                                  # the optimum: f = 0, g = 0 exactly
    x[1, 5] = 3.0e6                             # above 2^20: that chunk on the FP64 path
    x[2, min(300, nx - 1)] = 1e-30              # below 2^-60
    x[3, ::7] = 0.0
    x[4, ::5] = -0.0
    x[5, 126] = 2.0 ** 20                       # first value out of range
    x[5, 127] = 2.0 ** 20 - 1.0                 # largest in range
    x[6, nx // 2:nx // 2 + 60] = rng.uniform(-1e-12, 1e-12, 60)
    x[7] = 1.0 + rng.integers(-3, 4, nx) * 2.0 ** -52  # one ulp from the optimum
    x[8, -1] = 1e8                              # the last chunk alone out of range
    x[9, 0] = -7e5                              # in range (< 2^20)
    x[10, 127] = 1e60                           # chunk boundary: the carried t (~1e120) is out of range
    x[11, 127] = -3e7                           # chunk boundary, moderately out of range
    return x


@pytest.fixture
def double_float(monkeypatch):
    """Opt in to the double-float rosenbrock rows for one test."""
    monkeypatch.setenv("PGX_ROSENBROCK_DOUBLE_FLOAT", "1")


def test_rosenbrock_double_float_ranges(ctx, orc, double_float):
    rng = np.random.default_rng(31)
    for nx in (128, 1000, 1024, 4096):
        x = mixed_range_rows(rng, 16, nx)
        f, g = check_against_oracle(orc, ctx, N.ROSENBROCK, nx, x)
        assert f[0] == 0.0 and np.all(g[0] == 0.0)


def test_rosenbrock_double_float_matches_fp64_rows(ctx, orc, monkeypatch):
    x = W.rosenbrock_batch(256, 1000, seed=33)
    f64, g64 = P.rosenbrock(1000, ctx).batch_gradient(x)  # default: FP64 arithmetic
    monkeypatch.setenv("PGX_ROSENBROCK_DOUBLE_FLOAT", "1")
    f, g = P.rosenbrock(1000, ctx).batch_gradient(x)
    fl, fs = orc.batch_fitness_ld(N.ROSENBROCK, 1000, x)
    gl, gs = orc.batch_gradient_ld(N.ROSENBROCK, 1000, x)
    for a, b in ((f, fl), (f64, fl)):
        assert rel_err(a, b, fs) <= TOL
    for a, b in ((g, gl), (g64, gl)):
        assert rel_err(a, b, gs) <= TOL
    # the all-FP64 rows are close to rounding level
    assert rel_err(f64, fl, fs) <= 1e-15 and rel_err(g64, gl, gs) <= 1e-15


def test_rosenbrock_double_float_nonfinite(ctx, orc, double_float):
    x = W.rosenbrock_batch(4, 256, seed=34)
    x[0, 10] = math.nan
    x[1, 200] = math.inf
    x[2, 0] = -math.inf
    f = P.rosenbrock(256, ctx).batch_fitness(x)
    fr = orc.batch_fitness(N.ROSENBROCK, 256, x)
    for a, b in zip(f, fr):
        assert (math.isnan(a) and math.isnan(b)) or a == b or abs(a - b) <= 1e-13 * abs(b), (a, b)


# ------------------------------------------------- ackley, griewank, schwefel (fitness only)

FITNESS_ONLY = [(N.ACKLEY, "ackley"), (N.GRIEWANK, "griewank"), (N.SCHWEFEL, "schwefel")]


@pytest.mark.parametrize("kind,name", FITNESS_ONLY)
@pytest.mark.parametrize("dim", [1, 2, 3, 7, 31, 32, 33, 50, 255, 1000, 4096])
def test_fitness_only_problems_dims(ctx, orc, kind, name, dim):
    check_against_oracle(orc, ctx, kind, dim, W.uniform_batch(kind, dim, 37, seed=dim + 10 * kind), grad=False)


def test_fitness_only_known_answers(ctx):
    # tests/ackley.cpp:53-57, tests/griewank.cpp:52-56, tests/schwefel.cpp:52-56
    x1, x3 = [1.12], [-23.45, 12.34, 111.12]
    for cls, k1, k3 in ((P.ackley, 4.659037611351948, 21.941495638130885),
                        (P.griewank, 0.5646311537232878, 4.241511427781268),
                        (P.schwefel, 418.0067810680098, 1338.0260195323838)):
        assert math.isclose(cls(1, ctx).fitness(x1)[0], k1, rel_tol=1e-13)
        assert math.isclose(cls(3, ctx).fitness(x3)[0], k3, rel_tol=1e-13)


def test_fitness_only_problems_have_no_gradient(ctx):
    for cls in (P.ackley, P.griewank, P.schwefel):
        udp = cls(4, ctx)
        with pytest.raises(NotImplementedError):
            udp.gradient([0.1, 0.2, 0.3, 0.4])
        # the C ABI refuses too
        x = np.zeros(4)
        g = np.empty(4)
        st = N.lib().pgx_batch_gradient(ctx.handle, udp.kind, 4, N.ptr(x), 1, None, N.ptr(g))
        assert st == N.ERR_NOTIMPL


def test_fitness_only_problems_bounds_and_errors(ctx, orc):
    for kind, name in FITNESS_ONLY:
        lb, ub = N.problem_bounds(kind, 5)
        wl, wu = W.bounds(kind, 5)
        assert np.array_equal(lb, wl) and np.array_equal(ub, wu)
        with pytest.raises(ValueError, match="minimum 1 dimension"):
            P.from_kind(kind, 0, ctx)


def test_fitness_only_nonfinite_and_gpu_bfe(ctx, orc):
    for kind, name in FITNESS_ONLY:
        x = W.uniform_batch(kind, 9, 4, seed=kind)
        x[0, 2] = math.nan
        x[1, 1] = math.inf
        f = B.gpu_bfe()(B.problem(P.from_kind(kind, 9, ctx)), x.ravel())
        fr = orc.batch_fitness(kind, 9, x)
        for a, b in zip(f, fr):
            assert (math.isnan(a) and math.isnan(b)) or a == b or abs(a - b) <= 1e-12 * (1 + abs(b)), (name, a, b)


def test_translate_forwards_the_batch(ctx, orc):
    """translate{udp, t} (src/problems/translate.cpp:118-146): the batch shifted back and evaluated by the inner
    GPU UDP in one pass, through batch_fitness and through gpu_bfe."""
    rng = np.random.RandomState(8)
    for udp, kind, param in ((P.rosenbrock(50, ctx), N.ROSENBROCK, 50), (P.zdt(1, 30, ctx), None, None)):
        t = rng.uniform(-1, 1, udp.get_nx())
        tr = P.translate(udp, t)
        lb, ub = tr.get_bounds()
        assert np.array_equal(lb, udp.get_bounds()[0] + t)
        x = rng.uniform(0, 1, (300, udp.get_nx())) * (ub - lb) + lb
        f = tr.batch_fitness(x)
        assert np.array_equal(f, udp.batch_fitness(x - t))
        assert np.array_equal(B.gpu_bfe()(tr, x.ravel()), f)
    with pytest.raises(ValueError, match="Length of shift vector is: 3 while the problem dimension is: 50"):
        P.translate(P.rosenbrock(50, ctx), [1.0, 2.0, 3.0])
