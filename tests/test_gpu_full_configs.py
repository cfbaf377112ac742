"""Every value of the full benchmark configurations, on the GPU, against the
long-double oracle, and beside it the reference's own double arithmetic
(the oracle's mirror functions, which repeat rastrigin.cpp:62-72 /
rosenbrock.cpp:59-92 / lennard_jones.cpp:72-91 operation by operation):

- rastrigin fitness + gradient, 4096 x 50 (all rows);
- rosenbrock fitness + gradient, 65536 x 1000 (all rows);
- lennard_jones energy + gradient, 16384 clusters of 150 atoms (all rows);
- the 64-island mixed archipelago epoch the benchmark times (45 185 rows),
  fused, in place over the host arrays and staged through pinned buffers.

The bar is |gpu - exact| <= 1e-13 * scale per value, scale being the
first-order error bound of the reference's own evaluation (the sum of the
absolute values of the summed terms), computed in long double. Each test also
prints the plain relative error max |gpu - exact| / |exact| over all values
(fitness, and gradient components with exact != 0), and the same two
figures for the reference's double arithmetic on the same rows (run with -s).
For fitness values the plain relative error is within 1e-13 too; for
gradient components that nearly cancel (rastrigin's 2x against
20*pi*sin(2*pi*x), rosenbrock's chain terms) the plain relative error of any
double evaluation, the reference's included, exceeds it; the scale-relative
bar is the one both meet.
"""
import numpy as np
import pytest

from pagmo2_gb300 import _native as N
from pagmo2_gb300 import archipelago as A
from pagmo2_gb300 import problems as P
from pagmo2_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-13


def errors(got, want, scale):
    """(max error of scale, max plain relative error over nonzero exact values)."""
    got, want, scale = (np.asarray(a, dtype=np.float64).ravel() for a in (got, want, scale))
    of_scale = float(np.max(np.abs(got - want) / np.maximum(scale, np.finfo(float).tiny))) if got.size else 0.0
    nz = want != 0
    rel = float(np.max(np.abs(got[nz] - want[nz]) / np.abs(want[nz]))) if nz.any() else 0.0
    return of_scale, rel


def report(name, f, g, fl, fs, gl, gs, fr=None, gr=None):
    fe = errors(f, fl, fs)
    line = f"{name}: fitness {fe[0]:.2e} of scale, {fe[1]:.2e} relative"
    if fr is not None:
        e = errors(fr, fl, fs)
        line += f" (reference {e[0]:.2e}, {e[1]:.2e})"
    ge = (0.0, 0.0)
    if g is not None:
        ge = errors(g, gl, gs)
        line += f"; gradient {ge[0]:.2e} of scale, {ge[1]:.2e} relative"
        if gr is not None:
            e = errors(gr, gl, gs)
            line += f" (reference {e[0]:.2e}, {e[1]:.2e})"
    print("\nPARITY-FULL " + line)
    return fe, ge


def full_check(ctx, orc, name, kind, param, x, reference_gradient=True):
    udp = P.from_kind(kind, param, ctx)
    f, g = udp.batch_gradient(x)
    fl, fs = orc.batch_fitness_ld(kind, param, x)
    gl, gs = orc.batch_gradient_ld(kind, param, x)
    fr = orc.batch_fitness(kind, param, x)
    gr = orc.batch_gradient(kind, param, x) if reference_gradient else None
    fe, ge = report(name, f, g, fl, fs, gl, gs, fr, gr)
    assert fe[0] <= TOL, (name, "fitness", fe)
    assert fe[1] <= TOL, (name, "fitness, plain relative", fe)
    assert ge[0] <= TOL, (name, "gradient", ge)
    # the fitness-only kernel gives the same values as the fused one
    f_only = udp.batch_fitness(x)
    assert errors(f_only, fl, fs)[0] <= TOL
    return f, g


def test_config1_rastrigin_4096x50_every_value(ctx, orc):
    full_check(ctx, orc, "rastrigin 4096 x 50", N.RASTRIGIN, 50, W.rastrigin_batch())


def test_config2_rosenbrock_65536x1000_every_value(ctx, orc):
    full_check(ctx, orc, "rosenbrock 65536 x 1000", N.ROSENBROCK, 1000, W.rosenbrock_batch())


def test_config3_lennard_jones_16384x150_every_value(ctx, orc):
    # the reference has no lennard_jones gradient: the energy is compared with
    # its double evaluation, the gradient with the long-double oracle only
    full_check(ctx, orc, "lennard_jones 16384 x 150 atoms", N.LENNARD_JONES, 150, W.lj_batch(),
               reference_gradient=False)


@pytest.mark.parametrize("staged", [False, True], ids=["in_place", "staged"])
def test_config5_archipelago_64_islands_every_value(ctx, orc, monkeypatch, staged):
    """The benchmark's epoch: 64 islands (seed 5), every island fitness +
    gradient, every row of every island checked."""
    if staged:
        monkeypatch.setenv("PGX_EPOCH_STAGED", "1")
    else:
        monkeypatch.delenv("PGX_EPOCH_STAGED", raising=False)
    reqs = W.archipelago(64)
    shapes = [(r.kind, r.param, r.n, True) for r in reqs]
    batches = [r.dvs for r in reqs]
    assert sum(r.n for r in reqs) == 45185
    ep = A.Epoch(shapes, ctx)
    try:
        outs = ep.run(batches)
        again = ep.run(batches)
    finally:
        ep.close()
    worst = {}
    for (k, p, n, _), x, (f, g), (f2, g2) in zip(shapes, batches, outs, again):
        assert np.array_equal(f, f2) and np.array_equal(g, g2)  # deterministic
        fl, fs = orc.batch_fitness_ld(k, p, x)
        gl, gs = orc.batch_gradient_ld(k, p, x)
        fe, ge = errors(f, fl, fs), errors(g, gl, gs)
        assert fe[0] <= TOL and fe[1] <= TOL, (k, p, n, fe)
        assert ge[0] <= TOL, (k, p, n, ge)
        w = worst.setdefault(k, [0.0, 0.0, 0.0, 0.0])
        w[:] = [max(w[0], fe[0]), max(w[1], fe[1]), max(w[2], ge[0]), max(w[3], ge[1])]
    names = {N.RASTRIGIN: "rastrigin", N.ROSENBROCK: "rosenbrock", N.LENNARD_JONES: "lennard_jones"}
    for k, w in sorted(worst.items()):
        print(f"\nPARITY-FULL archipelago 64 islands ({'staged' if staged else 'in place'}), {names[k]} islands: "
              f"fitness {w[0]:.2e} of scale, {w[1]:.2e} relative; gradient {w[2]:.2e} of scale, {w[3]:.2e} relative")
