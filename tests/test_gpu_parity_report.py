"""Per-problem error report against the long-double oracle (the parity bar is
1e-13 of the first-order error bound `scale`; the plain relative error is
reported beside it), with the same figures for the reference's own double
arithmetic (the oracle's mirror functions) on the same rows: near a zero of a
gradient component both lose relative accuracy alike. Benchmark-shaped
batches; prints one line per problem (run with -s to see them) and asserts
the bar."""
import numpy as np
import pytest

from pagmo2_gb300 import _native as N
from pagmo2_gb300 import problems as P
from pagmo2_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-13

CASES = [  # (name, kind, param, rows, gradient)
    ("rastrigin 50", N.RASTRIGIN, 50, 4096, True),
    ("rosenbrock 1000", N.ROSENBROCK, 1000, 2048, True),
    ("lennard_jones 150 atoms", N.LENNARD_JONES, 150, 256, True),
    ("lennard_jones 20 atoms", N.LENNARD_JONES, 20, 2048, True),
    ("ackley 50", N.ACKLEY, 50, 4096, False),
    ("griewank 50", N.GRIEWANK, 50, 4096, False),
    ("schwefel 50", N.SCHWEFEL, 50, 4096, False),
]


def errors(got, want, scale):
    rel_scale = float(np.max(np.abs(got - want) / np.maximum(scale, np.finfo(float).tiny)))
    nz = np.abs(want) > 0
    rel = float(np.max(np.abs(got[nz] - want[nz]) / np.abs(want[nz]))) if nz.any() else 0.0
    return rel_scale, rel


@pytest.mark.parametrize("name,kind,param,rows,grad", CASES)
def test_error_report(ctx, orc, name, kind, param, rows, grad):
    x = W.uniform_batch(kind, param, rows, seed=31)
    udp = P.from_kind(kind, param, ctx)
    if grad:
        f, g = udp.batch_gradient(x)
    else:
        f, g = udp.batch_fitness(x), None
    fl, fs = orc.batch_fitness_ld(kind, param, x)
    fe = errors(f, fl, fs)
    fr = errors(orc.batch_fitness(kind, param, x), fl, fs)
    line = f"{name}: fitness {fe[0]:.2e} of scale, {fe[1]:.2e} relative (reference {fr[0]:.2e}, {fr[1]:.2e})"
    assert fe[0] <= TOL
    if grad:
        gl, gs = orc.batch_gradient_ld(kind, param, x)
        ge = errors(g.ravel(), gl.ravel(), gs.ravel())
        line += f"; gradient {ge[0]:.2e} of scale, {ge[1]:.2e} relative"
        if kind == N.LENNARD_JONES:
            line += " (no reference gradient)"
        else:
            gr = errors(orc.batch_gradient(kind, param, x).ravel(), gl.ravel(), gs.ravel())
            line += f" (reference {gr[0]:.2e}, {gr[1]:.2e})"
        assert ge[0] <= TOL
    print("\nPARITY " + line)
