"""Batched gradient-based refinement (pgx_refine_batch, pagmo2_gb300.algorithms
.gpu_mbh): monotonic basin hopping per individual (the scheme of
src/algorithms/mbh.cpp:102-200) with projected-gradient descent, every
individual at once on the GPU.

- The GPU loop equals its host restatement (oracle/refine.py) bit for bit when
  the restatement is fed the GPU's own fitness and gradient of each point.
- Fed the reference's problem::fitness and problem::gradient instead (the
  long-double oracle's gradient for lennard_jones, which has none in the
  reference), the same loop ends at the same points up to the last bits of
  the evaluations.
- On large batches: fitness never rises, points stay in the bounds, the
  returned fitness is the batch fitness of the returned points, and the
  evaluation count is within its bounds.
"""
import numpy as np
import pytest

from oracle import refine as R
from pagmo2_gb300 import _native as N
from pagmo2_gb300 import problems as P
from pagmo2_gb300 import workloads as W
from pagmo2_gb300.algorithms import gpu_mbh

pytestmark = pytest.mark.gpu

SMALL = [(N.RASTRIGIN, 10, 12), (N.RASTRIGIN, 50, 6), (N.ROSENBROCK, 10, 12), (N.ROSENBROCK, 40, 6),
         (N.LENNARD_JONES, 8, 6), (N.LENNARD_JONES, 40, 3)]
PARAMS = dict(hops=4, stop=3, steps=12, perturb=0.05, step0=0.05, step_min=1e-6, seed=11)


def host_loop(fg, x0, udp, kind):
    lb, ub = udp.get_bounds()
    out = [R.refine_one(fg, x0[r], lb, ub, r, PARAMS["hops"], PARAMS["stop"], PARAMS["steps"], PARAMS["perturb"],
                        PARAMS["step0"], PARAMS["step_min"], PARAMS["seed"], R.refine_lanes(kind, udp.get_nx()))
           for r in range(x0.shape[0])]
    return np.array([o[0] for o in out]), np.array([o[1] for o in out]), sum(o[2] for o in out)


@pytest.mark.parametrize("kind,param,n", SMALL)
def test_gpu_loop_equals_host_restatement_on_gpu_values(ctx, kind, param, n):
    udp = P.from_kind(kind, param, ctx)
    x0 = W.uniform_batch(kind, param, n, seed=7)
    xg, fgpu, evals = gpu_mbh(context=ctx, **PARAMS).refine(udp, x0)

    def gpu_point(x):
        f, g = udp.batch_gradient(x[None, :])
        return f[0], g[0]

    xh, fh, eh = host_loop(gpu_point, x0, udp, kind)
    assert np.array_equal(xh, xg), (kind, param)
    assert np.array_equal(fh, fgpu), (kind, param)
    assert eh == evals
    assert np.all(fgpu <= udp.batch_fitness(x0))


@pytest.mark.parametrize("kind,param,n", SMALL)
def test_gpu_loop_against_the_reference_arithmetic(ctx, orc, ref, kind, param, n):
    """The same loop on pagmo's own fitness and gradient: the GPU's values
    differ from the reference's in the last bits, so the trajectories agree
    to within a small tolerance unless an acceptance test falls on a tie."""
    udp = P.from_kind(kind, param, ctx)
    x0 = W.uniform_batch(kind, param, n, seed=7)
    xg, fgpu, _ = gpu_mbh(context=ctx, **PARAMS).refine(udp, x0)

    def ref_point(x):
        f = ref.fitness_rows(kind, param, x[None, :])[0]
        if kind == N.LENNARD_JONES:
            g = orc.batch_gradient_ld(kind, param, x[None, :])[0][0]
        else:
            g = ref.gradient_rows(kind, param, x[None, :])[0]
        return f, g

    xr, fr, _ = host_loop(ref_point, x0, udp, kind)
    lb, ub = udp.get_bounds()
    close_f = np.abs(fgpu - fr) <= 1e-9 * np.maximum(1.0, np.abs(fr))
    close_x = np.max(np.abs(xg - xr) / (ub - lb), axis=1) <= 1e-6
    agree = close_f & close_x
    print(f"\nREFINE vs reference {kind}/{param}: {int(agree.sum())}/{n} individuals agree; "
          f"max |f_gpu - f_ref| / max(1, |f_ref|) = {np.max(np.abs(fgpu - fr) / np.maximum(1.0, np.abs(fr))):.2e}")
    assert agree.sum() >= n - 1, (kind, param, fgpu, fr)


@pytest.mark.parametrize("kind,param,n", [(N.RASTRIGIN, 50, 65536), (N.ROSENBROCK, 1000, 8192),
                                          (N.LENNARD_JONES, 150, 1024)])
def test_large_batches(ctx, kind, param, n):
    udp = P.from_kind(kind, param, ctx)
    x0 = W.uniform_batch(kind, param, n, seed=3)
    f0 = udp.batch_fitness(x0)
    algo = gpu_mbh(hops=3, stop=2, steps=8, perturb=0.02, step0=0.02, step_min=1e-7, seed=5, context=ctx)
    x, f, evals = algo.refine(udp, x0)
    lb, ub = udp.get_bounds()
    assert np.all(x >= lb) and np.all(x <= ub)
    assert np.all(f <= f0)
    assert np.mean(f < f0) > 0.5  # most individuals improve
    fb = udp.batch_fitness(x)
    assert np.max(np.abs(fb - f) / np.maximum(1.0, np.abs(f))) <= 1e-12
    assert n * (1 + 1) <= evals <= n * (1 + 3 * (1 + 8))
    # an evolve keeps the better of the two
    xe, fe = algo.evolve(udp, x0, f0)
    assert np.all(fe <= f0)


def test_arguments_are_checked(ctx):
    udp = P.rastrigin(5, ctx)
    with pytest.raises(ValueError, match=r"The perturbation must be in \]0,1\]"):
        gpu_mbh(perturb=0.0, context=ctx)
    bad = gpu_mbh(context=ctx)
    bad.params.perturb = 1.5
    with pytest.raises(ValueError, match=r"The perturbation must be in \]0,1\]"):
        bad.refine(udp, np.zeros((2, 5)))
    bad = gpu_mbh(step0=0.01, step_min=0.1, context=ctx)
    with pytest.raises(ValueError, match="step_min"):
        bad.refine(udp, np.zeros((2, 5)))
    with pytest.raises(NotImplementedError):
        gpu_mbh(context=ctx).refine(P.ackley(5, ctx), np.zeros((2, 5)))
    x, f, e = gpu_mbh(context=ctx).refine(udp, np.zeros((0, 5)))
    assert x.shape == (0, 5) and f.shape == (0,) and e == 0
