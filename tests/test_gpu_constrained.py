"""hock_schittkowski_71 and the unconstrain meta-problem on the GPU (pgx_constrained_batch_fitness,
pgx_unconstrain_batch_fitness): every row bit for bit the oracle's restatement of the reference's arithmetic
(itself pinned bit for bit to the compiled reference), and the compiled reference's where it is built; every
penalty method, with and without constraint tolerances; batches larger than one pipeline chunk."""
import numpy as np
import pytest

from pagmo2_gb300 import problems as P
from test_oracle_constrained import METHODS, rows

pytestmark = pytest.mark.gpu


def test_hs71_rows(ctx, orc):
    h = P.hock_schittkowski_71(ctx)
    x = rows(7, 5000)
    f = h.batch_fitness(x).reshape(-1, 3)
    assert np.array_equal(f, orc.hs71_fitness(x))
    assert np.array_equal(h.fitness(x[3]), orc.hs71_fitness(x[3:4])[0])
    lb, ub = h.get_bounds()
    assert lb.tolist() == [1.0] * 4 and ub.tolist() == [5.0] * 4


@pytest.mark.parametrize("method", METHODS)
def test_unconstrain_rows(ctx, orc, method):
    h = P.hock_schittkowski_71(ctx)
    x = rows(11, 3000)
    w = [1.5, 0.25] if method == "weighted" else []
    for tol in (None, [1e-3, 0.5]):
        u = P.unconstrain(h, method, w, tol)
        assert np.array_equal(u.batch_fitness(x), orc.unconstrain_hs71(method, x, w, tol)), (method, tol)


@pytest.mark.parametrize("method", METHODS)
def test_unconstrain_against_reference(ctx, ref, method):
    h = P.hock_schittkowski_71(ctx)
    x = rows(13, 500)
    w = [0.75, 2.0] if method == "weighted" else []
    u = P.unconstrain(h, method, w, [0.0, 1e-2])
    assert np.array_equal(u.batch_fitness(x), ref.unconstrain_hs71(method, x, w, [0.0, 1e-2]))


def test_large_batch(ctx, orc):
    x = 1.0 + 4.0 * np.random.default_rng(1).random((3_000_000, 4))
    u = P.unconstrain(P.hock_schittkowski_71(ctx), "kuri")
    got = u.batch_fitness(x)
    assert np.array_equal(got[::997], orc.unconstrain_hs71("kuri", x[::997]))
    assert np.array_equal(got[-5:], orc.unconstrain_hs71("kuri", x[-5:]))
