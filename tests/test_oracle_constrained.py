"""Pins the oracle's hock_schittkowski_71 and unconstrain penalties (oracle/constrained.cpp) to the compiled
reference bit for bit, and checks the host side of the unconstrain meta-problem: its constructor's checks and
messages (src/problems/unconstrain.cpp:66-100, problem::set_c_tol, src/problem.cpp:620-636), which need no GPU."""
import numpy as np
import pytest

from pagmo2_gb300 import problems as P

METHODS = ["death penalty", "kuri", "weighted", "ignore_c", "ignore_o"]


def rows(seed=3, n=400):
    rng = np.random.default_rng(seed)
    x = 1.0 + 4.0 * rng.random((n, 4))
    x[:20] = np.round(x[:20])            # exact values: constraints exactly satisfied or violated
    x[20] = [1.0, 4.742999, 3.821150, 1.379408]  # near the known optimum
    x[21] = [1.0, 5.0, 5.0, 1.0]
    return x


def test_hs71_rows_bit_exact(orc, ref):
    x = rows()
    assert np.array_equal(orc.hs71_fitness(x), ref.hs71_fitness(x))


@pytest.mark.parametrize("method", METHODS)
def test_penalties_bit_exact(orc, ref, method):
    x = rows(5)
    w = [1.5, 0.25] if method == "weighted" else []
    for tol in (None, [1e-3, 0.5]):
        got = orc.unconstrain_hs71(method, x, w, tol)
        want = ref.unconstrain_hs71(method, x, w, tol)
        assert np.array_equal(got, want), (method, tol)


def test_constructor_messages():
    h = P.hock_schittkowski_71()
    with pytest.raises(ValueError, match="Length of weight vector is: 1 while the problem constraints are: 2"):
        P.unconstrain(h, "weighted", [1.0])
    with pytest.raises(ValueError, match=r"The method foo is not supported \(did you misspell\?\)"):
        P.unconstrain(h, "foo")
    with pytest.raises(ValueError, match="The weight vector needs to be empty to use the unconstrain method kuri"):
        P.unconstrain(h, "kuri", [1.0, 2.0])
    with pytest.raises(ValueError, match="Unconstrain can only be applied to constrained problems"):
        P.unconstrain(P.rastrigin(3))
    with pytest.raises(ValueError, match="The tolerance vector has a negative value at the index 1"):
        P.unconstrain(h, "kuri", c_tol=[0.0, -1.0])
    u = P.unconstrain(h, "ignore_o")
    assert u.get_nobj() == 1 and u.get_nx() == 4 and u.get_name() == "Hock Schittkowski 71 [unconstrained]"


def test_reference_messages(ref):
    x = rows()[:2]
    with pytest.raises(ValueError, match=r"The method foo is not supported \(did you misspell\?\)"):
        ref.unconstrain_hs71("foo", x)
    with pytest.raises(ValueError, match="Length of weight vector is: 1 while the problem constraints are: 2"):
        ref.unconstrain_hs71("weighted", x, [1.0])
