"""Pins the hypervolume oracle (oracle/hypervolume.cpp, long double) to the reference.

- the known answers of tests/hypervolume.cpp:229-297 (2 and 3 objectives);
- the compiled reference (hypervolume(points, true).compute(ref)) on random,
  tied, duplicated, dominated and border point sets, within 1e-12 relative
  (the reference's hv3d updates its sweep area by subtraction);
- the reference's own compute test cases for hv2d and hv3d
  (tests/hypervolume_test_data, read where the reference tree exists) within
  the tolerance its test list states (1e-8).
"""
from pathlib import Path

import numpy as np
import pytest

import oracle


def test_known_answers(orc):
    assert orc.hypervolume([[1, 2], [2, 1]], [3, 3]) == 3.0
    assert orc.hypervolume([[1, 2], [2, 1]], [2, 2]) == 0.0
    assert orc.hypervolume([[1, 1, 1], [2, 2, 2]], [3, 3, 3]) == 8.0
    assert orc.hypervolume([[1, 2, 1], [2, 1, 1]], [2, 2, 2]) == 0.0
    assert abs(orc.hypervolume([[2.3, 4.5], [3.4, 3.4], [6.0, 1.2]], [7, 7]) - 17.91) <= 1e-14
    assert abs(orc.hypervolume([[2.3, 4.5, 3.2], [3.4, 3.4, 3.4], [6.0, 1.2, 3.6]], [7, 7, 7]) - 66.386) <= 1e-13


def point_sets(rng):
    for n, m in ((1, 2), (2, 3), (17, 2), (128, 2), (128, 3), (700, 3), (2048, 3)):
        yield f"uniform {n}x{m}", rng.random((n, m)), np.full(m, 1.1)
    for n, m in ((200, 2), (300, 3)):
        p = np.floor(rng.random((n, m)) * 8) / 8  # ties and duplicates
        p[:5, 0] = 1.0  # on the border of the reference point in one coordinate
        yield f"grid {n}x{m}", p, np.full(m, 1.0)
    w = rng.dirichlet(np.ones(3), 500)  # a front on the simplex plus dominated layers
    yield "simplex layers", np.concatenate([w, w * 1.5, w * 2.0]), np.full(3, 2.5)


def test_against_compiled_reference(orc, ref):
    rng = np.random.default_rng(17)
    for label, p, r in point_sets(rng):
        want = ref.hypervolume(p, r)
        got = orc.hypervolume(p, r)
        assert abs(got - want) <= 1e-12 * max(abs(want), 1e-300), label


def read_cases(path):
    tok = path.read_text().split()
    pos = 0

    def nxt():
        nonlocal pos
        pos += 1
        return tok[pos - 1]
    for _ in range(int(nxt())):
        m, n = int(nxt()), int(nxt())
        r = np.array([float(nxt()) for _ in range(m)])
        p = np.array([float(nxt()) for _ in range(n * m)]).reshape(n, m)
        yield p, r, float(nxt())


@pytest.mark.parametrize("name", ["c_max_t100_d2_n128", "c_max_t100_d3_n128", "c_max_t1_d3_n2048"])
def test_reference_test_cases(orc, name):
    path = None if oracle.REF_ROOT is None else oracle.REF_ROOT / "tests" / "hypervolume_test_data" / "testcases" / name
    if path is None or not path.exists():
        pytest.skip("the reference's test data is only present where its tree is")
    for p, r, want in read_cases(path):
        assert abs(orc.hypervolume(p, r) - want) < 1e-8, name
