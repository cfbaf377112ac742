"""Pins the hypervolume oracle (oracle/hypervolume.cpp, long double) to the reference.

- the known answers of tests/hypervolume.cpp:229-297 (2 and 3 objectives);
- the compiled reference (hypervolume(points, true).compute(ref)) on random,
  tied, duplicated, dominated and border point sets, within 1e-12 relative
  (the reference's hv3d updates its sweep area by subtraction);
- the reference's own compute test cases for hv2d and hv3d
  (tests/hypervolume_test_data, read where the reference tree exists) within
  the tolerance its test list states (1e-8).

And the WFG oracle (orc_hvwfg, orc_hvwfg_contributions: double, the
reference's operation order):
- bit for bit against the compiled reference's hvwfg compute and
  contributions on random, tied, duplicated and dominated sets of 2 to 7
  objectives;
- the known contributions of tests/hypervolume.cpp:322-460;
- the reference's WFG compute, exclusive and least-contributor test cases
  (hypervolume_test_data: c_max_t1_d5_n1024, c_max_t1_d7_n64, e_max_d2/3/5,
  lc_max_d2/3) with their tolerances.
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


def wfg_sets(rng):
    for m in (2, 3, 4, 5, 6, 7):
        for n in (1, 2, 3, 5, 17, 40):
            yield f"uniform {n}x{m}", rng.random((n, m)), np.full(m, 1.2)
            g = np.floor(rng.random((n, m)) * 5) / 5  # ties, duplicates, dominated points
            yield f"grid {n}x{m}", g, np.full(m, 1.0)
    w = rng.dirichlet(np.ones(5), 60)  # a simplex front with dominated copies and duplicates
    yield "simplex 5", np.concatenate([w, w * 1.3, w[:10]]), np.full(5, 1.5)


def lift2(p, r):
    """The points and reference hv2d::contributions hands to hv3d (hv_hv2d.cpp:135-143)."""
    return np.column_stack([p, np.zeros(len(p))]), np.append(r, 1.0)


def test_wfg_oracle_bit_exact_with_compiled_reference(orc, ref):
    rng = np.random.default_rng(23)
    for label, p, r in wfg_sets(rng):
        m = p.shape[1]
        assert orc.hvwfg(p, r) == ref.hvwfg(p, r), label
        if m >= 4:
            assert orc.hvwfg(p, r) == ref.hypervolume(p, r), label
        c = orc.hvwfg_contributions(p, r)
        if len(p) > 1:  # a lone point's contribution is hypervolume's own product (hypervolume.cpp:303-307)
            assert np.array_equal(c, ref.hv_contributions(p, r, wfg=True)), label
            if m >= 4:
                assert np.array_equal(c, ref.hv_contributions(p, r)), label


# tests/hypervolume.cpp:322-460: (points, reference point, contributions)
KNOWN_CONTRIBUTIONS = [
    ([[1, 6.5], [1, 6], [1, 5], [2, 5], [3, 5], [3, 3], [4, 6.5], [4.5, 4], [5, 3], [5, 1.5], [7, 1.5], [7, 3.5]],
     [7, 6.5], [0, 0, 1, 0, 0, 3.5, 0, 0, 0, 3, 0, 0]),
    ([[1, 1]], [2, 2], [1]),
    ([[1, 1], [1, 1]], [2, 2], [0, 0]),
    ([[1, 1], [1, 1], [1, 1], [0.5, 0.5]], [2, 2], [0, 0, 0, 1.25]),
    ([[-6, -1, -6], [-1, -3, -5], [-3, -4, -4], [-4, -2, -3], [-5, -5, -2], [-2, -6, -1]], [0, 0, 0],
     [18, 2, 12, 1, 18, 2]),
    ([[-6, -1, -6], [-1, -3, -5], [-3, -4, -4], [-4, -2, -3], [-5, -5, -2], [-2, -6, -1], [-3, -1, -3],
      [-1, -1, -5], [-1, -2, -4], [-1, -3, -4], [-7, -7, 0], [0, -5, -5], [-7, 0, -7]], [0, 0, 0],
     [18, 2, 12, 1, 18, 2, 0, 0, 0, 0, 0, 0, 0]),
    ([[3, 3, 3], [4, 4, 4]], [5, 5, 5], [7, 0]),
    ([[3, 3, 3], [4, 4, 4], [3, 3, 3], [3, 3, 2], [3, 3, 1]], [5, 5, 5], [0, 0, 0, 0, 4]),
    ([[-1, -1, -1]] * 3 + [[-1000, -1000, -1000]], [0, 0, 0], [0, 0, 0, 999999999]),
    ([[1, 1, 1, 1], [4, 4, 4, 4], [3, 3, 3, 3]], [5, 5, 5, 5], [240, 0, 0]),
    ([[1, 1, 1, 1], [4, 4, 4, 4], [3, 3, 3, 3], [1, 1, 1, 1]], [5, 5, 5, 5], [0, 0, 0, 0]),
]


def test_wfg_oracle_known_contributions(orc):
    for p, r, want in KNOWN_CONTRIBUTIONS:
        p, r = np.array(p, dtype=float), np.array(r, dtype=float)
        if p.shape[1] == 2 and len(p) > 1:
            p, r = lift2(p, r)
        got = orc.hvwfg_contributions(p, r) if len(p) > 1 else [abs(np.prod(p[0] - r))]
        assert list(got) == [float(x) for x in want], (p.tolist(), list(got))
    # tests/hypervolume.cpp:258-309: volumes of 4 and 5 objectives
    assert orc.hvwfg([[1, 1, 1, 1], [2, 2, 2, 2]], [3, 3, 3, 3]) == 16.0
    assert orc.hvwfg([[1, 1, 1, 3], [2, 2, 2, 3]], [3, 3, 3, 3]) == 0.0
    assert orc.hvwfg([[1, 1, 1, 1], [1, 1, 1, 1]], [2, 2, 2, 2]) == 1.0
    assert orc.hvwfg([[1, 1, 1, 1], [1, 1, 1, 1], [0, 0, 0, 0]], [2, 2, 2, 2]) == 16.0
    assert orc.hvwfg([[2.3, 4.5, 3.2, 1.9, 6.0], [3.4, 3.4, 3.4, 2.1, 5.8], [6.0, 1.2, 3.6, 3.0, 6.0]],
                     [7, 7, 7, 7, 7]) == 373.21228


def read_typed(path, kind):
    """The reference's hypervolume test files: (points, reference point, answer) with the answer a volume
    (compute), (index, volume) (exclusive) or an index (least_contributor)."""
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
        if kind == "compute":
            yield p, r, float(nxt())
        elif kind == "exclusive":
            yield p, r, (int(nxt()), float(nxt()))
        else:
            yield p, r, int(nxt())


def test_data_path(name):
    path = None if oracle.REF_ROOT is None else oracle.REF_ROOT / "tests" / "hypervolume_test_data" / "testcases" / name
    if path is None or not path.exists():
        pytest.skip("the reference's test data is only present where its tree is")
    return path


test_data_path.__test__ = False


def test_wfg_reference_test_cases(orc):
    # compute wfg c_max_t1_d5_n1024 with the list's tolerance 1e-3 (testcases_list.txt)
    for p, r, want in read_typed(test_data_path("c_max_t1_d5_n1024"), "compute"):
        assert abs(orc.hvwfg(p, r) - want) < 1e-3
    # exclusive wfg e_max_d5, hv3d e_max_d3, hv2d e_max_d2 (1e-8): the contribution of the point
    for name in ("e_max_d2", "e_max_d3", "e_max_d5"):
        for p, r, (i, want) in read_typed(test_data_path(name), "exclusive"):
            q, rr = lift2(p, r) if p.shape[1] == 2 else (p, r)
            got = orc.hvwfg_contributions(q, rr)[i] if len(p) > 1 else orc.hvwfg(p, r)
            assert abs(got - want) < 1e-8, (name, got, want)
    # least_contributor wfg / hv3d lc_max_d3, hv2d lc_max_d2: the first smallest contribution
    for name in ("lc_max_d2", "lc_max_d3"):
        for p, r, want in read_typed(test_data_path(name), "least"):
            q, rr = lift2(p, r) if p.shape[1] == 2 else (p, r)
            got = int(np.argmin(orc.hvwfg_contributions(q, rr))) if len(p) > 1 else 0
            assert got == want, name


def test_wfg_reference_test_cases_against_compiled_reference(orc, ref):
    for name in ("c_max_t1_d5_n1024", "c_max_t1_d7_n64"):
        for p, r, _ in read_typed(test_data_path(name), "compute"):
            assert orc.hvwfg(p, r) == ref.hypervolume(p, r), name
