"""Host-side checks of the C ABI that need no GPU: the library loads, exports
every entry point include/pgx.h declares, validates arguments like the
reference (constructor errors, bounds) and fails loudly without a device."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from pagmo2_gb300 import _native as N
from pagmo2_gb300 import workloads as W

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    out = set()
    for h in (ROOT / "include").glob("*.h"):
        out |= set(re.findall(r"PGX_API[^;(]*?\b(pgx_\w+)\s*\(", h.read_text()))
    return out


def test_library_exports_every_declared_symbol():
    lib = N.lib()
    syms = declared_symbols()
    assert len(syms) >= 14
    for s in sorted(syms):
        assert hasattr(lib, s), s
    assert set(N.SIGNATURES) == syms, set(N.SIGNATURES) ^ syms
    assert lib.pgx_abi_version() == 1


def test_problem_validation_messages():
    with pytest.raises(ValueError, match="Rastrigin Function must have minimum 1 dimension, 0 requested"):
        N.problem_nx(N.RASTRIGIN, 0)
    with pytest.raises(ValueError, match="Rosenbrock Function must have minimum 2 dimensions, 1 requested"):
        N.problem_nx(N.ROSENBROCK, 1)
    for atoms in (0, 1, 2):
        with pytest.raises(ValueError, match="must be positive and greater than 2"):
            N.problem_nx(N.LENNARD_JONES, atoms)
    with pytest.raises(ValueError, match="Overflow caused by the number of atoms"):
        N.problem_nx(N.LENNARD_JONES, 0xFFFFFFFF // 2)
    with pytest.raises(ValueError, match="unknown problem kind"):
        N.problem_nx(9, 3)
    assert N.problem_nx(N.LENNARD_JONES, 150) == 444


def test_bounds_match_reference_udps():
    lb, ub = N.problem_bounds(N.RASTRIGIN, 1)
    assert lb.tolist() == [-5.12] and ub.tolist() == [5.12]
    lb, ub = N.problem_bounds(N.ROSENBROCK, 2)
    assert lb.tolist() == [-5.0, -5.0] and ub.tolist() == [10.0, 10.0]
    lb, ub = N.problem_bounds(N.LENNARD_JONES, 3)
    assert lb.tolist() == [-3, -3, -3] and ub.tolist() == [3, 3, 3]
    for kind, param in ((1, 7), (2, 9), (3, 150)):
        lb, ub = N.problem_bounds(kind, param)
        wl, wu = W.bounds(kind, param)
        assert np.array_equal(lb, wl) and np.array_equal(ub, wu)


def test_bounds_against_compiled_reference(ref):
    for kind, param in ((1, 11), (2, 13), (3, 40)):
        nx = N.problem_nx(kind, param)
        assert all(np.array_equal(a, b) for a, b in zip(N.problem_bounds(kind, param), ref.bounds(kind, param, nx)))


def test_no_device_fails_loudly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError):
        N.Context(0)


def test_workloads_are_seeded_and_in_bounds():
    a = W.rastrigin_batch(64, 50)
    b = W.rastrigin_batch(64, 50)
    assert np.array_equal(a, b) and a.min() >= -5.12 and a.max() <= 5.12
    x = W.lj_batch(8, 10)
    lb, ub = W.bounds(N.LENNARD_JONES, 10)
    assert np.all(x >= lb) and np.all(x <= ub)
    p = W.nsga2_points(2000, 3, layers=10)
    assert p.shape == (2000, 3)
    # 5 % exact duplicates
    assert np.unique(p, axis=0).shape[0] <= 1900 + 1
    isl = W.archipelago(64)
    assert len(isl) == 64 and all(32 <= r.n <= 4096 for r in isl)
    assert all(r.dvs.shape == (r.n, r.nx) for r in isl)


def test_workload_matches_mt19937_stream():
    # RandomState(seed).random_sample() is genrand_res53 of mt19937(seed)
    rs = np.random.RandomState(1)
    ints = rs.randint(0, 2**32, size=2, dtype=np.uint32)  # two raw 32-bit draws
    a, b = int(ints[0]) >> 5, int(ints[1]) >> 6
    u = (a * 67108864.0 + b) / 9007199254740992.0
    assert u == np.random.RandomState(1).random_sample()


def test_lj_encode_preserves_energy(orc):
    rs = np.random.RandomState(3)
    pos = rs.normal(size=(12, 3)) * 2
    dv = W.lj_encode(pos)
    d = np.linalg.norm(pos[:, None, :] - pos[None, :, :], axis=2)
    iu = np.triu_indices(12, 1)
    s = d[iu] ** -6
    e = 4 * np.sum(s * s - s)
    fl, _ = orc.batch_fitness_ld(3, 12, dv[None, :])
    assert abs(fl[0] - e) <= 1e-12 * np.sum(s * s + s) * 4


def test_build_id_is_this_builds_digest():
    """The library reports the digest its build recipe stamped it with (the
    autotuner's cache key starts with it)."""
    from pagmo2_gb300 import build as B

    bid = N.lib().pgx_build_id().decode()
    assert bid == (B.OUT / "libpgx.stamp").read_text()[:16]
