"""gpu_bfe: a user-defined batch fitness evaluator (UDBFE) backed by libpgx.

Mirrors the contract of pagmo's UDBFEs (include/pagmo/bfe.hpp:68-108,
src/batch_evaluators/thread_bfe.cpp:64-144): ``bfe(prob, dvs) -> fvs`` with dvs
row-major (n * nx) and fvs (n * nf). It evaluates the problems it knows on the
GPU in one pass; any other problem is rejected (there is no CPU fallback).
Like every UDBFE it does not increment the problem's fevals counter: the
type-erased pagmo::bfe does that (src/bfe.cpp:106-107, member_bfe.cpp:42-44).
The wrapper ``bfe`` below reproduces that accounting for Python callers.
"""
from __future__ import annotations

import numpy as np

from . import problems as P


class gpu_bfe:
    """Batch fitness evaluator running the GB300 kernels."""

    def get_name(self) -> str:
        return "GB300 batch fitness evaluator"

    def get_extra_info(self) -> str:
        return ""

    def get_thread_safety(self) -> str:
        return "basic"

    def __call__(self, prob, dvs) -> np.ndarray:
        udp = getattr(prob, "udp", prob)
        if isinstance(udp, P.translate):
            return udp.batch_fitness(dvs)
        if not isinstance(udp, (P._gpu_udp, P._gpu_mo_udp)):
            name = udp.get_name() if hasattr(udp, "get_name") else type(udp).__name__
            raise ValueError(f"Cannot use a gpu_bfe on the problem '{name}': only the GPU rastrigin, rosenbrock, "
                             "lennard_jones, ackley, griewank, schwefel, zdt and dtlz problems are supported")
        return udp.batch_fitness(dvs)


class problem:
    """Minimal stand-in for pagmo::problem's bookkeeping around a UDP: dims,
    the input/output checks of bfe::operator() and the fevals counter."""

    def __init__(self, udp):
        self.udp = udp
        self.fevals = 0
        self.gevals = 0

    def get_nx(self) -> int:
        return self.udp.get_nx()

    def get_nf(self) -> int:
        return self.udp.get_nf()

    def get_fevals(self) -> int:
        return self.fevals

    def get_name(self) -> str:
        return self.udp.get_name()

    def fitness(self, x):
        f = self.udp.fitness(x)
        self.fevals += 1
        return f

    def gradient(self, x):
        g = self.udp.gradient(x)
        self.gevals += 1
        return g


class bfe:
    """Type-erased batch evaluator, as pagmo::bfe::operator() (src/bfe.cpp:91-110):
    checks the input size, calls the UDBFE, checks the output, adds n to fevals."""

    def __init__(self, udbfe=None):
        self.udbfe = udbfe if udbfe is not None else gpu_bfe()

    def get_name(self) -> str:
        return self.udbfe.get_name()

    def __call__(self, prob: problem, dvs) -> np.ndarray:
        nx = prob.get_nx()
        a = np.asarray(dvs, dtype=np.float64).reshape(-1)
        if a.size % nx:
            raise ValueError(
                "Invalid argument for a batch fitness evaluation: the length of the vector representing the decision "
                f"vectors, {a.size}, is not an exact multiple of the dimension of the problem, {nx}")
        out = np.asarray(self.udbfe(prob, a))
        nf = prob.get_nf()
        if out.size % nf:
            raise ValueError(
                "An invalid result was produced by a batch fitness evaluation: the length of the vector representing "
                f"the fitness vectors, {out.size}, is not an exact multiple of the fitness dimension of the problem, "
                f"{nf}")
        if out.size // nf != a.size // nx:
            raise ValueError(
                "An invalid result was produced by a batch fitness evaluation: the number of produced fitness vectors, "
                f"{out.size // nf}, differs from the number of input decision vectors, {a.size // nx}")
        prob.fevals += a.size // nx
        return out
