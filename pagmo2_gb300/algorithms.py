"""Batched gradient-based local refinement (pgx_refine_batch).

gpu_mbh runs monotonic basin hopping, the scheme of pagmo's mbh
(src/algorithms/mbh.cpp:102-200), on every individual of a batch at once on
the GPU, with a projected-gradient descent driven by the batched adjoint as
the inner local optimiser: per individual, each trial perturbs the best point
within perturb * (ub - lb) (clipped to the bounds, as mbh does), takes up to
`steps` descent steps, and keeps the result when it lowers the fitness; an
individual stops after `stop` trials in a row without improvement, or after
`hops` trials. mbh takes an inner pagmo algorithm and accepts a whole
population when its best improves; here each individual is its own chain.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .problems import _as_rows


class gpu_mbh:
    """Monotonic basin hopping with gradient descent on a whole batch (GPU).

    hops: at most this many trials per individual; stop: trials in a row
    without improvement that end an individual's chain (mbh's stop); steps:
    projected-gradient steps per trial; perturb: perturbation half-width as a
    fraction of (ub - lb), in ]0, 1] (mbh's perturb); step0 / step_min: first
    and smallest step length of a descent, in box-scaled units; seed: the
    perturbations are a function of (seed, individual, trial, coordinate).
    """

    def __init__(self, hops: int = 10, stop: int = 5, steps: int = 20, perturb: float = 0.01, step0: float = 0.05,
                 step_min: float = 1e-8, seed: int = 0, context: N.Context | None = None):
        if not (0.0 < float(perturb) <= 1.0):
            raise ValueError(f"The perturbation must be in ]0,1], while a value of {perturb} was detected.")
        self.params = N.pgx_refine_params(int(hops), int(stop), int(steps), float(perturb), float(step0),
                                          float(step_min), int(seed) & 0xFFFFFFFFFFFFFFFF)
        self._ctx = context
        self.evals = 0

    @property
    def ctx(self) -> N.Context:
        return self._ctx if self._ctx is not None else N.default_context()

    def get_name(self) -> str:
        return "MBH with projected-gradient descent, every individual at once (GB300)"

    def set_seed(self, seed: int) -> None:
        self.params.seed = int(seed) & 0xFFFFFFFFFFFFFFFF

    def refine(self, udp, dvs):
        """(best decision vectors [n, nx], their fitness [n], evaluations made)
        for a GPU UDP with a gradient (rastrigin, rosenbrock, lennard_jones)."""
        nx = udp.get_nx()
        x = _as_rows(dvs, nx).copy()
        n = x.size // nx
        f = np.empty(n)
        ev = C.c_uint64(0)
        if n:
            N.check(N.lib().pgx_refine_batch(self.ctx.handle, udp.kind, udp.param, C.byref(self.params), N.ptr(x), n,
                                             N.ptr(f), C.byref(ev)))
        self.evals += ev.value
        return x.reshape(n, nx), f, ev.value

    def evolve(self, udp, dvs, fvs=None):
        """The population (decision vectors, fitness) after refinement; with
        fvs (the population's fitness) an individual keeps its point unless
        the refinement found a lower one."""
        x, f, _ = self.refine(udp, dvs)
        if fvs is not None:
            f0 = np.asarray(fvs, dtype=np.float64).reshape(-1)
            keep = ~(f < f0)
            x[keep] = _as_rows(dvs, udp.get_nx()).reshape(x.shape)[keep]
            f[keep] = f0[keep]
        return x, f
