"""GPU-backed user-defined problems mirroring pagmo's rastrigin, rosenbrock,
lennard_jones, ackley, griewank and schwefel UDPs
(src/problems/{rastrigin,rosenbrock,lennard_jones,ackley,griewank,schwefel}.cpp).

They expose the UDP interface pagmo's ``problem`` wraps (``fitness``,
``get_bounds``, ``get_name``, ``get_thread_safety``) plus the optional hooks the
batch path uses: ``batch_fitness`` (src/problem.cpp:413-425, picked by
member_bfe/default_bfe) and ``gradient`` (src/problem.cpp:456-467), and the
batch extension ``batch_gradient`` (fitness and gradient of a whole batch in
one pass; the reference has no batch gradient hook). Every evaluation runs on
the GPU through libpgx; the per-row ``fitness``/``gradient`` are one-row
batches (correct, but only the batch calls are fast).
"""
from __future__ import annotations

import numpy as np

from . import _native as N


def _as_rows(dvs, nx: int) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(dvs, dtype=np.float64)).reshape(-1)
    if a.size % nx:
        raise ValueError(
            "Invalid argument for a batch fitness evaluation: the length of the vector representing the decision "
            f"vectors, {a.size}, is not an exact multiple of the dimension of the problem, {nx}")
    return a


class _gpu_udp:
    kind = 0
    thread_safety = "constant"

    def __init__(self, param: int, context: N.Context | None = None):
        self.param = int(param)
        self._nx = N.problem_nx(self.kind, self.param)  # validates like the reference constructors
        self._ctx = context

    @property
    def ctx(self) -> N.Context:
        return self._ctx if self._ctx is not None else N.default_context()

    def get_nx(self) -> int:
        return self._nx

    def get_nobj(self) -> int:
        return 1

    def get_nf(self) -> int:
        return 1

    def get_bounds(self):
        lb, ub = N.problem_bounds(self.kind, self.param)
        return lb, ub

    def get_thread_safety(self) -> str:
        return self.thread_safety

    def batch_fitness(self, dvs) -> np.ndarray:
        x = _as_rows(dvs, self._nx)
        n = x.size // self._nx
        f = np.empty(n)
        if n:
            N.check(N.lib().pgx_batch_fitness(self.ctx.handle, self.kind, self.param, N.ptr(x), n, N.ptr(f)))
        return f

    def batch_gradient(self, dvs, with_fitness: bool = True):
        """(fitness[n], gradient[n, nx]) of a whole batch in one pass."""
        x = _as_rows(dvs, self._nx)
        n = x.size // self._nx
        g = np.empty((n, self._nx))
        f = np.empty(n) if with_fitness else None
        if n:
            N.check(N.lib().pgx_batch_gradient(self.ctx.handle, self.kind, self.param, N.ptr(x), n, N.ptr(f),
                                               N.ptr(g)))
        return (f, g) if with_fitness else g

    def fitness(self, x) -> np.ndarray:
        x = np.asarray(x, dtype=np.float64)
        if x.size != self._nx:
            raise ValueError(f"A decision vector is incompatible with a problem of type '{self.get_name()}': "
                             f"the number of dimensions of the problem is {self._nx}, while the decision vector "
                             f"has a size of {x.size} (the two values should be equal)")
        return self.batch_fitness(x)

    def gradient(self, x) -> np.ndarray:
        x = np.asarray(x, dtype=np.float64)
        if x.size != self._nx:
            raise ValueError(f"A decision vector is incompatible with a problem of type '{self.get_name()}': "
                             f"the number of dimensions of the problem is {self._nx}, while the decision vector "
                             f"has a size of {x.size} (the two values should be equal)")
        return self.batch_gradient(x, with_fitness=False).reshape(-1)


class rastrigin(_gpu_udp):
    """rastrigin{dim}: f = 10 n + sum(x_i^2 - 10 cos(2 pi x_i)) on [-5.12, 5.12]^n."""
    kind = N.RASTRIGIN

    def __init__(self, dim: int = 1, context=None):
        super().__init__(dim, context)

    def get_name(self) -> str:
        return "Rastrigin Function"

    def best_known(self):
        return np.zeros(self._nx)


class rosenbrock(_gpu_udp):
    """rosenbrock{dim}: f = sum 100 (x_i^2 - x_{i+1})^2 + (x_i - 1)^2 on [-5, 10]^n."""
    kind = N.ROSENBROCK

    def __init__(self, dim: int = 2, context=None):
        super().__init__(dim, context)

    def get_name(self) -> str:
        return "Multidimensional Rosenbrock Function"

    def best_known(self):
        return np.ones(self._nx)


class lennard_jones(_gpu_udp):
    """lennard_jones{atoms}: 4 sum_{i<j} (r^-12 - r^-6) with three pinned coordinates."""
    kind = N.LENNARD_JONES

    def __init__(self, atoms: int = 3, context=None):
        super().__init__(atoms, context)

    def get_name(self) -> str:
        return f"Lennard Jones Cluster ({self.param} atoms)"


class _fitness_only_udp(_gpu_udp):
    """The reference gives these UDPs no gradient: gradient requests raise
    NotImplementedError, as pagmo's problem::gradient raises
    not_implemented_error (src/problem.cpp:453-467)."""

    def has_gradient(self) -> bool:
        return False

    def batch_gradient(self, dvs, with_fitness: bool = True):
        raise NotImplementedError("The gradient has been requested but it is not implemented in the UDP")

    def gradient(self, x):
        raise NotImplementedError("The gradient has been requested but it is not implemented in the UDP")


class ackley(_fitness_only_udp):
    """ackley{dim}: f = -20 exp(-0.2 sqrt(sum x^2 / n)) - exp(sum cos(2 pi x) / n) + 20 + e on [-15, 30]^n."""
    kind = N.ACKLEY

    def __init__(self, dim: int = 1, context=None):
        super().__init__(dim, context)

    def get_name(self) -> str:
        return "Ackley Function"

    def best_known(self):
        return np.zeros(self._nx)


class griewank(_fitness_only_udp):
    """griewank{dim}: f = sum x^2 / 4000 - prod cos(x_i / sqrt(i + 1)) + 1 on [-600, 600]^n."""
    kind = N.GRIEWANK

    def __init__(self, dim: int = 1, context=None):
        super().__init__(dim, context)

    def get_name(self) -> str:
        return "Griewank Function"

    def best_known(self):
        return np.zeros(self._nx)


class schwefel(_fitness_only_udp):
    """schwefel{dim}: f = 418.9828872724338 n - sum x sin(sqrt|x|) on [-500, 500]^n."""
    kind = N.SCHWEFEL

    def __init__(self, dim: int = 1, context=None):
        super().__init__(dim, context)

    def get_name(self) -> str:
        return "Schwefel Function"

    def best_known(self):
        return np.full(self._nx, 420.9687)


def from_kind(kind: int, param: int, context=None) -> _gpu_udp:
    return {N.RASTRIGIN: rastrigin, N.ROSENBROCK: rosenbrock, N.LENNARD_JONES: lennard_jones, N.ACKLEY: ackley,
            N.GRIEWANK: griewank, N.SCHWEFEL: schwefel}[kind](param, context)
