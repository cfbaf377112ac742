"""GPU-backed user-defined problems mirroring pagmo's rastrigin, rosenbrock,
lennard_jones, ackley, griewank, schwefel, zdt and dtlz UDPs
(src/problems/{rastrigin,rosenbrock,lennard_jones,ackley,griewank,schwefel,zdt,dtlz}.cpp).

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

import ctypes as C

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


class _gpu_mo_udp:
    """ZDT / DTLZ on the GPU: fitness vectors of nobj objectives, batch fitness
    in pagmo's fvs layout (n rows of nobj, flattened), p_distance per vector
    or averaged over a population (src/problems/zdt.cpp, src/problems/dtlz.cpp)."""
    thread_safety = "constant"

    def __init__(self, spec: N.pgx_mo_problem, context: N.Context | None = None):
        self._spec = spec
        self._nx, self._nobj, self._nix = N.mo_problem_dims(spec)  # the reference constructors' checks
        self._ctx = context

    @property
    def ctx(self) -> N.Context:
        return self._ctx if self._ctx is not None else N.default_context()

    def get_nx(self) -> int:
        return self._nx

    def get_nobj(self) -> int:
        return self._nobj

    def get_nf(self) -> int:
        return self._nobj

    def get_nix(self) -> int:
        return self._nix

    def get_bounds(self):
        return N.mo_problem_bounds(self._spec)

    def get_thread_safety(self) -> str:
        return self.thread_safety

    def has_gradient(self) -> bool:
        return False

    def batch_fitness(self, dvs) -> np.ndarray:
        x = _as_rows(dvs, self._nx)
        n = x.size // self._nx
        f = np.empty(n * self._nobj)
        if n:
            N.check(N.lib().pgx_mo_batch_fitness(self.ctx.handle, C.byref(self._spec), N.ptr(x), n, N.ptr(f)))
        return f

    def batch_p_distance(self, dvs) -> np.ndarray:
        """p_distance of every decision vector of a batch."""
        x = _as_rows(dvs, self._nx)
        n = x.size // self._nx
        out = np.empty(n)
        if n:
            N.check(N.lib().pgx_mo_p_distance(self.ctx.handle, C.byref(self._spec), N.ptr(x), n, N.ptr(out)))
        return out

    def fitness(self, x) -> np.ndarray:
        x = np.asarray(x, dtype=np.float64)
        if x.size != self._nx:
            raise ValueError(f"A decision vector is incompatible with a problem of type '{self.get_name()}': "
                             f"the number of dimensions of the problem is {self._nx}, while the decision vector "
                             f"has a size of {x.size} (the two values should be equal)")
        return self.batch_fitness(x)

    def p_distance(self, x) -> float:
        """p_distance(x) of one decision vector, or the mean over a population
        (anything with get_x()), summed in row order as the reference does."""
        if hasattr(x, "get_x"):
            pts = np.asarray(x.get_x(), dtype=np.float64).reshape(-1, self._nx)
            if pts.shape[0] == 0:
                return float("nan")
            vals = self.batch_p_distance(pts)
            return float(np.cumsum(vals)[-1] / vals.size)
        return self._p_distance_vector(np.asarray(x, dtype=np.float64).reshape(-1))

    def _p_distance_vector(self, v: np.ndarray) -> float:
        # dtlz.cpp:156-163 checks the size
        if v.size != self._nx:
            raise ValueError(f"The size of the decision vector should be {self._nx} while {v.size} was detected")
        return float(self.batch_p_distance(v)[0])


class zdt(_gpu_mo_udp):
    """zdt{prob_id, param}: the six two-objective ZDT problems (param is the
    dimension, except for ZDT5 whose 30 + 5 (param - 1) bits it counts)."""

    def __init__(self, prob_id: int = 1, param: int = 30, context=None):
        self.prob_id, self.param = int(prob_id), int(param)
        super().__init__(N.mo_problem(N.ZDT, self.prob_id, self.param), context)

    def get_name(self) -> str:
        return f"ZDT{self.prob_id}"

    def _p_distance_vector(self, v: np.ndarray) -> float:
        # zdt.cpp:204-224 does not check the size: the metric of a vector of
        # another length is that of the same ZDT problem at that length
        if v.size == self._nx:
            return float(self.batch_p_distance(v)[0])
        if self.prob_id == 5:
            if v.size < 30:
                raise ValueError(f"a ZDT5 decision vector has at least 30 entries, {v.size} given")
            other = zdt(5, (v.size - 30) // 5 + 1, self._ctx)
            return float(other.batch_p_distance(v[:other.get_nx()])[0])
        if v.size < 2:
            raise ValueError(f"a ZDT decision vector has at least 2 entries, {v.size} given")
        return float(zdt(self.prob_id, v.size, self._ctx).batch_p_distance(v)[0])


class dtlz(_gpu_mo_udp):
    """dtlz{prob_id, dim, fdim, alpha}: the seven scalable DTLZ problems on [0, 1]^dim."""

    def __init__(self, prob_id: int = 1, dim: int = 5, fdim: int = 3, alpha: int = 100, context=None):
        self.prob_id, self.dim, self.fdim, self.alpha = int(prob_id), int(dim), int(fdim), int(alpha)
        super().__init__(N.mo_problem(N.DTLZ, self.prob_id, self.dim, self.fdim, self.alpha), context)

    def get_name(self) -> str:
        return f"DTLZ{self.prob_id}"


class hock_schittkowski_71:
    """hock_schittkowski_71 (src/problems/hock_schittkowski_71.cpp) on the GPU: four variables in [1, 5], one
    objective, one equality and one inequality constraint; batch_fitness gives n rows of [f, ceq, cineq], the
    reference's values bit for bit. pagmo's gradient and hessians of this UDP are not provided."""
    thread_safety = "constant"

    def __init__(self, context: N.Context | None = None):
        self._ctx = context
        self.kind, self.param = N.HS71, 0

    @property
    def ctx(self) -> N.Context:
        return self._ctx if self._ctx is not None else N.default_context()

    def get_nx(self) -> int:
        return 4

    def get_nobj(self) -> int:
        return 1

    def get_nec(self) -> int:
        return 1

    def get_nic(self) -> int:
        return 1

    def get_nf(self) -> int:
        return 3

    def get_bounds(self):
        lb, ub = np.empty(4), np.empty(4)
        N.check(N.lib().pgx_constrained_bounds(N.HS71, 0, N.ptr(lb), N.ptr(ub)))
        return lb, ub

    def get_name(self) -> str:
        return "Hock Schittkowski 71"

    def get_thread_safety(self) -> str:
        return self.thread_safety

    def has_gradient(self) -> bool:
        return False

    def batch_fitness(self, dvs) -> np.ndarray:
        x = _as_rows(dvs, 4)
        n = x.size // 4
        f = np.empty(3 * n)
        if n:
            N.check(N.lib().pgx_constrained_batch_fitness(self.ctx.handle, N.HS71, 0, N.ptr(x), n, N.ptr(f)))
        return f

    def fitness(self, x) -> np.ndarray:
        x = np.asarray(x, dtype=np.float64)
        if x.size != 4:
            raise ValueError(f"A decision vector is incompatible with a problem of type '{self.get_name()}': the "
                             f"number of dimensions of the problem is 4, while the decision vector has a size of "
                             f"{x.size} (the two values should be equal)")
        return self.batch_fitness(x)


class unconstrain:
    """unconstrain{udp, method, weights} (src/problems/unconstrain.cpp) around a constrained GPU UDP: the inner
    batch fitness and every row's penalty ("death penalty", "kuri", "weighted", "ignore_c", "ignore_o";
    unconstrain::penalize, :130-225) in one GPU pass, the reference's values bit for bit. c_tol: the inner
    problem's constraint tolerances (pagmo's problem::set_c_tol; default 0). Constructor checks and messages as
    the reference's (:66-100)."""

    def __init__(self, udp, method: str = "death penalty", weights=(), c_tol=None):
        nc = udp.get_nec() + udp.get_nic() if hasattr(udp, "get_nec") else 0
        if nc == 0:
            raise ValueError(f"Unconstrain can only be applied to constrained problems, the instance of "
                             f"{udp.get_name()} is not one.")
        w = np.ascontiguousarray(np.asarray(weights, dtype=np.float64).reshape(-1))
        if w.size != nc and method == "weighted":
            raise ValueError(f"Length of weight vector is: {w.size} while the problem constraints are: {nc}")
        if method not in N.UNCONSTRAIN_METHODS:
            raise ValueError(f"The method {method} is not supported (did you misspell?)")
        if w.size != 0 and method != "weighted":
            raise ValueError(f"The weight vector needs to be empty to use the unconstrain method {method}")
        if not hasattr(udp, "kind") or udp.kind != N.HS71:
            raise NotImplementedError(f"unconstrain on the GPU: the inner problem must be a constrained GPU UDP "
                                      f"(hock_schittkowski_71), not {udp.get_name()}")
        self.inner, self.method, self.weights = udp, method, w
        self.c_tol = np.zeros(nc) if c_tol is None else np.ascontiguousarray(np.asarray(c_tol, dtype=np.float64))
        if self.c_tol.size != nc:  # problem::set_c_tol's checks (src/problem.cpp:620-636)
            raise ValueError(f"The tolerance vector size should be: {nc}, while a size of: {self.c_tol.size} was "
                             f"detected.")
        for i, t in enumerate(self.c_tol):
            if np.isnan(t):
                raise ValueError(f"The tolerance vector has a NaN value at the index {i}")
            if t < 0:
                raise ValueError(f"The tolerance vector has a negative value at the index {i}")
        self._desc = N.pgx_unconstrain(N.UNCONSTRAIN_METHODS[method], N.ptr(self.weights) if w.size else None,
                                       w.size, N.ptr(self.c_tol))

    def get_nx(self) -> int:
        return self.inner.get_nx()

    def get_nobj(self) -> int:
        return 1 if self.method == "ignore_o" else self.inner.get_nobj()

    def get_nf(self) -> int:
        return self.get_nobj()

    def get_bounds(self):
        return self.inner.get_bounds()

    def get_name(self) -> str:
        return self.inner.get_name() + " [unconstrained]"

    def get_thread_safety(self) -> str:
        return self.inner.get_thread_safety()

    def has_gradient(self) -> bool:
        return False

    def batch_fitness(self, dvs) -> np.ndarray:
        nx = self.get_nx()
        x = _as_rows(dvs, nx)
        n = x.size // nx
        f = np.empty(n * self.get_nobj())
        if n:
            N.check(N.lib().pgx_unconstrain_batch_fitness(self.inner.ctx.handle, self.inner.kind, self.inner.param,
                                                          C.byref(self._desc), N.ptr(x), n, N.ptr(f)))
        return f

    def fitness(self, x) -> np.ndarray:
        return self.batch_fitness(np.asarray(x, dtype=np.float64).reshape(1, -1))


class translate:
    """translate{udp, translation} (src/problems/translate.cpp): f(x) = inner(x - translation), bounds shifted by
    the translation; batch_fitness shifts the whole batch back and forwards it to the inner problem's batch_fitness
    (translate.cpp:118-146), so a GPU UDP inside stays a one-pass GPU evaluation."""

    def __init__(self, udp, translation):
        self.inner = udp
        self.translation = np.ascontiguousarray(np.asarray(translation, dtype=np.float64).reshape(-1))
        if self.translation.size != udp.get_nx():
            raise ValueError(f"Length of shift vector is: {self.translation.size} while the problem dimension is: "
                             f"{udp.get_nx()}")
        self.thread_safety = getattr(udp, "thread_safety", "basic")

    def get_nx(self) -> int:
        return self.inner.get_nx()

    def get_nobj(self) -> int:
        return self.inner.get_nobj()

    def get_nf(self) -> int:
        return self.inner.get_nf()

    def get_bounds(self):
        lb, ub = self.inner.get_bounds()
        return lb + self.translation, ub + self.translation

    def get_name(self) -> str:
        return self.inner.get_name() + " [translated]"

    def get_thread_safety(self) -> str:
        return self.thread_safety

    def has_gradient(self) -> bool:
        return self.inner.has_gradient() if hasattr(self.inner, "has_gradient") else hasattr(self.inner, "gradient")

    def _back(self, dvs) -> np.ndarray:
        x = _as_rows(dvs, self.get_nx()).reshape(-1, self.get_nx())
        return (x - self.translation).reshape(-1)

    def batch_fitness(self, dvs) -> np.ndarray:
        return self.inner.batch_fitness(self._back(dvs))

    def fitness(self, x) -> np.ndarray:
        return self.inner.fitness(np.asarray(x, dtype=np.float64) - self.translation)

    def gradient(self, x) -> np.ndarray:
        return self.inner.gradient(np.asarray(x, dtype=np.float64) - self.translation)

    def batch_gradient(self, dvs, with_fitness: bool = True):
        return self.inner.batch_gradient(self._back(dvs), with_fitness)


def from_kind(kind: int, param: int, context=None) -> _gpu_udp:
    return {N.RASTRIGIN: rastrigin, N.ROSENBROCK: rosenbrock, N.LENNARD_JONES: lennard_jones, N.ACKLEY: ackley,
            N.GRIEWANK: griewank, N.SCHWEFEL: schwefel}[kind](param, context)
