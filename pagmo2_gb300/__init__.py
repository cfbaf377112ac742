"""GB300-native batch evaluation for pagmo.

The compute path is libpgx.so (hand-written sm_103a CUDA behind the C ABI of
include/pgx.h). This package is its Python host side, mirroring pagmo's
plugin interface for the batch-fitness path:

  problems:         rastrigin, rosenbrock, lennard_jones (GPU UDPs with
                    batch_fitness, gradient and batch_gradient); ackley,
                    griewank, schwefel (batch_fitness; no gradient, as in
                    the reference); zdt, dtlz (multi-objective batch_fitness
                    and p_distance); hock_schittkowski_71 (constrained) and
                    the unconstrain meta-problem around it; translate
  batch_evaluators: gpu_bfe (the UDBFE) and a bfe/problem pair reproducing
                    pagmo's input/output checks and fevals accounting
  multi_objective:  fast_non_dominated_sorting, crowding_distance,
                    nsga2_survival, select_best_N_mo, sort_population_mo,
                    hypervolume (2 to 16 objectives: compute, exclusive,
                    contributions, least / greatest contributor)
  algorithms:       gpu_mbh (monotonic basin hopping with gradient descent on
                    every individual of a batch at once)
  workloads:        seeded synthetic inputs
"""
from ._native import Context, default_context  # noqa: F401
from .algorithms import gpu_mbh  # noqa: F401
from .batch_evaluators import bfe, gpu_bfe, problem  # noqa: F401
from .multi_objective import (crowding_distance, fast_non_dominated_sorting, hypervolume,  # noqa: F401
                              nsga2_survival, select_best_N_mo, sort_population_mo)
from .problems import (ackley, dtlz, griewank, hock_schittkowski_71, lennard_jones, rastrigin,  # noqa: F401
                       rosenbrock, schwefel, translate, unconstrain, zdt)
