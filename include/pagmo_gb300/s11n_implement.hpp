// Include in exactly one translation unit of a program that serializes
// pagmo objects holding the GB300 plug-ins (islands, archipelagos,
// problems or bfes saved with Boost.Serialization): it instantiates the
// registrations whose keys gpu_bfe.hpp, gpu_problems.hpp and gpu_mbh.hpp declare, as
// pagmo's own PAGMO_S11N_*_IMPLEMENT macros do for its built-in plug-ins.
#ifndef PAGMO_GB300_S11N_IMPLEMENT_HPP
#define PAGMO_GB300_S11N_IMPLEMENT_HPP

#include "gpu_bfe.hpp"
#include "gpu_mbh.hpp"
#include "gpu_problems.hpp"

PAGMO_S11N_BFE_IMPLEMENT(pagmo_gb300::gpu_bfe)
PAGMO_S11N_ALGORITHM_IMPLEMENT(pagmo_gb300::gpu_mbh)
PAGMO_S11N_PROBLEM_IMPLEMENT(pagmo_gb300::gpu_rastrigin)
PAGMO_S11N_PROBLEM_IMPLEMENT(pagmo_gb300::gpu_rosenbrock)
PAGMO_S11N_PROBLEM_IMPLEMENT(pagmo_gb300::gpu_lennard_jones)
PAGMO_S11N_PROBLEM_IMPLEMENT(pagmo_gb300::gpu_ackley)
PAGMO_S11N_PROBLEM_IMPLEMENT(pagmo_gb300::gpu_griewank)
PAGMO_S11N_PROBLEM_IMPLEMENT(pagmo_gb300::gpu_schwefel)
PAGMO_S11N_PROBLEM_IMPLEMENT(pagmo_gb300::gpu_zdt)
PAGMO_S11N_PROBLEM_IMPLEMENT(pagmo_gb300::gpu_dtlz)
PAGMO_S11N_PROBLEM_IMPLEMENT(pagmo_gb300::gpu_hock_schittkowski_71)

#endif
