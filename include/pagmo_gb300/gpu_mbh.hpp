// gpu_mbh: a pagmo user-defined algorithm (UDA) that refines every individual
// of a population at once on a GB300 (pgx_refine_batch): monotonic basin
// hopping, the scheme of pagmo's mbh (src/algorithms/mbh.cpp:102-200), with a
// projected-gradient descent driven by the batched adjoint as the inner local
// optimiser, and each individual as its own chain (mbh perturbs the whole
// population and accepts it when its best improves).
//
// Problems: pagmo's rastrigin, rosenbrock and lennard_jones, and the GPU UDPs
// gpu_rastrigin, gpu_rosenbrock, gpu_lennard_jones; anything else is rejected
// with std::invalid_argument (there is no CPU fallback). An individual's
// decision vector and fitness change only when its chain found a lower
// fitness. The problem's fevals counter grows by the evaluations made (each is
// one fitness and one gradient evaluation; pagmo offers no way to add to the
// gevals counter from outside a problem).
#ifndef PAGMO_GB300_GPU_MBH_HPP
#define PAGMO_GB300_GPU_MBH_HPP

#include <cstdint>
#include <stdexcept>
#include <string>

#include <pagmo/algorithm.hpp>
#include <pagmo/population.hpp>
#include <pagmo/problem.hpp>
#include <pagmo/problems/lennard_jones.hpp>
#include <pagmo/problems/rastrigin.hpp>
#include <pagmo/problems/rosenbrock.hpp>
#include <pagmo/types.hpp>

#include "gpu_problems.hpp"
#include "pgx.hpp"

namespace pagmo_gb300
{

class gpu_mbh
{
public:
    // hops: at most this many trials per individual; stop: trials in a row
    // without improvement that end an individual's chain (mbh's stop); steps:
    // descent steps per trial; perturb: half-width of the perturbation as a
    // fraction of (ub - lb), in ]0, 1] (mbh's perturb); step0 / step_min: first
    // and smallest descent step in box-scaled units; seed: the perturbations
    // are a function of (seed, individual, trial, coordinate).
    explicit gpu_mbh(unsigned hops = 10u, unsigned stop = 5u, unsigned steps = 20u, double perturb = 0.01,
                     double step0 = 0.05, double step_min = 1e-8, unsigned seed = 0u, int device = 0)
        : m_device(device)
    {
        if (!(perturb > 0.0 && perturb <= 1.0))
            throw std::invalid_argument("The perturbation must be in ]0,1], while a value of "
                                        + std::to_string(perturb) + " was detected.");
        m_p.hops = hops;
        m_p.stop = stop;
        m_p.steps = steps;
        m_p.perturb = perturb;
        m_p.step0 = step0;
        m_p.step_min = step_min;
        m_p.seed = seed;
    }

    pagmo::population evolve(pagmo::population pop) const
    {
        const auto &prob = pop.get_problem();
        int kind = 0;
        std::uint64_t param = prob.get_nx();
        if (prob.extract<pagmo::rastrigin>() || prob.extract<gpu_rastrigin>()) {
            kind = PGX_RASTRIGIN;
        } else if (prob.extract<pagmo::rosenbrock>() || prob.extract<gpu_rosenbrock>()) {
            kind = PGX_ROSENBROCK;
        } else if (prob.extract<pagmo::lennard_jones>() || prob.extract<gpu_lennard_jones>()) {
            kind = PGX_LENNARD_JONES;
            param = (prob.get_nx() + 6u) / 3u;
        } else {
            throw std::invalid_argument("Cannot use gpu_mbh on the problem '" + prob.get_name()
                                        + "': only rastrigin, rosenbrock and lennard_jones are refined on the GPU");
        }
        const auto np = pop.size();
        if (np == 0u) return pop;
        const auto nx = prob.get_nx();
        pagmo::vector_double x(np * nx), f(np);
        for (decltype(pop.size()) i = 0; i < np; ++i)
            std::copy(pop.get_x()[i].begin(), pop.get_x()[i].end(), x.begin() + static_cast<std::ptrdiff_t>(i * nx));
        std::uint64_t evals = 0;
        check(pgx_refine_batch(device_context(m_device), kind, param, &m_p, x.data(), np, f.data(), &evals));
        prob.increment_fevals(evals);
        for (decltype(pop.size()) i = 0; i < np; ++i) {
            if (f[i] < pop.get_f()[i][0]) {
                pop.set_xf(i, pagmo::vector_double(x.begin() + static_cast<std::ptrdiff_t>(i * nx),
                                                   x.begin() + static_cast<std::ptrdiff_t>((i + 1u) * nx)),
                           pagmo::vector_double{f[i]});
            }
        }
        ++m_p.seed; // the next call perturbs differently, as a seeded pagmo UDA does
        return pop;
    }

    void set_seed(unsigned seed)
    {
        m_p.seed = seed;
    }

    std::string get_name() const
    {
        return "MBH with projected-gradient descent, every individual at once (GB300)";
    }

    std::string get_extra_info() const
    {
        return "\tTrials per individual: " + std::to_string(m_p.hops) + "\n\tStop: " + std::to_string(m_p.stop)
               + "\n\tDescent steps: " + std::to_string(m_p.steps) + "\n\tPerturbation: "
               + std::to_string(m_p.perturb) + "\n\tDevice: " + std::to_string(m_device) + "\n";
    }

    template <typename Archive>
    void serialize(Archive &ar, unsigned)
    {
        ar &m_p.hops;
        ar &m_p.stop;
        ar &m_p.steps;
        ar &m_p.perturb;
        ar &m_p.step0;
        ar &m_p.step_min;
        ar &m_p.seed;
        ar &m_device;
    }

private:
    mutable pgx_refine_params m_p{};
    int m_device = 0;
};

} // namespace pagmo_gb300

// Registration with pagmo's Boost.Serialization machinery (include/pagmo/algorithm.hpp):
// the key here, the implementation in one translation unit (pagmo_gb300/s11n_implement.hpp).
PAGMO_S11N_ALGORITHM_EXPORT_KEY(pagmo_gb300::gpu_mbh)

#endif
