// gpu_bfe: a user-defined batch fitness evaluator (UDBFE) for pagmo::bfe
// that evaluates pagmo's own rastrigin, rosenbrock, lennard_jones, ackley,
// griewank, schwefel, zdt and dtlz UDPs (DTLZ4 excepted), the GPU UDPs of
// gpu_problems.hpp, and any of these inside pagmo's translate, on a GB300.
//
// A UDBFE is a callable vector_double(const problem &, const vector_double &)
// (include/pagmo/bfe.hpp:68-108). Like every UDBFE it leaves the fevals
// counter alone: pagmo::bfe::operator() checks the output and adds the
// number of evaluated vectors itself (src/bfe.cpp:91-110,
// src/batch_evaluators/member_bfe.cpp:42-44). Any other problem is rejected
// with std::invalid_argument (there is no CPU fallback).
#ifndef PAGMO_GB300_GPU_BFE_HPP
#define PAGMO_GB300_GPU_BFE_HPP

#include <cstdint>
#include <stdexcept>
#include <string>

#include <pagmo/bfe.hpp>
#include <pagmo/problem.hpp>
#include <pagmo/problems/ackley.hpp>
#include <pagmo/problems/dtlz.hpp>
#include <pagmo/problems/griewank.hpp>
#include <pagmo/problems/lennard_jones.hpp>
#include <pagmo/problems/rastrigin.hpp>
#include <pagmo/problems/rosenbrock.hpp>
#include <pagmo/problems/schwefel.hpp>
#include <pagmo/problems/hock_schittkowski_71.hpp>
#include <pagmo/problems/translate.hpp>
#include <pagmo/problems/unconstrain.hpp>
#include <pagmo/problems/zdt.hpp>
#include <pagmo/threading.hpp>
#include <pagmo/types.hpp>

#include "gpu_problems.hpp"
#include "pgx.hpp"

namespace pagmo_gb300
{

class gpu_bfe
{
public:
    explicit gpu_bfe(int device = 0) : m_device(device) {}

    pagmo::vector_double operator()(const pagmo::problem &p, const pagmo::vector_double &dvs) const
    {
        if (const auto *g = p.extract<gpu_rastrigin>()) return g->batch_fitness(dvs);
        if (const auto *g = p.extract<gpu_rosenbrock>()) return g->batch_fitness(dvs);
        if (const auto *g = p.extract<gpu_lennard_jones>()) return g->batch_fitness(dvs);
        if (const auto *g = p.extract<gpu_ackley>()) return g->batch_fitness(dvs);
        if (const auto *g = p.extract<gpu_griewank>()) return g->batch_fitness(dvs);
        if (const auto *g = p.extract<gpu_schwefel>()) return g->batch_fitness(dvs);
        if (const auto *g = p.extract<gpu_zdt>()) return g->batch_fitness(dvs);
        if (const auto *g = p.extract<gpu_dtlz>()) return g->batch_fitness(dvs);
        if (const auto *g = p.extract<gpu_hock_schittkowski_71>()) return g->batch_fitness(dvs);
        if (p.extract<pagmo::zdt>() || p.extract<pagmo::dtlz>()) return mo_fitness(p, dvs);
        if (p.extract<pagmo::hock_schittkowski_71>()) {
            const std::uint64_t n = dvs.size() / 4u; // pagmo::bfe checked divisibility
            pagmo::vector_double fvs(3u * n);
            if (n)
                check(pgx_constrained_batch_fitness(device_context(m_device), PGX_HS71, 0u, dvs.data(), n,
                                                    fvs.data()));
            return fvs;
        }
        if (const auto *u = p.extract<pagmo::unconstrain>()) {
            // unconstrain::batch_fitness (src/problems/unconstrain.cpp:245-266):
            // the inner problem's batch evaluation (on the GPU for a GPU UDP),
            // then pagmo's own penalty; its method and weights are private
            if (u->get_inner_problem().has_batch_fitness()) return u->batch_fitness(dvs);
            throw std::invalid_argument("Cannot use a gpu_bfe on '" + p.get_name()
                                        + "': wrap a GPU UDP with batch_fitness (gpu_hock_schittkowski_71) "
                                          "in the unconstrain");
        }
        if (const auto *t = p.extract<pagmo::translate>()) {
            // translate::batch_fitness (src/problems/translate.cpp:118-146): the
            // decision vectors shifted back, then the inner problem's evaluation
            const auto &tr = t->get_translation();
            const auto nx = tr.size();
            pagmo::vector_double back(dvs.size());
            for (std::size_t i = 0; i < dvs.size(); ++i) back[i] = dvs[i] - tr[i % nx];
            return (*this)(t->get_inner_problem(), back);
        }
        int kind = 0;
        std::uint64_t param = p.get_nx();
        if (p.extract<pagmo::rastrigin>()) {
            kind = PGX_RASTRIGIN;
        } else if (p.extract<pagmo::rosenbrock>()) {
            kind = PGX_ROSENBROCK;
        } else if (p.extract<pagmo::lennard_jones>()) {
            kind = PGX_LENNARD_JONES;
            param = (p.get_nx() + 6u) / 3u;
        } else if (p.extract<pagmo::ackley>()) {
            kind = PGX_ACKLEY;
        } else if (p.extract<pagmo::griewank>()) {
            kind = PGX_GRIEWANK;
        } else if (p.extract<pagmo::schwefel>()) {
            kind = PGX_SCHWEFEL;
        } else {
            throw std::invalid_argument("Cannot use a gpu_bfe on the problem '" + p.get_name()
                                        + "': only rastrigin, rosenbrock, lennard_jones, ackley, griewank, "
                                          "schwefel, zdt, dtlz and hock_schittkowski_71 are evaluated on the GPU");
        }
        const std::uint64_t n = dvs.size() / p.get_nx(); // pagmo::bfe checked divisibility
        pagmo::vector_double fvs(n);
        if (n) check(pgx_batch_fitness(device_context(m_device), kind, param, dvs.data(), n, fvs.data()));
        return fvs;
    }

    std::string get_name() const
    {
        return "GB300 batch fitness evaluator";
    }
    // pagmo's zdt and dtlz: the problem id comes from get_name() ("ZDT3",
    // zdt.cpp:164-167; "DTLZ2", dtlz.cpp:169-172), the parameters from the
    // dimensions. DTLZ4's alpha is not readable through pagmo's public
    // interface, so pagmo::dtlz{4, ...} is refused (gpu_dtlz carries it).
    pagmo::vector_double mo_fitness(const pagmo::problem &p, const pagmo::vector_double &dvs) const
    {
        pgx_mo_problem mp{};
        const std::string name = p.get_name();
        const bool is_zdt = p.extract<pagmo::zdt>() != nullptr;
        mp.kind = is_zdt ? PGX_ZDT : PGX_DTLZ;
        mp.prob_id = static_cast<std::uint32_t>(std::stoul(name.substr(is_zdt ? 3u : 4u)));
        if (is_zdt) {
            mp.param = mp.prob_id == 5u ? (p.get_nx() - 30u) / 5u + 1u : p.get_nx();
        } else {
            if (mp.prob_id == 4u)
                throw std::invalid_argument("Cannot use a gpu_bfe on pagmo's DTLZ4: its alpha is not exposed by "
                                            "the problem; use pagmo_gb300::gpu_dtlz{4, dim, fdim, alpha}");
            mp.param = p.get_nx();
            mp.fdim = p.get_nobj();
            mp.alpha = 100u;
        }
        const std::uint64_t n = dvs.size() / p.get_nx(); // pagmo::bfe checked divisibility
        pagmo::vector_double fvs(n * p.get_nobj());
        if (n) check(pgx_mo_batch_fitness(device_context(m_device), &mp, dvs.data(), n, fvs.data()));
        return fvs;
    }

    std::string get_extra_info() const
    {
        return "\tDevice: " + std::to_string(m_device) + "\n";
    }

    // callable from concurrent island threads: the library serialises work
    // per device, and the object itself is never modified
    pagmo::thread_safety get_thread_safety() const
    {
        return pagmo::thread_safety::basic;
    }

    template <typename Archive>
    void serialize(Archive &ar, unsigned)
    {
        ar &m_device;
    }

private:
    int m_device = 0;
};

} // namespace pagmo_gb300

// Registration with pagmo's Boost.Serialization machinery (include/pagmo/bfe.hpp:54-62):
// the key here, the implementation in one translation unit (pagmo_gb300/s11n_implement.hpp).
PAGMO_S11N_BFE_EXPORT_KEY(pagmo_gb300::gpu_bfe)

#endif
