// GPU-backed user-defined problems for pagmo: the rastrigin, rosenbrock,
// lennard_jones, ackley, griewank, schwefel, zdt and dtlz UDPs
// (src/problems/*.cpp) with the same dimensions, bounds, names and
// constructor errors, whose evaluations run on a GB300 through libpgx.
//
// Besides fitness/get_bounds (the UDP minimum, include/pagmo/problem.hpp:436-448)
// they provide batch_fitness, which member_bfe and default_bfe pick
// (src/batch_evaluators/default_bfe.cpp:53-58), gradient
// (src/problem.cpp:456-467; dense, nf = 1) and the batch extension
// batch_gradient. Thread safety is constant: evaluations only read the object.
#ifndef PAGMO_GB300_GPU_PROBLEMS_HPP
#define PAGMO_GB300_GPU_PROBLEMS_HPP

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include <pagmo/population.hpp>
#include <pagmo/problem.hpp>
#include <pagmo/threading.hpp>
#include <pagmo/types.hpp>

#include "pgx.hpp"

namespace pagmo_gb300
{

namespace detail
{

// Fitness, batch fitness, bounds and serialization of a GPU UDP. Problems
// whose reference UDP has no gradient (ackley, griewank, schwefel) stop
// here, so pagmo's has_gradient is false for them and problem::gradient
// raises not_implemented_error, as for the reference UDPs.
template <int Kind>
class gpu_udp_fitness
{
public:
    gpu_udp_fitness() = default;
    explicit gpu_udp_fitness(std::uint64_t param, int device = 0) : m_param(param), m_device(device)
    {
        check(pgx_problem_nx(Kind, param, &m_nx)); // the reference constructors' checks and messages
    }

    pagmo::vector_double fitness(const pagmo::vector_double &x) const
    {
        return batch_fitness(x);
    }

    pagmo::vector_double batch_fitness(const pagmo::vector_double &dvs) const
    {
        const std::uint64_t n = rows(dvs);
        pagmo::vector_double f(n);
        if (n) check(pgx_batch_fitness(device_context(m_device), Kind, m_param, dvs.data(), n, f.data()));
        return f;
    }

    std::pair<pagmo::vector_double, pagmo::vector_double> get_bounds() const
    {
        std::pair<pagmo::vector_double, pagmo::vector_double> b{pagmo::vector_double(m_nx),
                                                                pagmo::vector_double(m_nx)};
        check(pgx_problem_bounds(Kind, m_param, b.first.data(), b.second.data()));
        return b;
    }

    pagmo::thread_safety get_thread_safety() const
    {
        return pagmo::thread_safety::constant;
    }

    std::uint64_t param() const
    {
        return m_param;
    }

    template <typename Archive>
    void serialize(Archive &ar, unsigned)
    {
        ar &m_param;
        ar &m_nx;
        ar &m_device;
    }

protected:
    std::uint64_t rows(const pagmo::vector_double &dvs) const
    {
        if (m_nx == 0 || dvs.size() % m_nx)
            throw std::invalid_argument("Invalid argument for a batch fitness evaluation: the length of the vector "
                                        "representing the decision vectors, "
                                        + std::to_string(dvs.size())
                                        + ", is not an exact multiple of the dimension of the problem, "
                                        + std::to_string(m_nx));
        return dvs.size() / m_nx;
    }

    std::uint64_t m_param = 0;
    std::uint64_t m_nx = 0;
    int m_device = 0;
};

// A GPU UDP with the gradient hook (rastrigin, rosenbrock, lennard_jones).
template <int Kind>
class gpu_udp : public gpu_udp_fitness<Kind>
{
public:
    gpu_udp() = default;
    explicit gpu_udp(std::uint64_t param, int device = 0) : gpu_udp_fitness<Kind>(param, device) {}

    pagmo::vector_double gradient(const pagmo::vector_double &x) const
    {
        return batch_gradient(x).second;
    }

    // (fitness, gradient) of a whole batch in one GPU pass: n fitness values
    // and n * nx gradient entries, row-major.
    std::pair<pagmo::vector_double, pagmo::vector_double> batch_gradient(const pagmo::vector_double &dvs) const
    {
        const std::uint64_t n = this->rows(dvs);
        std::pair<pagmo::vector_double, pagmo::vector_double> out{pagmo::vector_double(n),
                                                                  pagmo::vector_double(n * this->m_nx)};
        if (n)
            check(pgx_batch_gradient(device_context(this->m_device), Kind, this->m_param, dvs.data(), n,
                                     out.first.data(), out.second.data()));
        return out;
    }
};

} // namespace detail

// rastrigin{dim}: f = 10 n + sum (x_i^2 - 10 cos(2 pi x_i)) on [-5.12, 5.12]^n.
class gpu_rastrigin : public detail::gpu_udp<PGX_RASTRIGIN>
{
public:
    explicit gpu_rastrigin(unsigned dim = 1u, int device = 0) : gpu_udp(dim, device) {}
    std::string get_name() const
    {
        return "Rastrigin Function";
    }
    pagmo::vector_double best_known() const
    {
        return pagmo::vector_double(m_nx, 0.);
    }
};

// rosenbrock{dim}: f = sum 100 (x_i^2 - x_{i+1})^2 + (x_i - 1)^2 on [-5, 10]^n.
class gpu_rosenbrock : public detail::gpu_udp<PGX_ROSENBROCK>
{
public:
    explicit gpu_rosenbrock(pagmo::vector_double::size_type dim = 2u, int device = 0) : gpu_udp(dim, device) {}
    std::string get_name() const
    {
        return "Multidimensional Rosenbrock Function";
    }
    pagmo::vector_double best_known() const
    {
        return pagmo::vector_double(m_nx, 1.);
    }
};

// lennard_jones{atoms}: 4 sum_{i<j} (r^-12 - r^-6), three coordinates pinned.
class gpu_lennard_jones : public detail::gpu_udp<PGX_LENNARD_JONES>
{
public:
    explicit gpu_lennard_jones(unsigned atoms = 3u, int device = 0) : gpu_udp(atoms, device) {}
    std::string get_name() const
    {
        return "Lennard Jones Cluster (" + std::to_string(m_param) + " atoms)";
    }
};

// ackley{dim}: -20 exp(-0.2 sqrt(sum x^2 / n)) - exp(sum cos(2 pi x) / n) + 20 + e on [-15, 30]^n
// (src/problems/ackley.cpp). Fitness only, as the reference.
class gpu_ackley : public detail::gpu_udp_fitness<PGX_ACKLEY>
{
public:
    explicit gpu_ackley(unsigned dim = 1u, int device = 0) : gpu_udp_fitness(dim, device) {}
    std::string get_name() const
    {
        return "Ackley Function";
    }
    pagmo::vector_double best_known() const
    {
        return pagmo::vector_double(m_nx, 0.);
    }
};

// griewank{dim}: sum x^2 / 4000 - prod cos(x_i / sqrt(i + 1)) + 1 on [-600, 600]^n
// (src/problems/griewank.cpp). Fitness only, as the reference.
class gpu_griewank : public detail::gpu_udp_fitness<PGX_GRIEWANK>
{
public:
    explicit gpu_griewank(unsigned dim = 1u, int device = 0) : gpu_udp_fitness(dim, device) {}
    std::string get_name() const
    {
        return "Griewank Function";
    }
    pagmo::vector_double best_known() const
    {
        return pagmo::vector_double(m_nx, 0.);
    }
};

// schwefel{dim}: 418.9828872724338 n - sum x sin(sqrt|x|) on [-500, 500]^n
// (src/problems/schwefel.cpp). Fitness only, as the reference.
class gpu_schwefel : public detail::gpu_udp_fitness<PGX_SCHWEFEL>
{
public:
    explicit gpu_schwefel(unsigned dim = 1u, int device = 0) : gpu_udp_fitness(dim, device) {}
    std::string get_name() const
    {
        return "Schwefel Function";
    }
    pagmo::vector_double best_known() const
    {
        return pagmo::vector_double(m_nx, 420.9687);
    }
};

namespace detail
{

// ZDT / DTLZ on the GPU: fitness vectors of nobj objectives, batch_fitness in
// pagmo's fvs layout (n rows of nobj), p_distance of a vector or the mean over
// a population (src/problems/zdt.cpp:179-224, src/problems/dtlz.cpp:131-163).
class gpu_mo_udp
{
public:
    gpu_mo_udp() = default;
    gpu_mo_udp(int kind, unsigned prob_id, std::uint64_t param, std::uint64_t fdim, unsigned alpha, int device)
        : m_device(device)
    {
        m_p.kind = kind;
        m_p.prob_id = prob_id;
        m_p.param = param;
        m_p.fdim = fdim;
        m_p.alpha = alpha;
        check(pgx_mo_problem_dims(&m_p, &m_nx, &m_nobj, &m_nix)); // the reference constructors' checks
    }
    pagmo::vector_double fitness(const pagmo::vector_double &x) const
    {
        return batch_fitness(x);
    }
    pagmo::vector_double batch_fitness(const pagmo::vector_double &dvs) const
    {
        const std::uint64_t n = rows(dvs);
        pagmo::vector_double f(n * m_nobj);
        if (n) check(pgx_mo_batch_fitness(device_context(m_device), &m_p, dvs.data(), n, f.data()));
        return f;
    }
    pagmo::vector_double::size_type get_nobj() const
    {
        return m_nobj;
    }
    std::pair<pagmo::vector_double, pagmo::vector_double> get_bounds() const
    {
        std::pair<pagmo::vector_double, pagmo::vector_double> b{pagmo::vector_double(m_nx),
                                                                pagmo::vector_double(m_nx)};
        check(pgx_mo_problem_bounds(&m_p, b.first.data(), b.second.data()));
        return b;
    }
    pagmo::thread_safety get_thread_safety() const
    {
        return pagmo::thread_safety::constant;
    }
    // p_distance of every row of a batch.
    pagmo::vector_double batch_p_distance(const pagmo::vector_double &dvs) const
    {
        const std::uint64_t n = rows(dvs);
        pagmo::vector_double out(n);
        if (n) check(pgx_mo_p_distance(device_context(m_device), &m_p, dvs.data(), n, out.data()));
        return out;
    }
    // Mean p_distance over the population, summed in row order as the reference does.
    double p_distance(const pagmo::population &pop) const
    {
        pagmo::vector_double flat;
        flat.reserve(pop.size() * m_nx);
        for (const auto &x : pop.get_x()) flat.insert(flat.end(), x.begin(), x.end());
        const auto d = batch_p_distance(flat);
        double c = 0.0;
        for (double v : d) c += v;
        return c / static_cast<double>(pop.size());
    }
    template <typename Archive>
    void serialize(Archive &ar, unsigned)
    {
        ar &m_p.kind;
        ar &m_p.prob_id;
        ar &m_p.param;
        ar &m_p.fdim;
        ar &m_p.alpha;
        ar &m_nx;
        ar &m_nobj;
        ar &m_nix;
        ar &m_device;
    }

protected:
    std::uint64_t rows(const pagmo::vector_double &dvs) const
    {
        if (m_nx == 0 || dvs.size() % m_nx)
            throw std::invalid_argument("Invalid argument for a batch fitness evaluation: the length of the vector "
                                        "representing the decision vectors, "
                                        + std::to_string(dvs.size())
                                        + ", is not an exact multiple of the dimension of the problem, "
                                        + std::to_string(m_nx));
        return dvs.size() / m_nx;
    }
    pgx_mo_problem m_p{};
    std::uint64_t m_nx = 0, m_nobj = 0, m_nix = 0;
    int m_device = 0;
};

} // namespace detail

// zdt{prob_id, param}: the six two-objective ZDT problems (src/problems/zdt.cpp);
// param is the dimension, except for ZDT5, whose 30 + 5 (param - 1) bits it counts.
class gpu_zdt : public detail::gpu_mo_udp
{
public:
    explicit gpu_zdt(unsigned prob_id = 1u, unsigned param = 30u, int device = 0)
        : gpu_mo_udp(PGX_ZDT, prob_id, param, 0u, 0u, device)
    {
    }
    std::string get_name() const
    {
        return "ZDT" + std::to_string(m_p.prob_id);
    }
    pagmo::vector_double::size_type get_nix() const
    {
        return m_nix;
    }
    using gpu_mo_udp::p_distance;
    // zdt.cpp:204-224 does not check the size of x: the metric of a vector of
    // another length is that of the same ZDT problem at that length.
    double p_distance(const pagmo::vector_double &x) const
    {
        if (x.size() == m_nx) return batch_p_distance(x)[0];
        if (m_p.prob_id == 5u) {
            if (x.size() < 30u) throw std::invalid_argument("a ZDT5 decision vector has at least 30 entries");
            const gpu_zdt other(5u, static_cast<unsigned>((x.size() - 30u) / 5u + 1u), m_device);
            return other.batch_p_distance(pagmo::vector_double(x.begin(), x.begin() + other.m_nx))[0];
        }
        return gpu_zdt(m_p.prob_id, static_cast<unsigned>(x.size()), m_device).batch_p_distance(x)[0];
    }
};

// dtlz{prob_id, dim, fdim, alpha}: the seven scalable DTLZ problems on [0, 1]^dim
// (src/problems/dtlz.cpp).
class gpu_dtlz : public detail::gpu_mo_udp
{
public:
    explicit gpu_dtlz(unsigned prob_id = 1u, pagmo::vector_double::size_type dim = 5u,
                      pagmo::vector_double::size_type fdim = 3u, unsigned alpha = 100u, int device = 0)
        : gpu_mo_udp(PGX_DTLZ, prob_id, dim, fdim, alpha, device)
    {
    }
    std::string get_name() const
    {
        return "DTLZ" + std::to_string(m_p.prob_id);
    }
    using gpu_mo_udp::p_distance;
    double p_distance(const pagmo::vector_double &x) const
    {
        // dtlz.cpp:156-163
        if (x.size() != m_nx)
            throw std::invalid_argument("The size of the decision vector should be " + std::to_string(m_nx)
                                        + " while " + std::to_string(x.size()) + " was detected");
        return batch_p_distance(x)[0];
    }
};

// hock_schittkowski_71: four variables in [1, 5], one objective, one equality
// and one inequality constraint (src/problems/hock_schittkowski_71.cpp:48-69);
// batch_fitness on the GPU (n rows of [f, ceq, cineq], the reference's values
// bit for bit). Inside pagmo's unconstrain, whose batch_fitness forwards to the
// inner problem's (src/problems/unconstrain.cpp:245-266), the evaluations run
// on the GPU. pagmo's gradient and hessians of this UDP are not provided.
class gpu_hock_schittkowski_71
{
public:
    explicit gpu_hock_schittkowski_71(int device = 0) : m_device(device) {}
    pagmo::vector_double fitness(const pagmo::vector_double &x) const
    {
        return batch_fitness(x);
    }
    pagmo::vector_double batch_fitness(const pagmo::vector_double &dvs) const
    {
        if (dvs.size() % 4u)
            throw std::invalid_argument("Invalid argument for a batch fitness evaluation: the length of the vector "
                                        "representing the decision vectors, "
                                        + std::to_string(dvs.size())
                                        + ", is not an exact multiple of the dimension of the problem, 4");
        const std::uint64_t n = dvs.size() / 4u;
        pagmo::vector_double f(3u * n);
        if (n) check(pgx_constrained_batch_fitness(device_context(m_device), PGX_HS71, 0u, dvs.data(), n, f.data()));
        return f;
    }
    std::pair<pagmo::vector_double, pagmo::vector_double> get_bounds() const
    {
        std::pair<pagmo::vector_double, pagmo::vector_double> b{pagmo::vector_double(4), pagmo::vector_double(4)};
        check(pgx_constrained_bounds(PGX_HS71, 0u, b.first.data(), b.second.data()));
        return b;
    }
    pagmo::vector_double::size_type get_nec() const
    {
        return 1u;
    }
    pagmo::vector_double::size_type get_nic() const
    {
        return 1u;
    }
    std::string get_name() const
    {
        return "Hock Schittkowski 71";
    }
    pagmo::thread_safety get_thread_safety() const
    {
        return pagmo::thread_safety::constant;
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

// Registration with pagmo's Boost.Serialization machinery (include/pagmo/problem.hpp:67-76):
// the keys here, the implementations in one translation unit (pagmo_gb300/s11n_implement.hpp).
PAGMO_S11N_PROBLEM_EXPORT_KEY(pagmo_gb300::gpu_rastrigin)
PAGMO_S11N_PROBLEM_EXPORT_KEY(pagmo_gb300::gpu_rosenbrock)
PAGMO_S11N_PROBLEM_EXPORT_KEY(pagmo_gb300::gpu_lennard_jones)
PAGMO_S11N_PROBLEM_EXPORT_KEY(pagmo_gb300::gpu_ackley)
PAGMO_S11N_PROBLEM_EXPORT_KEY(pagmo_gb300::gpu_griewank)
PAGMO_S11N_PROBLEM_EXPORT_KEY(pagmo_gb300::gpu_schwefel)
PAGMO_S11N_PROBLEM_EXPORT_KEY(pagmo_gb300::gpu_zdt)
PAGMO_S11N_PROBLEM_EXPORT_KEY(pagmo_gb300::gpu_dtlz)
PAGMO_S11N_PROBLEM_EXPORT_KEY(pagmo_gb300::gpu_hock_schittkowski_71)

#endif
