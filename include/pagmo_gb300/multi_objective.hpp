// NSGA-II survival on a GB300 with pagmo's signatures:
// fast_non_dominated_sorting, crowding_distance, select_best_N_mo and
// sort_population_mo (include/pagmo/utils/multi_objective.hpp:72-81;
// src/utils/multi_objective.cpp:200-465), and the survival block of
// nsga2::evolve (src/algorithms/nsga2.cpp:183-206) in one call. Every output
// is identical to the reference's: ranks, domination counts, the fronts in the
// reference's order, dom_list, crowding distances and index lists, including
// the order of ties, which the device sorts leave as the reference's std::sort
// (GNU libstdc++) leaves them.
#ifndef PAGMO_GB300_MULTI_OBJECTIVE_HPP
#define PAGMO_GB300_MULTI_OBJECTIVE_HPP

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include <pagmo/population.hpp>
#include <pagmo/types.hpp>
#include <pagmo/utils/multi_objective.hpp>

#include "pgx.hpp"

namespace pagmo_gb300
{

namespace detail
{

inline std::vector<double> flatten(const std::vector<pagmo::vector_double> &points, std::uint64_t &m)
{
    m = points.empty() ? 0u : points[0].size();
    std::vector<double> flat;
    flat.reserve(points.size() * m);
    for (const auto &p : points) {
        if (p.size() != m)
            throw std::invalid_argument("Different number of objectives found in input fitnesses: "
                                        + std::to_string(m) + " and " + std::to_string(p.size())
                                        + ". I cannot define dominance");
        flat.insert(flat.end(), p.begin(), p.end());
    }
    return flat;
}

} // namespace detail

inline pagmo::fnds_return_type fast_non_dominated_sorting(const std::vector<pagmo::vector_double> &points,
                                                          int device = 0)
{
    const std::uint64_t n = points.size();
    if (n < 2u)
        throw std::invalid_argument("At least two points are needed for fast_non_dominated_sorting: "
                                    + std::to_string(n) + " detected.");
    std::uint64_t m = 0;
    const auto flat = detail::flatten(points, m);
    pgx_context *ctx = device_context(device);
    std::vector<std::int32_t> rank(n), dc(n), off(n + 1), idx(n);
    std::int32_t nf = 0;
    check(pgx_fnds(ctx, flat.data(), n, m, rank.data(), dc.data(), off.data(), idx.data(), &nf));
    std::vector<std::int64_t> dl_off(n + 1);
    std::uint64_t total = 0;
    int st = pgx_fnds_dom_list(ctx, flat.data(), n, m, dl_off.data(), nullptr, 0, &total);
    if (st != PGX_OK && st != PGX_ERR_CAPACITY) check(st);
    std::vector<std::int32_t> dl_idx(total > 0 ? total : 1);
    check(pgx_fnds_dom_list(ctx, flat.data(), n, m, dl_off.data(), dl_idx.data(), dl_idx.size(), &total));

    std::vector<std::vector<pagmo::pop_size_t>> fronts(static_cast<size_t>(nf)), dom_list(n);
    for (std::int32_t f = 0; f < nf; ++f)
        fronts[f].assign(idx.begin() + off[f], idx.begin() + off[f + 1]);
    for (std::uint64_t i = 0; i < n; ++i)
        dom_list[i].assign(dl_idx.begin() + dl_off[i], dl_idx.begin() + dl_off[i + 1]);
    return std::make_tuple(std::move(fronts), std::move(dom_list),
                           std::vector<pagmo::pop_size_t>(dc.begin(), dc.end()),
                           std::vector<pagmo::pop_size_t>(rank.begin(), rank.end()));
}

inline pagmo::vector_double crowding_distance(const std::vector<pagmo::vector_double> &front, int device = 0)
{
    const std::uint64_t n = front.size();
    if (n < 2u)
        throw std::invalid_argument("A non dominated front must contain at least two points: " + std::to_string(n)
                                    + " detected.");
    const std::uint64_t m = front[0].size();
    if (m < 2u)
        throw std::invalid_argument("Points in the non dominated front must contain at least two objectives: "
                                    + std::to_string(m) + " detected.");
    for (const auto &p : front)
        if (p.size() != m)
            throw std::invalid_argument("A non dominated front must contain points of uniform dimensionality. Some "
                                        "different sizes were instead detected.");
    std::uint64_t mm = 0;
    const auto flat = detail::flatten(front, mm);
    pagmo::vector_double out(n);
    check(pgx_crowding_distance(device_context(device), flat.data(), n, m, out.data()));
    return out;
}

// select_best_N_mo: the best N individuals (whole fronts, then the critical
// front by descending crowding distance).
inline std::vector<pagmo::pop_size_t> select_best_N_mo(const std::vector<pagmo::vector_double> &points,
                                                       pagmo::pop_size_t N, int device = 0)
{
    const std::uint64_t n = points.size();
    if (N == 0u || n == 0u) return {};
    if (n == 1u) return {0u};
    std::uint64_t m = 0;
    const auto flat = detail::flatten(points, m);
    std::vector<std::int32_t> out(N < n ? N : n);
    std::uint64_t cnt = 0;
    check(pgx_select_best_n_mo(device_context(device), flat.empty() ? nullptr : flat.data(), n, m, N, out.data(),
                               &cnt));
    return std::vector<pagmo::pop_size_t>(out.begin(), out.begin() + static_cast<std::ptrdiff_t>(cnt));
}

// sort_population_mo: the individuals ordered by (non-domination rank,
// descending crowding distance).
inline std::vector<pagmo::pop_size_t> sort_population_mo(const std::vector<pagmo::vector_double> &points,
                                                         int device = 0)
{
    const std::uint64_t n = points.size();
    if (n == 0u) return {};
    if (n == 1u) return {0u};
    std::uint64_t m = 0;
    const auto flat = detail::flatten(points, m);
    std::vector<std::int32_t> out(n);
    check(pgx_sort_population_mo(device_context(device), flat.empty() ? nullptr : flat.data(), n, m, out.data()));
    return std::vector<pagmo::pop_size_t>(out.begin(), out.end());
}

// The survival block of one NSGA-II generation: non-domination ranks, the
// fronts and every individual's crowding distance within its front.
struct nsga2_survival_result {
    std::vector<std::vector<pagmo::pop_size_t>> fronts;
    std::vector<pagmo::pop_size_t> rank;
    pagmo::vector_double crowding;
};

inline nsga2_survival_result nsga2_survival(const std::vector<pagmo::vector_double> &points, int device = 0)
{
    const std::uint64_t n = points.size();
    if (n < 2u)
        throw std::invalid_argument("At least two points are needed for fast_non_dominated_sorting: "
                                    + std::to_string(n) + " detected.");
    std::uint64_t m = 0;
    const auto flat = detail::flatten(points, m);
    std::vector<std::int32_t> rank(n), dc(n), off(n + 1), idx(n);
    std::int32_t nf = 0;
    nsga2_survival_result r;
    r.crowding.resize(n);
    check(pgx_nsga2_survival(device_context(device), flat.data(), n, m, rank.data(), dc.data(), off.data(),
                             idx.data(), &nf, r.crowding.data()));
    r.fronts.resize(static_cast<size_t>(nf));
    for (std::int32_t f = 0; f < nf; ++f) r.fronts[f].assign(idx.begin() + off[f], idx.begin() + off[f + 1]);
    r.rank.assign(rank.begin(), rank.end());
    return r;
}

namespace detail
{
// The points row-major, after hypervolume's construction and dimension checks
// (src/utils/hypervolume.cpp:406-449).
inline std::vector<double> hv_rows(const std::vector<pagmo::vector_double> &points, const pagmo::vector_double &ref)
{
    if (points.empty()) throw std::invalid_argument("Point set cannot be empty.");
    const auto m = points[0].size();
    if (m <= 1u) throw std::invalid_argument("Points of dimension > 1 required.");
    std::vector<double> flat;
    flat.reserve(points.size() * m);
    for (const auto &p : points) {
        if (p.size() != m) throw std::invalid_argument("All point set dimensions must be equal.");
        flat.insert(flat.end(), p.begin(), p.end());
    }
    if (ref.size() != m)
        throw std::invalid_argument("Point set dimensions and reference point dimension must be equal.");
    return flat;
}
} // namespace detail

// hypervolume(points).compute(ref) (src/utils/hypervolume.cpp:203-228) on the
// GPU for 2 to 16 objectives (hv2d / hv3d's value, hvwfg's bit for bit from 4
// objectives on), with the reference's checks and messages; more than 16
// objectives throw pagmo::not_implemented_error.
inline double hypervolume_compute(const std::vector<pagmo::vector_double> &points, const pagmo::vector_double &ref,
                                  int device = 0)
{
    const auto flat = detail::hv_rows(points, ref);
    double out = 0.0;
    check(pgx_hypervolume(device_context(device), flat.data(), points.size(), ref.size(), ref.data(), &out));
    return out;
}

// hypervolume(points).exclusive(p_idx, ref) (hypervolume.cpp:249-272).
inline double hypervolume_exclusive(const std::vector<pagmo::vector_double> &points, unsigned p_idx,
                                    const pagmo::vector_double &ref, int device = 0)
{
    const auto flat = detail::hv_rows(points, ref);
    double out = 0.0;
    check(pgx_hypervolume_exclusive(device_context(device), flat.data(), points.size(), ref.size(), ref.data(), p_idx,
                                    &out));
    return out;
}

// hypervolume(points).contributions(ref) (hypervolume.cpp:293-320), by
// hvwfg's limit sets.
inline std::vector<double> hypervolume_contributions(const std::vector<pagmo::vector_double> &points,
                                                     const pagmo::vector_double &ref, int device = 0)
{
    const auto flat = detail::hv_rows(points, ref);
    std::vector<double> out(points.size());
    check(pgx_hypervolume_contributions(device_context(device), flat.data(), points.size(), ref.size(), ref.data(),
                                        out.data()));
    return out;
}

// hypervolume(points).least_contributor(ref) / greatest_contributor(ref)
// (hypervolume.cpp:333-401).
inline unsigned long long hypervolume_least_contributor(const std::vector<pagmo::vector_double> &points,
                                                        const pagmo::vector_double &ref, int device = 0)
{
    const auto flat = detail::hv_rows(points, ref);
    std::uint64_t idx = 0;
    check(pgx_hypervolume_extreme_contributor(device_context(device), flat.data(), points.size(), ref.size(),
                                              ref.data(), 0, &idx));
    return idx;
}

inline unsigned long long hypervolume_greatest_contributor(const std::vector<pagmo::vector_double> &points,
                                                           const pagmo::vector_double &ref, int device = 0)
{
    const auto flat = detail::hv_rows(points, ref);
    std::uint64_t idx = 0;
    check(pgx_hypervolume_extreme_contributor(device_context(device), flat.data(), points.size(), ref.size(),
                                              ref.data(), 1, &idx));
    return idx;
}

// pagmo::hypervolume's interface (include/pagmo/utils/hypervolume.hpp:63-200)
// with every query on the GPU: the constructors' checks and messages
// (src/utils/hypervolume.cpp:46-80, 406-432), refpoint, get_points, compute,
// exclusive, contributions, least_contributor, greatest_contributor. The
// algorithm overloads (taking an hv_algorithm) are not provided: the GPU picks
// hv2d / hv3d / hvwfg as the reference's get_best_* do. The queries always
// check the reference point, whatever the verify flag; copy_points has no
// effect (the points are always copied to the device).
class hypervolume
{
public:
    hypervolume() = default;
    explicit hypervolume(const std::vector<pagmo::vector_double> &points, bool verify = true)
        : m_points(points), m_verify(verify)
    {
        if (m_verify) verify_after_construct();
    }
    explicit hypervolume(const pagmo::population &pop, bool verify = false) : m_verify(verify)
    {
        if (pop.get_problem().get_nc() > 0u)
            throw std::invalid_argument("The problem of the population is not unconstrained."
                                        "Only unconstrained populations can be used to construct hypervolume objects.");
        if (pop.get_problem().get_nobj() < 2u)
            throw std::invalid_argument("The problem of the population is not multiobjective."
                                        "Only multi-objective populations can be used to construct hypervolume "
                                        "objects.");
        m_points = pop.get_f();
        if (m_verify) verify_after_construct();
    }
    void set_copy_points(bool c)
    {
        m_copy_points = c;
    }
    bool get_copy_points() const
    {
        return m_copy_points;
    }
    void set_verify(bool v)
    {
        m_verify = v;
    }
    bool get_verify() const
    {
        return m_verify;
    }
    pagmo::vector_double refpoint(double offset = 0.0) const
    {
        if (m_points.empty()) return {};
        pagmo::vector_double r(m_points[0]);
        for (std::size_t k = 0; k < r.size(); ++k)
            for (std::size_t i = 1; i < m_points.size(); ++i) r[k] = std::max(r[k], m_points[i][k]);
        for (auto &c : r) c += offset;
        return r;
    }
    const std::vector<pagmo::vector_double> &get_points() const
    {
        return m_points;
    }
    double compute(const pagmo::vector_double &r) const
    {
        return hypervolume_compute(m_points, r, m_device);
    }
    double exclusive(unsigned p_idx, const pagmo::vector_double &r) const
    {
        return hypervolume_exclusive(m_points, p_idx, r, m_device);
    }
    std::vector<double> contributions(const pagmo::vector_double &r) const
    {
        return hypervolume_contributions(m_points, r, m_device);
    }
    unsigned long long least_contributor(const pagmo::vector_double &r) const
    {
        return hypervolume_least_contributor(m_points, r, m_device);
    }
    unsigned long long greatest_contributor(const pagmo::vector_double &r) const
    {
        return hypervolume_greatest_contributor(m_points, r, m_device);
    }
    // the GPU the queries run on (default 0)
    void set_device(int device)
    {
        m_device = device;
    }

private:
    void verify_after_construct() const
    {
        if (m_points.empty()) throw std::invalid_argument("Point set cannot be empty.");
        const auto m = m_points[0].size();
        if (m <= 1u) throw std::invalid_argument("Points of dimension > 1 required.");
        for (const auto &p : m_points)
            if (p.size() != m) throw std::invalid_argument("All point set dimensions must be equal.");
        for (const auto &p : m_points)
            for (double v : p)
                if (std::isnan(v))
                    throw std::invalid_argument("A nan value has been encountered in the hypervolume points. Cannot "
                                                "construct the hypervolume object");
    }

    std::vector<pagmo::vector_double> m_points;
    bool m_copy_points = true;
    bool m_verify = false;
    int m_device = 0;
};

} // namespace pagmo_gb300

#endif
