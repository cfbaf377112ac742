// NSGA-II survival on a GB300 with pagmo's signatures:
// fast_non_dominated_sorting and crowding_distance
// (include/pagmo/utils/multi_objective.hpp:72,75; src/utils/multi_objective.cpp:200-315),
// and the survival block of nsga2::evolve (src/algorithms/nsga2.cpp:183-206)
// in one call. Ranks, domination counts, the fronts (in the reference's
// order) and dom_list are identical to the reference's; crowding distances
// too, except that equal objective values are ordered as a stable sort would
// order them (the reference's std::sort leaves that order unspecified).
#ifndef PAGMO_GB300_MULTI_OBJECTIVE_HPP
#define PAGMO_GB300_MULTI_OBJECTIVE_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

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

} // namespace pagmo_gb300

#endif
