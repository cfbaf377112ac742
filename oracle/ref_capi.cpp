// C entry points over the reference's own compiled sources (pagmo 2.19.1),
// used only by the test suite and by the CPU leg of the benchmark to run the
// unmodified reference implementation of the batch-evaluation path.
//
// Every function catches exceptions and returns a status (0 = ok, 1 = the
// reference threw std::invalid_argument, 2 = any other exception); the
// message of the last error is available from ref_last_error().
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <pagmo/batch_evaluators/thread_bfe.hpp>
#include <pagmo/bfe.hpp>
#include <pagmo/problem.hpp>
#include <pagmo/problems/ackley.hpp>
#include <pagmo/problems/dtlz.hpp>
#include <pagmo/problems/griewank.hpp>
#include <pagmo/problems/hock_schittkowski_71.hpp>
#include <pagmo/problems/lennard_jones.hpp>
#include <pagmo/problems/rastrigin.hpp>
#include <pagmo/problems/rosenbrock.hpp>
#include <pagmo/problems/schwefel.hpp>
#include <pagmo/problems/unconstrain.hpp>
#include <pagmo/problems/zdt.hpp>
#include <pagmo/utils/hv_algos/hv_hvwfg.hpp>
#include <pagmo/utils/hypervolume.hpp>
#include <pagmo/utils/multi_objective.hpp>

namespace
{
thread_local std::string g_err;

pagmo::problem make_problem(int kind, std::uint64_t param)
{
    switch (kind) {
        case 1:
            return pagmo::problem{pagmo::rastrigin{static_cast<unsigned>(param)}};
        case 2:
            return pagmo::problem{pagmo::rosenbrock{static_cast<pagmo::vector_double::size_type>(param)}};
        case 3:
            return pagmo::problem{pagmo::lennard_jones{static_cast<unsigned>(param)}};
        case 4:
            return pagmo::problem{pagmo::ackley{static_cast<unsigned>(param)}};
        case 5:
            return pagmo::problem{pagmo::griewank{static_cast<unsigned>(param)}};
        case 6:
            return pagmo::problem{pagmo::schwefel{static_cast<unsigned>(param)}};
        default:
            throw std::invalid_argument("unknown problem kind " + std::to_string(kind));
    }
}

// family 7: pagmo::zdt{prob_id, param}; family 8: pagmo::dtlz{prob_id, dim, fdim, alpha}.
pagmo::problem make_mo_problem(int family, unsigned prob_id, std::uint64_t param, std::uint64_t fdim, unsigned alpha)
{
    if (family == 7) return pagmo::problem{pagmo::zdt{prob_id, static_cast<unsigned>(param)}};
    if (family == 8)
        return pagmo::problem{pagmo::dtlz{prob_id, static_cast<pagmo::vector_double::size_type>(param),
                                          static_cast<pagmo::vector_double::size_type>(fdim), alpha}};
    throw std::invalid_argument("unknown multi-objective family " + std::to_string(family));
}

template <typename F>
int guard(F &&f)
{
    try {
        f();
        return 0;
    } catch (const std::invalid_argument &e) {
        g_err = e.what();
        return 1;
    } catch (const std::exception &e) {
        g_err = e.what();
        return 2;
    }
}

std::vector<pagmo::vector_double> rows(const double *p, std::uint64_t n, std::uint64_t m)
{
    std::vector<pagmo::vector_double> out(n, pagmo::vector_double(m));
    for (std::uint64_t i = 0; i < n; ++i)
        for (std::uint64_t k = 0; k < m; ++k) out[i][k] = p[i * m + k];
    return out;
}
} // namespace

extern "C" {

const char *ref_last_error(void)
{
    return g_err.c_str();
}

// bfe{thread_bfe{}}(problem{udp}, dvs): the reference's multi-threaded batch path.
// fevals_out (nullable) receives the caller-side fevals counter after the call.
int ref_thread_bfe(int kind, std::uint64_t param, const double *dvs, std::uint64_t n_dvs, std::uint64_t nx,
                   double *fvs, std::uint64_t *fevals_out)
{
    return guard([&] {
        auto p = make_problem(kind, param);
        pagmo::bfe b{pagmo::thread_bfe{}};
        pagmo::vector_double in(dvs, dvs + n_dvs * nx);
        auto out = b(p, in);
        std::memcpy(fvs, out.data(), out.size() * sizeof(double));
        if (fevals_out) *fevals_out = p.get_fevals();
    });
}

// The decision vectors as the vector_double a pagmo algorithm hands its bfe,
// loaded once so that timing the evaluation does not time building it.
namespace
{
pagmo::vector_double g_loaded;
}

int ref_load_dvs(const double *dvs, std::uint64_t n_total)
{
    return guard([&] { g_loaded.assign(dvs, dvs + n_total); });
}

// bfe{thread_bfe{}}(problem{udp}, loaded dvs).
int ref_thread_bfe_loaded(int kind, std::uint64_t param, double *fvs)
{
    return guard([&] {
        auto p = make_problem(kind, param);
        pagmo::bfe b{pagmo::thread_bfe{}};
        auto out = b(p, g_loaded);
        std::memcpy(fvs, out.data(), out.size() * sizeof(double));
    });
}

// problem::gradient over the loaded rows on `threads` std::threads (pagmo has
// no batch gradient: this is the per-row API a user would parallelise).
int ref_gradient_loaded(int kind, std::uint64_t param, double *grads, int threads)
{
    return guard([&] {
        auto p = make_problem(kind, param);
        const std::uint64_t nx = p.get_nx(), n = g_loaded.size() / nx;
        const std::uint64_t nt = static_cast<std::uint64_t>(threads > 0 ? threads : 1);
        std::vector<std::thread> pool;
        std::vector<std::exception_ptr> errs(nt);
        for (std::uint64_t t = 0; t < nt; ++t) {
            pool.emplace_back([&, t]() {
                try {
                    pagmo::vector_double x(nx);
                    for (std::uint64_t i = t * n / nt; i < (t + 1) * n / nt; ++i) {
                        std::memcpy(x.data(), g_loaded.data() + i * nx, nx * sizeof(double));
                        const auto g = p.gradient(x);
                        std::memcpy(grads + i * nx, g.data(), nx * sizeof(double));
                    }
                } catch (...) {
                    errs[t] = std::current_exception();
                }
            });
        }
        for (auto &th : pool) th.join();
        for (auto &e : errs)
            if (e) std::rethrow_exception(e);
    });
}

// Serial problem::fitness over rows (the per-call path).
int ref_fitness_rows(int kind, std::uint64_t param, const double *dvs, std::uint64_t n_dvs, std::uint64_t nx,
                     double *fvs)
{
    return guard([&] {
        auto p = make_problem(kind, param);
        pagmo::vector_double x(nx);
        for (std::uint64_t i = 0; i < n_dvs; ++i) {
            std::memcpy(x.data(), dvs + i * nx, nx * sizeof(double));
            fvs[i] = p.fitness(x)[0];
        }
    });
}

// Serial problem::gradient over rows (rastrigin and rosenbrock provide one).
int ref_gradient_rows(int kind, std::uint64_t param, const double *dvs, std::uint64_t n_dvs, std::uint64_t nx,
                      double *grads)
{
    return guard([&] {
        auto p = make_problem(kind, param);
        pagmo::vector_double x(nx);
        for (std::uint64_t i = 0; i < n_dvs; ++i) {
            std::memcpy(x.data(), dvs + i * nx, nx * sizeof(double));
            auto g = p.gradient(x);
            std::memcpy(grads + i * nx, g.data(), nx * sizeof(double));
        }
    });
}

// problem::get_bounds of the reference UDP.
int ref_bounds(int kind, std::uint64_t param, double *lb, double *ub)
{
    return guard([&] {
        auto p = make_problem(kind, param);
        auto b = p.get_bounds();
        std::memcpy(lb, b.first.data(), b.first.size() * sizeof(double));
        std::memcpy(ub, b.second.data(), b.second.size() * sizeof(double));
    });
}

// hypervolume(points, true).compute(ref) (src/utils/hypervolume.cpp:203-228):
// errors come back as status 1 with the reference's message.
int ref_hypervolume(const double *pts, std::uint64_t n, std::uint64_t m, const double *r, double *out)
{
    return guard([&] {
        pagmo::hypervolume hv(rows(pts, n, m), true);
        *out = hv.compute(pagmo::vector_double(r, r + m));
    });
}

// hypervolume(points, true).exclusive(p_idx, ref), .contributions(ref),
// .least_contributor(ref), .greatest_contributor(ref)
// (src/utils/hypervolume.cpp:249-401), each with the algorithm the reference
// picks for the dimension; with wfg != 0, hvwfg() given explicitly.
int ref_hv_exclusive(const double *pts, std::uint64_t n, std::uint64_t m, const double *r, std::uint64_t p_idx,
                     double *out)
{
    return guard([&] {
        pagmo::hypervolume hv(rows(pts, n, m), true);
        *out = hv.exclusive(static_cast<unsigned>(p_idx), pagmo::vector_double(r, r + m));
    });
}

int ref_hv_contributions(const double *pts, std::uint64_t n, std::uint64_t m, const double *r, int wfg, double *out)
{
    return guard([&] {
        pagmo::hypervolume hv(rows(pts, n, m), true);
        const pagmo::vector_double rv(r, r + m);
        pagmo::hvwfg algo;
        const auto c = wfg ? hv.contributions(rv, algo) : hv.contributions(rv);
        std::copy(c.begin(), c.end(), out);
    });
}

int ref_hv_extreme(const double *pts, std::uint64_t n, std::uint64_t m, const double *r, int greatest,
                   std::uint64_t *idx)
{
    return guard([&] {
        pagmo::hypervolume hv(rows(pts, n, m), true);
        const pagmo::vector_double rv(r, r + m);
        *idx = greatest ? hv.greatest_contributor(rv) : hv.least_contributor(rv);
    });
}

// hock_schittkowski_71::fitness per row, and problem{unconstrain{problem with
// hock_schittkowski_71 and c_tol, method, weights}}.fitness per row
// (src/problems/unconstrain.cpp:104-225); method as its string.
int ref_hs71_fitness(const double *x, std::uint64_t n, double *out)
{
    return guard([&] {
        pagmo::problem p{pagmo::hock_schittkowski_71{}};
        for (std::uint64_t r = 0; r < n; ++r) {
            const auto f = p.fitness(pagmo::vector_double(x + 4u * r, x + 4u * r + 4u));
            std::copy(f.begin(), f.end(), out + 3u * r);
        }
    });
}

int ref_unconstrain_hs71(const char *method, const double *weights, std::uint64_t n_weights, const double *c_tol,
                         const double *x, std::uint64_t n, double *out)
{
    return guard([&] {
        pagmo::problem inner{pagmo::hock_schittkowski_71{}};
        if (c_tol) inner.set_c_tol(pagmo::vector_double(c_tol, c_tol + 2));
        pagmo::problem p{pagmo::unconstrain{inner, method, pagmo::vector_double(weights, weights + n_weights)}};
        const auto w = p.get_nf();
        for (std::uint64_t r = 0; r < n; ++r) {
            const auto f = p.fitness(pagmo::vector_double(x + 4u * r, x + 4u * r + 4u));
            std::copy(f.begin(), f.end(), out + w * r);
        }
    });
}

int ref_hvwfg_compute(const double *pts, std::uint64_t n, std::uint64_t m, const double *r, double *out)
{
    return guard([&] {
        pagmo::hypervolume hv(rows(pts, n, m), true);
        pagmo::hvwfg algo;
        *out = hv.compute(pagmo::vector_double(r, r + m), algo);
    });
}

// ZDT / DTLZ: dimensions (nx, nobj, nix) and bounds of the constructed problem;
// construction errors come back as status 1 with the reference's message.
int ref_mo_dims(int family, unsigned prob_id, std::uint64_t param, std::uint64_t fdim, unsigned alpha,
                std::uint64_t *nx, std::uint64_t *nobj, std::uint64_t *nix)
{
    return guard([&] {
        auto p = make_mo_problem(family, prob_id, param, fdim, alpha);
        *nx = p.get_nx();
        *nobj = p.get_nobj();
        *nix = p.get_nix();
    });
}

int ref_mo_bounds(int family, unsigned prob_id, std::uint64_t param, std::uint64_t fdim, unsigned alpha, double *lb,
                  double *ub)
{
    return guard([&] {
        auto p = make_mo_problem(family, prob_id, param, fdim, alpha);
        auto b = p.get_bounds();
        std::memcpy(lb, b.first.data(), b.first.size() * sizeof(double));
        std::memcpy(ub, b.second.data(), b.second.size() * sizeof(double));
    });
}

// bfe{thread_bfe{}} over n rows of a ZDT / DTLZ problem: fvs is n x nobj.
int ref_mo_thread_bfe(int family, unsigned prob_id, std::uint64_t param, std::uint64_t fdim, unsigned alpha,
                      const double *dvs, std::uint64_t n_dvs, std::uint64_t nx, double *fvs)
{
    return guard([&] {
        auto p = make_mo_problem(family, prob_id, param, fdim, alpha);
        pagmo::bfe b{pagmo::thread_bfe{}};
        pagmo::vector_double in(dvs, dvs + n_dvs * nx);
        auto out = b(p, in);
        std::memcpy(fvs, out.data(), out.size() * sizeof(double));
    });
}

// p_distance(x) of every row (zdt.cpp:204-224, dtlz.cpp:156-163).
int ref_mo_p_distance(int family, unsigned prob_id, std::uint64_t param, std::uint64_t fdim, unsigned alpha,
                      const double *dvs, std::uint64_t n_dvs, std::uint64_t nx, double *out)
{
    return guard([&] {
        pagmo::vector_double x(nx);
        if (family == 7) {
            pagmo::zdt udp{prob_id, static_cast<unsigned>(param)};
            for (std::uint64_t i = 0; i < n_dvs; ++i) {
                std::memcpy(x.data(), dvs + i * nx, nx * sizeof(double));
                out[i] = udp.p_distance(x);
            }
        } else {
            pagmo::dtlz udp{prob_id, static_cast<pagmo::vector_double::size_type>(param),
                            static_cast<pagmo::vector_double::size_type>(fdim), alpha};
            for (std::uint64_t i = 0; i < n_dvs; ++i) {
                std::memcpy(x.data(), dvs + i * nx, nx * sizeof(double));
                out[i] = udp.p_distance(x);
            }
        }
    });
}

// fast_non_dominated_sorting over n points of m objectives (row-major). Outputs:
// rank[n], dom_count[n], fronts flattened (front_offsets[n_fronts+1],
// front_indices[n]), dom_list flattened (dl_offsets[n+1], dl_indices up to
// dl_capacity entries; nullable).
int ref_fnds(const double *pts, std::uint64_t n, std::uint64_t m, std::uint64_t *rank, std::uint64_t *dom_count,
             std::uint64_t *front_offsets, std::uint64_t *front_indices, std::uint64_t *n_fronts,
             std::uint64_t *dl_offsets, std::uint64_t *dl_indices, std::uint64_t dl_capacity)
{
    return guard([&] {
        auto r = pagmo::fast_non_dominated_sorting(rows(pts, n, m));
        const auto &fr = std::get<0>(r);
        const auto &dl = std::get<1>(r);
        const auto &dc = std::get<2>(r);
        const auto &rk = std::get<3>(r);
        for (std::uint64_t i = 0; i < n; ++i) {
            rank[i] = rk[i];
            dom_count[i] = dc[i];
        }
        std::uint64_t pos = 0;
        front_offsets[0] = 0;
        for (std::size_t f = 0; f < fr.size(); ++f) {
            for (auto v : fr[f]) front_indices[pos++] = v;
            front_offsets[f + 1] = pos;
        }
        *n_fronts = fr.size();
        if (dl_offsets) {
            std::uint64_t q = 0;
            dl_offsets[0] = 0;
            for (std::uint64_t i = 0; i < n; ++i) {
                for (auto v : dl[i]) {
                    if (q >= dl_capacity) throw std::overflow_error("dom_list capacity exceeded");
                    dl_indices[q++] = v;
                }
                dl_offsets[i + 1] = q;
            }
        }
    });
}

// crowding_distance over one front of n points with m objectives (row-major).
int ref_crowding(const double *pts, std::uint64_t n, std::uint64_t m, double *out)
{
    return guard([&] {
        auto r = pagmo::crowding_distance(rows(pts, n, m));
        std::memcpy(out, r.data(), r.size() * sizeof(double));
    });
}

// select_best_N_mo over n points of m objectives: out[*n_out] indices.
int ref_select_best_n_mo(const double *pts, std::uint64_t n, std::uint64_t m, std::uint64_t N, std::uint64_t *out,
                         std::uint64_t *n_out)
{
    return guard([&] {
        const auto r = pagmo::select_best_N_mo(rows(pts, n, m), N);
        for (std::size_t i = 0; i < r.size(); ++i) out[i] = r[i];
        *n_out = r.size();
    });
}

// sort_population_mo over n points of m objectives: out[n].
int ref_sort_population_mo(const double *pts, std::uint64_t n, std::uint64_t m, std::uint64_t *out)
{
    return guard([&] {
        const auto r = pagmo::sort_population_mo(rows(pts, n, m));
        for (std::size_t i = 0; i < r.size(); ++i) out[i] = r[i];
    });
}

// pareto_dominance(a, b) for two m-vectors: returns 0/1 in *out.
int ref_pareto_dominance(const double *a, const double *b, std::uint64_t m, int *out)
{
    return guard([&] {
        *out = pagmo::pareto_dominance(pagmo::vector_double(a, a + m), pagmo::vector_double(b, b + m)) ? 1 : 0;
    });
}

} // extern "C"
