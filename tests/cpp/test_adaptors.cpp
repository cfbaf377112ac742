// Host-side checks of the pagmo adaptors (include/pagmo_gb300/) against the
// reference's own type machinery: the GPU UDPs are UDPs with batch_fitness
// and gradient, gpu_bfe is a UDBFE, errors are pagmo's, and without a GPU
// every evaluation fails loudly instead of falling back to the CPU.
// Exit status 0 = all checks passed; with PGX_TEST_HAVE_GPU=1 the
// evaluations are also compared with the reference's own results.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <stdexcept>
#include <string>
#include <vector>

#include <pagmo/algorithm.hpp>
#include <pagmo/batch_evaluators/member_bfe.hpp>
#include <pagmo/batch_evaluators/thread_bfe.hpp>
#include <pagmo/bfe.hpp>
#include <pagmo/population.hpp>
#include <pagmo/problem.hpp>
#include <pagmo/exceptions.hpp>
#include <pagmo/problems/ackley.hpp>
#include <pagmo/problems/dtlz.hpp>
#include <pagmo/problems/griewank.hpp>
#include <pagmo/problems/hock_schittkowski_71.hpp>
#include <pagmo/problems/lennard_jones.hpp>
#include <pagmo/problems/null_problem.hpp>
#include <pagmo/problems/rastrigin.hpp>
#include <pagmo/problems/rosenbrock.hpp>
#include <pagmo/problems/schwefel.hpp>
#include <pagmo/problems/translate.hpp>
#include <pagmo/problems/unconstrain.hpp>
#include <pagmo/problems/zdt.hpp>
#include <pagmo/utils/hypervolume.hpp>
#include <pagmo/utils/multi_objective.hpp>

#include <pagmo_gb300/gpu_bfe.hpp>
#include <pagmo_gb300/gpu_mbh.hpp>
#include <pagmo_gb300/gpu_problems.hpp>
#include <pagmo_gb300/multi_objective.hpp>
#include <pagmo_gb300/s11n_implement.hpp>

using namespace pagmo_gb300;

static int failures = 0;
#define CHECK(c)                                                                                                      \
    do {                                                                                                               \
        if (!(c)) {                                                                                                    \
            std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);                                        \
            ++failures;                                                                                                \
        }                                                                                                              \
    } while (0)

template <typename E, typename F>
bool throws_with(F &&f, const std::string &needle)
{
    try {
        f();
    } catch (const E &e) {
        return std::string(e.what()).find(needle) != std::string::npos;
    } catch (...) {
        return false;
    }
    return false;
}

// A byte-stream archive with Boost.Serialization's operator& (save: append the
// member's bytes; load: read them back in the same order), enough for the
// plain members the plug-ins' serialize() functions visit: the round trip
// Boost's archives make of an island's problem, algorithm or bfe.
struct byte_archive {
    std::vector<unsigned char> buf;
    std::size_t pos = 0;
    bool loading = false;
    template <typename T>
    byte_archive &operator&(T &v)
    {
        static_assert(std::is_trivially_copyable<T>::value, "plain members only");
        if (loading) {
            if (pos + sizeof(T) > buf.size()) throw std::runtime_error("archive exhausted");
            std::memcpy(&v, buf.data() + pos, sizeof(T));
            pos += sizeof(T);
        } else {
            const auto *q = reinterpret_cast<const unsigned char *>(&v);
            buf.insert(buf.end(), q, q + sizeof(T));
        }
        return *this;
    }
};

// src saved and loaded into a default-constructed T; every byte consumed
template <typename T>
T round_trip(T src)
{
    byte_archive a;
    src.serialize(a, 0u);
    T dst{};
    a.loading = true;
    dst.serialize(a, 0u);
    if (a.pos != a.buf.size()) throw std::runtime_error("archive not consumed");
    return dst;
}

template <typename T>
bool same_problem(const T &x, const T &y)
{
    const pagmo::problem a{x}, b{y};
    return a.get_nx() == b.get_nx() && a.get_nobj() == b.get_nobj() && a.get_nix() == b.get_nix()
           && a.get_bounds() == b.get_bounds() && a.get_name() == b.get_name()
           && a.get_extra_info() == b.get_extra_info();
}

static_assert(pagmo::is_udbfe<gpu_bfe>::value, "gpu_bfe must be a UDBFE");
static_assert(pagmo::is_udp<gpu_rastrigin>::value, "gpu_rastrigin must be a UDP");
static_assert(pagmo::is_udp<gpu_rosenbrock>::value, "gpu_rosenbrock must be a UDP");
static_assert(pagmo::is_udp<gpu_lennard_jones>::value, "gpu_lennard_jones must be a UDP");
static_assert(pagmo::has_batch_fitness<gpu_rosenbrock>::value, "batch_fitness hook");
static_assert(pagmo::has_gradient<gpu_rosenbrock>::value, "gradient hook");
static_assert(pagmo::has_gradient<gpu_lennard_jones>::value, "gradient hook");
static_assert(pagmo::has_batch_fitness<pagmo::translate>::value, "translate forwards batch_fitness");
static_assert(pagmo::is_udp<gpu_zdt>::value && pagmo::is_udp<gpu_dtlz>::value, "gpu_zdt / gpu_dtlz must be UDPs");
static_assert(pagmo::is_udp<gpu_hock_schittkowski_71>::value, "gpu_hock_schittkowski_71 must be a UDP");
static_assert(pagmo::has_batch_fitness<gpu_zdt>::value && pagmo::has_batch_fitness<gpu_dtlz>::value,
              "batch_fitness hook of the multi-objective UDPs");
static_assert(!pagmo::has_gradient<gpu_zdt>::value && !pagmo::has_gradient<gpu_dtlz>::value,
              "zdt and dtlz have no gradient in the reference");
static_assert(pagmo::has_get_nobj<gpu_dtlz>::value && pagmo::has_integer_part<gpu_zdt>::value, "nobj / nix hooks");
static_assert(pagmo::is_udp<gpu_ackley>::value && pagmo::is_udp<gpu_griewank>::value && pagmo::is_udp<gpu_schwefel>::value,
              "fitness-only GPU UDPs");
static_assert(!pagmo::has_gradient<gpu_ackley>::value && !pagmo::has_gradient<gpu_schwefel>::value,
              "no gradient where the reference has none");
static_assert(pagmo::has_batch_fitness<gpu_griewank>::value, "batch_fitness hook");

int main()
{
    const bool gpu = std::getenv("PGX_TEST_HAVE_GPU") && std::string(std::getenv("PGX_TEST_HAVE_GPU")) == "1";

    // problem facade: dims, bounds, hooks, thread safety
    pagmo::problem p{gpu_rosenbrock{10u}};
    CHECK(p.get_nx() == 10u && p.get_nf() == 1u);
    CHECK(p.has_batch_fitness() && p.has_gradient());
    CHECK(p.get_thread_safety() == pagmo::thread_safety::constant);
    CHECK(p.get_bounds() == pagmo::problem{pagmo::rosenbrock{10u}}.get_bounds());
    CHECK(pagmo::problem{gpu_rastrigin{7u}}.get_bounds() == pagmo::problem{pagmo::rastrigin{7u}}.get_bounds());
    CHECK(pagmo::problem{gpu_lennard_jones{5u}}.get_nx() == 9u);
    CHECK(pagmo::problem{gpu_lennard_jones{5u}}.get_name().find("Jones") != std::string::npos);

    // constructor errors are the reference's
    CHECK(throws_with<std::invalid_argument>([] { gpu_rastrigin{0u}; }, "must have minimum 1 dimension"));
    CHECK(throws_with<std::invalid_argument>([] { gpu_rosenbrock{1u}; }, "must have minimum 2 dimensions"));
    CHECK(throws_with<std::invalid_argument>([] { gpu_lennard_jones{2u}; }, "greater than 2"));
    CHECK(throws_with<std::invalid_argument>([] { gpu_ackley{0u}; }, "Ackley Function must have minimum 1"));
    CHECK(throws_with<std::invalid_argument>([] { gpu_griewank{0u}; }, "Griewank Function must have minimum 1"));
    CHECK(throws_with<std::invalid_argument>([] { gpu_schwefel{0u}; }, "Schwefel Function must have minimum 1"));
    CHECK(pagmo::problem{gpu_ackley{3u}}.get_bounds() == pagmo::problem{pagmo::ackley{3u}}.get_bounds());
    CHECK(pagmo::problem{gpu_griewank{3u}}.get_bounds() == pagmo::problem{pagmo::griewank{3u}}.get_bounds());
    CHECK(pagmo::problem{gpu_schwefel{3u}}.get_bounds() == pagmo::problem{pagmo::schwefel{3u}}.get_bounds());
    CHECK(pagmo::problem{gpu_schwefel{3u}}.get_name() == pagmo::problem{pagmo::schwefel{3u}}.get_name());
    // no gradient: pagmo's own not_implemented_error, before any device work
    CHECK(throws_with<pagmo::not_implemented_error>([] { pagmo::problem{gpu_ackley{3u}}.gradient({1., 2., 3.}); },
                                                    "gradient"));

    // ZDT / DTLZ: constructor errors, dimensions, bounds and names as the reference's
    CHECK(throws_with<std::invalid_argument>([] { gpu_zdt{7u, 23u}; }, "prob_id=7 was detected"));
    CHECK(throws_with<std::invalid_argument>([] { gpu_zdt{2u, 1u}; }, "minimum value of 2"));
    CHECK(throws_with<std::invalid_argument>([] { gpu_dtlz{9u, 7u, 3u, 100u}; }, "prob_id=9 was detected"));
    CHECK(throws_with<std::invalid_argument>([] { gpu_dtlz{1u, 7u, 1u, 100u}; }, "minimum of 2 objectives"));
    CHECK(throws_with<std::invalid_argument>([] { gpu_dtlz{1u, 3u, 3u, 100u}; }, "has to be larger"));
    for (unsigned id = 1u; id <= 6u; ++id) {
        const unsigned param = id == 4u ? 10u : 11u;
        pagmo::problem a{gpu_zdt{id, param}}, r{pagmo::zdt{id, param}};
        CHECK(a.get_nx() == r.get_nx() && a.get_nobj() == r.get_nobj() && a.get_nix() == r.get_nix());
        CHECK(a.get_bounds() == r.get_bounds() && a.get_name() == r.get_name());
    }
    for (unsigned id = 1u; id <= 7u; ++id) {
        pagmo::problem a{gpu_dtlz{id, 12u, 4u}}, r{pagmo::dtlz{id, 12u, 4u}};
        CHECK(a.get_nx() == r.get_nx() && a.get_nobj() == r.get_nobj() && a.get_nix() == r.get_nix());
        CHECK(a.get_bounds() == r.get_bounds() && a.get_name() == r.get_name());
    }
    CHECK(throws_with<std::invalid_argument>([] { gpu_dtlz{2u, 4u}.p_distance(pagmo::vector_double(3, 0.5)); },
                                             "The size of the decision vector should be 4 while 3 was detected"));

    // the UDBFE wrapped by pagmo::bfe
    pagmo::bfe b{gpu_bfe{}};
    CHECK(throws_with<std::invalid_argument>([&b] { b(pagmo::problem{pagmo::dtlz{4u}}, pagmo::vector_double(10, 0.5)); },
                                             "alpha is not exposed"));
    CHECK(b.get_name() == "GB300 batch fitness evaluator");
    CHECK(b.get_thread_safety() == pagmo::thread_safety::basic);
    CHECK(b.is<gpu_bfe>());
    CHECK(throws_with<std::invalid_argument>([&b] { b(pagmo::problem{pagmo::null_problem{}}, {0.5, 0.5}); },
                                             "Cannot use a gpu_bfe on the problem"));
    // pagmo::bfe's own input check runs before the UDBFE
    CHECK(throws_with<std::invalid_argument>([&b] { b(pagmo::problem{pagmo::rosenbrock{4u}}, {1., 2., 3.}); },
                                             "is not an exact multiple"));

    // multi-objective: argument errors before any device work
    CHECK(throws_with<std::invalid_argument>([] { fast_non_dominated_sorting({{1., 2.}}); },
                                             "At least two points"));
    CHECK(throws_with<std::invalid_argument>([] { crowding_distance({{1.}, {2.}}); }, "at least two objectives"));
    // select_best_N_mo / sort_population_mo corner cases need no device, as in the reference
    CHECK(select_best_N_mo({{1., 2.}, {3., 4.}}, 0u).empty());
    CHECK(select_best_N_mo({}, 10u).empty());
    CHECK((select_best_N_mo({{1., 2.}}, 10u) == std::vector<pagmo::pop_size_t>{0u}));
    CHECK((sort_population_mo({{1., 5., 2., 3.}}) == std::vector<pagmo::pop_size_t>{0u}));
    CHECK(sort_population_mo({}).empty());

    std::vector<double> dvs(40);
    for (size_t i = 0; i < dvs.size(); ++i) dvs[i] = -2.0 + 0.1 * static_cast<double>(i);
    if (!gpu) {
        // no device: evaluations fail loudly, never on the CPU
        pagmo::problem pr{pagmo::rosenbrock{4u}};
        CHECK(throws_with<std::runtime_error>([&] { b(pr, dvs); }, ""));
        CHECK(pr.get_fevals() == 0u);
        CHECK(throws_with<std::runtime_error>([&] { pagmo::problem{gpu_rosenbrock{4u}}.fitness({1., 1., 1., 1.}); },
                                              ""));
        CHECK(throws_with<std::runtime_error>([] { sort_population_mo({{1., 2.}, {2., 1.}}); }, ""));
        pagmo::problem pz{pagmo::zdt{1u, 4u}};
        CHECK(throws_with<std::runtime_error>([&] { b(pz, dvs); }, ""));
        CHECK(pz.get_fevals() == 0u);
        // translate{rosenbrock}: gpu_bfe reaches the inner problem (and the device)
        pagmo::problem pt{pagmo::translate{pagmo::rosenbrock{4u}, {0.1, 0.2, 0.3, 0.4}}};
        CHECK(throws_with<std::runtime_error>([&] { b(pt, dvs); }, ""));
        CHECK(!throws_with<std::invalid_argument>([&] { b(pt, dvs); }, "Cannot use a gpu_bfe"));
    } else {
        // with a device: bfe{gpu_bfe} against bfe{thread_bfe}, fevals counted once
        pagmo::problem pr{pagmo::rosenbrock{4u}};
        const auto f_gpu = b(pr, dvs);
        CHECK(pr.get_fevals() == 10u);
        const auto f_ref = pagmo::bfe{pagmo::thread_bfe{}}(pagmo::problem{pagmo::rosenbrock{4u}}, dvs);
        for (size_t i = 0; i < f_ref.size(); ++i) CHECK(std::abs(f_gpu[i] - f_ref[i]) <= 1e-13 * std::abs(f_ref[i]));
        pagmo::problem pg{gpu_rosenbrock{4u}};
        CHECK(pg.gradient({.1, .2, .3, .4}).size() == 4u);
        auto r = fast_non_dominated_sorting({{0, 7}, {1, 5}, {2, 3}, {4, 2}, {7, 1}, {10, 0}, {2, 6}, {4, 4}, {10, 2},
                                             {6, 6}, {9, 5}});
        auto w = pagmo::fast_non_dominated_sorting({{0, 7}, {1, 5}, {2, 3}, {4, 2}, {7, 1}, {10, 0}, {2, 6}, {4, 4},
                                                    {10, 2}, {6, 6}, {9, 5}});
        CHECK(r == w);
        // tie-heavy populations: the index lists equal the reference's, ties included
        std::vector<pagmo::vector_double> pop;
        unsigned seed = 7u;
        for (int i = 0; i < 150; ++i) {
            pagmo::vector_double f(3);
            for (auto &v : f) {
                seed = seed * 1103515245u + 12345u;
                v = static_cast<double>((seed >> 16) % 4u);
            }
            pop.push_back(f);
        }
        CHECK(sort_population_mo(pop) == pagmo::sort_population_mo(pop));
        for (pagmo::pop_size_t N : {1u, 7u, 50u, 75u, 149u, 150u, 300u})
            CHECK(select_best_N_mo(pop, N) == pagmo::select_best_N_mo(pop, N));
        const auto cd_gpu = crowding_distance(pop), cd_ref = pagmo::crowding_distance(pop);
        bool same = cd_gpu.size() == cd_ref.size();
        for (size_t i = 0; same && i < cd_ref.size(); ++i)
            same = (std::isnan(cd_gpu[i]) && std::isnan(cd_ref[i])) || cd_gpu[i] == cd_ref[i];
        CHECK(same);
        CHECK(throws_with<std::invalid_argument>([] { sort_population_mo({{1.}, {1.}, {2.}}); },
                                                 "at least two objectives"));
        // ackley, griewank, schwefel through bfe{gpu_bfe} against bfe{thread_bfe}
        std::vector<double> d3(30);
        for (size_t i = 0; i < d3.size(); ++i) d3[i] = -14.0 + 1.7 * static_cast<double>(i);
        for (auto prob : {pagmo::problem{pagmo::ackley{3u}}, pagmo::problem{pagmo::griewank{3u}},
                          pagmo::problem{pagmo::schwefel{3u}}}) {
            const auto fg = b(prob, d3);
            const auto fr = pagmo::bfe{pagmo::thread_bfe{}}(prob, d3);
            for (size_t i = 0; i < fr.size(); ++i) CHECK(std::abs(fg[i] - fr[i]) <= 1e-12 * (1.0 + std::abs(fr[i])));
        }
        // translate: around pagmo's rosenbrock through gpu_bfe, around a GPU UDP through its batch_fitness
        {
            const pagmo::vector_double shift{0.5, -0.25, 1.5, 2.0};
            pagmo::problem pt{pagmo::translate{pagmo::rosenbrock{4u}, shift}};
            pagmo::problem pg2{pagmo::translate{gpu_rosenbrock{4u}, shift}};
            CHECK(pg2.has_batch_fitness());
            const auto fr = pagmo::bfe{pagmo::thread_bfe{}}(pt, dvs);
            const auto f1 = b(pt, dvs);
            const auto f2 = pagmo::bfe{pagmo::member_bfe{}}(pg2, dvs);
            for (size_t i = 0; i < fr.size(); ++i) {
                CHECK(std::abs(f1[i] - fr[i]) <= 1e-13 * std::abs(fr[i]));
                CHECK(std::abs(f2[i] - fr[i]) <= 1e-13 * std::abs(fr[i]));
            }
        }
        // pagmo's zdt and dtlz through bfe{gpu_bfe}, and the GPU UDPs, against bfe{thread_bfe}
        std::vector<double> u(60);
        for (size_t i = 0; i < u.size(); ++i) u[i] = 0.0125 + 0.0163 * static_cast<double>(i % 61);
        for (auto prob : {pagmo::problem{pagmo::zdt{1u, 6u}}, pagmo::problem{pagmo::zdt{3u, 6u}},
                          pagmo::problem{pagmo::dtlz{2u, 6u, 3u}}, pagmo::problem{pagmo::dtlz{7u, 6u, 3u}},
                          pagmo::problem{gpu_zdt{2u, 6u}}, pagmo::problem{gpu_dtlz{4u, 6u, 3u, 100u}}}) {
            const auto fg = b(prob, u);
            const auto fr = pagmo::bfe{pagmo::thread_bfe{}}(prob, u);
            CHECK(fg.size() == fr.size());
            for (size_t i = 0; i < fr.size(); ++i) CHECK(std::abs(fg[i] - fr[i]) <= 1e-12 * (1.0 + std::abs(fr[i])));
        }
        // gpu_mbh through pagmo's algorithm: no individual gets worse, most improve,
        // the stored fitness is the problem's fitness of the stored point, fevals grow
        for (auto prob : {pagmo::problem{pagmo::rosenbrock{10u}}, pagmo::problem{gpu_rastrigin{20u}},
                          pagmo::problem{pagmo::lennard_jones{8u}}}) {
            pagmo::population pop{prob, 64u, 17u};
            const auto f0 = pop.get_f();
            const auto fe0 = pop.get_problem().get_fevals();
            pagmo::algorithm algo{gpu_mbh{4u, 3u, 10u, 0.05, 0.05, 1e-6, 3u}};
            CHECK(algo.get_name().find("GB300") != std::string::npos);
            pop = algo.evolve(pop);
            int better = 0;
            for (size_t i = 0; i < f0.size(); ++i) {
                CHECK(pop.get_f()[i][0] <= f0[i][0]);
                better += pop.get_f()[i][0] < f0[i][0];
                const double fx = pagmo::problem{prob}.fitness(pop.get_x()[i])[0];
                CHECK(std::abs(fx - pop.get_f()[i][0]) <= 1e-12 * (1.0 + std::abs(fx)));
            }
            CHECK(better > 32);
            CHECK(pop.get_problem().get_fevals() > fe0 + 64u);
        }
        // hock_schittkowski_71 through bfe{gpu_bfe}, and pagmo's unconstrain around the GPU UDP (its
        // batch_fitness forwards to the GPU) against the reference's own problems, bit for bit
        {
            std::vector<double> hx(4 * 50);
            for (size_t i = 0; i < hx.size(); ++i) hx[i] = 1.0 + std::fmod(0.731 * static_cast<double>(i * i + 3u), 4.0);
            pagmo::problem hr{pagmo::hock_schittkowski_71{}}, hg{gpu_hock_schittkowski_71{}};
            const auto fr = pagmo::bfe{pagmo::thread_bfe{}}(hr, hx);
            CHECK(b(hr, hx) == fr);
            CHECK(pagmo::bfe{pagmo::member_bfe{}}(hg, hx) == fr);
            for (const char *m : {"death penalty", "kuri", "ignore_c", "ignore_o"}) {
                pagmo::problem ur{pagmo::unconstrain{pagmo::hock_schittkowski_71{}, m}};
                pagmo::problem ug{pagmo::unconstrain{gpu_hock_schittkowski_71{}, m}};
                CHECK(ug.has_batch_fitness());
                const auto want = pagmo::bfe{pagmo::thread_bfe{}}(ur, hx);
                CHECK(pagmo::bfe{pagmo::member_bfe{}}(ug, hx) == want);
                CHECK(b(ug, hx) == want);
            }
            pagmo::problem uw{pagmo::unconstrain{gpu_hock_schittkowski_71{}, "weighted", {2.0, 0.5}}};
            CHECK(b(uw, hx)
                  == pagmo::bfe{pagmo::thread_bfe{}}(
                      pagmo::problem{pagmo::unconstrain{pagmo::hock_schittkowski_71{}, "weighted", {2.0, 0.5}}}, hx));
        }
        // hypervolume queries against pagmo::hypervolume: 5 objectives (hvwfg) bit for bit
        {
            std::vector<pagmo::vector_double> pts;
            for (unsigned i = 0; i < 40u; ++i) {
                pagmo::vector_double q(5);
                for (unsigned k = 0; k < 5u; ++k) q[k] = std::fmod(0.37 * (i + 1u) * (k + 2u) + 0.11 * k * k, 1.0);
                pts.push_back(q);
            }
            const pagmo::vector_double r(5, 1.5);
            pagmo::hypervolume h(pts);
            CHECK(hypervolume_compute(pts, r) == h.compute(r));
            CHECK(hypervolume_contributions(pts, r) == h.contributions(r));
            CHECK(hypervolume_exclusive(pts, 7u, r) == h.exclusive(7u, r));
            CHECK(hypervolume_least_contributor(pts, r) == h.least_contributor(r));
            CHECK(hypervolume_greatest_contributor(pts, r) == h.greatest_contributor(r));
            CHECK(throws_with<std::invalid_argument>([&] { hypervolume_exclusive(pts, 40u, r); },
                                                     "Index of the individual is out of bounds."));
            // the class mirror, from points and from a population
            pagmo_gb300::hypervolume hg(pts);
            CHECK(hg.compute(r) == h.compute(r) && hg.contributions(r) == h.contributions(r));
            CHECK(hg.least_contributor(r) == h.least_contributor(r) && hg.refpoint(0.5) == h.refpoint(0.5));
            pagmo::population zp{pagmo::problem{pagmo::zdt{1u, 10u}}, 30u, 7u};
            const pagmo_gb300::hypervolume hz(zp);
            const pagmo::hypervolume hzr(zp);
            CHECK(hz.compute(hzr.refpoint(1.0)) == hzr.compute(hzr.refpoint(1.0))
                  || std::abs(hz.compute(hzr.refpoint(1.0)) - hzr.compute(hzr.refpoint(1.0)))
                         <= 1e-13 * hzr.compute(hzr.refpoint(1.0)));
        }
    }
    // the hypervolume class mirror's construction checks (no GPU needed)
    CHECK(throws_with<std::invalid_argument>([] { pagmo_gb300::hypervolume h{std::vector<pagmo::vector_double>{}}; },
                                             "Point set cannot be empty."));
    CHECK(throws_with<std::invalid_argument>(
        [] { pagmo_gb300::hypervolume h{std::vector<pagmo::vector_double>{{1.0, 2.0}, {1.0}}}; },
        "All point set dimensions must be equal."));
    CHECK(throws_with<std::invalid_argument>(
        [] {
            pagmo::population p{pagmo::problem{pagmo::rosenbrock{3u}}, 4u, 1u};
            pagmo_gb300::hypervolume h{p};
        },
        "not multiobjective"));
    // gpu_mbh refuses problems it cannot refine (no CPU fallback) and bad perturbations
    CHECK(throws_with<std::invalid_argument>([] { gpu_mbh{10u, 5u, 20u, 0.0}; }, "The perturbation must be in ]0,1]"));
    CHECK(throws_with<std::invalid_argument>(
        [] {
            pagmo::population pop{pagmo::problem{pagmo::ackley{3u}}, 4u, 1u};
            gpu_mbh{}.evolve(pop);
        },
        "Cannot use gpu_mbh"));
    // serialize(): the members the plug-ins save come back, so a loaded problem,
    // algorithm or bfe is the saved one (the Boost registration itself is the
    // export-key / implement macro pair and needs Boost)
    CHECK(same_problem(round_trip(gpu_rastrigin{13u, 1}), gpu_rastrigin{13u, 1}));
    CHECK(round_trip(gpu_rastrigin{13u, 1}).param() == 13u);
    CHECK(same_problem(round_trip(gpu_rosenbrock{21u}), gpu_rosenbrock{21u}));
    CHECK(same_problem(round_trip(gpu_lennard_jones{9u}), gpu_lennard_jones{9u}));
    CHECK(same_problem(round_trip(gpu_ackley{5u}), gpu_ackley{5u}));
    CHECK(same_problem(round_trip(gpu_griewank{6u}), gpu_griewank{6u}));
    CHECK(same_problem(round_trip(gpu_schwefel{7u}), gpu_schwefel{7u}));
    CHECK(same_problem(round_trip(gpu_zdt{5u, 12u}), gpu_zdt{5u, 12u}));
    CHECK(same_problem(round_trip(gpu_dtlz{4u, 9u, 3u, 50u}), gpu_dtlz{4u, 9u, 3u, 50u}));
    CHECK(same_problem(round_trip(gpu_hock_schittkowski_71{}), gpu_hock_schittkowski_71{}));
    CHECK(round_trip(gpu_bfe{3}).get_extra_info() == gpu_bfe{3}.get_extra_info());
    CHECK(round_trip(gpu_mbh{7u, 3u, 11u, 0.2, 0.03, 1e-7, 99u, 2}).get_extra_info()
          == gpu_mbh(7u, 3u, 11u, 0.2, 0.03, 1e-7, 99u, 2).get_extra_info());
    CHECK(round_trip(gpu_mbh{7u, 3u, 11u, 0.2, 0.03, 1e-7, 99u, 2}).get_extra_info() != gpu_mbh{}.get_extra_info());

    if (failures) {
        std::fprintf(stderr, "%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("adaptor checks passed (%s)\n", gpu ? "with GPU" : "no GPU");
    return 0;
}
