// pagmo's own algorithms, compiled from the reference's sources, run twice on
// the same problem, population and seeds: once with bfe{thread_bfe{}} (the
// reference's CPU batch evaluator) and once with bfe{gpu_bfe{}}. This is the
// shape of the reference's bfe_usage tests (tests/nsga2.cpp:204-233,
// tests/moead_gen.cpp:258-287, tests/pso_gen.cpp:302-318, tests/nspso.cpp:202-229,
// tests/gaco.cpp:340-356, tests/maco.cpp:185-212), with the GPU bfe in place of
// the default one.
//
// Per case the program reports whether the two runs took the same decisions
// (final decision vectors bit-identical), whether the logs are bit-identical,
// and the largest relative difference of a logged or final fitness value.
// A case passes when the decisions are identical and every value is within
// 1e-12 relative (absolute floor 1e-14 for values near zero): the GPU's
// fitness values differ from the reference's in the last bits only (within
// 1e-13 of the error scale), and the same decisions show that no selection
// turned on such a difference. Exit status 0 = every case passed.
//
// Each run's initial population is evaluated by the run's own batch evaluator
// (pagmo's population(problem, bfe, size, seed) constructor, same decision
// vectors for both): NSGA-II copies offspring that neither crossover nor
// mutation changed, and such a clone must tie with its parent. A GPU run that
// started from parents evaluated by problem::fitness on the CPU would compare
// GPU clones with CPU parents, whose values can differ in the last bit, and
// pagmo's dominance test would then rank one above the other.
//
// Without PGX_TEST_HAVE_GPU=1 only the thread_bfe runs are made (the GPU bfe
// is then expected to fail loudly, which the other adaptor test checks).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <sstream>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include <pagmo/algorithm.hpp>
#include <pagmo/algorithms/gaco.hpp>
#include <pagmo/algorithms/maco.hpp>
#include <pagmo/algorithms/moead_gen.hpp>
#include <pagmo/algorithms/nsga2.hpp>
#include <pagmo/algorithms/nspso.hpp>
#include <pagmo/algorithms/pso_gen.hpp>
#include <pagmo/batch_evaluators/thread_bfe.hpp>
#include <pagmo/bfe.hpp>
#include <pagmo/population.hpp>
#include <pagmo/problem.hpp>
#include <pagmo/problems/dtlz.hpp>
#include <pagmo/problems/lennard_jones.hpp>
#include <pagmo/problems/rastrigin.hpp>
#include <pagmo/problems/rosenbrock.hpp>
#include <pagmo/problems/zdt.hpp>

#include <pagmo_gb300/gpu_bfe.hpp>
#include <pagmo_gb300/gpu_problems.hpp>
#include <pagmo_gb300/s11n_implement.hpp>

namespace
{

struct Diff {
    bool ints_equal = true;    // every integer field (generation, fevals, sizes) equal
    bool bit_identical = true; // every floating value bit for bit
    bool within_tol = true;
    double max_rel = 0.0;
};

void cmp_value(Diff &d, double a, double b)
{
    if (std::isnan(a) && std::isnan(b)) return;
    if (!(a == b)) d.bit_identical = false;
    const double scale = std::fmax(std::fabs(a), std::fabs(b));
    const double err = std::fabs(a - b);
    if (scale > 0.0) d.max_rel = std::fmax(d.max_rel, err / scale);
    if (!(err <= 1e-12 * scale + 1e-14)) d.within_tol = false;
}

template <typename T>
std::enable_if_t<std::is_integral<T>::value> cmp(Diff &d, T a, T b)
{
    if (a != b) d.ints_equal = false;
}
inline void cmp(Diff &d, double a, double b)
{
    cmp_value(d, a, b);
}
inline void cmp(Diff &d, const pagmo::vector_double &a, const pagmo::vector_double &b)
{
    if (a.size() != b.size()) {
        d.ints_equal = false;
        return;
    }
    for (std::size_t i = 0; i < a.size(); ++i) cmp_value(d, a[i], b[i]);
}
template <typename Tup, std::size_t... I>
void cmp_tuple(Diff &d, const Tup &a, const Tup &b, std::index_sequence<I...>)
{
    (cmp(d, std::get<I>(a), std::get<I>(b)), ...);
}
template <typename... T>
void cmp(Diff &d, const std::tuple<T...> &a, const std::tuple<T...> &b)
{
    cmp_tuple(d, a, b, std::index_sequence_for<T...>{});
}

// the algorithms print their log at verbosity > 0 (needed to record it)
struct Quiet {
    std::ostringstream sink;
    std::streambuf *old;
    Quiet() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~Quiet()
    {
        std::cout.rdbuf(old);
    }
};

int failures = 0;

template <typename UDA, typename Make>
void compare(const char *name, Make make, const pagmo::problem &prob, pagmo::population::size_type np,
             unsigned pop_seed, bool have_gpu, const pagmo::problem *prob_gpu_udp = nullptr)
{
    // prob_gpu_udp: the GPU run on a GPU UDP (every problem::fitness call on
    // the GPU too) instead of on the reference's own UDP
    const pagmo::population pop{prob, pagmo::bfe{pagmo::thread_bfe{}}, np, pop_seed};
    UDA cpu = make();
    cpu.set_verbosity(1u);
    cpu.set_bfe(pagmo::bfe{pagmo::thread_bfe{}});
    pagmo::population p_cpu;
    {
        Quiet q;
        p_cpu = cpu.evolve(pop);
    }
    if (!have_gpu) {
        std::printf("case %-34s thread_bfe only: %zu log lines, fevals %llu\n", name, cpu.get_log().size(),
                    static_cast<unsigned long long>(p_cpu.get_problem().get_fevals()));
        return;
    }
    const pagmo::population pop_gpu{prob_gpu_udp ? *prob_gpu_udp : prob, pagmo::bfe{pagmo_gb300::gpu_bfe{}}, np,
                                    pop_seed};
    if (pop_gpu.get_x() != pop.get_x()) {
        std::printf("case %-34s initial populations differ -> FAILED\n", name);
        ++failures;
        return;
    }
    UDA gpu = make();
    gpu.set_verbosity(1u);
    gpu.set_bfe(pagmo::bfe{pagmo_gb300::gpu_bfe{}});
    pagmo::population p_gpu;
    {
        Quiet q;
        p_gpu = gpu.evolve(pop_gpu);
    }
    Diff log_d, f_d;
    const auto &l1 = cpu.get_log();
    const auto &l2 = gpu.get_log();
    if (l1.size() != l2.size()) log_d.ints_equal = false;
    std::size_t first_diff = l1.size();
    for (std::size_t i = 0; i < l1.size() && i < l2.size(); ++i) {
        Diff line;
        cmp(line, l1[i], l2[i]);
        if (!line.bit_identical && first_diff == l1.size()) first_diff = i;
        cmp(log_d, l1[i], l2[i]);
    }
    const bool same_x = p_cpu.get_x() == p_gpu.get_x() && p_cpu.get_ID() == p_gpu.get_ID();
    const auto &f1 = p_cpu.get_f();
    const auto &f2 = p_gpu.get_f();
    if (f1.size() != f2.size()) f_d.ints_equal = false;
    for (std::size_t i = 0; i < f1.size() && i < f2.size(); ++i) cmp(f_d, f1[i], f2[i]);
    const bool fevals_equal = p_cpu.get_problem().get_fevals() == p_gpu.get_problem().get_fevals();
    const bool ok = same_x && fevals_equal && log_d.ints_equal && f_d.ints_equal && log_d.within_tol
                    && f_d.within_tol;
    std::printf("case %-34s decisions %s, log %s (%zu lines, first differing line %zd), "
                "max rel diff log %.3g final f %.3g, final f %s, fevals %llu %s -> %s\n",
                name, same_x ? "identical" : "DIFFER", log_d.bit_identical ? "bit-identical" : "not bit-identical",
                l1.size(), first_diff == l1.size() ? static_cast<std::ptrdiff_t>(-1)
                                                   : static_cast<std::ptrdiff_t>(first_diff),
                log_d.max_rel, f_d.max_rel, f_d.bit_identical ? "bit-identical" : "not bit-identical",
                static_cast<unsigned long long>(p_gpu.get_problem().get_fevals()), fevals_equal ? "(equal)" : "(DIFFER)",
                ok ? "ok" : "FAILED");
    if (!ok) ++failures;
}

// population::population(problem, bfe, size, seed) (src/population.cpp:82-103):
// the initial population evaluated through a bfe
void compare_population_init(const char *name, const pagmo::problem &prob, pagmo::population::size_type np,
                             unsigned seed)
{
    const pagmo::population a{prob, pagmo::bfe{pagmo::thread_bfe{}}, np, seed};
    const pagmo::population b{prob, pagmo::bfe{pagmo_gb300::gpu_bfe{}}, np, seed};
    Diff d;
    const auto &f1 = a.get_f();
    const auto &f2 = b.get_f();
    for (std::size_t i = 0; i < f1.size(); ++i) cmp(d, f1[i], f2[i]);
    const bool ok = a.get_x() == b.get_x() && f1.size() == f2.size() && d.ints_equal && d.within_tol
                    && a.get_problem().get_fevals() == b.get_problem().get_fevals();
    std::printf("init %-34s %zu individuals, max rel diff f %.3g, %s -> %s\n", name, f1.size(), d.max_rel,
                d.bit_identical ? "bit-identical" : "not bit-identical", ok ? "ok" : "FAILED");
    if (!ok) ++failures;
}

} // namespace

int main()
{
    using namespace pagmo;
    const char *env = std::getenv("PGX_TEST_HAVE_GPU");
    const bool have_gpu = env && std::string(env) == "1";

    // NSGA-II: the reference's own bfe test shape, a bit-exact integer problem, a longer run
    compare<nsga2>("nsga2 dtlz1(10,2) 24x10", [] { return nsga2{10u, 0.95, 10., 0.01, 50., 23u}; },
                   problem{dtlz{1u, 10u, 2u}}, 24u, 32u, have_gpu);
    compare<nsga2>("nsga2 zdt5(10) 24x10", [] { return nsga2{10u, 0.95, 10., 0.01, 50., 23u}; },
                   problem{zdt{5u, 10u}}, 24u, 32u, have_gpu);
    compare<nsga2>("nsga2 zdt1(30) 100x50", [] { return nsga2{50u, 0.95, 10., 0.01, 50., 7u}; },
                   problem{zdt{1u, 30u}}, 100u, 8u, have_gpu);
    compare<nsga2>("nsga2 dtlz2(12,3) 92x30", [] { return nsga2{30u, 0.95, 10., 0.01, 50., 11u}; },
                   problem{dtlz{2u, 12u, 3u}}, 92u, 12u, have_gpu);
    // MOEA/D (generational), NSPSO, MACO: multi-objective
    compare<moead_gen>("moead_gen zdt1(30) 24x10",
                       [] { return moead_gen{10u, "grid", "tchebycheff", 10u, 0.9, 0.5, 20., 0.9, 2u, true, 23u}; },
                       problem{zdt{1u, 30u}}, 24u, 32u, have_gpu);
    compare<nspso>("nspso dtlz2(12,3) 24x10",
                   [] { return nspso{10u, 0.6, 2.0, 2.0, 1.0, 0.5, 60u, "crowding distance", false, 23u}; },
                   problem{dtlz{2u, 12u, 3u}}, 24u, 32u, have_gpu);
    {
        const problem gp{pagmo_gb300::gpu_dtlz{2u, 12u, 3u}};
        compare<nsga2>("nsga2 gpu_dtlz2(12,3) UDP 92x30", [] { return nsga2{30u, 0.95, 10., 0.01, 50., 11u}; },
                       problem{dtlz{2u, 12u, 3u}}, 92u, 12u, have_gpu, &gp);
    }
    compare<maco>("maco dtlz1(10,2) 43x10", [] { return maco{10u, 43u, 1.0, 1u, 7u, 100000u, 0., false, 23u}; },
                  problem{dtlz{1u, 10u, 2u}}, 43u, 32u, have_gpu);
    // PSO (generational) and GACO: single objective, the three hot-path UDPs
    compare<pso_gen>("pso_gen rosenbrock(10) 30x40",
                     [] { return pso_gen{40u, 0.79, 2., 2., 0.1, 5u, 2u, 4u, false, 23u}; },
                     problem{rosenbrock{10u}}, 30u, 23u, have_gpu);
    compare<pso_gen>("pso_gen rastrigin(50) 64x40",
                     [] { return pso_gen{40u, 0.79, 2., 2., 0.1, 5u, 2u, 4u, false, 5u}; },
                     problem{rastrigin{50u}}, 64u, 6u, have_gpu);
    compare<pso_gen>("pso_gen lennard_jones(10) 32x30",
                     [] { return pso_gen{30u, 0.79, 2., 2., 0.1, 5u, 2u, 4u, false, 9u}; },
                     problem{lennard_jones{10u}}, 32u, 10u, have_gpu);
    compare<gaco>("gaco rosenbrock(10) 200x40",
                  [] { return gaco{40u, 10u, 1.0, 25.0, 0.01, 5u, 7u, 1000u, 1000u, 0.0, false, 23u}; },
                  problem{rosenbrock{10u}}, 200u, 23u, have_gpu);
    if (have_gpu) {
        compare_population_init("rosenbrock(1000) x 4096", problem{rosenbrock{1000u}}, 4096u, 3u);
        compare_population_init("lennard_jones(150) x 256", problem{lennard_jones{150u}}, 256u, 4u);
        compare_population_init("zdt1(30) x 20000", problem{zdt{1u, 30u}}, 20000u, 5u);
    }
    if (failures) {
        std::printf("%d case(s) FAILED\n", failures);
        return 1;
    }
    std::printf(have_gpu ? "uda checks passed (with GPU)\n" : "uda checks passed (thread_bfe only)\n");
    return 0;
}
