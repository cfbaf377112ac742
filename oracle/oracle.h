/*
 * CPU oracle for the pagmo batch-evaluation path (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain C++ restatement of the reference algorithms that the GPU
 * library replaces. It is the checker: only the test suite, the smoke check
 * and the CPU leg of the benchmark call it. The product library never links,
 * loads or falls back to it.
 *
 * Parity pin: tests/test_oracle.py checks every function here against the
 * golden vectors in tests/golden/ (produced by the reference's own sources,
 * compiled unmodified by oracle/Makefile) and against the known answers in
 * the reference's tests (tests/lennard_jones.cpp:59-60, tests/rastrigin.cpp:56-57,
 * tests/rosenbrock.cpp:70-79, tests/multi_objective.cpp:81-182).
 *
 * Two families:
 *  - "mirror" functions repeat the reference's double arithmetic in the same
 *    order, so they reproduce its results bit for bit (same libm);
 *  - "_ld" functions evaluate the same formulas in long double and also return
 *    a condition scale (the sum of the absolute values of the summed terms),
 *    used to state relative errors that survive cancellation.
 *
 * Problem kinds: 1 = rastrigin (param = dim), 2 = rosenbrock (param = dim),
 * 3 = lennard_jones (param = atoms, dim = 3*atoms-6), 4 = ackley, 5 = griewank,
 * 6 = schwefel (param = dim; fitness only, as in the reference).
 * Status codes: 0 ok, 1 invalid argument (message via orc_last_error()).
 */
#ifndef PGX_ORACLE_H
#define PGX_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

const char *orc_last_error(void);

/* ---- mirrors of the reference arithmetic (double) ---- */
double orc_rastrigin_fitness(const double *x, uint64_t n);
void orc_rastrigin_gradient(const double *x, uint64_t n, double *g);
double orc_rosenbrock_fitness(const double *x, uint64_t n);
void orc_rosenbrock_gradient(const double *x, uint64_t n, double *g);
double orc_lj_fitness(const double *x, uint64_t atoms);
double orc_ackley_fitness(const double *x, uint64_t n);
double orc_griewank_fitness(const double *x, uint64_t n);
double orc_schwefel_fitness(const double *x, uint64_t n);

/* ---- long-double oracle with condition scales ---- */
double orc_rastrigin_fitness_ld(const double *x, uint64_t n, double *scale);
void orc_rastrigin_gradient_ld(const double *x, uint64_t n, double *g, double *gscale);
double orc_rosenbrock_fitness_ld(const double *x, uint64_t n, double *scale);
void orc_rosenbrock_gradient_ld(const double *x, uint64_t n, double *g, double *gscale);
double orc_lj_fitness_ld(const double *x, uint64_t atoms, double *scale);
void orc_lj_gradient_ld(const double *x, uint64_t atoms, double *g, double *gscale);
double orc_ackley_fitness_ld(const double *x, uint64_t n, double *scale);
double orc_griewank_fitness_ld(const double *x, uint64_t n, double *scale);
double orc_schwefel_fitness_ld(const double *x, uint64_t n, double *scale);

/* ---- batch runners over row-major dvs (n rows of nx) ---- */
/* Mirror of bfe{thread_bfe{}}: static partition over nthreads std::threads,
   each row copied into a temporary vector and evaluated by the mirror fitness
   (thread_bfe.cpp:94-123). nthreads <= 0 -> hardware_concurrency. */
int orc_batch_fitness(int kind, uint64_t param, const double *dvs, uint64_t n, uint64_t nx, double *f, int nthreads);
/* Mirror gradients per row (rastrigin/rosenbrock: the reference's gradient();
   lennard_jones: the long-double formula rounded to double). */
int orc_batch_gradient(int kind, uint64_t param, const double *dvs, uint64_t n, uint64_t nx, double *g, int nthreads);
/* Long-double fitness (+scale) and gradient (+component scales) per row. */
int orc_batch_fitness_ld(int kind, uint64_t param, const double *dvs, uint64_t n, uint64_t nx, double *f,
                         double *scale, int nthreads);
int orc_batch_gradient_ld(int kind, uint64_t param, const double *dvs, uint64_t n, uint64_t nx, double *g,
                          double *gscale, int nthreads);

/* ---- multi-objective survival ---- */
int orc_pareto_dominance(const double *a, const double *b, uint64_t m);
/* fast_non_dominated_sorting (multi_objective.cpp:200-257). Fronts are
   flattened: front_offsets[0..n_fronts], front_indices[0..n). dom_list is
   flattened the same way (dl_offsets[0..n], dl_indices) when dl_offsets is
   non-null; dl_capacity bounds dl_indices. */
int orc_fnds(const double *pts, uint64_t n, uint64_t m, uint64_t *rank, uint64_t *dom_count,
             uint64_t *front_offsets, uint64_t *front_indices, uint64_t *n_fronts, uint64_t *dl_offsets,
             uint64_t *dl_indices, uint64_t dl_capacity);
/* crowding_distance of one front (multi_objective.cpp:280-315). */
int orc_crowding(const double *pts, uint64_t n, uint64_t m, double *out);
/* NSGA-II survival glue (nsga2.cpp:183-206): crowding per front for all points,
   fronts of size 1 or 2 get +inf. Needs the fronts from orc_fnds. */
int orc_nsga2_crowding(const double *pts, uint64_t n, uint64_t m, const uint64_t *front_offsets,
                       const uint64_t *front_indices, uint64_t n_fronts, double *out);
/* Same with stable != 0: ties between equal objective values keep their
   order in the front (std::stable_sort), the tie rule of the GPU kernels. */
int orc_crowding_ex(const double *pts, uint64_t n, uint64_t m, int stable, double *out);
int orc_nsga2_crowding_ex(const double *pts, uint64_t n, uint64_t m, const uint64_t *front_offsets,
                          const uint64_t *front_indices, uint64_t n_fronts, int stable, double *out);

/* ---- orderings (sorting.cpp) ----
   (key, value) pairs sorted by key in place: with std::sort (the reference's
   order of ties), with the restated libstdc++ introsort, with the same
   introsort partitioned in 32-wide chunks (the GPU's formulation), and with
   std::partial_sort(first, last, last) / the restated heapsort. */
const char *orc_sort_last_error(void);
uint64_t orc_depth_limit_hits(void);
void orc_std_sort_keys(long long *k, int32_t *v, uint64_t n);
void orc_introsort_keys(long long *k, int32_t *v, uint64_t n);
void orc_introsort_chunked_keys(long long *k, int32_t *v, uint64_t n);
void orc_introsort_lists_keys(long long *k, int32_t *v, uint64_t n);
void orc_heap_sort_keys(long long *k, int32_t *v, uint64_t n);
void orc_std_partial_sort_full(long long *k, int32_t *v, uint64_t n);
/* McIlroy's quicksort adversary against std::sort: n keys. */
void orc_quicksort_adversary(uint64_t n, long long *out);
/* select_best_N_mo (multi_objective.cpp:344-396) and sort_population_mo
   (:425-465). Errors: 1 with the message in orc_sort_last_error(). */
int orc_select_best_n_mo(const double *pts, uint64_t n, uint64_t m, uint64_t N, uint64_t *out, uint64_t *n_out);
int orc_sort_population_mo(const double *pts, uint64_t n, uint64_t m, uint64_t *out);

/* ---- ZDT (family 7) and DTLZ (family 8) multi-objective problems (mo_problems.cpp) ---- */
const char *orc_mo_last_error(void);
int orc_mo_dims(int family, unsigned prob_id, uint64_t param, uint64_t fdim, uint64_t *nx, uint64_t *nobj);
void orc_zdt_fitness(unsigned prob_id, const double *x, uint64_t n, double *f);
double orc_zdt_p_distance(unsigned prob_id, const double *x, uint64_t n);
void orc_dtlz_fitness(unsigned prob_id, uint64_t fdim, unsigned alpha, const double *x, uint64_t n, double *f);
double orc_dtlz_p_distance(unsigned prob_id, uint64_t fdim, const double *x, uint64_t n);
int orc_mo_batch_fitness(int family, unsigned prob_id, uint64_t param, uint64_t fdim, unsigned alpha,
                         const double *dvs, uint64_t n, uint64_t nx, double *f, int nthreads);
int orc_mo_batch_fitness_ld(int family, unsigned prob_id, uint64_t param, uint64_t fdim, unsigned alpha,
                            const double *dvs, uint64_t n, uint64_t nx, double *f, double *scale, int nthreads);
int orc_mo_batch_p_distance(int family, unsigned prob_id, uint64_t param, uint64_t fdim, const double *dvs,
                            uint64_t n, uint64_t nx, double *out, double *scale, int nthreads);

/* ---- hypervolume of 2 or 3 objectives, long double (hypervolume.cpp) ---- */
int orc_hypervolume_ld(const double *pts, uint64_t n, uint64_t m, const double *ref, double *out);

/* ---- WFG (hvwfg, stop dimension 2) in double, the reference's operation
   order: the volume, and every point's exclusive contribution ---- */
int orc_hvwfg(const double *pts, uint64_t n, uint64_t m, const double *ref, double *out);
int orc_hvwfg_contributions(const double *pts, uint64_t n, uint64_t m, const double *ref, double *out);

/* ---- hock_schittkowski_71 and unconstrain's penalties, double, the
   reference's operation order (constrained.cpp); method 0..4 = death penalty,
   kuri, weighted, ignore_c, ignore_o ---- */
void orc_hs71_fitness(const double *x, uint64_t n, double *f);
int orc_unconstrain_penalize(const double *f, uint64_t n, uint64_t nobj, uint64_t nec, uint64_t nic, int method,
                             const double *weights, const double *tol, double *out);

#ifdef __cplusplus
}
#endif
#endif
