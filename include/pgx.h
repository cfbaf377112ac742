/*
 * pgx -- GB300-native batch evaluation for pagmo (C ABI).
 *
 * This is the drop-in boundary of the library: plain C types only (pointers,
 * sizes, status codes), no CUDA or C++ types in any signature, so that the
 * pagmo adaptor headers (include/pagmo_gb300/), a ctypes/cffi binding or a
 * pybind11 module of pygmo can bind it directly.
 *
 * Each entry point names the reference interface it replaces, as a path in
 * the pagmo 2.19.1 source tree.
 *
 * Conventions
 *  - Decision vectors are row-major: n_dvs rows of nx doubles, exactly the
 *    layout pagmo::bfe receives (src/problem.cpp:383-392). Fitness vectors of
 *    the single-objective kinds are n_dvs doubles (nf = 1); those of the
 *    multi-objective ZDT and DTLZ problems (pgx_mo_*) are n_dvs rows of nobj
 *    doubles, again pagmo's fvs layout.
 *    Gradients are dense, n_dvs rows of nx doubles: for nf = 1 this is the
 *    layout of problem::gradient (src/problem.cpp:456-467, dense sparsity).
 *  - Problems: PGX_RASTRIGIN (param = dim >= 1), PGX_ROSENBROCK (param =
 *    dim >= 2), PGX_LENNARD_JONES (param = atoms >= 3, nx = 3*atoms - 6);
 *    PGX_ACKLEY, PGX_GRIEWANK, PGX_SCHWEFEL (param = dim >= 1) have no
 *    gradient in the reference, so gradient requests for them return
 *    PGX_ERR_NOTIMPL, and archipelago epochs take the first three kinds only.
 *  - Every function returns PGX_OK (0) or an error status; the message of the
 *    calling thread's last error is pgx_last_error(). PGX_ERR_INVALID maps to
 *    pagmo's std::invalid_argument. There is no CPU fallback: without a usable
 *    GB300 every compute entry point fails with PGX_ERR_CUDA/PGX_ERR_NODEVICE.
 *  - Host-buffer entry points are synchronous. *_device entry points take
 *    device pointers and a cudaStream_t passed as void* (NULL = the legacy
 *    default stream, as in CUDA) and are asynchronous on that stream.
 *  - A context is bound to one device. Calls on one context are serialised
 *    by an internal lock, so island threads may share it.
 */
#ifndef PGX_H
#define PGX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGX_ABI_VERSION 1

#if defined(__GNUC__)
#define PGX_API __attribute__((visibility("default")))
#else
#define PGX_API
#endif

/* status codes */
#define PGX_OK 0
#define PGX_ERR_INVALID 1  /* bad argument (pagmo: std::invalid_argument) */
#define PGX_ERR_CUDA 2     /* a CUDA runtime call failed */
#define PGX_ERR_TIMEOUT 3  /* a bounded device-side wait gave up */
#define PGX_ERR_CAPACITY 4 /* a size exceeds a fixed capacity */
#define PGX_ERR_NODEVICE 5 /* no CUDA device could be opened */
#define PGX_ERR_NOTIMPL 6  /* not provided by the UDP (pagmo: not_implemented_error) */

/* problem kinds (the reference UDPs) */
#define PGX_RASTRIGIN 1     /* src/problems/rastrigin.cpp */
#define PGX_ROSENBROCK 2    /* src/problems/rosenbrock.cpp */
#define PGX_LENNARD_JONES 3 /* src/problems/lennard_jones.cpp */
#define PGX_ACKLEY 4        /* src/problems/ackley.cpp (fitness only) */
#define PGX_GRIEWANK 5      /* src/problems/griewank.cpp (fitness only) */
#define PGX_SCHWEFEL 6      /* src/problems/schwefel.cpp (fitness only) */
#define PGX_ZDT 7           /* src/problems/zdt.cpp (multi-objective, pgx_mo_*) */
#define PGX_DTLZ 8          /* src/problems/dtlz.cpp (multi-objective, pgx_mo_*) */

typedef struct pgx_context pgx_context;
typedef struct pgx_epoch pgx_epoch;

/* ------------------------------------------------------------------ runtime */

/* ABI version of the loaded library (PGX_ABI_VERSION at build time). */
PGX_API int pgx_abi_version(void);

/* Identity of this build of the library: a digest of its sources and compiler
 * flags. The archipelago autotuner keys its cached choices by it, so a rebuilt
 * library re-tunes. No counterpart in the reference. */
PGX_API const char *pgx_build_id(void);

/* Message of the calling thread's most recent failing call ("" if none). */
PGX_API const char *pgx_last_error(void);

/* Opens a context on CUDA device `device`: a non-blocking stream, grow-only
   device and pinned staging buffers, cached graphs. */
PGX_API int pgx_context_create(int device, pgx_context **out);
PGX_API void pgx_context_destroy(pgx_context *ctx);

/* Number of kernels this library launched on `ctx` since creation (for the
   benchmark's launch accounting). */
PGX_API uint64_t pgx_context_launch_count(const pgx_context *ctx);

/* ------------------------------------------------------------ problem facts */

/* Decision-vector size for (kind, param): rastrigin::get_bounds
   (src/problems/rastrigin.cpp:80-85), rosenbrock (:72-75), lennard_jones
   (src/problems/lennard_jones.cpp:99-113); validates param as the UDP
   constructors do (rastrigin.cpp:46-52, rosenbrock.cpp:43-49,
   lennard_jones.cpp:51-63). */
PGX_API int pgx_problem_nx(int kind, uint64_t param, uint64_t *nx);

/* Box bounds, nx doubles each (same sources as above). */
PGX_API int pgx_problem_bounds(int kind, uint64_t param, double *lb, double *ub);

/* --------------------------------------------------------- batch evaluation */

/* Batch fitness, host buffers. Replaces the fitness loop that
   bfe{thread_bfe{}} / member_bfe run for one problem
   (src/batch_evaluators/thread_bfe.cpp:64-144, member_bfe.cpp:40-45,
   src/problem.cpp:413-425) with one GPU pass. dvs: n_dvs*nx, fvs: n_dvs.
   Does not touch any fevals counter (pagmo::bfe adds n_dvs itself,
   src/bfe.cpp:106-107). */
PGX_API int pgx_batch_fitness(pgx_context *ctx, int kind, uint64_t param, const double *dvs, uint64_t n_dvs, double *fvs);

/* Batch fitness + gradient, host buffers: fvs (nullable) n_dvs, grads
   n_dvs*nx. Row i of grads equals problem::gradient(dv_i) of the reference
   (src/problems/rastrigin.cpp:98-107, src/problems/rosenbrock.cpp:83-92);
   for lennard_jones, which has no reference gradient, it is dE/dx over the
   3*atoms-6 free coordinates (minus the forces), with the pair loop
   recomputed. */
PGX_API int pgx_batch_gradient(pgx_context *ctx, int kind, uint64_t param, const double *dvs, uint64_t n_dvs, double *fvs,
                       double *grads);

/* Device-resident variant of both calls: d_grads NULL = fitness only,
   d_fvs may be NULL when d_grads is not. Asynchronous on `stream`. */
PGX_API int pgx_batch_eval_device(pgx_context *ctx, int kind, uint64_t param, const double *d_dvs, uint64_t n_dvs,
                          double *d_fvs, double *d_grads, void *stream);

/* Self-test of the bounded device waits (no counterpart in the reference):
   runs a two-block cooperative kernel in which one block never reaches the
   grid barrier, so the other's wait gives up after spin_limit polls (about
   spin_limit x 100 ns; 1 .. 2^24) and flags the timeout. *timed_out receives
   1 when the wait gave up and returned, as the survival kernels' barriers do
   (their callers then report PGX_ERR_TIMEOUT); the context stays usable. */
PGX_API int pgx_selftest_barrier_timeout(pgx_context *ctx, uint64_t spin_limit, int32_t *timed_out);

/* Self-test of the reciprocal and its cube in the Lennard-Jones pair loops
   (no counterpart in the reference, whose pair sum divides and cubes in FP64:
   src/problems/lennard_jones.cpp:83): inv[i] = 1/d[i] and, when inv_cube is
   not null, inv_cube[i] = 1/d[i]^3 from the fixed-point core those loops use
   (the loops feed it the integer sum of the squared differences; here it
   gets d's significand), for host arrays of n values. For 2^-100 <= d <
   2^101: 1/d within one half unit of the last place of the exact value plus
   2^-10 units, 1/d^3 plus 2^-5 units; for the other positive normal d with a
   normal reciprocal (an FP64 Newton step, then two FP64 multiplies): 1/d
   within one unit. Other d are not covered (the pair loops flag d = 0 apart). */
PGX_API int pgx_selftest_lj_reciprocal(pgx_context *ctx, const double *d, uint64_t n, double *inv, double *inv_cube);

/* ------------------------------------- multi-objective test problems (ZDT, DTLZ) */

/* A ZDT or DTLZ problem as its reference constructor takes it:
   zdt(prob_id, param) (src/problems/zdt.cpp:55-66; param is the dimension,
   except for ZDT5 whose 30 + 5 (param - 1) bits it counts) and
   dtlz(prob_id, dim, fdim, alpha) (src/problems/dtlz.cpp:53-74; pagmo's
   defaults are dim 5, fdim 3, alpha 100). */
typedef struct pgx_mo_problem {
    int kind;         /* PGX_ZDT or PGX_DTLZ */
    uint32_t prob_id; /* ZDT 1-6, DTLZ 1-7 */
    uint64_t param;   /* ZDT: param; DTLZ: dim */
    uint64_t fdim;    /* DTLZ: number of objectives (>= 2, < dim); ignored for ZDT */
    uint32_t alpha;   /* DTLZ4's exponent; ignored otherwise */
} pgx_mo_problem;

/* get_nx / get_nobj / get_nix of the problem (zdt.cpp:108-158, zdt.hpp:154-157,
   dtlz.cpp:116-119, dtlz.hpp:116-119); validates it with the constructors'
   messages (PGX_ERR_INVALID). Any output pointer may be NULL. */
PGX_API int pgx_mo_problem_dims(const pgx_mo_problem *p, uint64_t *nx, uint64_t *nobj, uint64_t *nix);

/* Box bounds, nx doubles each (zdt.cpp:108-133, dtlz.cpp:116-119). */
PGX_API int pgx_mo_problem_bounds(const pgx_mo_problem *p, double *lb, double *ub);

/* Batch fitness, host buffers: dvs n_dvs*nx, fvs n_dvs*nobj (row i holds
   fitness(dv_i), zdt.cpp:76-100, dtlz.cpp:84-107). Replaces the fitness loop
   of bfe{thread_bfe{}} / member_bfe for these problems; touches no fevals. */
PGX_API int pgx_mo_batch_fitness(pgx_context *ctx, const pgx_mo_problem *p, const double *dvs, uint64_t n_dvs,
                                 double *fvs);

/* Device-resident variant, asynchronous on `stream`: d_fvs n_dvs*nobj, for
   example the points of a following pgx_nsga2_survival_device call. */
PGX_API int pgx_mo_batch_fitness_device(pgx_context *ctx, const pgx_mo_problem *p, const double *d_dvs,
                                        uint64_t n_dvs, double *d_fvs, void *stream);

/* p_distance(dv) of every row (zdt.cpp:204-224, dtlz.cpp:156-163): out
   n_dvs doubles. p_distance(population) is their mean, summed in row order
   (zdt.cpp:179-187, dtlz.cpp:131-139). */
PGX_API int pgx_mo_p_distance(pgx_context *ctx, const pgx_mo_problem *p, const double *dvs, uint64_t n_dvs,
                              double *out);

/* ------------------------------------------------------------- hypervolume */

/* hypervolume(points).compute(ref) (src/utils/hypervolume.cpp:203-228,
   with the algorithm the reference picks: hv2d, hv3d or hvwfg,
   src/utils/hv_algos/hv_hv2d.cpp:48-68, hv_hv3d.cpp:75-116,
   hv_hvwfg.cpp:64-69): the measure of the region the n points (row-major, m
   objectives) dominate, bounded by ref. The reference's checks and messages
   (hypervolume.cpp:406-449, hv_algorithm.cpp:226-258: empty set, NaN, a point
   outside or equal to the reference point) give PGX_ERR_INVALID; more than
   16 objectives give PGX_ERR_NOTIMPL. FP64. For 2 and 3 objectives the value
   differs from the reference's sweep by summation order only (non-negative
   slabs, no cancellation); for 4 to 16 it is the reference's hvwfg value bit
   for bit. */
PGX_API int pgx_hypervolume(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, const double *ref,
                            double *out);

/* Device-resident variant: d_points on the device, ref on the host (m
   doubles), the volume written to *d_out, asynchronous on `stream`. The
   input checks that need the points (NaN, points beyond ref) are the
   caller's. */
PGX_API int pgx_hypervolume_device(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m,
                                   const double *ref, double *d_out, void *stream);

/* hypervolume(points).exclusive(p_idx, ref) (hypervolume.cpp:249-272 with
   hv_algorithm::exclusive, hv_algorithm.cpp:93-106): the volume of all the
   points minus the volume without point p_idx, both on the GPU (a lone
   point: its volume). The reference's checks come first, then an index
   p_idx >= n gives PGX_ERR_INVALID ("Index of the individual is out of
   bounds."). */
PGX_API int pgx_hypervolume_exclusive(pgx_context *ctx, const double *points, uint64_t n, uint64_t m,
                                      const double *ref, uint64_t p_idx, double *out);

/* hypervolume(points).contributions(ref) (hypervolume.cpp:293-320): out[i] =
   the volume only point i dominates, by hvwfg's contributions
   (hv_hvwfg.cpp:79-105): vol(p_i) - hv(limit set of p_i). For 4 to 16
   objectives this is the algorithm the reference picks and the values are
   its bit for bit; for 3 objectives the reference's hv3d (HyCon3D,
   hv_hv3d.cpp:170-300) sums boxes instead and falls back to the same hvwfg
   when a point is dominated; for 2, hv2d hands hv3d the points with a third
   coordinate 0 and a reference 1, and so does this call. A lone point: its
   volume |prod (p_c - r_c)| (hypervolume.cpp:303-307). Checks as
   pgx_hypervolume. */
PGX_API int pgx_hypervolume_contributions(pgx_context *ctx, const double *points, uint64_t n, uint64_t m,
                                          const double *ref, double *out);

/* Device-resident variant: d_points and d_out (n doubles) on the device, ref
   on the host, asynchronous on `stream`. A NaN in d_out marks a point whose
   warp ran out of frame buffers (cannot happen with the fixed pool of m
   frames of n rows per warp; the host variant reports it). */
PGX_API int pgx_hypervolume_contributions_device(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m,
                                                 const double *ref, double *d_out, void *stream);

/* least_contributor(ref) (greatest = 0) or greatest_contributor(ref)
   (greatest = 1) (hypervolume.cpp:333-401, hv_algorithm.cpp:136-157 and
   329-349): the first index of the smallest / largest contribution, the
   contributions as pgx_hypervolume_contributions computes them; 0 for a
   lone point. */
PGX_API int pgx_hypervolume_extreme_contributor(pgx_context *ctx, const double *points, uint64_t n, uint64_t m,
                                                const double *ref, int greatest, uint64_t *idx);

/* ---------------------------------- constrained problems and unconstrain */

#define PGX_HS71 9 /* src/problems/hock_schittkowski_71.cpp: nx 4, one objective, one equality, one inequality */

/* hock_schittkowski_71 (param unused): dimensions and bounds [1, 5]^4
   (hock_schittkowski_71.cpp:66-69), and the batch fitness, n rows of
   [f, ceq, cineq] (pagmo's fvs layout, :48-55), bit for bit the reference's. */
PGX_API int pgx_constrained_dims(int kind, uint64_t param, uint64_t *nx, uint64_t *nobj, uint64_t *nec,
                                 uint64_t *nic);
PGX_API int pgx_constrained_bounds(int kind, uint64_t param, double *lb, double *ub);
PGX_API int pgx_constrained_batch_fitness(pgx_context *ctx, int kind, uint64_t param, const double *dvs,
                                          uint64_t n_dvs, double *fvs);

/* unconstrain{inner, method, weights} (src/problems/unconstrain.cpp): the
   methods "death penalty", "kuri", "weighted", "ignore_c", "ignore_o"; weights
   (n_weights = nec + nic) for "weighted" only; c_tol the inner problem's
   constraint tolerances (NULL: all 0, pagmo's default). */
#define PGX_UNCONSTRAIN_DEATH 0
#define PGX_UNCONSTRAIN_KURI 1
#define PGX_UNCONSTRAIN_WEIGHTED 2
#define PGX_UNCONSTRAIN_IGNORE_C 3
#define PGX_UNCONSTRAIN_IGNORE_O 4
typedef struct pgx_unconstrain {
    int method;
    const double *weights;
    uint64_t n_weights;
    const double *c_tol;
} pgx_unconstrain;

/* unconstrain::batch_fitness (unconstrain.cpp:245-266): the inner problem's
   batch fitness and unconstrain::penalize (:130-225) of every row in one
   kernel; out n rows of the inner problem's nobj objectives (one for
   "ignore_o"), bit for bit the reference's. The constructor's checks and
   messages (:66-100) give PGX_ERR_INVALID. */
PGX_API int pgx_unconstrain_batch_fitness(pgx_context *ctx, int kind, uint64_t param, const pgx_unconstrain *u,
                                          const double *dvs, uint64_t n_dvs, double *fvs);

/* --------------------------------------------------- NSGA-II survival (MO) */

/* fast_non_dominated_sorting (src/utils/multi_objective.cpp:200-257) over n
   points of m objectives, row-major host buffer. Outputs (host):
     rank[n], dom_count[n]                    -- bit-exact with the reference
     front_offsets[n+1], front_indices[n]     -- fronts in the reference's order
     *n_fronts
   Errors as the reference: n < 2 -> PGX_ERR_INVALID. m may be 0. */
PGX_API int pgx_fnds(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, int32_t *rank, int32_t *dom_count,
             int32_t *front_offsets, int32_t *front_indices, int32_t *n_fronts);

/* The dom_list member of fnds_return_type, flattened: dl_offsets[n+1] and
   dl_indices[capacity] (each list ascending, as the reference builds it).
   Returns PGX_ERR_CAPACITY and the needed size in *dl_total when capacity
   is too small (dl_indices may then be NULL). */
PGX_API int pgx_fnds_dom_list(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, int64_t *dl_offsets,
                      int32_t *dl_indices, uint64_t capacity, uint64_t *dl_total);

/* crowding_distance of one non-dominated front (src/utils/multi_objective.cpp:280-315).
   n >= 2 and m >= 2 or PGX_ERR_INVALID. Bit-exact with the reference,
   including tied objective values: the per-objective sorts leave ties in the
   order the reference's std::sort (GNU libstdc++ introsort) leaves them. */
PGX_API int pgx_crowding_distance(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, double *out);

/* NSGA-II survival block (src/algorithms/nsga2.cpp:183-206): fnds, then the
   crowding distance of every point within its front (fronts of one or two
   points get +inf). crowding[n]; the fnds outputs as in pgx_fnds. */
PGX_API int pgx_nsga2_survival(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, int32_t *rank,
                       int32_t *dom_count, int32_t *front_offsets, int32_t *front_indices, int32_t *n_fronts,
                       double *crowding);

/* select_best_N_mo (src/utils/multi_objective.cpp:344-396): the indices of
   the best N of n points of m objectives (whole fronts while they fit, then the
   critical front by descending crowding distance), min(N, n) of them in out,
   that count in *n_out. Bit-exact with the reference, ties included. Errors as
   the reference: a critical front with m < 2 -> PGX_ERR_INVALID. */
PGX_API int pgx_select_best_n_mo(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, uint64_t N,
                                 int32_t *out, uint64_t *n_out);

/* sort_population_mo (src/utils/multi_objective.cpp:425-465): out[n], the
   points ordered by (non-domination rank, descending crowding distance; a
   front of one point counts 0). Bit-exact with the reference, ties included.
   A front of two or more points with m < 2 -> PGX_ERR_INVALID. */
PGX_API int pgx_sort_population_mo(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, int32_t *out);

/* Device-resident variants, asynchronous on `stream`: d_out holds min(N, n)
   (resp. n) indices. d_status (nullable device int32) reads, once the stream
   has run: 0 ok, 1 the reference would have thrown (crowding over fewer than
   two objectives; d_out is then incomplete), -1 a grid barrier gave up, 2 an
   internal error of the device sort. */
PGX_API int pgx_select_best_n_mo_device(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m, uint64_t N,
                                        int32_t *d_out, int32_t *d_status, void *stream);
PGX_API int pgx_sort_population_mo_device(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m,
                                          int32_t *d_out, int32_t *d_status, void *stream);

/* Sorts (keys[i], values[i]) by key in place (host buffers) on the GPU,
   leaving equal keys in the order std::sort (GNU libstdc++ introsort) leaves
   them -- the order behind the three functions above. No counterpart in the
   reference; exported so callers (and tests) can reproduce std::sort's tie
   order. n <= 2^30. */
PGX_API int pgx_std_sort_i64(pgx_context *ctx, int64_t *keys, int32_t *values, uint64_t n);

/* Device-resident survival: all pointers are device memory; d_n_fronts is a
   device int32. Asynchronous on `stream`. The front peeling waits on grid
   barriers with a bounded spin (about a second); if one gives up, the call
   still returns and *d_n_fronts reads -1 once the stream has run. */
PGX_API int pgx_nsga2_survival_device(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m, int32_t *d_rank,
                              int32_t *d_dom_count, int32_t *d_front_offsets, int32_t *d_front_indices,
                              int32_t *d_n_fronts, double *d_crowding, void *stream);

/* Allocation-free variant of pgx_nsga2_survival_device, for callers that
   cannot call cudaMalloc when they evaluate (their device memory is already
   held by another allocator, or they must not risk the device-wide
   synchronisation cudaMalloc/cudaFree can cause). It has no counterpart in
   the reference. Same arguments, outputs and asynchronous behaviour as
   pgx_nsga2_survival_device, without a context: it runs on the current
   device, and its scratch is a fixed device array inside the library, so
   n <= 4096 and m <= 8, else PGX_ERR_CAPACITY. The first call on each device
   (and in each CUDA context) does a one-time set-up: it looks up that array's
   device address and loads the library's survival code and data on the device
   (under lazy module loading, the CUDA default, this is when the ~2.6 MB array
   is allocated). Make that first call before another allocator reserves the
   device's memory, and before any stream capture; later calls allocate
   nothing. All calls share the array and it keeps the last call's contents
   (each call re-initialises what it needs); calls whose work overlaps on the
   GPU race on it and must be serialised by the caller. */
PGX_API int pgx_nsga2_survival_device_noalloc(const double *d_points, uint64_t n, uint64_t m, int32_t *d_rank,
                                              int32_t *d_dom_count, int32_t *d_front_offsets,
                                              int32_t *d_front_indices, int32_t *d_n_fronts, double *d_crowding,
                                              void *stream);

/* ------------------------------------------------- archipelago epochs */

/* One island's request in a migration epoch: a batch of one problem. */
typedef struct pgx_request {
    int kind;           /* PGX_RASTRIGIN, PGX_ROSENBROCK or PGX_LENNARD_JONES */
    uint64_t param;     /* dim, or atoms for lennard_jones */
    uint64_t n_dvs;     /* rows */
    const double *dvs;  /* host, n_dvs * nx, row-major */
    double *fvs;        /* host, n_dvs (may be NULL when grads is set) */
    double *grads;      /* host, n_dvs * nx, or NULL for fitness only */
} pgx_request;

/* Plans a migration epoch for a fixed list of request shapes (the pointers
   are ignored here). The islands' rows are packed into one device buffer
   and cut into warp-sized tiles, costliest first; lanes per row and tile
   sizes come from an autotuner that times the candidates on this device
   once per (problem, dimension) and caches the choice. Host-to-device copy,
   one persistent fused kernel over all tiles and device-to-host copies are
   captured in CUDA graphs, one per pinned staging set (three sets, three
   streams), so consecutive epochs overlap. On a device that accesses
   pageable host memory coherently (cudaDevAttrPageableMemoryAccess, as GB300
   with Grace over NVLink-C2C) a second graph per set lets the kernel read
   the requests' dvs and write their fvs/grads in place, with no packing,
   copies or unpacking; it is taken for every epoch whose arrays are 16-byte
   aligned and whose outputs do not overlap its inputs, unless
   PGX_EPOCH_STAGED=1. Replaces the island-by-island
   bfe calls of an archipelago epoch (src/archipelago.cpp:325-330 ->
   src/island.cpp:428-655 -> src/bfe.cpp:91-110). */
PGX_API int pgx_epoch_create(pgx_context *ctx, const pgx_request *reqs, int n_reqs, pgx_epoch **out);

/* One synchronous epoch: packs every request's dvs into the next staging
   set, replays its graph, waits, unpacks fvs/grads (or evaluates the arrays
   in place, see above). Shapes must match the plan (PGX_ERR_INVALID
   otherwise). */
PGX_API int pgx_epoch_run(pgx_epoch *ep, const pgx_request *reqs);

/* Asynchronous pair over the staging sets: submit packs and launches
   one epoch and returns; collect waits for the oldest submitted epoch and
   unpacks it into the pointers given at its submit. At most three in flight.
   Every array of a submitted request must stay allocated, and its dvs
   unchanged, until the collect of that epoch returns: the kernel may read
   and write them in place while the epoch runs. */
PGX_API int pgx_epoch_submit(pgx_epoch *ep, const pgx_request *reqs);
PGX_API int pgx_epoch_collect(pgx_epoch *ep);

/* Device-resident replay of the fused kernel alone on the plan's device
   buffers of staging set 0 (inputs as last copied), asynchronous on
   `stream` (NULL: the plan's stream). For measurement. */
PGX_API int pgx_epoch_launch_device(pgx_epoch *ep, void *stream);

/* Number of tiles and the lanes per row the autotuner chose for request i. */
PGX_API int pgx_epoch_info(const pgx_epoch *ep, int i, int *lanes_per_row, uint64_t *n_tiles);

PGX_API void pgx_epoch_destroy(pgx_epoch *ep);

/* The island-by-island baseline: one plain host-buffer batch call per
   request, in order (pgx_batch_gradient, or pgx_batch_fitness when grads is
   NULL). */
PGX_API int pgx_requests_run_plain(pgx_context *ctx, const pgx_request *reqs, int n_reqs);

/* ------------------------------------------------ batched local refinement */

/* Parameters of pgx_refine_batch (see there). */
typedef struct pgx_refine_params {
    uint32_t hops;   /* at most this many perturb-and-descend trials per individual */
    uint32_t stop;   /* an individual's chain ends after this many trials in a row without improvement
                        (mbh's stop, src/algorithms/mbh.cpp:150-190) */
    uint32_t steps;  /* projected-gradient steps per trial */
    double perturb;  /* perturbation half-width as a fraction of (ub - lb), in ]0, 1] (mbh's perturb) */
    double step0;    /* first step length of a descent, in box-scaled units, in ]0, 1] */
    double step_min; /* a descent ends when its step length falls below this (0 < step_min <= step0) */
    uint64_t seed;   /* the perturbations are a function of (seed, individual, trial, coordinate) */
} pgx_refine_params;

/* Monotonic basin hopping on every individual of a batch at once, with the
   batched adjoint driving a projected-gradient local descent: the scheme of
   mbh::evolve (src/algorithms/mbh.cpp:102-200) applied to each individual as
   its own chain, with gradient descent as the inner optimiser (mbh takes a
   pagmo algorithm and accepts a whole population when its best improves; it
   has no batched counterpart). Per individual, starting from its decision
   vector x_best: each trial perturbs x_best uniformly within
   [max(x - perturb (ub - lb), lb), min(x + perturb (ub - lb), ub)] per
   coordinate, takes up to `steps` steps x <- clamp(x - eta s d / |d|, lb, ub)
   with s = ub - lb and d = s * gradient (a step is kept when it lowers the
   fitness, eta then doubling up to 1, else eta halves; the descent ends when
   eta < step_min), and replaces x_best when it ends lower. Kinds with a
   gradient only (rastrigin, rosenbrock, lennard_jones; else PGX_ERR_NOTIMPL).
   dvs (n_dvs x nx) is overwritten with the best points, fvs (n_dvs) receives
   their fitness, *evals (nullable) the number of fitness + gradient
   evaluations made. Synchronous. */
PGX_API int pgx_refine_batch(pgx_context *ctx, int kind, uint64_t param, const pgx_refine_params *params, double *dvs,
                             uint64_t n_dvs, double *fvs, uint64_t *evals);

/* The same on device buffers, asynchronous on `stream`: *d_evals (device,
   zeroed by the caller) accumulates the evaluations. */
PGX_API int pgx_refine_batch_device(pgx_context *ctx, int kind, uint64_t param, const pgx_refine_params *params,
                                    double *d_dvs, uint64_t n_dvs, double *d_fvs, unsigned long long *d_evals,
                                    void *stream);

/* ------------------------------------------------------------ measurement */

/* FP64 FMA throughput of the device in GFLOP/s (FMA = 2 flops), measured by a
   short DFMA-chain kernel: the denominator of the FP64 roofline. */
PGX_API int pgx_measure_fp64_peak(pgx_context *ctx, double *gflops);

#ifdef __cplusplus
}
#endif
#endif
