// Internal declarations shared by the pgx translation units: error state,
// the context object, device helpers and the kernel launchers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pgx.h"

// Digest of the sources and flags of this build, set by the build recipe.
#ifndef PGX_BUILD_ID
#define PGX_BUILD_ID "unversioned"
#endif

namespace pgx
{

// ------------------------------------------------------------------ errors

void set_error(const std::string &msg);
const char *get_error();

// Returns PGX_ERR_CUDA (and records the message) when `e` is an error.
int cuda_status(cudaError_t e, const char *what);

#define PGX_CUDA(call)                                                                                                 \
    do {                                                                                                               \
        cudaError_t pgx_e_ = (call);                                                                                   \
        if (pgx_e_ != cudaSuccess) return ::pgx::cuda_status(pgx_e_, #call);                                           \
    } while (0)

#define PGX_CHECK(cond, code, msg)                                                                                     \
    do {                                                                                                               \
        if (!(cond)) {                                                                                                 \
            ::pgx::set_error(msg);                                                                                     \
            return (code);                                                                                             \
        }                                                                                                              \
    } while (0)

#define PGX_TRY(expr)                                                                                                  \
    do {                                                                                                               \
        int pgx_s_ = (expr);                                                                                           \
        if (pgx_s_ != PGX_OK) return pgx_s_;                                                                           \
    } while (0)

// --------------------------------------------------------- device buffers

// Grow-only device allocation owned by a context.
struct dbuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t need);
    void release();
    template <typename T>
    T *as() const
    {
        return static_cast<T *>(ptr);
    }
};

// Grow-only pinned host allocation owned by a context.
struct hbuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t need);
    void release();
    template <typename T>
    T *as() const
    {
        return static_cast<T *>(ptr);
    }
};

} // namespace pgx

// The context (opaque to callers of the C ABI).
struct pgx_context {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr; // kernels
    cudaStream_t h2d = nullptr;    // host-to-device copies of the host pipelines
    cudaStream_t d2h = nullptr;    // device-to-host copies of the host pipelines
    std::mutex lock;
    uint64_t launches = 0;
    // device buffers of the host-buffer calls
    pgx::dbuf d_in, d_out, d_grad;
    std::vector<cudaEvent_t> chunk_ev;
    // survival: inputs/outputs of host calls, the scratch of a pass, small outputs
    pgx::dbuf s_points, s_state, s_outs, s_crowd;
    // batched refinement: per-individual working points and gradients
    pgx::dbuf r_work;
    // WFG hypervolume: work counter, status and the warps' frame pools
    pgx::dbuf h_wfg;
};

namespace pgx
{

// Scope guard: makes ctx->device current for the calling thread.
int use_device(pgx_context *ctx);

// ------------------------------------------------------- host row pipeline
// Launches the evaluation of nr rows already on the device (inputs din, nx per
// row; outputs dout and, when set, dgrad) on stream s, adding its kernel
// launches to *launches.
using row_launcher = std::function<int(const double *din, uint64_t nr, double *dout, double *dgrad, cudaStream_t s,
                                       uint64_t *launches)>;
// Host-buffer batch evaluation through the context's chunked upload /
// evaluate / download pipeline; out_w outputs per row in fvs.
int host_rows(pgx_context *ctx, uint64_t nx, uint64_t out_w, const double *dvs, uint64_t n, double *fvs, double *grads,
              const row_launcher &launch);

// ------------------------------------------------------------ problem facts

int problem_nx(int kind, uint64_t param, uint64_t *nx);

// ------------------------------------------------------ WFG hypervolume

// Most objectives the WFG kernels take (hv_wfg.cu).
constexpr uint32_t kWfgMaxObjectives = 16;
// The volume of n >= 1 device points of 2 <= m <= kWfgMaxObjectives
// objectives by pagmo's hvwfg (stop dimension 2), r on the host; *d_out on
// stream s. Bit-exact with the reference.
int launch_wfg_compute(pgx_context *ctx, const double *d_pts, uint32_t n, uint32_t m, const double *r,
                       double *d_out, cudaStream_t s);
// Every point's exclusive contribution (d_out[n]) as pagmo's
// hypervolume::contributions computes it for m >= 4 (hvwfg), and as hv3d /
// hv2d's contributions do when they fall back to hvwfg for m = 3 / 2.
int launch_wfg_contributions(pgx_context *ctx, const double *d_pts, uint32_t n, uint32_t m, const double *r,
                             double *d_out, cudaStream_t s);
// Synchronises ctx->stream and reads the status word of the last WFG warp
// kernel (nonzero: a warp ran out of frame buffers; its outputs are NaN).
int wfg_status(pgx_context *ctx, unsigned *status);

// -------------------------------------------------------------- launchers

// Lanes per row (1..32) used by the strided rastrigin/rosenbrock row kernels.
int lanes_per_row(uint32_t nx);
// Threads per block of the row kernels for n rows of `lanes` lanes: 256, or
// fewer so that small batches still give every SM a block.
int row_block_threads(uint64_t n, int lanes, int num_sms);

// Whether lennard_jones clusters of na atoms use the flattened pair walk.
bool lj_use_flat(uint32_t na);

// True when PGX_ROSENBROCK_DOUBLE_FLOAT=1: rosenbrock rows in double-float
// arithmetic on the FP32 pipe (an opt-in; the default is FP64 arithmetic).
bool rosenbrock_double_float();

// PGX_ERR_NOTIMPL unless the problem kind provides a gradient.
int check_has_gradient(int kind);

// rastrigin/rosenbrock with a forced row variant (lanes 1..32, or 0 for the
// 4-wide rosenbrock rows); for the autotuner.
int launch_rows_variant(int kind, uint64_t nx, const double *d_x, uint64_t n, double *d_f, double *d_g, int lanes,
                        cudaStream_t stream, int num_sms);

// Batch fitness (+ gradient when d_g != nullptr) for one problem on `stream`.
// Returns the number of kernel launches issued through *launches.
int launch_eval(int kind, uint64_t param, uint64_t nx, const double *d_x, uint64_t n, double *d_f, double *d_g,
                cudaStream_t stream, int num_sms, uint64_t *launches);

// Survival: fnds (+ crowding when d_crowd != nullptr) on device buffers.
struct survival_out {
    int32_t *rank = nullptr;
    int32_t *dom_count = nullptr;
    int32_t *front_offsets = nullptr; // n + 1 entries
    int32_t *front_indices = nullptr; // n entries
    int32_t *n_fronts = nullptr;      // one int32
    double *crowding = nullptr;       // n entries or nullptr
};
int launch_survival(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m, const survival_out &out,
                    cudaStream_t stream);

// Single-front crowding distance on device buffers.
int launch_crowding_single(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m, double *d_out,
                           cudaStream_t stream);

// select_best_N_mo / sort_population_mo on device buffers (d_out holds
// min(N, n) / n indices; d_status nullable: 0 ok, -1 barrier timeout, 1 fewer
// than two objectives where crowding is needed, 2 internal sort error).
int launch_select_best(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m, uint64_t N, int32_t *d_out,
                       int32_t *d_status, cudaStream_t stream);
int launch_sort_population(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m, int32_t *d_out,
                           int32_t *d_status, cudaStream_t stream);
// After a synchronisation: the error of the last select_best/sort_population
// pass of shape (n, m) on this context, as the reference would raise it.
int read_mo_status(pgx_context *ctx, uint64_t n, uint64_t m);
// std::sort-ordered in-place sort of device (key, value) pairs by one block;
// d_lists holds n int2 and d_pos 2 n int32 of scratch, *d_err receives a
// nonzero code on a broken invariant.
// d_state: sort_pairs_state_bytes() of device scratch (grid barrier state of
// the grid-wide sort used beyond 4096 pairs).
int launch_sort_pairs(pgx_context *ctx, long long *d_keys, int32_t *d_vals, uint64_t n, int *d_err, int2 *d_lists,
                      int32_t *d_pos, void *d_state, cudaStream_t stream);
size_t sort_pairs_state_bytes();
// Self-test of the bounded grid barriers (one block never arrives).
int run_barrier_timeout_test(pgx_context *ctx, uint64_t spin_limit, int32_t *timed_out);
// Self-test of the Lennard-Jones pair loops' 1/d and 1/d^3 (host in, host out; cube may be null).
int run_lj_reciprocal(pgx_context *ctx, const double *d, uint64_t n, double *inv, double *cube);

// Reads the device status word of the last survival pass of shape (n, m) on
// this context (after a stream synchronisation): PGX_ERR_TIMEOUT when a grid
// barrier gave up.
int read_survival_status(pgx_context *ctx, uint64_t n, uint64_t m);

// dom_list support: builds the "dominates" bit matrix (row i: the points i
// dominates) and per-row counts (device int64[n], owned by the context), then
// writes each row's set bits, ascending, at the given CSR offsets.
int build_dominates_rows(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m, int64_t **d_row_count,
                         cudaStream_t stream);
int extract_dom_list(pgx_context *ctx, uint64_t n, uint64_t m, const int64_t *d_offsets, int32_t *d_indices,
                     cudaStream_t stream);

} // namespace pgx
