// The C ABI of include/pgx.h: contexts, staging buffers, argument checks
// mirroring the reference's, and the host-buffer pipelines around the kernels.
#include "pgx_internal.cuh"

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace pgx
{

namespace
{
thread_local std::string t_err;

constexpr size_t kChunkBytes = size_t(32) << 20; // per-chunk input bytes of the host pipeline
constexpr int kMaxChunkEvents = 128;
} // namespace

void set_error(const std::string &msg)
{
    t_err = msg;
}

const char *get_error()
{
    return t_err.c_str();
}

int cuda_status(cudaError_t e, const char *what)
{
    t_err = std::string("CUDA error in ") + what + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? PGX_ERR_NODEVICE : PGX_ERR_CUDA;
}

int dbuf::ensure(size_t need)
{
    if (need <= bytes && ptr) return PGX_OK;
    release();
    size_t sz = std::max<size_t>(need, 256);
    PGX_CUDA(cudaMalloc(&ptr, sz));
    bytes = sz;
    return PGX_OK;
}

void dbuf::release()
{
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

int hbuf::ensure(size_t need)
{
    if (need <= bytes && ptr) return PGX_OK;
    release();
    size_t sz = std::max<size_t>(need, 256);
    PGX_CUDA(cudaMallocHost(&ptr, sz));
    bytes = sz;
    return PGX_OK;
}

void hbuf::release()
{
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    bytes = 0;
}

int use_device(pgx_context *ctx)
{
    PGX_CUDA(cudaSetDevice(ctx->device));
    return PGX_OK;
}

// rastrigin.cpp:46-52 (dim >= 1), rosenbrock.cpp:43-49 (dim >= 2),
// lennard_jones.cpp:51-63 (atoms >= 3, 3*(atoms-2) must fit an unsigned).
int problem_nx(int kind, uint64_t param, uint64_t *nx)
{
    switch (kind) {
        case PGX_RASTRIGIN:
            PGX_CHECK(param >= 1u, PGX_ERR_INVALID,
                      "Rastrigin Function must have minimum 1 dimension, " + std::to_string(param) + " requested");
            *nx = param;
            return PGX_OK;
        case PGX_ROSENBROCK:
            PGX_CHECK(param >= 2u, PGX_ERR_INVALID,
                      "Rosenbrock Function must have minimum 2 dimensions, " + std::to_string(param) + " requested");
            *nx = param;
            return PGX_OK;
        case PGX_LENNARD_JONES:
            PGX_CHECK(param >= 3u, PGX_ERR_INVALID,
                      "The number of atoms in a Lennard Jones Clusters problem must be positive and greater than 2, "
                      "while a number of "
                          + std::to_string(param) + " was detected.");
            PGX_CHECK(param - 2u <= 0xffffffffull / 3u, PGX_ERR_INVALID,
                      "Overflow caused by the number of atoms requested: " + std::to_string(param));
            *nx = 3u * param - 6u;
            return PGX_OK;
        case PGX_ACKLEY:
            PGX_CHECK(param >= 1u, PGX_ERR_INVALID,
                      "Ackley Function must have minimum 1 dimension, " + std::to_string(param) + " requested");
            *nx = param;
            return PGX_OK;
        case PGX_GRIEWANK:
            PGX_CHECK(param >= 1u, PGX_ERR_INVALID,
                      "Griewank Function must have minimum 1 dimension, " + std::to_string(param) + " requested");
            *nx = param;
            return PGX_OK;
        case PGX_SCHWEFEL:
            PGX_CHECK(param >= 1u, PGX_ERR_INVALID,
                      "Schwefel Function must have minimum 1 dimension, " + std::to_string(param) + " requested");
            *nx = param;
            return PGX_OK;
        default:
            set_error("unknown problem kind " + std::to_string(kind));
            return PGX_ERR_INVALID;
    }
}

// problem::gradient of a UDP without gradient (src/problem.cpp:453-467).
int check_has_gradient(int kind)
{
    PGX_CHECK(kind == PGX_RASTRIGIN || kind == PGX_ROSENBROCK || kind == PGX_LENNARD_JONES, PGX_ERR_NOTIMPL,
              "The gradient has been requested but it is not implemented in the UDP");
    return PGX_OK;
}

// Host-buffer batch evaluation: the rows are cut into chunks; chunk c's
// upload (h2d stream), evaluation (compute stream) and download (d2h stream)
// are chained by events, so uploads, kernels and downloads of consecutive
// chunks overlap. Each row has nx inputs, out_w outputs in fvs and, when
// grads is set, nx gradient entries.
int host_rows(pgx_context *ctx, uint64_t nx, uint64_t out_w, const double *dvs, uint64_t n, double *fvs, double *grads,
              const row_launcher &launch)
{
    PGX_CHECK(dvs != nullptr || n == 0, PGX_ERR_INVALID, "null decision vector buffer");
    PGX_CHECK(fvs != nullptr || grads != nullptr, PGX_ERR_INVALID, "no output buffer");
    if (n == 0) return PGX_OK;
    PGX_CHECK(n <= (uint64_t(1) << 40) / (nx > out_w ? nx : out_w), PGX_ERR_CAPACITY, "batch too large");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    const size_t row_in = nx * sizeof(double), row_out = out_w * sizeof(double);
    PGX_TRY(ctx->d_in.ensure(n * row_in));
    PGX_TRY(ctx->d_out.ensure(n * row_out));
    if (grads) PGX_TRY(ctx->d_grad.ensure(n * row_in));
    double *din = ctx->d_in.as<double>();
    double *dout = ctx->d_out.as<double>();
    double *dgrad = grads ? ctx->d_grad.as<double>() : nullptr;

    uint64_t rows = std::max<uint64_t>(1, kChunkBytes / row_in);
    uint64_t chunks = (n + rows - 1) / rows;
    if (chunks > kMaxChunkEvents / 2) {
        rows = (n + kMaxChunkEvents / 2 - 1) / (kMaxChunkEvents / 2);
        chunks = (n + rows - 1) / rows;
    }
    for (uint64_t c = 0; c < chunks; ++c) {
        const uint64_t r0 = c * rows, r1 = std::min(n, r0 + rows), nr = r1 - r0;
        cudaEvent_t up = ctx->chunk_ev[2 * c], done = ctx->chunk_ev[2 * c + 1];
        PGX_CUDA(cudaMemcpyAsync(din + r0 * nx, dvs + r0 * nx, nr * row_in, cudaMemcpyHostToDevice, ctx->h2d));
        PGX_CUDA(cudaEventRecord(up, ctx->h2d));
        PGX_CUDA(cudaStreamWaitEvent(ctx->stream, up, 0));
        uint64_t l = 0;
        PGX_TRY(launch(din + r0 * nx, nr, dout + r0 * out_w, dgrad ? dgrad + r0 * nx : nullptr, ctx->stream, &l));
        ctx->launches += l;
        PGX_CUDA(cudaEventRecord(done, ctx->stream));
        PGX_CUDA(cudaStreamWaitEvent(ctx->d2h, done, 0));
        if (fvs)
            PGX_CUDA(cudaMemcpyAsync(fvs + r0 * out_w, dout + r0 * out_w, nr * row_out, cudaMemcpyDeviceToHost,
                                     ctx->d2h));
        if (grads)
            PGX_CUDA(cudaMemcpyAsync(grads + r0 * nx, dgrad + r0 * nx, nr * row_in, cudaMemcpyDeviceToHost, ctx->d2h));
    }
    PGX_CUDA(cudaStreamSynchronize(ctx->d2h));
    PGX_CUDA(cudaStreamSynchronize(ctx->stream));
    return PGX_OK;
}

namespace
{

int host_eval(pgx_context *ctx, int kind, uint64_t param, const double *dvs, uint64_t n, double *fvs, double *grads)
{
    uint64_t nx = 0;
    PGX_TRY(problem_nx(kind, param, &nx));
    if (grads) PGX_TRY(check_has_gradient(kind));
    const int num_sms = ctx->num_sms;
    return host_rows(ctx, nx, 1, dvs, n, fvs, grads,
                     [&](const double *din, uint64_t nr, double *dout, double *dgrad, cudaStream_t s, uint64_t *l) {
                         return launch_eval(kind, param, nx, din, nr, dout, dgrad, s, num_sms, l);
                     });
}

struct dev_survival {
    double *points;
    int32_t *rank, *dom_count, *front_offsets, *front_indices, *n_fronts;
    double *crowding;
};

int alloc_survival(pgx_context *ctx, uint64_t n, uint64_t m, bool crowd, dev_survival *d)
{
    auto al = [](size_t b) { return (b + 255u) & ~size_t(255); };
    const size_t bp = al(n * std::max<uint64_t>(m, 1) * sizeof(double));
    const size_t bi = al(n * sizeof(int32_t));
    const size_t bo = al((n + 1) * sizeof(int32_t));
    const size_t bc = crowd ? al(n * sizeof(double)) : 0;
    PGX_TRY(ctx->s_points.ensure(bp + 3 * bi + bo + 256 + bc));
    char *p = ctx->s_points.as<char>();
    d->points = reinterpret_cast<double *>(p);
    p += bp;
    d->rank = reinterpret_cast<int32_t *>(p);
    p += bi;
    d->dom_count = reinterpret_cast<int32_t *>(p);
    p += bi;
    d->front_indices = reinterpret_cast<int32_t *>(p);
    p += bi;
    d->front_offsets = reinterpret_cast<int32_t *>(p);
    p += bo;
    d->n_fronts = reinterpret_cast<int32_t *>(p);
    p += 256;
    d->crowding = crowd ? reinterpret_cast<double *>(p) : nullptr;
    return PGX_OK;
}

int host_survival(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, int32_t *rank, int32_t *dom_count,
                  int32_t *front_offsets, int32_t *front_indices, int32_t *n_fronts, double *crowding)
{
    PGX_CHECK(n >= 2u, PGX_ERR_INVALID,
              "At least two points are needed for fast_non_dominated_sorting: " + std::to_string(n) + " detected.");
    PGX_CHECK(points != nullptr || m == 0, PGX_ERR_INVALID, "null points buffer");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    dev_survival d{};
    PGX_TRY(alloc_survival(ctx, n, m, crowding != nullptr, &d));
    cudaStream_t s = ctx->stream;
    if (m > 0) PGX_CUDA(cudaMemcpyAsync(d.points, points, n * m * sizeof(double), cudaMemcpyHostToDevice, s));
    survival_out o;
    o.rank = d.rank;
    o.dom_count = d.dom_count;
    o.front_offsets = d.front_offsets;
    o.front_indices = d.front_indices;
    o.n_fronts = d.n_fronts;
    o.crowding = d.crowding;
    PGX_TRY(launch_survival(ctx, d.points, n, m, o, s));
    int32_t nf = 0;
    PGX_CUDA(cudaMemcpyAsync(&nf, d.n_fronts, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (rank) PGX_CUDA(cudaMemcpyAsync(rank, d.rank, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (dom_count) PGX_CUDA(cudaMemcpyAsync(dom_count, d.dom_count, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (front_indices)
        PGX_CUDA(cudaMemcpyAsync(front_indices, d.front_indices, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (front_offsets)
        PGX_CUDA(cudaMemcpyAsync(front_offsets, d.front_offsets, (n + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (crowding) PGX_CUDA(cudaMemcpyAsync(crowding, d.crowding, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaStreamSynchronize(s));
    PGX_TRY(read_survival_status(ctx, n, m));
    if (n_fronts) *n_fronts = nf;
    if (crowding && m < 2u) {
        // crowding_distance throws for fewer than two objectives
        // (multi_objective.cpp:290-294); nsga2 only calls it on fronts of three or more points.
        std::vector<int32_t> off(n + 1);
        PGX_CUDA(cudaMemcpy(off.data(), d.front_offsets, (n + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost));
        for (int32_t f = 0; f < nf; ++f) {
            PGX_CHECK(off[f + 1] - off[f] < 3, PGX_ERR_INVALID,
                      "Points in the non dominated front must contain at least two objectives: " + std::to_string(m)
                          + " detected.");
        }
    }
    return PGX_OK;
}

} // namespace
} // namespace pgx

using namespace pgx;

extern "C" {

int pgx_abi_version(void)
{
    return PGX_ABI_VERSION;
}

const char *pgx_build_id(void)
{
    return PGX_BUILD_ID;
}

const char *pgx_last_error(void)
{
    return get_error();
}

int pgx_context_create(int device, pgx_context **out)
{
    PGX_CHECK(out != nullptr, PGX_ERR_INVALID, "null output pointer");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        set_error(std::string("no CUDA device available: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices"));
        return PGX_ERR_NODEVICE;
    }
    PGX_CHECK(device >= 0 && device < count, PGX_ERR_INVALID, "device index out of range");
    auto *ctx = new pgx_context();
    ctx->device = device;
    int st = PGX_OK;
    auto fail = [&](int code) {
        pgx_context_destroy(ctx);
        return code;
    };
    if ((st = use_device(ctx)) != PGX_OK) return fail(st);
    cudaError_t ce = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (ce != cudaSuccess) return fail(cuda_status(ce, "cudaDeviceGetAttribute"));
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
    if (!coop) {
        set_error("device does not support cooperative launches");
        return fail(PGX_ERR_NODEVICE);
    }
    for (cudaStream_t *s : {&ctx->stream, &ctx->h2d, &ctx->d2h}) {
        ce = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
        if (ce != cudaSuccess) return fail(cuda_status(ce, "cudaStreamCreateWithFlags"));
    }
    ctx->chunk_ev.resize(kMaxChunkEvents);
    for (auto &ev : ctx->chunk_ev) {
        ce = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (ce != cudaSuccess) return fail(cuda_status(ce, "cudaEventCreateWithFlags"));
    }
    *out = ctx;
    return PGX_OK;
}

void pgx_context_destroy(pgx_context *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    for (cudaStream_t s : {ctx->stream, ctx->h2d, ctx->d2h})
        if (s) cudaStreamSynchronize(s);
    for (auto &ev : ctx->chunk_ev)
        if (ev) cudaEventDestroy(ev);
    for (pgx::dbuf *b : {&ctx->d_in, &ctx->d_out, &ctx->d_grad, &ctx->s_points,
                         &ctx->s_state, &ctx->s_outs, &ctx->s_crowd, &ctx->r_work, &ctx->h_wfg})
        b->release();
    for (cudaStream_t s : {ctx->stream, ctx->h2d, ctx->d2h})
        if (s) cudaStreamDestroy(s);
    delete ctx;
}

uint64_t pgx_context_launch_count(const pgx_context *ctx)
{
    return ctx ? ctx->launches : 0;
}

int pgx_problem_nx(int kind, uint64_t param, uint64_t *nx)
{
    PGX_CHECK(nx != nullptr, PGX_ERR_INVALID, "null output pointer");
    return problem_nx(kind, param, nx);
}

int pgx_problem_bounds(int kind, uint64_t param, double *lb, double *ub)
{
    uint64_t nx = 0;
    PGX_TRY(problem_nx(kind, param, &nx));
    PGX_CHECK(lb != nullptr && ub != nullptr, PGX_ERR_INVALID, "null bounds buffer");
    for (uint64_t i = 0; i < nx; ++i) {
        if (kind == PGX_RASTRIGIN) {
            lb[i] = -5.12;
            ub[i] = 5.12;
        } else if (kind == PGX_ROSENBROCK) {
            lb[i] = -5.;
            ub[i] = 10.;
        } else if (kind == PGX_ACKLEY) { // ackley.cpp:85-90
            lb[i] = -15.;
            ub[i] = 30.;
        } else if (kind == PGX_GRIEWANK) { // griewank.cpp:84-89
            lb[i] = -600.;
            ub[i] = 600.;
        } else if (kind == PGX_SCHWEFEL) { // schwefel.cpp:78-83
            lb[i] = -500.;
            ub[i] = 500.;
        } else {
            const bool z = i != 0u && i % 3u == 0u;
            lb[i] = z ? 0.0 : -3.0;
            ub[i] = z ? 6.0 : 3.0;
        }
    }
    return PGX_OK;
}

int pgx_batch_fitness(pgx_context *ctx, int kind, uint64_t param, const double *dvs, uint64_t n_dvs, double *fvs)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(fvs != nullptr || n_dvs == 0, PGX_ERR_INVALID, "null fitness buffer");
    if (n_dvs == 0) return PGX_OK;
    return host_eval(ctx, kind, param, dvs, n_dvs, fvs, nullptr);
}

int pgx_batch_gradient(pgx_context *ctx, int kind, uint64_t param, const double *dvs, uint64_t n_dvs, double *fvs,
                       double *grads)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(grads != nullptr || n_dvs == 0, PGX_ERR_INVALID, "null gradient buffer");
    if (n_dvs == 0) return PGX_OK;
    return host_eval(ctx, kind, param, dvs, n_dvs, fvs, grads);
}

int pgx_batch_eval_device(pgx_context *ctx, int kind, uint64_t param, const double *d_dvs, uint64_t n_dvs,
                          double *d_fvs, double *d_grads, void *stream)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    uint64_t nx = 0;
    PGX_TRY(problem_nx(kind, param, &nx));
    if (d_grads) PGX_TRY(check_has_gradient(kind));
    PGX_CHECK(d_fvs != nullptr || d_grads != nullptr, PGX_ERR_INVALID, "no output buffer");
    if (n_dvs == 0) return PGX_OK;
    PGX_CHECK(d_dvs != nullptr, PGX_ERR_INVALID, "null decision vector buffer");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint64_t l = 0;
    PGX_TRY(launch_eval(kind, param, nx, d_dvs, n_dvs, d_fvs, d_grads, s, ctx->num_sms, &l));
    ctx->launches += l;
    return PGX_OK;
}

int pgx_fnds(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, int32_t *rank, int32_t *dom_count,
             int32_t *front_offsets, int32_t *front_indices, int32_t *n_fronts)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    return host_survival(ctx, points, n, m, rank, dom_count, front_offsets, front_indices, n_fronts, nullptr);
}

int pgx_nsga2_survival(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, int32_t *rank,
                       int32_t *dom_count, int32_t *front_offsets, int32_t *front_indices, int32_t *n_fronts,
                       double *crowding)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(crowding != nullptr, PGX_ERR_INVALID, "null crowding buffer");
    return host_survival(ctx, points, n, m, rank, dom_count, front_offsets, front_indices, n_fronts, crowding);
}

int pgx_nsga2_survival_device(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m, int32_t *d_rank,
                              int32_t *d_dom_count, int32_t *d_front_offsets, int32_t *d_front_indices,
                              int32_t *d_n_fronts, double *d_crowding, void *stream)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(d_crowding == nullptr || m >= 2u, PGX_ERR_INVALID,
              "Points in the non dominated front must contain at least two objectives: " + std::to_string(m)
                  + " detected.");
    PGX_CHECK(d_rank && d_dom_count && d_front_offsets && d_front_indices && d_n_fronts, PGX_ERR_INVALID,
              "null output buffer");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    survival_out o;
    o.rank = d_rank;
    o.dom_count = d_dom_count;
    o.front_offsets = d_front_offsets;
    o.front_indices = d_front_indices;
    o.n_fronts = d_n_fronts;
    o.crowding = d_crowding;
    return launch_survival(ctx, d_points, n, m, o, s);
}

int pgx_crowding_distance(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, double *out)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(n >= 2u, PGX_ERR_INVALID,
              "A non dominated front must contain at least two points: " + std::to_string(n) + " detected.");
    PGX_CHECK(m >= 2u, PGX_ERR_INVALID,
              "Points in the non dominated front must contain at least two objectives: " + std::to_string(m)
                  + " detected.");
    PGX_CHECK(points != nullptr && out != nullptr, PGX_ERR_INVALID, "null buffer");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    PGX_TRY(ctx->s_crowd.ensure(n * m * sizeof(double) + ((n * sizeof(double) + 255u) & ~size_t(255)) + 256));
    double *dp = ctx->s_crowd.as<double>();
    double *dout = reinterpret_cast<double *>(ctx->s_crowd.as<char>() + ((n * m * sizeof(double) + 255u) & ~size_t(255)));
    cudaStream_t s = ctx->stream;
    PGX_CUDA(cudaMemcpyAsync(dp, points, n * m * sizeof(double), cudaMemcpyHostToDevice, s));
    PGX_TRY(launch_crowding_single(ctx, dp, n, m, dout, s));
    PGX_CUDA(cudaMemcpyAsync(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaStreamSynchronize(s));
    return read_mo_status(ctx, n, m);
}

int pgx_select_best_n_mo(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, uint64_t N, int32_t *out,
                         uint64_t *n_out)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(n_out != nullptr, PGX_ERR_INVALID, "null count pointer");
    const uint64_t cnt = N < n ? N : n;
    *n_out = 0;
    PGX_CHECK(out != nullptr || cnt == 0, PGX_ERR_INVALID, "null output buffer");
    PGX_CHECK(points != nullptr || n * m == 0, PGX_ERR_INVALID, "null points buffer");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    const size_t bp = (n * m * sizeof(double) + 255u) & ~size_t(255);
    PGX_TRY(ctx->s_crowd.ensure(bp + n * sizeof(int32_t) + 256));
    double *dp = ctx->s_crowd.as<double>();
    int32_t *dout = reinterpret_cast<int32_t *>(ctx->s_crowd.as<char>() + bp);
    cudaStream_t s = ctx->stream;
    if (n * m) PGX_CUDA(cudaMemcpyAsync(dp, points, n * m * sizeof(double), cudaMemcpyHostToDevice, s));
    PGX_TRY(launch_select_best(ctx, dp, n, m, N, dout, nullptr, s));
    if (cnt) PGX_CUDA(cudaMemcpyAsync(out, dout, cnt * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaStreamSynchronize(s));
    if (n >= 2 && N > 0 && N < n) PGX_TRY(read_mo_status(ctx, n, m));
    *n_out = cnt;
    return PGX_OK;
}

int pgx_sort_population_mo(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, int32_t *out)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(out != nullptr || n == 0, PGX_ERR_INVALID, "null output buffer");
    PGX_CHECK(points != nullptr || n * m == 0, PGX_ERR_INVALID, "null points buffer");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    const size_t bp = (n * m * sizeof(double) + 255u) & ~size_t(255);
    PGX_TRY(ctx->s_crowd.ensure(bp + n * sizeof(int32_t) + 256));
    double *dp = ctx->s_crowd.as<double>();
    int32_t *dout = reinterpret_cast<int32_t *>(ctx->s_crowd.as<char>() + bp);
    cudaStream_t s = ctx->stream;
    if (n * m) PGX_CUDA(cudaMemcpyAsync(dp, points, n * m * sizeof(double), cudaMemcpyHostToDevice, s));
    PGX_TRY(launch_sort_population(ctx, dp, n, m, dout, nullptr, s));
    if (n) PGX_CUDA(cudaMemcpyAsync(out, dout, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaStreamSynchronize(s));
    if (n >= 2) PGX_TRY(read_mo_status(ctx, n, m));
    return PGX_OK;
}

int pgx_select_best_n_mo_device(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m, uint64_t N,
                                int32_t *d_out, int32_t *d_status, void *stream)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(d_out != nullptr || N == 0 || n == 0, PGX_ERR_INVALID, "null output buffer");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    return launch_select_best(ctx, d_points, n, m, N, d_out, d_status, static_cast<cudaStream_t>(stream));
}

int pgx_sort_population_mo_device(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m, int32_t *d_out,
                                  int32_t *d_status, void *stream)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(d_out != nullptr || n == 0, PGX_ERR_INVALID, "null output buffer");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    return launch_sort_population(ctx, d_points, n, m, d_out, d_status, static_cast<cudaStream_t>(stream));
}

int pgx_std_sort_i64(pgx_context *ctx, int64_t *keys, int32_t *values, uint64_t n)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK((keys != nullptr && values != nullptr) || n == 0, PGX_ERR_INVALID, "null buffer");
    if (n < 2) return PGX_OK;
    PGX_CHECK(n <= (1ull << 30), PGX_ERR_CAPACITY, "sort: more than 2^30 elements");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    const size_t bk = (n * sizeof(int64_t) + 255u) & ~size_t(255);
    const size_t bv = (n * sizeof(int32_t) + 255u) & ~size_t(255);
    const size_t bl = (n * 2u * sizeof(int32_t) + 255u) & ~size_t(255);
    const size_t bs = (sort_pairs_state_bytes() + 255u) & ~size_t(255);
    PGX_TRY(ctx->s_crowd.ensure(bk + bv + 2u * bl + 256 + bs));
    char *base = ctx->s_crowd.as<char>();
    void *dstate = base + bk + bv + 2u * bl + 256;
    long long *dk = reinterpret_cast<long long *>(base);
    int32_t *dv = reinterpret_cast<int32_t *>(base + bk);
    int2 *dl = reinterpret_cast<int2 *>(base + bk + bv);
    int32_t *dpos = reinterpret_cast<int32_t *>(base + bk + bv + bl);
    int *derr = reinterpret_cast<int *>(base + bk + bv + 2u * bl);
    cudaStream_t s = ctx->stream;
    PGX_CUDA(cudaMemsetAsync(derr, 0, sizeof(int), s));
    PGX_CUDA(cudaMemcpyAsync(dk, keys, n * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    PGX_CUDA(cudaMemcpyAsync(dv, values, n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    PGX_TRY(launch_sort_pairs(ctx, dk, dv, n, derr, dl, dpos, dstate, s));
    int err = 0;
    PGX_CUDA(cudaMemcpyAsync(keys, dk, n * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaMemcpyAsync(values, dv, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaMemcpyAsync(&err, derr, sizeof(int), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaStreamSynchronize(s));
    PGX_CHECK(err == 0, PGX_ERR_CUDA, "device sort: internal error " + std::to_string(err));
    return PGX_OK;
}

int pgx_selftest_barrier_timeout(pgx_context *ctx, uint64_t spin_limit, int32_t *timed_out)
{
    PGX_CHECK(ctx != nullptr && timed_out != nullptr, PGX_ERR_INVALID, "null argument");
    PGX_CHECK(spin_limit >= 1u && spin_limit <= (uint64_t(1) << 24), PGX_ERR_INVALID,
              "spin limit out of range [1, 2^24]");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    return run_barrier_timeout_test(ctx, spin_limit, timed_out);
}

int pgx_selftest_lj_reciprocal(pgx_context *ctx, const double *d, uint64_t n, double *inv, double *inv_cube)
{
    PGX_CHECK(ctx != nullptr && (n == 0 || (d != nullptr && inv != nullptr)), PGX_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    return run_lj_reciprocal(ctx, d, n, inv, inv_cube);
}

int pgx_fnds_dom_list(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, int64_t *dl_offsets,
                      int32_t *dl_indices, uint64_t capacity, uint64_t *dl_total)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(n >= 2u, PGX_ERR_INVALID,
              "At least two points are needed for fast_non_dominated_sorting: " + std::to_string(n) + " detected.");
    PGX_CHECK(dl_offsets != nullptr && dl_total != nullptr, PGX_ERR_INVALID, "null output buffer");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    cudaStream_t s = ctx->stream;
    PGX_TRY(ctx->s_crowd.ensure(n * std::max<uint64_t>(m, 1) * sizeof(double)));
    double *dp = ctx->s_crowd.as<double>();
    if (m > 0) PGX_CUDA(cudaMemcpyAsync(dp, points, n * m * sizeof(double), cudaMemcpyHostToDevice, s));
    int64_t *dcnt = nullptr;
    PGX_TRY(build_dominates_rows(ctx, dp, n, m, &dcnt, s));
    std::vector<int64_t> cnt(n);
    PGX_CUDA(cudaMemcpyAsync(cnt.data(), dcnt, n * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaStreamSynchronize(s));
    dl_offsets[0] = 0;
    for (uint64_t i = 0; i < n; ++i) dl_offsets[i + 1] = dl_offsets[i] + cnt[i];
    const uint64_t total = static_cast<uint64_t>(dl_offsets[n]);
    *dl_total = total;
    PGX_CHECK(total <= capacity, PGX_ERR_CAPACITY,
              "dom_list needs " + std::to_string(total) + " entries, capacity is " + std::to_string(capacity));
    if (total == 0) return PGX_OK;
    PGX_CHECK(dl_indices != nullptr, PGX_ERR_INVALID, "null dom_list index buffer");
    PGX_TRY(ctx->d_out.ensure((n + 1) * sizeof(int64_t)));
    PGX_TRY(ctx->d_grad.ensure(total * sizeof(int32_t)));
    PGX_CUDA(cudaMemcpyAsync(ctx->d_out.ptr, dl_offsets, (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    PGX_TRY(extract_dom_list(ctx, n, m, ctx->d_out.as<int64_t>(), ctx->d_grad.as<int32_t>(), s));
    PGX_CUDA(cudaMemcpyAsync(dl_indices, ctx->d_grad.ptr, total * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaStreamSynchronize(s));
    return PGX_OK;
}

} // extern "C"
