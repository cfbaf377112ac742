// Batched gradient-based local refinement: monotonic basin hopping (the
// scheme of pagmo's mbh, src/algorithms/mbh.cpp:102-200) run on every
// individual of a batch at once, with a projected-gradient descent driven by
// the batched adjoint as the inner local optimiser.
//
// Per individual (one group of lanes, a warp for lennard_jones), all in one
// launch:
//   x_best = the starting point, f_best = f(x_best)
//   trial t = 0, 1, ... while t < hops and fewer than `stop` trials in a row
//   failed to improve (mbh's stop):
//     x = uniform in [max(x_best - p (ub - lb), lb), min(x_best + p (ub - lb), ub)]
//         per coordinate (mbh.cpp:164-170; p = perturb), from a counter-based
//         generator keyed by (seed, individual, trial, coordinate)
//     `steps` projected-gradient steps from x: with s = ub - lb and
//         d = s * g(x) (the gradient in box-scaled coordinates), the trial
//         point is clamp(x - eta * s * d / |d|, lb, ub); it replaces x when its
//         fitness is lower (eta doubles, up to 1), else eta halves; the descent
//         ends early when eta < step_min or d = 0
//     x_best, f_best = x, f(x) when f(x) < f_best (monotonic acceptance)
// Every fitness and gradient comes from the same row routines as the batch
// evaluation (fitness_dev.cuh); one evaluation = one fitness + gradient. The
// loop's own arithmetic is rounded operation by operation (no contraction into
// FMAs) and |d|^2 is summed lane by lane (element i in lane i mod L, then the
// lanes' butterfly), so that a host restatement fed the same fitness and
// gradient values reproduces it bit for bit.
//
// mbh itself perturbs and re-optimises a whole population with an inner
// pagmo algorithm and accepts the population when its best improves; here each
// individual is its own chain, which is what lets the whole batch refine at
// once on the GPU.
#include "fitness_dev.cuh"
#include "pgx_internal.cuh"

#include <string>

namespace pgx
{
namespace
{
using namespace dev;

struct refine_args {
    double *x;                 // n x nx: in the starting points, out the best points
    double *f;                 // n: out the best fitness
    double *work;              // n x 4 nx: current point, trial point, their gradients
    double *fslot;             // n x 2: fitness of the current and the trial point
    unsigned long long *evals; // total evaluations (accumulated)
    uint64_t n;
    uint32_t nx, na;
    uint32_t hops, stop, steps;
    double perturb, step0, step_min;
    uint64_t seed;
};

// Bounds of coordinate i, as pgx_problem_bounds gives them (rastrigin.cpp:80-85,
// rosenbrock.cpp:72-75, lennard_jones.cpp:99-113).
template <int KIND>
__device__ __forceinline__ void refine_bounds(uint32_t i, double &lo, double &hi)
{
    if constexpr (KIND == PGX_RASTRIGIN) {
        lo = -5.12;
        hi = 5.12;
    } else if constexpr (KIND == PGX_ROSENBROCK) {
        lo = -5.;
        hi = 10.;
    } else {
        const bool z = i != 0u && i % 3u == 0u;
        lo = z ? 0.0 : -3.0;
        hi = z ? 6.0 : 3.0;
    }
}

// splitmix64's finaliser (Steele, Lea and Flood, 2014)
__device__ __forceinline__ uint64_t refine_mix(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Uniform [0, 1) with 53 random bits, a function of (seed, individual, trial,
// coordinate) only.
__device__ __forceinline__ double refine_uniform(uint64_t seed, uint64_t row, uint32_t trial, uint32_t coord)
{
    const uint64_t h =
        refine_mix(refine_mix(seed ^ refine_mix(row)) ^ ((static_cast<uint64_t>(trial) << 32) | coord));
    return static_cast<double>(h >> 11) * 0x1.0p-53;
}

template <int KIND, int L, int V, int LJV>
__device__ __forceinline__ void refine_eval(const double *xr, uint32_t nx, uint32_t na, double *sm, double *fo,
                                            double *gr)
{
    if constexpr (KIND == PGX_RASTRIGIN) {
        rastrigin_row<V, L, true>(xr, nx, fo, gr);
    } else if constexpr (KIND == PGX_ROSENBROCK) {
        rosenbrock_row<L, true>(xr, nx, fo, gr);
    } else if constexpr (LJV == 0) {
        lj_cluster_reg<1, true>(xr, na, nx, sm, fo, gr);
    } else {
        lj_cluster_flat<true>(xr, na, nx, sm, fo, gr);
    }
}

template <int KIND, int L, int V, int LJV>
__global__ void __launch_bounds__(128) refine_kernel(refine_args a)
{
    extern __shared__ double smem[];
    const unsigned sub = threadIdx.x & (L - 1);
    const unsigned mask = group_mask<L>();
    double *sm = KIND == PGX_LENNARD_JONES ? smem + static_cast<size_t>(threadIdx.x >> 5) * 6u * a.na : nullptr;
    const uint32_t nx = a.nx;
    const uint64_t per_block = blockDim.x / L;
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * per_block;
    for (uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / L; row < a.n;
         row += stride) {
        double *xb = a.x + row * nx;
        double *xc = a.work + row * 4u * nx;
        double *xt = xc + nx;
        double *gc = xt + nx;
        double *gt = gc + nx;
        double *fs = a.fslot + 2u * row;
        refine_eval<KIND, L, V, LJV>(xb, nx, a.na, sm, fs, gt);
        __syncwarp(mask);
        double fb = __ldcg(fs);
        unsigned long long evals = 1;
        uint32_t failed = 0;
        for (uint32_t trial = 0; trial < a.hops && failed < a.stop; ++trial) {
            for (uint32_t i = sub; i < nx; i += L) {
                double lo, hi;
                refine_bounds<KIND>(i, lo, hi);
                const double w = __dmul_rn(a.perturb, __dsub_rn(hi, lo));
                const double xl = fmax(__dsub_rn(xb[i], w), lo), xu = fmin(__dadd_rn(xb[i], w), hi);
                xc[i] = __dadd_rn(xl, __dmul_rn(__dsub_rn(xu, xl), refine_uniform(a.seed, row, trial, i)));
            }
            __syncwarp(mask);
            refine_eval<KIND, L, V, LJV>(xc, nx, a.na, sm, fs, gc);
            __syncwarp(mask);
            double fc = __ldcg(fs);
            ++evals;
            double eta = a.step0;
            for (uint32_t k = 0; k < a.steps && eta >= a.step_min; ++k) {
                double q = 0.0;
                for (uint32_t i = sub; i < nx; i += L) {
                    double lo, hi;
                    refine_bounds<KIND>(i, lo, hi);
                    const double d = __dmul_rn(__dsub_rn(hi, lo), gc[i]);
                    q = __dadd_rn(q, __dmul_rn(d, d));
                }
                q = group_sum<L>(q, mask);
                if (!(q > 0.0) || !isfinite(q)) break; // stationary, or no finite direction
                const double c = eta / sqrt(q);
                for (uint32_t i = sub; i < nx; i += L) {
                    double lo, hi;
                    refine_bounds<KIND>(i, lo, hi);
                    const double s = __dsub_rn(hi, lo);
                    const double t = __dmul_rn(__dmul_rn(c, s), __dmul_rn(s, gc[i]));
                    xt[i] = fmin(fmax(__dsub_rn(xc[i], t), lo), hi);
                }
                __syncwarp(mask);
                refine_eval<KIND, L, V, LJV>(xt, nx, a.na, sm, fs + 1, gt);
                __syncwarp(mask);
                const double ft = __ldcg(fs + 1);
                ++evals;
                if (ft < fc) {
                    double *t = xc;
                    xc = xt;
                    xt = t;
                    t = gc;
                    gc = gt;
                    gt = t;
                    fc = ft;
                    eta = fmin(2.0 * eta, 1.0);
                } else {
                    eta *= 0.5;
                }
            }
            if (fc < fb) {
                for (uint32_t i = sub; i < nx; i += L) xb[i] = xc[i];
                fb = fc;
                failed = 0;
            } else {
                ++failed;
            }
            __syncwarp(mask);
        }
        if (sub == 0) {
            a.f[row] = fb;
            atomicAdd(a.evals, evals);
        }
    }
}

template <typename K>
int launch_refine_kernel(K kernel, int lanes, size_t smem_per_warp, const refine_args &a, int num_sms,
                         cudaStream_t s)
{
    int warps = 4;
    if (smem_per_warp) {
        warps = static_cast<int>((96u * 1024u) / smem_per_warp);
        warps = warps > 4 ? 4 : (warps < 1 ? 1 : warps);
    }
    const int threads = 32 * warps;
    const size_t smem = smem_per_warp * static_cast<size_t>(warps);
    PGX_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem > 48u * 1024u ? smem : 48u * 1024u)));
    int occ = 0;
    PGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem));
    if (occ < 1) occ = 1;
    const uint64_t per_block = static_cast<uint64_t>(threads / lanes);
    const uint64_t need = (a.n + per_block - 1) / per_block;
    const uint64_t cap = static_cast<uint64_t>(num_sms) * static_cast<uint64_t>(occ);
    const int grid = static_cast<int>(need < cap ? (need ? need : 1) : cap);
    kernel<<<grid, threads, smem, s>>>(a);
    PGX_CUDA(cudaGetLastError());
    return PGX_OK;
}

int launch_refine(int kind, const refine_args &a, int num_sms, cudaStream_t s)
{
    if (kind == PGX_LENNARD_JONES) {
        const size_t per_warp = 6u * static_cast<size_t>(a.na) * sizeof(double);
        PGX_CHECK(per_warp <= 96u * 1024u, PGX_ERR_CAPACITY, "refinement: too many atoms for one cluster per warp");
        if (a.na <= 32u)
            return launch_refine_kernel(refine_kernel<PGX_LENNARD_JONES, 32, 32, 0>, 32, per_warp, a, num_sms, s);
        return launch_refine_kernel(refine_kernel<PGX_LENNARD_JONES, 32, 32, 1>, 32, per_warp, a, num_sms, s);
    }
    const int own = lanes_per_row(a.nx);
    if (kind == PGX_RASTRIGIN) {
        switch (rastrigin_width(own)) {
            case 8: return launch_refine_kernel(refine_kernel<PGX_RASTRIGIN, 8, 8, 0>, 8, 0, a, num_sms, s);
            case 16: return launch_refine_kernel(refine_kernel<PGX_RASTRIGIN, 16, 16, 0>, 16, 0, a, num_sms, s);
            default: return launch_refine_kernel(refine_kernel<PGX_RASTRIGIN, 32, 32, 0>, 32, 0, a, num_sms, s);
        }
    }
    switch (own) {
        case 32: return launch_refine_kernel(refine_kernel<PGX_ROSENBROCK, 32, 32, 0>, 32, 0, a, num_sms, s);
        case 16: return launch_refine_kernel(refine_kernel<PGX_ROSENBROCK, 16, 32, 0>, 16, 0, a, num_sms, s);
        case 8: return launch_refine_kernel(refine_kernel<PGX_ROSENBROCK, 8, 32, 0>, 8, 0, a, num_sms, s);
        case 4: return launch_refine_kernel(refine_kernel<PGX_ROSENBROCK, 4, 32, 0>, 4, 0, a, num_sms, s);
        case 2: return launch_refine_kernel(refine_kernel<PGX_ROSENBROCK, 2, 32, 0>, 2, 0, a, num_sms, s);
        default: return launch_refine_kernel(refine_kernel<PGX_ROSENBROCK, 1, 32, 0>, 1, 0, a, num_sms, s);
    }
}

int check_refine(int kind, uint64_t param, const pgx_refine_params *p, uint64_t *nx)
{
    PGX_CHECK(p != nullptr, PGX_ERR_INVALID, "null refinement parameters");
    PGX_TRY(problem_nx(kind, param, nx));
    PGX_CHECK(kind == PGX_RASTRIGIN || kind == PGX_ROSENBROCK || kind == PGX_LENNARD_JONES, PGX_ERR_NOTIMPL,
              "The gradient has been requested but it is not implemented in the UDP");
    // mbh's own check (src/algorithms/mbh.cpp:58-71): perturbation in ]0, 1]
    PGX_CHECK(p->perturb > 0.0 && p->perturb <= 1.0, PGX_ERR_INVALID,
              "The perturbation must be in ]0,1], while a value of " + std::to_string(p->perturb)
                  + " was detected.");
    PGX_CHECK(p->step0 > 0.0 && p->step0 <= 1.0 && p->step_min > 0.0 && p->step_min <= p->step0, PGX_ERR_INVALID,
              "refinement: need 0 < step_min <= step0 <= 1");
    PGX_CHECK(*nx < (1ull << 31), PGX_ERR_CAPACITY, "decision vector dimension exceeds 2^31-1");
    return PGX_OK;
}

// The refinement of n individuals on device buffers (working points and
// gradients in the context's grow-only buffer), asynchronous on s.
int refine_device(pgx_context *ctx, int kind, uint64_t param, uint64_t nx, const pgx_refine_params *p, double *d_x,
                  uint64_t n, double *d_f, unsigned long long *d_evals, cudaStream_t s)
{
    const size_t b_work = ((4u * n * nx * sizeof(double)) + 255u) & ~size_t(255);
    PGX_TRY(ctx->r_work.ensure(b_work + 2u * n * sizeof(double)));
    refine_args a{};
    a.x = d_x;
    a.f = d_f;
    a.work = ctx->r_work.as<double>();
    a.fslot = reinterpret_cast<double *>(ctx->r_work.as<char>() + b_work);
    a.evals = d_evals;
    a.n = n;
    a.nx = static_cast<uint32_t>(nx);
    a.na = kind == PGX_LENNARD_JONES ? static_cast<uint32_t>(param) : 0u;
    a.hops = p->hops;
    a.stop = p->stop;
    a.steps = p->steps;
    a.perturb = p->perturb;
    a.step0 = p->step0;
    a.step_min = p->step_min;
    a.seed = p->seed;
    PGX_TRY(launch_refine(kind, a, ctx->num_sms, s));
    ++ctx->launches;
    return PGX_OK;
}

} // namespace
} // namespace pgx

using namespace pgx;

extern "C" {

int pgx_refine_batch_device(pgx_context *ctx, int kind, uint64_t param, const pgx_refine_params *params, double *d_dvs,
                            uint64_t n_dvs, double *d_fvs, unsigned long long *d_evals, void *stream)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    uint64_t nx = 0;
    PGX_TRY(check_refine(kind, param, params, &nx));
    if (n_dvs == 0) return PGX_OK;
    PGX_CHECK(d_dvs != nullptr && d_fvs != nullptr && d_evals != nullptr, PGX_ERR_INVALID, "null buffer");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    return refine_device(ctx, kind, param, nx, params, d_dvs, n_dvs, d_fvs, d_evals,
                         static_cast<cudaStream_t>(stream));
}

int pgx_refine_batch(pgx_context *ctx, int kind, uint64_t param, const pgx_refine_params *params, double *dvs,
                     uint64_t n_dvs, double *fvs, uint64_t *evals)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    uint64_t nx = 0;
    PGX_TRY(check_refine(kind, param, params, &nx));
    if (evals) *evals = 0;
    if (n_dvs == 0) return PGX_OK;
    PGX_CHECK(dvs != nullptr && fvs != nullptr, PGX_ERR_INVALID, "null buffer");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    cudaStream_t s = ctx->stream;
    const size_t bx = n_dvs * nx * sizeof(double);
    const size_t bf = (n_dvs * sizeof(double) + 255u) & ~size_t(255);
    PGX_TRY(ctx->d_in.ensure(bx));
    PGX_TRY(ctx->d_out.ensure(bf + sizeof(unsigned long long)));
    double *dx = ctx->d_in.as<double>();
    double *df = ctx->d_out.as<double>();
    auto *dev_evals = reinterpret_cast<unsigned long long *>(ctx->d_out.as<char>() + bf);
    PGX_CUDA(cudaMemcpyAsync(dx, dvs, bx, cudaMemcpyHostToDevice, s));
    PGX_CUDA(cudaMemsetAsync(dev_evals, 0, sizeof(unsigned long long), s));
    PGX_TRY(refine_device(ctx, kind, param, nx, params, dx, n_dvs, df, dev_evals, s));
    PGX_CUDA(cudaMemcpyAsync(dvs, dx, bx, cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaMemcpyAsync(fvs, df, n_dvs * sizeof(double), cudaMemcpyDeviceToHost, s));
    unsigned long long e = 0;
    PGX_CUDA(cudaMemcpyAsync(&e, dev_evals, sizeof(e), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaStreamSynchronize(s));
    if (evals) *evals = e;
    return PGX_OK;
}

} // extern "C"
