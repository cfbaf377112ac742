// Multi-objective test problems ZDT (src/problems/zdt.cpp) and DTLZ
// (src/problems/dtlz.cpp): batch fitness and p_distance on the GPU, FP64.
//
// One group of G lanes evaluates one row (grid-stride over rows). The lanes
// split the row's distance function g (a sum over most of the row) and reduce
// it with shuffles; the objectives are then formed from g as the reference
// forms them. DTLZ1-6 objective i is the left-to-right product
// (1 + g) c_0 c_1 ... c_{m-2-i} s_{m-1-i}: the lanes compute the c_j, s_j
// (the sin/cos work) in parallel and the group walks the running product
// once, in the reference's order, each lane writing the objectives whose s it
// holds. Sums are reduced in a different order than the reference's running
// sums (differences of a few units of the last place of the summed
// magnitudes); every product, quotient and square root is the reference's.
#include "fitness_dev.cuh"
#include "pgx_internal.cuh"

#include <climits>
#include <string>

namespace pgx
{
namespace
{
using dev::cos_2pi;
using dev::fast_trig_arg;
using dev::group_mask;
using dev::group_sum;
using dev::signed_const;

// The reference's pi and pi/2 (include/pagmo/detail/constants.hpp:37-44).
constexpr double kPi = 3.1415926535897932384626433832795028841971693993;
constexpr double kPiHalf = kPi / 2.;

// cos(2 pi t) with its sign applied: the integer fixed-point routine for
// 2^-60 <= |t| < 2^40 (trig_fixed.h), else the FP64 polynomial or cospi.
__device__ __forceinline__ double cos_2pi_signed(double t)
{
    if (trigfx::in_range(t)) return trigfx::cos_2pi(t);
    if (!fast_trig_arg(t)) return cospi(t + t);
    int neg = 0;
    const double c = cos_2pi(t, neg);
    return signed_const(c, neg);
}

// sin and cos of the reference's argument: a * (pi/2) rounded once to a
// double (dtlz.cpp:303-314, 332-343 and 373-384 evaluate std::cos(a *
// detail::pi_half())), then sin and cos of that double. Evaluating the exact
// angle instead would give cos = 0 at a = 1 where the reference has
// cos(fl(pi/2)) = 6.1e-17: individuals at the upper bound, which the variation
// operators produce by clamping, would then tie where the reference ranks them
// by g, and pagmo's algorithms would take other decisions.
__device__ __forceinline__ void sincos_half_pi(double a, double &s, double &c)
{
    sincos(__dmul_rn(a, kPiHalf), &s, &c);
}

template <int G>
__device__ __forceinline__ uint32_t group_sum_u32(uint32_t v, unsigned mask)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, G);
    return v;
}

// ------------------------------------------------------------------- ZDT

// ID: the ZDT problem (1-6). pd: write p_distance (n values) instead of the
// two objectives (n x 2).
template <int G, int ID>
__global__ void __launch_bounds__(256) zdt_kernel(const double *__restrict__ x, uint64_t n, uint32_t nx, bool pd,
                                                  double *__restrict__ out)
{
    const unsigned sub = threadIdx.x & (G - 1);
    const unsigned mask = group_mask<G>();
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * (blockDim.x / G);
    for (uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / G; row < n; row += stride) {
        const double *xr = x + row * nx;
        if constexpr (ID == 5) {
            // ZDT5 (zdt.cpp:298-339; p_distance :384-421): counts of ones of
            // the rounded (floored for p_distance) string, integer sums.
            uint32_t u0 = 0, gv = 0;
            if (!pd)
                for (uint32_t i = sub; i < 30u; i += G) u0 += round(__ldg(xr + i)) == 1.0 ? 1u : 0u;
            const uint32_t nb = (nx - 30u) / 5u;
            for (uint32_t b = sub; b < nb; b += G) {
                uint32_t u = 0;
                const double *xb = xr + 30u + 5u * b;
#pragma unroll
                for (int j = 0; j < 5; ++j) {
                    const double v = __ldg(xb + j);
                    u += (pd ? floor(v) : round(v)) == 1.0 ? 1u : 0u;
                }
                gv += u < 5u ? 2u + u : 1u;
            }
            u0 = group_sum_u32<G>(u0, mask);
            gv = group_sum_u32<G>(gv, mask);
            if (sub == 0) {
                const double g = static_cast<double>(gv);
                if (pd) {
                    out[row] = g - static_cast<double>(nb + 1u) + 1;
                } else {
                    const double f0 = 1.0 + static_cast<double>(u0);
                    out[2 * row] = f0;
                    out[2 * row + 1] = g * (1. / f0);
                }
            }
            continue;
        } else {
            // sum over x[1..nx-1]: of x (ZDT1-3, 6) in an integer accumulator
            // (isum.h: within 2^-60 of the largest term per addition, rounded
            // once); of x^2 and cos(4 pi x) (ZDT4) in FP64, where the
            // fixed-point cosine already loads the integer pipes
            isum::sg_acc a1 = isum::make_signed();
            double s1 = 0.0, s2 = 0.0;
#pragma unroll 4
            for (uint32_t i = sub + 1u; i < nx; i += G) {
                const double xi = __ldg(xr + i);
                if constexpr (ID == 4) {
                    s1 = fma(xi, xi, s1);
                    s2 += cos_2pi_signed(xi + xi);
                } else {
                    isum::add_value(a1, xi);
                }
            }
            if constexpr (ID == 4) {
                s1 = group_sum<G>(s1, mask);
                s2 = group_sum<G>(s2, mask);
            } else {
                s1 = isum::value(dev::group_ssum<G>(a1, mask));
            }
            if (sub != 0) continue;
            const double x0 = __ldg(xr);
            const double nm1 = static_cast<double>(nx - 1u);
            if constexpr (ID == 4) {
                // zdt.cpp:281-296 / :371-382
                const double s = fma(-10.0, s2, s1);
                if (pd) {
                    out[row] = (1. + 10. * nm1 + s) - 1.;
                } else {
                    const double g = (1 + 10 * nm1) + s;
                    out[2 * row] = x0;
                    out[2 * row + 1] = g * (1. - sqrt(x0 / g));
                }
            } else if constexpr (ID == 6) {
                // zdt.cpp:341-356 / :423-434
                const double g = 1 + 9 * pow((s1 / nm1), 0.25);
                if (pd) {
                    out[row] = g - 1;
                } else {
                    const double f0 = 1 - exp(-4 * x0) * pow(sin(6 * kPi * x0), 6.0);
                    out[2 * row] = f0;
                    out[2 * row + 1] = g * (1 - (f0 / g) * (f0 / g));
                }
            } else {
                // zdt.cpp:233-279 / :358-369
                const double g = 1. + (9. * s1) / nm1;
                if (pd) {
                    out[row] = g - 1.;
                } else {
                    const double r = x0 / g;
                    double f1;
                    if constexpr (ID == 1)
                        f1 = g * (1. - sqrt(r));
                    else if constexpr (ID == 2)
                        f1 = g * (1. - r * r);
                    else
                        f1 = g * (1. - sqrt(r) - r * sin(10. * kPi * x0));
                    out[2 * row] = x0;
                    out[2 * row + 1] = f1;
                }
            }
        }
    }
}

// ------------------------------------------------------------------ DTLZ

// ID: the DTLZ problem (1-7); m objectives; pd: write the distance function
// g(x_M) (p_distance, dtlz.cpp:411-420) instead of the m objectives.
template <int G, int ID>
__global__ void __launch_bounds__(256) dtlz_kernel(const double *__restrict__ x, uint64_t n, uint32_t nx, uint32_t m,
                                                   uint32_t alpha, bool pd, double *__restrict__ out)
{
    const unsigned sub = threadIdx.x & (G - 1);
    const unsigned mask = group_mask<G>();
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * (blockDim.x / G);
    const uint32_t k = nx - (m - 1u);
    for (uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / G; row < n; row += stride) {
        const double *xr = x + row * nx;
        const double *xm = xr + (m - 1u);
        // distance function over x_M (dtlz.cpp:182-244)
        // sums as the problem takes them: of (x - 0.5)^2, of x and of x^0.1 in
        // integer accumulators (isum.h), of cos(20 pi (x - 0.5)) in FP64
        isum::sq_acc qs = isum::make();
        isum::sg_acc as = isum::make_signed();
        double sc = 0.0; // the cosines in FP64: their fixed-point evaluation already loads the integer pipes
#pragma unroll 4
        for (uint32_t i = sub; i < k; i += G) {
            const double xi = __ldg(xm + i);
            if constexpr (ID == 1 || ID == 3) {
                const double d = xi - 0.5;
                isum::add_square(qs, d);
                sc += cos_2pi_signed(10.0 * d); // cos(20 pi d)
            } else if constexpr (ID == 6) {
                isum::add_value(as, pow(xi, 0.1));
            } else if constexpr (ID == 7) {
                isum::add_value(as, xi);
            } else {
                const double d = xi - 0.5;
                isum::add_square(qs, d);
            }
        }
        double s;
        if constexpr (ID == 6 || ID == 7) {
            s = isum::value(dev::group_ssum<G>(as, mask));
        } else {
            s = isum::value(dev::group_isum<G>(qs, mask));
        }
        if constexpr (ID == 1 || ID == 3) sc = group_sum<G>(sc, mask);
        double g;
        if constexpr (ID == 1 || ID == 3) {
            g = 100. * ((s - sc) + static_cast<double>(k));
        } else if constexpr (ID == 7) {
            g = (9. / static_cast<double>(k)) * s;
        } else {
            g = s;
        }
        if (pd) {
            if (sub == 0) out[row] = g;
            continue;
        }
        double *fr = out + row * m;
        if constexpr (ID == 7) {
            // dtlz.cpp:388-408, h7 of :247-256
            const double opg = 1.0 + (1. + g);
            double y = 0.0;
            for (uint32_t i = sub; i + 1u < m; i += G) {
                const double xi = __ldg(xr + i);
                // dtlz.cpp:253: std::sin(3 * detail::pi() * f[i]), 3 pi rounded first
                const double sn = sin(__dmul_rn(3. * kPi, xi));
                y += (xi / opg) * (1.0 + sn);
                fr[i] = xi;
            }
            y = group_sum<G>(y, mask);
            if (sub == 0) fr[m - 1u] = opg * (static_cast<double>(m) - y);
        } else {
            // dtlz.cpp:258-386
            const double opg = 1. + g;
            const double head = ID == 1 ? 0.5 * opg : opg;
            [[maybe_unused]] double t = 0.0;
            if constexpr (ID == 5 || ID == 6) t = 1. / (2. * opg);
            double p = head;
            for (uint32_t base = 0; base + 1u < m; base += G) {
                const uint32_t j = base + sub;
                double cj = 1.0, sj = 0.0;
                if (j + 1u < m) {
                    const double xj = __ldg(xr + j);
                    if constexpr (ID == 1) {
                        cj = xj;
                        sj = 1. - xj;
                    } else {
                        double a = xj;
                        if constexpr (ID == 4) a = pow(xj, static_cast<double>(alpha));
                        if constexpr (ID == 5 || ID == 6) a = j == 0 ? xj : t + ((g * xj) / (1.0 + g));
                        sincos_half_pi(a, sj, cj);
                    }
                }
                const uint32_t cnt = m - 1u - base < static_cast<uint32_t>(G) ? m - 1u - base : G;
                for (uint32_t u = 0; u < cnt; ++u) {
                    const double cu = __shfl_sync(mask, cj, static_cast<int>(u), G);
                    if (sub == u) fr[m - 1u - (base + u)] = p * sj;
                    p = p * cu;
                }
            }
            if (sub == 0) fr[0] = p;
        }
    }
}

// ---------------------------------------------------------------- launches

struct mo_shape {
    int kind;
    uint32_t id, nx, nobj, alpha;
};

template <typename K, typename... A>
int launch_grid(K kernel, int lanes, uint64_t n, int num_sms, cudaStream_t s, A... args)
{
    const int threads = row_block_threads(n, lanes, num_sms);
    int occ = 0;
    PGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, 0));
    if (occ < 1) occ = 1;
    const uint64_t per_block = static_cast<uint64_t>(threads / lanes);
    const uint64_t need = (n + per_block - 1) / per_block;
    const uint64_t cap = static_cast<uint64_t>(num_sms) * static_cast<uint64_t>(occ);
    const int grid = static_cast<int>(need < cap ? (need ? need : 1) : cap);
    kernel<<<grid, threads, 0, s>>>(args...);
    PGX_CUDA(cudaGetLastError());
    return PGX_OK;
}

template <int G>
int launch_zdt(const mo_shape &p, const double *x, uint64_t n, bool pd, double *out, cudaStream_t s, int num_sms)
{
    switch (p.id) {
        case 1u:
            return launch_grid(zdt_kernel<G, 1>, G, n, num_sms, s, x, n, p.nx, pd, out);
        case 2u:
            return launch_grid(zdt_kernel<G, 2>, G, n, num_sms, s, x, n, p.nx, pd, out);
        case 3u:
            return launch_grid(zdt_kernel<G, 3>, G, n, num_sms, s, x, n, p.nx, pd, out);
        case 4u:
            return launch_grid(zdt_kernel<G, 4>, G, n, num_sms, s, x, n, p.nx, pd, out);
        case 5u:
            return launch_grid(zdt_kernel<G, 5>, G, n, num_sms, s, x, n, p.nx, pd, out);
        default:
            return launch_grid(zdt_kernel<G, 6>, G, n, num_sms, s, x, n, p.nx, pd, out);
    }
}

template <int G>
int launch_dtlz(const mo_shape &p, const double *x, uint64_t n, bool pd, double *out, cudaStream_t s, int num_sms)
{
    switch (p.id) {
        case 1u:
            return launch_grid(dtlz_kernel<G, 1>, G, n, num_sms, s, x, n, p.nx, p.nobj, p.alpha, pd, out);
        case 2u:
            return launch_grid(dtlz_kernel<G, 2>, G, n, num_sms, s, x, n, p.nx, p.nobj, p.alpha, pd, out);
        case 3u:
            return launch_grid(dtlz_kernel<G, 3>, G, n, num_sms, s, x, n, p.nx, p.nobj, p.alpha, pd, out);
        case 4u:
            return launch_grid(dtlz_kernel<G, 4>, G, n, num_sms, s, x, n, p.nx, p.nobj, p.alpha, pd, out);
        case 5u:
            return launch_grid(dtlz_kernel<G, 5>, G, n, num_sms, s, x, n, p.nx, p.nobj, p.alpha, pd, out);
        case 6u:
            return launch_grid(dtlz_kernel<G, 6>, G, n, num_sms, s, x, n, p.nx, p.nobj, p.alpha, pd, out);
        default:
            return launch_grid(dtlz_kernel<G, 7>, G, n, num_sms, s, x, n, p.nx, p.nobj, p.alpha, pd, out);
    }
}

// Lanes per row: 2, 8 or 32, after the widest group that keeps the row's main
// loop at least 94 % busy (a function of the problem only, so that a row's
// result does not depend on the batch it comes in).
int mo_lanes(const mo_shape &p)
{
    uint32_t work;
    if (p.kind == PGX_ZDT)
        work = p.id == 5u ? (p.nx - 30u) / 5u : p.nx - 1u;
    else
        work = p.nx - (p.nobj - 1u);
    const int l = lanes_per_row(work);
    return l >= 32 ? 32 : (l >= 8 ? 8 : 2);
}

int launch_mo(const mo_shape &p, const double *x, uint64_t n, bool pd, double *out, cudaStream_t s, int num_sms)
{
    if (n == 0) return PGX_OK;
    const int lanes = mo_lanes(p);
    if (p.kind == PGX_ZDT) {
        if (lanes == 32) return launch_zdt<32>(p, x, n, pd, out, s, num_sms);
        if (lanes == 8) return launch_zdt<8>(p, x, n, pd, out, s, num_sms);
        return launch_zdt<2>(p, x, n, pd, out, s, num_sms);
    }
    if (lanes == 32) return launch_dtlz<32>(p, x, n, pd, out, s, num_sms);
    if (lanes == 8) return launch_dtlz<8>(p, x, n, pd, out, s, num_sms);
    return launch_dtlz<2>(p, x, n, pd, out, s, num_sms);
}

// Validates a problem as the reference constructors do (zdt.cpp:55-66,
// dtlz.cpp:53-74) and derives its shape; sizes beyond the kernels' 32-bit
// indexing are rejected.
int mo_validate(const pgx_mo_problem *p, mo_shape *out, uint64_t *nix)
{
    PGX_CHECK(p != nullptr, PGX_ERR_INVALID, "null problem");
    mo_shape sh{p->kind, p->prob_id, 0, 0, p->alpha};
    uint64_t nx = 0, nobj = 0, ni = 0;
    if (p->kind == PGX_ZDT) {
        PGX_CHECK(p->param <= UINT_MAX, PGX_ERR_INVALID,
                  "ZDT parameter " + std::to_string(p->param) + " does not fit the reference's unsigned parameter");
        PGX_CHECK(p->param >= 2u, PGX_ERR_INVALID,
                  "ZDT test problems must have a minimum value of 2 for the constructing parameter (representing "
                  "the dimension except for ZDT5), "
                      + std::to_string(p->param) + " requested");
        PGX_CHECK(p->prob_id >= 1u && p->prob_id <= 6u, PGX_ERR_INVALID,
                  "ZDT test suite contains six (prob_id=[1 ... 6]) problems, prob_id=" + std::to_string(p->prob_id)
                      + " was detected");
        nx = p->prob_id == 5u ? 30u + 5u * (p->param - 1u) : p->param;
        nobj = 2u;
        ni = p->prob_id == 5u ? nx : 0u;
    } else if (p->kind == PGX_DTLZ) {
        PGX_CHECK(p->prob_id >= 1u && p->prob_id <= 7u, PGX_ERR_INVALID,
                  "DTLZ test suite contains seven (prob_id = [1 ... 7]) problems, prob_id="
                      + std::to_string(p->prob_id) + " was detected");
        PGX_CHECK(p->fdim >= 2u, PGX_ERR_INVALID,
                  "DTLZ test problem have a minimum of 2 objectives: fdim=" + std::to_string(p->fdim)
                      + " was detected");
        PGX_CHECK(p->fdim <= UINT64_MAX / 3u, PGX_ERR_INVALID, "The number of objectives is too large");
        PGX_CHECK(p->param <= UINT64_MAX / 3u, PGX_ERR_INVALID, "The problem dimension is too large");
        PGX_CHECK(p->param > p->fdim, PGX_ERR_INVALID,
                  "The problem dimension has to be larger than the number of objectives.");
        nx = p->param;
        nobj = p->fdim;
    } else {
        set_error("unknown multi-objective problem kind " + std::to_string(p->kind));
        return PGX_ERR_INVALID;
    }
    PGX_CHECK(nx < (1ull << 31), PGX_ERR_CAPACITY, "decision vector dimension exceeds 2^31-1");
    sh.nx = static_cast<uint32_t>(nx);
    sh.nobj = static_cast<uint32_t>(nobj);
    *out = sh;
    if (nix) *nix = ni;
    return PGX_OK;
}

int mo_host(pgx_context *ctx, const pgx_mo_problem *p, const double *dvs, uint64_t n, bool pd, double *out)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    mo_shape sh{};
    PGX_TRY(mo_validate(p, &sh, nullptr));
    PGX_CHECK(out != nullptr || n == 0, PGX_ERR_INVALID, "null output buffer");
    if (n == 0) return PGX_OK;
    const int num_sms = ctx->num_sms;
    return host_rows(ctx, sh.nx, pd ? 1u : sh.nobj, dvs, n, out, nullptr,
                     [&](const double *din, uint64_t nr, double *dout, double *, cudaStream_t s, uint64_t *l) {
                         *l = 1;
                         return launch_mo(sh, din, nr, pd, dout, s, num_sms);
                     });
}

} // namespace
} // namespace pgx

using namespace pgx;

extern "C" {

int pgx_mo_problem_dims(const pgx_mo_problem *p, uint64_t *nx, uint64_t *nobj, uint64_t *nix)
{
    mo_shape sh{};
    uint64_t ni = 0;
    PGX_TRY(mo_validate(p, &sh, &ni));
    if (nx) *nx = sh.nx;
    if (nobj) *nobj = sh.nobj;
    if (nix) *nix = ni;
    return PGX_OK;
}

int pgx_mo_problem_bounds(const pgx_mo_problem *p, double *lb, double *ub)
{
    mo_shape sh{};
    PGX_TRY(mo_validate(p, &sh, nullptr));
    PGX_CHECK(lb != nullptr && ub != nullptr, PGX_ERR_INVALID, "null bounds buffer");
    for (uint32_t i = 0; i < sh.nx; ++i) {
        // ZDT4: x0 in [0, 1], the others in [-5, 5] (zdt.cpp:118-125); every
        // other ZDT and DTLZ problem: [0, 1].
        const bool wide = sh.kind == PGX_ZDT && sh.id == 4u && i != 0u;
        lb[i] = wide ? -5. : 0.;
        ub[i] = wide ? 5. : 1.;
    }
    return PGX_OK;
}

int pgx_mo_batch_fitness(pgx_context *ctx, const pgx_mo_problem *p, const double *dvs, uint64_t n_dvs, double *fvs)
{
    return mo_host(ctx, p, dvs, n_dvs, false, fvs);
}

int pgx_mo_p_distance(pgx_context *ctx, const pgx_mo_problem *p, const double *dvs, uint64_t n_dvs, double *out)
{
    return mo_host(ctx, p, dvs, n_dvs, true, out);
}

int pgx_mo_batch_fitness_device(pgx_context *ctx, const pgx_mo_problem *p, const double *d_dvs, uint64_t n_dvs,
                                double *d_fvs, void *stream)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    mo_shape sh{};
    PGX_TRY(mo_validate(p, &sh, nullptr));
    if (n_dvs == 0) return PGX_OK;
    PGX_CHECK(d_dvs != nullptr && d_fvs != nullptr, PGX_ERR_INVALID, "null device buffer");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    PGX_TRY(launch_mo(sh, d_dvs, n_dvs, false, d_fvs, static_cast<cudaStream_t>(stream), ctx->num_sms));
    ctx->launches += 1;
    return PGX_OK;
}

} // extern "C"
