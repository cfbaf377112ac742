// A constrained UDP and pagmo's unconstrain meta-problem on the GPU.
//
// hock_schittkowski_71 (src/problems/hock_schittkowski_71.cpp:48-55): four
// variables in [1, 5], one objective, one equality and one inequality
// constraint; a row's fitness is [f, ceq, cineq] in the reference's operation
// order (explicitly rounded operations, no contraction into FMA), so it is the
// reference's bit for bit.
//
// unconstrain::batch_fitness (src/problems/unconstrain.cpp:245-266) forwards the
// batch to the inner problem's batch_fitness and penalises every row
// (unconstrain::penalize, :130-225): here both run in one kernel, the inner
// row's fitness kept in registers. The penalties follow the reference
// operation by operation: feasibility by problem::feasibility_f
// (src/problem.cpp:709-721) with the tolerances c_tol, the Kuri penalty
// DBL_MAX * (1 - satisfied / nc), the weighted sum over the violated
// constraints in index order, and ignore_o's norms sqrt(sum of squared
// violations) of the equalities plus that of the inequalities
// (include/pagmo/utils/constrained.hpp:49-80).
#include "pgx_internal.cuh"

#include <algorithm>
#include <cfloat>
#include <string>

namespace pgx
{
namespace
{

constexpr uint32_t kMaxCon = 8; // constraints a penalty takes by value

struct con_shape {
    uint32_t nx, nobj, nec, nic;
};

int con_validate(int kind, uint64_t param, con_shape *sh)
{
    (void)param;
    PGX_CHECK(kind == PGX_HS71, PGX_ERR_INVALID, "unknown constrained problem kind " + std::to_string(kind));
    *sh = con_shape{4u, 1u, 1u, 1u};
    return PGX_OK;
}

// hock_schittkowski_71::fitness
__device__ __forceinline__ void hs71_row(const double *x, double *f)
{
    const double x0 = x[0], x1 = x[1], x2 = x[2], x3 = x[3];
    f[0] = __dadd_rn(__dmul_rn(__dmul_rn(x0, x3), __dadd_rn(__dadd_rn(x0, x1), x2)), x2);
    f[1] = __dsub_rn(
        __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(x0, x0), __dmul_rn(x1, x1)), __dmul_rn(x2, x2)), __dmul_rn(x3, x3)),
        40.);
    f[2] = __dsub_rn(25., __dmul_rn(__dmul_rn(__dmul_rn(x0, x1), x2), x3));
}

struct penalty {
    int method; // PGX_UNCONSTRAIN_*
    uint32_t nobj, nec, nic;
    double tol[kMaxCon];
    double w[kMaxCon];
};

__device__ __forceinline__ double std_max0(double a)
{
    return a < 0. ? 0. : a; // std::max(a, 0.)
}

// detail::test_eq_constraints / test_ineq_constraints over f[nobj ..): the
// number satisfied and the two sums of squared violations
__device__ __forceinline__ void test_constraints(const penalty &u, const double *f, uint32_t *sat, double *l2e,
                                                 double *l2i)
{
    uint32_t n = 0;
    double a = 0., b = 0.;
    for (uint32_t i = 0; i < u.nec; ++i) {
        const double err = std_max0(__dsub_rn(fabs(f[u.nobj + i]), u.tol[i]));
        a = __dadd_rn(a, __dmul_rn(err, err));
        n += err <= 0. ? 1u : 0u;
    }
    for (uint32_t i = 0; i < u.nic; ++i) {
        const double err = std_max0(__dsub_rn(f[u.nobj + u.nec + i], u.tol[u.nec + i]));
        b = __dadd_rn(b, __dmul_rn(err, err));
        n += err <= 0. ? 1u : 0u;
    }
    *sat = n;
    *l2e = a;
    *l2i = b;
}

// unconstrain::penalize of one row f (nobj + nec + nic values) into out
__device__ void penalize(const penalty &u, const double *f, double *out)
{
    const uint32_t nc = u.nec + u.nic;
    uint32_t sat = 0;
    double l2e = 0., l2i = 0.;
    switch (u.method) {
        case PGX_UNCONSTRAIN_DEATH:
            test_constraints(u, f, &sat, &l2e, &l2i);
            for (uint32_t k = 0; k < u.nobj; ++k) out[k] = sat == nc ? f[k] : DBL_MAX;
            break;
        case PGX_UNCONSTRAIN_KURI: {
            test_constraints(u, f, &sat, &l2e, &l2i);
            const double p = __dmul_rn(DBL_MAX, __dsub_rn(1., __ddiv_rn(static_cast<double>(sat), static_cast<double>(nc))));
            for (uint32_t k = 0; k < u.nobj; ++k) out[k] = sat == nc ? f[k] : p;
        } break;
        case PGX_UNCONSTRAIN_WEIGHTED: {
            double p = 0.;
            for (uint32_t i = 0; i < nc; ++i) {
                const double c = i < u.nec ? __dsub_rn(fabs(f[u.nobj + i]), u.tol[i]) : __dsub_rn(f[u.nobj + i], u.tol[i]);
                if (!(c <= 0.)) p = __dadd_rn(p, __dmul_rn(u.w[i], c));
            }
            for (uint32_t k = 0; k < u.nobj; ++k) out[k] = __dadd_rn(f[k], p);
        } break;
        case PGX_UNCONSTRAIN_IGNORE_C:
            for (uint32_t k = 0; k < u.nobj; ++k) out[k] = f[k];
            break;
        default: // PGX_UNCONSTRAIN_IGNORE_O
            test_constraints(u, f, &sat, &l2e, &l2i);
            out[0] = __dadd_rn(__dsqrt_rn(l2e), __dsqrt_rn(l2i));
    }
}

// One thread per row: the inner fitness, then (penalise != 0) the penalty.
__global__ void hs71_kernel(const double *__restrict__ x, uint64_t n, double *__restrict__ out, penalty pen,
                            int penalise)
{
    for (uint64_t r = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; r < n;
         r += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const double xr[4] = {x[4u * r], x[4u * r + 1u], x[4u * r + 2u], x[4u * r + 3u]};
        double f[3];
        hs71_row(xr, f);
        if (penalise) {
            double o[3];
            penalize(pen, f, o);
            const uint32_t w = pen.method == PGX_UNCONSTRAIN_IGNORE_O ? 1u : pen.nobj;
            for (uint32_t k = 0; k < w; ++k) out[r * w + k] = o[k];
        } else {
            out[3u * r] = f[0];
            out[3u * r + 1u] = f[1];
            out[3u * r + 2u] = f[2];
        }
    }
}

int launch_con(const con_shape &sh, const double *d_x, uint64_t n, double *d_out, const penalty *pen, cudaStream_t s,
               int num_sms)
{
    (void)sh;
    const int threads = 256;
    const uint64_t want = (n + threads - 1u) / threads;
    const int grid = static_cast<int>(std::min<uint64_t>(want, static_cast<uint64_t>(num_sms) * 16u));
    penalty p{};
    if (pen) p = *pen;
    hs71_kernel<<<grid, threads, 0, s>>>(d_x, n, d_out, p, pen ? 1 : 0);
    PGX_CUDA(cudaGetLastError());
    return PGX_OK;
}

// unconstrain's constructor checks (unconstrain.cpp:66-100) on the C ABI's
// method code and weights, and the penalty's parameters
int make_penalty(const con_shape &sh, const pgx_unconstrain *u, penalty *out)
{
    PGX_CHECK(u != nullptr, PGX_ERR_INVALID, "null unconstrain descriptor");
    const uint32_t nc = sh.nec + sh.nic;
    PGX_CHECK(nc > 0u, PGX_ERR_INVALID,
              "Unconstrain can only be applied to constrained problems, the instance of the problem is not one.");
    PGX_CHECK(u->method >= PGX_UNCONSTRAIN_DEATH && u->method <= PGX_UNCONSTRAIN_IGNORE_O, PGX_ERR_INVALID,
              "The method " + std::to_string(u->method) + " is not supported (did you misspell?)");
    PGX_CHECK(u->n_weights == nc || u->method != PGX_UNCONSTRAIN_WEIGHTED, PGX_ERR_INVALID,
              "Length of weight vector is: " + std::to_string(u->n_weights) +
                  " while the problem constraints are: " + std::to_string(nc));
    PGX_CHECK(u->n_weights == 0u || u->method == PGX_UNCONSTRAIN_WEIGHTED, PGX_ERR_INVALID,
              "The weight vector needs to be empty to use the unconstrain method " +
                  std::string(u->method == PGX_UNCONSTRAIN_DEATH  ? "death penalty"
                              : u->method == PGX_UNCONSTRAIN_KURI ? "kuri"
                              : u->method == PGX_UNCONSTRAIN_IGNORE_C ? "ignore_c"
                                                                      : "ignore_o"));
    PGX_CHECK(nc <= kMaxCon, PGX_ERR_CAPACITY, "unconstrain: more than 8 constraints");
    PGX_CHECK(u->n_weights == 0u || u->weights != nullptr, PGX_ERR_INVALID, "null weights");
    penalty p{};
    p.method = u->method;
    p.nobj = sh.nobj;
    p.nec = sh.nec;
    p.nic = sh.nic;
    for (uint32_t i = 0; i < nc; ++i) {
        p.tol[i] = u->c_tol ? u->c_tol[i] : 0.;
        p.w[i] = u->n_weights ? u->weights[i] : 0.;
    }
    *out = p;
    return PGX_OK;
}

} // namespace
} // namespace pgx

using namespace pgx;

extern "C" {

int pgx_constrained_dims(int kind, uint64_t param, uint64_t *nx, uint64_t *nobj, uint64_t *nec, uint64_t *nic)
{
    con_shape sh{};
    PGX_TRY(con_validate(kind, param, &sh));
    if (nx) *nx = sh.nx;
    if (nobj) *nobj = sh.nobj;
    if (nec) *nec = sh.nec;
    if (nic) *nic = sh.nic;
    return PGX_OK;
}

int pgx_constrained_bounds(int kind, uint64_t param, double *lb, double *ub)
{
    con_shape sh{};
    PGX_TRY(con_validate(kind, param, &sh));
    PGX_CHECK(lb != nullptr && ub != nullptr, PGX_ERR_INVALID, "null bounds buffer");
    for (uint32_t i = 0; i < sh.nx; ++i) { // hock_schittkowski_71.cpp:66-69
        lb[i] = 1.;
        ub[i] = 5.;
    }
    return PGX_OK;
}

int pgx_constrained_batch_fitness(pgx_context *ctx, int kind, uint64_t param, const double *dvs, uint64_t n_dvs,
                                  double *fvs)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    con_shape sh{};
    PGX_TRY(con_validate(kind, param, &sh));
    PGX_CHECK(fvs != nullptr || n_dvs == 0, PGX_ERR_INVALID, "null fitness buffer");
    if (n_dvs == 0) return PGX_OK;
    const int num_sms = ctx->num_sms;
    return host_rows(ctx, sh.nx, sh.nobj + sh.nec + sh.nic, dvs, n_dvs, fvs, nullptr,
                     [&](const double *din, uint64_t nr, double *dout, double *, cudaStream_t s, uint64_t *l) {
                         *l = 1;
                         return launch_con(sh, din, nr, dout, nullptr, s, num_sms);
                     });
}

int pgx_unconstrain_batch_fitness(pgx_context *ctx, int kind, uint64_t param, const pgx_unconstrain *u,
                                  const double *dvs, uint64_t n_dvs, double *fvs)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    con_shape sh{};
    PGX_TRY(con_validate(kind, param, &sh));
    penalty pen{};
    PGX_TRY(make_penalty(sh, u, &pen));
    PGX_CHECK(fvs != nullptr || n_dvs == 0, PGX_ERR_INVALID, "null fitness buffer");
    if (n_dvs == 0) return PGX_OK;
    const int num_sms = ctx->num_sms;
    const uint64_t w = pen.method == PGX_UNCONSTRAIN_IGNORE_O ? 1u : sh.nobj;
    return host_rows(ctx, sh.nx, w, dvs, n_dvs, fvs, nullptr,
                     [&](const double *din, uint64_t nr, double *dout, double *, cudaStream_t s, uint64_t *l) {
                         *l = 1;
                         return launch_con(sh, din, nr, dout, &pen, s, num_sms);
                     });
}

} // extern "C"
