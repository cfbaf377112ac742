/*
 * CPU oracle for the constrained UDP and the unconstrain meta-problem (TEST
 * INFRASTRUCTURE ONLY: the tests and the smoke check use it; the product
 * library never links or loads it).
 *
 * hock_schittkowski_71::fitness (src/problems/hock_schittkowski_71.cpp:48-55)
 * and unconstrain::penalize (src/problems/unconstrain.cpp:130-225, with
 * problem::feasibility_f, src/problem.cpp:709-721, and the constraint tests of
 * include/pagmo/utils/constrained.hpp:49-80) restated in double in the
 * reference's order of operations: bit for bit the reference's values
 * (tests/test_oracle_constrained.py pins them to the compiled reference).
 */
#include "oracle.h"

#include <cfloat>
#include <cmath>

namespace
{
double max0(double a)
{
    return a < 0. ? 0. : a; // std::max(a, 0.)
}

// satisfied constraints and the two sums of squared violations of one row
void tests(const double *f, uint64_t nobj, uint64_t nec, uint64_t nic, const double *tol, uint64_t *sat, double *l2e,
           double *l2i)
{
    uint64_t n = 0;
    double a = 0., b = 0.;
    for (uint64_t i = 0; i < nec; ++i) {
        const double err = max0(std::fabs(f[nobj + i]) - tol[i]);
        a += err * err;
        n += err <= 0. ? 1u : 0u;
    }
    for (uint64_t i = 0; i < nic; ++i) {
        const double err = max0(f[nobj + nec + i] - tol[nec + i]);
        b += err * err;
        n += err <= 0. ? 1u : 0u;
    }
    *sat = n;
    *l2e = a;
    *l2i = b;
}
} // namespace

extern "C" {

void orc_hs71_fitness(const double *x, uint64_t n, double *f)
{
    for (uint64_t r = 0; r < n; ++r) {
        const double *v = x + 4u * r;
        double *o = f + 3u * r;
        o[0] = v[0] * v[3] * (v[0] + v[1] + v[2]) + v[2];
        o[1] = v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3] - 40.;
        o[2] = 25. - v[0] * v[1] * v[2] * v[3];
    }
}

int orc_unconstrain_penalize(const double *f, uint64_t n, uint64_t nobj, uint64_t nec, uint64_t nic, int method,
                             const double *weights, const double *tol, double *out)
{
    const uint64_t nc = nec + nic, nf = nobj + nc;
    const uint64_t w = method == 4 ? 1u : nobj;
    for (uint64_t r = 0; r < n; ++r) {
        const double *row = f + r * nf;
        double *o = out + r * w;
        uint64_t sat = 0;
        double l2e = 0., l2i = 0.;
        switch (method) {
            case 0: // death penalty
                tests(row, nobj, nec, nic, tol, &sat, &l2e, &l2i);
                for (uint64_t k = 0; k < nobj; ++k) o[k] = sat == nc ? row[k] : DBL_MAX;
                break;
            case 1: { // kuri
                tests(row, nobj, nec, nic, tol, &sat, &l2e, &l2i);
                const double p = DBL_MAX * (1. - static_cast<double>(sat) / static_cast<double>(nc));
                for (uint64_t k = 0; k < nobj; ++k) o[k] = sat == nc ? row[k] : p;
            } break;
            case 2: { // weighted
                double p = 0.;
                for (uint64_t i = 0; i < nc; ++i) {
                    const double c = i < nec ? std::fabs(row[nobj + i]) - tol[i] : row[nobj + i] - tol[i];
                    if (!(c <= 0.)) p += weights[i] * c;
                }
                for (uint64_t k = 0; k < nobj; ++k) o[k] = row[k] + p;
            } break;
            case 3: // ignore_c
                for (uint64_t k = 0; k < nobj; ++k) o[k] = row[k];
                break;
            case 4: // ignore_o
                tests(row, nobj, nec, nic, tol, &sat, &l2e, &l2i);
                o[0] = std::sqrt(l2e) + std::sqrt(l2i);
                break;
            default:
                return 1;
        }
    }
    return 0;
}

} // extern "C"
