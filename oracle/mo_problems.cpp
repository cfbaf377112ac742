/*
 * CPU oracle for the multi-objective test problems ZDT and DTLZ
 * (TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU leg of the
 * benchmark use it; the product library never links or loads it).
 *
 * Restates src/problems/zdt.cpp and src/problems/dtlz.cpp of pagmo 2.19.1:
 *  - mirror functions (double) repeat the reference's arithmetic in the same
 *    order with the same libm calls, so they reproduce its results bit for bit;
 *    tests/test_oracle_mo_problems.py pins them to the reference's known answers
 *    (tests/zdt.cpp, tests/dtlz.cpp) and to the compiled reference;
 *  - "_ld" functions evaluate the mathematics in long double and return, per
 *    objective, a first-order error scale: every rounded operation of the
 *    reference's formula contributes the magnitude of its result, propagated
 *    through the rest of the formula by the absolute partial derivatives (the
 *    reference's pi and pi/2 count as rounded constants, each libm call as one
 *    more rounding of its result). A double evaluation of the formula differs
 *    from the long-double value by about 2^-53 x scale; tests allow 1e-13 x
 *    scale.
 *
 * Families (the problem kinds of the GPU library): 7 = ZDT (prob_id 1-6,
 * param), 8 = DTLZ (prob_id 1-7, dim, fdim, alpha). Status codes: 0 ok, 1 invalid argument (orc_mo_last_error()).
 */
#include "oracle.h"
#include "rows.hpp"

#include <cmath>
#include <limits>
#include <string>
#include <vector>

namespace
{
thread_local std::string mo_err;

constexpr double k_pi = 3.1415926535897932384626433832795028841971693993; // constants.hpp:37-40
constexpr double k_pi_half = k_pi / 2.;                                      // constants.hpp:41-44

using ld = long double;
const ld k_pi_ld = 3.1415926535897932384626433832795028841971693993L;

// ------------------------------------------------------------ argument checks

// zdt.cpp:55-66 and the dimensions of zdt.cpp:108-158; dtlz.cpp:53-74.
bool mo_dims(int family, unsigned id, uint64_t param, uint64_t fdim, uint64_t *nx, uint64_t *nobj)
{
    if (family == 7) {
        if (param < 2u) {
            mo_err = "ZDT test problems must have a minimum value of 2 for the constructing parameter (representing "
                     "the dimension except for ZDT5), "
                     + std::to_string(param) + " requested";
            return false;
        }
        if (id == 0u || id > 6u) {
            mo_err = "ZDT test suite contains six (prob_id=[1 ... 6]) problems, prob_id=" + std::to_string(id)
                     + " was detected";
            return false;
        }
        *nx = id == 5u ? 30u + 5u * (param - 1u) : param;
        *nobj = 2u;
        return true;
    }
    if (family == 8) {
        if (id == 0u || id > 7u) {
            mo_err = "DTLZ test suite contains seven (prob_id = [1 ... 7]) problems, prob_id=" + std::to_string(id)
                     + " was detected";
            return false;
        }
        if (fdim < 2u) {
            mo_err = "DTLZ test problem have a minimum of 2 objectives: fdim=" + std::to_string(fdim)
                     + " was detected";
            return false;
        }
        if (fdim > std::numeric_limits<uint64_t>::max() / 3u) {
            mo_err = "The number of objectives is too large";
            return false;
        }
        if (param > std::numeric_limits<uint64_t>::max() / 3u) {
            mo_err = "The problem dimension is too large";
            return false;
        }
        if (param <= fdim) {
            mo_err = "The problem dimension has to be larger than the number of objectives.";
            return false;
        }
        *nx = param;
        *nobj = fdim;
        return true;
    }
    mo_err = "unknown multi-objective family " + std::to_string(family);
    return false;
}

// ------------------------------------------------------------- ZDT mirrors

// zdt.cpp:233-279: g = 1 + 9 sum(x[1:]) / (N - 1), all three of ZDT1-3.
double zdt_g123(const double *x, uint64_t n)
{
    double s = 0.;
    for (uint64_t i = 1u; i < n; ++i) s += x[i];
    return 1. + (9. * s) / static_cast<double>(n - 1u);
}

// zdt.cpp:281-296: g = 1 + 10 (N - 1) + sum(x^2 - 10 cos(4 pi x)).
double zdt_g4(const double *x, uint64_t n)
{
    double g = 1 + 10 * static_cast<double>(n - 1u);
    for (uint64_t i = 1u; i < n; ++i) g += x[i] * x[i] - 10. * std::cos(4. * k_pi * x[i]);
    return g;
}

// Counts of ones of the rounded (fitness) or floored (p_distance) ZDT5 string:
// u0 over the first 30 bits, then v(u) = u < 5 ? 2 + u : 1 summed over the
// following 5-bit groups (zdt.cpp:298-339, :384-421).
template <typename R>
void zdt5_counts(const double *x, uint64_t n, R round_fn, uint64_t *u0, double *g)
{
    uint64_t c0 = 0;
    for (uint64_t i = 0; i < 30u; ++i) c0 += round_fn(x[i]) == 1. ? 1u : 0u;
    double s = 0.;
    for (uint64_t b = 30u; b + 5u <= n; b += 5u) {
        uint64_t u = 0;
        for (uint64_t j = 0; j < 5u; ++j) u += round_fn(x[b + j]) == 1. ? 1u : 0u;
        s += static_cast<double>(u < 5u ? 2u + u : 1u);
    }
    *u0 = c0;
    *g = s;
}

void zdt_fitness(unsigned id, const double *x, uint64_t n, double *f)
{
    switch (id) {
        case 1u: { // zdt.cpp:233-247
            const double g = zdt_g123(x, n);
            f[0] = x[0];
            f[1] = g * (1. - std::sqrt(x[0] / g));
            return;
        }
        case 2u: { // zdt.cpp:249-263
            const double g = zdt_g123(x, n);
            f[0] = x[0];
            f[1] = g * (1. - (x[0] / g) * (x[0] / g));
            return;
        }
        case 3u: { // zdt.cpp:265-279
            const double g = zdt_g123(x, n);
            f[0] = x[0];
            f[1] = g * (1. - std::sqrt(x[0] / g) - x[0] / g * std::sin(10. * k_pi * x[0]));
            return;
        }
        case 4u: { // zdt.cpp:281-296
            const double g = zdt_g4(x, n);
            f[0] = x[0];
            f[1] = g * (1. - std::sqrt(x[0] / g));
            return;
        }
        case 5u: { // zdt.cpp:298-339
            uint64_t u0 = 0;
            double g = 0.;
            zdt5_counts(x, n, [](double v) { return std::round(v); }, &u0, &g);
            f[0] = 1.0 + static_cast<double>(u0);
            f[1] = g * (1. / f[0]);
            return;
        }
        default: { // zdt.cpp:341-356
            const double f0 = 1 - std::exp(-4 * x[0]) * std::pow(std::sin(6 * k_pi * x[0]), 6);
            double s = 0.;
            for (uint64_t i = 1u; i < n; ++i) s += x[i];
            const double g = 1 + 9 * std::pow((s / static_cast<double>(n - 1u)), 0.25);
            f[0] = f0;
            f[1] = g * (1 - (f0 / g) * (f0 / g));
            return;
        }
    }
}

double zdt_p_distance(unsigned id, const double *x, uint64_t n)
{
    switch (id) {
        case 1u:
        case 2u:
        case 3u: { // zdt.cpp:358-369
            double c = 0.;
            c += zdt_g123(x, n);
            return c - 1.;
        }
        case 4u: { // zdt.cpp:371-382
            double s = 0.;
            for (uint64_t j = 1u; j < n; ++j) s += x[j] * x[j] - 10. * std::cos(4. * k_pi * x[j]);
            double c = 0.;
            c += 1. + 10. * static_cast<double>(n - 1u) + s;
            return c - 1.;
        }
        case 5u: { // zdt.cpp:384-421 (floor, and no first-30 count)
            uint64_t u0 = 0;
            double g = 0.;
            zdt5_counts(x, n, [](double v) { return std::floor(v); }, &u0, &g);
            const uint64_t groups = (n - 30u) / 5u + 1u;
            double c = 0.;
            c += g;
            return c - static_cast<double>(groups) + 1;
        }
        default: { // zdt.cpp:423-434
            double s = 0.;
            for (uint64_t j = 1u; j < n; ++j) s += x[j];
            double c = 0.;
            c += 1. + 9. * std::pow((s / static_cast<double>(n - 1u)), 0.25);
            return c - 1;
        }
    }
}

// ------------------------------------------------------------- DTLZ mirrors

// dtlz.cpp:182-244: the distance function over x_M = x[fdim-1 .. n-1].
double dtlz_g(unsigned id, const double *xm, uint64_t k)
{
    double y = 0.;
    switch (id) {
        case 1u:
        case 3u:
            for (uint64_t i = 0; i < k; ++i) y += std::pow(xm[i] - 0.5, 2) - std::cos(20. * k_pi * (xm[i] - 0.5));
            return 100. * (y + static_cast<double>(k));
        case 6u:
            for (uint64_t i = 0; i < k; ++i) y += std::pow(xm[i], 0.1);
            return y;
        case 7u:
            for (uint64_t i = 0; i < k; ++i) y += xm[i];
            return (9. / static_cast<double>(k)) * y;
        default: // 2, 4, 5
            for (uint64_t i = 0; i < k; ++i) y += std::pow(xm[i] - 0.5, 2);
            return y;
    }
}

// Shape functions of DTLZ1-6 (dtlz.cpp:258-386). Objective i is the running
// product (1 + g) c_0 c_1 ... c_{m-2-i}, times s_{m-1-i} for i > 0, multiplied
// left to right as the reference does; each objective's product is formed
// afresh, exactly as in the reference's nested loops.
template <typename C, typename S>
void dtlz_shape(uint64_t m, double head, C c, S s, double *f)
{
    f[0] = head;
    for (uint64_t i = 0; i + 1u < m; ++i) f[0] *= c(i);
    for (uint64_t i = 1u; i + 1u < m; ++i) {
        f[i] = head;
        for (uint64_t j = 0; j < m - (i + 1u); ++j) f[i] *= c(j);
        f[i] *= s(m - (i + 1u));
    }
}

void dtlz_fitness(unsigned id, uint64_t m, unsigned alpha, const double *x, uint64_t n, double *f)
{
    const double *xm = x + (m - 1u);
    const uint64_t k = n - (m - 1u);
    switch (id) {
        case 1u: { // dtlz.cpp:258-287
            const double g = dtlz_g(id, xm, k);
            dtlz_shape(
                m, 0.5 * (1. + g), [&](uint64_t j) { return x[j]; }, [&](uint64_t j) { return 1. - x[j]; }, f);
            f[m - 1u] = 0.5 * (1. - x[0]) * (1. + g);
            return;
        }
        case 2u:
        case 3u: { // dtlz.cpp:289-316
            const double g = dtlz_g(id, xm, k);
            dtlz_shape(
                m, 1. + g, [&](uint64_t j) { return std::cos(x[j] * k_pi_half); },
                [&](uint64_t j) { return std::sin(x[j] * k_pi_half); }, f);
            f[m - 1u] = (1. + g) * std::sin(x[0] * k_pi_half);
            return;
        }
        case 4u: { // dtlz.cpp:318-345
            const double g = dtlz_g(id, xm, k);
            dtlz_shape(
                m, 1. + g, [&](uint64_t j) { return std::cos(std::pow(x[j], alpha) * k_pi_half); },
                [&](uint64_t j) { return std::sin(std::pow(x[j], alpha) * k_pi_half); }, f);
            f[m - 1u] = (1. + g) * std::sin(std::pow(x[0], alpha) * k_pi_half);
            return;
        }
        case 5u:
        case 6u: { // dtlz.cpp:347-386
            const double g = dtlz_g(id, xm, k);
            std::vector<double> theta(m, 0.);
            theta[0] = x[0];
            const double t = 1. / (2. * (1. + g));
            for (uint64_t i = 1u; i < m; ++i) theta[i] = t + ((g * x[i]) / (1.0 + g));
            dtlz_shape(
                m, 1. + g, [&](uint64_t j) { return std::cos(theta[j] * k_pi_half); },
                [&](uint64_t j) { return std::sin(theta[j] * k_pi_half); }, f);
            f[m - 1u] = (1. + g) * std::sin(theta[0] * k_pi_half);
            return;
        }
        default: { // dtlz.cpp:388-408 with h7 of dtlz.cpp:247-256
            const double g = 1. + dtlz_g(id, xm, k);
            for (uint64_t i = 0; i + 1u < m; ++i) f[i] = x[i];
            double y = 0.;
            for (uint64_t i = 0; i + 1u < m; ++i) y += (f[i] / (1.0 + g)) * (1.0 + std::sin(3 * k_pi * f[i]));
            f[m - 1u] = (1. + g) * (static_cast<double>(m) - y);
            return;
        }
    }
}

// ------------------------------------------------ long double with error scales

// A value and its error scale (in units of the unit roundoff u = 2^-53): the
// magnitude of every rounding that produced it, carried through the
// operations by their absolute partial derivatives. Products and sin/cos also
// carry the second-order term (u m_a m_b, u m_a^2 / 2): where two factors are
// both near zero (DTLZ's cos(pi/2 x) at x = 1, which the reference evaluates
// to 6e-17 and an exact reduction to 0) the first-order bound alone vanishes.
constexpr ld kU = 1.0L / 9007199254740992.0L; // 2^-53

struct em {
    ld v, m;
};
em exact(ld v)
{
    return {v, 0};
}
em rounded_const(ld v)
{
    return {v, fabsl(v)};
}
em operator+(em a, em b)
{
    const ld v = a.v + b.v;
    return {v, a.m + b.m + fabsl(v)};
}
em operator-(em a, em b)
{
    const ld v = a.v - b.v;
    return {v, a.m + b.m + fabsl(v)};
}
em operator*(em a, em b)
{
    const ld v = a.v * b.v;
    return {v, a.m * fabsl(b.v) + fabsl(a.v) * b.m + kU * a.m * b.m + fabsl(v)};
}
em operator/(em a, em b)
{
    const ld v = a.v / b.v;
    return {v, a.m / fabsl(b.v) + fabsl(a.v) * b.m / (b.v * b.v) + fabsl(v)};
}
// A libm call y = fn(a) with derivative d at a: one rounding of its own.
em call(ld y, ld d, em a)
{
    return {y, fabsl(d) * a.m + fabsl(y)};
}
em e_sqrt(em a)
{
    const ld y = sqrtl(a.v);
    if (a.m == 0) return {y, fabsl(y)};
    if (a.v <= 0) return {y, std::numeric_limits<ld>::infinity()};
    return call(y, 0.5L / y, a);
}
em e_sin(em a)
{
    em r = call(sinl(a.v), cosl(a.v), a);
    r.m += 0.5L * kU * a.m * a.m;
    return r;
}
em e_cos(em a)
{
    em r = call(cosl(a.v), sinl(a.v), a);
    r.m += 0.5L * kU * a.m * a.m;
    return r;
}
em e_exp(em a)
{
    const ld y = expl(a.v);
    return call(y, y, a);
}
em e_pow(em a, ld p)
{
    const ld y = powl(a.v, p);
    if (a.m == 0) return {y, fabsl(y)};
    if (a.v == 0) return {y, p >= 1 ? 0.0L : std::numeric_limits<ld>::infinity()};
    return call(y, p * powl(a.v, p - 1), a);
}
// A sum of many terms: the terms' own scales plus one rounding of the sum of
// their magnitudes (the scale convention of the single-objective oracle; the
// GPU's reduction trees and the reference's running sum both stay far inside
// 1e-13 of it).
struct em_sum {
    ld v = 0, m = 0, a = 0;
    void add(em t)
    {
        v += t.v;
        m += t.m;
        a += fabsl(t.v);
    }
    em get() const
    {
        return {v, m + a};
    }
};

em e_sum(const double *x, uint64_t b, uint64_t e)
{
    em_sum s;
    for (uint64_t i = b; i < e; ++i) s.add(exact(x[i]));
    return s.get();
}

void zdt_fitness_ld(unsigned id, const double *x, uint64_t n, double *f, double *sc)
{
    const em x0 = exact(x[0]);
    const em nm1 = exact(static_cast<ld>(n - 1u));
    em f0 = x0, f1{};
    switch (id) {
        case 1u:
        case 2u:
        case 3u:
        case 4u: {
            em g{};
            if (id == 4u) {
                em_sum acc;
                acc.add(exact(1) + exact(10) * nm1);
                const em four_pi = rounded_const(4 * k_pi_ld);
                for (uint64_t i = 1u; i < n; ++i) {
                    const em xi = exact(x[i]);
                    acc.add(xi * xi - exact(10) * e_cos(four_pi * xi));
                }
                g = acc.get();
            } else {
                g = exact(1) + (exact(9) * e_sum(x, 1u, n)) / nm1;
            }
            const em r = x0 / g;
            if (id == 2u)
                f1 = g * (exact(1) - r * r);
            else if (id == 3u)
                f1 = g * (exact(1) - e_sqrt(r) - r * e_sin(rounded_const(10 * k_pi_ld) * x0));
            else
                f1 = g * (exact(1) - e_sqrt(r));
            break;
        }
        case 5u: {
            uint64_t u0 = 0;
            double g = 0.;
            zdt5_counts(x, n, [](double v) { return std::round(v); }, &u0, &g);
            f0 = exact(1 + static_cast<ld>(u0));
            f1 = exact(g) * (exact(1) / f0);
            break;
        }
        default: {
            const em s6 = e_sin(rounded_const(6 * k_pi_ld) * x0);
            f0 = exact(1) - e_exp(exact(-4) * x0) * e_pow(s6, 6);
            const em g = exact(1) + exact(9) * e_pow(e_sum(x, 1u, n) / nm1, 0.25L);
            const em q = f0 / g;
            f1 = g * (exact(1) - q * q);
            break;
        }
    }
    f[0] = static_cast<double>(f0.v);
    f[1] = static_cast<double>(f1.v);
    if (sc) {
        sc[0] = static_cast<double>(f0.m);
        sc[1] = static_cast<double>(f1.m);
    }
}

em dtlz_g_ld(unsigned id, const double *xm, uint64_t k)
{
    em_sum y;
    switch (id) {
        case 1u:
        case 3u: {
            const em twenty_pi = rounded_const(20 * k_pi_ld);
            for (uint64_t i = 0; i < k; ++i) {
                const em d = exact(xm[i]) - exact(0.5L);
                y.add(d * d - e_cos(twenty_pi * d));
            }
            return exact(100) * (y.get() + exact(static_cast<ld>(k)));
        }
        case 6u:
            for (uint64_t i = 0; i < k; ++i) y.add(e_pow(exact(xm[i]), 0.1L));
            return y.get();
        case 7u:
            for (uint64_t i = 0; i < k; ++i) y.add(exact(xm[i]));
            return (exact(9) / exact(static_cast<ld>(k))) * y.get();
        default:
            for (uint64_t i = 0; i < k; ++i) {
                const em d = exact(xm[i]) - exact(0.5L);
                y.add(d * d);
            }
            return y.get();
    }
}

void dtlz_fitness_ld(unsigned id, uint64_t m, unsigned alpha, const double *x, uint64_t n, double *f, double *sc)
{
    const double *xm = x + (m - 1u);
    const uint64_t k = n - (m - 1u);
    std::vector<em> out(m), c(m), s(m);
    const em half_pi = rounded_const(k_pi_ld / 2);
    if (id == 7u) {
        const em g = exact(1) + dtlz_g_ld(id, xm, k);
        const em three_pi = rounded_const(3 * k_pi_ld);
        em_sum y;
        for (uint64_t i = 0; i + 1u < m; ++i) {
            out[i] = exact(x[i]);
            y.add((out[i] / (exact(1) + g)) * (exact(1) + e_sin(three_pi * out[i])));
        }
        out[m - 1u] = (exact(1) + g) * (exact(static_cast<ld>(m)) - y.get());
    } else {
        const em g = dtlz_g_ld(id, xm, k);
        em head = exact(1) + g;
        if (id == 1u) head = exact(0.5L) * head;
        std::vector<em> theta(m);
        if (id == 5u || id == 6u) {
            theta[0] = exact(x[0]);
            const em t = exact(1) / (exact(2) * (exact(1) + g));
            for (uint64_t i = 1u; i < m; ++i) theta[i] = t + (g * exact(x[i])) / (exact(1) + g);
        }
        for (uint64_t j = 0; j < m; ++j) {
            if (id == 1u) {
                c[j] = exact(x[j]);
                s[j] = exact(1) - exact(x[j]);
                continue;
            }
            em a = exact(x[j]);
            if (id == 4u) a = e_pow(a, static_cast<ld>(alpha));
            if (id == 5u || id == 6u) a = theta[j];
            c[j] = e_cos(a * half_pi);
            s[j] = e_sin(a * half_pi);
        }
        em p = head;
        for (uint64_t j = 0; j + 1u < m; ++j) {
            out[m - 1u - j] = p * s[j];
            p = p * c[j];
        }
        out[0] = p;
    }
    for (uint64_t i = 0; i < m; ++i) {
        f[i] = static_cast<double>(out[i].v);
        if (sc) sc[i] = static_cast<double>(out[i].m);
    }
}

// p_distance in long double: the distance functions above, shifted as the
// reference's p_distance shifts them.
double mo_p_distance_ld(int family, unsigned id, uint64_t m, const double *x, uint64_t n, double *sc)
{
    em r{};
    if (family == 7) {
        const em nm1 = exact(static_cast<ld>(n - 1u));
        if (id <= 3u) {
            r = exact(1) + (exact(9) * e_sum(x, 1u, n)) / nm1 - exact(1);
        } else if (id == 4u) {
            const em four_pi = rounded_const(4 * k_pi_ld);
            em_sum s;
            for (uint64_t j = 1u; j < n; ++j) {
                const em xj = exact(x[j]);
                s.add(xj * xj - exact(10) * e_cos(four_pi * xj));
            }
            r = exact(1) + exact(10) * nm1 + s.get() - exact(1);
        } else if (id == 5u) {
            r = exact(zdt_p_distance(5u, x, n));
        } else {
            r = exact(1) + exact(9) * e_pow(e_sum(x, 1u, n) / nm1, 0.25L) - exact(1);
        }
    } else {
        r = dtlz_g_ld(id, x + (m - 1u), n - (m - 1u));
    }
    if (sc) *sc = static_cast<double>(r.m);
    return static_cast<double>(r.v);
}

} // namespace

extern "C" {

const char *orc_mo_last_error(void)
{
    return mo_err.c_str();
}

int orc_mo_dims(int family, unsigned prob_id, uint64_t param, uint64_t fdim, uint64_t *nx, uint64_t *nobj)
{
    return mo_dims(family, prob_id, param, fdim, nx, nobj) ? 0 : 1;
}

void orc_zdt_fitness(unsigned prob_id, const double *x, uint64_t n, double *f)
{
    zdt_fitness(prob_id, x, n, f);
}

double orc_zdt_p_distance(unsigned prob_id, const double *x, uint64_t n)
{
    return zdt_p_distance(prob_id, x, n);
}

void orc_dtlz_fitness(unsigned prob_id, uint64_t fdim, unsigned alpha, const double *x, uint64_t n, double *f)
{
    dtlz_fitness(prob_id, fdim, alpha, x, n, f);
}

double orc_dtlz_p_distance(unsigned prob_id, uint64_t fdim, const double *x, uint64_t n)
{
    // dtlz.cpp:156-163 and :411-420: the distance function of x_M.
    return dtlz_g(prob_id, x + (fdim - 1u), n - (fdim - 1u));
}

// Rows of a batch: f is n x nobj, row-major (the layout of pagmo's fvs).
int orc_mo_batch_fitness(int family, unsigned prob_id, uint64_t param, uint64_t fdim, unsigned alpha,
                         const double *dvs, uint64_t n, uint64_t nx, double *f, int nthreads)
{
    uint64_t want = 0, nobj = 0;
    if (!mo_dims(family, prob_id, param, fdim, &want, &nobj)) return 1;
    if (nx != want) {
        mo_err = "decision vectors of " + std::to_string(nx) + " entries, the problem has " + std::to_string(want);
        return 1;
    }
    orc_detail::parallel_rows(n, nthreads, [&](uint64_t b, uint64_t e) {
        for (; b != e; ++b) {
            if (family == 7)
                zdt_fitness(prob_id, dvs + b * nx, nx, f + b * nobj);
            else
                dtlz_fitness(prob_id, nobj, alpha, dvs + b * nx, nx, f + b * nobj);
        }
    });
    return 0;
}

int orc_mo_batch_fitness_ld(int family, unsigned prob_id, uint64_t param, uint64_t fdim, unsigned alpha,
                            const double *dvs, uint64_t n, uint64_t nx, double *f, double *scale, int nthreads)
{
    uint64_t want = 0, nobj = 0;
    if (!mo_dims(family, prob_id, param, fdim, &want, &nobj)) return 1;
    if (nx != want) {
        mo_err = "decision vectors of " + std::to_string(nx) + " entries, the problem has " + std::to_string(want);
        return 1;
    }
    orc_detail::parallel_rows(n, nthreads, [&](uint64_t b, uint64_t e) {
        for (; b != e; ++b) {
            double *sc = scale ? scale + b * nobj : nullptr;
            if (family == 7)
                zdt_fitness_ld(prob_id, dvs + b * nx, nx, f + b * nobj, sc);
            else
                dtlz_fitness_ld(prob_id, nobj, alpha, dvs + b * nx, nx, f + b * nobj, sc);
        }
    });
    return 0;
}

// p_distance of every row (the reference's per-vector convergence metric);
// with `scale` non-null the long-double values and their error scales.
int orc_mo_batch_p_distance(int family, unsigned prob_id, uint64_t param, uint64_t fdim, const double *dvs,
                            uint64_t n, uint64_t nx, double *out, double *scale, int nthreads)
{
    uint64_t want = 0, nobj = 0;
    if (!mo_dims(family, prob_id, param, fdim, &want, &nobj)) return 1;
    if (nx != want) {
        mo_err = "decision vectors of " + std::to_string(nx) + " entries, the problem has " + std::to_string(want);
        return 1;
    }
    orc_detail::parallel_rows(n, nthreads, [&](uint64_t b, uint64_t e) {
        for (; b != e; ++b) {
            const double *x = dvs + b * nx;
            if (scale)
                out[b] = mo_p_distance_ld(family, prob_id, nobj, x, nx, scale + b);
            else
                out[b] = family == 7 ? zdt_p_distance(prob_id, x, nx) : orc_dtlz_p_distance(prob_id, nobj, x, nx);
        }
    });
    return 0;
}

} // extern "C"
