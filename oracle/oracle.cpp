// CPU oracle for the pagmo batch-evaluation path (TEST INFRASTRUCTURE ONLY).
// See oracle.h for the contract. Reference citations are paths inside the
// pagmo 2.19.1 source tree.
//
// Compile with -ffp-contract=off so that the mirror functions do not fuse
// multiply-adds (the reference is compiled the same way by oracle/Makefile,
// and x86-64 builds of pagmo never contract without -mfma).
#include "oracle.h"
#include "rows.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace
{
using orc_detail::parallel_rows;
using orc_detail::resolve_threads;

thread_local std::string g_err;

// The reference's pi (include/pagmo/detail/constants.hpp:37-40) and its
// rastrigin angular frequency omega = 2*pi (src/problems/rastrigin.cpp:65).
constexpr double k_pi = 3.1415926535897932384626433832795028841971693993;
constexpr double k_omega = 2. * k_pi;

using ld = long double;

// Pinned-atom decode of a lennard_jones decision vector
// (src/problems/lennard_jones.cpp:132-151): atom 0 is the origin, atom 1 sits
// on the z axis at x[0], atom 2 in the y-z plane at (x[1], x[2]), and atom
// k >= 3 is x[3(k-2) .. 3(k-2)+2].
inline double lj_coord(const double *x, unsigned atom, unsigned c)
{
    if (atom == 0u) return 0.0;
    if (atom == 1u) return c < 2u ? 0.0 : x[0];
    if (atom == 2u) return c == 0u ? 0.0 : x[c];
    return x[3u * (atom - 2u) + c];
}

// Index of the decision variable that holds coordinate c of an atom, or -1 if
// the coordinate is pinned.
inline long lj_var(unsigned atom, unsigned c)
{
    if (atom == 0u) return -1;
    if (atom == 1u) return c == 2u ? 0 : -1;
    if (atom == 2u) return c == 0u ? -1 : static_cast<long>(c);
    return static_cast<long>(3u * (atom - 2u) + c);
}

// NaN-aware ordering of include/pagmo/detail/custom_comparisons.hpp:54-89:
// NaN sorts after every number, two NaNs are unordered.
inline bool lt_f(double a, double b)
{
    if (!std::isnan(a)) return std::isnan(b) ? true : a < b;
    return false;
}
inline bool gt_f(double a, double b)
{
    if (!std::isnan(a)) return std::isnan(b) ? false : a > b;
    return !std::isnan(b);
}

// pareto_dominance (src/utils/multi_objective.cpp:97-113).
inline bool dominates(const double *a, const double *b, uint64_t m)
{
    bool strict = false;
    for (uint64_t i = 0; i < m; ++i) {
        if (gt_f(a[i], b[i])) return false;
        if (lt_f(a[i], b[i])) strict = true;
    }
    return strict;
}

bool check_kind(int kind, uint64_t param, uint64_t nx)
{
    switch (kind) {
        case 1:
            if (param < 1u || nx != param) break;
            return true;
        case 2:
            if (param < 2u || nx != param) break;
            return true;
        case 3:
            if (param < 3u || nx != 3u * param - 6u) break;
            return true;
        case 4:
        case 5:
        case 6:
            if (param < 1u || nx != param) break;
            return true;
        default:
            break;
    }
    g_err = "invalid problem kind/parameter/dimension: kind " + std::to_string(kind) + ", param "
            + std::to_string(param) + ", nx " + std::to_string(nx);
    return false;
}

// Per-row fitness as pagmo's problem::fitness returns it: a fresh vector.
std::vector<double> row_fitness(int kind, uint64_t param, const std::vector<double> &x)
{
    switch (kind) {
        case 1:
            return {orc_rastrigin_fitness(x.data(), x.size())};
        case 2:
            return {orc_rosenbrock_fitness(x.data(), x.size())};
        case 4:
            return {orc_ackley_fitness(x.data(), x.size())};
        case 5:
            return {orc_griewank_fitness(x.data(), x.size())};
        case 6:
            return {orc_schwefel_fitness(x.data(), x.size())};
        default:
            return {orc_lj_fitness(x.data(), param)};
    }
}
} // namespace

extern "C" {

const char *orc_last_error(void)
{
    return g_err.c_str();
}

// ---------------------------------------------------------------- mirrors

// src/problems/rastrigin.cpp:62-72: sum of x^2 - 10 cos(omega x), then + 10 n.
double orc_rastrigin_fitness(const double *x, uint64_t n)
{
    double f = 0.;
    for (uint64_t i = 0; i < n; ++i) {
        f += x[i] * x[i] - 10. * std::cos(k_omega * x[i]);
    }
    f += 10. * static_cast<double>(n);
    return f;
}

// src/problems/rastrigin.cpp:98-107.
void orc_rastrigin_gradient(const double *x, uint64_t n, double *g)
{
    for (uint64_t i = 0; i < n; ++i) {
        g[i] = 2 * x[i] + 10.0 * k_omega * std::sin(k_omega * x[i]);
    }
}

// src/problems/rosenbrock.cpp:59-66.
double orc_rosenbrock_fitness(const double *x, uint64_t n)
{
    double r = 0.;
    for (uint64_t i = 0; i + 1u < n; ++i) {
        const double t = x[i] * x[i] - x[i + 1];
        const double u = x[i] - 1;
        r += 100. * t * t + u * u;
    }
    return r;
}

// src/problems/rosenbrock.cpp:83-92.
void orc_rosenbrock_gradient(const double *x, uint64_t n, double *g)
{
    g[0] = -400. * x[0] * (x[1] - x[0] * x[0]) - 2. * (1 - x[0]);
    for (uint64_t i = 1; i + 1u < n; ++i) {
        g[i] = -400. * x[i] * (x[i + 1u] - x[i] * x[i]) - 2. * (1 - x[i]) + 200. * (x[i] - x[i - 1u] * x[i - 1u]);
    }
    g[n - 1u] = 200. * (x[n - 1u] - x[n - 2u] * x[n - 2u]);
}

// src/problems/lennard_jones.cpp:72-91: pairs i < j in row-major order,
// r^2 through std::pow(.,2), r^-6 = pow(r^2, -3); a zero distance overwrites
// the running sum with DBL_MAX and the loop continues; finally times 4.
double orc_lj_fitness(const double *x, uint64_t atoms)
{
    const unsigned na = static_cast<unsigned>(atoms);
    double f = 0.;
    for (unsigned i = 0u; i < na - 1u; ++i) {
        for (unsigned j = i + 1u; j < na; ++j) {
            const double dist = std::pow(lj_coord(x, i, 0) - lj_coord(x, j, 0), 2)
                                + std::pow(lj_coord(x, i, 1) - lj_coord(x, j, 1), 2)
                                + std::pow(lj_coord(x, i, 2) - lj_coord(x, j, 2), 2);
            if (dist == 0.0) {
                f = std::numeric_limits<double>::max();
            } else {
                const double sixth = std::pow(dist, -3);
                f += (std::pow(sixth, 2) - sixth);
            }
        }
    }
    return 4 * f;
}

// ---------------------------------------------------------------- long double

double orc_rastrigin_fitness_ld(const double *x, uint64_t n, double *scale)
{
    const ld om = static_cast<ld>(k_omega);
    ld f = 0, s = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const ld xi = x[i];
        const ld c = cosl(om * xi);
        f += xi * xi - 10.0L * c;
        s += xi * xi + 10.0L * fabsl(c);
    }
    f += 10.0L * static_cast<ld>(n);
    s += 10.0L * static_cast<ld>(n);
    if (scale) *scale = static_cast<double>(s);
    return static_cast<double>(f);
}

void orc_rastrigin_gradient_ld(const double *x, uint64_t n, double *g, double *gscale)
{
    const ld om = static_cast<ld>(k_omega);
    for (uint64_t i = 0; i < n; ++i) {
        const ld xi = x[i];
        const ld sn = sinl(om * xi);
        g[i] = static_cast<double>(2.0L * xi + 10.0L * om * sn);
        if (gscale) gscale[i] = static_cast<double>(2.0L * fabsl(xi) + 10.0L * om * fabsl(sn));
    }
}

double orc_rosenbrock_fitness_ld(const double *x, uint64_t n, double *scale)
{
    // Condition scale: first-order error bound of the reference's evaluation.
    // The terms are non-negative, but t = x_i^2 - x_{i+1} is formed from a
    // rounded x_i^2, which contributes 2*100*|t|*x_i^2 per term.
    ld r = 0, s = 0;
    for (uint64_t i = 0; i + 1u < n; ++i) {
        const ld xi = x[i], xn = x[i + 1];
        const ld t = xi * xi - xn, u = xi - 1.0L;
        r += 100.0L * t * t + u * u;
        s += 100.0L * t * t + u * u + 200.0L * fabsl(t) * xi * xi;
    }
    if (scale) *scale = static_cast<double>(s);
    return static_cast<double>(r);
}

void orc_rosenbrock_gradient_ld(const double *x, uint64_t n, double *g, double *gscale)
{
    // gscale: first-order error bound, counting the rounded squares inside
    // both chain terms (400 |x_i| x_i^2 and 200 x_{i-1}^2).
    for (uint64_t i = 0; i < n; ++i) {
        ld v = 0, s = 0;
        const ld xi = x[i];
        if (i + 1u < n) {
            const ld t = static_cast<ld>(x[i + 1]) - xi * xi;
            const ld a = -400.0L * xi * t;
            const ld b = -2.0L * (1.0L - xi);
            v += a + b;
            s += fabsl(a) + fabsl(b) + 400.0L * fabsl(xi) * xi * xi;
        }
        if (i > 0u) {
            const ld xp = x[i - 1];
            const ld c = 200.0L * (xi - xp * xp);
            v += c;
            s += fabsl(c) + 200.0L * xp * xp;
        }
        g[i] = static_cast<double>(v);
        if (gscale) gscale[i] = static_cast<double>(s);
    }
}

double orc_lj_fitness_ld(const double *x, uint64_t atoms, double *scale)
{
    const unsigned na = static_cast<unsigned>(atoms);
    ld f = 0, s = 0;
    bool zero = false;
    for (unsigned i = 0u; i + 1u < na; ++i) {
        for (unsigned j = i + 1u; j < na; ++j) {
            ld d = 0;
            for (unsigned c = 0; c < 3u; ++c) {
                const ld dc = static_cast<ld>(lj_coord(x, i, c)) - static_cast<ld>(lj_coord(x, j, c));
                d += dc * dc;
            }
            if (d == 0) {
                zero = true;
                continue;
            }
            const ld six = 1.0L / (d * d * d);
            f += six * six - six;
            s += six * six + six;
        }
    }
    if (scale) *scale = static_cast<double>(4.0L * s);
    if (zero) return std::isnan(static_cast<double>(f)) ? static_cast<double>(f) : HUGE_VAL;
    return static_cast<double>(4.0L * f);
}

// dE/dx for the free coordinates. With d = |r_i - r_j|^2 and s = d^-3,
// E = 4 sum_{i<j} (s^2 - s) gives dE/dr_i = sum_{j != i} -24 s (2s - 1) / d (r_i - r_j).
void orc_lj_gradient_ld(const double *x, uint64_t atoms, double *g, double *gscale)
{
    const unsigned na = static_cast<unsigned>(atoms);
    std::vector<ld> G(3u * na, 0.0L), S(3u * na, 0.0L);
    for (unsigned i = 0u; i + 1u < na; ++i) {
        for (unsigned j = i + 1u; j < na; ++j) {
            ld dv[3], d = 0;
            for (unsigned c = 0; c < 3u; ++c) {
                dv[c] = static_cast<ld>(lj_coord(x, i, c)) - static_cast<ld>(lj_coord(x, j, c));
                d += dv[c] * dv[c];
            }
            const ld inv = 1.0L / d;
            const ld six = inv * inv * inv;
            const ld coef = -24.0L * six * (2.0L * six - 1.0L) * inv;
            const ld cabs = 24.0L * six * (2.0L * six + 1.0L) * inv;
            for (unsigned c = 0; c < 3u; ++c) {
                G[3u * i + c] += coef * dv[c];
                G[3u * j + c] -= coef * dv[c];
                S[3u * i + c] += cabs * fabsl(dv[c]);
                S[3u * j + c] += cabs * fabsl(dv[c]);
            }
        }
    }
    for (unsigned a = 1u; a < na; ++a) {
        for (unsigned c = 0; c < 3u; ++c) {
            const long v = lj_var(a, c);
            if (v < 0) continue;
            g[v] = static_cast<double>(G[3u * a + c]);
            if (gscale) gscale[v] = static_cast<double>(S[3u * a + c]);
        }
    }
}

// ------------------------------------------- ackley, griewank, schwefel

// src/problems/ackley.cpp:62-77, in the reference's operation order.
double orc_ackley_fitness(const double *x, uint64_t n)
{
    const double omega = 2. * k_pi;
    double s1 = 0., s2 = 0.;
    const double nepero = std::exp(1.0);
    for (uint64_t i = 0; i < n; ++i) {
        s1 += x[i] * x[i];
        s2 += std::cos(omega * x[i]);
    }
    return -20 * std::exp(-0.2 * std::sqrt(1.0 / static_cast<double>(n) * s1))
           - std::exp(1.0 / static_cast<double>(n) * s2) + 20 + nepero;
}

// src/problems/griewank.cpp:62-76.
double orc_griewank_fitness(const double *x, uint64_t n)
{
    const double fr = 4000.;
    double retval = 0., p = 1.;
    for (uint64_t i = 0; i < n; ++i) retval += x[i] * x[i];
    for (uint64_t i = 0; i < n; ++i) p *= std::cos(x[i] / std::sqrt(static_cast<double>(i) + 1.0));
    return retval / fr - p + 1.;
}

// src/problems/schwefel.cpp:62-70.
double orc_schwefel_fitness(const double *x, uint64_t n)
{
    double f = 0.;
    for (uint64_t i = 0; i < n; ++i) f += x[i] * std::sin(std::sqrt(std::abs(x[i])));
    return 418.9828872724338 * static_cast<double>(n) - f;
}

// Long-double versions. scale = first-order error bound of the reference's
// FP64 evaluation: the magnitudes of the combined terms plus the effect of
// its rounded arguments (omega*x in ackley, x/sqrt(i+1) in griewank,
// sqrt|x| in schwefel), each per unit roundoff.
double orc_ackley_fitness_ld(const double *x, uint64_t n, double *scale)
{
    const ld om = static_cast<ld>(k_omega);
    ld s1 = 0, s2 = 0, arg = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const ld xi = x[i];
        s1 += xi * xi;
        s2 += cosl(om * xi);
        arg += fabsl(om * xi);
    }
    const ld nn = static_cast<ld>(n), r = sqrtl(s1 / nn);
    const ld a = 20.0L * expl(-0.2L * r), b = expl(s2 / nn), e = expl(1.0L);
    if (scale) *scale = static_cast<double>(a * (1.0L + 0.2L * r) + b * (1.0L + arg / nn) + 20.0L + e);
    return static_cast<double>(-a - b + 20.0L + e);
}

double orc_griewank_fitness_ld(const double *x, uint64_t n, double *scale)
{
    std::vector<ld> c(n), sn(n), arg(n), pre(n + 1), suf(n + 1);
    ld sum = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const ld xi = x[i];
        sum += xi * xi;
        arg[i] = xi / sqrtl(static_cast<ld>(i) + 1.0L);
        c[i] = cosl(arg[i]);
        sn[i] = sinl(arg[i]);
    }
    pre[0] = 1;
    for (uint64_t i = 0; i < n; ++i) pre[i + 1] = pre[i] * c[i];
    suf[n] = 1;
    for (uint64_t i = n; i-- > 0;) suf[i] = suf[i + 1] * c[i];
    ld sens = 0;
    for (uint64_t i = 0; i < n; ++i) sens += fabsl(pre[i] * suf[i + 1] * sn[i] * arg[i]);
    const ld p = pre[n];
    if (scale) *scale = static_cast<double>(sum / 4000.0L + 1.0L + fabsl(p) * static_cast<ld>(2u * n) + 2.0L * sens);
    return static_cast<double>(sum / 4000.0L - p + 1.0L);
}

double orc_schwefel_fitness_ld(const double *x, uint64_t n, double *scale)
{
    ld f = 0, s = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const ld xi = x[i], q = sqrtl(fabsl(xi));
        const ld t = xi * sinl(q);
        f += t;
        s += fabsl(t) + fabsl(xi * cosl(q)) * q;
    }
    const ld c = 418.9828872724338L * static_cast<ld>(n);
    if (scale) *scale = static_cast<double>(c + s);
    return static_cast<double>(c - f);
}

// ---------------------------------------------------------------- batch runners

int orc_batch_fitness(int kind, uint64_t param, const double *dvs, uint64_t n, uint64_t nx, double *f, int nthreads)
{
    if (!check_kind(kind, param, nx)) return 1;
    parallel_rows(n, nthreads, [&](uint64_t b, uint64_t e) {
        // thread_bfe.cpp:94-123: one temporary dv per chunk, a fresh fitness
        // vector per row.
        std::vector<double> tmp(nx);
        for (; b != e; ++b) {
            std::copy(dvs + b * nx, dvs + (b + 1u) * nx, tmp.begin());
            const auto fv = row_fitness(kind, param, tmp);
            f[b] = fv[0];
        }
    });
    return 0;
}

int orc_batch_gradient(int kind, uint64_t param, const double *dvs, uint64_t n, uint64_t nx, double *g, int nthreads)
{
    if (!check_kind(kind, param, nx)) return 1;
    if (kind >= 4) {
        g_err = "The gradient has been requested but it is not implemented in the UDP";
        return 1;
    }
    parallel_rows(n, nthreads, [&](uint64_t b, uint64_t e) {
        std::vector<double> tmp(nx), out(nx);
        for (; b != e; ++b) {
            std::copy(dvs + b * nx, dvs + (b + 1u) * nx, tmp.begin());
            if (kind == 1)
                orc_rastrigin_gradient(tmp.data(), nx, out.data());
            else if (kind == 2)
                orc_rosenbrock_gradient(tmp.data(), nx, out.data());
            else
                orc_lj_gradient_ld(tmp.data(), param, out.data(), nullptr);
            std::copy(out.begin(), out.end(), g + b * nx);
        }
    });
    return 0;
}

int orc_batch_fitness_ld(int kind, uint64_t param, const double *dvs, uint64_t n, uint64_t nx, double *f,
                         double *scale, int nthreads)
{
    if (!check_kind(kind, param, nx)) return 1;
    parallel_rows(n, nthreads, [&](uint64_t b, uint64_t e) {
        for (; b != e; ++b) {
            const double *x = dvs + b * nx;
            double *sc = scale ? scale + b : nullptr;
            if (kind == 1)
                f[b] = orc_rastrigin_fitness_ld(x, nx, sc);
            else if (kind == 2)
                f[b] = orc_rosenbrock_fitness_ld(x, nx, sc);
            else if (kind == 4)
                f[b] = orc_ackley_fitness_ld(x, nx, sc);
            else if (kind == 5)
                f[b] = orc_griewank_fitness_ld(x, nx, sc);
            else if (kind == 6)
                f[b] = orc_schwefel_fitness_ld(x, nx, sc);
            else
                f[b] = orc_lj_fitness_ld(x, param, sc);
        }
    });
    return 0;
}

int orc_batch_gradient_ld(int kind, uint64_t param, const double *dvs, uint64_t n, uint64_t nx, double *g,
                          double *gscale, int nthreads)
{
    if (!check_kind(kind, param, nx)) return 1;
    if (kind >= 4) {
        g_err = "The gradient has been requested but it is not implemented in the UDP";
        return 1;
    }
    parallel_rows(n, nthreads, [&](uint64_t b, uint64_t e) {
        for (; b != e; ++b) {
            const double *x = dvs + b * nx;
            double *gs = gscale ? gscale + b * nx : nullptr;
            if (kind == 1)
                orc_rastrigin_gradient_ld(x, nx, g + b * nx, gs);
            else if (kind == 2)
                orc_rosenbrock_gradient_ld(x, nx, g + b * nx, gs);
            else
                orc_lj_gradient_ld(x, param, g + b * nx, gs);
        }
    });
    return 0;
}

// ---------------------------------------------------------------- multi-objective

int orc_pareto_dominance(const double *a, const double *b, uint64_t m)
{
    return dominates(a, b, m) ? 1 : 0;
}

// Restatement of fast_non_dominated_sorting (src/utils/multi_objective.cpp:200-257)
// over flat arrays.
int orc_fnds(const double *pts, uint64_t n, uint64_t m, uint64_t *rank, uint64_t *dom_count, uint64_t *front_offsets,
             uint64_t *front_indices, uint64_t *n_fronts, uint64_t *dl_offsets, uint64_t *dl_indices,
             uint64_t dl_capacity)
{
    if (n < 2u) {
        g_err = "At least two points are needed for fast_non_dominated_sorting: " + std::to_string(n) + " detected.";
        return 1;
    }
    std::vector<std::vector<uint64_t>> dl(n);
    std::vector<uint64_t> dc(n, 0u);
    // :212-227 -- for each i, the pairs (i, j < i) in ascending j.
    for (uint64_t i = 0; i < n; ++i) {
        for (uint64_t j = 0; j < i; ++j) {
            if (dominates(pts + i * m, pts + j * m, m)) {
                dl[i].push_back(j);
                ++dc[j];
            } else if (dominates(pts + j * m, pts + i * m, m)) {
                dl[j].push_back(i);
                ++dc[i];
            }
        }
    }
    // :228-254 -- first front in index order, later fronts in traversal order.
    std::vector<uint64_t> cur, cnt(dc);
    for (uint64_t i = 0; i < n; ++i) {
        if (dc[i] == 0u) {
            rank[i] = 0u;
            cur.push_back(i);
        }
    }
    uint64_t pos = 0, nf = 0, level = 0;
    front_offsets[0] = 0;
    while (!cur.empty()) {
        for (auto v : cur) front_indices[pos++] = v;
        front_offsets[++nf] = pos;
        std::vector<uint64_t> next;
        for (auto p : cur) {
            for (auto q : dl[p]) {
                if (--cnt[q] == 0u) {
                    rank[q] = level + 1u;
                    next.push_back(q);
                }
            }
        }
        ++level;
        cur.swap(next);
    }
    *n_fronts = nf;
    for (uint64_t i = 0; i < n; ++i) dom_count[i] = dc[i];
    if (dl_offsets) {
        uint64_t q = 0;
        dl_offsets[0] = 0;
        for (uint64_t i = 0; i < n; ++i) {
            for (auto v : dl[i]) {
                if (q >= dl_capacity) {
                    g_err = "dom_list capacity exceeded";
                    return 1;
                }
                dl_indices[q++] = v;
            }
            dl_offsets[i + 1] = q;
        }
    }
    return 0;
}

// Restatement of crowding_distance (src/utils/multi_objective.cpp:280-315),
// including its use of std::sort (not stable) with the NaN-aware comparator:
// with the same standard library the order of tied values is the reference's.
int orc_crowding(const double *pts, uint64_t n, uint64_t m, double *out)
{
    return orc_crowding_ex(pts, n, m, 0, out);
}

// stable != 0: std::stable_sort instead of std::sort, i.e. equal objective
// values keep their order in the front (the GPU's documented tie rule).
int orc_crowding_ex(const double *pts, uint64_t n, uint64_t m, int stable, double *out)
{
    if (n < 2u) {
        g_err = "A non dominated front must contain at least two points: " + std::to_string(n) + " detected.";
        return 1;
    }
    if (m < 2u) {
        g_err = "Points in the non dominated front must contain at least two objectives: " + std::to_string(m)
                + " detected.";
        return 1;
    }
    std::vector<uint64_t> idx(n);
    std::iota(idx.begin(), idx.end(), uint64_t(0));
    std::fill(out, out + n, 0.);
    for (uint64_t i = 0; i < m; ++i) {
        const auto cmp = [i, m, pts](uint64_t a, uint64_t b) { return lt_f(pts[a * m + i], pts[b * m + i]); };
        if (stable)
            std::stable_sort(idx.begin(), idx.end(), cmp);
        else
            std::sort(idx.begin(), idx.end(), cmp);
        out[idx[0]] = std::numeric_limits<double>::infinity();
        out[idx[n - 1u]] = std::numeric_limits<double>::infinity();
        const double df = pts[idx[n - 1u] * m + i] - pts[idx[0] * m + i];
        for (uint64_t j = 1u; j + 1u < n; ++j) {
            out[idx[j]] += (pts[idx[j + 1u] * m + i] - pts[idx[j - 1u] * m + i]) / df;
        }
    }
    return 0;
}

// src/algorithms/nsga2.cpp:183-206.
int orc_nsga2_crowding(const double *pts, uint64_t n, uint64_t m, const uint64_t *front_offsets,
                       const uint64_t *front_indices, uint64_t n_fronts, double *out)
{
    return orc_nsga2_crowding_ex(pts, n, m, front_offsets, front_indices, n_fronts, 0, out);
}

int orc_nsga2_crowding_ex(const double *pts, uint64_t n, uint64_t m, const uint64_t *front_offsets,
                          const uint64_t *front_indices, uint64_t n_fronts, int stable, double *out)
{
    std::vector<double> buf, cd;
    for (uint64_t f = 0; f < n_fronts; ++f) {
        const uint64_t b = front_offsets[f], e = front_offsets[f + 1];
        const uint64_t k = e - b;
        if (k == 1u || k == 2u) {
            for (uint64_t t = b; t < e; ++t) out[front_indices[t]] = std::numeric_limits<double>::infinity();
            continue;
        }
        buf.resize(k * m);
        cd.resize(k);
        for (uint64_t t = 0; t < k; ++t)
            std::memcpy(buf.data() + t * m, pts + front_indices[b + t] * m, m * sizeof(double));
        const int st = orc_crowding_ex(buf.data(), k, m, stable, cd.data());
        if (st) return st;
        for (uint64_t t = 0; t < k; ++t) out[front_indices[b + t]] = cd[t];
    }
    (void)n;
    return 0;
}

} // extern "C"
