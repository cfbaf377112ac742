// Host check of the fixed-point sin/cos(2 pi x) (pagmo2_gb300/csrc/trig_fixed.h)
// used by the rastrigin and ackley rows, in both rounding forms of to_double:
// x over every binade of the range (2^-60 .. 2^40), near the multiples of 1/4
// and exact multiples of 1/2, against long double with an exact reduction
// r = x - rint(2x)/2. Bounds: cos within 2^-53 absolute, sin within 2^-52
// relative (both about one unit of the last place). Prints "<values> <worst
// cos error> <worst sin relative error>"; exit 1 on a violation.
#include "trig_fixed.h"

#include <cmath>
#include <cstdio>
#include <random>

int main()
{
    using namespace pgx::trigfx;
    const long double pi = 3.141592653589793238462643383279502884L;
    std::mt19937_64 g(20261204);
    long values = 0, violations = 0;
    long double worst_c = 0, worst_s = 0;
    auto check = [&](double x) {
        if (!in_range(x)) return;
        double s, c, sv, cv;
        sincos_2pi(x, s, c);
        sincos_2pi<true>(x, sv, cv); // the conversion form: the same values up to the rounding of ties
        const double c1 = cos_2pi(x), c1v = cos_2pi<true>(x);
        const long double k = std::rint(2.0L * x);
        const long double r = static_cast<long double>(x) - k / 2;
        const long double sign = std::fmod(std::fabs(k), 2.0L) == 1.0L ? -1.0L : 1.0L;
        const long double ce = sign * std::cos(2 * pi * r), se = sign * std::sin(2 * pi * r);
        for (int form = 0; form < 2; ++form) {
            const double cc = form ? cv : c, ss = form ? sv : s;
            const long double dc = std::fabs(static_cast<long double>(cc) - ce);
            const long double ds = se == 0 ? std::fabs(static_cast<long double>(ss)) : std::fabs((ss - se) / se);
            if (dc > worst_c) worst_c = dc;
            if (ds > worst_s) worst_s = ds;
            if (dc > std::ldexp(1.0L, -53) || ds > std::ldexp(1.0L, -52)) ++violations;
        }
        if (c1 != c || c1v != cv) ++violations;
        ++values;
    };
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    for (int e = -60; e < 40; ++e)
        for (int i = 0; i < 20000; ++i) check(std::ldexp(U(g), e + 1));
    for (int i = 0; i < 200000; ++i) {
        const double q = std::floor(U(g) * 4000.0) / 4.0; // a multiple of 1/4
        check(q);
        check(std::nextafter(q, 1e9));
        check(std::nextafter(q, -1e9));
        check(q + std::ldexp(U(g), -30));
    }
    for (double x : {0.0, -0.0, 0.5, -0.5, 1.0, 0.25, -0.25, 0.75, 1e-18, -3e-18, 123456.5, 1099511627775.5})
        check(x);
    std::printf("%ld %.3Le %.3Le\n", values, worst_c, worst_s);
    return violations == 0 ? 0 : 1;
}
