// Host check of the integer sum-of-squares accumulator
// (pagmo2_gb300/csrc/isum.h) used by the Rosenbrock row loops: random terms
// spread over up to 2^200 in magnitude, 1..200 per sum, added one at a time
// and four at a time (sum4); each sum must lie within 2^-53 + n 2^-60 of the
// exact one (long double) relative, and the special values must follow FP64
// semantics; signed sums within 2^-53 of the result plus n 2^-60 of the
// largest magnitude. Prints "<sums> <worst relative error> <worst signed error
// as a fraction of its bound>"; exit 1 on a violation.
#include "isum.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <limits>
#include <random>

int main()
{
    using namespace pgx::isum;
    std::mt19937_64 g(20261204);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    long sums = 0, violations = 0;
    long double worst = 0;
    for (int trial = 0; trial < 40000; ++trial) {
        const int n = 1 + static_cast<int>(g() % 200u);
        const int spread = (trial % 4 == 0) ? 200 : (trial % 4 == 1) ? 40 : (trial % 4 == 2) ? 4 : 0;
        sq_acc one = make(), four = make();
        long double exact = 0;
        sq_term t[4];
        int k = 0;
        for (int i = 0; i < n; ++i) {
            const double v = std::ldexp(U(g), static_cast<int>(g() % static_cast<uint64_t>(spread + 1)) - spread / 2);
            add_square(one, v);
            t[k++] = square(v, four.flags);
            if (k == 4) {
                add(four, sum4(t[0], t[1], t[2], t[3]));
                k = 0;
            }
            exact += static_cast<long double>(v) * v;
        }
        while (k > 0 && k < 4) t[k++] = sq_term{0u, kEmptyExp};
        if (k == 4) add(four, sum4(t[0], t[1], t[2], t[3]));
        const long double bound = std::ldexp(1.0L, -53) + n * std::ldexp(1.0L, -60);
        for (const sq_acc &a : {one, four}) {
            const long double rel = exact == 0 ? 0 : std::fabs(static_cast<long double>(value(a)) - exact) / exact;
            if (rel > worst) worst = rel;
            if (rel > bound) ++violations;
            ++sums;
        }
    }
    // FP64 semantics of the special values
    sq_acc a = make();
    add_square(a, 1.0);
    add_square(a, std::numeric_limits<double>::infinity());
    violations += !(std::isinf(value(a)) && value(a) > 0);
    a = make();
    add_square(a, std::numeric_limits<double>::infinity());
    add_square(a, std::numeric_limits<double>::quiet_NaN());
    violations += !std::isnan(value(a));
    a = make();
    add_square(a, 1e200);
    violations += !std::isinf(value(a));
    a = make();
    add_square(a, 1e-200);
    add_square(a, 4.9e-324);
    violations += value(a) != 0.0;
    a = make();
    add_square(a, 3e-160);
    violations += value(a) != 3e-160 * 3e-160; // a subnormal square, as FP64 rounds it
    a = make();
    violations += value(a) != 0.0;
    a = make();
    add_square(a, -3.0);
    add_square(a, 4.0);
    violations += value(a) != 25.0;
    // signed sums: values of both signs over 2^-100 .. 2^100; the error is
    // bounded by 2^-53 of the result plus n 2^-60 of the largest magnitude
    long double worst_signed = 0;
    for (int trial = 0; trial < 40000; ++trial) {
        const int n = 1 + static_cast<int>(g() % 200u);
        const int spread = (trial % 3 == 0) ? 200 : (trial % 3 == 1) ? 20 : 0;
        sg_acc acc = make_signed();
        long double exact = 0, big = 0;
        for (int i = 0; i < n; ++i) {
            const double v = std::ldexp(U(g), static_cast<int>(g() % static_cast<uint64_t>(spread + 1)) - spread / 2);
            add_value(acc, v);
            exact += v;
            big = std::max<long double>(big, std::fabs(static_cast<long double>(v)));
        }
        const long double err = std::fabs(static_cast<long double>(value(acc)) - exact);
        const long double bound = std::ldexp(1.0L, -53) * std::fabs(exact) + n * std::ldexp(1.0L, -60) * big;
        if (bound > 0 && err / bound > worst_signed) worst_signed = err / bound;
        if (err > bound) ++violations;
    }
    {
        sg_acc a = make_signed();
        add_value(a, 1.5);
        add_value(a, -1.5);
        violations += value(a) != 0.0;
        a = make_signed();
        add_value(a, std::numeric_limits<double>::infinity());
        add_value(a, -std::numeric_limits<double>::infinity());
        violations += !std::isnan(value(a));
        a = make_signed();
        add_value(a, -std::numeric_limits<double>::infinity());
        add_value(a, 3.0);
        violations += !(std::isinf(value(a)) && value(a) < 0);
        a = make_signed();
        add_value(a, 0.1);
        add_value(a, 0.2);
        add_value(a, -0.3);
        violations += std::fabs(value(a)) > 1e-16;
        a = make_signed();
        add_value(a, -2.5);
        add_value(a, 4.9e-324);
        violations += value(a) != -2.5;
    }
    std::printf("%ld %.3Le %.3Le\n", sums, worst, worst_signed);
    return violations == 0 ? 0 : 1;
}
