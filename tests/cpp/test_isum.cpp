// Host check of the integer sum-of-squares accumulator
// (pagmo2_gb300/csrc/isum.h) used by the Rosenbrock row loops: random terms
// spread over up to 2^200 in magnitude, 1..200 per sum, added one at a time
// and four at a time (sum4); each sum must lie within 2^-53 + n 2^-60 of the
// exact one (long double) relative, and the special values must follow FP64
// semantics. Prints "<sums> <worst relative error>"; exit 1 on a violation.
#include "isum.h"

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
    std::printf("%ld %.3Le\n", sums, worst);
    return violations == 0 ? 0 : 1;
}
