// Host check of the fixed-point reciprocal (pagmo2_gb300/csrc/rcp_fixed.h)
// used by the Lennard-Jones pair loops: for seeds one unit of the last place
// either side of the correctly rounded single-precision reciprocal (the
// device's approximate reciprocal is within one unit), the result must be
// within 0.5 + 2^-10 units of the last place of 1/d, and the cube within
// 0.5 + 2^-5 units of the last place of 1/d^3, measured in long double.
// Prints "<values> <worst error in ulp> <not correctly rounded> <worst cube
// error in ulp>"; exit 1 on a violation.
#include "rcp_fixed.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

namespace
{
uint64_t bits_of(double d)
{
    uint64_t b;
    std::memcpy(&b, &d, 8);
    return b;
}
double from_bits(uint64_t b)
{
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}
uint32_t fbits_of(float f)
{
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}
float ffrom_bits(uint32_t b)
{
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}
} // namespace

int main()
{
    using namespace pgx::rcpfx;
    std::mt19937_64 g(20261204);
    long values = 0, violations = 0, not_cr = 0;
    long double worst = 0, worst3 = 0;
    auto check = [&](double d, int seed_offset) {
        const uint64_t b = bits_of(d);
        const uint32_t ex = static_cast<uint32_t>(b >> 52) & 0x7ffu;
        const uint64_t f = b & ((1ull << 52) - 1u);
        const float m23 = ffrom_bits(seed_input_bits(f));
        const uint32_t yb = fbits_of(1.0f / m23) + static_cast<uint32_t>(seed_offset);
        const double r = from_bits(rcp_bits(ex, f, seed_q32(yb)));
        uint64_t ib, cb;
        rcp_and_cube_bits(ex, f, seed_q32(yb), &ib, &cb);
        const long double exact = 1.0L / static_cast<long double>(d);
        int e2;
        std::frexp(static_cast<double>(exact), &e2);
        const long double ulp = std::ldexp(1.0L, e2 - 53);
        const long double err = std::fabs(static_cast<long double>(r) - exact) / ulp;
        if (err > worst) worst = err;
        if (err > 0.5L + 1.0L / 1024.0L || ib != bits_of(r)) ++violations;
        if (r != 1.0 / d) ++not_cr;
        // 1/d^3 from 1/d exactly: long double keeps 64 bits, so exact^3 is
        // within 2^-62 relative; the bound leaves room for that
        const long double inv = 1.0L / static_cast<long double>(d);
        const long double exact3 = inv * inv * inv;
        std::frexp(static_cast<double>(exact3), &e2);
        const long double err3 = std::fabs(static_cast<long double>(from_bits(cb)) - exact3) / std::ldexp(1.0L, e2 - 53);
        if (err3 > worst3) worst3 = err3;
        if (err3 > 0.5L + 1.0L / 32.0L) ++violations;
        ++values;
    };
    for (int k = 0; k < 2000000; ++k) {
        const double m = 1.0 + static_cast<double>(g() >> 12) * 0x1p-52;
        check(std::ldexp(m, static_cast<int>(g() % 201u) - 100), static_cast<int>(g() % 3u) - 1);
    }
    const uint64_t edges[] = {0u, 1u, 2u, 3u, (1ull << 52) - 1u, (1ull << 52) - 2u, 1ull << 51, (1ull << 29) - 1u,
                              1ull << 29, (1ull << 52) - (1ull << 29), 0x5555555555555ull, 0xaaaaaaaaaaaaaull};
    for (int e = -100; e <= 100; ++e)
        for (uint64_t f : edges)
            for (int off = -1; off <= 1; ++off)
                check(from_bits((static_cast<uint64_t>(1023 + e) << 52) | f), off);
    std::printf("%ld %.6Lf %ld %.6Lf\n", values, worst, not_cr, worst3);
    return violations == 0 ? 0 : 1;
}
