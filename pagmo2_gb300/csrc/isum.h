// Sums of squares with integer arithmetic (no FP64 instruction).
//
// Rosenbrock's fitness is two sums of squares, sum t_i^2 and sum (x_i - 1)^2;
// as FP64 FMAs they are a third of the FP64 instructions of the fused
// fitness + gradient row loop, on a pipe that retires two lanes per SM per
// clock while the integer pipes are mostly idle. Here each square is formed
// from the 53-bit significand with 32 x 32-bit integer multiplies and added to
// a floating accumulator held in integers:
//  - v = m 2^(ex - 1075) with m the significand (2^52 <= m < 2^53), so
//    v^2 = m^2 2^(2 ex - 2150) and p = floor(m^2 / 2^44) (2^60 <= p < 2^62,
//    the three partial products truncated: below 2^-59 relative) gives
//    v^2 = p 2^q, q = 2 ex - 2106;
//  - the accumulator is m_acc 2^e_acc with m_acc < 2^62: both operands are
//    aligned to the larger exponent (truncating the smaller one by at most one
//    unit of 2^e, i.e. below 2^-60 of the sum) and added; a sum that reaches
//    2^62 is halved (one more unit); four squares can first be summed the same
//    way among themselves (sum4) and added once;
//  - zero and subnormal v add nothing (their FP64 squares underflow below the
//    smallest subnormal), infinity and NaN set sticky flags that the result
//    reports as +inf and NaN, as the FP64 sums would; the exponent is an
//    integer, so sums past the double range overflow only when read.
// Every addition is thus within 2^-58 of the exact sum relative (FP64 FMAs:
// 2^-53), and value() rounds once.
// The header compiles as plain C++ too, so that it can be checked on the host.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>

#if defined(__CUDACC__)
#define PGX_ISUM_HD __host__ __device__ __forceinline__
#else
#define PGX_ISUM_HD inline
#endif

namespace pgx
{
namespace isum
{

struct sq_acc {
    uint64_t m;     // significand, < 2^62
    int32_t e;      // exponent of its unit
    uint32_t flags; // 1: an infinity was added, 2: a NaN
};

constexpr int32_t kEmptyExp = -(1 << 20); // below any square's exponent

PGX_ISUM_HD sq_acc make()
{
    return sq_acc{0u, kEmptyExp, 0u};
}

PGX_ISUM_HD uint64_t bits_of(double v)
{
#if defined(__CUDA_ARCH__)
    return static_cast<uint64_t>(__double_as_longlong(v));
#else
    uint64_t b;
    std::memcpy(&b, &v, 8);
    return b;
#endif
}

PGX_ISUM_HD int32_t imax(int32_t a, int32_t b)
{
    return a > b ? a : b;
}

PGX_ISUM_HD int32_t imin(int32_t a, int32_t b)
{
    return a < b ? a : b;
}

// v^2 = p 2^q (2^60 <= p < 2^62); zero and subnormal v give p = 0, and
// infinity or NaN p = 0 with the flag set in *flags.
struct sq_term {
    uint64_t p;
    int32_t q;
};

PGX_ISUM_HD sq_term square(double v, uint32_t &flags)
{
    const uint64_t b = bits_of(v);
    const uint32_t hi = static_cast<uint32_t>(b >> 32);
    const uint32_t ex = (hi >> 20) & 0x7ffu;
    if (ex == 0u || ex == 0x7ffu) {
        if (ex) flags |= (b << 12) != 0u ? 2u : 1u;
        return sq_term{0u, kEmptyExp};
    }
    const uint32_t mh = (hi & 0xfffffu) | 0x100000u;
    const uint32_t ml = static_cast<uint32_t>(b);
    const uint64_t p = ((static_cast<uint64_t>(mh) * mh) << 20) + ((static_cast<uint64_t>(mh) * ml) >> 11)
                       + ((static_cast<uint64_t>(ml) * ml) >> 44);
    return sq_term{p, 2 * static_cast<int32_t>(ex) - 2106};
}

// |v| = p 2^q (2^61 <= p < 2^62 for normal v, exact), for sums of
// non-negative values; zero gives p = 0, infinity and NaN set the flags.
PGX_ISUM_HD sq_term magnitude(double v, uint32_t &flags)
{
    const uint64_t b = bits_of(v);
    const uint32_t ex = static_cast<uint32_t>(b >> 52) & 0x7ffu;
    if (ex == 0x7ffu) {
        flags |= (b << 12) != 0u ? 2u : 1u;
        return sq_term{0u, kEmptyExp};
    }
    const uint64_t f = b & ((1ull << 52) - 1u);
    if (ex == 0u) return sq_term{f << 9, -1083}; // subnormal (or zero): f 2^-1074
    return sq_term{(f | (1ull << 52)) << 9, static_cast<int32_t>(ex) - 1084};
}

// a + b + c (each p < 2^62) aligned to the largest exponent, each truncated by
// less than one unit: the result's p may reach 3 2^62 (below 2^64)
PGX_ISUM_HD sq_term sum3(sq_term a, sq_term b, sq_term c)
{
    const int32_t qm = imax(imax(a.q, b.q), c.q);
    const uint64_t s = (a.p >> imin(qm - a.q, 63)) + (b.p >> imin(qm - b.q, 63)) + (c.p >> imin(qm - c.q, 63));
    return sq_term{s, qm};
}

// a + b + c + d aligned to the largest exponent (each truncated by less than
// one unit), then brought below 2^62 (two more bits at most)
PGX_ISUM_HD sq_term sum4(sq_term a, sq_term b, sq_term c, sq_term d)
{
    const int32_t qm = imax(imax(a.q, b.q), imax(c.q, d.q));
    uint64_t s = (a.p >> imin(qm - a.q, 63)) + (b.p >> imin(qm - b.q, 63));
    s += (c.p >> imin(qm - c.q, 63)) + (d.p >> imin(qm - d.q, 63));
    if (s >> 62) return sq_term{s >> 2, qm + 2};
    return sq_term{s, qm};
}

// acc += p 2^q (p < 2^62)
PGX_ISUM_HD void add(sq_acc &a, sq_term t)
{
    const int32_t big = imax(a.e, t.q);
    a.m = (a.m >> imin(big - a.e, 63)) + (t.p >> imin(big - t.q, 63));
    a.e = big;
    if (a.m >> 62) {
        a.m >>= 1;
        a.e += 1;
    }
}

// acc += v^2
PGX_ISUM_HD void add_square(sq_acc &a, double v)
{
    add(a, square(v, a.flags));
}

PGX_ISUM_HD int clz64(uint64_t v)
{
#if defined(__CUDA_ARCH__)
    return __clzll(static_cast<long long>(v));
#else
    return __builtin_clzll(v);
#endif
}

// The sum rounded to a double (overflowing to +inf), its bits assembled with
// integer operations; a subnormal result takes ldexp.
PGX_ISUM_HD double value(const sq_acc &a)
{
    if (a.flags & 2u) return std::numeric_limits<double>::quiet_NaN();
    if (a.flags & 1u) return std::numeric_limits<double>::infinity();
    if (a.m == 0u) return 0.0;
    const int lz = clz64(a.m);
    const uint64_t n = a.m << lz;                   // [2^63, 2^64): value n 2^(e - lz)
    const int32_t be = a.e - lz + 63 + 1023;        // biased exponent of the leading bit
    if (be < 1) return std::ldexp(static_cast<double>(a.m), a.e);
    if (be > 2046) return std::numeric_limits<double>::infinity();
    const uint64_t nr = n + 1024u;                  // to nearest, ties away
    const uint64_t mant = nr < n ? (1ull << 53) : (nr >> 11);
    // the implicit bit adds one to the exponent field, a carry to 2^53 two
    // (be = 2046 with a carry gives the bits of +inf)
    const uint64_t b = (static_cast<uint64_t>(be - 1) << 52) + mant;
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(static_cast<long long>(b));
#else
    double d;
    std::memcpy(&d, &b, 8);
    return d;
#endif
}

// ---------------------------------------------------------------- signed sums
//
// Sums of doubles of any sign (ZDT's sum of x, DTLZ's sums of cosines): the
// same floating accumulator with a signed significand. Each value enters
// exactly (its 53-bit significand shifted up 9 bits) and is aligned to the
// larger exponent, truncated toward minus infinity by at most one unit of
// 2^e (below 2^-60 of the largest magnitude added); cancellation needs no
// renormalisation (the result's error stays within 2^-60 per addition of the
// largest magnitude, the sum of |terms| of a first-order error bound).
// Infinities and NaN follow FP64: +inf + -inf and NaN give NaN.
struct sg_acc {
    int64_t m;      // |m| < 2^62
    int32_t e;
    uint32_t flags; // 1: +inf added, 2: -inf added, 4: NaN added
};

PGX_ISUM_HD sg_acc make_signed()
{
    return sg_acc{0, kEmptyExp, 0u};
}

// acc += s p 2^q (p < 2^62, s the sign)
PGX_ISUM_HD void add_signed(sg_acc &a, int64_t sp, int32_t q)
{
    const int32_t big = imax(a.e, q);
    a.m = (a.m >> imin(big - a.e, 63)) + (sp >> imin(big - q, 63));
    a.e = big;
    const int64_t mag = a.m < 0 ? -a.m : a.m;
    if (mag >> 62) {
        a.m >>= 1;
        a.e += 1;
    }
}

// acc += v
PGX_ISUM_HD void add_value(sg_acc &a, double v)
{
    const uint64_t b = bits_of(v);
    const uint32_t ex = static_cast<uint32_t>(b >> 52) & 0x7ffu;
    if (ex == 0x7ffu) {
        a.flags |= (b << 12) != 0u ? 4u : ((b >> 63) ? 2u : 1u);
        return;
    }
    const uint64_t f = b & ((1ull << 52) - 1u);
    const uint64_t p = (ex ? (f | (1ull << 52)) : f) << 9;
    const int32_t q = (ex ? static_cast<int32_t>(ex) : 1) - 1084;
    add_signed(a, (b >> 63) ? -static_cast<int64_t>(p) : static_cast<int64_t>(p), q);
}

// The sum rounded to a double (to nearest, ties away; overflowing to +-inf).
PGX_ISUM_HD double value(const sg_acc &a)
{
    if ((a.flags & 4u) || (a.flags & 3u) == 3u) return std::numeric_limits<double>::quiet_NaN();
    if (a.flags & 1u) return std::numeric_limits<double>::infinity();
    if (a.flags & 2u) return -std::numeric_limits<double>::infinity();
    if (a.m == 0) return 0.0;
    const bool neg = a.m < 0;
    const sq_acc mag{static_cast<uint64_t>(neg ? -a.m : a.m), a.e, 0u};
    const double v = value(mag);
    return neg ? -v : v;
}

} // namespace isum
} // namespace pgx
