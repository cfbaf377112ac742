// sin(2 pi x) and cos(2 pi x) with integer arithmetic (no FP64 instruction,
// or one conversion per result: to_double).
//
// Rastrigin, Ackley and the multi-objective test problems spend most of their
// FP64 instructions on sin/cos(2 pi x) polynomials; GB300's FP64 pipe retires
// two lanes per SM per clock while the integer pipes sit mostly idle. Here:
//  - reduction, exact: with |x| = m 2^e (m the 53-bit significand),
//    2|x| = k + f with k = rint(2|x|) and |f| <= 1/2 computed on m's bits, so
//    r = f / 2 = +-R 2^er exactly (|r| <= 1/4) and
//    sin(2 pi |x|) = (-1)^k sin(2 pi r), cos(2 pi |x|) = (-1)^k cos(2 pi r);
//  - z = r^2 in Q64 from the normalised R (a 64 x 64-bit high product);
//  - sin(2 pi r) = r S(z) and cos(2 pi r) = 1 + z H(z), S and H of degree 8
//    on z in [0, 1/16] (interpolation errors 1.3e-18 and 4.1e-19; coefficients
//    in Q55 from gen_trig_coeffs.py), evaluated by Horner's rule on signed
//    64-bit fixed point (each step truncates by at most 2^-55);
//  - sin keeps r's relative precision (S >= 4 multiplies the normalised R),
//    so it is within about 2^-56 of the exact value relative; cos is within
//    about 2^-55 absolute; both are rounded to doubles once.
// Valid for 2^-60 <= |x| < 2^40 and x = 0; callers route the rest elsewhere.
// The header compiles as plain C++ too, so that it can be checked on the host.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define PGX_TRIG_HD __host__ __device__ __forceinline__
#else
#define PGX_TRIG_HD inline
#endif

namespace pgx
{
namespace trigfx
{

// sin(2 pi r) / r and (cos(2 pi r) - 1) / r^2 as polynomials in z = r^2, Q55,
// lowest degree first (gen_trig_coeffs.py); scalars so that device code can
// use them as immediates
constexpr int64_t kS0 = 226375608064910089LL, kS1 = -1489491798437810757LL, kS2 = 2940138961849612574LL,
                  kS3 = -2763619851199646660LL, kS4 = 1515324146322002856LL, kS5 = -543841781022845872LL,
                  kS6 = 137627413933948365LL, kS7 = -25859085110711807LL, kS8 = 3635195912119868LL;
constexpr int64_t kH0 = -711179947248643885LL, kH1 = 2339688245777237824LL, kH2 = -3078906321026659378LL,
                  kH3 = 2170541955464940332LL, kH4 = -952106241398342809LL, kH5 = 284754897436682737LL,
                  kH6 = -61767157157176774LL, kH7 = 10155930143671935LL, kH8 = -1273060735599591LL;

PGX_TRIG_HD uint64_t bits_of(double v)
{
#if defined(__CUDA_ARCH__)
    return static_cast<uint64_t>(__double_as_longlong(v));
#else
    uint64_t b;
    std::memcpy(&b, &v, 8);
    return b;
#endif
}

PGX_TRIG_HD double from_bits(uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(static_cast<long long>(b));
#else
    double d;
    std::memcpy(&d, &b, 8);
    return d;
#endif
}

PGX_TRIG_HD int64_t mul_hi_s64(int64_t a, int64_t b)
{
#if defined(__CUDA_ARCH__)
    return __mul64hi(a, b);
#else
    return static_cast<int64_t>((static_cast<__int128>(a) * b) >> 64);
#endif
}

PGX_TRIG_HD uint64_t mul_hi_u64(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return static_cast<uint64_t>((static_cast<unsigned __int128>(a) * b) >> 64);
#endif
}

PGX_TRIG_HD int clz64(uint64_t v)
{
#if defined(__CUDA_ARCH__)
    return __clzll(static_cast<long long>(v));
#else
    return __builtin_clzll(v);
#endif
}

// True when x is handled here: 2^-60 <= |x| < 2^40, or x = +-0.
PGX_TRIG_HD bool in_range(double x)
{
    const uint32_t ex = static_cast<uint32_t>(bits_of(x) >> 52) & 0x7ffu;
    return (ex - (1023u - 60u) < 100u) || (bits_of(x) << 1) == 0u;
}

// The double nearest to p 2^e (p > 0, result normal), with the sign bit s,
// in two forms with one rounding each: CVT = false rounds the significand
// with integer operations (about twenty; ties away from zero), CVT = true
// converts p with one instruction (ties to even) and scales it through the
// exponent field. The conversion made the rastrigin rows, where the integer
// pipe binds, 7 % faster and the ackley and ZDT4 rows, whose FP64 pipe is
// busier, 5-9 % slower.
template <bool CVT = false>
PGX_TRIG_HD double to_double(uint64_t p, int32_t e, uint64_t s)
{
    if constexpr (CVT) {
#if defined(__CUDA_ARCH__)
        const double v = __ull2double_rn(p);
#else
        const double v = static_cast<double>(p);
#endif
        return from_bits((bits_of(v) + (static_cast<uint64_t>(static_cast<int64_t>(e)) << 52)) | (s << 63));
    } else {
        const int lz = clz64(p);
        const uint64_t n = p << lz;
        const uint64_t nr = n + 1024u;
        const uint64_t mant = nr < n ? (1ull << 53) : (nr >> 11);
        // value n 2^(e - lz): leading bit at 2^(e - lz + 63); the implicit bit adds one to the exponent field
        return from_bits((s << 63) | ((static_cast<uint64_t>(e - lz + 63 + 1022) << 52) + mant));
    }
}

struct reduced {
    uint64_t rn;  // |r| normalised: rn 2^re, 2^63 <= rn < 2^64, or 0 when r = 0
    int32_t re;
    uint32_t neg; // 1: r < 0 (for |x|)
    uint32_t odd; // k mod 2
};

// 2|x| = k + 2r, |r| <= 1/4 (x in range)
PGX_TRIG_HD reduced reduce(double x)
{
    const uint64_t b = bits_of(x);
    const uint32_t ex = static_cast<uint32_t>(b >> 52) & 0x7ffu;
    const uint64_t m = (b & ((1ull << 52) - 1u)) | (1ull << 52);
    reduced red{0u, 0, 0u, 0u};
    if ((b << 1) == 0u) return red;
    const int32_t s = 1074 - static_cast<int32_t>(ex); // 2|x| = m 2^-s
    int64_t fi;                                        // 2r = fi 2^-s
    if (s <= 0) {
        red.odd = s == 0 ? static_cast<uint32_t>(m & 1u) : 0u;
        return red; // 2|x| is an integer
    }
    if (s > 53) {
        fi = static_cast<int64_t>(m); // 2|x| < 1/2: k = 0
    } else {
        const uint64_t k = (m + (1ull << (s - 1))) >> s;
        red.odd = static_cast<uint32_t>(k & 1u);
        fi = static_cast<int64_t>(m) - static_cast<int64_t>(k << s);
    }
    if (fi == 0) return red;
    red.neg = fi < 0 ? 1u : 0u;
    const uint64_t a = static_cast<uint64_t>(fi < 0 ? -fi : fi);
    const int lz = clz64(a);
    red.rn = a << lz;
    red.re = -s - 1 - lz; // r = fi 2^(-s-1) = rn 2^(-s-1-lz)
    return red;
}

// z = r^2 in Q64 (z <= 1/16: below 2^60)
PGX_TRIG_HD int64_t z_q64(const reduced &r)
{
    if (r.rn == 0u) return 0;
    const uint64_t sq = mul_hi_u64(r.rn, r.rn); // r^2 = sq 2^(2 re + 64)
    const int32_t sh = -(2 * r.re + 128);       // z 2^64 = sq 2^-sh, sh >= 4
    return sh >= 64 ? 0 : static_cast<int64_t>(sq >> sh);
}

PGX_TRIG_HD int64_t poly_s(int64_t z)
{
    int64_t a = kS8;
    a = mul_hi_s64(a, z) + kS7;
    a = mul_hi_s64(a, z) + kS6;
    a = mul_hi_s64(a, z) + kS5;
    a = mul_hi_s64(a, z) + kS4;
    a = mul_hi_s64(a, z) + kS3;
    a = mul_hi_s64(a, z) + kS2;
    a = mul_hi_s64(a, z) + kS1;
    return mul_hi_s64(a, z) + kS0;
}

PGX_TRIG_HD int64_t poly_h(int64_t z)
{
    int64_t a = kH8;
    a = mul_hi_s64(a, z) + kH7;
    a = mul_hi_s64(a, z) + kH6;
    a = mul_hi_s64(a, z) + kH5;
    a = mul_hi_s64(a, z) + kH4;
    a = mul_hi_s64(a, z) + kH3;
    a = mul_hi_s64(a, z) + kH2;
    a = mul_hi_s64(a, z) + kH1;
    return mul_hi_s64(a, z) + kH0;
}

// cos(2 pi x), x in range
template <bool CVT = false>
PGX_TRIG_HD double cos_2pi(double x)
{
    const reduced r = reduce(x);
    const int64_t z = z_q64(r);
    const int64_t c = (int64_t{1} << 55) + mul_hi_s64(poly_h(z), z); // cos(2 pi r) in Q55, >= 0
    if (c <= 0) return 0.0;
    return to_double<CVT>(static_cast<uint64_t>(c), -55, r.odd);
}

// sin(2 pi x) and cos(2 pi x), x in range
template <bool CVT = false>
PGX_TRIG_HD void sincos_2pi(double x, double &s, double &c)
{
    const reduced r = reduce(x);
    const int64_t z = z_q64(r);
    const int64_t cq = (int64_t{1} << 55) + mul_hi_s64(poly_h(z), z);
    c = cq <= 0 ? 0.0 : to_double<CVT>(static_cast<uint64_t>(cq), -55, r.odd);
    const uint64_t sx = bits_of(x) >> 63;
    if (r.rn == 0u) {
        s = from_bits((sx ^ r.odd) << 63); // a zero of the sine, signed as r (+0 for x = +-0: x)
        if ((bits_of(x) << 1) == 0u) s = x;
        return;
    }
    // |sin(2 pi r)| = rn 2^re S(z), S(z) >= 4 in Q55
    const uint64_t p = mul_hi_u64(r.rn, static_cast<uint64_t>(poly_s(z)));
    s = to_double<CVT>(p, r.re + 64 - 55, sx ^ r.odd ^ r.neg);
}

} // namespace trigfx
} // namespace pgx
