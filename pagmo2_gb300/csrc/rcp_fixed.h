// Double-precision reciprocal and its cube with integer arithmetic (no FP64
// instruction).
//
// On GB300 the FP64 pipe retires two lanes per SM per clock while the integer
// pipes are mostly idle in the Lennard-Jones pair loop, so 1/r^2 and r^-6 are
// computed there with integer multiplies: Newton-Raphson division (a seed y0
// of 1/m, then y = y0 (1 + e + e^2) with the exact residual e = 1 - m y0, the
// truncated series of 1 / (1 - e)), carried out in 64/96-bit fixed point.
//
// For d = m 2^k (1 <= m < 2, 52-bit fraction f), with a seed y0 = Y0 / 2^32
// of 1/m whose residual satisfies |e| <= 2^-21:
//  - m y0 = u Y0 / 2^95 with u = m 2^63, so e = (2^95 - u Y0) / 2^95 is
//    formed exactly from a 64 x 32-bit product and kept in Q83 (|e| 2^83 <=
//    2^62);
//  - e^2 comes from the top 33 bits of e (absolute error below 2^-72);
//  - y 2^64 = Y0 2^32 + Y0 (e + e^2) 2^32, the second term from the high
//    half of a 64 x 64-bit product;
//  - the dropped e^3 is below 2^-63 and the truncations below 2^-64, so the
//    fixed-point y (Q64, in [1/2, 1)) is within 2^-62 of 1/m relative;
//    rounding it to 53 bits gives a result within 0.51 units of the last
//    place of 1/d (faithful: the correctly rounded value except within 2^-10
//    units of the last place of a midpoint);
//  - y^3 from two more 64 x 64-bit high products (each truncation below 2^-61
//    relative) is within 2^-59 of 1/m^3, so r^-6 = y^3 2^-3k rounds to within
//    0.52 units of the last place (two FP64 multiplies of the rounded 1/d give
//    up to about 2 units).
// The header compiles as plain C++ too, so that the fixed-point part can be
// checked on the host with any seed of the stated accuracy.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define PGX_RCP_HD __host__ __device__ __forceinline__
#else
#define PGX_RCP_HD inline
#endif

namespace pgx
{
namespace rcpfx
{

// floor(a b / 2^64) for signed 64-bit a, b
PGX_RCP_HD int64_t mul_hi_s64(int64_t a, int64_t b)
{
#if defined(__CUDA_ARCH__)
    return __mul64hi(a, b);
#else
    return static_cast<int64_t>((static_cast<__int128>(a) * b) >> 64);
#endif
}

// floor(a b / 2^64) for unsigned 64-bit a, b
PGX_RCP_HD uint64_t mul_hi_u64(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return static_cast<uint64_t>((static_cast<unsigned __int128>(a) * b) >> 64);
#endif
}

// leading zero bits of a nonzero 64-bit value
PGX_RCP_HD int clz_u64(uint64_t v)
{
#if defined(__CUDA_ARCH__)
    return __clzll(static_cast<long long>(v));
#else
    return __builtin_clzll(v);
#endif
}

// The seed's Q32 form from the bits of a float y0 that approximates 1/m,
// 1/2 < 1/m <= 1: y0 in [1/2, 1) is exact in Q32; 1 and values below 1/2
// (possible one unit of the last place away from the range) are clamped.
PGX_RCP_HD uint32_t seed_q32(uint32_t y0_bits)
{
    if (y0_bits >= 0x3f800000u) return 0xffffffffu;
    if (y0_bits < 0x3f000000u) return 0x80000000u;
    return ((y0_bits & 0x7fffffu) | 0x800000u) << 8;
}

// The float whose value is m = 1 + f52 2^-52 truncated to 23 fraction bits
// (the seed's input).
PGX_RCP_HD uint32_t seed_input_bits(uint64_t f52)
{
    return 0x3f800000u | static_cast<uint32_t>(f52 >> 29);
}

// 1/m in Q64 for m = u / 2^63, any 64-bit significand 2^63 <= u < 2^64:
// 2^63 <= z < 2^64 (1/2 <= 1/m < 1 up to the error above; m = 1 gives
// 2^64 - 1). y0q: the seed in Q32.
PGX_RCP_HD uint64_t rcp_q64_u(uint64_t u, uint32_t y0q)
{
    const uint64_t pl = static_cast<uint64_t>(static_cast<uint32_t>(u)) * y0q;
    const uint64_t ph = static_cast<uint64_t>(static_cast<uint32_t>(u >> 32)) * y0q + (pl >> 32);
    // D = 2^95 - u Y0 = T 2^32 - (pl mod 2^32); e = D / 2^95, ef = D / 2^12 = e 2^83
    const int64_t t = static_cast<int64_t>((1ull << 63) - ph);
    const int64_t ef = t * (int64_t{1} << 20) - static_cast<int64_t>(static_cast<uint32_t>(pl) >> 12);
    const int64_t eh = ef >> 31;                // e 2^52
    const int64_t c = ef + ((eh * eh) >> 21);   // (e + e^2) 2^83
    const int64_t corr = mul_hi_s64(static_cast<int64_t>(static_cast<uint64_t>(y0q) << 31), c) >> 18; // y0 c 2^64
    return (static_cast<uint64_t>(y0q) << 32) + static_cast<uint64_t>(corr);
}

// The float whose value is u / 2^63 truncated to 23 fraction bits.
PGX_RCP_HD uint32_t seed_input_bits_u(uint64_t u)
{
    return 0x3f800000u | (static_cast<uint32_t>(u >> 40) & 0x7fffffu);
}

// 1/m in Q64 for a double's significand m = 1 + f52 2^-52.
PGX_RCP_HD uint64_t rcp_q64(uint64_t f52, uint32_t y0q)
{
    return rcp_q64_u((1ull << 63) | (f52 << 11), y0q);
}

// z in [2^63, 2^64) rounded to a 53-bit mantissa (implicit bit included):
// a value in [2^52, 2^53], 2^53 when z rounds up to 2^64.
PGX_RCP_HD uint64_t round_q64(uint64_t z)
{
    const uint64_t zr = z + 1024u;
    return zr < z ? (1ull << 53) : (zr >> 11);
}

// 53-bit mantissa of 1/m rounded to nearest (see round_q64).
PGX_RCP_HD uint64_t rcp_mantissa(uint64_t f52, uint32_t y0q)
{
    return round_q64(rcp_q64(f52, y0q));
}

// Bits of 1/d for d = (1 + f52 2^-52) 2^(ex - 1023), ex the biased exponent,
// when the result is normal (923 <= ex <= 1123 in the callers).
PGX_RCP_HD uint64_t rcp_bits(uint32_t ex, uint64_t f52, uint32_t y0q)
{
    const uint64_t mant = rcp_mantissa(f52, y0q);
    // the implicit bit (2^52) adds one to the exponent field, a carry to 2^53 two
    return (static_cast<uint64_t>(2044u - ex) << 52) + mant;
}

// Bits of 1/d and of 1/d^3 (d as above, 923 <= ex <= 1123: both normal).
PGX_RCP_HD void rcp_and_cube_bits(uint32_t ex, uint64_t f52, uint32_t y0q, uint64_t *inv_bits, uint64_t *cube_bits)
{
    const uint64_t z = rcp_q64(f52, y0q);
    *inv_bits = (static_cast<uint64_t>(2044u - ex) << 52) + round_q64(z);
    const uint64_t z3 = mul_hi_u64(mul_hi_u64(z, z), z); // y^3 2^64, in [2^61, 2^64)
    const int lz = clz_u64(z3);                          // 0, 1 or 2
    // y^3 = (z3 << lz) 2^-64 2^-lz; 1/d^3 = y^3 2^(-3 (ex - 1023))
    *cube_bits = (static_cast<uint64_t>(4090u - 3u * ex - static_cast<uint32_t>(lz)) << 52) + round_q64(z3 << lz);
}

} // namespace rcpfx
} // namespace pgx
