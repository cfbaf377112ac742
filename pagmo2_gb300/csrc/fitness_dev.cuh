// Device routines of the batch fitness/gradient path, shared by the
// per-problem kernels (fitness.cu) and the fused archipelago kernel
// (epoch.cu). Every routine evaluates whole rows with a fixed group of lanes,
// in FP64 arithmetic or in integer arithmetic that is exact or closer to the
// exact result than the FP64 operations it replaces (isum.h, rcp_fixed.h,
// trig_fixed.h), except the opt-in rosenbrock_row_v4_ff, which works in
// double-float arithmetic on the FP32 pipe.
//
// GB300's FP64 pipe retires two lanes per SM per clock, so these routines are
// written for the fewest FP64 instructions per element; integer and shuffle
// work is cheap by comparison.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "isum.h"
#include "rcp_fixed.h"
#include "trig_fixed.h"

namespace pgx
{
namespace dev
{

constexpr unsigned kFull = 0xffffffffu;

// 2*pi and 10*(2*pi) as the reference rounds them (src/problems/rastrigin.cpp:65, :104).
constexpr double kOmega = 2. * 3.1415926535897932384626433832795028841971693993;
constexpr double k10Omega = 10.0 * kOmega;

// Lanes of the calling thread's group of G consecutive lanes (G | 32).
template <int G>
__device__ __forceinline__ unsigned group_mask()
{
    if constexpr (G == 32) {
        return kFull;
    } else {
        const unsigned lane = threadIdx.x & 31u;
        return ((1u << G) - 1u) << (lane & ~static_cast<unsigned>(G - 1));
    }
}

template <int G>
__device__ __forceinline__ double group_sum(double v, unsigned mask)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, G);
    return v;
}

// Total of the integer sum-of-squares accumulators of a group of G lanes
// (xor butterfly on integer shuffles: every lane gets the same total, no FP64
// instruction).
template <int G>
__device__ __forceinline__ isum::sq_acc group_isum(isum::sq_acc a, unsigned mask)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        const unsigned long long m = __shfl_xor_sync(mask, static_cast<unsigned long long>(a.m), o, G);
        const int e = __shfl_xor_sync(mask, a.e, o, G);
        a.flags |= __shfl_xor_sync(mask, a.flags, o, G);
        isum::add(a, isum::sq_term{m, e});
    }
    return a;
}

// The same for the signed accumulators (isum::sg_acc).
template <int G>
__device__ __forceinline__ isum::sg_acc group_ssum(isum::sg_acc a, unsigned mask)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        const long long m = __shfl_xor_sync(mask, static_cast<long long>(a.m), o, G);
        const int e = __shfl_xor_sync(mask, a.e, o, G);
        a.flags |= __shfl_xor_sync(mask, a.flags, o, G);
        isum::add_signed(a, m, e);
    }
    return a;
}

// +1.0 or -1.0, and a constant with its sign flipped, built with integer
// operations so that signs cost no FP64 instruction: callers fold them into
// the FMA that consumes the value.
__device__ __forceinline__ double unit_sign(int neg)
{
    return __longlong_as_double(0x3ff0000000000000LL | (static_cast<long long>(neg & 1) << 63));
}

__device__ __forceinline__ double signed_const(double v, int neg)
{
    return __longlong_as_double(__double_as_longlong(v) ^ (static_cast<long long>(neg & 1) << 63));
}

// ------------------------------------------------------------ sin/cos(2 pi x)
//
// Method: exact argument reduction in units of the period, then polynomials.
// With k = rint(4x) (one FMA against the 1.5*2^52 rounding constant, valid for
// |x| < 2^49) and r = x - k/4 (exact: Sterbenz), 2 pi x = k pi/2 + 2 pi r with
// |2 pi r| <= pi/4. sin(2 pi r) = r S(r^2) and cos(2 pi r) = 1 + r^2 C(r^2),
// S and C near-minimax (Chebyshev interpolation) fits on r^2 in [0, 1/64],
// |error| about 2e-16 including rounding; cos is exactly 1 at r = 0, so
// integer x give cos = 1, sin = +-0 exactly. The quadrant k mod 4 swaps the
// pair and decides the signs, returned as flags (s_neg, c_neg) for the
// caller's FMA. Callers route |x| >= 2^40, infinities and NaN to CUDA's
// sincospi/cospi.
constexpr double kRound52 = 0x1.8p52;

__device__ __forceinline__ bool fast_trig_arg(double x)
{
    const unsigned e = (static_cast<unsigned>(__double2hiint(x)) >> 20) & 0x7ffu;
    return e < 1023u + 40u;
}

__device__ __forceinline__ void sincos_2pi(double x, double &s, int &s_neg, double &c, int &c_neg)
{
    const double t = fma(x, 4.0, kRound52);
    const int k = __double2loint(t);
    const double r = fma(t - kRound52, -0.25, x);
    const double z = r * r;
    double ps = 0x1.e3f38399551bfp+1;
    ps = fma(ps, z, -0x1.e30071afc3e59p+3);
    ps = fma(ps, z, 0x1.50782fda12d96p+5);
    ps = fma(ps, z, -0x1.32d2cce2e5b19p+6);
    ps = fma(ps, z, 0x1.466bc677587f8p+6);
    ps = fma(ps, z, -0x1.4abbce625be41p+5);
    ps = fma(ps, z, 0x1.921fb54442d18p+2);
    const double sr = r * ps;
    double pc = 0x1.f4b536b457d9ep+2;
    pc = fma(pc, z, -0x1.a6cc32d07dc98p+4);
    pc = fma(pc, z, 0x1.e1f50093e4c8fp+5);
    pc = fma(pc, z, -0x1.55d3c7e10153fp+6);
    pc = fma(pc, z, 0x1.03c1f081b4b74p+6);
    pc = fma(pc, z, -0x1.3bd3cc9be45dbp+4);
    const double cr = fma(pc, z, 1.0);
    const int q = k & 3;
    const bool swap = (q & 1) != 0;
    c = swap ? sr : cr;
    s = swap ? cr : sr;
    c_neg = ((q + 1) >> 1) & 1; // negative in quadrants 1, 2
    s_neg = (q >> 1) & 1;       // negative in quadrants 2, 3
}

// cos(2 pi x) alone: half-period reduction k = rint(2x), r = x - k/2,
// cos(2 pi x) = (-1)^k (1 + r^2 H(r^2)), H fitted on r^2 in [0, 1/16].
// Returns the magnitude; *neg = k mod 2.
__device__ __forceinline__ double cos_2pi(double x, int &neg)
{
    const double t = fma(x, 2.0, kRound52);
    const int k = __double2loint(t);
    const double r = fma(t - kRound52, -0.5, x);
    const double z = r * r;
    double p = 0x1.179a329ef4140p-2;
    p = fma(p, z, -0x1.b6a6feabe52e9p+0);
    p = fma(p, z, 0x1.f9d2c1f3b2167p+2);
    p = fma(p, z, -0x1.a6d1f12b0bef2p+4);
    p = fma(p, z, 0x1.e1f5068620bcbp+5);
    p = fma(p, z, -0x1.55d3c7e3c9051p+6);
    p = fma(p, z, 0x1.03c1f081b5a9fp+6);
    p = fma(p, z, -0x1.3bd3cc9be45dep+4);
    neg = k & 1;
    return fma(p, z, 1.0);
}

// ------------------------------------------------------------------ rastrigin
//
// f = sum_i (x_i^2 - 10 cos(2 pi x_i)) + 10 n  (src/problems/rastrigin.cpp:62-72),
// accumulated as sum x^2 and sum cos apart; g_i = 2 x_i + 10 omega sin(2 pi x_i)
// (:98-107). One group of G lanes per row, lanes strided over coordinates.
// For 2^-60 <= |x| < 2^40 (the usual case) sin and cos come from the integer
// fixed-point routines of trig_fixed.h and 2x is an exponent increment. The
// integer pipe binds these rows, so the FP64 pipe takes the sums: per element
// the x^2 FMA, the cos add, the gradient's FMA and the two conversions of the
// fixed-point results (21 FP64 instructions with FP64 polynomials). Other x
// take the FP64 polynomials (|x| < 2^-60) or CUDA's sincospi/cospi.

// 2x exactly for zero or a normal x whose double 2x is finite
__device__ __forceinline__ double twice_exact(double x)
{
    const long long b = __double_as_longlong(x);
    return (b << 1) == 0 ? x : __longlong_as_double(b + (1LL << 52));
}

// One element's contribution: x^2 into sx, cos(2 pi x) into sc and, with the
// gradient, g = 2x + 10 omega sin(2 pi x) stored.
template <bool GRAD>
__device__ __forceinline__ void rastrigin_element(double xi, double &sx, double &sc, double *gi)
{
    sx = fma(xi, xi, sx);
    if (trigfx::in_range(xi)) {
        if (GRAD) {
            double s, c;
            trigfx::sincos_2pi<true>(xi, s, c);
            sc += c;
            *gi = fma(k10Omega, s, twice_exact(xi));
        } else {
            sc += trigfx::cos_2pi<true>(xi);
        }
        return;
    }
    double s = 0.0, c;
    int s_neg = 0, c_neg = 0;
    if (fast_trig_arg(xi)) {
        if (GRAD)
            sincos_2pi(xi, s, s_neg, c, c_neg);
        else
            c = cos_2pi(xi, c_neg);
    } else {
        if (GRAD)
            sincospi(xi + xi, &s, &c);
        else
            c = cospi(xi + xi);
    }
    sc = fma(c, unit_sign(c_neg), sc);
    if (GRAD) *gi = fma(signed_const(k10Omega, s_neg), s, xi + xi);
}

// A row's two sums in one fixed order, whatever the number of lanes G that
// evaluates it: element i belongs to virtual lane v = i mod V, each virtual
// lane sums its elements in index order, and the V partial sums are combined
// by the butterfly of a V-lane xor reduction (offsets V/2, ..., 1; each step
// adds the partner's sum to one's own). V depends on the dimension only
// (rastrigin_width). Lane `sub` of a group of G | V lanes holds the J = V/G
// virtual lanes sub + G j: the butterfly's steps with offsets >= G join them
// inside the thread (offset G h joins j and j + h), the others cross the group
// by shuffles. Empty virtual lanes (v >= nx) hold +0, which every step adds
// exactly. The result is therefore bit-identical for every G, and the number
// of lanes follows the batch size (more per row for small batches) without
// changing any value.
struct rastrigin_part {
    double sx; // sum of x^2
    double sc; // sum of cos(2 pi x)
};

__device__ __forceinline__ void rastrigin_join(rastrigin_part &a, const rastrigin_part &b)
{
    a.sx = a.sx + b.sx;
    a.sc = a.sc + b.sc;
}

template <int V, int G, bool GRAD>
__device__ __forceinline__ void rastrigin_row(const double *__restrict__ xr, uint32_t nx, double *f_out,
                                              double *__restrict__ gr)
{
    static_assert(G >= 4 && G <= V && V <= 32 && (G & (G - 1)) == 0 && (V & (V - 1)) == 0,
                  "rastrigin rows: 4 <= G <= V <= 32, powers of two");
    constexpr int J = V / G;
    const unsigned sub = threadIdx.x & (G - 1);
    const unsigned mask = group_mask<G>();
    rastrigin_part acc[J];
#pragma unroll
    for (int j = 0; j < J; ++j) acc[j] = rastrigin_part{0.0, 0.0};
    // chunks of V elements; the next element's load is issued before this
    // one's arithmetic
    double xn = sub < nx ? __ldg(xr + sub) : 0.0;
    for (uint32_t base = 0; base < nx; base += V) {
#pragma unroll
        for (int j = 0; j < J; ++j) {
            const uint32_t i = base + sub + static_cast<uint32_t>(G * j);
            const double xi = xn;
            const uint32_t inext = j + 1 < J ? i + G : base + V + sub;
            if (inext < nx) xn = __ldg(xr + inext);
            if (i < nx) rastrigin_element<GRAD>(xi, acc[j].sx, acc[j].sc, GRAD ? gr + i : nullptr);
        }
    }
#pragma unroll
    for (int h = J / 2; h >= 1; h >>= 1) {
#pragma unroll
        for (int j = 0; j < h; ++j) rastrigin_join(acc[j], acc[j + h]);
    }
    const double sxv = group_sum<G>(acc[0].sx, mask);
    const double scv = group_sum<G>(acc[0].sc, mask);
    if (sub == 0 && f_out) *f_out = fma(-10.0, scv, sxv) + 10.0 * static_cast<double>(nx);
}

// The canonical width V of a rastrigin row, from its dimension alone: the
// lanes the dimension would take by itself (lanes_for_dim) when that is 16 or
// 32, else 8.
__host__ __device__ inline int rastrigin_width(int lanes_for_dim)
{
    return lanes_for_dim >= 16 ? (lanes_for_dim >= 32 ? 32 : 16) : 8;
}

// Lanes per rastrigin row for a batch of n rows: all V for batches of at most
// one 256-thread block's worth of lanes per SM (latency-bound: shorter chains
// per lane), else the dimension's own choice (at least 4). Results do not
// depend on it.
__host__ __device__ inline int rastrigin_lanes(int lanes_for_dim, uint64_t n, int num_sms)
{
    const int v = rastrigin_width(lanes_for_dim);
    const uint64_t cap = static_cast<uint64_t>(num_sms > 0 ? num_sms : 1) * 256u;
    if (n * static_cast<uint64_t>(v) <= cap) return v;
    return lanes_for_dim < 4 ? 4 : (lanes_for_dim > v ? v : lanes_for_dim);
}

// ----------------------------------------------------------------- rosenbrock
//
// With t_i = x_{i+1} - x_i^2 and c_i = 2 x_i - 2 (src/problems/rosenbrock.cpp:59-66, 83-92):
//   f   = 100 sum t_i^2 + sum (x_i - 1)^2        (i < n-1)
//   g_i = 200 (t_{i-1} - 2 x_i t_i) + c_i        (i < n-1, t_{-1} = 0)
//   g_{n-1} = 200 t_{n-2}
// Fitness + gradient: 5 FP64 instructions per element (t, 2x, 2x-2,
// t_{i-1} - 2x t, 200 b + c), 4 in the vector variant where 2x is an integer
// exponent increment; fitness only: 2 (t, x-1). The sums of t^2 and
// (2x-2)^2 or (x-1)^2 are exact integer accumulations (isum.h).

// Scalar variant: one group of G lanes per row, element i in lane i mod G;
// x_{i+1} from the next lane (the last lane takes the next chunk's head),
// t_{i-1} from the previous lane.
template <int G, bool GRAD>
__device__ __forceinline__ void rosenbrock_row(const double *__restrict__ xr, uint32_t nx, double *f_out,
                                               double *__restrict__ gr)
{
    const unsigned sub = threadIdx.x & (G - 1);
    const unsigned mask = group_mask<G>();
    isum::sq_acc acc_t = isum::make(), acc_u = isum::make();
    double t_carry = 0.0;
    double x_cur = sub < nx ? __ldg(xr + sub) : 0.0;
    for (uint32_t base = 0; base < nx; base += G) {
        const uint32_t i = base + sub;
        const double x_nxt = (i + G < nx) ? __ldg(xr + i + G) : 0.0;
        double xn = __shfl_down_sync(mask, x_cur, 1, G);
        const double head = __shfl_sync(mask, x_nxt, 0, G);
        if (sub == G - 1) xn = head;
        const bool has_next = i + 1u < nx;
        const double t = has_next ? fma(-x_cur, x_cur, xn) : 0.0;
        if (GRAD) {
            double t_prev = __shfl_up_sync(mask, t, 1, G);
            if (sub == 0) t_prev = t_carry;
            t_carry = __shfl_sync(mask, t, G - 1, G);
            if (i < nx) {
                const double w = x_cur + x_cur;
                const double c = w - 2.0;
                double gi;
                if (has_next) {
                    isum::add_square(acc_t, t);
                    isum::add_square(acc_u, c);
                    gi = fma(200.0, fma(-w, t, t_prev), c);
                } else {
                    gi = 200.0 * t_prev;
                }
                gr[i] = gi;
            }
        } else if (has_next) {
            isum::add_square(acc_t, t);
            isum::add_square(acc_u, x_cur - 1.0);
        }
        x_cur = x_nxt;
    }
    const double st = isum::value(group_isum<G>(acc_t, mask));
    const double su = isum::value(group_isum<G>(acc_u, mask));
    // with the gradient the second sum is over c^2 = 4 (x-1)^2
    if (sub == 0 && f_out) *f_out = GRAD ? fma(100.0, st, 0.25 * su) : fma(100.0, st, su);
}

// 2x by incrementing the exponent field: exact for normal x whose double is
// finite (biased exponent 1..0x7fd); an integer add instead of an FP64 one.
__device__ __forceinline__ bool doubling_ok(double x)
{
    const unsigned e = (static_cast<unsigned>(__double2hiint(x)) >> 20) & 0x7ffu;
    return e - 1u < 0x7fdu;
}

__device__ __forceinline__ double twice_normal(double x)
{
    return __hiloint2double(__double2hiint(x) + 0x00100000, __double2loint(x));
}

// Vector variant: one warp per row, each lane owning 4 consecutive elements
// (two 16-byte loads), so a warp step covers 128 elements with a quarter of
// the loads and shuffles of the scalar variant. Needs nx % 4 == 0 and a
// 16-byte aligned row start.
template <bool GRAD>
__device__ __forceinline__ void rosenbrock_row_v4(const double *__restrict__ xr, uint32_t nx, double *f_out,
                                                  double *__restrict__ gr)
{
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t slots = nx >> 2;
    const double2 *x2 = reinterpret_cast<const double2 *>(xr);
    isum::sq_acc acc_t = isum::make(), acc_u = isum::make();
    double t_carry = 0.0;
    double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
    if (lane < slots) {
        a = __ldg(x2 + 2u * lane);
        b = __ldg(x2 + 2u * lane + 1u);
    }
    for (uint32_t base = 0; base < slots; base += 32u) {
        const uint32_t s = base + lane;
        const bool act = s < slots;
        const uint32_t sn = s + 32u;
        double2 na = make_double2(0.0, 0.0), nb = make_double2(0.0, 0.0);
        if (sn < slots) {
            na = __ldg(x2 + 2u * sn);
            nb = __ldg(x2 + 2u * sn + 1u);
        }
        const double x0 = a.x, x1 = a.y, x2v = b.x, x3 = b.y;
        double xn = __shfl_down_sync(kFull, x0, 1);
        const double head = __shfl_sync(kFull, na.x, 0);
        if (lane == 31u) xn = head;
        const bool last_has_next = s + 1u < slots;
        const double t0 = fma(-x0, x0, x1);
        const double t1 = fma(-x1, x1, x2v);
        const double t2 = fma(-x2v, x2v, x3);
        const double t3 = last_has_next ? fma(-x3, x3, xn) : 0.0;
        if (GRAD) {
            double tp = __shfl_up_sync(kFull, t3, 1);
            if (lane == 0) tp = t_carry;
            t_carry = __shfl_sync(kFull, t3, 31);
            // 2x exactly by an exponent increment when every element of the
            // warp is a normal number whose double is finite, else by an add
            const bool ok = !act || (doubling_ok(x0) && doubling_ok(x1) && doubling_ok(x2v) && doubling_ok(x3));
            double w0, w1, w2, w3;
            if (__all_sync(kFull, ok)) {
                w0 = twice_normal(x0);
                w1 = twice_normal(x1);
                w2 = twice_normal(x2v);
                w3 = twice_normal(x3);
            } else {
                w0 = x0 + x0;
                w1 = x1 + x1;
                w2 = x2v + x2v;
                w3 = x3 + x3;
            }
            if (act) {
                const double c0 = w0 - 2.0, c1 = w1 - 2.0, c2 = w2 - 2.0, c3 = w3 - 2.0;
                isum::add_square(acc_t, t0);
                isum::add_square(acc_t, t1);
                isum::add_square(acc_t, t2);
                isum::add_square(acc_u, c0);
                isum::add_square(acc_u, c1);
                isum::add_square(acc_u, c2);
                double2 g01, g23;
                g01.x = fma(200.0, fma(-w0, t0, tp), c0);
                g01.y = fma(200.0, fma(-w1, t1, t0), c1);
                g23.x = fma(200.0, fma(-w2, t2, t1), c2);
                if (last_has_next) {
                    isum::add_square(acc_t, t3);
                    isum::add_square(acc_u, c3);
                    g23.y = fma(200.0, fma(-w3, t3, t2), c3);
                } else {
                    g23.y = 200.0 * t2;
                }
                double2 *g2 = reinterpret_cast<double2 *>(gr);
                g2[2u * s] = g01;
                g2[2u * s + 1u] = g23;
            }
        } else if (act) {
            isum::add(acc_t, isum::sum4(isum::square(t0, acc_t.flags), isum::square(t1, acc_t.flags),
                                        isum::square(t2, acc_t.flags), isum::square(t3, acc_t.flags)));
            isum::add(acc_u, isum::sum4(isum::square(x0 - 1.0, acc_u.flags), isum::square(x1 - 1.0, acc_u.flags),
                                        isum::square(x2v - 1.0, acc_u.flags),
                                        last_has_next ? isum::square(x3 - 1.0, acc_u.flags)
                                                      : isum::sq_term{0u, isum::kEmptyExp}));
        }
        a = na;
        b = nb;
    }
    const double st = isum::value(group_isum<32>(acc_t, kFull));
    const double su = isum::value(group_isum<32>(acc_u, kFull));
    if (lane == 0 && f_out) *f_out = GRAD ? fma(100.0, st, 0.25 * su) : fma(100.0, st, su);
}

// ------------------------------------------------ ackley, griewank, schwefel
//
// Fitness only: the reference gives these UDPs no gradient. One group of G
// lanes per row, lanes strided over coordinates, sums (and griewank's product)
// reduced with shuffles; the closing expressions keep the reference's order.

// e as std::exp(1.0) rounds it.
constexpr double kNepero = 2.71828182845904523536;

template <int G>
__device__ __forceinline__ double group_prod(double v, unsigned mask)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v *= __shfl_xor_sync(mask, v, o, G);
    return v;
}

// f = -20 exp(-0.2 sqrt(s1/n)) - exp(s2/n) + 20 + e, s1 = sum x^2,
// s2 = sum cos(2 pi x) (src/problems/ackley.cpp:62-77).
template <int G>
__device__ __forceinline__ void ackley_row(const double *__restrict__ xr, uint32_t nx, double *f_out)
{
    const unsigned sub = threadIdx.x & (G - 1);
    const unsigned mask = group_mask<G>();
    isum::sq_acc sq = isum::make();
    double s2 = 0.0;
    double xn = sub < nx ? __ldg(xr + sub) : 0.0;
    for (uint32_t i = sub; i < nx; i += G) {
        const double xi = xn;
        if (i + G < nx) xn = __ldg(xr + i + G);
        isum::add_square(sq, xi);
        if (trigfx::in_range(xi)) {
            s2 += trigfx::cos_2pi(xi);
        } else {
            int c_neg = 0;
            const double c = fast_trig_arg(xi) ? cos_2pi(xi, c_neg) : cospi(xi + xi);
            s2 = fma(c, unit_sign(c_neg), s2);
        }
    }
    const double s1 = isum::value(group_isum<G>(sq, mask));
    s2 = group_sum<G>(s2, mask);
    if (sub == 0 && f_out) {
        const double inv_n = 1.0 / static_cast<double>(nx);
        *f_out = -20.0 * exp(-0.2 * sqrt(inv_n * s1)) - exp(inv_n * s2) + 20.0 + kNepero;
    }
}

// f = sum x^2 / 4000 - prod cos(x_i / sqrt(i + 1)) + 1 (src/problems/griewank.cpp:62-76);
// the division and square root are correctly rounded as in the reference.
// sqrt(i + 1) depends on the column only: `root` holds it (the same correctly
// rounded value) for the first `n_root` columns, computed once per block.
template <int G>
__device__ __forceinline__ void griewank_row(const double *__restrict__ xr, uint32_t nx, double *f_out,
                                             const double *root = nullptr, uint32_t n_root = 0)
{
    const unsigned sub = threadIdx.x & (G - 1);
    const unsigned mask = group_mask<G>();
    double s = 0.0, p = 1.0;
    double xn = sub < nx ? __ldg(xr + sub) : 0.0;
    for (uint32_t i = sub; i < nx; i += G) {
        const double xi = xn;
        if (i + G < nx) xn = __ldg(xr + i + G);
        s = fma(xi, xi, s);
        const double r = i < n_root ? root[i] : sqrt(static_cast<double>(i) + 1.0);
        p *= cos(xi / r);
    }
    s = group_sum<G>(s, mask);
    p = group_prod<G>(p, mask);
    if (sub == 0 && f_out) *f_out = s / 4000.0 - p + 1.0;
}

// f = 418.9828872724338 n - sum x sin(sqrt|x|) (src/problems/schwefel.cpp:62-70).
template <int G>
__device__ __forceinline__ void schwefel_row(const double *__restrict__ xr, uint32_t nx, double *f_out)
{
    const unsigned sub = threadIdx.x & (G - 1);
    const unsigned mask = group_mask<G>();
    double s = 0.0;
    double xn = sub < nx ? __ldg(xr + sub) : 0.0;
    for (uint32_t i = sub; i < nx; i += G) {
        const double xi = xn;
        if (i + G < nx) xn = __ldg(xr + i + G);
        s = fma(xi, sin(sqrt(fabs(xi))), s);
    }
    s = group_sum<G>(s, mask);
    if (sub == 0 && f_out) *f_out = 418.9828872724338 * static_cast<double>(nx) - s;
}

// ------------------------------------------------- rosenbrock on the FP32 pipe
//
// GB300 retires 2 FP64 lanes per SM per clock but ~115 FP32 and ~90 integer
// lanes (and converts between float and double on the FP64 pipe too). This
// variant evaluates rosenbrock rows in double-float arithmetic: every value is
// an unevaluated sum hi + lo of two floats (48 significant bits), operated on
// with error-free transformations -- Knuth's two-sum, Dekker/Møller's
// fast-two-sum, and the FMA product error e = fma(a, b, -a*b) -- so each
// result carries a relative error of about 2^-47 of the magnitudes it is formed
// from. Doubles are split into (hi, lo) and rebuilt from them with integer bit
// operations (no conversion instructions); the only FP64 instruction left per
// element adds the two halves of the gradient component. Fitness and gradients
// therefore stay within ~2e-14 of the first-order error bound of the
// reference's own FP64 evaluation (inside the 1e-13 parity tolerance). It is
// an opt-in (PGX_ROSENBROCK_DOUBLE_FLOAT=1): the default rows compute in FP64
// arithmetic, as the reference does.
//
// Range: the split and every intermediate stay finite floats when each
// element is 0 or 2^-60 <= |x| < 2^20 (|t| < 2^41, so a lane's sum of t^2 over
// any row of up to 2^31 elements stays below 2^115, and 400 x t < 2^70); the
// low parts of values below about 2^-100 may lose bits to float underflow,
// which is far below the error bound because such rows' terms are dominated
// by (x - 1)^2 ~ 1. A
// warp processes a chunk of 128 elements on this path only if all of them are
// in range; otherwise that chunk takes the FP64 path (the same arithmetic as
// rosenbrock_row_v4), with the running t carried across in both forms.

struct ff {
    float h, l; // value h + l
};

__device__ __forceinline__ ff ff_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ ff ff_fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// x = h + l with h = x rounded to a 24-bit mantissa and l the signed rest
// (29 bits, |l| <= 2^-24 |h|) rounded to a float: |x - h - l| <= 2^-48 |x|.
// ok = x is 0 or in the range of the FP32-pipe path (biased exponent in
// [1023-60, 1023+19]); h and l are meaningful only then.
__device__ __forceinline__ ff ff_split(double x, bool &ok)
{
    const unsigned hi = static_cast<unsigned>(__double2hiint(x)), lo = static_cast<unsigned>(__double2loint(x));
    const unsigned sign = hi & 0x80000000u, e = (hi >> 20) & 0x7ffu;
    const bool zero = ((hi << 1) | lo) == 0u;
    ok = e - 963u <= 1042u - 963u || zero;
    // round to nearest at bit 29 of the mantissa: add 2^28 with carry
    const unsigned lr = lo + 0x10000000u;
    const unsigned hr = hi + (lr < lo ? 1u : 0u);
    // float bits: exponent e - 896 (the top exponent bits drop out of hr << 3)
    const unsigned hb = ((hr << 3) + 0x40000000u) & 0x7fffffffu;
    const float h = __uint_as_float(zero ? sign : sign | hb | (lr >> 29));
    // the rest: signed 29-bit integer (lo's low bits minus the rounding) * 2^(e - 1075)
    const int rr = static_cast<int>(lo << 3) >> 3;
    const unsigned es = e < 963u ? 963u : e;
    const float scale = __uint_as_float(sign | ((es - 948u) << 23));
    return {h, __fmul_rn(__int2float_rn(rr), scale)};
}

// The double of a float, exactly, by bit operations (zero and subnormal
// floats give a signed zero).
__device__ __forceinline__ double ff_float_to_double(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned sign = b & 0x80000000u, mag = b & 0x7fffffffu;
    if (mag < 0x00800000u) return __hiloint2double(static_cast<int>(sign), 0);
    return __hiloint2double(static_cast<int>(sign | ((mag >> 3) + 0x38000000u)), static_cast<int>(b << 29));
}

// h + l as one double (one FP64 add).
__device__ __forceinline__ double ff_to_double(ff v)
{
    return ff_float_to_double(v.h) + ff_float_to_double(v.l);
}

// t = y - x^2 (x^2 = p + pe exactly up to the dropped l(x)^2 term).
__device__ __forceinline__ ff ff_rosen_t(ff x, ff y)
{
    const float p = __fmul_rn(x.h, x.h);
    float pe = __fmaf_rn(x.h, x.h, -p);
    pe = __fmaf_rn(__fmul_rn(2.0f, x.h), x.l, pe);
    const ff s = ff_two_sum(y.h, -p);
    return ff_fast_two_sum(s.h, __fadd_rn(s.l, __fsub_rn(y.l, pe)));
}

// acc += v^2 (v = h + l, non-negative terms: no renormalisation needed).
__device__ __forceinline__ void ff_acc_square(ff &acc, ff v)
{
    const float q = __fmul_rn(v.h, v.h);
    float qe = __fmaf_rn(v.h, v.h, -q);
    qe = __fmaf_rn(__fmul_rn(2.0f, v.h), v.l, qe);
    const ff s = ff_two_sum(acc.h, q);
    acc.h = s.h;
    acc.l = __fadd_rn(acc.l, __fadd_rn(s.l, qe));
}

// u = x - 1.
__device__ __forceinline__ ff ff_minus_one(ff x)
{
    const ff s = ff_two_sum(x.h, -1.0f);
    return ff_fast_two_sum(s.h, __fadd_rn(s.l, x.l));
}

// g = 200 (tp - 2 x t) + 2 u, as a double.
__device__ __forceinline__ double ff_rosen_grad(ff x, ff t, ff tp, ff u)
{
    const float a = __fmul_rn(x.h, t.h);
    float ae = __fmaf_rn(x.h, t.h, -a);
    ae = __fmaf_rn(x.h, t.l, ae);
    ae = __fmaf_rn(x.l, t.h, ae);
    const ff w = ff_two_sum(tp.h, __fmul_rn(-2.0f, a));
    const float wl = __fadd_rn(w.l, __fmaf_rn(-2.0f, ae, tp.l));
    const float b = __fmul_rn(w.h, 200.0f);
    float be = __fmaf_rn(w.h, 200.0f, -b);
    be = __fmaf_rn(wl, 200.0f, be);
    const ff g = ff_two_sum(b, __fmul_rn(2.0f, u.h));
    return ff_to_double({g.h, __fadd_rn(g.l, __fmaf_rn(2.0f, u.l, be))});
}

__device__ __forceinline__ ff ff_group_sum32(ff v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(kFull, v.h, o), ol = __shfl_xor_sync(kFull, v.l, o);
        const ff s = ff_two_sum(v.h, oh);
        v = ff_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(v.l, ol)));
    }
    return v;
}

// One warp per row, each lane owning 4 consecutive elements per 128-element
// chunk, as rosenbrock_row_v4 (nx % 4 == 0, 16-byte aligned rows).
template <bool GRAD>
__device__ __forceinline__ void rosenbrock_row_v4_ff(const double *__restrict__ xr, uint32_t nx, double *f_out,
                                                     double *__restrict__ gr)
{
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t slots = nx >> 2;
    const double2 *x2 = reinterpret_cast<const double2 *>(xr);
    ff acc_t{0.f, 0.f}, acc_u{0.f, 0.f};  // FP32-pipe chunks: sum t^2, sum u^2
    double dacc_t = 0.0, dacc_u = 0.0;    // FP64 chunks: sum t^2, sum (2u)^2
    ff carry{0.f, 0.f};                    // t of the previous chunk's last element
    double carry_d = 0.0;
    bool carry_is_ff = true;
    double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
    if (lane < slots) {
        a = __ldg(x2 + 2u * lane);
        b = __ldg(x2 + 2u * lane + 1u);
    }
    for (uint32_t base = 0; base < slots; base += 32u) {
        const uint32_t s = base + lane;
        const bool act = s < slots;
        const uint32_t sn = s + 32u;
        double2 na = make_double2(0.0, 0.0), nb = make_double2(0.0, 0.0);
        if (sn < slots) {
            na = __ldg(x2 + 2u * sn);
            nb = __ldg(x2 + 2u * sn + 1u);
        }
        const double x0 = a.x, x1 = a.y, x2v = b.x, x3 = b.y;
        double xn = __shfl_down_sync(kFull, x0, 1);
        const double head = __shfl_sync(kFull, na.x, 0);
        if (lane == 31u) xn = head;
        const bool last_has_next = s + 1u < slots;
        bool k0, k1, k2, k3, kn;
        const ff f0 = ff_split(x0, k0), f1 = ff_split(x1, k1), f2 = ff_split(x2v, k2), f3 = ff_split(x3, k3);
        const ff fn = ff_split(last_has_next ? xn : 0.0, kn);
        // the t carried in from an FP64 chunk must itself be in range
        bool kc = true;
        const ff carry_in = carry_is_ff ? carry : ff_split(carry_d, kc);
        if (__all_sync(kFull, (!act || (k0 && k1 && k2 && k3 && kn)) && kc)) {
            carry = carry_in;
            carry_is_ff = true;
            const ff t0 = ff_rosen_t(f0, f1), t1 = ff_rosen_t(f1, f2), t2 = ff_rosen_t(f2, f3);
            const ff t3 = last_has_next ? ff_rosen_t(f3, fn) : ff{0.f, 0.f};
            ff tp;
            tp.h = __shfl_up_sync(kFull, t3.h, 1);
            tp.l = __shfl_up_sync(kFull, t3.l, 1);
            if (lane == 0) tp = carry;
            carry.h = __shfl_sync(kFull, t3.h, 31);
            carry.l = __shfl_sync(kFull, t3.l, 31);
            if (act) {
                const ff u0 = ff_minus_one(f0), u1 = ff_minus_one(f1), u2 = ff_minus_one(f2);
                ff_acc_square(acc_t, t0);
                ff_acc_square(acc_t, t1);
                ff_acc_square(acc_t, t2);
                ff_acc_square(acc_u, u0);
                ff_acc_square(acc_u, u1);
                ff_acc_square(acc_u, u2);
                ff u3{0.f, 0.f};
                if (last_has_next) {
                    u3 = ff_minus_one(f3);
                    ff_acc_square(acc_t, t3);
                    ff_acc_square(acc_u, u3);
                }
                if (GRAD) {
                    double2 g01, g23;
                    g01.x = ff_rosen_grad(f0, t0, tp, u0);
                    g01.y = ff_rosen_grad(f1, t1, t0, u1);
                    g23.x = ff_rosen_grad(f2, t2, t1, u2);
                    if (last_has_next) {
                        g23.y = ff_rosen_grad(f3, t3, t2, u3);
                    } else {
                        // g_{n-1} = 200 t_{n-2}
                        const float bh = __fmul_rn(t2.h, 200.0f);
                        const float bl = __fmaf_rn(t2.l, 200.0f, __fmaf_rn(t2.h, 200.0f, -bh));
                        g23.y = ff_to_double({bh, bl});
                    }
                    double2 *g2 = reinterpret_cast<double2 *>(gr);
                    g2[2u * s] = g01;
                    g2[2u * s + 1u] = g23;
                }
            }
        } else {
            if (carry_is_ff) {
                carry_d = ff_to_double(carry);
                carry_is_ff = false;
            }
            const double t0 = fma(-x0, x0, x1);
            const double t1 = fma(-x1, x1, x2v);
            const double t2 = fma(-x2v, x2v, x3);
            const double t3 = last_has_next ? fma(-x3, x3, xn) : 0.0;
            double tp = __shfl_up_sync(kFull, t3, 1);
            if (lane == 0) tp = carry_d;
            carry_d = __shfl_sync(kFull, t3, 31);
            if (act) {
                const double c0 = (x0 + x0) - 2.0, c1 = (x1 + x1) - 2.0, c2 = (x2v + x2v) - 2.0;
                dacc_t = fma(t0, t0, dacc_t);
                dacc_t = fma(t1, t1, dacc_t);
                dacc_t = fma(t2, t2, dacc_t);
                dacc_u = fma(c0, c0, dacc_u);
                dacc_u = fma(c1, c1, dacc_u);
                dacc_u = fma(c2, c2, dacc_u);
                double c3 = 0.0;
                if (last_has_next) {
                    c3 = (x3 + x3) - 2.0;
                    dacc_t = fma(t3, t3, dacc_t);
                    dacc_u = fma(c3, c3, dacc_u);
                }
                if (GRAD) {
                    double2 g01, g23;
                    g01.x = fma(200.0, fma(-(x0 + x0), t0, tp), c0);
                    g01.y = fma(200.0, fma(-(x1 + x1), t1, t0), c1);
                    g23.x = fma(200.0, fma(-(x2v + x2v), t2, t1), c2);
                    g23.y = last_has_next ? fma(200.0, fma(-(x3 + x3), t3, t2), c3) : 200.0 * t2;
                    double2 *g2 = reinterpret_cast<double2 *>(gr);
                    g2[2u * s] = g01;
                    g2[2u * s + 1u] = g23;
                }
            }
        }
        a = na;
        b = nb;
    }
    acc_t = ff_group_sum32(acc_t);
    acc_u = ff_group_sum32(acc_u);
    dacc_t = group_sum<32>(dacc_t, kFull);
    dacc_u = group_sum<32>(dacc_u, kFull);
    if (lane == 0 && f_out) {
        const double st = ff_to_double(acc_t) + dacc_t, su = ff_to_double(acc_u) + 0.25 * dacc_u;
        *f_out = fma(100.0, st, su);
    }
}

// ------------------------------------------------------------- lennard_jones
//
// E = 4 sum_{i<j} (s^2 - s), s = r_ij^-6 (src/problems/lennard_jones.cpp:72-91);
// dE/dr_i = -24 sum_j s (2 s - 1) / r^2 (r_i - r_j). One warp per cluster.
// Coordinates are decoded into shared memory (structure of arrays) with the
// reference's pinned-atom convention (:132-151): atom 0 at the origin, atom 1
// at (0, 0, x0), atom 2 at (0, x1, x2), atom k >= 3 at x[3(k-2) .. 3(k-2)+2];
// in the flattened 3N layout P[p] = x[p-6] for p >= 7, P[5] = x[0], else 0.
// The i<j pairs are walked as a half ring, pair (i, i+k mod N) for
// k = 1..N/2 (k = N/2 only for i < N/2 when N is even), so every lane does
// the same number of pairs. A zero distance makes the reference overwrite
// its sum with DBL_MAX and end at +inf (:81-82, :89); a NaN term keeps NaN.

// 1/d: the hardware approximation refined by one cubic Newton step
// (y1 = y0 (1 + e + e^2), e = 1 - d y0). d = +inf gives 0 (not NaN).
__device__ __forceinline__ double lj_rcp(double d)
{
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
    const double e = fma(-d, y, 1.0);
    const double r = fma(y, fma(e, e, e), y);
    return (__double_as_longlong(y) << 1) == 0 ? y : r;
}

// Fixed-point 1/d and s = d^-3 for d = (u / 2^63) 2^k, 2^63 <= u < 2^64
// (rcp_fixed.h): 1/d = z 2^(-64 - k), s = n3 2^(-64 - l3 - 3k) with
// 2^63 <= n3 < 2^64. The seed is the FP32 approximate reciprocal of u's
// leading bits.
struct lj_fixed {
    uint64_t z, n3;
    int l3;
};

__device__ __forceinline__ lj_fixed lj_fixed_core(uint64_t u)
{
    float yf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(__uint_as_float(rcpfx::seed_input_bits_u(u))));
    lj_fixed r;
    r.z = rcpfx::rcp_q64_u(u, rcpfx::seed_q32(__float_as_uint(yf)));
    const uint64_t z3 = rcpfx::mul_hi_u64(rcpfx::mul_hi_u64(r.z, r.z), r.z);
    r.l3 = isum::clz64(z3);
    r.n3 = z3 << r.l3;
    return r;
}

// 1/d and s rounded to doubles (-100 <= k <= 100: both normal)
__device__ __forceinline__ double lj_fixed_inv(const lj_fixed &r, int32_t k)
{
    return __longlong_as_double(
        static_cast<long long>((static_cast<uint64_t>(1021 - k) << 52) + rcpfx::round_q64(r.z)));
}

__device__ __forceinline__ uint64_t lj_fixed_s_bits(const lj_fixed &r, int32_t k)
{
    return (static_cast<uint64_t>(1021 - 3 * k - r.l3) << 52) + rcpfx::round_q64(r.n3);
}

// The force coefficient (2 s^2 - s) / d = (2s - 1) s (1/d) in fixed point,
// rounded to a double once. With s = n3 2^Es (Es = -64 - l3 - 3k), 2s - 1 is
// formed exactly as W 2^Ec, Ec = max(Es + 3, -62) (the 1 drops below the last
// unit only when 2s > 2^62), s (1/d) = pm 2^(-64 - l3 - 4k) with pm the high
// half of n3 z, and the product's high half gives the result to within 2^-60
// of max(2s, 1) s / d relative: as close as the FP64 fma(2s, s, -s) / d of
// rounded s and 1/d, or closer.
__device__ __forceinline__ double lj_fixed_coef(const lj_fixed &r, int32_t k)
{
    const int32_t es = -64 - r.l3 - 3 * k;
    const int32_t ec = es + 3 > -62 ? es + 3 : -62;
    const int sh = ec - es - 1 < 63 ? ec - es - 1 : 63;               // 2s = n3 2^(es+1) in units of 2^ec
    const int64_t one = ec <= 0 ? (int64_t{1} << (-ec)) : 0;          // 1 in units of 2^ec
    const int64_t w = static_cast<int64_t>(r.n3 >> sh) - one;         // (2s - 1) = w 2^ec
    const uint64_t pm = rcpfx::mul_hi_u64(r.n3, r.z);                 // s (1/d) = pm 2^(-64 - l3 - 4k)
    const int64_t q = rcpfx::mul_hi_s64(w, static_cast<int64_t>(pm >> 1)); // coef = q 2^(ec - l3 - 4k + 1)
    if (q == 0) return 0.0;
    const uint64_t mag = static_cast<uint64_t>(q < 0 ? -q : q);
    return trigfx::to_double(mag, ec - r.l3 - 4 * k + 1, q < 0 ? 1u : 0u);
}

// The pair loops' 1/d and d^-3 for a double d (self-test): d = (u / 2^63) 2^k
// with u from d's significand; outside 2^-100 .. 2^100, lj_rcp and two FP64
// multiplies.
__device__ __forceinline__ void lj_rcp_cube(double d, double &inv, double &s)
{
    const uint64_t b = static_cast<uint64_t>(__double_as_longlong(d));
    const int32_t k = static_cast<int32_t>((b >> 52) & 0x7ffu) - 1023;
    if (k < -100 || k > 100 || (b >> 63)) {
        inv = lj_rcp(d);
        s = inv * inv * inv;
        return;
    }
    const lj_fixed r = lj_fixed_core((1ull << 63) | (b << 11));
    inv = lj_fixed_inv(r, k);
    s = __longlong_as_double(static_cast<long long>(lj_fixed_s_bits(r, k)));
}

// One pair from its FP64 coordinate differences, with integer arithmetic
// where it is exact or closer than FP64: d = dx^2 + dy^2 + dz^2 as the
// aligned sum of the three squares (isum.h, within 2^-59 of the exact d), 1/d
// and s = d^-3 in fixed point from that sum (rcp_fixed.h: Newton-Raphson
// division seeded by the FP32 approximate reciprocal, then two 64 x 64-bit
// products), and the energy as two integer sums E12 += s^2, E6 += s
// (E = 4 (E12 - E6)). With the gradient, coef = (2 s^2 - s) / d in fixed point
// as well (lj_fixed_coef). The FP64 formulation spends 13 FP64 instructions per
// pair on the energy and 2 more on coef, on a pipe that retires two lanes per
// SM per clock. Sums outside 2^-100 .. 2^100 and
// infinite or NaN differences take the FP64 formulas (lj_rcp). A zero
// distance sets *zero and gives coef = NaN (the reference's 1/0 in the
// gradient).
template <bool GRAD>
__device__ __forceinline__ void lj_pair(double dx, double dy, double dz, isum::sq_acc &e12, isum::sq_acc &e6,
                                        int &zero, double &coef)
{
    uint32_t fl = 0u;
    const isum::sq_term d3 = isum::sum3(isum::square(dx, fl), isum::square(dy, fl), isum::square(dz, fl));
    if (d3.p == 0u && fl == 0u) {
        zero = 1;
        if (GRAD) coef = __longlong_as_double(0x7ff8000000000000LL);
        return;
    }
    const int lz = d3.p ? isum::clz64(d3.p) : 0;
    const int32_t k = d3.q - lz + 63; // d = (u / 2^63) 2^k
    if (fl != 0u || k < -100 || k > 100) {
        const double d = fma(dx, dx, fma(dy, dy, dz * dz));
        if (__double_as_longlong(d) == 0) {
            zero = 1;
            if (GRAD) coef = __longlong_as_double(0x7ff8000000000000LL);
            return;
        }
        const double inv = lj_rcp(d);
        const double s = inv * inv * inv;
        isum::add_square(e12, s);
        isum::add(e6, isum::magnitude(s, e6.flags));
        if (GRAD) coef = fma(s + s, s, -s) * inv;
        return;
    }
    const lj_fixed r = lj_fixed_core(d3.p << lz);
    isum::add(e6, isum::sq_term{r.n3 >> 2, -62 - r.l3 - 3 * k});                                 // s
    isum::add(e12, isum::sq_term{rcpfx::mul_hi_u64(r.n3, r.n3) >> 2, -62 - 2 * r.l3 - 6 * k}); // s^2
    if (GRAD) coef = lj_fixed_coef(r, k);
}

// 4 (E12 - E6) over the warp, or +inf after a zero distance (NaN stays NaN).
__device__ __forceinline__ double lj_energy(isum::sq_acc e12, isum::sq_acc e6, int zero)
{
    const double a = isum::value(group_isum<32>(e12, kFull));
    const double b = isum::value(group_isum<32>(e6, kFull));
    const double e = a - b;
    return __any_sync(kFull, zero) ? (isnan(e) ? e : HUGE_VAL) : 4.0 * e;
}

__device__ __forceinline__ void lj_decode(const double *__restrict__ xr, uint32_t na, double *px, double *py,
                                          double *pz, double *gx, double *gy, double *gz, bool zero_g)
{
    const unsigned lane = threadIdx.x & 31u;
    for (uint32_t p = lane; p < 3u * na; p += 32u) {
        double v = 0.0;
        if (p == 5u)
            v = __ldg(xr);
        else if (p >= 7u)
            v = __ldg(xr + (p - 6u));
        const uint32_t at = p / 3u, cc = p - 3u * at;
        (cc == 0u ? px : (cc == 1u ? py : pz))[at] = v;
        if (zero_g) (cc == 0u ? gx : (cc == 1u ? gy : gz))[at] = 0.0;
    }
    __syncwarp();
}

// Writes -24 * G[atom(v)][coord(v)] for every free coordinate v.
__device__ __forceinline__ void lj_store_gradient(uint32_t nx, const double *gx, const double *gy, const double *gz,
                                                  double *__restrict__ gr)
{
    const unsigned lane = threadIdx.x & 31u;
    for (uint32_t v = lane; v < nx; v += 32u) {
        uint32_t at, cc;
        if (v < 3u) {
            at = v == 0u ? 1u : 2u;
            cc = v == 1u ? 1u : 2u;
        } else {
            at = v / 3u + 2u;
            cc = v - 3u * (v / 3u);
        }
        gr[v] = -24.0 * (cc == 0u ? gx : (cc == 1u ? gy : gz))[at];
    }
}

// Register variant (N <= 32*MA): lane l owns atoms l, l+32, ..., whose
// positions and force sums stay in registers; only the reaction on the
// partner atom goes through shared memory. Per pair, fitness + gradient:
// 9 FP64 instructions (3 differences, 3 own and 3 reaction FMAs; lj_pair
// does the rest on the integer pipes); fitness only: 3.
template <int MA, bool GRAD>
__device__ __forceinline__ void lj_cluster_reg(const double *__restrict__ xr, uint32_t na, uint32_t nx, double *sm,
                                               double *f_out, double *__restrict__ gr)
{
    const unsigned lane = threadIdx.x & 31u;
    double *px = sm, *py = px + na, *pz = py + na;
    double *gx = pz + na, *gy = gx + na, *gz = gy + na;
    lj_decode(xr, na, px, py, pz, gx, gy, gz, GRAD);
    double ox[MA], oy[MA], oz[MA], fx[MA], fy[MA], fz[MA];
#pragma unroll
    for (int m = 0; m < MA; ++m) {
        const uint32_t i = 32u * m + lane;
        ox[m] = i < na ? px[i] : 0.0;
        oy[m] = i < na ? py[i] : 0.0;
        oz[m] = i < na ? pz[i] : 0.0;
        fx[m] = fy[m] = fz[m] = 0.0;
    }
    isum::sq_acc e12 = isum::make(), e6 = isum::make();
    int zero = 0;
    const bool even = (na & 1u) == 0u;
    const uint32_t kmax = na / 2u;
    for (uint32_t k = 1u; k <= kmax; ++k) {
        const uint32_t ilim = (even && k == kmax) ? kmax : na;
#pragma unroll
        for (int m = 0; m < MA; ++m) {
            const uint32_t i = 32u * m + lane;
            if (i < ilim) {
                uint32_t j = i + k;
                if (j >= na) j -= na;
                const double dx = ox[m] - px[j], dy = oy[m] - py[j], dz = oz[m] - pz[j];
                double coef = 0.0; // (2 s^2 - s) / r^2
                lj_pair<GRAD>(dx, dy, dz, e12, e6, zero, coef);
                if (GRAD) {
                    fx[m] = fma(coef, dx, fx[m]);
                    fy[m] = fma(coef, dy, fy[m]);
                    fz[m] = fma(coef, dz, fz[m]);
                    gx[j] = fma(-coef, dx, gx[j]);
                    gy[j] = fma(-coef, dy, gy[j]);
                    gz[j] = fma(-coef, dz, gz[j]);
                }
            }
        }
        // the partners of one step are distinct; the next step may revisit them
        if (GRAD) __syncwarp();
    }
    const double energy = lj_energy(e12, e6, zero);
    if (lane == 0 && f_out) *f_out = energy;
    if (GRAD) {
#pragma unroll
        for (int m = 0; m < MA; ++m) {
            const uint32_t i = 32u * m + lane;
            if (i < na) {
                gx[i] += fx[m];
                gy[i] += fy[m];
                gz[i] += fz[m];
            }
        }
        __syncwarp();
        lj_store_gradient(nx, gx, gy, gz, gr);
    }
    __syncwarp();
}

// Flattened variant (N >= 33): the half-ring pairs (k, i) are enumerated in
// one sequence and the 32 lanes take 32 consecutive pairs per step, so every
// lane is busy (the register variant idles the lanes beyond N in its last
// chunk). A step spans at most two values of k; since N >= 33, its lanes
// still hold distinct i and distinct j, so both sides of the pairs are
// accumulated in shared memory in two conflict-free phases.
template <bool GRAD>
__device__ __forceinline__ void lj_cluster_flat(const double *__restrict__ xr, uint32_t na, uint32_t nx, double *sm,
                                                double *f_out, double *__restrict__ gr)
{
    const unsigned lane = threadIdx.x & 31u;
    double *px = sm, *py = px + na, *pz = py + na;
    double *gx = pz + na, *gy = gx + na, *gz = gy + na;
    lj_decode(xr, na, px, py, pz, gx, gy, gz, GRAD);
    const bool even = (na & 1u) == 0u;
    const uint32_t kmax = na / 2u;
    const uint32_t pairs = na * (na - 1u) / 2u;
    isum::sq_acc e12 = isum::make(), e6 = isum::make();
    int zero = 0;
    uint32_t k = 1u, i = lane; // pair number q0 + lane, q0 = 0
    for (uint32_t q0 = 0; q0 < pairs; q0 += 32u) {
        const bool act = q0 + lane < pairs;
        uint32_t j = i + k;
        if (j >= na) j -= na;
        double dx = 0.0, dy = 0.0, dz = 0.0, coef = 0.0;
        if (act) {
            dx = px[i] - px[j];
            dy = py[i] - py[j];
            dz = pz[i] - pz[j];
            lj_pair<GRAD>(dx, dy, dz, e12, e6, zero, coef);
        }
        if (GRAD) {
            if (act) {
                gx[i] = fma(coef, dx, gx[i]);
                gy[i] = fma(coef, dy, gy[i]);
                gz[i] = fma(coef, dz, gz[i]);
            }
            __syncwarp();
            if (act) {
                gx[j] = fma(-coef, dx, gx[j]);
                gy[j] = fma(-coef, dy, gy[j]);
                gz[j] = fma(-coef, dz, gz[j]);
            }
            __syncwarp();
        }
        // advance this lane's pair by 32 in the (k, i) sequence
        i += 32u;
        for (;;) {
            const uint32_t ilim = (even && k == kmax) ? kmax : na;
            if (i < ilim || k >= kmax) break;
            i -= ilim;
            ++k;
        }
    }
    const double energy = lj_energy(e12, e6, zero);
    if (lane == 0 && f_out) *f_out = energy;
    if (GRAD) {
        __syncwarp();
        lj_store_gradient(nx, gx, gy, gz, gr);
    }
    __syncwarp();
}

// Shared-memory variant for any N: both sides of each pair go through shared
// memory, in two conflict-free phases (the lanes of one step hold distinct i
// and distinct j).
template <bool GRAD>
__device__ __forceinline__ void lj_cluster_smem(const double *__restrict__ xr, uint32_t na, uint32_t nx, double *sm,
                                                double *f_out, double *__restrict__ gr)
{
    const unsigned lane = threadIdx.x & 31u;
    double *px = sm, *py = px + na, *pz = py + na;
    double *gx = pz + na, *gy = gx + na, *gz = gy + na;
    lj_decode(xr, na, px, py, pz, gx, gy, gz, GRAD);
    isum::sq_acc e12 = isum::make(), e6 = isum::make();
    int zero = 0;
    const bool even = (na & 1u) == 0u;
    const uint32_t kmax = na / 2u;
    for (uint32_t k = 1u; k <= kmax; ++k) {
        const uint32_t ilim = (even && k == kmax) ? kmax : na;
        for (uint32_t i0 = 0u; i0 < ilim; i0 += 32u) {
            const uint32_t i = i0 + lane;
            const bool act = i < ilim;
            uint32_t j = i + k;
            if (j >= na) j -= na;
            double dx = 0.0, dy = 0.0, dz = 0.0, coef = 0.0;
            if (act) {
                dx = px[i] - px[j];
                dy = py[i] - py[j];
                dz = pz[i] - pz[j];
                lj_pair<GRAD>(dx, dy, dz, e12, e6, zero, coef);
            }
            if (GRAD) {
                if (act) {
                    gx[i] = fma(coef, dx, gx[i]);
                    gy[i] = fma(coef, dy, gy[i]);
                    gz[i] = fma(coef, dz, gz[i]);
                }
                __syncwarp();
                if (act) {
                    gx[j] = fma(-coef, dx, gx[j]);
                    gy[j] = fma(-coef, dy, gy[j]);
                    gz[j] = fma(-coef, dz, gz[j]);
                }
                __syncwarp();
            }
        }
    }
    const double energy = lj_energy(e12, e6, zero);
    if (lane == 0 && f_out) *f_out = energy;
    if (GRAD) {
        __syncwarp();
        lj_store_gradient(nx, gx, gy, gz, gr);
    }
    __syncwarp();
}

} // namespace dev
} // namespace pgx
