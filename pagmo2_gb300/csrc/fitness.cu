// Batch fitness and gradient kernels for the three single-objective UDPs of
// the reference: rastrigin (src/problems/rastrigin.cpp:62-72, 98-107),
// rosenbrock (src/problems/rosenbrock.cpp:59-66, 83-92) and lennard_jones
// (src/problems/lennard_jones.cpp:72-91, 132-151).
//
// All arithmetic is FP64. On GB300 the FP64 pipe, not HBM, bounds these
// kernels, so the formulations below aim at the fewest FP64 instructions per
// element while keeping every result within 1e-13 (relative to the sum of
// absolute terms) of the reference:
//  - rastrigin evaluates cos(2 pi x) as cospi(2x): 2x is exact, so the
//    argument reduction is exact too (the reference rounds omega*x first);
//  - rosenbrock shares t = x_{i+1} - x_i^2 between the fitness and both
//    gradient terms it feeds, and accumulates sum t^2 and sum (x-1)^2 apart;
//  - lennard_jones walks the i<j pairs as a "half ring" (pair (i, i+k mod N)
//    for k = 1..N/2) so every lane of a warp does the same number of pairs,
//    and the backward pass applies each pair force to both atoms (the
//    reaction through shared memory) instead of visiting every pair twice.
#include "pgx_internal.cuh"

#include <cmath>

namespace pgx
{
namespace
{

// 2*pi and 10*(2*pi) as the reference rounds them (rastrigin.cpp:65, :104).
constexpr double kOmega = 2. * 3.1415926535897932384626433832795028841971693993;
constexpr double k10Omega = 10.0 * kOmega;

constexpr unsigned kFull = 0xffffffffu;

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

// ------------------------------------------------------------------ rastrigin

// One group of G lanes per decision vector, lanes strided over coordinates.
// f = sum_i (x_i^2 - 10 cos(2 pi x_i)) + 10 n; g_i = 2 x_i + 10 omega sin(2 pi x_i).
template <int G, bool GRAD>
__global__ void __launch_bounds__(256) rastrigin_kernel(const double *__restrict__ x, uint64_t n, uint32_t nx,
                                                        double *__restrict__ f, double *__restrict__ g)
{
    const unsigned sub = threadIdx.x & (G - 1);
    const unsigned mask = group_mask<G>();
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * (blockDim.x / G);
    for (uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / G; row < n; row += stride) {
        const double *xr = x + row * nx;
        double acc = 0.0;
        for (uint32_t i = sub; i < nx; i += G) {
            const double xi = __ldg(xr + i);
            const double y = xi + xi;
            if (GRAD) {
                double s, c;
                sincospi(y, &s, &c);
                acc += fma(xi, xi, -10.0 * c);
                g[row * nx + i] = fma(k10Omega, s, y);
            } else {
                acc += fma(xi, xi, -10.0 * cospi(y));
            }
        }
        acc = group_sum<G>(acc, mask);
        if (sub == 0 && f) f[row] = acc + 10.0 * static_cast<double>(nx);
    }
}

// ----------------------------------------------------------------- rosenbrock

// One group of G lanes per decision vector; element i of a chunk sits in lane
// i mod G, x_{i+1} comes from the next lane (the last lane takes the next
// chunk's first element), t_{i-1} from the previous lane.
// With t_i = x_{i+1} - x_i^2 and c_i = 2 x_i - 2:
//   f   = 100 sum t_i^2 + sum (x_i - 1)^2                 (i < n-1)
//   g_i = 200 (t_{i-1} - 2 x_i t_i) + c_i                 (0 <= i < n-1, t_{-1} = 0)
//   g_{n-1} = 200 t_{n-2}
template <int G, bool GRAD>
__global__ void __launch_bounds__(256) rosenbrock_kernel(const double *__restrict__ x, uint64_t n, uint32_t nx,
                                                         double *__restrict__ f, double *__restrict__ g)
{
    const unsigned sub = threadIdx.x & (G - 1);
    const unsigned mask = group_mask<G>();
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * (blockDim.x / G);
    for (uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / G; row < n; row += stride) {
        const double *xr = x + row * nx;
        double *gr = GRAD ? g + row * nx : nullptr;
        double acc_t = 0.0, acc_u = 0.0, t_carry = 0.0;
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
                        acc_t = fma(t, t, acc_t);
                        acc_u = fma(c, c, acc_u);
                        gi = fma(200.0, fma(-w, t, t_prev), c);
                    } else {
                        gi = 200.0 * t_prev;
                    }
                    gr[i] = gi;
                }
            } else if (has_next) {
                const double u = x_cur - 1.0;
                acc_t = fma(t, t, acc_t);
                acc_u = fma(u, u, acc_u);
            }
            x_cur = x_nxt;
        }
        acc_t = group_sum<G>(acc_t, mask);
        acc_u = group_sum<G>(acc_u, mask);
        // with the gradient the second sum is over c^2 = 4 (x-1)^2
        if (sub == 0 && f) f[row] = GRAD ? fma(100.0, acc_t, 0.25 * acc_u) : fma(100.0, acc_t, acc_u);
    }
}

// ------------------------------------------------------------- lennard_jones

// One warp per cluster. Atom coordinates are decoded into shared memory (SoA)
// with the reference's pinned-atom convention: atom 0 at the origin, atom 1 at
// (0, 0, x0), atom 2 at (0, x1, x2), atom k >= 3 at x[3(k-2) .. 3(k-2)+2];
// in the flattened 3N layout P[p] = x[p-6] for p >= 7, P[5] = x[0], else 0.
//
// Energy: E = 4 sum_{i<j} (s^2 - s), s = r_ij^-6. A zero distance makes the
// reference overwrite its running sum with DBL_MAX (lennard_jones.cpp:81-82)
// and the final 4* turns it into +inf; a NaN term keeps it NaN.
// Gradient: dE/dr_i = -24 sum_j s (2 s - 1) / r^2 (r_i - r_j).
template <bool GRAD>
__global__ void __launch_bounds__(128) lj_kernel(const double *__restrict__ x, uint64_t n, uint32_t na, uint32_t nx,
                                                 double *__restrict__ f, double *__restrict__ g)
{
    extern __shared__ double smem[];
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const unsigned wpb = blockDim.x >> 5;
    double *px = smem + static_cast<size_t>(warp) * (GRAD ? 6u : 3u) * na;
    double *py = px + na;
    double *pz = py + na;
    double *gx = pz + na;
    double *gy = gx + na;
    double *gz = gy + na;
    const bool even = (na & 1u) == 0u;
    const uint32_t kmax = na / 2u; // for odd na this is (na-1)/2
    for (uint64_t c = static_cast<uint64_t>(blockIdx.x) * wpb + warp; c < n;
         c += static_cast<uint64_t>(gridDim.x) * wpb) {
        const double *xr = x + c * nx;
        for (uint32_t p = lane; p < 3u * na; p += 32u) {
            double v = 0.0;
            if (p == 5u)
                v = __ldg(xr);
            else if (p >= 7u)
                v = __ldg(xr + (p - 6u));
            const uint32_t a = p / 3u, cc = p - 3u * a;
            (cc == 0u ? px : (cc == 1u ? py : pz))[a] = v;
            if (GRAD) (cc == 0u ? gx : (cc == 1u ? gy : gz))[a] = 0.0;
        }
        __syncwarp();
        double e = 0.0;
        int zero = 0;
        for (uint32_t k = 1u; k <= kmax; ++k) {
            const uint32_t ilim = (even && k == kmax) ? kmax : na;
            for (uint32_t i0 = 0u; i0 < ilim; i0 += 32u) {
                const uint32_t i = i0 + lane;
                const bool act = i < ilim;
                uint32_t j = i + k;
                if (j >= na) j -= na;
                double fxv = 0.0, fyv = 0.0, fzv = 0.0;
                if (act) {
                    const double dx = px[i] - px[j], dy = py[i] - py[j], dz = pz[i] - pz[j];
                    const double d = fma(dx, dx, fma(dy, dy, dz * dz));
                    const double inv = 1.0 / d;
                    const double s = inv * inv * inv;
                    if (d != 0.0)
                        e += fma(s, s, -s);
                    else
                        zero = 1;
                    if (GRAD) {
                        const double coef = fma(s, s + s, -s) * inv;
                        fxv = coef * dx;
                        fyv = coef * dy;
                        fzv = coef * dz;
                    }
                }
                if (GRAD) {
                    // lanes hold distinct i and distinct j: two conflict-free phases
                    if (act) {
                        gx[i] += fxv;
                        gy[i] += fyv;
                        gz[i] += fzv;
                    }
                    __syncwarp();
                    if (act) {
                        gx[j] -= fxv;
                        gy[j] -= fyv;
                        gz[j] -= fzv;
                    }
                    __syncwarp();
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(kFull, e, o);
        zero = __any_sync(kFull, zero);
        if (lane == 0 && f) f[c] = zero ? (isnan(e) ? e : HUGE_VAL) : 4.0 * e;
        if (GRAD) {
            for (uint32_t v = lane; v < nx; v += 32u) {
                uint32_t a, cc;
                if (v < 3u) {
                    a = v == 0u ? 1u : 2u;
                    cc = v == 1u ? 1u : 2u;
                } else {
                    a = v / 3u + 2u;
                    cc = v - 3u * (v / 3u);
                }
                const double gv = (cc == 0u ? gx : (cc == 1u ? gy : gz))[a];
                g[c * nx + v] = -24.0 * gv;
            }
        }
        __syncwarp();
    }
}

template <typename K>
int grid_for(K kernel, int threads, size_t smem, uint64_t work_items, int per_block, int num_sms, int *grid)
{
    int occ = 0;
    PGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem));
    if (occ < 1) occ = 1;
    const uint64_t need = (work_items + per_block - 1) / per_block;
    const uint64_t cap = static_cast<uint64_t>(num_sms) * occ;
    *grid = static_cast<int>(need < cap ? (need ? need : 1) : cap);
    return PGX_OK;
}

template <int G>
int launch_rows(int kind, bool grad, const double *x, uint64_t n, uint32_t nx, double *f, double *g,
                cudaStream_t s, int num_sms)
{
    constexpr int threads = 256;
    constexpr int per_block = threads / G;
    int grid = 1;
    if (kind == PGX_RASTRIGIN) {
        if (grad) {
            PGX_TRY(grid_for(rastrigin_kernel<G, true>, threads, 0, n, per_block, num_sms, &grid));
            rastrigin_kernel<G, true><<<grid, threads, 0, s>>>(x, n, nx, f, g);
        } else {
            PGX_TRY(grid_for(rastrigin_kernel<G, false>, threads, 0, n, per_block, num_sms, &grid));
            rastrigin_kernel<G, false><<<grid, threads, 0, s>>>(x, n, nx, f, g);
        }
    } else {
        if (grad) {
            PGX_TRY(grid_for(rosenbrock_kernel<G, true>, threads, 0, n, per_block, num_sms, &grid));
            rosenbrock_kernel<G, true><<<grid, threads, 0, s>>>(x, n, nx, f, g);
        } else {
            PGX_TRY(grid_for(rosenbrock_kernel<G, false>, threads, 0, n, per_block, num_sms, &grid));
            rosenbrock_kernel<G, false><<<grid, threads, 0, s>>>(x, n, nx, f, g);
        }
    }
    PGX_CUDA(cudaGetLastError());
    return PGX_OK;
}

} // namespace

int launch_eval(int kind, uint64_t param, uint64_t nx, const double *d_x, uint64_t n, double *d_f, double *d_g,
                cudaStream_t stream, int num_sms, uint64_t *launches)
{
    if (n == 0) return PGX_OK;
    PGX_CHECK(nx < (1ull << 31), PGX_ERR_CAPACITY, "decision vector dimension exceeds 2^31-1");
    const bool grad = d_g != nullptr;
    const uint32_t nx32 = static_cast<uint32_t>(nx);
    if (kind == PGX_RASTRIGIN || kind == PGX_ROSENBROCK) {
        int st;
        if (nx <= 48)
            st = launch_rows<8>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms);
        else if (nx <= 256)
            st = launch_rows<16>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms);
        else
            st = launch_rows<32>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms);
        if (st == PGX_OK && launches) ++*launches;
        return st;
    }
    if (kind == PGX_LENNARD_JONES) {
        const uint32_t na = static_cast<uint32_t>(param);
        const size_t per_warp = static_cast<size_t>(grad ? 6u : 3u) * na * sizeof(double);
        PGX_CHECK(per_warp <= 200u * 1024u, PGX_ERR_CAPACITY, "lennard_jones: too many atoms for one cluster per warp");
        int wpb = static_cast<int>((96u * 1024u) / per_warp);
        if (wpb > 4) wpb = 4;
        if (wpb < 1) wpb = 1;
        const int threads = 32 * wpb;
        const size_t smem = per_warp * wpb;
        int grid = 1;
        if (grad) {
            PGX_CUDA(cudaFuncSetAttribute(lj_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(smem > 48u * 1024u ? smem : 48u * 1024u)));
            PGX_TRY(grid_for(lj_kernel<true>, threads, smem, n, wpb, num_sms, &grid));
            lj_kernel<true><<<grid, threads, smem, stream>>>(d_x, n, na, nx32, d_f, d_g);
        } else {
            PGX_CUDA(cudaFuncSetAttribute(lj_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(smem > 48u * 1024u ? smem : 48u * 1024u)));
            PGX_TRY(grid_for(lj_kernel<false>, threads, smem, n, wpb, num_sms, &grid));
            lj_kernel<false><<<grid, threads, smem, stream>>>(d_x, n, na, nx32, d_f, d_g);
        }
        PGX_CUDA(cudaGetLastError());
        if (launches) ++*launches;
        return PGX_OK;
    }
    set_error("unknown problem kind " + std::to_string(kind));
    return PGX_ERR_INVALID;
}

} // namespace pgx
