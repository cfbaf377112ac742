// Hypervolume of 2 or 3 objectives on the GPU (pagmo's hypervolume::compute,
// src/utils/hypervolume.cpp:203-228, which picks hv2d for two objectives and
// hv3d for three: src/utils/hv_algos/hv_hv2d.cpp:48-68, hv_hv3d.cpp:75-116),
// and the C ABI of the hypervolume queries: compute (4 or more objectives by
// hvwfg in hv_wfg.cu), exclusive, contributions and the least and greatest
// contributors (hypervolume.cpp:249-401).
//
// The dominated region is summed as non-negative slabs (no cancellation):
//  - 2D: with the points sorted by y, the staircase width W(t) = max over the
//    first t+1 points of (r_x - x), and HV = sum_t (y_{t+1} - y_t) W(t) with
//    y_n = r_y (hv2d's own sweep, summed as a tree).
//  - 3D: with the points sorted by z, level i holds the 2D area A_i of the
//    points up to level i, and HV = sum_i (z_{i+1} - z_i) A_i with z_n = r_z.
//    Every level is an independent thread: over the points in y order
//    (staged through shared memory for a block of levels), the running
//    maximum of (r_x - x) among the points whose z rank is at most i, summed
//    run by run between the points that widen it. O(n^2) integer work, FP64
//    only at those points, all levels in parallel.
// Order: both sorts are counting ranks over the NaN-aware int64 order keys
// (ties by index); a tie does not change any slab (its step is zero). The
// widths r_x - x are non-negative on valid input, so their running maximum
// is taken on the IEEE bit patterns with integer operations.
#include "pgx_internal.cuh"

#include <algorithm>
#include <climits>
#include <cmath>
#include <sstream>
#include <string>
#include <vector>

namespace pgx
{
namespace
{

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ long long hv_key(double v)
{
    if (isnan(v)) return LLONG_MAX;
    if (v == 0.0) return 0;
    const long long b = __double_as_longlong(v);
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

// order keys kyz[c * n + t]: c = 0 the y coordinate; for 3D also c = 1 the z
// coordinate and c = 2 the x coordinate
__global__ void hv_keys_kernel(const double *__restrict__ pts, uint32_t n, uint32_t m, long long *__restrict__ kyz)
{
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const double *p = pts + static_cast<uint64_t>(t) * m;
        kyz[t] = hv_key(p[1]);
        if (m == 3u) {
            kyz[static_cast<uint64_t>(n) + t] = hv_key(p[2]);
            kyz[2ull * n + t] = hv_key(p[0]);
        }
    }
}

// Ranks by coordinate c + 1 (ties by index) in two steps. hv_runs_kernel:
// block b sorts the (key, index) pairs of points [b R, (b + 1) R) (R =
// kRun) by a bitonic network in shared memory, padding with (LLONG_MAX,
// INT_MAX), which no point's pair exceeds, and writes the sorted run.
// hv_rank_kernel: a point's rank is the number of pairs below its own, summed
// over every run by binary search (pairs are distinct, so this is its
// position). blockIdx.y = c.
constexpr uint32_t kRun = 2048;

struct key_idx {
    long long k;
    long long i;
};

__device__ __forceinline__ bool pair_less(const key_idx &a, const key_idx &b)
{
    return a.k < b.k || (a.k == b.k && a.i < b.i);
}

__global__ void __launch_bounds__(1024) hv_runs_kernel(const long long *__restrict__ kyz, uint32_t n,
                                                       key_idx *__restrict__ runs)
{
    __shared__ key_idx s[kRun];
    const uint32_t c = blockIdx.y, nb = gridDim.x;
    const long long *k = kyz + static_cast<uint64_t>(c) * n;
    const uint32_t t0 = blockIdx.x * kRun;
    for (uint32_t j = threadIdx.x; j < kRun; j += blockDim.x) {
        const uint32_t t = t0 + j;
        s[j] = t < n ? key_idx{k[t], static_cast<long long>(t)} : key_idx{LLONG_MAX, INT_MAX};
    }
    __syncthreads();
    for (uint32_t size = 2; size <= kRun; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t j = threadIdx.x; j < kRun / 2u; j += blockDim.x) {
                const uint32_t lo = 2u * stride * (j / stride) + (j % stride), hi = lo + stride;
                const bool up = (lo & size) == 0u;
                const key_idx a = s[lo], b = s[hi];
                if (pair_less(b, a) == up) {
                    s[lo] = b;
                    s[hi] = a;
                }
            }
            __syncthreads();
        }
    }
    key_idx *out = runs + (static_cast<uint64_t>(c) * nb + blockIdx.x) * kRun;
    for (uint32_t j = threadIdx.x; j < kRun; j += blockDim.x) out[j] = s[j];
}

__global__ void hv_rank_kernel(const long long *__restrict__ kyz, uint32_t n, const key_idx *__restrict__ runs,
                               uint32_t nb, int32_t *__restrict__ rank)
{
    const uint32_t c = blockIdx.y;
    const long long *k = kyz + static_cast<uint64_t>(c) * n;
    const key_idx *rc = runs + static_cast<uint64_t>(c) * nb * kRun;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const key_idx x{k[t], static_cast<long long>(t)};
        uint32_t r = 0;
        for (uint32_t b = 0; b < nb; ++b) {
            const key_idx *run = rc + static_cast<uint64_t>(b) * kRun;
            uint32_t pos = 0;
#pragma unroll
            for (uint32_t step = kRun / 2u; step > 0; step >>= 1)
                if (pair_less(run[pos + step - 1u], x)) pos += step;
            r += pos + (pair_less(run[pos], x) ? 1u : 0u) * (pos == kRun - 1u ? 1u : 0u);
        }
        rank[static_cast<uint64_t>(c) * n + t] = static_cast<int32_t>(r);
    }
}

// points into y order: ys and, for 2D, the widths r_x - x as bits; for 3D
// the 32-bit width keys (n - 1 - the x rank: a larger key never has a smaller
// width) beside the z ranks, the widths as doubles, and the z values in z
// order
__global__ void hv_scatter_kernel(const double *__restrict__ pts, uint32_t n, uint32_t m, double rx,
                                  const int32_t *__restrict__ rank, double *__restrict__ ys,
                                  long long *__restrict__ wbits, int2 *__restrict__ wk, double *__restrict__ wv,
                                  double *__restrict__ zs)
{
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const double *p = pts + static_cast<uint64_t>(t) * m;
        const int32_t ry = rank[t];
        ys[ry] = p[1];
        const double w = rx - p[0];
        if (m == 3u) {
            const int32_t rz = rank[static_cast<uint64_t>(n) + t], rxk = rank[2ull * n + t];
            wk[ry] = make_int2(static_cast<int>(n) - 1 - rxk, rz);
            wv[ry] = w;
            zs[rz] = p[2];
        } else {
            wbits[ry] = __double_as_longlong(w);
        }
    }
}

__device__ __forceinline__ long long warp_incl_max(long long v)
{
    const unsigned lane = threadIdx.x & 31u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long u = __shfl_up_sync(kFull, v, o);
        if (static_cast<int>(lane) >= o && u > v) v = u;
    }
    return v;
}

// 2D, one warp: A = sum_t (y_{t+1} - y_t) * max_{t' <= t} w[t'] over the points
// in y order (y_n = r_y). The running maximum W changes only at "records" (a
// point widening the staircase), so A is summed run by run, W_run * (y at the
// next record - y at this record), the last run ending at r_y: two FP64
// operations per record instead of two per point.
__global__ void hv_area2_kernel(const double *__restrict__ ys, const long long *__restrict__ wbits, uint32_t n,
                                double ry, double *__restrict__ out)
{
    const unsigned lane = threadIdx.x & 31u;
    long long carry = 0;               // bits of the running maximum so far (+0.0: no point yet)
    double pend_w = 0.0, pend_y = 0.0; // the open run: its width and where it starts
    double a = 0.0;
    for (uint32_t t0 = 0; t0 < n; t0 += 32u) {
        const uint32_t t = t0 + lane;
        const bool valid = t < n;
        long long v = valid ? wbits[t] : 0;
        v = warp_incl_max(v);
        if (carry > v) v = carry;
        long long prev = __shfl_up_sync(kFull, v, 1);
        if (lane == 0) prev = carry;
        const bool rec = valid && v != prev;
        const uint32_t b = __ballot_sync(kFull, rec);
        if (b) {
            const double y = rec ? ys[t] : 0.0;
            const double w = __longlong_as_double(v);
            const uint32_t nb = b & ~((2u << lane) - 1u); // records after this lane
            const double ynx = __shfl_sync(kFull, y, nb ? __ffs(nb) - 1 : static_cast<int>(lane));
            if (rec && nb) a = fma(w, ynx - y, a);
            if (static_cast<int>(lane) == __ffs(b) - 1 && pend_w > 0.0) a = fma(pend_w, y - pend_y, a);
            const int last = 31 - __clz(b);
            pend_w = __shfl_sync(kFull, w, last);
            pend_y = __shfl_sync(kFull, y, last);
        }
        carry = __shfl_sync(kFull, v, 31);
    }
    if (lane == 0 && pend_w > 0.0) a = fma(pend_w, ry - pend_y, a);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(kFull, a, o);
    if (lane == 0) *out = a;
}

// 3D: one thread per level i (the points of z rank <= i), the points in y
// order staged through shared memory for the whole block (asynchronous
// copies, two tiles in flight): the same run-by-run sum as the 2D kernel,
// with a warp covering 32 levels per point (a record, a point widening the
// staircase, costs one FMA on its own lane).
constexpr int kLevelThreads = 64;
constexpr uint32_t kLevelTile = 1024;

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(static_cast<unsigned>(__cvta_generic_to_shared(smem))),
                 "l"(gmem));
}

__global__ void __launch_bounds__(kLevelThreads)
    hv_levels3_kernel(const double *__restrict__ ys, const int2 *__restrict__ wk, const double *__restrict__ wv,
                      const double *__restrict__ zs, uint32_t n, double ry, double rz, double *__restrict__ term)
{
    __shared__ __align__(16) int2 s_k[2][kLevelTile]; // read two entries at a time (16-byte loads)
    __shared__ double s_y[2][kLevelTile];
    __shared__ double s_w[2][kLevelTile];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lim = i < n ? static_cast<int>(i) : -1; // z rank <= i
    int v = -1;                                       // running maximum width key (-1: no point yet)
    double pend_w = 0.0, pend_y = 0.0, a = 0.0;
    const uint32_t tiles = (n + kLevelTile - 1u) / kLevelTile;
    auto stage = [&](uint32_t t, uint32_t buf) {
        const uint32_t t0 = t * kLevelTile;
        const uint32_t cnt = n - t0 < kLevelTile ? n - t0 : kLevelTile;
        for (uint32_t j = threadIdx.x; j < cnt; j += blockDim.x) {
            cp_async8(&s_k[buf][j], wk + t0 + j);
            cp_async8(&s_y[buf][j], ys + t0 + j);
            cp_async8(&s_w[buf][j], wv + t0 + j);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    stage(0u, 0u);
    for (uint32_t t = 0; t < tiles; ++t) {
        const uint32_t buf = t & 1u;
        if (t + 1u < tiles) {
            stage(t + 1u, buf ^ 1u);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        const uint32_t cnt = n - t * kLevelTile < kLevelTile ? n - t * kLevelTile : kLevelTile;
        const int4 *k2 = reinterpret_cast<const int4 *>(s_k[buf]); // two points per 16-byte load
        // four points per warp-uniform test; the records inside are rare
        for (uint32_t j = 0; j < cnt; j += 4u) {
            const int4 e01 = k2[j >> 1], e23 = k2[(j >> 1) + 1u]; // staged past cnt: masked below
            int c[4];
            c[0] = e01.y <= lim ? e01.x : -1;
            c[1] = (j + 1u < cnt && e01.w <= lim) ? e01.z : -1;
            c[2] = (j + 2u < cnt && e23.y <= lim) ? e23.x : -1;
            c[3] = (j + 3u < cnt && e23.w <= lim) ? e23.z : -1;
            const int mx = max(max(c[0], c[1]), max(c[2], c[3]));
            if (__any_sync(kFull, mx > v)) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (c[q] > v) {
                        const double y = s_y[buf][j + q];
                        if (pend_w > 0.0) a = fma(pend_w, y - pend_y, a);
                        pend_w = s_w[buf][j + q];
                        pend_y = y;
                        v = c[q];
                    }
                }
            }
        }
        __syncthreads(); // the buffer is staged again two tiles on
    }
    if (i < n) {
        if (pend_w > 0.0) a = fma(pend_w, ry - pend_y, a);
        const double dz = (i + 1u < n ? zs[i + 1u] : rz) - zs[i];
        term[i] = dz == 0.0 ? 0.0 : dz * a;
    }
}

// out = sum of term[0 .. L) in a fixed tree (one block)
__global__ void hv_sum_kernel(const double *__restrict__ term, uint32_t L, double *__restrict__ out)
{
    __shared__ double part[1024];
    double s = 0.0;
    for (uint32_t i = threadIdx.x; i < L; i += blockDim.x) s += term[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (unsigned h = blockDim.x / 2u; h > 0; h >>= 1) {
        if (threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = part[0];
}

// hypervolume::verify_after_construct and verify_before_compute with
// hv_algorithm::assert_minimisation (src/utils/hypervolume.cpp:406-449,
// src/utils/hv_algos/hv_algorithm.cpp:226-258), on host data.
int hv_check(const double *pts, uint64_t n, uint64_t m, const double *r)
{
    PGX_CHECK(n > 0u, PGX_ERR_INVALID, "Point set cannot be empty.");
    PGX_CHECK(m > 1u, PGX_ERR_INVALID, "Points of dimension > 1 required.");
    for (uint64_t i = 0; i < n * m; ++i)
        PGX_CHECK(!std::isnan(pts[i]), PGX_ERR_INVALID,
                  "A nan value has been encountered in the hypervolume points. Cannot construct the hypervolume object");
    PGX_CHECK(m <= kWfgMaxObjectives, PGX_ERR_NOTIMPL,
              "hypervolume on the GPU: at most " + std::to_string(kWfgMaxObjectives) + " objectives; " +
                  std::to_string(m) + " given");
    for (uint64_t i = 0; i < n; ++i) {
        bool outside = false, all_equal = true;
        for (uint64_t k = 0; k < m; ++k) {
            outside |= r[k] < pts[i * m + k];
            all_equal &= r[k] == pts[i * m + k];
        }
        if (outside || all_equal) {
            std::string sp("("), sr("(");
            for (uint64_t k = 0; k < m; ++k) {
                sp += std::to_string(pts[i * m + k]);
                sr += std::to_string(r[k]);
                sp += k + 1 < m ? ", " : ")";
                sr += k + 1 < m ? ", " : ")";
            }
            std::ostringstream ss;
            ss << "Reference point is invalid: another point seems to be outside the reference point boundary, or "
                  "be equal to it:"
               << std::endl
               << " P[" << i << "]\t= " << sp << std::endl
               << " R\t= " << sr << std::endl;
            set_error(ss.str());
            return PGX_ERR_INVALID;
        }
    }
    return PGX_OK;
}

size_t align256(size_t b)
{
    return (b + 255u) & ~size_t(255);
}

// All kernels on stream s over device points; *d_out receives the volume
// (4 or more objectives: hvwfg, hv_wfg.cu).
int launch_hypervolume(pgx_context *ctx, const double *d_pts, uint32_t n, uint32_t m, const double *r,
                       double *d_out, cudaStream_t s)
{
    if (m >= 4u) return launch_wfg_compute(ctx, d_pts, n, m, r, d_out, s);
    const uint32_t nc = m == 3u ? 3u : 1u; // coordinates ranked: y (and z, x for 3D)
    const int sms = ctx->num_sms;
    const int g1 = static_cast<int>(std::min<uint64_t>((n + 255u) / 256u, static_cast<uint64_t>(sms) * 8u));
    const uint32_t nb = (n + kRun - 1u) / kRun; // sorted runs per coordinate
    const size_t b_keys = align256(static_cast<size_t>(n) * nc * 8u);
    const size_t b_rank = align256(static_cast<size_t>(n) * nc * 4u);
    const size_t b_runs = align256(static_cast<size_t>(nb) * kRun * nc * sizeof(key_idx));
    const size_t b_d = align256(static_cast<size_t>(n) * 8u);
    PGX_TRY(ctx->s_crowd.ensure(b_keys + b_rank + b_runs + 6u * b_d + 256u));
    char *base = ctx->s_crowd.as<char>();
    long long *kyz = reinterpret_cast<long long *>(base);
    int32_t *rank = reinterpret_cast<int32_t *>(base + b_keys);
    key_idx *runs = reinterpret_cast<key_idx *>(base + b_keys + b_rank);
    char *arr = base + b_keys + b_rank + b_runs; // six arrays of n doubles
    double *ys = reinterpret_cast<double *>(arr);
    long long *wbits = reinterpret_cast<long long *>(arr + b_d);
    double *zs = reinterpret_cast<double *>(arr + 2u * b_d);
    double *term = reinterpret_cast<double *>(arr + 3u * b_d);
    int2 *wk = reinterpret_cast<int2 *>(arr + 4u * b_d);
    double *wv = reinterpret_cast<double *>(arr + 5u * b_d);
    hv_keys_kernel<<<g1, 256, 0, s>>>(d_pts, n, m, kyz);
    PGX_CUDA(cudaGetLastError());
    hv_runs_kernel<<<dim3(nb, nc), 1024, 0, s>>>(kyz, n, runs);
    PGX_CUDA(cudaGetLastError());
    hv_rank_kernel<<<dim3(static_cast<unsigned>((n + 127u) / 128u), nc), 128, 0, s>>>(kyz, n, runs, nb, rank);
    PGX_CUDA(cudaGetLastError());
    hv_scatter_kernel<<<g1, 256, 0, s>>>(d_pts, n, m, r[0], rank, ys, wbits, m == 3u ? wk : nullptr,
                                         m == 3u ? wv : nullptr, m == 3u ? zs : nullptr);
    PGX_CUDA(cudaGetLastError());
    if (m == 3u) {
        const int g3 = static_cast<int>((n + kLevelThreads - 1u) / kLevelThreads);
        hv_levels3_kernel<<<g3, kLevelThreads, 0, s>>>(ys, wk, wv, zs, n, r[1], r[2], term);
        PGX_CUDA(cudaGetLastError());
        hv_sum_kernel<<<1, 1024, 0, s>>>(term, n, d_out);
    } else {
        hv_area2_kernel<<<1, 32, 0, s>>>(ys, wbits, n, r[1], d_out);
    }
    PGX_CUDA(cudaGetLastError());
    ctx->launches += m == 3u ? 6 : 5;
    return PGX_OK;
}

// *out = a - b
__global__ void hv_sub_kernel(const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ out)
{
    if (threadIdx.x == 0) *out = __dsub_rn(*a, *b);
}

// *idx = the first index of the smallest (greatest = 0) or largest
// (greatest = 1) of c[0 .. n): hv_algorithm::extreme_contributor's strict
// scan from index 0 (hv_algorithm.cpp:329-349), as a reduction that prefers
// the lower index on ties.
__global__ void __launch_bounds__(1024) hv_extreme_kernel(const double *__restrict__ c, uint32_t n, int greatest,
                                                          unsigned long long *__restrict__ idx)
{
    __shared__ double sv[1024];
    __shared__ uint32_t si[1024];
    double best = 0.0;
    uint32_t bi = UINT32_MAX;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = c[i];
        if (bi == UINT32_MAX || (greatest ? v > best : v < best)) {
            best = v;
            bi = i;
        }
    }
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    for (unsigned h = blockDim.x / 2u; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            const double v = sv[threadIdx.x + h];
            const uint32_t j = si[threadIdx.x + h];
            const uint32_t i = si[threadIdx.x];
            const bool take = j != UINT32_MAX &&
                              (i == UINT32_MAX || (greatest ? v > sv[threadIdx.x] : v < sv[threadIdx.x]) ||
                               (v == sv[threadIdx.x] && j < i));
            if (take) {
                sv[threadIdx.x] = v;
                si[threadIdx.x] = j;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *idx = si[0];
}

// The checks of hypervolume's construction and compute on host data, the
// point count and the device, then the points on the device (s_points):
// returns their address; tail_bytes more are reserved after them.
int upload_points(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, const double *ref,
                  size_t tail_bytes, double **dp, char **tail)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK((points != nullptr || n == 0) && ref != nullptr, PGX_ERR_INVALID, "null buffer");
    PGX_TRY(hv_check(points, n, m, ref));
    PGX_CHECK(n < (1u << 24), PGX_ERR_CAPACITY, "hypervolume: more than 2^24 points");
    PGX_TRY(use_device(ctx));
    const size_t bp = align256(static_cast<size_t>(n) * m * 8u);
    PGX_TRY(ctx->s_points.ensure(bp + tail_bytes));
    *dp = ctx->s_points.as<double>();
    *tail = ctx->s_points.as<char>() + bp;
    PGX_CUDA(cudaMemcpyAsync(*dp, points, static_cast<size_t>(n) * m * 8u, cudaMemcpyHostToDevice, ctx->stream));
    return PGX_OK;
}

int wfg_ok(pgx_context *ctx)
{
    unsigned st = 0;
    PGX_TRY(wfg_status(ctx, &st));
    PGX_CHECK(st == 0u, PGX_ERR_CAPACITY, "hypervolume (WFG): a warp ran out of frame buffers");
    return PGX_OK;
}

} // namespace
} // namespace pgx

using namespace pgx;

extern "C" {

int pgx_hypervolume(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, const double *ref, double *out)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(out != nullptr && (points != nullptr || n == 0) && ref != nullptr, PGX_ERR_INVALID, "null buffer");
    PGX_TRY(hv_check(points, n, m, ref));
    PGX_CHECK(n < (1u << 24), PGX_ERR_CAPACITY, "hypervolume: more than 2^24 points");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    const size_t bp = align256(static_cast<size_t>(n) * m * 8u);
    PGX_TRY(ctx->s_points.ensure(bp + 256u));
    double *dp = ctx->s_points.as<double>();
    double *dout = reinterpret_cast<double *>(ctx->s_points.as<char>() + bp);
    cudaStream_t s = ctx->stream;
    PGX_CUDA(cudaMemcpyAsync(dp, points, static_cast<size_t>(n) * m * 8u, cudaMemcpyHostToDevice, s));
    PGX_TRY(launch_hypervolume(ctx, dp, static_cast<uint32_t>(n), static_cast<uint32_t>(m), ref, dout, s));
    PGX_CUDA(cudaMemcpyAsync(out, dout, sizeof(double), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaStreamSynchronize(s));
    return PGX_OK;
}

int pgx_hypervolume_device(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m, const double *ref,
                           double *d_out, void *stream)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(d_points != nullptr && d_out != nullptr && ref != nullptr, PGX_ERR_INVALID, "null buffer");
    PGX_CHECK(n > 0u, PGX_ERR_INVALID, "Point set cannot be empty.");
    PGX_CHECK(m > 1u, PGX_ERR_INVALID, "Points of dimension > 1 required.");
    PGX_CHECK(m <= kWfgMaxObjectives, PGX_ERR_NOTIMPL,
              "hypervolume on the GPU: at most " + std::to_string(kWfgMaxObjectives) + " objectives; " +
                  std::to_string(m) + " given");
    PGX_CHECK(n < (1u << 24), PGX_ERR_CAPACITY, "hypervolume: more than 2^24 points");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    return launch_hypervolume(ctx, d_points, static_cast<uint32_t>(n), static_cast<uint32_t>(m), ref, d_out,
                              static_cast<cudaStream_t>(stream));
}

int pgx_hypervolume_exclusive(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, const double *ref,
                              uint64_t p_idx, double *out)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(out != nullptr && (points != nullptr || n == 0) && ref != nullptr, PGX_ERR_INVALID, "null buffer");
    PGX_TRY(hv_check(points, n, m, ref)); // before the index, as hypervolume::exclusive (hypervolume.cpp:251-256)
    PGX_CHECK(p_idx < n, PGX_ERR_INVALID, "Index of the individual is out of bounds.");
    std::lock_guard<std::mutex> g(ctx->lock);
    const size_t bl = align256(static_cast<size_t>(n) * m * 8u);
    double *dp = nullptr;
    char *tail = nullptr;
    PGX_TRY(upload_points(ctx, points, n, m, ref, bl + 256u, &dp, &tail));
    double *less = reinterpret_cast<double *>(tail);
    double *d3 = reinterpret_cast<double *>(tail + bl); // volume of all, of all but p_idx, their difference
    cudaStream_t s = ctx->stream;
    const auto nn = static_cast<uint32_t>(n), mm = static_cast<uint32_t>(m);
    if (n == 1u) {
        // hv_algorithm::exclusive of a lone point: the volume (hv_algorithm.cpp:96-98)
        PGX_TRY(launch_hypervolume(ctx, dp, nn, mm, ref, d3 + 2, s));
    } else {
        const size_t row = static_cast<size_t>(m) * 8u;
        if (p_idx > 0u) PGX_CUDA(cudaMemcpyAsync(less, dp, p_idx * row, cudaMemcpyDeviceToDevice, s));
        if (p_idx + 1u < n)
            PGX_CUDA(cudaMemcpyAsync(less + p_idx * m, dp + (p_idx + 1u) * m, (n - p_idx - 1u) * row,
                                     cudaMemcpyDeviceToDevice, s));
        PGX_TRY(launch_hypervolume(ctx, dp, nn, mm, ref, d3, s));
        PGX_TRY(launch_hypervolume(ctx, less, nn - 1u, mm, ref, d3 + 1, s));
        hv_sub_kernel<<<1, 32, 0, s>>>(d3, d3 + 1, d3 + 2);
        PGX_CUDA(cudaGetLastError());
        ++ctx->launches;
    }
    PGX_CUDA(cudaMemcpyAsync(out, d3 + 2, sizeof(double), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaStreamSynchronize(s));
    if (m >= 4u) PGX_TRY(wfg_ok(ctx));
    return PGX_OK;
}

int pgx_hypervolume_contributions(pgx_context *ctx, const double *points, uint64_t n, uint64_t m, const double *ref,
                                  double *out)
{
    PGX_CHECK(out != nullptr, PGX_ERR_INVALID, "null buffer");
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    std::lock_guard<std::mutex> g(ctx->lock);
    const size_t bo = align256(static_cast<size_t>(n) * 8u);
    double *dp = nullptr;
    char *tail = nullptr;
    PGX_TRY(upload_points(ctx, points, n, m, ref, bo, &dp, &tail));
    double *dc = reinterpret_cast<double *>(tail);
    PGX_TRY(launch_wfg_contributions(ctx, dp, static_cast<uint32_t>(n), static_cast<uint32_t>(m), ref, dc,
                                     ctx->stream));
    PGX_CUDA(cudaMemcpyAsync(out, dc, static_cast<size_t>(n) * 8u, cudaMemcpyDeviceToHost, ctx->stream));
    return wfg_ok(ctx);
}

int pgx_hypervolume_contributions_device(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m,
                                         const double *ref, double *d_out, void *stream)
{
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    PGX_CHECK(d_points != nullptr && d_out != nullptr && ref != nullptr, PGX_ERR_INVALID, "null buffer");
    PGX_CHECK(n > 0u, PGX_ERR_INVALID, "Point set cannot be empty.");
    PGX_CHECK(m > 1u, PGX_ERR_INVALID, "Points of dimension > 1 required.");
    PGX_CHECK(m <= kWfgMaxObjectives, PGX_ERR_NOTIMPL,
              "hypervolume on the GPU: at most " + std::to_string(kWfgMaxObjectives) + " objectives; " +
                  std::to_string(m) + " given");
    PGX_CHECK(n < (1u << 24), PGX_ERR_CAPACITY, "hypervolume: more than 2^24 points");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    return launch_wfg_contributions(ctx, d_points, static_cast<uint32_t>(n), static_cast<uint32_t>(m), ref, d_out,
                                    static_cast<cudaStream_t>(stream));
}

int pgx_hypervolume_extreme_contributor(pgx_context *ctx, const double *points, uint64_t n, uint64_t m,
                                        const double *ref, int greatest, uint64_t *idx)
{
    PGX_CHECK(idx != nullptr, PGX_ERR_INVALID, "null buffer");
    PGX_CHECK(ctx != nullptr, PGX_ERR_INVALID, "null context");
    std::lock_guard<std::mutex> g(ctx->lock);
    const size_t bo = align256(static_cast<size_t>(n) * 8u);
    double *dp = nullptr;
    char *tail = nullptr;
    PGX_TRY(upload_points(ctx, points, n, m, ref, bo + 256u, &dp, &tail));
    if (n == 1u) { // hypervolume.cpp:339-342, hv_algorithm.cpp:332-335
        *idx = 0;
        return PGX_OK;
    }
    double *dc = reinterpret_cast<double *>(tail);
    auto *di = reinterpret_cast<unsigned long long *>(tail + bo);
    cudaStream_t s = ctx->stream;
    PGX_TRY(launch_wfg_contributions(ctx, dp, static_cast<uint32_t>(n), static_cast<uint32_t>(m), ref, dc, s));
    hv_extreme_kernel<<<1, 1024, 0, s>>>(dc, static_cast<uint32_t>(n), greatest ? 1 : 0, di);
    PGX_CUDA(cudaGetLastError());
    ++ctx->launches;
    unsigned long long h = 0;
    PGX_CUDA(cudaMemcpyAsync(&h, di, sizeof(h), cudaMemcpyDeviceToHost, s));
    PGX_TRY(wfg_ok(ctx));
    *idx = h;
    return PGX_OK;
}

} // extern "C"
