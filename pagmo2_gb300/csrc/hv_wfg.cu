// WFG hypervolume on the GPU: pagmo's hvwfg with stop dimension 2
// (src/utils/hv_algos/hv_hvwfg.cpp), the algorithm hypervolume::compute picks
// for 4 or more objectives and hypervolume::contributions for 4 or more
// (src/utils/hypervolume.cpp:488-537); hv3d's contributions fall back to it
// (hv_hv3d.cpp:229-231), hv2d's run hv3d on the points with a third
// coordinate 0 and a reference 1 (hv_hv2d.cpp:133-146).
//
// The recursion, per frame of k points in d coordinates (hv_hvwfg.cpp:196-272):
//   k = 1: vol(p) = |prod over c = d-1 .. 0 of (r_c - p_c)|;
//   k = 2: vol(p0) + vol(p1) - prod over c = 0 .. d-1 of (r_c - max(p0_c, p1_c));
//   d = 2: hv2d's sweep over the points sorted by the second coordinate;
//   else: the frame sorted by hvwfg::cmp_points (descending, last coordinate
//   first) and H += |(p_j[d-1] - r_{d-1}) * (vol_{d-1}(p_j) - hv(L_j))| in
//   that order, L_j the limit set of p_j over the points after it: max(q, p_j)
//   over the first d-1 coordinates, non-dominated, one copy of equal points
//   (hvwfg::limitset, hv_hvwfg.cpp:134-193).
// A point's contribution is vol_m(p) - hv(limit set of p over every other
// point, m coordinates) (hvwfg::contributions, hv_hvwfg.cpp:79-105); the
// volume is the sum, in sorted order, of the top level's terms.
//
// GPU layout: one warp per top-level term (compute) or per point
// (contributions), taken from a work counter in index order (the early terms
// of the sorted set have the most candidates). The warp's lanes share the
// limit-set filter (32 candidates at a time against the kept set, then
// against each other, then the kept points the survivors cover are removed),
// the counting-rank sorts of a frame and the closed forms; the recursion
// below the top level runs on an explicit stack, its frames in the warp's
// slice of a scratch pool (m buffers of n rows). A frame's kept set is the
// unique non-dominated subset of its candidates whatever order they are
// filtered in, every frame of more than two points is sorted by a strict
// order before it is used, and the two-point form is symmetric, so the
// arithmetic is the reference's: every operation is the reference's
// IEEE double operation in the reference's order (explicit round-to-nearest
// intrinsics: no contraction into FMA), and the volumes and contributions
// equal the reference's bit for bit.
#include "pgx_internal.cuh"

#include <algorithm>

namespace pgx
{
namespace
{

constexpr unsigned kMask = 0xffffffffu;
constexpr int kWarpsPerBlock = 4;

struct wfg_ref {
    double r[kWfgMaxObjectives];
};

__device__ __forceinline__ double std_max(double a, double b)
{
    return a < b ? b : a; // std::max(a, b)
}

// |prod over c = d-1 .. 0 of (r_c - p_c)| (hv_algorithm::volume_between on
// pointers, hv_algorithm.cpp:73-82)
__device__ __forceinline__ double vol(const double *r, const double *p, uint32_t d)
{
    double v = 1.0;
    for (int c = static_cast<int>(d) - 1; c >= 0; --c) v = __dmul_rn(v, __dsub_rn(r[c], p[c]));
    return v < 0.0 ? -v : v;
}

__device__ __forceinline__ unsigned lanes_below(unsigned lane)
{
    return (1u << lane) - 1u;
}

// The limit set of p over the rows t of src in [begin, end), t != skip
// (stride src_stride): max(row, p) over the first dc coordinates, filtered to
// the non-dominated ones with one copy of equal points, written to dst
// (stride dc). Returns the number kept. Warp-uniform arguments.
template <int DM>
__device__ uint32_t limit_set(const double *src, uint32_t src_stride, uint32_t begin, uint32_t end, uint32_t skip,
                              const double *p, uint32_t dc, double *dst, unsigned lane)
{
    uint32_t K = 0;
    for (uint32_t base = begin; base < end; base += 32u) {
        const uint32_t t = base + lane;
        const bool valid = t < end && t != skip;
        double s[DM];
#pragma unroll
        for (int c = 0; c < DM; ++c)
            s[c] = (valid && c < static_cast<int>(dc)) ? std_max(src[static_cast<uint64_t>(t) * src_stride + c], p[c])
                                                       : 0.0;
        bool alive = valid;
        // a kept point <= s in every coordinate (dominating or equal): s goes
        for (uint32_t q = 0; q < K; ++q) {
            if (!__any_sync(kMask, alive)) break;
            const double *kq = dst + static_cast<uint64_t>(q) * dc;
            bool le = true;
#pragma unroll
            for (int c = 0; c < DM; ++c)
                if (c < static_cast<int>(dc)) le &= kq[c] <= s[c];
            alive &= !le;
        }
        // within the batch: a live candidate that dominates s, or equals it
        // from a higher lane (a candidate a kept point removed is no witness
        // needed: that kept point also covers whatever it dominates)
        const unsigned live = __ballot_sync(kMask, alive);
        if (__popc(live) > 1) {
            for (unsigned rest = live; rest; rest &= rest - 1u) {
                const int u = __ffs(rest) - 1;
                bool le = true, lt = false;
#pragma unroll
                for (int c = 0; c < DM; ++c) {
                    if (c < static_cast<int>(dc)) {
                        const double su = __shfl_sync(kMask, s[c], u);
                        le &= su <= s[c];
                        lt |= su < s[c];
                    }
                }
                if (u != static_cast<int>(lane) && le && (lt || u > static_cast<int>(lane))) alive = false;
            }
        }
        const unsigned surv = __ballot_sync(kMask, alive);
        if (surv == 0u) continue;
        // the kept points a survivor covers go (in place, order kept), the
        // survivors are appended
        uint32_t nk = 0;
        for (uint32_t c0 = 0; c0 < K; c0 += 32u) {
            const uint32_t q = c0 + lane;
            const bool has = q < K;
            double qr[DM];
#pragma unroll
            for (int c = 0; c < DM; ++c)
                qr[c] = (has && c < static_cast<int>(dc)) ? dst[static_cast<uint64_t>(q) * dc + c] : 0.0;
            bool keep = has;
            for (unsigned rs = surv; rs; rs &= rs - 1u) {
                const int u = __ffs(rs) - 1;
                bool cov = true;
#pragma unroll
                for (int c = 0; c < DM; ++c)
                    if (c < static_cast<int>(dc)) cov &= __shfl_sync(kMask, s[c], u) <= qr[c];
                keep &= !cov;
            }
            const unsigned km = __ballot_sync(kMask, keep);
            __syncwarp();
            if (keep) {
                double *o = dst + static_cast<uint64_t>(nk + __popc(km & lanes_below(lane))) * dc;
#pragma unroll
                for (int c = 0; c < DM; ++c)
                    if (c < static_cast<int>(dc)) o[c] = qr[c];
            }
            nk += __popc(km);
            __syncwarp();
        }
        if (alive) {
            double *o = dst + static_cast<uint64_t>(nk + __popc(surv & lanes_below(lane))) * dc;
#pragma unroll
            for (int c = 0; c < DM; ++c)
                if (c < static_cast<int>(dc)) o[c] = s[c];
        }
        K = nk + __popc(surv);
        __syncwarp();
    }
    return K;
}

// Rows of src (K rows of d) into dst in order: by_y = false, hvwfg::cmp_points
// (descending, last coordinate first: hv_hvwfg.cpp:276-286); by_y = true,
// ascending second coordinate (hv2d, hv_hv2d.cpp:79-81). Ties by row index
// (a frame's rows are distinct, so they never decide an order there).
template <int DM>
__device__ void sort_rows(const double *src, uint32_t K, uint32_t d, bool by_y, double *dst, unsigned lane)
{
    for (uint32_t i0 = 0; i0 < K; i0 += 32u) {
        const uint32_t i = i0 + lane;
        const bool has = i < K;
        double mine[DM];
#pragma unroll
        for (int c = 0; c < DM; ++c)
            mine[c] = (has && c < static_cast<int>(d)) ? src[static_cast<uint64_t>(i) * d + c] : 0.0;
        uint32_t rank = 0;
        for (uint32_t j = 0; j < K; ++j) {
            const double *rj = src + static_cast<uint64_t>(j) * d;
            int dec = 0; // +1: row j first, -1: this row first
            if (by_y) {
                const double a = rj[1];
                dec = a < mine[1] ? 1 : (a > mine[1] ? -1 : 0);
            } else {
#pragma unroll
                for (int c = DM - 1; c >= 0; --c) {
                    if (c < static_cast<int>(d) && dec == 0) {
                        const double a = rj[c];
                        dec = a > mine[c] ? 1 : (a < mine[c] ? -1 : 0);
                    }
                }
            }
            rank += (dec > 0 || (dec == 0 && j < i)) ? 1u : 0u;
        }
        if (has) {
            double *o = dst + static_cast<uint64_t>(rank) * d;
#pragma unroll
            for (int c = 0; c < DM; ++c)
                if (c < static_cast<int>(d)) o[c] = mine[c];
        }
    }
    __syncwarp();
}

// The frames of a warp: m buffers of bd doubles, taken and given back by bit.
struct frame_pool {
    double *base;
    uint64_t bd;
    unsigned free;

    __device__ int take()
    {
        if (free == 0u) return -1;
        const int b = __ffs(free) - 1;
        free &= ~(1u << b);
        return b;
    }
    __device__ void give(int b)
    {
        free |= 1u << b;
    }
    __device__ double *at(int b) const
    {
        return base + static_cast<uint64_t>(b) * bd;
    }
};

// hv of a frame of 1 or 2 points, or of 2 coordinates (tmp: a free buffer
// for the sort by y when k > 2)
template <int DM>
__device__ double closed_form(const double *r, const double *f, uint32_t K, uint32_t d, double *tmp, unsigned lane)
{
    if (K == 1u) return vol(r, f, d);
    if (K == 2u) {
        const double h = __dadd_rn(vol(r, f, d), vol(r, f + d, d));
        double isect = 1.0;
        for (uint32_t c = 0; c < d; ++c) isect = __dmul_rn(isect, __dsub_rn(r[c], std_max(f[c], f[d + c])));
        return __dsub_rn(h, isect);
    }
    sort_rows<DM>(f, K, 2u, true, tmp, lane);
    double area = 0.0, w = __dsub_rn(r[0], tmp[0]);
    for (uint32_t t = 0; t + 1u < K; ++t) {
        area = __dadd_rn(area, __dmul_rn(__dsub_rn(tmp[2u * (t + 1u) + 1u], tmp[2u * t + 1u]), w));
        w = std_max(w, __dsub_rn(r[0], tmp[2u * (t + 1u)]));
    }
    return __dadd_rn(area, __dmul_rn(__dsub_rn(r[1], tmp[2u * (K - 1u) + 1u]), w));
}

// |(p[d-1] - r[d-1]) * ex|, the term a point of a frame of d coordinates adds
__device__ __forceinline__ double slice_term(const double *r, const double *p, uint32_t d, double ex)
{
    return fabs(__dmul_rn(__dsub_rn(p[d - 1u], r[d - 1u]), ex));
}

// hv of the frame in buffer `buf` (K points of d coordinates, K >= 1); the
// frame's buffer and every buffer taken below are given back. *fail is set
// when the pool runs dry (it cannot: a level holds one buffer, a sort or the
// sweep one more, and there are at most m - 1 levels).
template <int DM>
__device__ double frame_hv(const double *r, frame_pool &pool, int buf, uint32_t K, uint32_t d, unsigned lane,
                           bool *fail)
{
    int st_buf[DM];
    uint32_t st_k[DM], st_d[DM];
    int st_j[DM];
    double st_h[DM];
    int sp = 0;
    st_buf[0] = buf;
    st_k[0] = K;
    st_d[0] = d;
    st_j[0] = -1;
    st_h[0] = 0.0;
    for (;;) {
        const int j = st_j[sp];
        const uint32_t kk = st_k[sp], dd = st_d[sp];
        const double *f = pool.at(st_buf[sp]);
        double val;
        if (j < 0) {
            if (kk <= 2u || dd == 2u) {
                int tb = -1;
                if (kk > 2u && (tb = pool.take()) < 0) {
                    *fail = true;
                    return 0.0;
                }
                val = closed_form<DM>(r, f, kk, dd, tb >= 0 ? pool.at(tb) : nullptr, lane);
                if (tb >= 0) pool.give(tb);
            } else {
                const int sb = pool.take();
                if (sb < 0) {
                    *fail = true;
                    return 0.0;
                }
                sort_rows<DM>(f, kk, dd, false, pool.at(sb), lane);
                pool.give(st_buf[sp]);
                st_buf[sp] = sb;
                st_j[sp] = 0;
                st_h[sp] = 0.0;
                continue;
            }
        } else if (static_cast<uint32_t>(j) < kk) {
            const double *p = f + static_cast<uint64_t>(j) * dd;
            const int cb = pool.take();
            if (cb < 0) {
                *fail = true;
                return 0.0;
            }
            double *child = pool.at(cb);
            const uint32_t ck = limit_set<DM>(f, dd, static_cast<uint32_t>(j) + 1u, kk, kk, p, dd - 1u, child, lane);
            if (ck <= 1u) {
                double ex = vol(r, p, dd - 1u);
                if (ck == 1u) ex = __dsub_rn(ex, vol(r, child, dd - 1u));
                pool.give(cb);
                st_h[sp] = __dadd_rn(st_h[sp], slice_term(r, p, dd, ex));
                st_j[sp] = j + 1;
                continue;
            }
            ++sp;
            st_buf[sp] = cb;
            st_k[sp] = ck;
            st_d[sp] = dd - 1u;
            st_j[sp] = -1;
            st_h[sp] = 0.0;
            continue;
        } else {
            val = st_h[sp];
        }
        // level sp is done with value val: its parent's term j completes
        pool.give(st_buf[sp]);
        if (sp == 0) return val;
        --sp;
        const uint32_t pd = st_d[sp];
        const int pj = st_j[sp];
        const double *p = pool.at(st_buf[sp]) + static_cast<uint64_t>(pj) * pd;
        st_h[sp] = __dadd_rn(st_h[sp], slice_term(r, p, pd, __dsub_rn(vol(r, p, pd - 1u), val)));
        st_j[sp] = pj + 1;
    }
}

struct wfg_args {
    const double *pts;  // n rows of m; sorted by cmp_points for the terms of a volume
    uint32_t n, m;
    int contributions;  // 0: out[i] = the top-level term of sorted point i; 1: the contribution of point i
    double *out;        // n
    double *pool;       // per warp: m buffers of bd doubles
    uint64_t bd;
    unsigned *next;     // work counter (zero at launch)
    unsigned *status;   // set when a warp's pool ran dry
};

template <int DM>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) wfg_kernel(wfg_args a, wfg_ref ref)
{
    __shared__ double s_r[DM];
    if (threadIdx.x < DM) s_r[threadIdx.x] = threadIdx.x < a.m ? ref.r[threadIdx.x] : 0.0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t gw = static_cast<uint64_t>(blockIdx.x) * kWarpsPerBlock + (threadIdx.x >> 5);
    const uint32_t m = a.m;
    const uint32_t dc = a.contributions ? m : m - 1u; // coordinates of the first frame
    frame_pool pool{a.pool + gw * m * a.bd, a.bd, (1u << m) - 1u};
    for (;;) {
        unsigned item = 0;
        if (lane == 0) item = atomicAdd(a.next, 1u);
        item = __shfl_sync(kMask, item, 0);
        if (item >= a.n) break;
        const double *p = a.pts + static_cast<uint64_t>(item) * m;
        const int b0 = pool.take(); // the pool is full here
        const uint32_t k0 = a.contributions ? limit_set<DM>(a.pts, m, 0u, a.n, item, p, dc, pool.at(b0), lane)
                                            : limit_set<DM>(a.pts, m, item + 1u, a.n, a.n, p, dc, pool.at(b0), lane);
        double ex = vol(s_r, p, dc);
        bool fail = false;
        if (k0 == 0u) {
            pool.give(b0);
        } else {
            ex = __dsub_rn(ex, frame_hv<DM>(s_r, pool, b0, k0, dc, lane, &fail));
        }
        if (fail) {
            if (lane == 0) {
                atomicOr(a.status, 1u);
                a.out[item] = __longlong_as_double(0x7ff8000000000000LL);
            }
            pool.free = (1u << m) - 1u;
            continue;
        }
        if (lane == 0) a.out[item] = a.contributions ? ex : slice_term(s_r, p, m, ex);
    }
}

// Ranks of the points by hvwfg::cmp_points over m coordinates (ties by index)
// and the points written in that order: one thread per point, the others
// staged through shared memory.
constexpr int kRankThreads = 128;

__global__ void __launch_bounds__(kRankThreads)
    wfg_sort_points_kernel(const double *__restrict__ pts, uint32_t n, uint32_t m, double *__restrict__ sorted)
{
    __shared__ double tile[kRankThreads * kWfgMaxObjectives];
    const uint32_t i = blockIdx.x * kRankThreads + threadIdx.x;
    double mine[kWfgMaxObjectives];
    for (uint32_t c = 0; c < m; ++c) mine[c] = i < n ? pts[static_cast<uint64_t>(i) * m + c] : 0.0;
    uint32_t rank = 0;
    for (uint32_t j0 = 0; j0 < n; j0 += kRankThreads) {
        const uint32_t cnt = min(static_cast<uint32_t>(kRankThreads), n - j0);
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < cnt * m; e += kRankThreads)
            tile[e] = pts[static_cast<uint64_t>(j0) * m + e];
        __syncthreads();
        if (i < n) {
            for (uint32_t jj = 0; jj < cnt; ++jj) {
                const double *rj = tile + jj * m;
                int dec = 0;
                for (int c = static_cast<int>(m) - 1; c >= 0 && dec == 0; --c)
                    dec = rj[c] > mine[c] ? 1 : (rj[c] < mine[c] ? -1 : 0);
                rank += (dec > 0 || (dec == 0 && j0 + jj < i)) ? 1u : 0u;
            }
        }
    }
    if (i < n)
        for (uint32_t c = 0; c < m; ++c) sorted[static_cast<uint64_t>(rank) * m + c] = mine[c];
}

// out = the sum of term[0 .. n) in index order from 0.0 (compute_hv's
// H += ..., hv_hvwfg.cpp:262-266)
__global__ void wfg_sum_kernel(const double *__restrict__ term, uint32_t n, double *__restrict__ out)
{
    if (threadIdx.x != 0) return;
    double h = 0.0;
    for (uint32_t i = 0; i < n; ++i) h = __dadd_rn(h, term[i]);
    *out = h;
}

// The volume of one or two points (compute_hv's inclusion-exclusion,
// hv_hvwfg.cpp:201-211) and, with contribution_of_one, hypervolume's
// contribution of a lone point: |prod over c = 0 .. m-1 of (p_c - r_c)|
// (hypervolume.cpp:303-307 with volume_between on vectors,
// hv_algorithm.cpp:61-71).
__global__ void wfg_small_kernel(const double *__restrict__ pts, uint32_t n, uint32_t m, wfg_ref ref,
                                 int contribution_of_one, double *__restrict__ out)
{
    if (threadIdx.x != 0) return;
    const double *r = ref.r;
    if (contribution_of_one) {
        double v = 1.0;
        for (uint32_t c = 0; c < m; ++c) v = __dmul_rn(v, __dsub_rn(pts[c], r[c]));
        *out = v < 0.0 ? -v : v;
        return;
    }
    if (n == 1u) {
        *out = vol(r, pts, m);
        return;
    }
    const double h = __dadd_rn(vol(r, pts, m), vol(r, pts + m, m));
    double isect = 1.0;
    for (uint32_t c = 0; c < m; ++c) isect = __dmul_rn(isect, __dsub_rn(r[c], std_max(pts[c], pts[m + c])));
    *out = __dsub_rn(h, isect);
}

// 2-objective points as hv2d::contributions hands them to hv3d: a third
// coordinate 0 (hv_hv2d.cpp:135-143)
__global__ void wfg_lift2_kernel(const double *__restrict__ pts, uint32_t n, double *__restrict__ out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        out[3ull * i] = pts[2ull * i];
        out[3ull * i + 1u] = pts[2ull * i + 1u];
        out[3ull * i + 2u] = 0.0;
    }
}

size_t round256(size_t b)
{
    return (b + 255u) & ~size_t(255);
}

// Scratch of the warp kernel over n points of m coordinates: [points n*m |
// out n | counter, status | pool]; the number of warps fits the pool in
// kPoolBytes (at least one warp).
constexpr size_t kPoolBytes = size_t(1) << 30;

int run_warps(pgx_context *ctx, const double *d_pts, uint32_t n, uint32_t m, const wfg_ref &ref, int contributions,
              double *d_out, cudaStream_t s)
{
    const uint64_t bd = static_cast<uint64_t>(n) * m; // a frame: at most n rows of at most m coordinates
    const size_t per_warp = static_cast<size_t>(m) * bd * sizeof(double);
    PGX_CHECK(per_warp <= (size_t(4) << 30), PGX_ERR_CAPACITY,
              "hypervolume (WFG): " + std::to_string(n) + " points of " + std::to_string(m) +
                  " objectives need more than 4 GiB of frames per warp");
    const uint64_t want = std::min<uint64_t>(n, static_cast<uint64_t>(ctx->num_sms) * 16u);
    const uint64_t fit = std::max<uint64_t>(1u, kPoolBytes / per_warp);
    uint64_t warps = std::min(want, fit);
    const unsigned blocks = static_cast<unsigned>((warps + kWarpsPerBlock - 1u) / kWarpsPerBlock);
    warps = static_cast<uint64_t>(blocks) * kWarpsPerBlock; // every warp of the grid has its slice
    const size_t b_ctl = 256u;
    PGX_TRY(ctx->h_wfg.ensure(b_ctl + warps * per_warp));
    unsigned *ctl = ctx->h_wfg.as<unsigned>();
    PGX_CUDA(cudaMemsetAsync(ctl, 0, b_ctl, s));
    wfg_args a{};
    a.pts = d_pts;
    a.n = n;
    a.m = m;
    a.contributions = contributions;
    a.out = d_out;
    a.pool = reinterpret_cast<double *>(ctx->h_wfg.as<char>() + b_ctl);
    a.bd = bd;
    a.next = ctl;
    a.status = ctl + 1;
    if (m <= 4u) {
        wfg_kernel<4><<<blocks, kWarpsPerBlock * 32, 0, s>>>(a, ref);
    } else if (m <= 8u) {
        wfg_kernel<8><<<blocks, kWarpsPerBlock * 32, 0, s>>>(a, ref);
    } else {
        wfg_kernel<16><<<blocks, kWarpsPerBlock * 32, 0, s>>>(a, ref);
    }
    PGX_CUDA(cudaGetLastError());
    ++ctx->launches;
    return PGX_OK;
}

// A call that runs no warp kernel leaves a zero status behind.
int clear_status(pgx_context *ctx, cudaStream_t s)
{
    if (ctx->h_wfg.ptr != nullptr) PGX_CUDA(cudaMemsetAsync(ctx->h_wfg.ptr, 0, 256u, s));
    return PGX_OK;
}

wfg_ref make_ref(const double *r, uint32_t m)
{
    wfg_ref w{};
    for (uint32_t c = 0; c < m; ++c) w.r[c] = r[c];
    return w;
}

} // namespace

int launch_wfg_compute(pgx_context *ctx, const double *d_pts, uint32_t n, uint32_t m, const double *r,
                       double *d_out, cudaStream_t s)
{
    PGX_CHECK(m >= 2u && m <= kWfgMaxObjectives, PGX_ERR_NOTIMPL,
              "hypervolume on the GPU: at most " + std::to_string(kWfgMaxObjectives) + " objectives; " +
                  std::to_string(m) + " given");
    const wfg_ref ref = make_ref(r, m);
    if (n <= 2u) {
        PGX_TRY(clear_status(ctx, s));
        wfg_small_kernel<<<1, 32, 0, s>>>(d_pts, n, m, ref, 0, d_out);
        PGX_CUDA(cudaGetLastError());
        ++ctx->launches;
        return PGX_OK;
    }
    const size_t b_pts = round256(static_cast<size_t>(n) * m * sizeof(double));
    const size_t b_terms = round256(static_cast<size_t>(n) * sizeof(double));
    PGX_TRY(ctx->s_crowd.ensure(b_pts + b_terms));
    double *sorted = ctx->s_crowd.as<double>();
    double *terms = reinterpret_cast<double *>(ctx->s_crowd.as<char>() + b_pts);
    wfg_sort_points_kernel<<<(n + kRankThreads - 1u) / kRankThreads, kRankThreads, 0, s>>>(d_pts, n, m, sorted);
    PGX_CUDA(cudaGetLastError());
    PGX_TRY(run_warps(ctx, sorted, n, m, ref, 0, terms, s));
    wfg_sum_kernel<<<1, 32, 0, s>>>(terms, n, d_out);
    PGX_CUDA(cudaGetLastError());
    ctx->launches += 2;
    return PGX_OK;
}

int launch_wfg_contributions(pgx_context *ctx, const double *d_pts, uint32_t n, uint32_t m, const double *r,
                             double *d_out, cudaStream_t s)
{
    PGX_CHECK(m >= 2u && m <= kWfgMaxObjectives, PGX_ERR_NOTIMPL,
              "hypervolume on the GPU: at most " + std::to_string(kWfgMaxObjectives) + " objectives; " +
                  std::to_string(m) + " given");
    if (n == 1u) {
        PGX_TRY(clear_status(ctx, s));
        wfg_small_kernel<<<1, 32, 0, s>>>(d_pts, n, m, make_ref(r, m), 1, d_out);
        PGX_CUDA(cudaGetLastError());
        ++ctx->launches;
        return PGX_OK;
    }
    if (m == 2u) {
        PGX_TRY(ctx->s_crowd.ensure(static_cast<size_t>(n) * 3u * sizeof(double)));
        double *lifted = ctx->s_crowd.as<double>();
        const unsigned g = static_cast<unsigned>(std::min<uint64_t>((n + 255u) / 256u, 4096u));
        wfg_lift2_kernel<<<g, 256, 0, s>>>(d_pts, n, lifted);
        PGX_CUDA(cudaGetLastError());
        ++ctx->launches;
        const double r3[3] = {r[0], r[1], 1.0};
        return run_warps(ctx, lifted, n, 3u, make_ref(r3, 3u), 1, d_out, s);
    }
    return run_warps(ctx, d_pts, n, m, make_ref(r, m), 1, d_out, s);
}

int wfg_status(pgx_context *ctx, unsigned *status)
{
    *status = 0;
    if (ctx->h_wfg.ptr == nullptr) return PGX_OK;
    PGX_CUDA(cudaMemcpyAsync(status, ctx->h_wfg.as<unsigned>() + 1, sizeof(unsigned), cudaMemcpyDeviceToHost,
                             ctx->stream));
    PGX_CUDA(cudaStreamSynchronize(ctx->stream));
    return PGX_OK;
}

} // namespace pgx
