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
// of the sorted set have the most candidates); the frames of the first levels
// are split into one work item per sub-term, level by level (see wfg_level),
// and the deepest level recurses on an explicit stack, its frames in the
// warp's slice of a scratch pool (m buffers of n rows). A warp's lanes share
// the limit-set filter (32 candidates at a time against the kept set, then
// against each other, then the kept points the survivors cover are removed),
// the counting-rank sorts of a frame and the closed forms. Every comparison
// (limit sets, sorts, maxima) runs on 64-bit integer order keys of the
// coordinates (the IEEE bit pattern with negatives mirrored, -0.0 read as
// +0.0, which the reference compares equal): the frames hold keys, and only
// the volumes and terms turn them back into doubles (GB300's FP64 pipe is far
// too narrow for the comparisons). A frame's kept set is the unique
// non-dominated subset of its candidates whatever order they are filtered in,
// every frame of more than two points is sorted by a strict order before it is
// used, and the two-point form is symmetric, so the arithmetic is the
// reference's: every operation is the reference's IEEE double operation in the
// reference's order (explicit round-to-nearest intrinsics: no contraction into
// FMA), and the volumes and contributions equal the reference's bit for bit.
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

using okey = long long; // order key of a coordinate

__device__ __forceinline__ okey to_key(double v)
{
    const long long b = __double_as_longlong(v == 0.0 ? 0.0 : v);
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

__device__ __forceinline__ double from_key(okey k)
{
    return __longlong_as_double(k >= 0 ? k : (k ^ 0x7fffffffffffffffLL));
}

__device__ __forceinline__ double std_max(double a, double b)
{
    return a < b ? b : a; // std::max(a, b)
}

// |prod over c = d-1 .. 0 of (r_c - p_c)| (hv_algorithm::volume_between on
// pointers, hv_algorithm.cpp:73-82)
__device__ __forceinline__ double vol(const double *r, const okey *p, uint32_t d)
{
    double v = 1.0;
    for (int c = static_cast<int>(d) - 1; c >= 0; --c) v = __dmul_rn(v, __dsub_rn(r[c], from_key(p[c])));
    return v < 0.0 ? -v : v;
}

// the same on plain doubles
__device__ __forceinline__ double vol_d(const double *r, const double *p, uint32_t d)
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
__device__ uint32_t limit_set(const okey *src, uint32_t src_stride, uint32_t begin, uint32_t end, uint32_t skip,
                              const okey *p, uint32_t dc, okey *dst, unsigned lane)
{
    uint32_t K = 0;
    for (uint32_t base = begin; base < end; base += 32u) {
        const uint32_t t = base + lane;
        const bool valid = t < end && t != skip;
        okey s[DM];
#pragma unroll
        for (int c = 0; c < DM; ++c)
            s[c] = (valid && c < static_cast<int>(dc)) ? max(src[static_cast<uint64_t>(t) * src_stride + c], p[c]) : 0;
        bool alive = valid;
        // a kept point <= s in every coordinate (dominating or equal): s goes
        for (uint32_t q = 0; q < K; ++q) {
            if (!__any_sync(kMask, alive)) break;
            const okey *kq = dst + static_cast<uint64_t>(q) * dc;
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
                        const okey su = __shfl_sync(kMask, s[c], u);
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
            okey qr[DM];
#pragma unroll
            for (int c = 0; c < DM; ++c)
                qr[c] = (has && c < static_cast<int>(dc)) ? dst[static_cast<uint64_t>(q) * dc + c] : 0;
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
                okey *o = dst + static_cast<uint64_t>(nk + __popc(km & lanes_below(lane))) * dc;
#pragma unroll
                for (int c = 0; c < DM; ++c)
                    if (c < static_cast<int>(dc)) o[c] = qr[c];
            }
            nk += __popc(km);
            __syncwarp();
        }
        if (alive) {
            okey *o = dst + static_cast<uint64_t>(nk + __popc(surv & lanes_below(lane))) * dc;
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
__device__ void sort_rows(const okey *src, uint32_t K, uint32_t d, bool by_y, okey *dst, unsigned lane)
{
    for (uint32_t i0 = 0; i0 < K; i0 += 32u) {
        const uint32_t i = i0 + lane;
        const bool has = i < K;
        okey mine[DM];
#pragma unroll
        for (int c = 0; c < DM; ++c)
            mine[c] = (has && c < static_cast<int>(d)) ? src[static_cast<uint64_t>(i) * d + c] : 0;
        uint32_t rank = 0;
        for (uint32_t j = 0; j < K; ++j) {
            const okey *rj = src + static_cast<uint64_t>(j) * d;
            int dec = 0; // +1: row j first, -1: this row first
            if (by_y) {
                const okey a = rj[1];
                dec = a < mine[1] ? 1 : (a > mine[1] ? -1 : 0);
            } else {
#pragma unroll
                for (int c = DM - 1; c >= 0; --c) {
                    if (c < static_cast<int>(d) && dec == 0) {
                        const okey a = rj[c];
                        dec = a > mine[c] ? 1 : (a < mine[c] ? -1 : 0);
                    }
                }
            }
            rank += (dec > 0 || (dec == 0 && j < i)) ? 1u : 0u;
        }
        if (has) {
            okey *o = dst + static_cast<uint64_t>(rank) * d;
#pragma unroll
            for (int c = 0; c < DM; ++c)
                if (c < static_cast<int>(d)) o[c] = mine[c];
        }
    }
    __syncwarp();
}

// The frames of a warp: m buffers of bd doubles, taken and given back by bit.
struct frame_pool {
    okey *base;
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
    __device__ okey *at(int b) const
    {
        return base + static_cast<uint64_t>(b) * bd;
    }
};

// hv of a frame of 1 or 2 points, or of 2 coordinates (tmp: a free buffer
// for the sort by y when k > 2)
template <int DM>
__device__ double closed_form(const double *r, const okey *f, uint32_t K, uint32_t d, okey *tmp, unsigned lane)
{
    if (K == 1u) return vol(r, f, d);
    if (K == 2u) {
        const double h = __dadd_rn(vol(r, f, d), vol(r, f + d, d));
        double isect = 1.0;
        for (uint32_t c = 0; c < d; ++c) isect = __dmul_rn(isect, __dsub_rn(r[c], from_key(max(f[c], f[d + c]))));
        return __dsub_rn(h, isect);
    }
    sort_rows<DM>(f, K, 2u, true, tmp, lane);
    double area = 0.0, w = __dsub_rn(r[0], from_key(tmp[0]));
    for (uint32_t t = 0; t + 1u < K; ++t) {
        area = __dadd_rn(area, __dmul_rn(__dsub_rn(from_key(tmp[2u * (t + 1u) + 1u]), from_key(tmp[2u * t + 1u])), w));
        w = std_max(w, __dsub_rn(r[0], from_key(tmp[2u * (t + 1u)])));
    }
    return __dadd_rn(area, __dmul_rn(__dsub_rn(r[1], from_key(tmp[2u * (K - 1u) + 1u])), w));
}

// |(p[d-1] - r[d-1]) * ex|, the term a point of a frame of d coordinates adds
__device__ __forceinline__ double slice_term(const double *r, const okey *p, uint32_t d, double ex)
{
    return fabs(__dmul_rn(__dsub_rn(from_key(p[d - 1u]), r[d - 1u]), ex));
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
        const okey *f = pool.at(st_buf[sp]);
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
            const okey *p = f + static_cast<uint64_t>(j) * dd;
            const int cb = pool.take();
            if (cb < 0) {
                *fail = true;
                return 0.0;
            }
            okey *child = pool.at(cb);
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
        const okey *p = pool.at(st_buf[sp]) + static_cast<uint64_t>(pj) * pd;
        st_h[sp] = __dadd_rn(st_h[sp], slice_term(r, p, pd, __dsub_rn(vol(r, p, pd - 1u), val)));
        st_j[sp] = pj + 1;
    }
}

// The work of one volume or one set of contributions is split into levels of
// rows: wfg_top_kernel takes the items (the top-level terms of a volume, or
// the points of the contributions), builds each item's limit set (its
// "frame") and finishes the items whose frame has at most two points or two
// coordinates; every other frame is sorted into the level-1 row list, one row
// per sub-term. wfg_rows_kernel(l) takes the rows of level l: row j of a frame
// gives the sub-term |(f_j[d-1] - r_{d-1}) * (vol_{d-1}(f_j) - hv(limit set
// of f_j over the rows after it))|; the row's own frame (that limit set) goes
// to level l + 1 the same way while levels remain, else the recursion below it
// runs on the warp's own stack. wfg_join_kernel(l) adds each row's sub-terms
// of level l + 1 in order (compute_hv's H += ..., hv_hvwfg.cpp:262-266) and
// finishes the row, and wfg_items_kernel finishes the items from level 1. The
// operations and their order are those of one recursion, split between warps.
constexpr int kMaxLevels = 4;

struct wfg_level {
    okey *frames;                  // the frames of this level's rows, rows of d keys
    uint32_t *row_parent;          // per row: its item (level 1) or its row of the level above
    double *row_term;              // per row: its sub-term
    uint32_t *frame_k;             // per parent: rows of its frame here (0: none)
    unsigned long long *frame_off; // per parent: its first row here
    unsigned long long *rows_used; // rows handed out (zero at launch)
    uint64_t row_cap;
    uint64_t parents;              // entries of frame_k / frame_off
};

struct wfg_args {
    const okey *pts;    // n rows of m keys; sorted by cmp_points for the terms of a volume
    uint32_t n, m;
    int contributions;  // 0: out[i] = the top-level term of sorted point i; 1: the contribution of point i
    double *out;        // n
    okey *pool;         // per warp: m buffers of bd keys
    uint64_t bd;
    unsigned *next;     // work counters (zero at launch): [0] items, [2 + l] rows of level l
    unsigned *status;   // set when a warp's pool ran dry
    int levels;         // row levels in use, 1 .. kMaxLevels
    wfg_level lv[kMaxLevels + 2]; // lv[1 .. levels]; lv[levels + 1] unused
};

__device__ __forceinline__ uint32_t first_dims(const wfg_args &a)
{
    return a.contributions ? a.m : a.m - 1u; // coordinates of the items' frames
}

// Row g of level l when it belongs to a frame stored at that level: its frame's
// rows k, first row off and index j; false for rows of a frame past the
// list's end (never written: any values).
__device__ __forceinline__ bool row_of(const wfg_args &a, int l, unsigned long long g, uint32_t *k,
                                       unsigned long long *off)
{
    const wfg_level &L = a.lv[l];
    const uint32_t parent = L.row_parent[g];
    if (parent >= L.parents) return false;
    *k = L.frame_k[parent];
    *off = L.frame_off[parent];
    return *k != 0u && g >= *off && g < *off + *k && *off + *k <= L.row_cap;
}

// The frame `buf` (k points of d coordinates, k > 2, d > 2) into level l's
// list, one row per point, sorted; the parent's entries set. Returns false
// when the list is full (the caller recurses instead).
template <int DM>
__device__ bool store_frame(const wfg_args &a, int l, uint64_t parent, const okey *buf, uint32_t k, uint32_t d,
                            unsigned lane)
{
    const wfg_level &L = a.lv[l];
    unsigned long long row0 = 0;
    if (lane == 0) row0 = atomicAdd(L.rows_used, static_cast<unsigned long long>(k));
    row0 = __shfl_sync(kMask, row0, 0);
    if (row0 + k > L.row_cap) return false;
    sort_rows<DM>(buf, k, d, false, L.frames + row0 * d, lane);
    for (uint32_t t = lane; t < k; t += 32u) L.row_parent[row0 + t] = static_cast<uint32_t>(parent);
    if (lane == 0) {
        L.frame_k[parent] = k;
        L.frame_off[parent] = row0;
    }
    return true;
}

__device__ __forceinline__ void mark_failed(const wfg_args &a, uint32_t item, unsigned lane)
{
    if (lane == 0) {
        atomicOr(a.status, 1u);
        a.out[item] = __longlong_as_double(0x7ff8000000000000LL);
    }
}

template <int DM>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) wfg_top_kernel(wfg_args a, wfg_ref ref)
{
    __shared__ double s_r[DM];
    if (threadIdx.x < DM) s_r[threadIdx.x] = threadIdx.x < a.m ? ref.r[threadIdx.x] : 0.0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t gw = static_cast<uint64_t>(blockIdx.x) * kWarpsPerBlock + (threadIdx.x >> 5);
    const uint32_t m = a.m;
    const uint32_t dc = first_dims(a);
    frame_pool pool{a.pool + gw * m * a.bd, a.bd, (1u << m) - 1u};
    for (;;) {
        unsigned item = 0;
        if (lane == 0) item = atomicAdd(a.next, 1u);
        item = __shfl_sync(kMask, item, 0);
        if (item >= a.n) break;
        const okey *p = a.pts + static_cast<uint64_t>(item) * m;
        const int b0 = pool.take(); // the pool is full here
        const uint32_t k0 = a.contributions ? limit_set<DM>(a.pts, m, 0u, a.n, item, p, dc, pool.at(b0), lane)
                                            : limit_set<DM>(a.pts, m, item + 1u, a.n, a.n, p, dc, pool.at(b0), lane);
        double ex = vol(s_r, p, dc);
        bool fail = false;
        if (k0 == 0u) {
            pool.give(b0);
        } else if (k0 <= 2u || dc == 2u) {
            const int tb = k0 > 2u ? pool.take() : -1;
            ex = __dsub_rn(ex, closed_form<DM>(s_r, pool.at(b0), k0, dc, tb >= 0 ? pool.at(tb) : nullptr, lane));
            if (tb >= 0) pool.give(tb);
            pool.give(b0);
        } else if (store_frame<DM>(a, 1, item, pool.at(b0), k0, dc, lane)) {
            pool.give(b0);
            continue;
        } else {
            // the level-1 list is full: this warp finishes the item alone
            ex = __dsub_rn(ex, frame_hv<DM>(s_r, pool, b0, k0, dc, lane, &fail));
        }
        if (fail) {
            mark_failed(a, item, lane);
            if (lane == 0) a.lv[1].frame_k[item] = 0;
            pool.free = (1u << m) - 1u;
            continue;
        }
        if (lane == 0) {
            a.lv[1].frame_k[item] = 0;
            a.out[item] = a.contributions ? ex : slice_term(s_r, p, m, ex);
        }
    }
}

template <int DM>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) wfg_rows_kernel(wfg_args a, wfg_ref ref, int l)
{
    __shared__ double s_r[DM];
    if (threadIdx.x < DM) s_r[threadIdx.x] = threadIdx.x < a.m ? ref.r[threadIdx.x] : 0.0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t gw = static_cast<uint64_t>(blockIdx.x) * kWarpsPerBlock + (threadIdx.x >> 5);
    const uint32_t m = a.m;
    const uint32_t d = first_dims(a) - static_cast<uint32_t>(l - 1); // coordinates of this level's rows
    const wfg_level &L = a.lv[l];
    const unsigned long long used = *L.rows_used;
    const unsigned long long rows = used < L.row_cap ? used : L.row_cap;
    const bool deeper = l < a.levels; // a level below for the rows' own frames
    frame_pool pool{a.pool + gw * m * a.bd, a.bd, (1u << m) - 1u};
    for (;;) {
        unsigned g = 0;
        if (lane == 0) g = atomicAdd(a.next + 2 + l, 1u);
        g = __shfl_sync(kMask, g, 0);
        if (g >= rows) break;
        uint32_t k = 0;
        unsigned long long off = 0;
        if (!row_of(a, l, g, &k, &off)) continue;
        const uint32_t j = static_cast<uint32_t>(g - off);
        const okey *f = L.frames + off * d;
        const okey *p = f + static_cast<uint64_t>(j) * d;
        const int cb = pool.take();
        const uint32_t ck = limit_set<DM>(f, d, j + 1u, k, k, p, d - 1u, pool.at(cb), lane);
        double ex = vol(s_r, p, d - 1u);
        bool fail = false;
        if (ck == 0u) {
            pool.give(cb);
        } else if (ck <= 2u || d - 1u == 2u) {
            const int tb = ck > 2u ? pool.take() : -1;
            ex = __dsub_rn(ex, closed_form<DM>(s_r, pool.at(cb), ck, d - 1u, tb >= 0 ? pool.at(tb) : nullptr, lane));
            if (tb >= 0) pool.give(tb);
            pool.give(cb);
        } else if (deeper && store_frame<DM>(a, l + 1, g, pool.at(cb), ck, d - 1u, lane)) {
            pool.give(cb);
            continue; // wfg_join_kernel(l) finishes the row
        } else {
            ex = __dsub_rn(ex, frame_hv<DM>(s_r, pool, cb, ck, d - 1u, lane, &fail));
        }
        if (fail) {
            if (lane == 0) {
                atomicOr(a.status, 1u);
                L.row_term[g] = __longlong_as_double(0x7ff8000000000000LL);
            }
            pool.free = (1u << m) - 1u;
        } else if (lane == 0) {
            L.row_term[g] = slice_term(s_r, p, d, ex);
        }
        if (lane == 0 && deeper) a.lv[l + 1].frame_k[g] = 0;
    }
}

// The rows of level l whose frame went to level l + 1: H = the sum of that
// frame's sub-terms in order from 0.0, then the row's sub-term.
__global__ void wfg_join_kernel(wfg_args a, wfg_ref ref, int l)
{
    const uint32_t d = first_dims(a) - static_cast<uint32_t>(l - 1);
    const wfg_level &L = a.lv[l], &C = a.lv[l + 1];
    const unsigned long long used = *L.rows_used;
    const unsigned long long rows = used < L.row_cap ? used : L.row_cap;
    for (unsigned long long g = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; g < rows;
         g += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
        uint32_t k = 0;
        unsigned long long off = 0;
        if (!row_of(a, l, g, &k, &off)) continue;
        const uint32_t ck = C.frame_k[g];
        const unsigned long long coff = C.frame_off[g];
        if (ck == 0u || coff + ck > C.row_cap) continue;
        double h = 0.0;
        for (uint32_t t = 0; t < ck; ++t) h = __dadd_rn(h, C.row_term[coff + t]);
        const okey *p = L.frames + (off + (g - off)) * d;
        L.row_term[g] = slice_term(ref.r, p, d, __dsub_rn(vol(ref.r, p, d - 1u), h));
    }
}

// The items with a frame at level 1: H = the sum of their rows' sub-terms in
// order from 0.0, then the item's value as wfg_top_kernel would give it.
__global__ void wfg_items_kernel(wfg_args a, wfg_ref ref)
{
    const uint32_t m = a.m;
    const uint32_t dc = first_dims(a);
    const wfg_level &L = a.lv[1];
    for (uint32_t item = blockIdx.x * blockDim.x + threadIdx.x; item < a.n; item += gridDim.x * blockDim.x) {
        const uint32_t k0 = L.frame_k[item];
        if (k0 == 0u) continue;
        const unsigned long long off = L.frame_off[item];
        double h = 0.0;
        for (uint32_t j = 0; j < k0; ++j) h = __dadd_rn(h, L.row_term[off + j]);
        const okey *p = a.pts + static_cast<uint64_t>(item) * m;
        const double ex = __dsub_rn(vol(ref.r, p, dc), h);
        a.out[item] = a.contributions ? ex : slice_term(ref.r, p, m, ex);
    }
}

// The points as order keys (keys[i * m + c]).
__global__ void wfg_keys_kernel(const double *__restrict__ pts, uint64_t total, okey *__restrict__ keys)
{
    for (uint64_t e = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        keys[e] = to_key(pts[e]);
}

// Ranks of the points by hvwfg::cmp_points over m coordinates (ties by
// index): block (x, y) counts, for its 64 points, the points of slice y of
// the others that come first (staged in shared memory), added to rank[]
// (zero at launch).
constexpr int kRankThreads = 64;
constexpr uint32_t kRankSlices = 8;

__global__ void __launch_bounds__(kRankThreads)
    wfg_rank_kernel(const okey *__restrict__ keys, uint32_t n, uint32_t m, unsigned *__restrict__ rank)
{
    __shared__ okey tile[kRankThreads * kWfgMaxObjectives];
    const uint32_t i = blockIdx.x * kRankThreads + threadIdx.x;
    okey mine[kWfgMaxObjectives];
    for (uint32_t c = 0; c < m; ++c) mine[c] = i < n ? keys[static_cast<uint64_t>(i) * m + c] : 0;
    const uint32_t per = (n + kRankSlices - 1u) / kRankSlices;
    const uint32_t j_begin = blockIdx.y * per, j_end = min(n, j_begin + per);
    uint32_t cnt = 0;
    for (uint32_t j0 = j_begin; j0 < j_end; j0 += kRankThreads) {
        const uint32_t len = min(static_cast<uint32_t>(kRankThreads), j_end - j0);
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < len * m; e += kRankThreads) tile[e] = keys[static_cast<uint64_t>(j0) * m + e];
        __syncthreads();
        if (i < n) {
            for (uint32_t jj = 0; jj < len; ++jj) {
                const okey *rj = tile + jj * m;
                int dec = 0;
                for (int c = static_cast<int>(m) - 1; c >= 0 && dec == 0; --c)
                    dec = rj[c] > mine[c] ? 1 : (rj[c] < mine[c] ? -1 : 0);
                cnt += (dec > 0 || (dec == 0 && j0 + jj < i)) ? 1u : 0u;
            }
        }
    }
    if (i < n && cnt) atomicAdd(rank + i, cnt);
}

// sorted[rank[i]] = keys[i] (rows of m)
__global__ void wfg_scatter_kernel(const okey *__restrict__ keys, uint32_t n, uint32_t m,
                                   const unsigned *__restrict__ rank, okey *__restrict__ sorted)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (uint32_t c = 0; c < m; ++c) sorted[static_cast<uint64_t>(rank[i]) * m + c] = keys[static_cast<uint64_t>(i) * m + c];
}

// out = the sum of term[0 .. n) in index order from 0.0 (compute_hv's
// H += ..., hv_hvwfg.cpp:262-266): the block stages the terms in shared
// memory, one thread adds them in order.
constexpr int kSumThreads = 1024;

__global__ void __launch_bounds__(kSumThreads) wfg_sum_kernel(const double *__restrict__ term, uint32_t n,
                                                              double *__restrict__ out)
{
    __shared__ double s[kSumThreads];
    double h = 0.0;
    for (uint32_t base = 0; base < n; base += kSumThreads) {
        const uint32_t len = min(static_cast<uint32_t>(kSumThreads), n - base);
        __syncthreads();
        if (threadIdx.x < len) s[threadIdx.x] = term[base + threadIdx.x];
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (; t + 4u <= len; t += 4u) {
                const double a = s[t], b = s[t + 1u], c = s[t + 2u], d = s[t + 3u];
                h = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(h, a), b), c), d);
            }
            for (; t < len; ++t) h = __dadd_rn(h, s[t]);
        }
    }
    if (threadIdx.x == 0) *out = h;
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
        *out = vol_d(r, pts, m);
        return;
    }
    const double h = __dadd_rn(vol_d(r, pts, m), vol_d(r, pts + m, m));
    double isect = 1.0;
    for (uint32_t c = 0; c < m; ++c) isect = __dmul_rn(isect, __dsub_rn(r[c], std_max(pts[c], pts[m + c])));
    *out = __dsub_rn(h, isect);
}

// 2-objective points as hv2d::contributions hands them to hv3d, as keys: a
// third coordinate 0 (hv_hv2d.cpp:135-143)
__global__ void wfg_lift2_kernel(const double *__restrict__ pts, uint32_t n, okey *__restrict__ out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        out[3ull * i] = to_key(pts[2ull * i]);
        out[3ull * i + 1u] = to_key(pts[2ull * i + 1u]);
        out[3ull * i + 2u] = to_key(0.0);
    }
}

size_t round256(size_t b)
{
    return (b + 255u) & ~size_t(255);
}

// Scratch of the split kernels over n points of m coordinates: [counters,
// status, rows handed out | per level: per parent frame rows and first row,
// per row parent, sub-term and d keys | pool]; each level's list holds up to
// row_cap rows (past it a frame is finished by the warp that built it), the
// number of warps fits the pool in kPoolBytes (at least one warp).
constexpr size_t kPoolBytes = size_t(1) << 30;
constexpr uint64_t kRowCap = uint64_t(1) << 20;

int run_warps(pgx_context *ctx, const okey *d_keys, uint32_t n, uint32_t m, const wfg_ref &ref, int contributions,
              double *d_out, cudaStream_t s)
{
    const uint64_t bd = static_cast<uint64_t>(n) * m; // a frame: at most n rows of at most m coordinates
    const size_t per_warp = static_cast<size_t>(m) * bd * sizeof(okey);
    PGX_CHECK(per_warp <= (size_t(4) << 30), PGX_ERR_CAPACITY,
              "hypervolume (WFG): " + std::to_string(n) + " points of " + std::to_string(m) +
                  " objectives need more than 4 GiB of frames per warp");
    const uint32_t dc = contributions ? m : m - 1u;
    // levels 1 .. dc - 2 hold rows of dc .. 3 coordinates (a row of 3 has a frame of 2: closed form)
    const int levels = static_cast<int>(std::min<uint32_t>(kMaxLevels, dc > 3u ? dc - 2u : 1u));
    const uint64_t row_cap = std::max<uint64_t>(64u, std::min<uint64_t>(static_cast<uint64_t>(n) * n, kRowCap));
    const uint64_t want = std::min<uint64_t>(std::max<uint64_t>(n, 1024u), static_cast<uint64_t>(ctx->num_sms) * 16u);
    const uint64_t fit = std::max<uint64_t>(1u, kPoolBytes / per_warp);
    uint64_t warps = std::min(want, fit);
    const unsigned blocks = static_cast<unsigned>((warps + kWarpsPerBlock - 1u) / kWarpsPerBlock);
    warps = static_cast<uint64_t>(blocks) * kWarpsPerBlock; // every warp of the grid has its slice
    const size_t b_ctl = 256u;
    size_t head = b_ctl;
    size_t lv_off[kMaxLevels + 2][5] = {};
    for (int l = 1; l <= levels; ++l) {
        const uint64_t parents = l == 1 ? n : row_cap;
        const uint32_t d = dc - static_cast<uint32_t>(l - 1);
        lv_off[l][0] = head; // frame_k
        head += round256(parents * sizeof(uint32_t));
        lv_off[l][1] = head; // frame_off
        head += round256(parents * sizeof(unsigned long long));
        lv_off[l][2] = head; // row_parent
        head += round256(row_cap * sizeof(uint32_t));
        lv_off[l][3] = head; // row_term
        head += round256(row_cap * sizeof(double));
        lv_off[l][4] = head; // frames
        head += round256(row_cap * d * sizeof(okey));
    }
    PGX_TRY(ctx->h_wfg.ensure(head + warps * per_warp));
    char *base = ctx->h_wfg.as<char>();
    unsigned *ctl = reinterpret_cast<unsigned *>(base);
    PGX_CUDA(cudaMemsetAsync(ctl, 0, b_ctl, s));
    wfg_args a{};
    a.pts = d_keys;
    a.n = n;
    a.m = m;
    a.contributions = contributions;
    a.out = d_out;
    a.pool = reinterpret_cast<okey *>(base + head);
    a.bd = bd;
    a.next = ctl;
    a.status = ctl + 1;
    a.levels = levels;
    for (int l = 1; l <= levels; ++l) {
        wfg_level &L = a.lv[l];
        L.frame_k = reinterpret_cast<uint32_t *>(base + lv_off[l][0]);
        L.frame_off = reinterpret_cast<unsigned long long *>(base + lv_off[l][1]);
        L.row_parent = reinterpret_cast<uint32_t *>(base + lv_off[l][2]);
        L.row_term = reinterpret_cast<double *>(base + lv_off[l][3]);
        L.frames = reinterpret_cast<okey *>(base + lv_off[l][4]);
        L.rows_used = reinterpret_cast<unsigned long long *>(base + 64u + 8u * static_cast<size_t>(l));
        L.row_cap = row_cap;
        L.parents = l == 1 ? n : row_cap;
    }
    const int threads = kWarpsPerBlock * 32;
    auto launch_rows = [&](int l) {
        if (m <= 4u)
            wfg_rows_kernel<4><<<blocks, threads, 0, s>>>(a, ref, l);
        else if (m <= 8u)
            wfg_rows_kernel<8><<<blocks, threads, 0, s>>>(a, ref, l);
        else
            wfg_rows_kernel<16><<<blocks, threads, 0, s>>>(a, ref, l);
    };
    if (m <= 4u)
        wfg_top_kernel<4><<<blocks, threads, 0, s>>>(a, ref);
    else if (m <= 8u)
        wfg_top_kernel<8><<<blocks, threads, 0, s>>>(a, ref);
    else
        wfg_top_kernel<16><<<blocks, threads, 0, s>>>(a, ref);
    PGX_CUDA(cudaGetLastError());
    for (int l = 1; l <= levels; ++l) {
        launch_rows(l);
        PGX_CUDA(cudaGetLastError());
    }
    const unsigned jb = static_cast<unsigned>(std::min<uint64_t>((row_cap + 127u) / 128u, 4096u));
    for (int l = levels - 1; l >= 1; --l) {
        wfg_join_kernel<<<jb, 128, 0, s>>>(a, ref, l);
        PGX_CUDA(cudaGetLastError());
    }
    wfg_items_kernel<<<(n + 127u) / 128u, 128, 0, s>>>(a, ref);
    PGX_CUDA(cudaGetLastError());
    ctx->launches += 2u + 2u * static_cast<uint64_t>(levels);
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
    // keys | sorted keys | ranks | terms
    const size_t b_keys = round256(static_cast<size_t>(n) * m * sizeof(okey));
    const size_t b_rank = round256(static_cast<size_t>(n) * sizeof(unsigned));
    const size_t b_terms = round256(static_cast<size_t>(n) * sizeof(double));
    PGX_TRY(ctx->s_crowd.ensure(2u * b_keys + b_rank + b_terms));
    char *base = ctx->s_crowd.as<char>();
    okey *keys = reinterpret_cast<okey *>(base);
    okey *sorted = reinterpret_cast<okey *>(base + b_keys);
    unsigned *rank = reinterpret_cast<unsigned *>(base + 2u * b_keys);
    double *terms = reinterpret_cast<double *>(base + 2u * b_keys + b_rank);
    const uint64_t total = static_cast<uint64_t>(n) * m;
    const unsigned g = static_cast<unsigned>(std::min<uint64_t>((total + 255u) / 256u, 8192u));
    wfg_keys_kernel<<<g, 256, 0, s>>>(d_pts, total, keys);
    PGX_CUDA(cudaGetLastError());
    PGX_CUDA(cudaMemsetAsync(rank, 0, static_cast<size_t>(n) * sizeof(unsigned), s));
    wfg_rank_kernel<<<dim3((n + kRankThreads - 1u) / kRankThreads, kRankSlices), kRankThreads, 0, s>>>(keys, n, m,
                                                                                                     rank);
    PGX_CUDA(cudaGetLastError());
    wfg_scatter_kernel<<<(n + 255u) / 256u, 256, 0, s>>>(keys, n, m, rank, sorted);
    PGX_CUDA(cudaGetLastError());
    PGX_TRY(run_warps(ctx, sorted, n, m, ref, 0, terms, s));
    wfg_sum_kernel<<<1, kSumThreads, 0, s>>>(terms, n, d_out);
    PGX_CUDA(cudaGetLastError());
    ctx->launches += 4;
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
    const uint32_t mk = m == 2u ? 3u : m; // 2 objectives: hv3d's points with a third coordinate 0
    PGX_TRY(ctx->s_crowd.ensure(static_cast<size_t>(n) * mk * sizeof(okey)));
    okey *keys = ctx->s_crowd.as<okey>();
    if (m == 2u) {
        const unsigned g = static_cast<unsigned>(std::min<uint64_t>((n + 255u) / 256u, 4096u));
        wfg_lift2_kernel<<<g, 256, 0, s>>>(d_pts, n, keys);
        PGX_CUDA(cudaGetLastError());
        ++ctx->launches;
        const double r3[3] = {r[0], r[1], 1.0};
        return run_warps(ctx, keys, n, 3u, make_ref(r3, 3u), 1, d_out, s);
    }
    const uint64_t total = static_cast<uint64_t>(n) * m;
    const unsigned g = static_cast<unsigned>(std::min<uint64_t>((total + 255u) / 256u, 8192u));
    wfg_keys_kernel<<<g, 256, 0, s>>>(d_pts, total, keys);
    PGX_CUDA(cudaGetLastError());
    ++ctx->launches;
    return run_warps(ctx, keys, n, m, make_ref(r, m), 1, d_out, s);
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
