// std::sort's order, on the GPU.
//
// pagmo sorts with std::sort (crowding_distance, src/utils/multi_objective.cpp:
// 301-306; select_best_N_mo :386-389; sort_population_mo :455-462). std::sort
// is not stable: the order it leaves tied elements in is a property of the
// standard library, here GNU libstdc++'s introsort (bits/stl_algo.h, unchanged
// in this respect since GCC 4.9), which the reference is built against. These
// routines leave exactly the permutation that algorithm leaves:
//
//   introsort_loop(first, last, depth = 2 floor(log2 n)):
//     while last - first > 16:
//       if depth == 0: heapsort [first, last) (make_heap, sort_heap); return
//       --depth
//       move the median of (first+1, mid, last-1) into first
//       cut = Hoare partition of [first+1, last) around *first
//       introsort_loop(cut, last, depth); last = cut
//   insertion sort over the whole array
//
// GPU formulation (one thread block per sort):
//  - Ranges are processed level by level (a level = one recursion depth), each
//    range by one warp; the ranges of a level are disjoint, so the order in
//    which warps take them does not change the result.
//  - The sequential loop swaps the i-th "left stopper" (position p > first
//    with !(x[p] < pivot), in ascending order) with the i-th "right stopper"
//    (!(pivot < x[p]), in descending order) for as long as the former lies
//    below the latter, and returns min(next left stopper, last swapped right
//    stopper) -- the first left stopper if nothing was swapped. A partition
//    here compacts every left and right stopper of the range in position order
//    (ballots over the original values: by one warp for ranges up to
//    kBlockRange, by block scans for longer ones), K = the number of pairs i
//    with left[i] < right[i] (a prefix of i), the K swaps run in parallel, and
//    the cut is min(left[K], right[K-1]) (left[0] when K = 0) -- the same
//    pairs and cut as the sequential loop.
//  - Ranges of 16 or fewer elements are final: the closing insertion sort of
//    the whole array moves no element across a partition boundary, so it
//    equals a stable sort of each such range, which a half warp computes by
//    counting, for each element, the smaller keys and the equal keys before it.
//  - A range whose depth budget is spent is heapsorted by one lane, with
//    libstdc++'s make_heap/sort_heap sift order.
// The oracle restates the same algorithm twice (oracle/sorting.cpp) and the
// tests check both restatements and this code against std::sort itself.
#pragma once

#include <cstdint>

namespace pgx
{
namespace dev
{

constexpr unsigned kSortFull = 0xffffffffu;

// Composite key (sort_population_mo): rank, then descending crowding.
struct key2 {
    long long a, b;
};

__device__ __forceinline__ bool key_less(long long x, long long y)
{
    return x < y;
}
__device__ __forceinline__ bool key_less(const key2 &x, const key2 &y)
{
    return x.a < y.a || (x.a == y.a && x.b < y.b);
}

// (key, value) pairs in shared or global memory.
template <typename K>
struct sort_view {
    K *k;
    int32_t *v;
    __device__ __forceinline__ void swap(int a, int b) const
    {
        const K t = k[a];
        k[a] = k[b];
        k[b] = t;
        const int32_t u = v[a];
        v[a] = v[b];
        v[b] = u;
    }
};

// Control words of one block's sort (shared memory).
struct sort_ctl {
    int take;     // next small range of the current level
    int ncur;     // small ranges in the current level
    int nnext;    // small ranges queued for the next level
    int nbig;     // block-partitioned ranges in the current level
    int nbignext; // block-partitioned ranges queued for the next level
    int pad[3];
};

// Ranges longer than this are partitioned by the whole block.
constexpr int kBlockRange = 512;

// Bookkeeping of one block's sort: level lists of small ranges (2 * small_cap,
// small_cap >= n / 17 + 1) and of block-partitioned ranges (2 * big_cap,
// big_cap >= n / kBlockRange + 1), and n + n stopper positions.
struct sort_work {
    int2 *small;
    int small_cap;
    int2 *big;
    int big_cap;
    int *pos_l;
    int *pos_r;
};

// Error codes written to the sort's error word (never expected; each marks a
// broken invariant of the algorithm rather than bad input).
enum : int { kSortErrListFull = 1, kSortErrNoSentinel = 2, kSortErrGuard = 3 };

__device__ __forceinline__ int floor_log2_int(int n)
{
    return 31 - __clz(n);
}

template <typename K>
__device__ void median_to_first(const sort_view<K> &x, int result, int a, int b, int c)
{
    if (key_less(x.k[a], x.k[b])) {
        if (key_less(x.k[b], x.k[c]))
            x.swap(result, b);
        else if (key_less(x.k[a], x.k[c]))
            x.swap(result, c);
        else
            x.swap(result, a);
    } else if (key_less(x.k[a], x.k[c])) {
        x.swap(result, a);
    } else if (key_less(x.k[b], x.k[c])) {
        x.swap(result, c);
    } else {
        x.swap(result, b);
    }
}

template <typename K>
__device__ void insertion_sort(const sort_view<K> &x, int first, int last)
{
    for (int i = first + 1; i < last; ++i) {
        const K vk = x.k[i];
        const int32_t vv = x.v[i];
        int j = i;
        while (j > first && key_less(vk, x.k[j - 1])) {
            x.k[j] = x.k[j - 1];
            x.v[j] = x.v[j - 1];
            --j;
        }
        x.k[j] = vk;
        x.v[j] = vv;
    }
}

// libstdc++'s heap sift (__adjust_heap followed by __push_heap) on
// x[first .. first+len), placing (vk, vv) from the hole.
template <typename K>
__device__ void adjust_heap(const sort_view<K> &x, int first, int hole, int len, K vk, int32_t vv)
{
    const int top = hole;
    int child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (key_less(x.k[first + child], x.k[first + child - 1])) --child;
        x.k[first + hole] = x.k[first + child];
        x.v[first + hole] = x.v[first + child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        x.k[first + hole] = x.k[first + child - 1];
        x.v[first + hole] = x.v[first + child - 1];
        hole = child - 1;
    }
    int parent = (hole - 1) / 2;
    while (hole > top && key_less(x.k[first + parent], vk)) {
        x.k[first + hole] = x.k[first + parent];
        x.v[first + hole] = x.v[first + parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    x.k[first + hole] = vk;
    x.v[first + hole] = vv;
}

// make_heap then sort_heap (std::partial_sort(first, last, last)).
template <typename K>
__device__ void heap_sort(const sort_view<K> &x, int first, int last)
{
    const int len = last - first;
    if (len >= 2) {
        for (int parent = (len - 2) / 2;; --parent) {
            adjust_heap(x, first, parent, len, x.k[first + parent], x.v[first + parent]);
            if (parent == 0) break;
        }
    }
    for (int l = len; l > 1;) {
        --l;
        const K vk = x.k[first + l];
        const int32_t vv = x.v[first + l];
        x.k[first + l] = x.k[first];
        x.v[first + l] = x.v[first];
        adjust_heap(x, first, 0, l, vk, vv);
    }
}

// Stable sort of a leaf x[first .. first+len) (len <= 16) by one half warp:
// every lane of the half calls it with its half's leaf (len 0: nothing).
template <typename K>
__device__ __forceinline__ K shfl16(const K &v, int src);
template <>
__device__ __forceinline__ long long shfl16<long long>(const long long &v, int src)
{
    return __shfl_sync(kSortFull, v, src, 16);
}
template <>
__device__ __forceinline__ key2 shfl16<key2>(const key2 &v, int src)
{
    return key2{__shfl_sync(kSortFull, v.a, src, 16), __shfl_sync(kSortFull, v.b, src, 16)};
}

template <typename K>
__device__ void halfwarp_leaf_sort(const sort_view<K> &x, int first, int len)
{
    const int sub = static_cast<int>(threadIdx.x & 15u);
    const bool act = sub < len;
    K kv{};
    int32_t vv = 0;
    if (act) {
        kv = x.k[first + sub];
        vv = x.v[first + sub];
    }
    int pos = 0;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const K kj = shfl16(kv, j);
        if (act && j < len && (key_less(kj, kv) || (j < sub && !key_less(kv, kj)))) ++pos;
    }
    __syncwarp();
    if (act) {
        x.k[first + pos] = kv;
        x.v[first + pos] = vv;
    }
    __syncwarp();
}

// The whole block: median-of-three into `first`, then the Hoare partition of
// [first+1, last) from the compacted stopper lists; returns the cut (same
// value in every thread). scan: 64 ints of shared memory.
template <typename K>
__device__ int block_partition(const sort_view<K> &x, int first, int last, const sort_work &w, int *scan, int *err)
{
    const unsigned lane = threadIdx.x & 31u;
    const int warp = static_cast<int>(threadIdx.x >> 5), nwarps = static_cast<int>(blockDim.x >> 5);
    const unsigned below = (1u << lane) - 1u;
    if (threadIdx.x == 0) median_to_first(x, first, first + 1, first + (last - first) / 2, last - 1);
    __syncthreads();
    const K pv = x.k[first];
    int nl = 0, nr = 0; // stoppers so far (uniform)
    for (int t0 = first + 1; t0 < last; t0 += blockDim.x) {
        const int p = t0 + static_cast<int>(threadIdx.x);
        bool fl = false, fr = false;
        if (p < last) {
            const K kp = x.k[p];
            fl = !key_less(kp, pv);
            fr = !key_less(pv, kp);
        }
        const unsigned bl = __ballot_sync(kSortFull, fl), br = __ballot_sync(kSortFull, fr);
        if (lane == 0) {
            scan[warp] = __popc(bl);
            scan[32 + warp] = __popc(br);
        }
        __syncthreads();
        // exclusive prefix of the warps' counts: each warp scans the (up to 32)
        // counts with shuffles
        int cl = static_cast<int>(lane) < nwarps ? scan[lane] : 0;
        int cr = static_cast<int>(lane) < nwarps ? scan[32 + lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int tl = __shfl_up_sync(kSortFull, cl, o), tr = __shfl_up_sync(kSortFull, cr, o);
            if (static_cast<int>(lane) >= o) {
                cl += tl;
                cr += tr;
            }
        }
        const int totl = __shfl_sync(kSortFull, cl, 31), totr = __shfl_sync(kSortFull, cr, 31);
        const int offl = warp > 0 ? __shfl_sync(kSortFull, cl, warp - 1) : 0;
        const int offr = warp > 0 ? __shfl_sync(kSortFull, cr, warp - 1) : 0;
        if (fl) w.pos_l[nl + offl + __popc(bl & below)] = p;
        if (fr) w.pos_r[nr + offr + __popc(br & below)] = p;
        nl += totl;
        nr += totr;
        __syncthreads();
    }
    // pair i = (pos_l[i], pos_r[nr-1-i]); the swappable pairs are a prefix
    const int mx = min(nl, nr);
    int kk = 0;
    for (int i0 = 0; i0 < mx; i0 += blockDim.x) {
        const int i = i0 + static_cast<int>(threadIdx.x);
        const bool ok = i < mx && w.pos_l[i] < w.pos_r[nr - 1 - i];
        const int c = __syncthreads_count(ok);
        kk += c;
        if (c < static_cast<int>(blockDim.x)) break;
    }
    for (int i = threadIdx.x; i < kk; i += blockDim.x) x.swap(w.pos_l[i], w.pos_r[nr - 1 - i]);
    int cut;
    if (nl == 0) {
        if (threadIdx.x == 0) atomicExch(err, kSortErrNoSentinel);
        cut = last - 1;
    } else if (kk == 0) {
        cut = w.pos_l[0];
    } else {
        cut = w.pos_r[nr - kk];
        if (kk < nl) cut = min(cut, w.pos_l[kk]);
    }
    __syncthreads();
    return cut;
}

// One warp: median-of-three into `first`, then the Hoare partition of
// [first+1, last) around it from compacted stopper lists, as block_partition
// does with the whole block: one sweep of ballots over 32-position chunks
// lists every left stopper (!(x[p] < pivot)) and right stopper
// (!(pivot < x[p])) in position order into pos_l / pos_r at offset `first`
// (the ranges a level's warps hold are disjoint, so are these areas), the
// swappable pairs are a prefix counted by ballots, the swaps run on all lanes,
// and the cut is min(left[K], right[K-1]) (left[0] when K = 0). All 32 lanes
// call it with the same arguments; returns the cut.
template <typename K>
__device__ int warp_partition(const sort_view<K> &x, int first, int last, const sort_work &w, int *err)
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned below = (1u << lane) - 1u;
    if (lane == 0) median_to_first(x, first, first + 1, first + (last - first) / 2, last - 1);
    __syncwarp();
    const K pv = x.k[first];
    int *pl = w.pos_l + first, *pr = w.pos_r + first;
    int nl = 0, nr = 0;
    for (int t0 = first + 1; t0 < last; t0 += 32) {
        const int p = t0 + static_cast<int>(lane);
        bool fl = false, fr = false;
        if (p < last) {
            const K kp = x.k[p];
            fl = !key_less(kp, pv);
            fr = !key_less(pv, kp);
        }
        const unsigned bl = __ballot_sync(kSortFull, fl), br = __ballot_sync(kSortFull, fr);
        if (fl) pl[nl + __popc(bl & below)] = p;
        if (fr) pr[nr + __popc(br & below)] = p;
        nl += __popc(bl);
        nr += __popc(br);
    }
    __syncwarp();
    // pair i = (pl[i], pr[nr-1-i]); the swappable pairs are a prefix
    const int mx = min(nl, nr);
    int kk = 0;
    for (int i0 = 0; i0 < mx; i0 += 32) {
        const int i = i0 + static_cast<int>(lane);
        const unsigned b = __ballot_sync(kSortFull, i < mx && pl[i] < pr[nr - 1 - i]);
        kk += __popc(b);
        if (b != kSortFull) break;
    }
    for (int i = static_cast<int>(lane); i < kk; i += 32) x.swap(pl[i], pr[nr - 1 - i]);
    __syncwarp();
    if (nl == 0) {
        if (lane == 0) atomicExch(err, kSortErrNoSentinel);
        return last - 1;
    }
    if (kk == 0) return pl[0];
    const int cut = pr[nr - kk];
    return kk < nl ? min(cut, pl[kk]) : cut;
}

// Ranges of 17..kBlockRange elements wait in a ring of int4 (first, last,
// depth budget, publication ticket + 1) shared by the block's warps: any
// warp takes the next ticket, waits until that slot is published (or until no
// range is outstanding), partitions the range and publishes its children. The
// ranges outstanding at any time are disjoint and longer than 16, so at most
// n / 17 of them exist and a ring of n / 17 + 1 slots never overwrites a slot
// before its range is done. ctl->take: next ticket to take; ctl->nnext: next
// ticket to publish; ctl->ncur: ranges outstanding.
constexpr unsigned long long kRingSpinLimit = 1ull << 22;

__device__ __forceinline__ void ring_push(int4 *ring, int cap, sort_ctl *ctl, int a, int b, int d)
{
    const int t = atomicAdd(&ctl->nnext, 1);
    int4 *slot = ring + (t % cap);
    slot->x = a;
    slot->y = b;
    slot->z = d;
    __threadfence_block();
    atomicExch(&slot->w, t + 1);
}

// A child [a, b) of a partition with depth budget d: to the next level's
// block-partition list, to the ring, or (16 or fewer) left for the caller's
// leaf sort. Returns 1 when it went to the ring.
__device__ __forceinline__ int place_child(int a, int b, int d, int2 *big_next, const sort_work &w, int4 *ring,
                                           int cap, sort_ctl *ctl, int *err)
{
    const int len = b - a;
    if (len > kBlockRange) {
        const int slot = atomicAdd(&ctl->nbignext, 1);
        if (slot < w.big_cap)
            big_next[slot] = make_int2(a, b);
        else
            atomicExch(err, kSortErrListFull);
        return 0;
    }
    if (len > 16) {
        atomicAdd(&ctl->ncur, 1);
        ring_push(ring, cap, ctl, a, b, d);
        return 1;
    }
    return 0;
}

// Sorts x[0 .. n) by key with std::sort's order of ties. Every thread of the
// block calls it (blockDim.x a multiple of 32, at most 1024). slots_all: 64
// ints per warp of shared memory; ctl in shared memory. depth0 >= 0 continues
// an introsort whose depth budget at this range is depth0 (a subrange of a
// larger sort); -1 starts one (2 floor(log2 n)). Ends with a __syncthreads.
//
// Ranges longer than kBlockRange are partitioned level by level by the whole
// block; the shorter ones they produce go to the ring, which the warps then
// drain, each taking ranges as they come (no barrier between levels: a warp
// goes on with other ranges while deeper parts of the recursion proceed).
// Ranges are disjoint and each carries the depth budget the sequential
// recursion would give it, so the order of the work does not change the result.
template <typename K>
__device__ void block_std_sort(const sort_view<K> &x, int n, const sort_work &w, sort_ctl *ctl, int *slots_all,
                               int *err, int depth0 = -1)
{
    const unsigned lane = threadIdx.x & 31u;
    const int warp = static_cast<int>(threadIdx.x >> 5);
    if (n <= 16) {
        if (warp == 0) halfwarp_leaf_sort(x, 0, lane < 16u ? n : 0);
        __syncthreads();
        return;
    }
    int depth = depth0 >= 0 ? depth0 : 2 * floor_log2_int(n);
    int4 *ring = reinterpret_cast<int4 *>(w.small); // 2 small_cap int2 = small_cap int4
    const int cap = w.small_cap;
    int2 *big_cur = w.big, *big_next = w.big + w.big_cap;
    for (int i = threadIdx.x; i < cap; i += blockDim.x) ring[i].w = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        ctl->take = 0;
        ctl->nnext = 0;
        ctl->ncur = 0;
        ctl->nbig = 0;
        ctl->nbignext = 0;
        if (n > kBlockRange) {
            big_cur[0] = make_int2(0, n);
            ctl->nbig = 1;
        } else {
            atomicAdd(&ctl->ncur, 1);
            ring_push(ring, cap, ctl, 0, n, depth);
        }
    }
    __syncthreads();
    // ---- ranges longer than kBlockRange, one level at a time, by the whole block
    for (;;) {
        const int nbig = min(ctl->nbig, w.big_cap);
        if (nbig == 0) break;
        __syncthreads();
        for (int t = 0; t < nbig; ++t) {
            const int2 r = big_cur[t];
            if (depth == 0) {
                if (threadIdx.x == 0) heap_sort(x, r.x, r.y);
                __syncthreads();
                continue;
            }
            const int cut = block_partition(x, r.x, r.y, w, slots_all, err);
            if (threadIdx.x == 0) place_child(r.x, cut, depth - 1, big_next, w, ring, cap, ctl, err);
            if (threadIdx.x == 32 || (blockDim.x == 32 && threadIdx.x == 1))
                place_child(cut, r.y, depth - 1, big_next, w, ring, cap, ctl, err);
            if (warp == 0) {
                const int a = lane < 16u ? r.x : cut, len = lane < 16u ? cut - r.x : r.y - cut;
                halfwarp_leaf_sort(x, a, len <= 16 ? len : 0);
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            ctl->nbig = ctl->nbignext;
            ctl->nbignext = 0;
        }
        int2 *t = big_cur;
        big_cur = big_next;
        big_next = t;
        --depth;
        __syncthreads();
    }
    // ---- the ring: every warp takes ranges until none is outstanding
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(&ctl->take, 1);
        t = __shfl_sync(kSortFull, t, 0);
        volatile int4 *slot = ring + (t % cap);
        bool got = false;
        for (unsigned long long spins = 0;; ++spins) {
            int seq = 0, pend = 0;
            if (lane == 0) {
                seq = slot->w;
                pend = *reinterpret_cast<volatile int *>(&ctl->ncur);
            }
            seq = __shfl_sync(kSortFull, seq, 0);
            pend = __shfl_sync(kSortFull, pend, 0);
            if (seq == t + 1) {
                got = true;
                break;
            }
            if (pend == 0) break;
            if (spins > kRingSpinLimit) {
                if (lane == 0) atomicExch(err, kSortErrGuard);
                break;
            }
            __nanosleep(32);
        }
        if (!got) break;
        __threadfence_block();
        const int a = slot->x, b = slot->y, d = slot->z;
        if (d == 0) {
            if (lane == 0) heap_sort(x, a, b);
            __syncwarp();
        } else {
            const int cut = warp_partition(x, a, b, w, err);
            if (lane == 0) place_child(a, cut, d - 1, big_next, w, ring, cap, ctl, err);
            if (lane == 1) place_child(cut, b, d - 1, big_next, w, ring, cap, ctl, err);
            const int la = lane < 16u ? a : cut, len = lane < 16u ? cut - a : b - cut;
            halfwarp_leaf_sort(x, la, len <= 16 ? len : 0);
        }
        __syncwarp();
        if (lane == 0) atomicSub(&ctl->ncur, 1);
    }
    __syncthreads();
}

} // namespace dev
} // namespace pgx
