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
//  - A warp partitions its range without scratch: the sequential loop swaps
//    the i-th "left stopper" (position p > first with !(x[p] < pivot), in
//    ascending order) with the i-th "right stopper" (!(pivot < x[p]), in
//    descending order) for as long as the former lies below the latter, and
//    returns min(next left stopper, last swapped right stopper) -- the first
//    left stopper if nothing was swapped. The warp finds the stoppers with
//    ballots over 32-position chunks taken alternately from both ends (each
//    chunk clipped, when it is loaded, to positions no swap has touched, so
//    its flags are those of the original values) and pairs them in order.
//  - Ranges of 16 or fewer elements are final: the closing insertion sort of
//    the whole array moves no element across a partition boundary, so it
//    equals an insertion sort of each such range, done by one lane.
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
    int take;  // next range of the current level
    int ncur;  // ranges in the current level
    int nnext; // ranges queued for the next level
    int pad;
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

// One warp: median-of-three into `first`, then the Hoare partition of
// [first+1, last) around it; returns the cut. `slots` is 64 ints of this
// warp's shared memory. All 32 lanes call it with the same arguments.
template <typename K>
__device__ int warp_partition(const sort_view<K> &x, int first, int last, int *slots, int *err)
{
    const unsigned lane = threadIdx.x & 31u;
    if (lane == 0) median_to_first(x, first, first + 1, first + (last - first) / 2, last - 1);
    __syncwarp();
    const K pv = x.k[first];
    int lo = first + 1, hi = last - 1; // next unscanned position from each end
    int lastL = first, lastR = last;   // last swapped left / right stopper
    unsigned lmask = 0u, rmask = 0u;   // unpaired stoppers of the current chunks
    int lbase = 0, rbase = 0;
    const unsigned below = (1u << lane) - 1u;
    // every pass either pairs a stopper or returns; chunk loads advance lo/hi
    for (int pass = 0; pass <= last - first; ++pass) {
        while (lmask == 0u && lo < lastR) {
            const int p = lo + static_cast<int>(lane);
            const bool st = p < lastR && !key_less(x.k[p], pv);
            lmask = __ballot_sync(kSortFull, st);
            lbase = lo;
            lo = min(lo + 32, lastR);
        }
        if (lmask == 0u) {
            // no left stopper below the last swapped right stopper
            if (lastR == last) {
                if (lane == 0) atomicExch(err, kSortErrNoSentinel);
                return last - 1;
            }
            return lastR;
        }
        while (rmask == 0u && hi > lastL) {
            const int p = hi - static_cast<int>(lane);
            const bool st = p > lastL && !key_less(pv, x.k[p]);
            rmask = __ballot_sync(kSortFull, st);
            rbase = hi;
            hi = max(hi - 32, lastL);
        }
        if (rmask == 0u) return min(lbase + __ffs(lmask) - 1, lastR);
        const int mm = min(__popc(lmask), __popc(rmask));
        if ((lmask >> lane) & 1u) {
            const int r = __popc(lmask & below);
            if (r < mm) slots[r] = lbase + static_cast<int>(lane);
        }
        if ((rmask >> lane) & 1u) {
            const int r = __popc(rmask & below);
            if (r < mm) slots[32 + r] = rbase - static_cast<int>(lane);
        }
        __syncwarp();
        int lp = 0, rp = 0;
        bool ok = false;
        if (static_cast<int>(lane) < mm) {
            lp = slots[lane];
            rp = slots[32 + lane];
            ok = lp < rp;
        }
        // left positions ascend and right ones descend with the pair index, so
        // the pairs that may swap are a prefix
        const int v = __popc(__ballot_sync(kSortFull, ok));
        if (ok) x.swap(lp, rp);
        __syncwarp();
        if (v > 0) {
            lastL = __shfl_sync(kSortFull, lp, v - 1);
            lastR = __shfl_sync(kSortFull, rp, v - 1);
        }
        if (v < mm) return min(__shfl_sync(kSortFull, lp, v), lastR);
        for (int j = 0; j < mm; ++j) {
            lmask &= lmask - 1u;
            rmask &= rmask - 1u;
        }
    }
    if (lane == 0) atomicExch(err, kSortErrGuard);
    return last - 1;
}

// Sorts x[0 .. n) by key with std::sort's order of ties. Every thread of the
// block calls it (blockDim.x a multiple of 32). lists: 2 * list_cap ranges
// (list_cap >= n / 17 + 1); slots_all: 64 ints per warp of shared memory; ctl
// in shared memory. Ends with a __syncthreads.
template <typename K>
__device__ void block_std_sort(const sort_view<K> &x, int n, int2 *lists, int list_cap, sort_ctl *ctl, int *slots_all,
                               int *err)
{
    const unsigned lane = threadIdx.x & 31u;
    int *slots = slots_all + (threadIdx.x >> 5) * 64;
    if (n <= 16) {
        if (threadIdx.x == 0 && n > 1) insertion_sort(x, 0, n);
        __syncthreads();
        return;
    }
    int depth = 2 * floor_log2_int(n);
    int2 *cur = lists, *nxt = lists + list_cap;
    if (threadIdx.x == 0) {
        cur[0] = make_int2(0, n);
        ctl->ncur = 1;
    }
    __syncthreads();
    for (;;) {
        const int ncur = ctl->ncur;
        if (ncur == 0) break;
        __syncthreads();
        if (threadIdx.x == 0) {
            ctl->take = 0;
            ctl->nnext = 0;
        }
        __syncthreads();
        for (;;) {
            int t = 0;
            if (lane == 0) t = atomicAdd(&ctl->take, 1);
            t = __shfl_sync(kSortFull, t, 0);
            if (t >= ncur) break;
            const int2 r = cur[t];
            if (depth == 0) {
                if (lane == 0) heap_sort(x, r.x, r.y);
                __syncwarp();
                continue;
            }
            const int cut = warp_partition(x, r.x, r.y, slots, err);
            if (lane < 2u) {
                const int a = lane == 0 ? r.x : cut, b = lane == 0 ? cut : r.y;
                if (b - a > 16) {
                    const int slot = atomicAdd(&ctl->nnext, 1);
                    if (slot < list_cap)
                        nxt[slot] = make_int2(a, b);
                    else
                        atomicExch(err, kSortErrListFull);
                } else {
                    insertion_sort(x, a, b);
                }
            }
            __syncwarp();
        }
        __syncthreads();
        if (threadIdx.x == 0) ctl->ncur = min(ctl->nnext, list_cap);
        int2 *t = cur;
        cur = nxt;
        nxt = t;
        --depth;
        __syncthreads();
    }
    __syncthreads();
}

} // namespace dev
} // namespace pgx
