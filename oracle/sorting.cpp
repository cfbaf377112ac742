// CPU oracle, part 2 (TEST INFRASTRUCTURE ONLY): the orderings of the
// reference's multi-objective utilities.
//
// pagmo sorts with std::sort (crowding_distance, multi_objective.cpp:301-306;
// select_best_N_mo, :386-389; sort_population_mo, :455-462). std::sort is not
// stable, so which of two tied elements comes first is decided by the standard
// library's algorithm: here GNU libstdc++ (GCC 13, bits/stl_algo.h), the library
// the reference is built against in this container and on the GPU hosts. Its
// published algorithm is introsort:
//   __introsort_loop(first, last, 2*floor(log2(n))):
//     while last - first > 16:
//       depth == 0 -> heapsort the range (make_heap + sort_heap), return
//       --depth; median of (first+1, mid, last-1) swapped into first,
//       cut = Hoare partition of [first+1, last) around *first;
//       recurse on [cut, last); last = cut
//   then one insertion sort over the whole array.
// orc_introsort_keys restates it; orc_introsort_chunked_keys and
// orc_introsort_lists_keys restate it with the partition computed the two ways
// the GPU does (stoppers paired in 32-wide chunks; complete stopper lists);
// all three are checked against std::sort by the tests.
#include "oracle.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <string>
#include <vector>

namespace
{
thread_local std::string g_err2;
thread_local uint64_t g_depth_limit_hits = 0; // introsort ranges that fell back to heapsort

using key_t = long long;

struct arr {
    key_t *k;
    int32_t *v;
    void swap(long a, long b)
    {
        std::swap(k[a], k[b]);
        std::swap(v[a], v[b]);
    }
};

inline long floor_log2(long n)
{
    long r = 0;
    while (n > 1) {
        n >>= 1;
        ++r;
    }
    return r;
}

// libstdc++ __move_median_to_first(result, a, b, c).
void median_to_first(arr &x, long result, long a, long b, long c)
{
    const key_t *k = x.k;
    if (k[a] < k[b]) {
        if (k[b] < k[c])
            x.swap(result, b);
        else if (k[a] < k[c])
            x.swap(result, c);
        else
            x.swap(result, a);
    } else if (k[a] < k[c])
        x.swap(result, a);
    else if (k[b] < k[c])
        x.swap(result, c);
    else
        x.swap(result, b);
}

// libstdc++ __unguarded_partition(first + 1, last, pivot = first).
long hoare_partition(arr &x, long first, long last)
{
    const key_t pv = x.k[first];
    long lo = first + 1, hi = last;
    while (true) {
        while (x.k[lo] < pv) ++lo;
        --hi;
        while (pv < x.k[hi]) --hi;
        if (!(lo < hi)) return lo;
        x.swap(lo, hi);
        ++lo;
    }
}

// The same cut and the same swaps, found the GPU's way. Left stoppers are the
// positions p >= first+1 with !(k[p] < pivot), right stoppers the positions
// with !(pivot < k[p]); the sequential loop swaps the i-th left stopper with
// the i-th right stopper (left ascending, right descending) while the former
// lies below the latter, and returns min(next left stopper, last swapped right
// stopper) -- or the first left stopper when nothing was swapped. Chunks of 32
// positions are scanned from each side, each clipped at load time to the part
// no swap has touched yet (so every stopper flag is the one of the original
// value), and their stoppers are paired in order.
long chunked_partition(arr &x, long first, long last)
{
    const key_t pv = x.k[first];
    long lo = first + 1, hi = last - 1, lastL = first, lastR = last;
    unsigned lmask = 0, rmask = 0;
    long lbase = 0, rbase = 0;
    while (true) {
        while (lmask == 0u && lo < lastR) {
            for (int lane = 0; lane < 32; ++lane) {
                const long p = lo + lane;
                if (p < lastR && !(x.k[p] < pv)) lmask |= 1u << lane;
            }
            lbase = lo;
            lo = std::min(lo + 32, lastR);
        }
        if (lmask == 0u) return lastR;
        while (rmask == 0u && hi > lastL) {
            for (int lane = 0; lane < 32; ++lane) {
                const long p = hi - lane;
                if (p > lastL && !(pv < x.k[p])) rmask |= 1u << lane;
            }
            rbase = hi;
            hi = std::max(hi - 32, lastL);
        }
        if (rmask == 0u) return std::min(lbase + __builtin_ctz(lmask), lastR);
        long lp[32], rp[32];
        int nl = 0, nr = 0;
        for (int b = 0; b < 32; ++b) {
            if ((lmask >> b) & 1u) lp[nl++] = lbase + b;
            if ((rmask >> b) & 1u) rp[nr++] = rbase - b;
        }
        const int mm = std::min(nl, nr);
        int v = 0;
        while (v < mm && lp[v] < rp[v]) ++v;
        for (int j = 0; j < v; ++j) x.swap(lp[j], rp[j]);
        if (v > 0) {
            lastL = lp[v - 1];
            lastR = rp[v - 1];
        }
        if (v < mm) return std::min(lp[v], lastR);
        for (int j = 0; j < mm; ++j) {
            lmask &= lmask - 1u;
            rmask &= rmask - 1u;
        }
    }
}

// The same cut and swaps from the complete stopper lists (the GPU's
// formulation for long ranges): left stoppers L[0..nl) ascending and right
// stoppers R[0..nr) descending, all flagged on the original values; K = the
// number of i with L[i] < R[i] (a prefix), swap those K pairs, cut =
// min(L[K], R[K-1]), or L[0] when K = 0.
long lists_partition(arr &x, long first, long last)
{
    const key_t pv = x.k[first];
    std::vector<long> L, R;
    for (long p = first + 1; p < last; ++p)
        if (!(x.k[p] < pv)) L.push_back(p);
    for (long p = last - 1; p > first; --p)
        if (!(pv < x.k[p])) R.push_back(p);
    size_t K = 0;
    while (K < L.size() && K < R.size() && L[K] < R[K]) ++K;
    for (size_t i = 0; i < K; ++i) x.swap(L[i], R[i]);
    if (K == 0) return L[0];
    return K < L.size() ? std::min(L[K], R[K - 1]) : R[K - 1];
}

// libstdc++ __adjust_heap / __push_heap on x[first .. first+len).
void adjust_heap(arr &x, long first, long hole, long len, key_t vk, int32_t vv)
{
    const long top = hole;
    long child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (x.k[first + child] < x.k[first + child - 1]) --child;
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
    long parent = (hole - 1) / 2;
    while (hole > top && x.k[first + parent] < vk) {
        x.k[first + hole] = x.k[first + parent];
        x.v[first + hole] = x.v[first + parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    x.k[first + hole] = vk;
    x.v[first + hole] = vv;
}

// std::__partial_sort(first, last, last): make_heap then sort_heap.
void heap_sort(arr &x, long first, long last)
{
    const long len = last - first;
    if (len >= 2) {
        long parent = (len - 2) / 2;
        while (true) {
            adjust_heap(x, first, parent, len, x.k[first + parent], x.v[first + parent]);
            if (parent == 0) break;
            --parent;
        }
    }
    for (long l = len; l > 1;) {
        --l;
        const key_t vk = x.k[first + l];
        const int32_t vv = x.v[first + l];
        x.k[first + l] = x.k[first];
        x.v[first + l] = x.v[first];
        adjust_heap(x, first, 0, l, vk, vv);
    }
}

void insertion_sort(arr &x, long first, long last)
{
    for (long i = first + 1; i < last; ++i) {
        const key_t vk = x.k[i];
        const int32_t vv = x.v[i];
        long j = i;
        while (j > first && vk < x.k[j - 1]) {
            x.k[j] = x.k[j - 1];
            x.v[j] = x.v[j - 1];
            --j;
        }
        x.k[j] = vk;
        x.v[j] = vv;
    }
}

// Partition formulation of a restated introsort.
enum class part { hoare, chunked, lists };

template <part P>
void introsort_loop(arr &x, long first, long last, long depth)
{
    while (last - first > 16) {
        if (depth == 0) {
            ++g_depth_limit_hits;
            heap_sort(x, first, last);
            return;
        }
        --depth;
        median_to_first(x, first, first + 1, first + (last - first) / 2, last - 1);
        const long cut = P == part::chunked ? chunked_partition(x, first, last)
                         : P == part::lists ? lists_partition(x, first, last)
                                            : hoare_partition(x, first, last);
        introsort_loop<P>(x, cut, last, depth);
        last = cut;
    }
}

template <part P>
void introsort(key_t *k, int32_t *v, long n)
{
    if (n < 2) return;
    arr x{k, v};
    introsort_loop<P>(x, 0, n, 2 * floor_log2(n));
    insertion_sort(x, 0, n);
}

// NaN-aware orders of include/pagmo/detail/custom_comparisons.hpp:54-89.
inline bool lt_f(double a, double b)
{
    if (!std::isnan(a)) return std::isnan(b) ? true : a < b;
    return false;
}
inline bool gt_f(double a, double b)
{
    if (!std::isnan(a)) return std::isnan(b) ? false : a > b;
    return !std::isnan(b);
}

} // namespace

extern "C" {

const char *orc_sort_last_error(void)
{
    return g_err2.c_str();
}

// Number of ranges the restated introsorts of this thread handed to heapsort.
uint64_t orc_depth_limit_hits(void)
{
    return g_depth_limit_hits;
}

void orc_std_sort_keys(long long *k, int32_t *v, uint64_t n)
{
    std::vector<uint64_t> o(n);
    std::iota(o.begin(), o.end(), uint64_t(0));
    std::sort(o.begin(), o.end(), [k](uint64_t a, uint64_t b) { return k[a] < k[b]; });
    std::vector<long long> k2(n);
    std::vector<int32_t> v2(n);
    for (uint64_t i = 0; i < n; ++i) {
        k2[i] = k[o[i]];
        v2[i] = v[o[i]];
    }
    std::copy(k2.begin(), k2.end(), k);
    std::copy(v2.begin(), v2.end(), v);
}

void orc_introsort_keys(long long *k, int32_t *v, uint64_t n)
{
    introsort<part::hoare>(k, v, static_cast<long>(n));
}

void orc_introsort_chunked_keys(long long *k, int32_t *v, uint64_t n)
{
    introsort<part::chunked>(k, v, static_cast<long>(n));
}

void orc_introsort_lists_keys(long long *k, int32_t *v, uint64_t n)
{
    introsort<part::lists>(k, v, static_cast<long>(n));
}

void orc_heap_sort_keys(long long *k, int32_t *v, uint64_t n)
{
    arr x{k, v};
    heap_sort(x, 0, static_cast<long>(n));
}

void orc_std_partial_sort_full(long long *k, int32_t *v, uint64_t n)
{
    std::vector<uint64_t> o(n);
    std::iota(o.begin(), o.end(), uint64_t(0));
    std::partial_sort(o.begin(), o.end(), o.end(), [k](uint64_t a, uint64_t b) { return k[a] < k[b]; });
    std::vector<long long> k2(n);
    std::vector<int32_t> v2(n);
    for (uint64_t i = 0; i < n; ++i) {
        k2[i] = k[o[i]];
        v2[i] = v[o[i]];
    }
    std::copy(k2.begin(), k2.end(), k);
    std::copy(v2.begin(), v2.end(), v);
}

// McIlroy's adversary ("A Killer Adversary for Quicksort", Software: Practice
// and Experience 29(4), 1999): values are fixed lazily during a std::sort so
// that its pivots are as bad as possible; the values fixed by the end are an
// input that drives the introsort into its depth limit (heapsort).
void orc_quicksort_adversary(uint64_t n, long long *out)
{
    std::vector<long long> val(n, static_cast<long long>(n));
    const long long gas = static_cast<long long>(n);
    long long nsolid = 0;
    uint64_t candidate = 0;
    std::vector<uint64_t> ptr(n);
    std::iota(ptr.begin(), ptr.end(), uint64_t(0));
    std::sort(ptr.begin(), ptr.end(), [&](uint64_t x, uint64_t y) {
        if (val[x] == gas && val[y] == gas) {
            if (x == candidate)
                val[x] = nsolid++;
            else
                val[y] = nsolid++;
        }
        if (val[x] == gas)
            candidate = x;
        else if (val[y] == gas)
            candidate = y;
        return val[x] < val[y];
    });
    for (uint64_t i = 0; i < n; ++i) out[i] = val[i];
}

// select_best_N_mo (src/utils/multi_objective.cpp:344-396), restated over flat
// arrays with the reference's calls (fast_non_dominated_sorting, crowding
// distance with std::sort, std::sort by greater_than_f). out[*n_out].
int orc_select_best_n_mo(const double *pts, uint64_t n, uint64_t m, uint64_t N, uint64_t *out, uint64_t *n_out)
{
    *n_out = 0;
    if (N == 0u || n == 0u) return 0;
    if (n == 1u) {
        out[0] = 0;
        *n_out = 1;
        return 0;
    }
    if (N >= n) {
        for (uint64_t i = 0; i < n; ++i) out[i] = i;
        *n_out = n;
        return 0;
    }
    std::vector<uint64_t> rank(n), dc(n), off(n + 1), idx(n);
    uint64_t nf = 0;
    int st = orc_fnds(pts, n, m, rank.data(), dc.data(), off.data(), idx.data(), &nf, nullptr, nullptr, 0);
    if (st) {
        g_err2 = orc_last_error();
        return st;
    }
    uint64_t cnt = 0, f = 0;
    for (; f < nf; ++f) {
        const uint64_t sz = off[f + 1] - off[f];
        if (cnt + sz <= N) {
            for (uint64_t t = off[f]; t < off[f + 1]; ++t) out[cnt++] = idx[t];
            if (cnt == N) {
                *n_out = cnt;
                return 0;
            }
        } else {
            break;
        }
    }
    const uint64_t L = off[f + 1] - off[f];
    std::vector<double> buf(L * m), cds(L);
    for (uint64_t t = 0; t < L; ++t) std::memcpy(buf.data() + t * m, pts + idx[off[f] + t] * m, m * sizeof(double));
    st = orc_crowding(buf.data(), L, m, cds.data());
    if (st) {
        g_err2 = orc_last_error();
        return st;
    }
    std::vector<uint64_t> o(L);
    std::iota(o.begin(), o.end(), uint64_t(0));
    std::sort(o.begin(), o.end(), [&cds](uint64_t a, uint64_t b) { return gt_f(cds[a], cds[b]); });
    const uint64_t remaining = N - cnt;
    for (uint64_t i = 0; i < remaining; ++i) out[cnt++] = idx[off[f] + o[i]];
    *n_out = cnt;
    return 0;
}

// sort_population_mo (src/utils/multi_objective.cpp:425-465). out[n].
int orc_sort_population_mo(const double *pts, uint64_t n, uint64_t m, uint64_t *out)
{
    if (n == 0u) return 0;
    if (n == 1u) {
        out[0] = 0;
        return 0;
    }
    std::vector<uint64_t> rank(n), dc(n), off(n + 1), idx(n);
    uint64_t nf = 0;
    int st = orc_fnds(pts, n, m, rank.data(), dc.data(), off.data(), idx.data(), &nf, nullptr, nullptr, 0);
    if (st) {
        g_err2 = orc_last_error();
        return st;
    }
    std::vector<double> crowd(n), buf, cds;
    for (uint64_t f = 0; f < nf; ++f) {
        const uint64_t L = off[f + 1] - off[f];
        if (L == 1u) {
            crowd[idx[off[f]]] = 0.;
            continue;
        }
        buf.resize(L * m);
        cds.resize(L);
        for (uint64_t t = 0; t < L; ++t)
            std::memcpy(buf.data() + t * m, pts + idx[off[f] + t] * m, m * sizeof(double));
        st = orc_crowding(buf.data(), L, m, cds.data());
        if (st) {
            g_err2 = orc_last_error();
            return st;
        }
        for (uint64_t t = 0; t < L; ++t) crowd[idx[off[f] + t]] = cds[t];
    }
    std::vector<uint64_t> o(n);
    std::iota(o.begin(), o.end(), uint64_t(0));
    std::sort(o.begin(), o.end(), [&](uint64_t a, uint64_t b) {
        if (rank[a] == rank[b]) return gt_f(crowd[a], crowd[b]);
        return rank[a] < rank[b];
    });
    std::copy(o.begin(), o.end(), out);
    return 0;
}

} // extern "C"
