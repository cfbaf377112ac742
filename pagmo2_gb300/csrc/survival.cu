// NSGA-II survival on the GPU: fast non-dominated sorting
// (src/utils/multi_objective.cpp:200-257) and crowding distance (:280-315,
// applied per front as src/algorithms/nsga2.cpp:183-206 does).
//
// Pipeline (all on one stream):
//  1. order_keys: each objective value becomes an int64 key whose signed order
//     is the reference's NaN-aware order (include/pagmo/detail/
//     custom_comparisons.hpp:54-89): -0 and +0 are equal, every NaN sorts above
//     +inf and NaNs are equal to each other. Dominance then needs integer
//     compares only (the FP64 pipe of GB300 is narrow).
//  2. dominance_kernel: the "dominated-by" bit matrix Dt, row j holding bit i
//     when point i dominates point j, built 32x256 pairs per CTA with
//     __ballot_sync; dom_count[j] = popcount of row j.
//  3. peel2_kernel (peel_kernel beyond 131072 points): a cooperative
//     persistent kernel peels fronts. Front k+1 is
//     every unassigned point whose row has no unassigned dominator. The
//     reference's order inside a front (first front ascending; later fronts in
//     the order its dom_list traversal appends them) is rebuilt exactly: a
//     point q of front k+1 is appended when its last dominator in front k is
//     processed, so the order is by (max position of q's dominators in front k,
//     q).
//  4. front_crowding: one block per front sorts the front's members objective
//     after objective with std::sort's exact order (introsort.cuh; each sort
//     starts from the previous objective's order, as the reference's loop
//     does) and adds the reference's neighbour differences over the objective
//     range, in objective order per point.
// select_best_N_mo (:344-396) and sort_population_mo (:425-465) reuse 1-4 and
// the same sort.
#include "introsort.cuh"
#include "pgx_internal.cuh"

#include <algorithm>
#include <climits>
#include <cmath>

namespace pgx
{
namespace
{

constexpr unsigned kFull = 0xffffffffu;
constexpr unsigned long long kSpinLimit = 1ull << 24; // x (64 ns sleep + a poll): a second or more

__device__ __forceinline__ long long order_key(double v)
{
    if (isnan(v)) return LLONG_MAX;
    if (v == 0.0) return 0;
    const long long b = __double_as_longlong(v);
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

__global__ void order_keys_kernel(const double *__restrict__ pts, uint32_t n, uint32_t m, long long *__restrict__ keys)
{
    const uint64_t total = static_cast<uint64_t>(n) * m;
    for (uint64_t t = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < total;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint32_t i = static_cast<uint32_t>(t / m), k = static_cast<uint32_t>(t - static_cast<uint64_t>(i) * m);
        keys[static_cast<uint64_t>(k) * n + i] = order_key(pts[t]);
    }
}

// a dominates b: no objective worse, at least one better.
template <int M>
__device__ __forceinline__ bool dom_fixed(const long long (&a)[M], const long long *b, int stride)
{
    bool le = true, lt = false;
#pragma unroll
    for (int k = 0; k < M; ++k) {
        const long long bv = b[k * stride];
        le &= a[k] <= bv;
        lt |= a[k] < bv;
    }
    return le && lt;
}

// Symmetric tiles for 1 <= m <= 4: one warp compares a block of 32 points i
// (its lanes) with a block of 32 points j (staged in shared memory) for
// I-block <= J-block only. Per objective two compares, a_i < a_j and
// a_i > a_j, give both directions: i dominates j iff no ">" and some "<",
// j dominates i iff no "<" and some ">". The i-dominates-j bits of the 32 rows
// j come from ballots (one word per row, coalesced through shared memory);
// the j-dominates-i bits of each lane's row i collect in a register word.
// A diagonal tile writes its rows once. dom_count comes from a popcount pass.
template <int M>
__global__ void __launch_bounds__(256) dominance_sym_kernel(const long long *__restrict__ keys, uint32_t n,
                                                            uint32_t W8, uint32_t *__restrict__ Dt)
{
    __shared__ long long jk[M][32];
    __shared__ uint32_t tile[32][9];
    const uint32_t bj = blockIdx.y;              // J-block
    const uint32_t bi0 = blockIdx.x * 8u;        // first I-block of this CTA
    if (bi0 > bj) return;                        // whole CTA above the diagonal
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t J0 = bj * 32u;
    for (unsigned t = threadIdx.x; t < static_cast<unsigned>(M) * 32u; t += blockDim.x) {
        const unsigned k = t >> 5, jj = t & 31u;
        const uint32_t j = J0 + jj;
        jk[k][jj] = j < n ? keys[static_cast<uint64_t>(k) * n + j] : 0;
    }
    __syncthreads();
    const uint32_t bi = bi0 + warp;
    const bool active = bi <= bj;                // warp-uniform
    const uint32_t i = bi * 32u + lane;
    const bool iv = active && i < n;
    long long ik[M];
#pragma unroll
    for (int k = 0; k < M; ++k) ik[k] = iv ? keys[static_cast<uint64_t>(k) * n + i] : 0;
    uint32_t row_i = 0u; // bit jj: j = J0 + jj dominates i
    if (active) {
        for (unsigned jj = 0; jj < 32u; ++jj) {
            bool any_lt = false, any_gt = false;
#pragma unroll
            for (int k = 0; k < M; ++k) {
                const long long b = jk[k][jj];
                any_lt |= ik[k] < b;
                any_gt |= ik[k] > b;
            }
            const bool valid = iv && J0 + jj < n;
            const bool i_dom_j = valid && any_lt && !any_gt;
            const bool j_dom_i = valid && any_gt && !any_lt;
            const unsigned word = __ballot_sync(kFull, i_dom_j);
            if (lane == 0) tile[jj][warp] = word;
            row_i |= static_cast<uint32_t>(j_dom_i) << jj;
        }
        // the rows i of an off-diagonal tile: word J-block of row i
        if (bi != bj && i < n) Dt[static_cast<uint64_t>(i) * W8 + bj] = row_i;
    }
    __syncthreads();
    // the rows j: words bi0 .. bi0+7 of rows J0 .. J0+31 (blocks at or below the diagonal)
    const unsigned jj = threadIdx.x >> 3, ww = threadIdx.x & 7u;
    const uint32_t j = J0 + jj;
    if (j < n && bi0 + ww <= bj) Dt[static_cast<uint64_t>(j) * W8 + bi0 + ww] = tile[jj][ww];
}

// dom_count[j] = popcount of row j of Dt (one warp per row).
__global__ void row_popcount_kernel(const uint32_t *__restrict__ Dt, uint32_t n, uint32_t W8,
                                    int32_t *__restrict__ dom_count)
{
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t warps = static_cast<uint64_t>(gridDim.x) * (blockDim.x >> 5);
    for (uint64_t r = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
        int c = 0;
        for (uint32_t w = lane; w < W8; w += 32u) c += __popc(Dt[r * W8 + w]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(kFull, c, o);
        if (lane == 0) dom_count[r] = c;
    }
}

// ------------------------------------------------ packed-rank dominance
//
// For n <= kRankPoints and m <= 4 the dominance tiles compare ranks instead of
// 64-bit order keys: the rank of a point in objective k is the number of
// points with a smaller key there (equal keys, equal ranks, so the order and
// the ties of every objective are kept, and with them the dominance relation).
// Ranks are below 2^15; two share a 32-bit word as 16-bit fields whose top bit
// is a guard: for words a and b, ((b | G) - a) & G == G exactly when no field
// of a exceeds b's (a field's subtraction borrows from its guard bit only
// then, and never from the next field). So "no objective worse" costs one
// OR, one subtraction and one AND per word, for both directions of a pair.
constexpr uint32_t kRankPoints = 32768;
constexpr uint32_t kRankRun = 1024; // keys per sorted run
constexpr uint32_t kRankGuard = 0x80008000u;

// Sorted runs of kRankRun keys of each objective (bitonic network in shared
// memory; grid: runs x objectives).
__global__ void __launch_bounds__(kRankRun / 2) rank_runs_kernel(const long long *__restrict__ keys, uint32_t n,
                                                                 long long *__restrict__ runs)
{
    __shared__ long long sk[kRankRun];
    const uint32_t k = blockIdx.y, nb = gridDim.x;
    const uint32_t t0 = blockIdx.x * kRankRun;
    for (uint32_t j = threadIdx.x; j < kRankRun; j += blockDim.x) {
        const uint32_t t = t0 + j;
        sk[j] = t < n ? keys[static_cast<uint64_t>(k) * n + t] : LLONG_MAX;
    }
    __syncthreads();
    for (uint32_t size = 2; size <= kRankRun; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t j = threadIdx.x; j < kRankRun / 2u; j += blockDim.x) {
                const uint32_t lo = 2u * stride * (j / stride) + (j % stride), hi = lo + stride;
                const bool up = (lo & size) == 0u;
                const long long a = sk[lo], b = sk[hi];
                if ((b < a) == up) {
                    sk[lo] = b;
                    sk[hi] = a;
                }
            }
            __syncthreads();
        }
    }
    long long *out = runs + (static_cast<uint64_t>(k) * nb + blockIdx.x) * kRankRun;
    for (uint32_t j = threadIdx.x; j < kRankRun; j += blockDim.x) out[j] = sk[j];
}

// Each point's ranks (keys below its own, summed over the runs), added into
// the packed words pa = r0 | r1 << 16, pb = r2 | r3 << 16 (zeroed before):
// block (run b of objective k, chunk c of the points) holds the run in shared
// memory and counts, for each point of the chunk, the run's keys below the
// point's key by binary search (the padding keys LLONG_MAX are never below a
// point's key: NaN's key is LLONG_MAX too). A field's sum is the rank, below
// 2^15, so the additions never carry into the next field.
__global__ void __launch_bounds__(256) rank_search_kernel(const long long *__restrict__ keys, uint32_t n,
                                                          const long long *__restrict__ runs, uint32_t nb,
                                                          uint32_t *__restrict__ pa, uint32_t *__restrict__ pb)
{
    __shared__ long long sk[kRankRun];
    const uint32_t k = blockIdx.y / nb, b = blockIdx.y - k * nb;
    const long long *run = runs + (static_cast<uint64_t>(k) * nb + b) * kRankRun;
    for (uint32_t j = threadIdx.x; j < kRankRun; j += blockDim.x) sk[j] = run[j];
    __syncthreads();
    uint32_t *dst = (k >> 1) ? pb : pa;
    const uint32_t shift = 16u * (k & 1u);
    const uint32_t t1 = min(n, (blockIdx.x + 1u) * 1024u);
    for (uint32_t t = blockIdx.x * 1024u + threadIdx.x; t < t1; t += blockDim.x) {
        const long long x = keys[static_cast<uint64_t>(k) * n + t];
        uint32_t lo = 0;
#pragma unroll
        for (uint32_t step = kRankRun / 2u; step > 0; step >>= 1)
            if (sk[lo + step - 1u] < x) lo += step;
        lo += sk[lo] < x ? 1u : 0u;
        if (lo) atomicAdd(dst + t, lo << shift);
    }
}

// dominance_sym_kernel on packed ranks (NW = 1: m <= 2, NW = 2: m <= 4).
template <int NW>
__global__ void __launch_bounds__(256) dominance_sym_packed_kernel(const uint32_t *__restrict__ pa,
                                                                   const uint32_t *__restrict__ pb, uint32_t n,
                                                                   uint32_t W8, uint32_t *__restrict__ Dt)
{
    __shared__ uint4 jw[32]; // per candidate j: its words a, b and a | guard, b | guard
    __shared__ uint32_t tile[32][9];
    const uint32_t bj = blockIdx.y;
    const uint32_t bi0 = blockIdx.x * 8u;
    if (bi0 > bj) return;
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t J0 = bj * 32u;
    if (threadIdx.x < 32u) {
        const uint32_t j = J0 + threadIdx.x;
        const uint32_t a = j < n ? pa[j] : 0u, b = j < n && NW == 2 ? pb[j] : 0u;
        jw[threadIdx.x] = make_uint4(a, b, a | kRankGuard, b | kRankGuard);
    }
    __syncthreads();
    const uint32_t bi = bi0 + warp;
    const bool active = bi <= bj;
    const uint32_t i = bi * 32u + lane;
    const bool iv = active && i < n;
    const uint32_t ia = iv ? pa[i] : 0u, ib = iv && NW == 2 ? pb[i] : 0u;
    const uint32_t iag = ia | kRankGuard, ibg = ib | kRankGuard;
    const uint32_t jn = n - J0 < 32u ? n - J0 : 32u; // candidates of this tile
    uint32_t row_i = 0u;
    // pair (i, jj): i dominates jj / jj dominates i (valid: both points exist)
    const auto pair = [&](unsigned jj, bool valid, bool &i_dom_j, bool &j_dom_i) {
        const uint4 w = jw[jj];
        // no borrow into a guard bit: every field of the first word no smaller
        uint32_t c_ij = w.z - ia; // i no worse than j in every field
        uint32_t c_ji = iag - w.x; // j no worse than i
        if (NW == 2) {
            c_ij &= w.w - ib;
            c_ji &= ibg - w.y;
        }
        const bool le_ij = (c_ij & kRankGuard) == kRankGuard, le_ji = (c_ji & kRankGuard) == kRankGuard;
        // both ways no worse: every field equal, neither dominates
        i_dom_j = valid && le_ij && !le_ji;
        j_dom_i = valid && le_ji && !le_ij;
    };
    if (active) {
        if (jn == 32u && __all_sync(kFull, iv)) {
            // a full tile (nearly all of them): no validity tests per pair
#pragma unroll
            for (unsigned jj = 0; jj < 32u; ++jj) {
                bool idj, jdi;
                pair(jj, true, idj, jdi);
                const unsigned word = __ballot_sync(kFull, idj);
                if (lane == 0) tile[jj][warp] = word;
                row_i |= static_cast<uint32_t>(jdi) << jj;
            }
        } else {
            for (unsigned jj = 0; jj < 32u; ++jj) {
                bool idj, jdi;
                pair(jj, iv && jj < jn, idj, jdi);
                const unsigned word = __ballot_sync(kFull, idj);
                if (lane == 0) tile[jj][warp] = word;
                row_i |= static_cast<uint32_t>(jdi) << jj;
            }
        }
        if (bi != bj && i < n) Dt[static_cast<uint64_t>(i) * W8 + bj] = row_i;
    }
    __syncthreads();
    const unsigned jj = threadIdx.x >> 3, ww = threadIdx.x & 7u;
    const uint32_t j = J0 + jj;
    if (j < n && bi0 + ww <= bj) Dt[static_cast<uint64_t>(j) * W8 + bi0 + ww] = tile[jj][ww];
}

// CTA tile: 32 dominated candidates j (rows of Dt) x 256 dominators i (8 words).
// Warp w tests i = 32*(w0+w) + lane against each j and ballots the row word.
// M > 0: objectives in registers; M == 0: runtime m, keys read from global.
template <int M>
__global__ void __launch_bounds__(256) dominance_kernel(const long long *__restrict__ keys, uint32_t n, uint32_t m,
                                                        uint32_t W, uint32_t W8, uint32_t *__restrict__ Dt,
                                                        int32_t *__restrict__ dom_count)
{
    constexpr int MS = M > 0 ? M : 1;
    __shared__ long long jk[MS][32];
    __shared__ uint32_t tile[32][9];
    const uint32_t J0 = blockIdx.y * 32u;
    const uint32_t w0 = blockIdx.x * 8u;
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    if constexpr (M > 0) {
        for (unsigned t = threadIdx.x; t < static_cast<unsigned>(M) * 32u; t += blockDim.x) {
            const unsigned k = t >> 5, jj = t & 31u;
            const uint32_t j = J0 + jj;
            jk[k][jj] = j < n ? keys[static_cast<uint64_t>(k) * n + j] : 0;
        }
    }
    const uint32_t w = w0 + warp;
    const uint32_t i = w * 32u + lane;
    const bool iv = (w < W) && (i < n);
    long long ik[MS];
    if (M > 0) {
#pragma unroll
        for (int k = 0; k < MS; ++k) ik[k] = iv ? keys[static_cast<uint64_t>(k) * n + i] : 0;
    }
    __syncthreads();
    for (unsigned jj = 0; jj < 32u; ++jj) {
        const uint32_t j = J0 + jj;
        bool d = false;
        if (iv && j < n) {
            if (M > 0) {
                d = dom_fixed<MS>(ik, &jk[0][jj], 32);
            } else {
                bool le = true, lt = false;
                for (uint32_t k = 0; k < m; ++k) {
                    const long long a = keys[static_cast<uint64_t>(k) * n + i];
                    const long long b = keys[static_cast<uint64_t>(k) * n + j];
                    le &= a <= b;
                    lt |= a < b;
                }
                d = le && lt;
            }
        }
        const unsigned word = __ballot_sync(kFull, d);
        if (lane == 0) tile[jj][warp] = word;
    }
    __syncthreads();
    const unsigned jj = threadIdx.x >> 3, ww = threadIdx.x & 7u;
    const uint32_t j = J0 + jj;
    const uint32_t word = tile[jj][ww];
    if (j < n && w0 + ww < W8) Dt[static_cast<uint64_t>(j) * W8 + w0 + ww] = word;
    int c = __popc(word);
    c += __shfl_xor_sync(kFull, c, 4);
    c += __shfl_xor_sync(kFull, c, 2);
    c += __shfl_xor_sync(kFull, c, 1);
    if (ww == 0 && j < n && c) atomicAdd(&dom_count[j], c);
}

struct peel_state {
    unsigned bar_count;
    unsigned bar_gen;
    int err;      // a grid barrier gave up
    int n_fronts;
    int counts[2];
    int status;   // kStatusNeedTwoObjectives: crowding over fewer than two objectives
    int sort_err; // broken invariant of the device sort (never expected)
    int gs[72];   // grid sort: [0] shared-memory ranges, [1 + level] block-partitioned ranges per level
    int fronts_done; // fused crowding: fronts whose members and offsets are complete
    int peel_done;   // fused crowding: the peel has ended (n_fronts final)
    unsigned peel_arrivals; // peel_sync: arrivals so far (zero at the start of the pass)
};

constexpr int kStatusNeedTwoObjectives = 1;

// Grid-wide barrier for a cooperative launch (of its first nblocks blocks, all
// of them when 0); gives up (and flags st->err) after about a second
// (spin_limit polls) instead of waiting forever.
__device__ bool grid_sync(peel_state *st, unsigned long long spin_limit = kSpinLimit, unsigned nblocks = 0)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = &st->bar_gen;
        const unsigned g0 = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(&st->bar_count, 1u);
        if (arrived == (nblocks ? nblocks : gridDim.x) - 1u) {
            atomicExch(&st->bar_count, 0u);
            __threadfence();
            atomicAdd(&st->bar_gen, 1u);
        } else {
            unsigned long long spins = 0;
            volatile int *verr = &st->err;
            while (*vgen == g0) {
                if (*verr) break; // another block gave up: do not wait for it
                if (++spins > spin_limit) {
                    atomicExch(&st->err, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *reinterpret_cast<volatile int *>(&st->err) == 0;
}

// The peel's barrier over its first nb blocks: one counter of arrivals that
// only grows (it starts at zero for the pass), so the last arrival itself
// releases the others (round r ends when the count reaches (r + 1) nb); no
// reset, no second atomic. Gives up like grid_sync.
__device__ bool peel_sync(peel_state *st, unsigned nb)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        // the arrival releases the block's writes (ordered before it by the
        // block barrier), the polls acquire the other blocks'
        unsigned a;
        asm volatile("atom.add.release.gpu.u32 %0, [%1], 1;" : "=r"(a) : "l"(&st->peel_arrivals) : "memory");
        const unsigned target = (a / nb + 1u) * nb;
        volatile int *verr = &st->err;
        for (unsigned long long spins = 0;; ++spins) {
            unsigned v;
            asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(v) : "l"(&st->peel_arrivals) : "memory");
            if (v >= target) break;
            if (*verr) break;
            if (spins > kSpinLimit) {
                atomicExch(&st->err, 1);
                break;
            }
            __nanosleep(16);
        }
    }
    __syncthreads();
    return *reinterpret_cast<volatile int *>(&st->err) == 0;
}

constexpr int kTile = 2048; // (key, index) pairs per shared-memory tile

// Front peeling, one front per iteration, two grid barriers per front.
//
// Phase A: every unassigned point j whose row of Dt has no unassigned
// dominator joins front k. Warps take 4-candidate slices of the rem bit set
// and scan each candidate's row cooperatively (256 words per step, early
// exit). A member's ordering key is the highest position, in front k-1, of
// one of its dominators: a reverse scan over front k-1's positions (staged in
// shared memory; 128 at a time, ballots) stops at the first hit.
// Phase C: the position of a member is the number of members with a smaller
// (key, index), counted against shared-memory tiles; members are written to
// front_indices, ranked, and cleared from rem.
constexpr int kPeelThreads = 1024; // one block per SM: few arrivals per grid barrier
constexpr int kLocalMembers = 1024; // members a block collects before one global append
constexpr int kRemWords = 4096;     // rem staged in shared memory up to 131072 points

__global__ void __launch_bounds__(kPeelThreads) peel_kernel(const uint32_t *__restrict__ Dt, uint32_t n, uint32_t W,
                                                            uint32_t W8, uint32_t *rem, int32_t *list, int32_t *keyv,
                                                            int32_t *rank, int32_t *front_offsets,
                                                            int32_t *front_indices, peel_state *st)
{
    extern __shared__ int32_t sh[]; // kTile keys, then kTile indices
    __shared__ int32_t s_list[kLocalMembers], s_key[kLocalMembers];
    __shared__ uint32_t s_rem[kRemWords];
    __shared__ int s_cnt, s_base;
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthreads = gridDim.x * blockDim.x;
    const uint32_t gwarp = tid >> 5, nwarps = nthreads >> 5;
    int off = 0, off_prev = 0, size_prev = 0;
    int k = 0;
    for (;; ++k) {
        int *cnt = &st->counts[k & 1];
        // front k-1's members, by position, in shared memory when they fit
        const bool prev_in_smem = size_prev <= 2 * kTile;
        if (k > 0 && prev_in_smem)
            for (int t = threadIdx.x; t < size_prev; t += blockDim.x) sh[t] = __ldcg(front_indices + off_prev + t);
        // the unassigned set, read by every row scan of this phase
        const bool rem_in_smem = W <= static_cast<uint32_t>(kRemWords);
        if (rem_in_smem)
            for (uint32_t w = threadIdx.x; w < W; w += blockDim.x) s_rem[w] = __ldcg(rem + w);
        if (threadIdx.x == 0) s_cnt = 0;
        __syncthreads();
        // ---- Phase A (tasks: 4-candidate slices of the rem bit set)
        const uint32_t tasks = W * 8u;
        for (uint32_t t = gwarp; t < tasks; t += nwarps) {
            const uint32_t w = t >> 3, sub = t & 7u;
            uint32_t cand = (__ldcg(rem + w) >> (sub * 4u)) & 0xfu;
            while (cand) {
                const uint32_t b = static_cast<uint32_t>(__ffs(cand) - 1);
                cand &= cand - 1u;
                const uint32_t j = w * 32u + sub * 4u + b;
                const uint32_t *row = Dt + static_cast<uint64_t>(j) * W8;
                bool hit = false;
                for (uint32_t base = 0; base < W; base += 256u) { // 8 independent loads per lane
                    uint32_t v = 0u;
#pragma unroll
                    for (uint32_t u = 0; u < 8u; ++u) {
                        const uint32_t ww = base + u * 32u + lane;
                        if (ww < W) v |= __ldg(row + ww) & (rem_in_smem ? s_rem[ww] : __ldcg(rem + ww));
                    }
                    if (__any_sync(kFull, v != 0u)) {
                        hit = true;
                        break;
                    }
                }
                if (hit) continue;
                int key = 0;
                if (k > 0) {
                    key = -1;
                    for (int top = size_prev - 1; top >= 0 && key < 0; top -= 128) { // 4 x 32 positions per step
                        unsigned bal[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const int p = top - 32 * u - static_cast<int>(lane);
                            bool h = false;
                            if (p >= 0) {
                                const uint32_t d = static_cast<uint32_t>(
                                    prev_in_smem ? sh[p] : __ldcg(front_indices + off_prev + p));
                                h = (__ldg(row + (d >> 5)) >> (d & 31u)) & 1u;
                            }
                            bal[u] = __ballot_sync(kFull, h);
                        }
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            if (key < 0 && bal[u]) key = top - 32 * u - (__ffs(bal[u]) - 1);
                        }
                    }
                }
                if (lane == 0) {
                    const int ls = atomicAdd(&s_cnt, 1);
                    if (ls < kLocalMembers) {
                        s_list[ls] = static_cast<int32_t>(j);
                        s_key[ls] = key;
                    } else {
                        const int s = atomicAdd(cnt, 1);
                        list[s] = static_cast<int32_t>(j);
                        keyv[s] = key;
                    }
                }
            }
        }
        // one global append per block
        __syncthreads();
        const int local = min(s_cnt, kLocalMembers);
        if (threadIdx.x == 0) s_base = local ? atomicAdd(cnt, local) : 0;
        __syncthreads();
        for (int t = threadIdx.x; t < local; t += blockDim.x) {
            list[s_base + t] = s_list[t];
            keyv[s_base + t] = s_key[t];
        }
        if (!grid_sync(st)) {
            if (threadIdx.x == 0) atomicExch(&st->n_fronts, -1);
            return;
        }
        const int L = *reinterpret_cast<volatile int *>(cnt);
        if (L == 0) break;
        // ---- Phase C
        if (L <= kTile) {
            // the whole front in shared memory; one warp per member, lanes
            // splitting the comparisons
            for (int t = threadIdx.x; t < L; t += blockDim.x) {
                sh[t] = __ldcg(keyv + t);
                sh[kTile + t] = __ldcg(list + t);
            }
            __syncthreads();
            for (uint32_t s = gwarp; s < static_cast<uint32_t>(L); s += nwarps) {
                const int q = sh[kTile + s], kq = sh[s];
                int p = 0;
                for (int t = static_cast<int>(lane); t < L; t += 32) {
                    const int kt = sh[t], qt = sh[kTile + t];
                    p += (kt < kq) | ((kt == kq) & (qt < q));
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(kFull, p, o);
                if (lane == 0) {
                    front_indices[off + p] = q;
                    rank[q] = k;
                    atomicAnd(rem + (q >> 5), ~(1u << (q & 31)));
                }
            }
        } else {
        // large fronts: one thread per member against shared-memory tiles (the
        // loop bound is uniform per block, so __syncthreads is safe)
        for (uint32_t s0 = blockIdx.x * blockDim.x; s0 < static_cast<uint32_t>(L); s0 += nthreads) {
            const uint32_t s = s0 + threadIdx.x;
            const bool act = s < static_cast<uint32_t>(L);
            const int q = act ? __ldcg(list + s) : 0;
            const int kq = act ? __ldcg(keyv + s) : 0;
            int p = 0;
            for (int t0 = 0; t0 < L; t0 += kTile) {
                const int lim = min(kTile, L - t0);
                __syncthreads();
                for (int t = threadIdx.x; t < lim; t += blockDim.x) {
                    sh[t] = __ldcg(keyv + t0 + t);
                    sh[kTile + t] = __ldcg(list + t0 + t);
                }
                __syncthreads();
                if (act) {
                    for (int t = 0; t < lim; ++t) {
                        const int kt = sh[t], qt = sh[kTile + t];
                        p += (kt < kq) | ((kt == kq) & (qt < q));
                    }
                }
            }
            if (act) {
                front_indices[off + p] = q;
                rank[q] = k;
                atomicAnd(rem + (q >> 5), ~(1u << (q & 31)));
            }
        }
        }
        if (tid == 0) {
            st->counts[(k + 1) & 1] = 0;
            front_offsets[k + 1] = off + L;
        }
        off_prev = off;
        size_prev = L;
        off += L;
        if (!grid_sync(st)) {
            if (threadIdx.x == 0) atomicExch(&st->n_fronts, -1);
            return;
        }
    }
    if (tid == 0) {
        // a barrier that gave up elsewhere leaves the fronts incomplete: report -1
        st->n_fronts = *reinterpret_cast<volatile int *>(&st->err) ? -1 : k;
        front_offsets[0] = 0;
    }
}

// Front peeling with witnesses and one grid barrier per front (n <= 131072
// points, the unassigned set staged in every block's shared memory).
//
// Front 0 is every point with no dominator: its members, in ascending index
// order (the reference's first front), come from the dom_count == 0 bit set
// and its prefix popcounts, which every block computes for itself.
// For k >= 1, Phase A finds the members of front k. Each unassigned point j
// keeps a witness wit[j], an unassigned dominator found earlier, and the
// resume word res[j], the first word of its row that held an unassigned
// dominator then (both in the shared memory of the block that owns j's word):
// while the witness stays unassigned, j is settled by one shared-memory bit
// test. When the witness is peeled, j's row of Dt is scanned again from
// res[j] (the words before it held no unassigned dominator, and the
// unassigned set only shrinks); no unassigned dominator left makes j a member
// of front k. Otherwise every lane proposes one unassigned dominator from the
// first nonzero word of its part of the scanned window and the new witness is
// the proposal with the most dominators itself, which is likely peeled late,
// so that j is rescanned seldom. A block first tests the witnesses of the points of its own rem
// words, queueing the points that need a scan, then its warps scan the queue.
// A member's ordering key is the highest position, in front k-1, of one of
// its dominators (the reference appends q when its last dominator in front
// k-1 is processed): for k = 1 the highest-index dominator among front 0's
// bits (positions there follow indices); for k >= 2 a reverse scan of front
// k-1 by position.
// After the barrier, every block loads the L members of front k and counts
// their positions (by key, then index) itself, clears them from its rem copy
// and keeps them by position for the next front's keys; block b writes
// front_indices and rank for the positions p with p % gridDim.x == b. No
// second barrier is needed: nothing of front k is read from global memory
// before the next barrier. A front larger than kTile takes the grid-wide
// counting of peel_kernel and a second barrier instead.
constexpr int kQueue = 4096; // witness rescans queued per block and front
// Up to this many points every block keeps the previous front's membership
// bits and each member's position there (16 bits) in shared memory, and a
// member's key comes out of its own row scan (no second pass over the row).
constexpr uint32_t kPosPoints = 32768;

// ------------------------------------------------------------ crowding and orders

constexpr int kSortThreads = 1024;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortSmemCap = 4096;                                // (key, value) pairs kept in shared memory
constexpr int kSortSmemSmall = kSortSmemCap / 16 + 2;             // short ranges per level list
constexpr int kSortSmemBig = kSortSmemCap / dev::kBlockRange + 2; // block-partitioned ranges per level list
constexpr size_t kSortSmemBytes = static_cast<size_t>(kSortSmemCap) * (sizeof(dev::key2) + 3u * sizeof(int32_t))
                                  + 2u * (kSortSmemSmall + kSortSmemBig) * sizeof(int2);

// Where one block sorts L pairs: its shared memory when they fit, else the
// caller's slices of the global work arrays (L keys, L values, L ranges, 2 L
// positions).
template <typename K>
struct sort_area {
    K *k;
    int32_t *v;
    dev::sort_work w;
};

template <typename K>
__device__ sort_area<K> pick_area(unsigned char *smem, int L, K *gk, int32_t *gv, int2 *gl, int32_t *gpos)
{
    sort_area<K> a;
    if (L <= kSortSmemCap) {
        unsigned char *q = smem;
        a.k = reinterpret_cast<K *>(q);
        q += kSortSmemCap * sizeof(dev::key2);
        a.w.small = reinterpret_cast<int2 *>(q);
        a.w.small_cap = kSortSmemSmall;
        q += 2u * kSortSmemSmall * sizeof(int2);
        a.w.big = reinterpret_cast<int2 *>(q);
        a.w.big_cap = kSortSmemBig;
        q += 2u * kSortSmemBig * sizeof(int2);
        a.v = reinterpret_cast<int32_t *>(q);
        q += kSortSmemCap * sizeof(int32_t);
        a.w.pos_l = reinterpret_cast<int *>(q);
        q += kSortSmemCap * sizeof(int32_t);
        a.w.pos_r = reinterpret_cast<int *>(q);
    } else {
        a.k = gk;
        a.v = gv;
        // the small-range list doubles as a ring of int4: start it on a 16-byte boundary
        int2 *g0 = gl + ((reinterpret_cast<uintptr_t>(gl) & 15u) ? 1 : 0);
        a.w.big_cap = L / dev::kBlockRange + 2;
        a.w.small_cap = (L - 1 - 2 * a.w.big_cap) / 2;
        a.w.small = g0;
        a.w.big = g0 + 2 * a.w.small_cap;
        a.w.pos_l = gpos;
        a.w.pos_r = gpos + L;
    }
    return a;
}

// crowding_distance (multi_objective.cpp:280-315) of one front of L >= 2
// members (point indices, in front order), by one block, into cd[point]. Per
// objective: std::sort of the member list by that objective (starting from the
// previous objective's order), ends := +inf, interior += (f[next] - f[prev]) /
// (f[last] - f[first]).
__device__ void front_crowding(const double *__restrict__ pts, uint32_t n, uint32_t m,
                               const long long *__restrict__ keys, const int32_t *members, int L,
                               const sort_area<long long> &a, dev::sort_ctl *ctl, int *slots, int *err, double *cd)
{
    for (int p = threadIdx.x; p < L; p += blockDim.x) {
        const int32_t q = __ldcg(members + p); // written by other blocks of a fused peel
        a.v[p] = q;
        cd[q] = 0.0;
    }
    __syncthreads();
    for (uint32_t k = 0; k < m; ++k) {
        const long long *kk = keys + static_cast<uint64_t>(k) * n;
        for (int p = threadIdx.x; p < L; p += blockDim.x) a.k[p] = kk[a.v[p]];
        __syncthreads();
        dev::block_std_sort(dev::sort_view<long long>{a.k, a.v}, L, a.w, ctl, slots, err);
        const int32_t q0 = a.v[0], q1 = a.v[L - 1];
        const double df = pts[static_cast<uint64_t>(q1) * m + k] - pts[static_cast<uint64_t>(q0) * m + k];
        for (int p = 1 + static_cast<int>(threadIdx.x); p < L - 1; p += blockDim.x) {
            const int32_t q = a.v[p];
            cd[q] += (pts[static_cast<uint64_t>(a.v[p + 1]) * m + k] - pts[static_cast<uint64_t>(a.v[p - 1]) * m + k])
                     / df;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            cd[q0] = HUGE_VAL;
            cd[q1] = HUGE_VAL;
        }
        __syncthreads();
    }
}

// How fronts of one and two points are treated.
enum : int {
    kCrowdNsga2 = 0,         // nsga2.cpp:188-193: +inf for fronts of 1 or 2 points
    kCrowdSortPopulation = 1 // multi_objective.cpp:441-446: 0 for a single point, else crowding_distance
};

struct peel2_args {
    const uint32_t *Dt;
    const int32_t *dom_count;
    uint32_t n, W, W8;
    int32_t *wit;       // n first witnesses (-1: none) and
    int32_t *res;       // n their resume words, from witness_init_kernel
    int32_t *list;      // 2 n: members of fronts k (parity k & 1)
    int32_t *keyv;      // 2 n: their ordering keys
    int32_t *cnt;       // n + 2 per-front member counters, zeroed
    int32_t *rank, *front_offsets, *front_indices;
    peel_state *st;
    // blocks [0, npeel) peel; with crowding (cd set), blocks [npeel, gridDim.x)
    // compute the crowding distances of the fronts of up to kSortSmemCap
    // members as the peel completes them (longer fronts: big_crowding_kernel)
    uint32_t npeel;
    const double *pts;
    uint32_t m;
    const long long *keys;
    double *cd;
    int crowd_mode;
};

// Blocks of the fused peel that compute crowding distances.
constexpr int kCrowdBlocks = 16;

// The crowding blocks of peel2_kernel: block c of C takes fronts c, c + C, ...,
// each once the peel has published it (st->fronts_done), with a bounded wait.
__device__ void crowd_role(const peel2_args &a, int c, int C)
{
    extern __shared__ __align__(16) unsigned char sort_smem[];
    __shared__ dev::sort_ctl ctl;
    __shared__ int slots[kSortWarps * 64];
    __shared__ int s_go;
    for (int f = c;; f += C) {
        if (threadIdx.x == 0) {
            int go = 0;
            volatile int *vd = &a.st->fronts_done, *vp = &a.st->peel_done, *ve = &a.st->err, *vn = &a.st->n_fronts;
            for (unsigned long long spins = 0;; ++spins) {
                if (*vd > f) {
                    go = 1;
                    break;
                }
                if (*ve) break;
                if (*vp && *vn <= f) break;
                if (spins > kSpinLimit) {
                    atomicExch(&a.st->err, 1);
                    break;
                }
                __nanosleep(256);
            }
            __threadfence();
            s_go = go;
        }
        __syncthreads();
        if (!s_go) return;
        const int off = __ldcg(a.front_offsets + f), L = __ldcg(a.front_offsets + f + 1) - off;
        const int32_t *mem = a.front_indices + off;
        if (L == 1 || (L == 2 && a.crowd_mode == kCrowdNsga2)) {
            if (static_cast<int>(threadIdx.x) < L) a.cd[__ldcg(mem + threadIdx.x)] = a.crowd_mode == kCrowdNsga2 ? HUGE_VAL : 0.0;
        } else if (L <= kSortSmemCap) {
            const sort_area<long long> area = pick_area<long long>(sort_smem, L, nullptr, nullptr, nullptr, nullptr);
            front_crowding(a.pts, a.n, a.m, a.keys, mem, L, area, &ctl, slots, &a.st->sort_err, a.cd);
        }
        __syncthreads();
    }
}

// In-place exclusive prefix sum of h[0, R) by the whole block (R <= 4
// entries per thread here); wtot holds 32 ints of scratch.
__device__ void block_exclusive_scan(int32_t *h, int R, int *wtot)
{
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int per = (R + static_cast<int>(blockDim.x) - 1) / static_cast<int>(blockDim.x);
    const int b0 = min(R, static_cast<int>(threadIdx.x) * per), b1 = min(R, b0 + per);
    int local = 0;
    for (int i = b0; i < b1; ++i) local += h[i];
    int incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kFull, incl, o);
        if (static_cast<int>(lane) >= o) incl += t;
    }
    if (lane == 31u) wtot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int t = lane < nwarp ? wtot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(kFull, t, o);
            if (static_cast<int>(lane) >= o) t += u;
        }
        if (lane < nwarp) wtot[lane] = t;
    }
    __syncthreads();
    int run = incl - local + (warp > 0 ? wtot[warp - 1] : 0);
    for (int i = b0; i < b1; ++i) {
        const int c = h[i];
        h[i] = run;
        run += c;
    }
    __syncthreads();
}

__device__ __forceinline__ bool bit_of(const uint32_t *s, int32_t q)
{
    return (s[q >> 5] >> (q & 31)) & 1u;
}

// rem (the valid points) minus front 0 (the points without dominators): the
// unassigned set when front 1 is peeled.
__global__ void rem_outside_front0_kernel(const int32_t *__restrict__ dom_count, uint32_t n, uint32_t W,
                                          uint32_t *__restrict__ rem)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < W; w += warps) {
        const uint32_t q = w * 32u + lane;
        const uint32_t z = __ballot_sync(kFull, q < n && __ldg(dom_count + q) == 0);
        if (lane == 0) rem[w] &= ~z;
    }
}

// Every point's first witness and resume word, before the peel and on every
// SM at full occupancy (one warp per point): the first word of its row of Dt
// holding a dominator outside front 0 is the resume word, and the witness is,
// of one such dominator per lane (from the lane's first nonzero word), the one
// with the most dominators itself, as the peel's rescans choose. Points with
// no dominator outside front 0 (front 1) and front 0 itself get -1.
__global__ void __launch_bounds__(256) witness_init_kernel(const uint32_t *__restrict__ Dt,
                                                           const int32_t *__restrict__ dom_count,
                                                           const uint32_t *__restrict__ rem, uint32_t n, uint32_t W,
                                                           uint32_t W8, int32_t *__restrict__ wit,
                                                           int32_t *__restrict__ res)
{
    extern __shared__ uint32_t s_u[]; // W8 words: rem (words from W on are zero)
    for (uint32_t w = threadIdx.x; w < W8; w += blockDim.x) s_u[w] = w < W ? __ldg(rem + w) : 0u;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < n; j += warps) {
        int32_t found = -1, resume = -1;
        if (__ldg(dom_count + j) > 0) {
            const uint32_t *row = Dt + static_cast<uint64_t>(j) * W8;
            for (uint32_t base = 0; base < W && found < 0; base += 512u) {
                uint4 x[4];
#pragma unroll
                for (uint32_t u = 0; u < 4u; ++u) {
                    const uint32_t wi = base + 4u * (u * 32u + lane);
                    x[u] = make_uint4(0u, 0u, 0u, 0u);
                    if (wi < W) {
                        const uint4 d = __ldg(reinterpret_cast<const uint4 *>(row + wi));
                        const uint4 r = *reinterpret_cast<const uint4 *>(s_u + wi);
                        x[u] = make_uint4(d.x & r.x, d.y & r.y, d.z & r.z, d.w & r.w);
                    }
                }
                int cand = -1;
#pragma unroll
                for (uint32_t u = 0; u < 4u; ++u) {
                    const uint32_t c = x[u].x ? 0u : (x[u].y ? 1u : (x[u].z ? 2u : 3u));
                    const uint32_t xv = x[u].x ? x[u].x : (x[u].y ? x[u].y : (x[u].z ? x[u].z : x[u].w));
                    if (cand < 0 && xv)
                        cand = static_cast<int>((base + 4u * (u * 32u + lane) + c) * 32u) + (31 - __clz(xv));
                    const uint32_t bb = __ballot_sync(kFull, xv != 0u);
                    if (resume < 0 && bb) {
                        const int l0 = __ffs(bb) - 1;
                        const uint32_t cl = __shfl_sync(kFull, c, l0);
                        resume = static_cast<int32_t>(base + 4u * (u * 32u + static_cast<uint32_t>(l0)) + cl);
                    }
                }
                if (resume >= 0) {
                    int best = cand >= 0 ? __ldg(dom_count + cand) : -1, bq = cand;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        const int ob = __shfl_xor_sync(kFull, best, o), oq = __shfl_xor_sync(kFull, bq, o);
                        if (ob > best || (ob == best && oq < bq)) {
                            best = ob;
                            bq = oq;
                        }
                    }
                    found = bq;
                }
            }
        }
        if (lane == 0) {
            wit[j] = found;
            res[j] = resume;
        }
    }
}

__global__ void __launch_bounds__(kPeelThreads) peel2_kernel(peel2_args a)
{
    if (blockIdx.x >= a.npeel) {
        crowd_role(a, static_cast<int>(blockIdx.x - a.npeel), static_cast<int>(gridDim.x - a.npeel));
        return;
    }
    const uint32_t P = a.npeel; // the peeling blocks
    extern __shared__ __align__(16) uint32_t dyn[];
    const uint32_t W = a.W, n = a.n;
    uint32_t *s_rem = dyn;                                          // W
    uint32_t *s_Z = s_rem + W;                                      // W: front 0
    int32_t *s_Zp = reinterpret_cast<int32_t *>(s_Z + W);           // W: exclusive prefix popcounts of s_Z
    int32_t *s_prev = s_Zp + W;                                     // 2 kTile: front k-1 by position
    int32_t *s_key = s_prev + 2 * kTile;                            // kTile
    int32_t *s_idx = s_key + kTile;                                 // kTile
    int32_t *s_queue = s_idx + kTile;                               // kQueue
    int32_t *s_wit = s_queue + kQueue;                              // 32 wpb: witnesses of this block's points
    int32_t *s_res = s_wit + 32u * ((W + P - 1u) / P); // 32 wpb: their rescans' resume words
    uint32_t *s_pbits = reinterpret_cast<uint32_t *>(s_res + 32u * ((W + P - 1u) / P)); // W
    uint16_t *s_pos = reinterpret_cast<uint16_t *>(s_pbits + W); // n: positions in the previous front
    const bool pos_maps = n <= kPosPoints;
    uint16_t *s_dc = s_pos + ((n + 1u) & ~1u); // n: domination counts (pos_maps only; n <= kPosPoints < 65536)
    __shared__ int32_t s_list[kLocalMembers], s_lkey[kLocalMembers];
    __shared__ int s_cnt, s_base, s_qn, s_wtot[32];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned nwarp_b = blockDim.x >> 5;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    // this block's rem words in Phase A
    const uint32_t wpb = (W + P - 1u) / P;
    const uint32_t w_lo = min(W, blockIdx.x * wpb), w_hi = min(W, w_lo + wpb);
    const int32_t j_lo = static_cast<int32_t>(32u * w_lo); // this block's points: [j_lo, 32 w_hi)
    for (uint32_t t = threadIdx.x; t < 32u * wpb; t += blockDim.x) {
        const uint32_t j = static_cast<uint32_t>(j_lo) + t;
        s_wit[t] = j < n ? __ldg(a.wit + j) : -1;
        s_res[t] = j < n ? __ldg(a.res + j) : -1;
    }
    if (pos_maps)
        for (uint32_t t = threadIdx.x; t < n; t += blockDim.x) s_dc[t] = static_cast<uint16_t>(__ldg(a.dom_count + t));

    // ---- front 0 from dom_count (every block for itself)
    for (uint32_t w = warp; w < W; w += nwarp_b) {
        const uint32_t q = w * 32u + lane;
        const bool valid = q < n;
        const bool zero = valid && __ldg(a.dom_count + q) == 0;
        const uint32_t z = __ballot_sync(kFull, zero), v = __ballot_sync(kFull, valid);
        if (lane == 0) {
            s_Z[w] = z;
            s_rem[w] = v & ~z;
        }
    }
    __syncthreads();
    {
        // exclusive prefix popcounts of s_Z: each thread a run of consecutive words
        const uint32_t per = (W + blockDim.x - 1u) / blockDim.x;
        const uint32_t b0 = min(W, threadIdx.x * per), b1 = min(W, b0 + per);
        int local = 0;
        for (uint32_t w = b0; w < b1; ++w) local += __popc(s_Z[w]);
        int incl = local;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, o);
            if (static_cast<int>(lane) >= o) incl += t;
        }
        if (lane == 31u) s_wtot[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            int t = lane < nwarp_b ? s_wtot[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(kFull, t, o);
                if (static_cast<int>(lane) >= o) t += u;
            }
            if (lane < nwarp_b) s_wtot[lane] = t; // inclusive warp totals
        }
        __syncthreads();
        int run = incl - local + (warp > 0 ? s_wtot[warp - 1] : 0);
        for (uint32_t w = b0; w < b1; ++w) {
            s_Zp[w] = run;
            run += __popc(s_Z[w]);
        }
    }
    __syncthreads();
    const int L0 = s_wtot[nwarp_b - 1];
    // front 0's global writes, spread over the blocks by word
    for (uint32_t w = blockIdx.x * nwarp_b + warp; w < W; w += P * nwarp_b) {
        const uint32_t z = s_Z[w];
        if ((z >> lane) & 1u) {
            const uint32_t q = w * 32u + lane;
            const int p = s_Zp[w] + __popc(z & ((1u << lane) - 1u));
            a.front_indices[p] = static_cast<int32_t>(q);
            a.rank[q] = 0;
        }
    }
    if (tid == 0) a.front_offsets[1] = L0;
    if (pos_maps) {
        // front 0's membership bits and positions (every block for itself)
        for (uint32_t w = threadIdx.x; w < W; w += blockDim.x) s_pbits[w] = s_Z[w];
        for (uint32_t w = warp; w < W; w += nwarp_b) {
            const uint32_t z = s_Z[w];
            if ((z >> lane) & 1u) s_pos[w * 32u + lane] = static_cast<uint16_t>(s_Zp[w] + __popc(z & ((1u << lane) - 1u)));
        }
    }
    int off = L0, off_prev = 0, size_prev = L0;
    bool prev_global = false; // front k-1 by position only in global memory (a large front)
    bool pos_ok = pos_maps;   // front k-1's bits and positions are in s_pbits / s_pos
    int k = 1;
    for (; off < static_cast<int>(n); ++k) {
        if (threadIdx.x == 0) {
            s_cnt = 0;
            s_qn = 0;
        }
        if (prev_global && size_prev <= 2 * kTile) {
            for (int t = threadIdx.x; t < size_prev; t += blockDim.x) s_prev[t] = __ldcg(a.front_indices + off_prev + t);
        }
        const bool prev_in_smem = k >= 2 && size_prev <= 2 * kTile;
        __syncthreads();
        // ---- Phase A, stage 1: witness tests over this block's words
        for (uint32_t w = w_lo + warp; w < w_hi; w += nwarp_b) {
            const uint32_t bits = s_rem[w];
            if (!bits) continue;
            const int32_t j = static_cast<int32_t>(w * 32u + lane);
            const bool cand = (bits >> lane) & 1u;
            bool need = false;
            if (cand) {
                const int32_t wj = s_wit[j - j_lo];
                need = !(wj >= 0 && bit_of(s_rem, wj));
            }
            const uint32_t b = __ballot_sync(kFull, need);
            if (b) {
                int base = 0;
                if (lane == 0) base = atomicAdd(&s_qn, __popc(b));
                base = __shfl_sync(kFull, base, 0);
                if (need) s_queue[base + __popc(b & ((1u << lane) - 1u))] = j;
            }
        }
        __syncthreads();
        // ---- stage 2: scans of the queued rows
        const int qn = s_qn;
        for (int t = static_cast<int>(warp); t < qn; t += static_cast<int>(nwarp_b)) {
            const int32_t j = s_queue[t];
            const uint32_t *row = a.Dt + static_cast<uint64_t>(j) * a.W8;
            // 512 words per round from the resume word, four per 16-byte load
            // (rows start on 32-byte boundaries; words from W on are masked)
            const int32_t rj = s_res[j - j_lo];
            const uint32_t ws = (rj >= 0 ? static_cast<uint32_t>(rj) : 0u) & ~3u;
            int32_t found = -1, resume = -1;
            int pkey = -1; // this lane's highest position in front k-1 among the dominators seen
            for (uint32_t base = ws; base < W && found < 0; base += 512u) {
                uint4 x[4];
#pragma unroll
                for (uint32_t u = 0; u < 4u; ++u) {
                    const uint32_t wi = base + 4u * (u * 32u + lane);
                    x[u] = make_uint4(0u, 0u, 0u, 0u);
                    if (wi < W) {
                        const uint4 d = __ldg(reinterpret_cast<const uint4 *>(row + wi));
                        const uint4 r = *reinterpret_cast<const uint4 *>(s_rem + wi);
                        x[u].x = d.x & r.x;
                        x[u].y = wi + 1u < W ? d.y & r.y : 0u;
                        x[u].z = wi + 2u < W ? d.z & r.z : 0u;
                        x[u].w = wi + 3u < W ? d.w & r.w : 0u;
                        if (pos_ok) {
                            // dominators in front k-1 (all at or after the resume
                            // word: they were unassigned at every earlier scan)
                            const uint32_t dw[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
                            for (uint32_t c = 0; c < 4u; ++c) {
                                uint32_t pb = wi + c < W ? dw[c] & s_pbits[wi + c] : 0u;
                                while (pb) {
                                    const int b = __ffs(pb) - 1;
                                    pkey = max(pkey, static_cast<int>(s_pos[(wi + c) * 32u + static_cast<uint32_t>(b)]));
                                    pb &= pb - 1u;
                                }
                            }
                        }
                    }
                }
                // the first word holding an unassigned dominator: rescans resume there
                // (the words before it hold none, and the unassigned set only shrinks)
                int cand = -1; // this lane's proposal: a dominator from its first nonzero word
#pragma unroll
                for (uint32_t u = 0; u < 4u; ++u) {
                    const uint32_t c = x[u].x ? 0u : (x[u].y ? 1u : (x[u].z ? 2u : 3u));
                    const uint32_t xv = x[u].x ? x[u].x : (x[u].y ? x[u].y : (x[u].z ? x[u].z : x[u].w));
                    if (cand < 0 && xv)
                        cand = static_cast<int>((base + 4u * (u * 32u + lane) + c) * 32u) + (31 - __clz(xv));
                    const uint32_t bb = __ballot_sync(kFull, xv != 0u);
                    if (resume < 0 && bb) {
                        const int l0 = __ffs(bb) - 1;
                        const uint32_t cl = __shfl_sync(kFull, c, l0);
                        resume = static_cast<int32_t>(base + 4u * (u * 32u + static_cast<uint32_t>(l0)) + cl);
                    }
                }
                if (resume >= 0) {
                    // the witness: of the lanes' proposals, the dominator with the
                    // most dominators itself (likely in a later front, so j is
                    // rescanned less often)
                    int best = cand >= 0 ? (pos_maps ? static_cast<int>(s_dc[cand]) : __ldg(a.dom_count + cand)) : -1,
                        bq = cand;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        const int ob = __shfl_xor_sync(kFull, best, o), oq = __shfl_xor_sync(kFull, bq, o);
                        if (ob > best || (ob == best && oq < bq)) {
                            best = ob;
                            bq = oq;
                        }
                    }
                    found = bq;
                }
            }
            if (found >= 0) {
                if (lane == 0) {
                    s_wit[j - j_lo] = found;
                    s_res[j - j_lo] = resume;
                }
                continue;
            }
            // a member of front k: its key
            int key = -1;
            if (pos_ok) {
                // the scan above read every word that can hold its front k-1 dominators
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) pkey = max(pkey, __shfl_xor_sync(kFull, pkey, o));
                key = pkey;
            } else if (k == 1) {
                // the highest-index dominator among front 0 (positions follow indices there)
                for (int top = static_cast<int>(W) - 1; top >= 0 && key < 0; top -= 256) {
                    uint32_t x[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int ww = top - u * 32 - static_cast<int>(lane);
                        x[u] = ww >= 0 ? (__ldg(row + ww) & s_Z[ww]) : 0u;
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const uint32_t bb = __ballot_sync(kFull, x[u] != 0u);
                        if (key < 0 && bb) {
                            const int l0 = __ffs(bb) - 1; // lowest lane = highest word of this group
                            const uint32_t xv = __shfl_sync(kFull, x[u], l0);
                            const int ww = top - u * 32 - l0;
                            const int hb = 31 - __clz(xv);
                            key = s_Zp[ww] + __popc(s_Z[ww] & ((hb == 0) ? 0u : (0xffffffffu >> (32 - hb))));
                        }
                    }
                }
            } else {
                // 256 positions per round: every lane's 8 row-word loads are in
                // flight together, then the ballots
                for (int top = size_prev - 1; top >= 0 && key < 0; top -= 256) {
                    uint32_t hw[8], hb[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int p = top - 32 * u - static_cast<int>(lane);
                        hw[u] = 0u;
                        hb[u] = 0u;
                        if (p >= 0) {
                            const uint32_t d = static_cast<uint32_t>(prev_in_smem ? s_prev[p]
                                                                                  : __ldcg(a.front_indices + off_prev + p));
                            hw[u] = __ldg(row + (d >> 5));
                            hb[u] = d & 31u;
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const unsigned bal = __ballot_sync(kFull, (hw[u] >> hb[u]) & 1u);
                        if (key < 0 && bal) key = top - 32 * u - (__ffs(bal) - 1);
                    }
                }
            }
            if (lane == 0) {
                const int ls = atomicAdd(&s_cnt, 1);
                if (ls < kLocalMembers) {
                    s_list[ls] = j;
                    s_lkey[ls] = key;
                } else {
                    const int s = atomicAdd(a.cnt + k, 1);
                    a.list[(k & 1) * n + s] = j;
                    a.keyv[(k & 1) * n + s] = key;
                }
            }
        }
        __syncthreads();
        const int local = min(s_cnt, kLocalMembers);
        if (threadIdx.x == 0) s_base = local ? atomicAdd(a.cnt + k, local) : 0;
        __syncthreads();
        for (int t = threadIdx.x; t < local; t += blockDim.x) {
            a.list[(k & 1) * n + s_base + t] = s_list[t];
            a.keyv[(k & 1) * n + s_base + t] = s_lkey[t];
        }
        if (!peel_sync(a.st, P)) {
            if (threadIdx.x == 0) atomicExch(&a.st->n_fronts, -1);
            return;
        }
        // fronts 0 .. k-1 are complete in global memory (their last writes came
        // before this barrier): the crowding blocks may take them (published by
        // a warp with no part in the next steps' first loads)
        if (P < gridDim.x && blockIdx.x == 0 && threadIdx.x == blockDim.x - 32u) {
            __threadfence();
            atomicExch(&a.st->fronts_done, k);
        }
        const int L = *reinterpret_cast<volatile int *>(a.cnt + k);
        if (L == 0) break; // cannot happen while points remain (a dominance cycle would need one); guards the loop
        const int32_t *lst = a.list + (k & 1) * n;
        const int32_t *kv = a.keyv + (k & 1) * n;
        // keys are positions in front k-1: [0, size_prev)
        const int R = size_prev;
        if (L <= kTile && R <= kQueue) {
            // ---- Phase C in every block: a counting sort by key, ties by index
            int32_t *h = s_queue;              // R bucket counters, then bucket starts / ends
            int32_t *s_blist = s_prev + kTile; // members in bucket order
            for (int t = threadIdx.x; t < R; t += blockDim.x) h[t] = 0;
            if (pos_maps)
                for (uint32_t w = threadIdx.x; w < W; w += blockDim.x) s_pbits[w] = 0u;
            for (int t = threadIdx.x; t < L; t += blockDim.x) {
                int kq = __ldcg(kv + t);
                if (kq < 0 || kq >= R) { // a member without a dominator in front k-1: never expected
                    atomicExch(&a.st->sort_err, 1);
                    kq = kq < 0 ? 0 : R - 1;
                }
                s_key[t] = kq;
                s_idx[t] = __ldcg(lst + t);
            }
            __syncthreads();
            for (int t = threadIdx.x; t < L; t += blockDim.x) atomicAdd(h + s_key[t], 1);
            __syncthreads();
            block_exclusive_scan(h, R, s_wtot);
            constexpr int kPer = kTile / kPeelThreads;
            int b0[kPer], pos[kPer];
#pragma unroll
            for (int i = 0; i < kPer; ++i) {
                const int t = threadIdx.x + i * kPeelThreads;
                b0[i] = t < L ? h[s_key[t]] : 0;
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < kPer; ++i) {
                const int t = threadIdx.x + i * kPeelThreads;
                if (t < L) s_blist[atomicAdd(h + s_key[t], 1)] = t;
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < kPer; ++i) {
                const int t = threadIdx.x + i * kPeelThreads;
                pos[i] = 0;
                if (t < L) {
                    const int e = h[s_key[t]], q = s_idx[t];
                    int p = b0[i];
                    for (int u = b0[i]; u < e; ++u) p += s_idx[s_blist[u]] < q;
                    pos[i] = p;
                }
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < kPer; ++i) {
                const int t = threadIdx.x + i * kPeelThreads;
                if (t < L) {
                    const int q = s_idx[t], p = pos[i];
                    s_prev[p] = q; // front k by position, for the keys of front k+1
                    atomicAnd(s_rem + (q >> 5), ~(1u << (q & 31)));
                    if (pos_maps) {
                        s_pos[q] = static_cast<uint16_t>(p);
                        atomicOr(s_pbits + (q >> 5), 1u << (q & 31));
                    }
                    if (p % static_cast<int>(P) == static_cast<int>(blockIdx.x)) {
                        a.front_indices[off + p] = q;
                        a.rank[q] = k;
                    }
                }
            }
            prev_global = false;
            pos_ok = pos_maps;
        } else {
            // ---- a large front: block b ranks members [m_lo, m_hi), one warp per
            // member, lanes splitting the comparisons against shared-memory tiles;
            // then a barrier (the next keys read front k from global memory)
            for (int t = threadIdx.x; t < L; t += blockDim.x) {
                const int q = __ldcg(lst + t);
                atomicAnd(s_rem + (q >> 5), ~(1u << (q & 31)));
            }
            const int mpb = (L + static_cast<int>(P) - 1) / static_cast<int>(P);
            const int m_lo = min(L, static_cast<int>(blockIdx.x) * mpb), m_hi = min(L, m_lo + mpb);
            int32_t *cntm = s_queue; // mpb <= kQueue (checked on the host)
            for (int t = threadIdx.x; t < m_hi - m_lo; t += blockDim.x) cntm[t] = 0;
            for (int t0 = 0; t0 < L; t0 += kTile) {
                const int lim = min(kTile, L - t0);
                __syncthreads();
                for (int t = threadIdx.x; t < lim; t += blockDim.x) {
                    s_key[t] = __ldcg(kv + t0 + t);
                    s_idx[t] = __ldcg(lst + t0 + t);
                }
                __syncthreads();
                for (int sidx = m_lo + static_cast<int>(warp); sidx < m_hi; sidx += static_cast<int>(nwarp_b)) {
                    const int q = __ldcg(lst + sidx), kq = __ldcg(kv + sidx);
                    int p = 0;
                    for (int t = static_cast<int>(lane); t < lim; t += 32) {
                        const int kt = s_key[t], qt = s_idx[t];
                        p += (kt < kq) | ((kt == kq) & (qt < q));
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(kFull, p, o);
                    if (lane == 0) cntm[sidx - m_lo] += p;
                }
            }
            __syncthreads();
            for (int sidx = m_lo + static_cast<int>(threadIdx.x); sidx < m_hi; sidx += static_cast<int>(blockDim.x)) {
                const int q = __ldcg(lst + sidx), p = cntm[sidx - m_lo];
                a.front_indices[off + p] = q;
                a.rank[q] = k;
            }
            prev_global = true;
            pos_ok = false;
            if (!peel_sync(a.st, P)) {
                if (threadIdx.x == 0) atomicExch(&a.st->n_fronts, -1);
                return;
            }
        }
        if (tid == 0) a.front_offsets[k + 1] = off + L;
        off_prev = off;
        size_prev = L;
        off += L;
        __syncthreads();
    }
    if (P < gridDim.x) {
        // the last front's writes, then every front to the crowding blocks
        const bool ok = peel_sync(a.st, P);
        if (tid == 0) {
            a.st->n_fronts = (!ok || *reinterpret_cast<volatile int *>(&a.st->err)) ? -1 : k;
            a.front_offsets[0] = 0;
            __threadfence();
            atomicExch(&a.st->fronts_done, k);
            atomicExch(&a.st->peel_done, 1);
        }
        return;
    }
    if (tid == 0) {
        a.st->n_fronts = *reinterpret_cast<volatile int *>(&a.st->err) ? -1 : k;
        a.front_offsets[0] = 0;
    }
}

// Crowding distance of every point within its front: blocks take fronts
// f = blockIdx.x, blockIdx.x + gridDim.x, ... (n_fronts read on the device).
__global__ void __launch_bounds__(kSortThreads) front_crowding_kernel(
    const double *__restrict__ pts, uint32_t n, uint32_t m, const long long *__restrict__ keys,
    const int32_t *__restrict__ front_offsets, const int32_t *__restrict__ front_indices,
    const int32_t *__restrict__ n_fronts, int mode, unsigned char *wkey, int32_t *widx, int2 *wlist, int32_t *wpos,
    double *cd, peel_state *st)
{
    extern __shared__ __align__(16) unsigned char sort_smem[];
    __shared__ dev::sort_ctl ctl;
    __shared__ int slots[kSortWarps * 64];
    const int nf = *n_fronts; // -1 after a barrier timeout: nothing to do
    for (int f = blockIdx.x; f < nf; f += gridDim.x) {
        const int off = front_offsets[f], L = front_offsets[f + 1] - off;
        const int32_t *mem = front_indices + off;
        if (L == 1 || (L == 2 && mode == kCrowdNsga2)) {
            if (static_cast<int>(threadIdx.x) < L) cd[mem[threadIdx.x]] = mode == kCrowdNsga2 ? HUGE_VAL : 0.0;
            continue;
        }
        if (m < 2u) {
            if (threadIdx.x == 0) atomicExch(&st->status, kStatusNeedTwoObjectives);
            continue;
        }
        if (L > kSortSmemCap) continue; // big_crowding_kernel
        const sort_area<long long> a =
            pick_area<long long>(sort_smem, L, reinterpret_cast<long long *>(wkey) + off, widx + off, wlist + off,
                                 wpos + 2 * off);
        front_crowding(pts, n, m, keys, mem, L, a, &ctl, slots, &st->sort_err, cd);
    }
}

// ---------------------------------------------------------- grid-wide sorts
//
// Sorts longer than kSortSmemCap run on every block of a cooperative launch
// (one block of kGridSortThreads per SM), still with std::sort's exact
// permutation: the introsort's levels are processed in order, each range
// longer than kSortSmemCap partitioned by one block (block_partition: the
// same median-of-three and Hoare pairs as the sequential loop), the levels
// separated by grid barriers; ranges of 17..kSortSmemCap elements are then
// sorted by one block each in shared memory, continuing the introsort with
// the depth budget they were created with, and ranges of 16 or fewer are
// sorted as leaves when they appear. Ranges of one level are disjoint, so the
// blocks that take them do not change the result.
constexpr int kGridSortThreads = 1024;
constexpr int kGridSortWarps = kGridSortThreads / 32;

struct grid_sort_mem {
    int2 *lists;  // L int2 of scratch: two level lists, the shared-memory ranges and their depths
    int32_t *pos; // 2 L stopper positions
};

// Queues child [a, b) (depth budget d) of a partition by the grid.
__device__ __forceinline__ void grid_queue(int a, int b, int d, int2 *next, int big_cap, int2 *bot, int2 *bot_d,
                                           int bot_cap, int *nnext, int *nbot, int *err)
{
    const int len = b - a;
    if (len > kSortSmemCap) {
        const int slot = atomicAdd(nnext, 1);
        if (slot < big_cap)
            next[slot] = make_int2(a, b);
        else
            atomicExch(err, dev::kSortErrListFull);
    } else if (len > 16) {
        const int slot = atomicAdd(nbot, 1);
        if (slot < bot_cap) {
            bot[slot] = make_int2(a, b);
            bot_d[slot] = make_int2(d, 0);
        } else {
            atomicExch(err, dev::kSortErrListFull);
        }
    }
}

// Every block of the cooperative launch calls it with the same arguments
// (L > kSortSmemCap). Returns false when a grid barrier gave up.
template <typename K>
__device__ bool grid_std_sort(const dev::sort_view<K> &x, int L, const grid_sort_mem &g, peel_state *st,
                              unsigned char *sort_smem, dev::sort_ctl *ctl, int *slots, int *err)
{
    const int big_cap = L / (kSortSmemCap + 1) + 2, bot_cap = L / 17 + 2;
    int2 *big[2] = {g.lists, g.lists + big_cap};
    int2 *bot = g.lists + 2 * big_cap, *bot_d = bot + bot_cap;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int i = 0; i < 72; ++i) st->gs[i] = 0;
        st->gs[1] = 1;
        big[0][0] = make_int2(0, L);
    }
    if (!grid_sync(st)) return false;
    const unsigned lane = threadIdx.x & 31u;
    const int warp = static_cast<int>(threadIdx.x >> 5);
    int depth = 2 * dev::floor_log2_int(L);
    for (int level = 0; level < 70; ++level, --depth) {
        const int nbig = min(*reinterpret_cast<volatile int *>(&st->gs[1 + level]), big_cap);
        if (nbig == 0) break;
        int2 *cur = big[level & 1], *next = big[(level + 1) & 1];
        for (int t = blockIdx.x; t < nbig; t += gridDim.x) {
            const int2 r = cur[t];
            if (depth == 0) {
                if (threadIdx.x == 0) dev::heap_sort(x, r.x, r.y);
                __syncthreads();
                continue;
            }
            dev::sort_work w{};
            w.pos_l = g.pos + r.x;
            w.pos_r = g.pos + L + r.x;
            const int cut = dev::block_partition(x, r.x, r.y, w, slots, err);
            if (threadIdx.x == 0)
                grid_queue(r.x, cut, depth - 1, next, big_cap, bot, bot_d, bot_cap, &st->gs[2 + level], &st->gs[0], err);
            if (threadIdx.x == 32)
                grid_queue(cut, r.y, depth - 1, next, big_cap, bot, bot_d, bot_cap, &st->gs[2 + level], &st->gs[0], err);
            if (warp == 0) {
                const int a = lane < 16u ? r.x : cut, len = lane < 16u ? cut - r.x : r.y - cut;
                dev::halfwarp_leaf_sort(x, a, len <= 16 ? len : 0);
            }
            __syncthreads();
        }
        if (!grid_sync(st)) return false;
    }
    // the shared-memory ranges, one block each
    const int nbot = min(*reinterpret_cast<volatile int *>(&st->gs[0]), bot_cap);
    for (int t = blockIdx.x; t < nbot; t += gridDim.x) {
        const int2 r = bot[t];
        const int d = bot_d[t].x, len = r.y - r.x;
        const sort_area<K> a = pick_area<K>(sort_smem, len, nullptr, nullptr, nullptr, nullptr);
        for (int i = threadIdx.x; i < len; i += blockDim.x) {
            a.k[i] = x.k[r.x + i];
            a.v[i] = x.v[r.x + i];
        }
        __syncthreads();
        dev::block_std_sort(dev::sort_view<K>{a.k, a.v}, len, a.w, ctl, slots, err, d);
        for (int i = threadIdx.x; i < len; i += blockDim.x) {
            x.k[r.x + i] = a.k[i];
            x.v[r.x + i] = a.v[i];
        }
        __syncthreads();
    }
    return grid_sync(st);
}

// Crowding distance of one front longer than kSortSmemCap by every block of a
// cooperative launch: the same per-objective sorts as front_crowding, each
// starting from the previous objective's order, and the same neighbour
// differences. kb, v: L keys and values of scratch. Returns false when a grid
// barrier gave up.
__device__ bool grid_front_crowding(const double *__restrict__ pts, uint32_t n, uint32_t m,
                                    const long long *__restrict__ keys, const int32_t *mem, int L, long long *kb,
                                    int32_t *v, const grid_sort_mem &g, peel_state *st, unsigned char *sort_smem,
                                    dev::sort_ctl *ctl, int *slots, double *cd)
{
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x, gn = gridDim.x * blockDim.x;
    for (uint32_t p = gt; p < static_cast<uint32_t>(L); p += gn) {
        const int32_t q = mem[p];
        v[p] = q;
        cd[q] = 0.0;
    }
    if (!grid_sync(st)) return false;
    for (uint32_t k = 0; k < m; ++k) {
        const long long *kk = keys + static_cast<uint64_t>(k) * n;
        for (uint32_t p = gt; p < static_cast<uint32_t>(L); p += gn) kb[p] = kk[v[p]];
        if (!grid_sync(st)) return false;
        if (!grid_std_sort(dev::sort_view<long long>{kb, v}, L, g, st, sort_smem, ctl, slots, &st->sort_err))
            return false;
        const int32_t q0 = v[0], q1 = v[L - 1];
        const double df = pts[static_cast<uint64_t>(q1) * m + k] - pts[static_cast<uint64_t>(q0) * m + k];
        for (uint32_t p = 1u + gt; p < static_cast<uint32_t>(L - 1); p += gn) {
            const int32_t q = v[p];
            cd[q] += (pts[static_cast<uint64_t>(v[p + 1]) * m + k] - pts[static_cast<uint64_t>(v[p - 1]) * m + k])
                     / df;
        }
        if (!grid_sync(st)) return false;
        if (gt == 0) {
            cd[q0] = HUGE_VAL;
            cd[q1] = HUGE_VAL;
        }
        if (!grid_sync(st)) return false;
    }
    return true;
}

// The fronts longer than kSortSmemCap (front_crowding_kernel skips them), one
// after the other.
__global__ void __launch_bounds__(kGridSortThreads) big_crowding_kernel(
    const double *__restrict__ pts, uint32_t n, uint32_t m, const long long *__restrict__ keys,
    const int32_t *__restrict__ front_offsets, const int32_t *__restrict__ front_indices,
    const int32_t *__restrict__ n_fronts, unsigned char *wkey, int32_t *widx, int2 *wlist, int32_t *wpos, double *cd,
    peel_state *st)
{
    extern __shared__ __align__(16) unsigned char sort_smem[];
    __shared__ dev::sort_ctl ctl;
    __shared__ int slots[kGridSortWarps * 64];
    const int nf = *n_fronts;
    if (m < 2u) return; // front_crowding_kernel reports it
    for (int f = 0; f < nf; ++f) {
        const int off = front_offsets[f], L = front_offsets[f + 1] - off;
        if (L <= kSortSmemCap) continue;
        const grid_sort_mem g{wlist + off, wpos + 2 * off};
        if (!grid_front_crowding(pts, n, m, keys, front_indices + off, L, reinterpret_cast<long long *>(wkey) + off,
                                 widx + off, g, st, sort_smem, &ctl, slots, cd))
            return;
    }
}

// The critical front of select_best_N_mo when it is longer than kSortSmemCap
// (select_best_kernel copies the whole fronts before it and leaves the rest):
// the critical front's crowding and its descending sort, by the whole grid.
__global__ void __launch_bounds__(kGridSortThreads) select_best_big_kernel(
    const double *__restrict__ pts, uint32_t n, uint32_t m, uint32_t N, const long long *__restrict__ keys,
    const int32_t *__restrict__ front_offsets, const int32_t *__restrict__ front_indices,
    const int32_t *__restrict__ n_fronts, unsigned char *wkey, int32_t *widx, int2 *wlist, int32_t *wpos, double *wcd,
    int32_t *out, peel_state *st)
{
    extern __shared__ __align__(16) unsigned char sort_smem[];
    __shared__ dev::sort_ctl ctl;
    __shared__ int slots[kGridSortWarps * 64];
    const int nf = *n_fronts;
    if (nf < 1 || m < 2u) return;
    int lo = 0, hi = nf - 1; // first front whose end passes N
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (static_cast<uint32_t>(front_offsets[mid + 1]) > N)
            hi = mid;
        else
            lo = mid + 1;
    }
    const int off = front_offsets[lo], L = front_offsets[lo + 1] - off;
    if (L <= kSortSmemCap || static_cast<uint32_t>(off) == N) return;
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x, gn = gridDim.x * blockDim.x;
    const int32_t *mem = front_indices + off; // the whole fronts before it: copied by select_best_kernel
    long long *kb = reinterpret_cast<long long *>(wkey) + off;
    int32_t *v = widx + off;
    const grid_sort_mem g{wlist + off, wpos + 2 * off};
    if (!grid_front_crowding(pts, n, m, keys, mem, L, kb, v, g, st, sort_smem, &ctl, slots, wcd)) return;
    for (uint32_t p = gt; p < static_cast<uint32_t>(L); p += gn) {
        kb[p] = ~order_key(wcd[mem[p]]); // descending, NaN first: greater_than_f
        v[p] = static_cast<int32_t>(p);
    }
    if (!grid_sync(st)) return;
    if (!grid_std_sort(dev::sort_view<long long>{kb, v}, L, g, st, sort_smem, &ctl, slots, &st->sort_err)) return;
    const uint32_t remaining = N - static_cast<uint32_t>(off);
    for (uint32_t j = gt; j < remaining; j += gn) out[off + j] = mem[v[j]];
}

// sort_population_mo's final sort of 0..n-1 by (rank, descending crowding)
// for n > kSortSmemCap, by the whole grid.
__global__ void __launch_bounds__(kGridSortThreads) sort_population_big_kernel(
    const int32_t *__restrict__ rank, const double *__restrict__ crowd, uint32_t n, const int32_t *__restrict__ n_fronts,
    unsigned char *wkey, int32_t *widx, int2 *wlist, int32_t *wpos, int32_t *out, peel_state *st)
{
    extern __shared__ __align__(16) unsigned char sort_smem[];
    __shared__ dev::sort_ctl ctl;
    __shared__ int slots[kGridSortWarps * 64];
    if (*n_fronts < 1 || *reinterpret_cast<volatile int *>(&st->status) != 0) return;
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x, gn = gridDim.x * blockDim.x;
    dev::key2 *kb = reinterpret_cast<dev::key2 *>(wkey);
    for (uint32_t q = gt; q < n; q += gn) {
        kb[q] = dev::key2{rank[q], ~order_key(crowd[q])};
        widx[q] = static_cast<int32_t>(q);
    }
    if (!grid_sync(st)) return;
    const grid_sort_mem g{wlist, wpos};
    if (!grid_std_sort(dev::sort_view<dev::key2>{kb, widx}, static_cast<int>(n), g, st, sort_smem, &ctl, slots,
                       &st->sort_err))
        return;
    for (uint32_t j = gt; j < n; j += gn) out[j] = widx[j];
}

// select_best_N_mo (multi_objective.cpp:344-396) for 2 <= n, 1 <= N < n, by
// one block after the fronts are known: whole fronts while they fit, then the
// critical front's members by descending crowding distance (std::sort of the
// positions 0..L-1 with greater_than_f, ties in std::sort's order).
__global__ void __launch_bounds__(kSortThreads) select_best_kernel(
    const double *__restrict__ pts, uint32_t n, uint32_t m, uint32_t N, const long long *__restrict__ keys,
    const int32_t *__restrict__ front_offsets, const int32_t *__restrict__ front_indices,
    const int32_t *__restrict__ n_fronts, unsigned char *wkey, int32_t *widx, int2 *wlist, int32_t *wpos, double *wcd,
    int32_t *out,
    peel_state *st)
{
    extern __shared__ __align__(16) unsigned char sort_smem[];
    __shared__ dev::sort_ctl ctl;
    __shared__ int slots[kSortWarps * 64];
    __shared__ int s_front;
    const int nf = *n_fronts;
    if (nf < 1) return; // barrier timeout, reported through st->err
    if (threadIdx.x == 0) {
        // first front whose end passes N (front_offsets[nf] = n > N)
        int lo = 0, hi = nf - 1;
        while (lo < hi) {
            const int mid = (lo + hi) / 2;
            if (static_cast<uint32_t>(front_offsets[mid + 1]) > N)
                hi = mid;
            else
                lo = mid + 1;
        }
        s_front = lo;
    }
    __syncthreads();
    const int c = s_front;
    const int off = front_offsets[c], L = front_offsets[c + 1] - off;
    for (int p = threadIdx.x; p < off; p += blockDim.x) out[p] = front_indices[p];
    if (static_cast<uint32_t>(off) == N) return;
    if (m < 2u) {
        if (threadIdx.x == 0) atomicExch(&st->status, kStatusNeedTwoObjectives);
        return;
    }
    if (L > kSortSmemCap) return; // select_best_big_kernel
    const int32_t *mem = front_indices + off;
    const sort_area<long long> a =
        pick_area<long long>(sort_smem, L, reinterpret_cast<long long *>(wkey) + off, widx + off, wlist + off,
                                 wpos + 2 * off);
    front_crowding(pts, n, m, keys, mem, L, a, &ctl, slots, &st->sort_err, wcd);
    for (int p = threadIdx.x; p < L; p += blockDim.x) {
        a.k[p] = ~order_key(wcd[mem[p]]); // descending, NaN first: greater_than_f
        a.v[p] = p;
    }
    __syncthreads();
    dev::block_std_sort(dev::sort_view<long long>{a.k, a.v}, L, a.w, &ctl, slots, &st->sort_err);
    const int remaining = static_cast<int>(N) - off;
    for (int j = threadIdx.x; j < remaining; j += blockDim.x) out[off + j] = mem[a.v[j]];
}

// sort_population_mo's final std::sort (multi_objective.cpp:455-462) of
// 0..n-1 by (rank, descending crowding), by one block.
__global__ void __launch_bounds__(kSortThreads) sort_population_kernel(
    const int32_t *__restrict__ rank, const double *__restrict__ crowd, uint32_t n, const int32_t *__restrict__ n_fronts,
    unsigned char *wkey, int32_t *widx, int2 *wlist, int32_t *wpos, int32_t *out, peel_state *st)
{
    extern __shared__ __align__(16) unsigned char sort_smem[];
    __shared__ dev::sort_ctl ctl;
    __shared__ int slots[kSortWarps * 64];
    if (*n_fronts < 1 || st->status != 0) return;
    const int L = static_cast<int>(n);
    const sort_area<dev::key2> a =
        pick_area<dev::key2>(sort_smem, L, reinterpret_cast<dev::key2 *>(wkey), widx, wlist, wpos);
    for (int q = threadIdx.x; q < L; q += blockDim.x) {
        a.k[q] = dev::key2{rank[q], ~order_key(crowd[q])};
        a.v[q] = q;
    }
    __syncthreads();
    dev::block_std_sort(dev::sort_view<dev::key2>{a.k, a.v}, L, a.w, &ctl, slots, &st->sort_err);
    for (int j = threadIdx.x; j < L; j += blockDim.x) out[j] = a.v[j];
}

// (key, value) pairs of a caller's device buffers sorted in place by one
// block, with std::sort's order of ties.
__global__ void __launch_bounds__(kSortThreads) sort_pairs_kernel(long long *k, int32_t *v, uint32_t n, int2 *wlist,
                                                                  int32_t *wpos, int *err)
{
    extern __shared__ __align__(16) unsigned char sort_smem[];
    __shared__ dev::sort_ctl ctl;
    __shared__ int slots[kSortWarps * 64];
    const int L = static_cast<int>(n);
    const sort_area<long long> a = pick_area<long long>(sort_smem, L, k, v, wlist, wpos);
    const bool staged = a.k != k;
    if (staged) {
        for (int p = threadIdx.x; p < L; p += blockDim.x) {
            a.k[p] = k[p];
            a.v[p] = v[p];
        }
    }
    __syncthreads();
    dev::block_std_sort(dev::sort_view<long long>{a.k, a.v}, L, a.w, &ctl, slots, err);
    if (staged) {
        for (int p = threadIdx.x; p < L; p += blockDim.x) {
            k[p] = a.k[p];
            v[p] = a.v[p];
        }
    }
}

// The same for n > kSortSmemCap, by the whole grid (cooperative launch).
__global__ void __launch_bounds__(kGridSortThreads) sort_pairs_grid_kernel(long long *k, int32_t *v, uint32_t n,
                                                                          int2 *wlist, int32_t *wpos, peel_state *st,
                                                                          int *err)
{
    extern __shared__ __align__(16) unsigned char sort_smem[];
    __shared__ dev::sort_ctl ctl;
    __shared__ int slots[kGridSortWarps * 64];
    const grid_sort_mem g{wlist, wpos};
    if (!grid_std_sort(dev::sort_view<long long>{k, v}, static_cast<int>(n), g, st, sort_smem, &ctl, slots, err)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(err, 100); // a grid barrier gave up
    }
}

// Self-test of the bounded grid barrier: block 1 never arrives, so block 0's
// wait runs out after spin_limit polls and flags st->err, and the kernel
// returns. Launched cooperatively with two blocks (both resident).
__global__ void barrier_timeout_test_kernel(peel_state *st, unsigned long long spin_limit)
{
    if (blockIdx.x != 0) return;
    grid_sync(st, spin_limit);
}

// out[i] = i (corner cases of select_best_N_mo / sort_population_mo).
__global__ void iota_kernel(int32_t *out, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = static_cast<int32_t>(i);
}

// Device status word of the MO entry points: 0 ok, -1 a grid barrier gave up,
// 1 crowding over fewer than two objectives (the reference throws), 2 broken
// sort invariant.
__global__ void mo_status_kernel(const peel_state *st, int32_t *status)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
        *status = st->err ? -1 : st->status ? 1 : st->sort_err ? 2 : 0;
}

// One front holding every point: rank 0, identity order.
__global__ void single_front_kernel(uint32_t n, int32_t *rank, int32_t *front_offsets, int32_t *front_indices,
                                    int32_t *n_fronts)
{
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        rank[q] = 0;
        front_indices[q] = static_cast<int32_t>(q);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        front_offsets[0] = 0;
        front_offsets[1] = static_cast<int32_t>(n);
        *n_fronts = 1;
    }
}

// Dominates-matrix rows (bit j of row i: i dominates j) for the dom_list output.
template <int M>
__global__ void __launch_bounds__(256) dominates_rows_kernel(const long long *__restrict__ keys, uint32_t n, uint32_t m,
                                                             uint32_t W, uint32_t W8, uint32_t *__restrict__ D,
                                                             int64_t *__restrict__ row_count)
{
    constexpr int MS = M > 0 ? M : 1;
    __shared__ long long ik_s[MS][32];
    __shared__ uint32_t tile[32][9];
    const uint32_t I0 = blockIdx.y * 32u;
    const uint32_t w0 = blockIdx.x * 8u;
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    if constexpr (M > 0) {
        for (unsigned t = threadIdx.x; t < static_cast<unsigned>(M) * 32u; t += blockDim.x) {
            const unsigned k = t >> 5, ii = t & 31u;
            const uint32_t i = I0 + ii;
            ik_s[k][ii] = i < n ? keys[static_cast<uint64_t>(k) * n + i] : 0;
        }
    }
    const uint32_t w = w0 + warp;
    const uint32_t j = w * 32u + lane;
    const bool jv = (w < W) && (j < n);
    long long jk[MS];
    if (M > 0) {
#pragma unroll
        for (int k = 0; k < MS; ++k) jk[k] = jv ? keys[static_cast<uint64_t>(k) * n + j] : 0;
    }
    __syncthreads();
    for (unsigned ii = 0; ii < 32u; ++ii) {
        const uint32_t i = I0 + ii;
        bool d = false;
        if (jv && i < n) {
            bool le = true, lt = false;
            if (M > 0) {
#pragma unroll
                for (int k = 0; k < MS; ++k) {
                    const long long a = ik_s[k][ii];
                    le &= a <= jk[k];
                    lt |= a < jk[k];
                }
            } else {
                for (uint32_t k = 0; k < m; ++k) {
                    const long long a = keys[static_cast<uint64_t>(k) * n + i];
                    const long long b = keys[static_cast<uint64_t>(k) * n + j];
                    le &= a <= b;
                    lt |= a < b;
                }
            }
            d = le && lt;
        }
        const unsigned word = __ballot_sync(kFull, d);
        if (lane == 0) tile[ii][warp] = word;
    }
    __syncthreads();
    const unsigned ii = threadIdx.x >> 3, ww = threadIdx.x & 7u;
    const uint32_t i = I0 + ii;
    const uint32_t word = tile[ii][ww];
    if (i < n && w0 + ww < W8) D[static_cast<uint64_t>(i) * W8 + w0 + ww] = word;
    int c = __popc(word);
    c += __shfl_xor_sync(kFull, c, 4);
    c += __shfl_xor_sync(kFull, c, 2);
    c += __shfl_xor_sync(kFull, c, 1);
    if (ww == 0 && i < n && c) atomicAdd(reinterpret_cast<unsigned long long *>(&row_count[i]), static_cast<unsigned long long>(c));
}

// Writes the set bits of each D row, ascending, at its CSR offset.
__global__ void dom_list_extract_kernel(const uint32_t *__restrict__ D, uint32_t n, uint32_t W, uint32_t W8,
                                        const int64_t *__restrict__ offsets, int32_t *__restrict__ out)
{
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = gwarp; i < n; i += nwarps) {
        const uint32_t *row = D + static_cast<uint64_t>(i) * W8;
        int64_t base = offsets[i];
        for (uint32_t b = 0; b < W; b += 32u) {
            const uint32_t w = b + lane;
            uint32_t bits = w < W ? row[w] : 0u;
            const int c = __popc(bits);
            // exclusive prefix over lanes
            int pre = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(kFull, pre, o);
                if (lane >= static_cast<unsigned>(o)) pre += v;
            }
            const int total = __shfl_sync(kFull, pre, 31);
            int64_t at = base + pre - c;
            while (bits) {
                const int t = __ffs(bits) - 1;
                bits &= bits - 1u;
                out[at++] = static_cast<int32_t>(w * 32u + t);
            }
            base += total;
        }
    }
}

int blocks_for(uint64_t work, int threads, int num_sms)
{
    const uint64_t need = (work + threads - 1) / threads;
    const uint64_t cap = static_cast<uint64_t>(num_sms) * 8u;
    return static_cast<int>(need < 1 ? 1 : (need < cap ? need : cap));
}

int launch_dominance(const long long *keys, uint32_t n, uint32_t m, uint32_t W, uint32_t W8, uint32_t *Dt,
                     int32_t *dom_count, long long *runs, uint32_t *packed, int num_sms, cudaStream_t s,
                     uint64_t *launches)
{
    if (m >= 1u && m <= 4u && n <= kRankPoints && runs != nullptr) {
        if (W8 > W)
            PGX_CUDA(cudaMemset2DAsync(Dt + W, static_cast<size_t>(W8) * 4u, 0, static_cast<size_t>(W8 - W) * 4u, n,
                                       s));
        const uint32_t nb = (n + kRankRun - 1u) / kRankRun;
        rank_runs_kernel<<<dim3(nb, m), kRankRun / 2u, 0, s>>>(keys, n, runs);
        PGX_CUDA(cudaGetLastError());
        uint32_t *pa = packed, *pb = packed + n;
        PGX_CUDA(cudaMemsetAsync(packed, 0, 2u * static_cast<size_t>(n) * sizeof(uint32_t), s));
        rank_search_kernel<<<dim3((n + 1023u) / 1024u, nb * m), 256, 0, s>>>(keys, n, runs, nb, pa, pb);
        PGX_CUDA(cudaGetLastError());
        dim3 grid((W + 7u) / 8u, W);
        if (m <= 2u)
            dominance_sym_packed_kernel<1><<<grid, 256, 0, s>>>(pa, pb, n, W8, Dt);
        else
            dominance_sym_packed_kernel<2><<<grid, 256, 0, s>>>(pa, pb, n, W8, Dt);
        PGX_CUDA(cudaGetLastError());
        const int blocks = static_cast<int>(std::min<uint64_t>((static_cast<uint64_t>(n) + 7u) / 8u, 65535u));
        row_popcount_kernel<<<blocks, 256, 0, s>>>(Dt, n, W8, dom_count);
        PGX_CUDA(cudaGetLastError());
        *launches += 4;
        return PGX_OK;
    }
    *launches += m <= 4u ? 2 : 1; // dominance tiles (+ row popcounts)
    if (m >= 1u && m <= 4u) {
        // symmetric tiles cover words 0 .. W-1 of every row; zero the padding words W .. W8-1
        if (W8 > W)
            PGX_CUDA(cudaMemset2DAsync(Dt + W, static_cast<size_t>(W8) * 4u, 0, static_cast<size_t>(W8 - W) * 4u, n,
                                       s));
        dim3 grid((W + 7u) / 8u, W);
        switch (m) {
            case 1: dominance_sym_kernel<1><<<grid, 256, 0, s>>>(keys, n, W8, Dt); break;
            case 2: dominance_sym_kernel<2><<<grid, 256, 0, s>>>(keys, n, W8, Dt); break;
            case 3: dominance_sym_kernel<3><<<grid, 256, 0, s>>>(keys, n, W8, Dt); break;
            default: dominance_sym_kernel<4><<<grid, 256, 0, s>>>(keys, n, W8, Dt); break;
        }
        PGX_CUDA(cudaGetLastError());
        const int blocks = static_cast<int>(std::min<uint64_t>((static_cast<uint64_t>(n) + 7u) / 8u, 65535u));
        row_popcount_kernel<<<blocks, 256, 0, s>>>(Dt, n, W8, dom_count);
        PGX_CUDA(cudaGetLastError());
        return PGX_OK;
    }
    dim3 grid((W8 + 7u) / 8u, (n + 31u) / 32u);
    dominance_kernel<0><<<grid, 256, 0, s>>>(keys, n, m, W, W8, Dt, dom_count);
    PGX_CUDA(cudaGetLastError());
    return PGX_OK;
}

int launch_dominates_rows(const long long *keys, uint32_t n, uint32_t m, uint32_t W, uint32_t W8, uint32_t *D,
                          int64_t *row_count, cudaStream_t s)
{
    dim3 grid((W8 + 7u) / 8u, (n + 31u) / 32u);
    switch (m) {
        case 1: dominates_rows_kernel<1><<<grid, 256, 0, s>>>(keys, n, m, W, W8, D, row_count); break;
        case 2: dominates_rows_kernel<2><<<grid, 256, 0, s>>>(keys, n, m, W, W8, D, row_count); break;
        case 3: dominates_rows_kernel<3><<<grid, 256, 0, s>>>(keys, n, m, W, W8, D, row_count); break;
        case 4: dominates_rows_kernel<4><<<grid, 256, 0, s>>>(keys, n, m, W, W8, D, row_count); break;
        default: dominates_rows_kernel<0><<<grid, 256, 0, s>>>(keys, n, m, W, W8, D, row_count); break;
    }
    PGX_CUDA(cudaGetLastError());
    return PGX_OK;
}

__global__ void init_rem_kernel(uint32_t *rem, uint32_t n, uint32_t W8)
{
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < W8; w += gridDim.x * blockDim.x) {
        const uint32_t lo = w * 32u;
        uint32_t v = 0u;
        if (lo + 32u <= n)
            v = kFull;
        else if (lo < n)
            v = (1u << (n - lo)) - 1u;
        rem[w] = v;
    }
}

constexpr uint64_t kMaxPoints = 1u << 19; // 524288 points: a 32 GiB bit matrix

constexpr size_t align256(size_t b)
{
    return (b + 255u) & ~static_cast<size_t>(255u);
}

// Device scratch of one survival pass (global memory beyond the inputs and
// outputs). Laid out back to back, each piece 256-byte aligned.
struct survival_scratch {
    long long *keys;     // m * n order keys (objective-major)
    uint32_t *Dt;        // n * W8 dominated-by bit matrix
    peel_state *st;      // barrier, counters, status
    uint32_t *rem;       // W8 unassigned-point bit set
    int32_t *list;       // 2 n members of the front being built (two parities)
    int32_t *keyv;       // 2 n their ordering keys
    int32_t *wit;        // n peeling witnesses
    int32_t *cnt;        // n + 2 per-front member counters
    unsigned char *wkey; // n * 16 B sort keys of fronts too large for shared memory
    int32_t *widx;       // n sort values
    int2 *wlist;         // n sort ranges
    int32_t *wpos;       // 2 n sort stopper positions
    double *wcd;         // n crowding distances (select_best_N_mo, sort_population_mo)
    long long *runs;     // m * ceil(n / kRankRun) * kRankRun sorted key runs (n <= kRankPoints, m <= 4)
};

constexpr uint64_t rank_runs_bytes(uint64_t n, uint64_t m)
{
    return n <= kRankPoints && m >= 1u && m <= 4u ? m * ((n + kRankRun - 1u) / kRankRun) * kRankRun * 8u : 0u;
}

constexpr size_t survival_scratch_bytes(uint64_t n, uint64_t m)
{
    return align256(n * (m > 0 ? m : 1) * sizeof(long long))
           + align256(n * ((((n + 31u) / 32u) + 7u) & ~uint64_t(7)) * 4u) + align256(sizeof(peel_state))
           + align256(((((n + 31u) / 32u) + 7u) & ~uint64_t(7)) * 4u) + 2u * align256(2u * n * 4u)
           + align256(n * 4u) + align256((n + 2u) * 4u) + align256(n * 16u)
           + align256(n * 4u) + align256(n * sizeof(int2)) + align256(2u * n * 4u) + align256(n * sizeof(double))
           + align256(rank_runs_bytes(n, m));
}

survival_scratch carve_survival_scratch(void *base, uint64_t n, uint64_t m)
{
    const uint64_t mm = m > 0 ? m : 1;
    const uint64_t W8 = (((n + 31u) / 32u) + 7u) & ~uint64_t(7);
    char *p = static_cast<char *>(base);
    survival_scratch s{};
    s.keys = reinterpret_cast<long long *>(p);
    p += align256(n * mm * sizeof(long long));
    s.Dt = reinterpret_cast<uint32_t *>(p);
    p += align256(n * W8 * 4u);
    s.st = reinterpret_cast<peel_state *>(p);
    p += align256(sizeof(peel_state));
    s.rem = reinterpret_cast<uint32_t *>(p);
    p += align256(W8 * 4u);
    s.list = reinterpret_cast<int32_t *>(p);
    p += align256(2u * n * 4u);
    s.keyv = reinterpret_cast<int32_t *>(p);
    p += align256(2u * n * 4u);
    s.wit = reinterpret_cast<int32_t *>(p);
    p += align256(n * 4u);
    s.cnt = reinterpret_cast<int32_t *>(p);
    p += align256((n + 2u) * 4u);
    s.wkey = reinterpret_cast<unsigned char *>(p);
    p += align256(n * 16u);
    s.widx = reinterpret_cast<int32_t *>(p);
    p += align256(n * 4u);
    s.wlist = reinterpret_cast<int2 *>(p);
    p += align256(n * sizeof(int2));
    s.wpos = reinterpret_cast<int32_t *>(p);
    p += align256(2u * n * 4u);
    s.wcd = reinterpret_cast<double *>(p);
    p += align256(n * sizeof(double));
    s.runs = rank_runs_bytes(n, m) ? reinterpret_cast<long long *>(p) : nullptr;
    return s;
}

// Kernels launch_front_crowding issues for n points of m objectives.
constexpr int crowding_launches(uint32_t n, uint32_t m)
{
    return n > static_cast<uint32_t>(kSortSmemCap) && m >= 2u ? 2 : 1;
}

// Cooperative launch of a grid-sort kernel: one block of kGridSortThreads per
// SM (the grid barriers need every block resident).
template <typename... A>
int launch_cooperative_sort_kernel(const void *kernel, int num_sms, cudaStream_t s, A... args)
{
    PGX_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(kSortSmemBytes)));
    int occ = 0;
    PGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kGridSortThreads, kSortSmemBytes));
    PGX_CHECK(occ >= 1, PGX_ERR_CUDA, "grid sort kernel cannot be resident");
    void *argv[] = {static_cast<void *>(&args)...};
    PGX_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(num_sms), dim3(kGridSortThreads), argv, kSortSmemBytes, s));
    return PGX_OK;
}

int launch_front_crowding(const survival_scratch &sc, const double *d_points, uint32_t n, uint32_t m,
                          const int32_t *front_offsets, const int32_t *front_indices, const int32_t *n_fronts,
                          int mode, double *cd, int num_sms, cudaStream_t s)
{
    PGX_CUDA(cudaFuncSetAttribute(front_crowding_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(kSortSmemBytes)));
    const int grid = static_cast<int>(std::min<uint64_t>(n, static_cast<uint64_t>(num_sms) * 2u));
    front_crowding_kernel<<<grid, kSortThreads, kSortSmemBytes, s>>>(d_points, n, m, sc.keys, front_offsets,
                                                                     front_indices, n_fronts, mode, sc.wkey, sc.widx,
                                                                     sc.wlist, sc.wpos, cd, sc.st);
    PGX_CUDA(cudaGetLastError());
    if (n > static_cast<uint32_t>(kSortSmemCap) && m >= 2u) {
        // fronts longer than the shared-memory sorts: every SM on each of them
        PGX_TRY(launch_cooperative_sort_kernel(reinterpret_cast<const void *>(big_crowding_kernel), num_sms, s,
                                               d_points, n, m, sc.keys, front_offsets, front_indices, n_fronts,
                                               sc.wkey, sc.widx, sc.wlist, sc.wpos, cd, sc.st));
    }
    return PGX_OK;
}

// The whole survival pass on `stream` over caller-provided scratch: clears
// what must start at zero, builds keys and the bit matrix, peels the fronts
// (cooperative launch) and, when out.crowding is set, computes the crowding
// distances. *launches counts the kernels launched.
int run_survival(const survival_scratch &sc, const double *d_points, uint32_t n, uint32_t m,
                 const survival_out &out, int num_sms, cudaStream_t s, uint64_t *launches)
{
    const uint32_t W = (n + 31u) / 32u;
    const uint32_t W8 = (W + 7u) & ~7u;
    PGX_CUDA(cudaMemsetAsync(out.dom_count, 0, static_cast<size_t>(n) * sizeof(int32_t), s));
    PGX_CUDA(cudaMemsetAsync(sc.st, 0, sizeof(peel_state), s));
    PGX_CUDA(cudaMemsetAsync(out.front_offsets, 0, (static_cast<size_t>(n) + 1u) * sizeof(int32_t), s));
    init_rem_kernel<<<blocks_for(W8, 256, num_sms), 256, 0, s>>>(sc.rem, n, W8);
    PGX_CUDA(cudaGetLastError());
    *launches += 1;
    if (m > 0) {
        order_keys_kernel<<<blocks_for(static_cast<uint64_t>(n) * m, 256, num_sms), 256, 0, s>>>(d_points, n, m,
                                                                                                 sc.keys);
        PGX_CUDA(cudaGetLastError());
        // the packed ranks borrow the keyv area (2 n words), free until the peel
        PGX_TRY(launch_dominance(sc.keys, n, m, W, W8, sc.Dt, out.dom_count, sc.runs,
                                 reinterpret_cast<uint32_t *>(sc.keyv), num_sms, s, launches));
        *launches += 1; // keys
    } else {
        PGX_CUDA(cudaMemsetAsync(sc.Dt, 0, static_cast<size_t>(n) * W8 * sizeof(uint32_t), s));
    }

    // cooperative peel: every block resident at once (the grid barrier needs it);
    // with crowding, kCrowdBlocks of the blocks compute the crowding distances
    // of each front as soon as the others have peeled it
    const bool fused = out.crowding != nullptr && m >= 2u && num_sms > 2 * kCrowdBlocks;
    const uint32_t npeel = static_cast<uint32_t>(fused ? num_sms - kCrowdBlocks : num_sms);
    const uint32_t wpb = (W + npeel - 1u) / npeel;
    bool crowded = false;
    if (W <= static_cast<uint32_t>(kRemWords) && 32u * wpb <= static_cast<uint32_t>(kQueue)
        && n <= static_cast<uint64_t>(kQueue) * npeel) {
        size_t smem2 = (3u * static_cast<size_t>(W) + 4u * kTile + kQueue + 64u * wpb) * sizeof(int32_t)
                       + (n <= kPosPoints ? static_cast<size_t>(W) * 4u + 2u * ((static_cast<size_t>(n) * 2u + 3u) & ~size_t(3))
                                          : 0u);
        if (fused) smem2 = std::max(smem2, kSortSmemBytes);
        PGX_CUDA(cudaFuncSetAttribute(peel2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(smem2)));
        int occ2 = 0;
        PGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, peel2_kernel, kPeelThreads, smem2));
        PGX_CHECK(occ2 >= 1, PGX_ERR_CUDA, "peel kernel cannot be resident");
        PGX_CUDA(cudaMemsetAsync(sc.cnt, 0, (static_cast<size_t>(n) + 2u) * sizeof(int32_t), s));
        // first witnesses, on every SM (sc.widx holds their resume words until the crowding sorts)
        rem_outside_front0_kernel<<<blocks_for(static_cast<uint64_t>(W) * 32u, 256, num_sms), 256, 0, s>>>(
            out.dom_count, n, W, sc.rem);
        PGX_CUDA(cudaGetLastError());
        {
            const uint64_t wblocks = std::min<uint64_t>((static_cast<uint64_t>(n) + 7u) / 8u,
                                                        static_cast<uint64_t>(num_sms) * 8u);
            witness_init_kernel<<<static_cast<unsigned>(wblocks), 256, static_cast<size_t>(W8) * 4u, s>>>(
                sc.Dt, out.dom_count, sc.rem, n, W, W8, sc.wit, sc.widx);
            PGX_CUDA(cudaGetLastError());
        }
        *launches += 2;
        peel2_args pa{sc.Dt, out.dom_count, n, W, W8, sc.wit, sc.widx, sc.list, sc.keyv, sc.cnt,
                      out.rank, out.front_offsets, out.front_indices, sc.st, npeel, d_points, m, sc.keys,
                      fused ? out.crowding : nullptr, kCrowdNsga2};
        void *args2[] = {&pa};
        PGX_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(peel2_kernel), dim3(num_sms),
                                             dim3(kPeelThreads), args2, smem2, s));
        *launches += 1;
        crowded = fused;
    } else {
    const size_t smem = 2u * kTile * sizeof(int32_t);
    int occ = 0;
    PGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, peel_kernel, kPeelThreads, smem));
    PGX_CHECK(occ >= 1, PGX_ERR_CUDA, "peel kernel cannot be resident");
    if (occ > 1) occ = 1;
    const int grid = num_sms * occ;
    {
        const uint32_t *a0 = sc.Dt;
        uint32_t a1 = n, a2 = W, a3 = W8;
        uint32_t *a4 = sc.rem;
        int32_t *a5 = sc.list, *a6 = sc.keyv, *a7 = out.rank, *a8 = out.front_offsets, *a9 = out.front_indices;
        peel_state *a10 = sc.st;
        void *args[] = {&a0, &a1, &a2, &a3, &a4, &a5, &a6, &a7, &a8, &a9, &a10};
        PGX_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(peel_kernel), dim3(grid), dim3(kPeelThreads), args,
                                             smem, s));
        *launches += 1;
    }
    }
    PGX_CUDA(cudaMemcpyAsync(out.n_fronts, &sc.st->n_fronts, sizeof(int32_t), cudaMemcpyDeviceToDevice, s));

    if (crowded) {
        if (n > static_cast<uint32_t>(kSortSmemCap)) {
            // fronts longer than the shared-memory sorts: every SM on each of them
            PGX_TRY(launch_cooperative_sort_kernel(reinterpret_cast<const void *>(big_crowding_kernel), num_sms, s,
                                                   d_points, n, m, sc.keys, out.front_offsets, out.front_indices,
                                                   out.n_fronts, sc.wkey, sc.widx, sc.wlist, sc.wpos, out.crowding,
                                                   sc.st));
            *launches += 1;
        }
    } else if (out.crowding) {
        PGX_TRY(launch_front_crowding(sc, d_points, n, m, out.front_offsets, out.front_indices, out.n_fronts,
                                      kCrowdNsga2, out.crowding, num_sms, s));
        *launches += crowding_launches(n, m);
    }
    return PGX_OK;
}

int check_survival_shape(uint64_t n, uint64_t m)
{
    PGX_CHECK(n >= 2u, PGX_ERR_INVALID,
              "At least two points are needed for fast_non_dominated_sorting: " + std::to_string(n) + " detected.");
    PGX_CHECK(n <= kMaxPoints, PGX_ERR_CAPACITY, "fast_non_dominated_sorting: more than 524288 points");
    PGX_CHECK(m <= 4096u, PGX_ERR_CAPACITY, "fast_non_dominated_sorting: more than 4096 objectives");
    return PGX_OK;
}

} // namespace

int launch_survival(pgx_context *ctx, const double *d_points, uint64_t n, uint64_t m, const survival_out &out,
                    cudaStream_t s)
{
    PGX_TRY(check_survival_shape(n, m));
    PGX_TRY(ctx->s_state.ensure(survival_scratch_bytes(n, m)));
    const survival_scratch sc = carve_survival_scratch(ctx->s_state.ptr, n, m);
    return run_survival(sc, d_points, static_cast<uint32_t>(n), static_cast<uint32_t>(m), out, ctx->num_sms, s,
                        &ctx->launches);
}

// After a synchronisation: PGX_ERR_TIMEOUT when a grid barrier of the last
// survival pass on this context gave up.
int read_survival_status(pgx_context *ctx, uint64_t n, uint64_t m)
{
    const survival_scratch sc = carve_survival_scratch(ctx->s_state.ptr, n, m);
    peel_state st{};
    PGX_CUDA(cudaMemcpy(&st, sc.st, sizeof(peel_state), cudaMemcpyDeviceToHost));
    PGX_CHECK(st.err == 0, PGX_ERR_TIMEOUT, "fast_non_dominated_sorting: a grid barrier timed out on the device");
    PGX_CHECK(st.sort_err == 0, PGX_ERR_CUDA, "device sort: internal error " + std::to_string(st.sort_err));
    return PGX_OK;
}

int launch_crowding_single(pgx_context *ctx, const double *d_points, uint64_t n64, uint64_t m64, double *d_out,
                           cudaStream_t s)
{
    PGX_CHECK(n64 >= 2u, PGX_ERR_INVALID,
              "A non dominated front must contain at least two points: " + std::to_string(n64) + " detected.");
    PGX_CHECK(m64 >= 2u, PGX_ERR_INVALID,
              "Points in the non dominated front must contain at least two objectives: " + std::to_string(m64)
                  + " detected.");
    PGX_CHECK(n64 <= kMaxPoints && m64 <= 4096u, PGX_ERR_CAPACITY, "crowding_distance: input too large");
    const uint32_t n = static_cast<uint32_t>(n64), m = static_cast<uint32_t>(m64);
    const int sms = ctx->num_sms;
    // keys, status and the sort work arrays come from the survival scratch layout (no bit matrix use)
    PGX_TRY(ctx->s_state.ensure(survival_scratch_bytes(n, m)));
    const survival_scratch sc = carve_survival_scratch(ctx->s_state.ptr, n, m);
    const size_t b_rank = align256(static_cast<size_t>(n) * 4u);
    const size_t b_off = align256(2u * 4u);
    PGX_TRY(ctx->s_outs.ensure(2u * b_rank + b_off + 256u));
    int32_t *rank = ctx->s_outs.as<int32_t>();
    int32_t *front_indices = reinterpret_cast<int32_t *>(ctx->s_outs.as<char>() + b_rank);
    int32_t *front_offsets = reinterpret_cast<int32_t *>(ctx->s_outs.as<char>() + 2u * b_rank);
    int32_t *n_fronts = reinterpret_cast<int32_t *>(ctx->s_outs.as<char>() + 2u * b_rank + b_off);
    const uint64_t nm = static_cast<uint64_t>(n) * m;
    PGX_CUDA(cudaMemsetAsync(sc.st, 0, sizeof(peel_state), s));
    single_front_kernel<<<blocks_for(n, 256, sms), 256, 0, s>>>(n, rank, front_offsets, front_indices, n_fronts);
    PGX_CUDA(cudaGetLastError());
    order_keys_kernel<<<blocks_for(nm, 256, sms), 256, 0, s>>>(d_points, n, m, sc.keys);
    PGX_CUDA(cudaGetLastError());
    PGX_TRY(launch_front_crowding(sc, d_points, n, m, front_offsets, front_indices, n_fronts, kCrowdSortPopulation,
                                  d_out, sms, s));
    ctx->launches += 2 + crowding_launches(n, m);
    return PGX_OK;
}

// Output buffers of an fnds pass the MO entry points need but do not return.
struct fnds_bufs {
    survival_out o;
};

int fnds_buffers(pgx_context *ctx, uint32_t n, fnds_bufs *b)
{
    const size_t bn = align256(static_cast<size_t>(n) * 4u);
    const size_t bo = align256((static_cast<size_t>(n) + 1u) * 4u);
    PGX_TRY(ctx->s_outs.ensure(3u * bn + bo + 256u));
    char *p = ctx->s_outs.as<char>();
    b->o.rank = reinterpret_cast<int32_t *>(p);
    b->o.dom_count = reinterpret_cast<int32_t *>(p + bn);
    b->o.front_indices = reinterpret_cast<int32_t *>(p + 2u * bn);
    b->o.front_offsets = reinterpret_cast<int32_t *>(p + 3u * bn);
    b->o.n_fronts = reinterpret_cast<int32_t *>(p + 3u * bn + bo);
    b->o.crowding = nullptr;
    return PGX_OK;
}

int finish_status(const survival_scratch &sc, int32_t *d_status, cudaStream_t s, uint64_t *launches)
{
    if (d_status) {
        mo_status_kernel<<<1, 32, 0, s>>>(sc.st, d_status);
        PGX_CUDA(cudaGetLastError());
        ++*launches;
    }
    return PGX_OK;
}

int launch_iota(int32_t *d_out, uint64_t n, int num_sms, cudaStream_t s, uint64_t *launches)
{
    if (n == 0) return PGX_OK;
    iota_kernel<<<blocks_for(n, 256, num_sms), 256, 0, s>>>(d_out, static_cast<uint32_t>(n));
    PGX_CUDA(cudaGetLastError());
    ++*launches;
    return PGX_OK;
}

int build_dominates_rows(pgx_context *ctx, const double *d_points, uint64_t n64, uint64_t m64, int64_t **d_row_count,
                         cudaStream_t s)
{
    PGX_TRY(check_survival_shape(n64, m64));
    const uint32_t n = static_cast<uint32_t>(n64), m = static_cast<uint32_t>(m64);
    const uint32_t W = (n + 31u) / 32u;
    const uint32_t W8 = (W + 7u) & ~7u;
    const int sms = ctx->num_sms;
    PGX_TRY(ctx->s_state.ensure(survival_scratch_bytes(n, m)));
    const survival_scratch sc = carve_survival_scratch(ctx->s_state.ptr, n, m);
    PGX_TRY(ctx->s_outs.ensure(static_cast<size_t>(n) * sizeof(int64_t)));
    int64_t *cnt = ctx->s_outs.as<int64_t>();
    PGX_CUDA(cudaMemsetAsync(cnt, 0, static_cast<size_t>(n) * sizeof(int64_t), s));
    if (m > 0) {
        order_keys_kernel<<<blocks_for(static_cast<uint64_t>(n) * m, 256, sms), 256, 0, s>>>(d_points, n, m, sc.keys);
        PGX_CUDA(cudaGetLastError());
        PGX_TRY(launch_dominates_rows(sc.keys, n, m, W, W8, sc.Dt, cnt, s));
        ctx->launches += 2;
    } else {
        PGX_CUDA(cudaMemsetAsync(sc.Dt, 0, static_cast<size_t>(n) * W8 * sizeof(uint32_t), s));
    }
    *d_row_count = cnt;
    return PGX_OK;
}

int extract_dom_list(pgx_context *ctx, uint64_t n64, uint64_t m64, const int64_t *d_offsets, int32_t *d_indices,
                     cudaStream_t s)
{
    const uint32_t n = static_cast<uint32_t>(n64);
    const uint32_t W = (n + 31u) / 32u;
    const uint32_t W8 = (W + 7u) & ~7u;
    const survival_scratch sc = carve_survival_scratch(ctx->s_state.ptr, n64, m64);
    dom_list_extract_kernel<<<blocks_for(static_cast<uint64_t>(n) * 32u, 256, ctx->num_sms), 256, 0, s>>>(
        sc.Dt, n, W, W8, d_offsets, d_indices);
    PGX_CUDA(cudaGetLastError());
    ++ctx->launches;
    return PGX_OK;
}

int launch_select_best(pgx_context *ctx, const double *d_points, uint64_t n64, uint64_t m64, uint64_t N64,
                       int32_t *d_out, int32_t *d_status, cudaStream_t s)
{
    const int sms = ctx->num_sms;
    if (d_status) PGX_CUDA(cudaMemsetAsync(d_status, 0, sizeof(int32_t), s));
    if (N64 == 0 || n64 == 0) return PGX_OK;
    if (n64 == 1 || N64 >= n64) return launch_iota(d_out, n64, sms, s, &ctx->launches);
    PGX_TRY(check_survival_shape(n64, m64));
    const uint32_t n = static_cast<uint32_t>(n64), m = static_cast<uint32_t>(m64), N = static_cast<uint32_t>(N64);
    PGX_TRY(ctx->s_state.ensure(survival_scratch_bytes(n, m)));
    const survival_scratch sc = carve_survival_scratch(ctx->s_state.ptr, n, m);
    fnds_bufs fb;
    PGX_TRY(fnds_buffers(ctx, n, &fb));
    PGX_TRY(run_survival(sc, d_points, n, m, fb.o, sms, s, &ctx->launches));
    PGX_CUDA(cudaFuncSetAttribute(select_best_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(kSortSmemBytes)));
    select_best_kernel<<<1, kSortThreads, kSortSmemBytes, s>>>(d_points, n, m, N, sc.keys, fb.o.front_offsets,
                                                               fb.o.front_indices, fb.o.n_fronts, sc.wkey, sc.widx,
                                                               sc.wlist, sc.wpos, sc.wcd, d_out, sc.st);
    PGX_CUDA(cudaGetLastError());
    ++ctx->launches;
    if (n > static_cast<uint32_t>(kSortSmemCap) && m >= 2u) {
        // a critical front longer than the shared-memory sorts: every SM on it
        PGX_TRY(launch_cooperative_sort_kernel(reinterpret_cast<const void *>(select_best_big_kernel), sms, s,
                                               d_points, n, m, N, sc.keys, fb.o.front_offsets, fb.o.front_indices,
                                               fb.o.n_fronts, sc.wkey, sc.widx, sc.wlist, sc.wpos, sc.wcd, d_out,
                                               sc.st));
        ++ctx->launches;
    }
    return finish_status(sc, d_status, s, &ctx->launches);
}

int launch_sort_population(pgx_context *ctx, const double *d_points, uint64_t n64, uint64_t m64, int32_t *d_out,
                           int32_t *d_status, cudaStream_t s)
{
    const int sms = ctx->num_sms;
    if (d_status) PGX_CUDA(cudaMemsetAsync(d_status, 0, sizeof(int32_t), s));
    if (n64 == 0) return PGX_OK;
    if (n64 == 1) return launch_iota(d_out, 1, sms, s, &ctx->launches);
    PGX_TRY(check_survival_shape(n64, m64));
    const uint32_t n = static_cast<uint32_t>(n64), m = static_cast<uint32_t>(m64);
    PGX_TRY(ctx->s_state.ensure(survival_scratch_bytes(n, m)));
    const survival_scratch sc = carve_survival_scratch(ctx->s_state.ptr, n, m);
    fnds_bufs fb;
    PGX_TRY(fnds_buffers(ctx, n, &fb));
    PGX_TRY(run_survival(sc, d_points, n, m, fb.o, sms, s, &ctx->launches));
    PGX_TRY(launch_front_crowding(sc, d_points, n, m, fb.o.front_offsets, fb.o.front_indices, fb.o.n_fronts,
                                  kCrowdSortPopulation, sc.wcd, sms, s));
    if (n > static_cast<uint32_t>(kSortSmemCap)) {
        PGX_TRY(launch_cooperative_sort_kernel(reinterpret_cast<const void *>(sort_population_big_kernel), sms, s,
                                               static_cast<const int32_t *>(fb.o.rank),
                                               static_cast<const double *>(sc.wcd), n,
                                               static_cast<const int32_t *>(fb.o.n_fronts), sc.wkey, sc.widx,
                                               sc.wlist, sc.wpos, d_out, sc.st));
    } else {
        PGX_CUDA(cudaFuncSetAttribute(sort_population_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(kSortSmemBytes)));
        sort_population_kernel<<<1, kSortThreads, kSortSmemBytes, s>>>(fb.o.rank, sc.wcd, n, fb.o.n_fronts, sc.wkey,
                                                                       sc.widx, sc.wlist, sc.wpos, d_out, sc.st);
        PGX_CUDA(cudaGetLastError());
    }
    ctx->launches += 1 + crowding_launches(n, m);
    return finish_status(sc, d_status, s, &ctx->launches);
}

// Runs barrier_timeout_test_kernel on scratch state of its own; *timed_out
// receives the barrier's error flag (1 expected).
int run_barrier_timeout_test(pgx_context *ctx, uint64_t spin_limit, int32_t *timed_out)
{
    PGX_TRY(ctx->s_crowd.ensure(align256(sizeof(peel_state))));
    peel_state *st = ctx->s_crowd.as<peel_state>();
    cudaStream_t s = ctx->stream;
    PGX_CUDA(cudaMemsetAsync(st, 0, sizeof(peel_state), s));
    unsigned long long limit = spin_limit;
    void *args[] = {&st, &limit};
    PGX_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(barrier_timeout_test_kernel), dim3(2),
                                         dim3(32), args, 0, s));
    ++ctx->launches;
    peel_state h{};
    PGX_CUDA(cudaMemcpyAsync(&h, st, sizeof(peel_state), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaStreamSynchronize(s));
    *timed_out = h.err;
    return PGX_OK;
}

size_t sort_pairs_state_bytes()
{
    return sizeof(peel_state);
}

int launch_sort_pairs(pgx_context *ctx, long long *d_keys, int32_t *d_vals, uint64_t n64, int *d_err, int2 *d_lists,
                      int32_t *d_pos, void *d_state, cudaStream_t s)
{
    if (n64 < 2) return PGX_OK;
    PGX_CHECK(n64 <= (1ull << 30), PGX_ERR_CAPACITY, "sort: more than 2^30 elements");
    if (n64 > static_cast<uint64_t>(kSortSmemCap)) {
        PGX_CUDA(cudaMemsetAsync(d_state, 0, sizeof(peel_state), s));
        PGX_TRY(launch_cooperative_sort_kernel(reinterpret_cast<const void *>(sort_pairs_grid_kernel), ctx->num_sms,
                                               s, d_keys, d_vals, static_cast<uint32_t>(n64), d_lists, d_pos,
                                               static_cast<peel_state *>(d_state), d_err));
        ++ctx->launches;
        return PGX_OK;
    }
    PGX_CUDA(cudaFuncSetAttribute(sort_pairs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(kSortSmemBytes)));
    sort_pairs_kernel<<<1, kSortThreads, kSortSmemBytes, s>>>(d_keys, d_vals, static_cast<uint32_t>(n64), d_lists,
                                                              d_pos, d_err);
    PGX_CUDA(cudaGetLastError());
    ++ctx->launches;
    return PGX_OK;
}

// After a synchronisation, for the last select_best/sort_population pass of
// shape (n, m) on this context: the reference's error for crowding over fewer
// than two objectives, or a timeout / internal error.
int read_mo_status(pgx_context *ctx, uint64_t n, uint64_t m)
{
    const survival_scratch sc = carve_survival_scratch(ctx->s_state.ptr, n, m);
    peel_state st{};
    PGX_CUDA(cudaMemcpy(&st, sc.st, sizeof(peel_state), cudaMemcpyDeviceToHost));
    PGX_CHECK(st.err == 0, PGX_ERR_TIMEOUT, "fast_non_dominated_sorting: a grid barrier timed out on the device");
    PGX_CHECK(st.status == 0, PGX_ERR_INVALID,
              "Points in the non dominated front must contain at least two objectives: " + std::to_string(m)
                  + " detected.");
    PGX_CHECK(st.sort_err == 0, PGX_ERR_CUDA, "device sort: internal error " + std::to_string(st.sort_err));
    return PGX_OK;
}

} // namespace pgx

// ---------------------------------------------------------------------------
// Allocation-free NSGA-II survival.
//
// Some callers cannot call cudaMalloc at the time they evaluate a population:
// an application whose device memory is already claimed by another allocator
// (a framework's caching allocator that reserved most of HBM up front), or a
// latency-bound island thread that must not risk the implicit device-wide
// synchronisation cudaMalloc and cudaFree can cause. pgx_nsga2_survival_device
// grows context buffers on demand, so this variant instead takes its scratch
// (order keys, the dominance bit matrix, peel state, per-objective orders)
// from one array compiled into the library: g_noalloc_scratch, sized for at
// most kNoAllocMaxPoints points and kNoAllocMaxObjectives objectives (about
// 2.6 MB). Larger inputs are rejected with PGX_ERR_CAPACITY. The array is
// device memory of the library's survival module: a device holds it from the
// moment that module is loaded there (at the first call on the device under
// lazy module loading, the default) until the process exits.
//
// Host code cannot use the array's name as a device address (it names a host
// stand-in), so the first call on each device does a set-up with that device
// current: it looks up the array's address with cudaGetSymbolAddress (which
// loads the module, allocating the array) and loads every kernel this pass can
// launch (cudaFuncGetAttributes), so that no later call loads code or data and
// allocates nothing. The set-up is keyed by the device, the current CUDA
// context and the array's address: a call in another context (a driver-API
// context, or the primary context re-created after cudaDeviceReset) repeats
// it. Make the first call on a device before another allocator reserves that
// device's memory and before any stream capture. All calls share the one array
// and it keeps the last call's contents: every pass clears what must start at
// zero itself, and calls whose work overlaps on the GPU (different streams, or
// different host threads) race on the array and must be serialised by the
// caller.
namespace pgx
{
namespace
{

constexpr uint64_t kNoAllocMaxPoints = 4096;
constexpr uint64_t kNoAllocMaxObjectives = 8;
constexpr int kNoAllocMaxDevices = 64;

// the largest layout of at most kNoAllocMaxPoints points and kNoAllocMaxObjectives
// objectives (up to 4 objectives the layout adds the sorted rank runs)
constexpr size_t kNoAllocBytes = survival_scratch_bytes(kNoAllocMaxPoints, kNoAllocMaxObjectives)
                                         > survival_scratch_bytes(kNoAllocMaxPoints, 4)
                                     ? survival_scratch_bytes(kNoAllocMaxPoints, kNoAllocMaxObjectives)
                                     : survival_scratch_bytes(kNoAllocMaxPoints, 4);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

struct noalloc_device {
    void *context = nullptr; // the CUDA context the set-up ran in
    void *scratch = nullptr; // device address of g_noalloc_scratch in that context
    int num_sms = 0;
};

std::mutex g_noalloc_lock;
noalloc_device g_noalloc_devices[kNoAllocMaxDevices];

// The driver's cuCtxGetCurrent, reached through the runtime (no link-time
// dependency on the driver library); null if unavailable.
using ctx_get_current_fn = int (*)(void **);
ctx_get_current_fn ctx_get_current()
{
    static const ctx_get_current_fn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess
            || q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<ctx_get_current_fn>(p);
    }();
    return fn;
}

// Loads every kernel a survival pass of at most kNoAllocMaxPoints points can
// launch, so that none is loaded (and allocated for) at a later call.
int noalloc_load_kernels()
{
    const void *kernels[] = {
        reinterpret_cast<const void *>(init_rem_kernel),
        reinterpret_cast<const void *>(order_keys_kernel),
        reinterpret_cast<const void *>(dominance_sym_kernel<1>),
        reinterpret_cast<const void *>(dominance_sym_kernel<2>),
        reinterpret_cast<const void *>(dominance_sym_kernel<3>),
        reinterpret_cast<const void *>(dominance_sym_kernel<4>),
        reinterpret_cast<const void *>(dominance_kernel<0>),
        reinterpret_cast<const void *>(row_popcount_kernel),
        reinterpret_cast<const void *>(rank_runs_kernel),
        reinterpret_cast<const void *>(rank_search_kernel),
        reinterpret_cast<const void *>(dominance_sym_packed_kernel<1>),
        reinterpret_cast<const void *>(dominance_sym_packed_kernel<2>),
        reinterpret_cast<const void *>(rem_outside_front0_kernel),
        reinterpret_cast<const void *>(witness_init_kernel),
        reinterpret_cast<const void *>(peel2_kernel),
        reinterpret_cast<const void *>(peel_kernel),
        reinterpret_cast<const void *>(front_crowding_kernel),
        reinterpret_cast<const void *>(big_crowding_kernel),
    };
    for (const void *k : kernels) {
        cudaFuncAttributes a{};
        PGX_CUDA(cudaFuncGetAttributes(&a, k));
    }
    return PGX_OK;
}

// Set-up per (device, context), run with that device current.
int noalloc_setup(int device, noalloc_device *out)
{
    std::lock_guard<std::mutex> g(g_noalloc_lock);
    noalloc_device &d = g_noalloc_devices[device];
    void *context = nullptr;
    if (const ctx_get_current_fn get = ctx_get_current()) {
        if (get(&context) != 0) context = nullptr;
    }
    void *p = nullptr;
    PGX_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    if (d.scratch != p || d.context != context || d.num_sms == 0) {
        PGX_TRY(noalloc_load_kernels());
        int sms = 0;
        PGX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        d.num_sms = sms;
        d.context = context;
        d.scratch = p;
    }
    *out = d;
    return PGX_OK;
}

} // namespace
} // namespace pgx

extern "C" int pgx_nsga2_survival_device_noalloc(const double *d_points, uint64_t n, uint64_t m, int32_t *d_rank,
                                                 int32_t *d_dom_count, int32_t *d_front_offsets,
                                                 int32_t *d_front_indices, int32_t *d_n_fronts, double *d_crowding,
                                                 void *stream)
{
    using namespace pgx;
    PGX_CHECK(n >= 2u, PGX_ERR_INVALID,
              "At least two points are needed for fast_non_dominated_sorting: " + std::to_string(n) + " detected.");
    PGX_CHECK(n <= kNoAllocMaxPoints && m <= kNoAllocMaxObjectives, PGX_ERR_CAPACITY,
              "pgx_nsga2_survival_device_noalloc: at most " + std::to_string(kNoAllocMaxPoints) + " points and "
                  + std::to_string(kNoAllocMaxObjectives) + " objectives, got " + std::to_string(n) + " x "
                  + std::to_string(m));
    PGX_CHECK(d_crowding == nullptr || m >= 2u, PGX_ERR_INVALID,
              "Points in the non dominated front must contain at least two objectives: " + std::to_string(m)
                  + " detected.");
    PGX_CHECK(d_points != nullptr || m == 0, PGX_ERR_INVALID, "null points buffer");
    PGX_CHECK(d_rank && d_dom_count && d_front_offsets && d_front_indices && d_n_fronts, PGX_ERR_INVALID,
              "null output buffer");
    PGX_CHECK(survival_scratch_bytes(n, m) <= sizeof(g_noalloc_scratch), PGX_ERR_CAPACITY,
              "pgx_nsga2_survival_device_noalloc: scratch layout exceeds the static array");
    int device = 0;
    PGX_CUDA(cudaGetDevice(&device));
    PGX_CHECK(device >= 0 && device < kNoAllocMaxDevices, PGX_ERR_CAPACITY, "device ordinal too large");
    noalloc_device nd;
    PGX_TRY(noalloc_setup(device, &nd));
    const survival_scratch sc = carve_survival_scratch(nd.scratch, n, m);
    survival_out o;
    o.rank = d_rank;
    o.dom_count = d_dom_count;
    o.front_offsets = d_front_offsets;
    o.front_indices = d_front_indices;
    o.n_fronts = d_n_fronts;
    o.crowding = d_crowding;
    uint64_t launches = 0;
    return run_survival(sc, d_points, static_cast<uint32_t>(n), static_cast<uint32_t>(m), o, nd.num_sms,
                        static_cast<cudaStream_t>(stream), &launches);
}
