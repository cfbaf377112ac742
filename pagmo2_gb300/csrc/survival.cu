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
//  3. peel_kernel: a cooperative persistent kernel peels fronts. Front k+1 is
//     every unassigned point whose row has no unassigned dominator. The
//     reference's order inside a front (first front ascending; later fronts in
//     the order its dom_list traversal appends them) is rebuilt exactly: a
//     point q of front k+1 is appended when its last dominator in front k is
//     processed, so the order is by (max position of q's dominators in front k,
//     q).
//  4. crowding_rank / crowding_accumulate: for each front and objective the
//     sorted position of every point (ties broken by position in the front),
//     then the reference's neighbour differences over the objective range, in
//     objective order per point.
#include "pgx_internal.cuh"

#include <climits>
#include <cmath>

namespace pgx
{
namespace
{

constexpr unsigned kFull = 0xffffffffu;
constexpr unsigned long long kSpinLimit = 1ull << 22; // x 256 ns sleep: about one second

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
    int err;
    int n_fronts;
    int counts[2];
};

// Grid-wide barrier for a cooperative launch; gives up (and flags st->err)
// after about a second instead of waiting forever.
__device__ bool grid_sync(peel_state *st)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = &st->bar_gen;
        const unsigned g0 = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(&st->bar_count, 1u);
        if (arrived == gridDim.x - 1u) {
            atomicExch(&st->bar_count, 0u);
            __threadfence();
            atomicAdd(&st->bar_gen, 1u);
        } else {
            unsigned long long spins = 0;
            while (*vgen == g0) {
                if (++spins > kSpinLimit) {
                    atomicExch(&st->err, 1);
                    break;
                }
                __nanosleep(256);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *reinterpret_cast<volatile int *>(&st->err) == 0;
}

__device__ __forceinline__ int warp_max(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(kFull, v, o));
    return v;
}

// Front peeling. masks[0..2*W8): the bit sets of the current and the next
// front, alternating by iteration parity. rem[W8]: unassigned points.
__global__ void __launch_bounds__(256) peel_kernel(const uint32_t *__restrict__ Dt, uint32_t n, uint32_t W,
                                                   uint32_t W8, uint32_t *rem, uint32_t *masks, int32_t *pos,
                                                   int32_t *list, int32_t *keyv, int32_t *rank, int32_t *front_offsets,
                                                   int32_t *front_indices, peel_state *st)
{
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthreads = gridDim.x * blockDim.x;
    const uint32_t gwarp = tid >> 5, nwarps = nthreads >> 5;
    int offset = 0;
    int k = 0;
    for (;; ++k) {
        uint32_t *next = masks + static_cast<size_t>(k & 1) * W8;
        uint32_t *cur = masks + static_cast<size_t>((k + 1) & 1) * W8;
        int *cnt = &st->counts[k & 1];
        // Phase A: members of front k.
        for (uint32_t j = gwarp; j < n; j += nwarps) {
            if (!((__ldcg(rem + (j >> 5)) >> (j & 31u)) & 1u)) continue;
            const uint32_t *row = Dt + static_cast<uint64_t>(j) * W8;
            bool hit = false;
            for (uint32_t b = 0; b < W; b += 32u) {
                const uint32_t w = b + lane;
                const uint32_t v = w < W ? (__ldg(row + w) & __ldcg(rem + w)) : 0u;
                if (__any_sync(kFull, v != 0u)) {
                    hit = true;
                    break;
                }
            }
            if (!hit && lane == 0) {
                const int s = atomicAdd(cnt, 1);
                list[s] = static_cast<int32_t>(j);
                atomicOr(next + (j >> 5), 1u << (j & 31u));
            }
        }
        if (!grid_sync(st)) return;
        const int L = *reinterpret_cast<volatile int *>(cnt);
        if (L == 0) break;
        // Phase B: retire front k from rem; ordering key of each member.
        for (uint32_t w = tid; w < W; w += nthreads) rem[w] = __ldcg(rem + w) & ~__ldcg(next + w);
        if (k == 0) {
            for (uint32_t s = tid; s < static_cast<uint32_t>(L); s += nthreads) keyv[s] = 0;
        } else {
            for (uint32_t s = gwarp; s < static_cast<uint32_t>(L); s += nwarps) {
                const uint32_t q = static_cast<uint32_t>(__ldcg(list + s));
                const uint32_t *row = Dt + static_cast<uint64_t>(q) * W8;
                int best = -1;
                for (uint32_t w = lane; w < W; w += 32u) {
                    uint32_t bits = __ldg(row + w) & __ldcg(cur + w);
                    while (bits) {
                        const int t = __ffs(bits) - 1;
                        bits &= bits - 1u;
                        best = max(best, __ldcg(pos + w * 32u + t));
                    }
                }
                best = warp_max(best);
                if (lane == 0) keyv[s] = best;
            }
        }
        if (!grid_sync(st)) return;
        // Phase C: position of each member = rank of (key, index) in the front.
        for (uint32_t s = tid; s < static_cast<uint32_t>(L); s += nthreads) {
            const int q = __ldcg(list + s);
            const int kq = __ldcg(keyv + s);
            int p = 0;
            for (int t = 0; t < L; ++t) {
                const int kt = __ldcg(keyv + t);
                const int qt = __ldcg(list + t);
                p += (kt < kq) || (kt == kq && qt < q);
            }
            front_indices[offset + p] = q;
            rank[q] = k;
            pos[q] = p;
        }
        for (uint32_t w = tid; w < W8; w += nthreads) cur[w] = 0u;
        if (tid == 0) {
            st->counts[(k + 1) & 1] = 0;
            front_offsets[k + 1] = offset + L;
        }
        offset += L;
        if (!grid_sync(st)) return;
    }
    if (tid == 0) {
        st->n_fronts = k;
        front_offsets[0] = 0;
    }
}

// Sorted position of every point of a front of size >= 3 along each objective;
// sorted[k*n + off + p] = point. Ties keep front order.
__global__ void crowding_rank_kernel(const long long *__restrict__ keys, uint32_t n, uint32_t m,
                                     const int32_t *__restrict__ rank, const int32_t *__restrict__ pos,
                                     const int32_t *__restrict__ front_offsets,
                                     const int32_t *__restrict__ front_indices, int32_t *__restrict__ sorted,
                                     int32_t *__restrict__ inv_pos)
{
    const uint64_t total = static_cast<uint64_t>(n) * m;
    for (uint64_t t = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < total;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint32_t k = static_cast<uint32_t>(t / n), q = static_cast<uint32_t>(t - static_cast<uint64_t>(k) * n);
        const int f = rank[q];
        const int off = front_offsets[f], end = front_offsets[f + 1];
        if (end - off < 3) continue;
        const long long *kk = keys + static_cast<uint64_t>(k) * n;
        const long long kq = kk[q];
        const int pq = pos[q];
        int p = 0;
        for (int s = off; s < end; ++s) {
            const long long v = kk[front_indices[s]];
            p += (v < kq) || (v == kq && (s - off) < pq);
        }
        sorted[static_cast<uint64_t>(k) * n + off + p] = static_cast<int32_t>(q);
        inv_pos[static_cast<uint64_t>(k) * n + q] = p;
    }
}

// crowding_distance per point: ends of each objective get +inf (assignment),
// interior points add (f[next] - f[prev]) / (f[last] - f[first]); fronts of
// one or two points are +inf (nsga2.cpp:188-193).
__global__ void crowding_accumulate_kernel(const double *__restrict__ pts, uint32_t n, uint32_t m,
                                           const int32_t *__restrict__ rank, const int32_t *__restrict__ front_offsets,
                                           const int32_t *__restrict__ sorted, const int32_t *__restrict__ inv_pos,
                                           double *__restrict__ out)
{
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int f = rank[q];
        const int off = front_offsets[f], end = front_offsets[f + 1];
        const int sz = end - off;
        if (sz < 3) {
            out[q] = HUGE_VAL;
            continue;
        }
        double cd = 0.0;
        for (uint32_t k = 0; k < m; ++k) {
            const int32_t *srt = sorted + static_cast<uint64_t>(k) * n + off;
            const int p = inv_pos[static_cast<uint64_t>(k) * n + q];
            if (p == 0 || p == sz - 1) {
                cd = HUGE_VAL;
            } else {
                const double df = pts[static_cast<uint64_t>(srt[sz - 1]) * m + k] - pts[static_cast<uint64_t>(srt[0]) * m + k];
                cd += (pts[static_cast<uint64_t>(srt[p + 1]) * m + k] - pts[static_cast<uint64_t>(srt[p - 1]) * m + k]) / df;
            }
        }
        out[q] = cd;
    }
}

// One front holding every point: rank 0, identity order.
__global__ void single_front_kernel(uint32_t n, int32_t *rank, int32_t *pos, int32_t *front_offsets,
                                    int32_t *front_indices)
{
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        rank[q] = 0;
        pos[q] = static_cast<int32_t>(q);
        front_indices[q] = static_cast<int32_t>(q);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        front_offsets[0] = 0;
        front_offsets[1] = static_cast<int32_t>(n);
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
                     int32_t *dom_count, cudaStream_t s)
{
    dim3 grid((W8 + 7u) / 8u, (n + 31u) / 32u);
    switch (m) {
        case 1: dominance_kernel<1><<<grid, 256, 0, s>>>(keys, n, m, W, W8, Dt, dom_count); break;
        case 2: dominance_kernel<2><<<grid, 256, 0, s>>>(keys, n, m, W, W8, Dt, dom_count); break;
        case 3: dominance_kernel<3><<<grid, 256, 0, s>>>(keys, n, m, W, W8, Dt, dom_count); break;
        case 4: dominance_kernel<4><<<grid, 256, 0, s>>>(keys, n, m, W, W8, Dt, dom_count); break;
        default: dominance_kernel<0><<<grid, 256, 0, s>>>(keys, n, m, W, W8, Dt, dom_count); break;
    }
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

constexpr uint64_t kMaxPoints = 1u << 19; // 524288 points: a 32 GiB bit matrix

// Scratch layout inside ctx->s_state (device): peel_state, rem, masks, pos,
// list, keyv, sorted, inv_pos.
struct scratch_view {
    peel_state *st;
    uint32_t *rem, *masks;
    int32_t *pos, *list, *keyv, *sorted, *inv_pos;
};

size_t align256(size_t b)
{
    return (b + 255u) & ~static_cast<size_t>(255u);
}

int carve_scratch(pgx_context *ctx, uint64_t n, uint64_t m, uint32_t W8, scratch_view *v)
{
    const size_t mm = m > 0 ? m : 1;
    const size_t b_st = align256(sizeof(peel_state));
    const size_t b_rem = align256(W8 * 4u);
    const size_t b_masks = align256(2u * W8 * 4u);
    const size_t b_n = align256(n * 4u);
    const size_t b_nm = align256(n * mm * 4u);
    PGX_TRY(ctx->s_state.ensure(b_st + b_rem + b_masks + 3u * b_n + 2u * b_nm));
    char *p = ctx->s_state.as<char>();
    v->st = reinterpret_cast<peel_state *>(p);
    p += b_st;
    v->rem = reinterpret_cast<uint32_t *>(p);
    p += b_rem;
    v->masks = reinterpret_cast<uint32_t *>(p);
    p += b_masks;
    v->pos = reinterpret_cast<int32_t *>(p);
    p += b_n;
    v->list = reinterpret_cast<int32_t *>(p);
    p += b_n;
    v->keyv = reinterpret_cast<int32_t *>(p);
    p += b_n;
    v->sorted = reinterpret_cast<int32_t *>(p);
    p += b_nm;
    v->inv_pos = reinterpret_cast<int32_t *>(p);
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

} // namespace

int launch_survival(pgx_context *ctx, const double *d_points, uint64_t n64, uint64_t m64, const survival_out &out,
                    cudaStream_t s)
{
    PGX_CHECK(n64 >= 2u, PGX_ERR_INVALID,
              "At least two points are needed for fast_non_dominated_sorting: " + std::to_string(n64) + " detected.");
    PGX_CHECK(n64 <= kMaxPoints, PGX_ERR_CAPACITY, "fast_non_dominated_sorting: more than 524288 points");
    PGX_CHECK(m64 <= 4096u, PGX_ERR_CAPACITY, "fast_non_dominated_sorting: more than 4096 objectives");
    const uint32_t n = static_cast<uint32_t>(n64), m = static_cast<uint32_t>(m64);
    const uint32_t W = (n + 31u) / 32u;
    const uint32_t W8 = (W + 7u) & ~7u;
    const int sms = ctx->num_sms;

    PGX_TRY(ctx->s_keys.ensure(static_cast<size_t>(n) * (m ? m : 1) * sizeof(long long)));
    PGX_TRY(ctx->s_dommat.ensure(static_cast<size_t>(n) * W8 * sizeof(uint32_t)));
    scratch_view v{};
    PGX_TRY(carve_scratch(ctx, n, m, W8, &v));
    long long *keys = ctx->s_keys.as<long long>();
    uint32_t *Dt = ctx->s_dommat.as<uint32_t>();

    PGX_CUDA(cudaMemsetAsync(out.dom_count, 0, static_cast<size_t>(n) * sizeof(int32_t), s));
    PGX_CUDA(cudaMemsetAsync(v.st, 0, sizeof(peel_state), s));
    PGX_CUDA(cudaMemsetAsync(v.masks, 0, 2u * W8 * sizeof(uint32_t), s));
    PGX_CUDA(cudaMemsetAsync(out.front_offsets, 0, (static_cast<size_t>(n) + 1u) * sizeof(int32_t), s));
    init_rem_kernel<<<blocks_for(W8, 256, sms), 256, 0, s>>>(v.rem, n, W8);
    PGX_CUDA(cudaGetLastError());
    ++ctx->launches;
    if (m > 0) {
        order_keys_kernel<<<blocks_for(static_cast<uint64_t>(n) * m, 256, sms), 256, 0, s>>>(d_points, n, m, keys);
        PGX_CUDA(cudaGetLastError());
        PGX_TRY(launch_dominance(keys, n, m, W, W8, Dt, out.dom_count, s));
        ctx->launches += 2;
    } else {
        PGX_CUDA(cudaMemsetAsync(Dt, 0, static_cast<size_t>(n) * W8 * sizeof(uint32_t), s));
    }

    // cooperative peel: every block resident at once (the grid barrier needs it)
    int occ = 0;
    PGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, peel_kernel, 256, 0));
    if (occ < 1) occ = 1;
    if (occ > 2) occ = 2;
    const int grid = sms * occ;
    {
        const uint32_t *a0 = Dt;
        uint32_t a1 = n, a2 = W, a3 = W8;
        uint32_t *a4 = v.rem, *a5 = v.masks;
        int32_t *a6 = v.pos, *a7 = v.list, *a8 = v.keyv, *a9 = out.rank, *a10 = out.front_offsets,
                *a11 = out.front_indices;
        peel_state *a12 = v.st;
        void *args[] = {&a0, &a1, &a2, &a3, &a4, &a5, &a6, &a7, &a8, &a9, &a10, &a11, &a12};
        PGX_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(peel_kernel), dim3(grid), dim3(256), args,
                                             0, s));
        ++ctx->launches;
    }
    PGX_CUDA(cudaMemcpyAsync(out.n_fronts, &v.st->n_fronts, sizeof(int32_t), cudaMemcpyDeviceToDevice, s));

    if (out.crowding) {
        if (m > 0) {
            const uint64_t nm = static_cast<uint64_t>(n) * m;
            crowding_rank_kernel<<<blocks_for(nm, 256, sms), 256, 0, s>>>(keys, n, m, out.rank, v.pos,
                                                                          out.front_offsets, out.front_indices,
                                                                          v.sorted, v.inv_pos);
            PGX_CUDA(cudaGetLastError());
            ++ctx->launches;
        }
        crowding_accumulate_kernel<<<blocks_for(n, 256, sms), 256, 0, s>>>(d_points, n, m, out.rank,
                                                                           out.front_offsets, v.sorted, v.inv_pos,
                                                                           out.crowding);
        PGX_CUDA(cudaGetLastError());
        ++ctx->launches;
    }
    return PGX_OK;
}

int survival_status(pgx_context *ctx)
{
    PGX_CHECK(ctx->s_state.ptr != nullptr, PGX_ERR_INVALID, "survival_status before any survival call");
    int err = 0;
    PGX_CUDA(cudaMemcpy(&err, &reinterpret_cast<peel_state *>(ctx->s_state.ptr)->err, sizeof(int),
                        cudaMemcpyDeviceToHost));
    PGX_CHECK(err == 0, PGX_ERR_TIMEOUT, "fast_non_dominated_sorting: a grid barrier timed out on the device");
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
    PGX_CHECK(n64 < (1ull << 30) && m64 <= 4096u, PGX_ERR_CAPACITY, "crowding_distance: input too large");
    const uint32_t n = static_cast<uint32_t>(n64), m = static_cast<uint32_t>(m64);
    const int sms = ctx->num_sms;
    const uint32_t W8 = (((n + 31u) / 32u) + 7u) & ~7u;
    PGX_TRY(ctx->s_keys.ensure(static_cast<size_t>(n) * m * sizeof(long long)));
    scratch_view v{};
    PGX_TRY(carve_scratch(ctx, n, m, W8, &v));
    const size_t b_rank = align256(static_cast<size_t>(n) * 4u);
    PGX_TRY(ctx->s_outs.ensure(b_rank + align256((static_cast<size_t>(n) + 1u) * 4u)));
    int32_t *rank = ctx->s_outs.as<int32_t>();
    int32_t *front_offsets = reinterpret_cast<int32_t *>(ctx->s_outs.as<char>() + b_rank);
    int32_t *front_indices = v.list;
    long long *keys = ctx->s_keys.as<long long>();
    const uint64_t nm = static_cast<uint64_t>(n) * m;
    single_front_kernel<<<blocks_for(n, 256, sms), 256, 0, s>>>(n, rank, v.pos, front_offsets, front_indices);
    PGX_CUDA(cudaGetLastError());
    order_keys_kernel<<<blocks_for(nm, 256, sms), 256, 0, s>>>(d_points, n, m, keys);
    PGX_CUDA(cudaGetLastError());
    crowding_rank_kernel<<<blocks_for(nm, 256, sms), 256, 0, s>>>(keys, n, m, rank, v.pos, front_offsets,
                                                                  front_indices, v.sorted, v.inv_pos);
    PGX_CUDA(cudaGetLastError());
    crowding_accumulate_kernel<<<blocks_for(n, 256, sms), 256, 0, s>>>(d_points, n, m, rank, front_offsets, v.sorted,
                                                                       v.inv_pos, d_out);
    PGX_CUDA(cudaGetLastError());
    ctx->launches += 4;
    return PGX_OK;
}

int build_dominates_rows(pgx_context *ctx, const double *d_points, uint64_t n64, uint64_t m64, int64_t **d_row_count,
                         cudaStream_t s)
{
    PGX_CHECK(n64 >= 2u, PGX_ERR_INVALID,
              "At least two points are needed for fast_non_dominated_sorting: " + std::to_string(n64) + " detected.");
    PGX_CHECK(n64 <= kMaxPoints, PGX_ERR_CAPACITY, "fast_non_dominated_sorting: more than 524288 points");
    PGX_CHECK(m64 <= 4096u, PGX_ERR_CAPACITY, "fast_non_dominated_sorting: more than 4096 objectives");
    const uint32_t n = static_cast<uint32_t>(n64), m = static_cast<uint32_t>(m64);
    const uint32_t W = (n + 31u) / 32u;
    const uint32_t W8 = (W + 7u) & ~7u;
    const int sms = ctx->num_sms;
    PGX_TRY(ctx->s_keys.ensure(static_cast<size_t>(n) * (m ? m : 1) * sizeof(long long)));
    PGX_TRY(ctx->s_dommat.ensure(static_cast<size_t>(n) * W8 * sizeof(uint32_t)));
    PGX_TRY(ctx->s_outs.ensure(static_cast<size_t>(n) * sizeof(int64_t)));
    int64_t *cnt = ctx->s_outs.as<int64_t>();
    PGX_CUDA(cudaMemsetAsync(cnt, 0, static_cast<size_t>(n) * sizeof(int64_t), s));
    if (m > 0) {
        long long *keys = ctx->s_keys.as<long long>();
        order_keys_kernel<<<blocks_for(static_cast<uint64_t>(n) * m, 256, sms), 256, 0, s>>>(d_points, n, m, keys);
        PGX_CUDA(cudaGetLastError());
        PGX_TRY(launch_dominates_rows(keys, n, m, W, W8, ctx->s_dommat.as<uint32_t>(), cnt, s));
        ctx->launches += 2;
    } else {
        PGX_CUDA(cudaMemsetAsync(ctx->s_dommat.ptr, 0, static_cast<size_t>(n) * W8 * sizeof(uint32_t), s));
    }
    *d_row_count = cnt;
    return PGX_OK;
}

int extract_dom_list(pgx_context *ctx, uint64_t n64, const int64_t *d_offsets, int32_t *d_indices, cudaStream_t s)
{
    const uint32_t n = static_cast<uint32_t>(n64);
    const uint32_t W = (n + 31u) / 32u;
    const uint32_t W8 = (W + 7u) & ~7u;
    dom_list_extract_kernel<<<blocks_for(static_cast<uint64_t>(n) * 32u, 256, ctx->num_sms), 256, 0, s>>>(
        ctx->s_dommat.as<uint32_t>(), n, W, W8, d_offsets, d_indices);
    PGX_CUDA(cudaGetLastError());
    ++ctx->launches;
    return PGX_OK;
}

} // namespace pgx
