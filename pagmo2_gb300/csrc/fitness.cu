// Batch fitness and gradient kernels for the three single-objective UDPs of
// the reference: rastrigin (src/problems/rastrigin.cpp:62-72, 98-107),
// rosenbrock (src/problems/rosenbrock.cpp:59-66, 83-92) and lennard_jones
// (src/problems/lennard_jones.cpp:72-91, 132-151). The per-row arithmetic
// lives in fitness_dev.cuh; this file maps rows onto the grid and picks the
// variant for each shape.
#include "fitness_dev.cuh"
#include "pgx_internal.cuh"

#include <cstdlib>

namespace pgx
{

// Threads per block for n rows of `lanes` lanes: 256, or fewer for batches
// that would not give every SM a block (4096 rows of 4 lanes fill only 64
// blocks of 256): the blocks shrink (to 64 threads at least) until the grid
// covers the SMs. The lanes per row, and so every row's result, stay the same.
int row_block_threads(uint64_t n, int lanes, int num_sms)
{
    const uint64_t total = n * static_cast<uint64_t>(lanes);
    const uint64_t sms = static_cast<uint64_t>(num_sms > 0 ? num_sms : 1);
    if (total >= 256u * sms) return 256;
    uint64_t t = (total + sms - 1u) / sms;
    t = (t + 31u) & ~uint64_t(31);
    if (t < 64u) t = 64u;
    if (t < static_cast<uint64_t>(lanes)) t = static_cast<uint64_t>(lanes);
    return static_cast<int>(t > 256u ? 256u : t);
}

namespace
{

using namespace dev;

template <int V, int G, bool GRAD>
__global__ void __launch_bounds__(256) rastrigin_kernel(const double *__restrict__ x, uint64_t n, uint32_t nx,
                                                        double *__restrict__ f, double *__restrict__ g)
{
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * (blockDim.x / G);
    for (uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / G; row < n; row += stride)
        rastrigin_row<V, G, GRAD>(x + row * nx, nx, f ? f + row : nullptr, GRAD ? g + row * nx : nullptr);
}

template <int G, bool GRAD>
__global__ void __launch_bounds__(256) rosenbrock_kernel(const double *__restrict__ x, uint64_t n, uint32_t nx,
                                                         double *__restrict__ f, double *__restrict__ g)
{
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * (blockDim.x / G);
    for (uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / G; row < n; row += stride)
        rosenbrock_row<G, GRAD>(x + row * nx, nx, f ? f + row : nullptr, GRAD ? g + row * nx : nullptr);
}

// Griewank's per-column square roots kept in shared memory (8 KiB).
constexpr uint32_t kGriewankRoots = 1024;

// Fitness-only rows of ackley, griewank and schwefel.
template <int G, int KIND>
__global__ void __launch_bounds__(256) row_f_kernel(const double *__restrict__ x, uint64_t n, uint32_t nx,
                                                    double *__restrict__ f, double *__restrict__ g)
{
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * (blockDim.x / G);
    [[maybe_unused]] uint32_t n_root = 0;
    [[maybe_unused]] const double *root = nullptr;
    if constexpr (KIND == PGX_GRIEWANK) {
        __shared__ double roots[kGriewankRoots];
        n_root = nx < kGriewankRoots ? nx : kGriewankRoots;
        for (uint32_t i = threadIdx.x; i < n_root; i += blockDim.x) roots[i] = sqrt(static_cast<double>(i) + 1.0);
        __syncthreads();
        root = roots;
    }
    for (uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / G; row < n; row += stride) {
        double *fo = f ? f + row : nullptr;
        if constexpr (KIND == PGX_ACKLEY)
            ackley_row<G>(x + row * nx, nx, fo);
        else if constexpr (KIND == PGX_GRIEWANK)
            griewank_row<G>(x + row * nx, nx, fo, root, n_root);
        else
            schwefel_row<G>(x + row * nx, nx, fo);
    }
    (void)g;
}

template <bool GRAD>
__global__ void __launch_bounds__(256) rosenbrock_v4_kernel(const double *__restrict__ x, uint64_t n, uint32_t nx,
                                                            double *__restrict__ f, double *__restrict__ g)
{
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * (blockDim.x / 32u);
    for (uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / 32u; row < n; row += stride)
        rosenbrock_row_v4<GRAD>(x + row * nx, nx, f ? f + row : nullptr, GRAD ? g + row * nx : nullptr);
}

template <bool GRAD>
__global__ void __launch_bounds__(256, 4) rosenbrock_v4ff_kernel(const double *__restrict__ x, uint64_t n, uint32_t nx,
                                                              double *__restrict__ f, double *__restrict__ g)
{
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * (blockDim.x / 32u);
    for (uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / 32u; row < n; row += stride)
        rosenbrock_row_v4_ff<GRAD>(x + row * nx, nx, f ? f + row : nullptr, GRAD ? g + row * nx : nullptr);
}

template <int MA, bool GRAD>
__global__ void __launch_bounds__(128) lj_reg_kernel(const double *__restrict__ x, uint64_t n, uint32_t na,
                                                     uint32_t nx, double *__restrict__ f, double *__restrict__ g)
{
    extern __shared__ double smem[];
    const unsigned warp = threadIdx.x >> 5;
    const unsigned wpb = blockDim.x >> 5;
    double *sm = smem + static_cast<size_t>(warp) * (GRAD ? 6u : 3u) * na;
    for (uint64_t c = static_cast<uint64_t>(blockIdx.x) * wpb + warp; c < n; c += static_cast<uint64_t>(gridDim.x) * wpb)
        lj_cluster_reg<MA, GRAD>(x + c * nx, na, nx, sm, f ? f + c : nullptr, GRAD ? g + c * nx : nullptr);
}

template <bool GRAD>
__global__ void __launch_bounds__(128) lj_flat_kernel(const double *__restrict__ x, uint64_t n, uint32_t na,
                                                      uint32_t nx, double *__restrict__ f, double *__restrict__ g)
{
    extern __shared__ double smem[];
    const unsigned warp = threadIdx.x >> 5;
    const unsigned wpb = blockDim.x >> 5;
    double *sm = smem + static_cast<size_t>(warp) * (GRAD ? 6u : 3u) * na;
    for (uint64_t c = static_cast<uint64_t>(blockIdx.x) * wpb + warp; c < n; c += static_cast<uint64_t>(gridDim.x) * wpb)
        lj_cluster_flat<GRAD>(x + c * nx, na, nx, sm, f ? f + c : nullptr, GRAD ? g + c * nx : nullptr);
}

template <bool GRAD>
__global__ void __launch_bounds__(128) lj_smem_kernel(const double *__restrict__ x, uint64_t n, uint32_t na,
                                                      uint32_t nx, double *__restrict__ f, double *__restrict__ g)
{
    extern __shared__ double smem[];
    const unsigned warp = threadIdx.x >> 5;
    const unsigned wpb = blockDim.x >> 5;
    double *sm = smem + static_cast<size_t>(warp) * (GRAD ? 6u : 3u) * na;
    for (uint64_t c = static_cast<uint64_t>(blockIdx.x) * wpb + warp; c < n; c += static_cast<uint64_t>(gridDim.x) * wpb)
        lj_cluster_smem<GRAD>(x + c * nx, na, nx, sm, f ? f + c : nullptr, GRAD ? g + c * nx : nullptr);
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

template <typename K>
int launch_simple(K kernel, int lanes, const double *x, uint64_t n, uint32_t nx, double *f, double *g,
                  cudaStream_t s, int num_sms)
{
    const int threads = row_block_threads(n, lanes, num_sms);
    int grid = 1;
    PGX_TRY(grid_for(kernel, threads, 0, n, threads / lanes, num_sms, &grid));
    kernel<<<grid, threads, 0, s>>>(x, n, nx, f, g);
    PGX_CUDA(cudaGetLastError());
    return PGX_OK;
}

template <int G>
int launch_rows(int kind, bool grad, const double *x, uint64_t n, uint32_t nx, double *f, double *g, cudaStream_t s,
                int num_sms)
{
    constexpr int pb = G; // lanes per row
    switch (kind) {
        case PGX_ROSENBROCK:
            return grad ? launch_simple(rosenbrock_kernel<G, true>, pb, x, n, nx, f, g, s, num_sms)
                        : launch_simple(rosenbrock_kernel<G, false>, pb, x, n, nx, f, g, s, num_sms);
        case PGX_ACKLEY:
            return launch_simple(row_f_kernel<G, PGX_ACKLEY>, pb, x, n, nx, f, nullptr, s, num_sms);
        case PGX_GRIEWANK:
            return launch_simple(row_f_kernel<G, PGX_GRIEWANK>, pb, x, n, nx, f, nullptr, s, num_sms);
        default:
            return launch_simple(row_f_kernel<G, PGX_SCHWEFEL>, pb, x, n, nx, f, nullptr, s, num_sms);
    }
}

template <int V, int G>
int launch_rastrigin_vg(bool grad, const double *x, uint64_t n, uint32_t nx, double *f, double *g, cudaStream_t s,
                        int num_sms)
{
    return grad ? launch_simple(rastrigin_kernel<V, G, true>, G, x, n, nx, f, g, s, num_sms)
                : launch_simple(rastrigin_kernel<V, G, false>, G, x, n, nx, f, g, s, num_sms);
}

// rastrigin rows of canonical width V (8, 16, 32) on G lanes (4 <= G <= V)
int launch_rastrigin(int V, int G, bool grad, const double *x, uint64_t n, uint32_t nx, double *f, double *g,
                     cudaStream_t s, int num_sms)
{
    switch (V * 64 + G) {
        case 8 * 64 + 4: return launch_rastrigin_vg<8, 4>(grad, x, n, nx, f, g, s, num_sms);
        case 8 * 64 + 8: return launch_rastrigin_vg<8, 8>(grad, x, n, nx, f, g, s, num_sms);
        case 16 * 64 + 4: return launch_rastrigin_vg<16, 4>(grad, x, n, nx, f, g, s, num_sms);
        case 16 * 64 + 8: return launch_rastrigin_vg<16, 8>(grad, x, n, nx, f, g, s, num_sms);
        case 16 * 64 + 16: return launch_rastrigin_vg<16, 16>(grad, x, n, nx, f, g, s, num_sms);
        case 32 * 64 + 4: return launch_rastrigin_vg<32, 4>(grad, x, n, nx, f, g, s, num_sms);
        case 32 * 64 + 8: return launch_rastrigin_vg<32, 8>(grad, x, n, nx, f, g, s, num_sms);
        case 32 * 64 + 16: return launch_rastrigin_vg<32, 16>(grad, x, n, nx, f, g, s, num_sms);
        case 32 * 64 + 32: return launch_rastrigin_vg<32, 32>(grad, x, n, nx, f, g, s, num_sms);
        default:
            set_error("rastrigin rows: " + std::to_string(G) + " lanes for width " + std::to_string(V));
            return PGX_ERR_INVALID;
    }
}

} // namespace

// Lanes per row for the strided row kernels: the widest group (coalesced
// loads, fewest sequential steps) that keeps at least 94% of its lanes busy;
// the FP64 pipe spends a full warp instruction on partly idle warps.
int lanes_per_row(uint32_t nx)
{
    for (uint32_t g = 32; g >= 2; g >>= 1) {
        const uint32_t steps = (nx + g - 1) / g;
        if (nx >= g && 100u * nx >= 94u * g * steps) return static_cast<int>(g);
    }
    return nx >= 2 ? 2 : 1;
}

// lennard_jones: the flattened pair walk when the register variant (lane l
// owns atoms l, l+32, ...) would leave more than 5% of its lanes idle.
bool lj_use_flat(uint32_t na)
{
    const uint32_t ma = (na + 31u) / 32u;
    return na >= 33u && 100u * na < 95u * 32u * ma;
}

namespace
{

template <typename K>
int launch_lj(K kernel, bool grad, const double *x, uint64_t n, uint32_t na, uint32_t nx, double *f, double *g,
              cudaStream_t s, int num_sms)
{
    const size_t per_warp = static_cast<size_t>(grad ? 6u : 3u) * na * sizeof(double);
    int wpb = static_cast<int>((96u * 1024u) / per_warp);
    if (wpb > 4) wpb = 4;
    if (wpb < 1) wpb = 1;
    const int threads = 32 * wpb;
    const size_t smem = per_warp * wpb;
    PGX_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem > 48u * 1024u ? smem : 48u * 1024u)));
    int grid = 1;
    PGX_TRY(grid_for(kernel, threads, smem, n, wpb, num_sms, &grid));
    kernel<<<grid, threads, smem, s>>>(x, n, na, nx, f, g);
    PGX_CUDA(cudaGetLastError());
    return PGX_OK;
}

template <int MA>
int launch_lj_reg(bool grad, const double *x, uint64_t n, uint32_t na, uint32_t nx, double *f, double *g,
                  cudaStream_t s, int num_sms)
{
    return grad ? launch_lj(lj_reg_kernel<MA, true>, true, x, n, na, nx, f, g, s, num_sms)
                : launch_lj(lj_reg_kernel<MA, false>, false, x, n, na, nx, f, g, s, num_sms);
}

} // namespace

// Rosenbrock rows are evaluated in FP64 arithmetic. PGX_ROSENBROCK_DOUBLE_FLOAT=1
// in the environment (read at every launch) opts in to the double-float rows
// (about 2x faster on GB300, error within 2e-14 of the FP64 error bound, not
// FP64 arithmetic).
bool rosenbrock_double_float()
{
    const char *v = std::getenv("PGX_ROSENBROCK_DOUBLE_FLOAT");
    return v != nullptr && v[0] == '1';
}

int launch_eval(int kind, uint64_t param, uint64_t nx, const double *d_x, uint64_t n, double *d_f, double *d_g,
                cudaStream_t stream, int num_sms, uint64_t *launches)
{
    if (n == 0) return PGX_OK;
    PGX_CHECK(nx < (1ull << 31), PGX_ERR_CAPACITY, "decision vector dimension exceeds 2^31-1");
    const bool grad = d_g != nullptr;
    const uint32_t nx32 = static_cast<uint32_t>(nx);
    int st = PGX_OK;
    if (kind == PGX_ROSENBROCK && nx >= 128 && nx % 4 == 0 && reinterpret_cast<uintptr_t>(d_x) % 16 == 0
        && (!grad || reinterpret_cast<uintptr_t>(d_g) % 16 == 0)) {
        if (!rosenbrock_double_float())
            st = grad ? launch_simple(rosenbrock_v4_kernel<true>, 32, d_x, n, nx32, d_f, d_g, stream, num_sms)
                      : launch_simple(rosenbrock_v4_kernel<false>, 32, d_x, n, nx32, d_f, d_g, stream, num_sms);
        else
            st = grad ? launch_simple(rosenbrock_v4ff_kernel<true>, 32, d_x, n, nx32, d_f, d_g, stream, num_sms)
                      : launch_simple(rosenbrock_v4ff_kernel<false>, 32, d_x, n, nx32, d_f, d_g, stream, num_sms);
    } else if (kind == PGX_RASTRIGIN || kind == PGX_ROSENBROCK || kind == PGX_ACKLEY || kind == PGX_GRIEWANK
               || kind == PGX_SCHWEFEL) {
        PGX_CHECK(!grad || kind <= PGX_ROSENBROCK, PGX_ERR_NOTIMPL,
                  "The gradient has been requested but it is not implemented in the UDP");
        if (kind == PGX_RASTRIGIN) {
            const int own = lanes_per_row(nx32);
            st = launch_rastrigin(dev::rastrigin_width(own), dev::rastrigin_lanes(own, n, num_sms), grad, d_x, n, nx32,
                                  d_f, d_g, stream, num_sms);
            if (st == PGX_OK && launches) ++*launches;
            return st;
        }
        switch (lanes_per_row(nx32)) {
            case 32: st = launch_rows<32>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms); break;
            case 16: st = launch_rows<16>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms); break;
            case 8: st = launch_rows<8>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms); break;
            case 4: st = launch_rows<4>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms); break;
            case 2: st = launch_rows<2>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms); break;
            default: st = launch_rows<1>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms); break;
        }
    } else if (kind == PGX_LENNARD_JONES) {
        const uint32_t na = static_cast<uint32_t>(param);
        const size_t per_warp = static_cast<size_t>(grad ? 6u : 3u) * na * sizeof(double);
        PGX_CHECK(per_warp <= 200u * 1024u, PGX_ERR_CAPACITY,
                  "lennard_jones: too many atoms for one cluster per warp");
        if (lj_use_flat(na)) {
            st = grad ? launch_lj(lj_flat_kernel<true>, true, d_x, n, na, nx32, d_f, d_g, stream, num_sms)
                      : launch_lj(lj_flat_kernel<false>, false, d_x, n, na, nx32, d_f, d_g, stream, num_sms);
            if (st == PGX_OK && launches) ++*launches;
            return st;
        }
        switch ((na + 31u) / 32u) {
            case 1: st = launch_lj_reg<1>(grad, d_x, n, na, nx32, d_f, d_g, stream, num_sms); break;
            case 2: st = launch_lj_reg<2>(grad, d_x, n, na, nx32, d_f, d_g, stream, num_sms); break;
            case 3: st = launch_lj_reg<3>(grad, d_x, n, na, nx32, d_f, d_g, stream, num_sms); break;
            case 4: st = launch_lj_reg<4>(grad, d_x, n, na, nx32, d_f, d_g, stream, num_sms); break;
            case 5: st = launch_lj_reg<5>(grad, d_x, n, na, nx32, d_f, d_g, stream, num_sms); break;
            case 6: st = launch_lj_reg<6>(grad, d_x, n, na, nx32, d_f, d_g, stream, num_sms); break;
            case 7: st = launch_lj_reg<7>(grad, d_x, n, na, nx32, d_f, d_g, stream, num_sms); break;
            case 8: st = launch_lj_reg<8>(grad, d_x, n, na, nx32, d_f, d_g, stream, num_sms); break;
            default:
                st = grad ? launch_lj(lj_smem_kernel<true>, true, d_x, n, na, nx32, d_f, d_g, stream, num_sms)
                          : launch_lj(lj_smem_kernel<false>, false, d_x, n, na, nx32, d_f, d_g, stream, num_sms);
        }
    } else {
        set_error("unknown problem kind " + std::to_string(kind));
        return PGX_ERR_INVALID;
    }
    if (st == PGX_OK && launches) ++*launches;
    return st;
}

// Same as launch_eval for rastrigin/rosenbrock with the variant forced:
// lanes = 1..32 strided rows with that many lanes per row, lanes = 0 the
// 4-wide rosenbrock rows. Used by the autotuner.
int launch_rows_variant(int kind, uint64_t nx, const double *d_x, uint64_t n, double *d_f, double *d_g, int lanes,
                        cudaStream_t stream, int num_sms)
{
    if (n == 0) return PGX_OK;
    const bool grad = d_g != nullptr;
    const uint32_t nx32 = static_cast<uint32_t>(nx);
    if (lanes == 0) {
        PGX_CHECK(kind == PGX_ROSENBROCK && nx % 4 == 0 && reinterpret_cast<uintptr_t>(d_x) % 16 == 0,
                  PGX_ERR_INVALID, "4-wide rows need rosenbrock, nx % 4 == 0 and aligned rows");
        return grad ? launch_simple(rosenbrock_v4_kernel<true>, 32, d_x, n, nx32, d_f, d_g, stream, num_sms)
                    : launch_simple(rosenbrock_v4_kernel<false>, 32, d_x, n, nx32, d_f, d_g, stream, num_sms);
    }
    if (kind == PGX_RASTRIGIN)
        return launch_rastrigin(dev::rastrigin_width(lanes_per_row(nx32)), lanes, grad, d_x, n, nx32, d_f, d_g, stream,
                                num_sms);
    switch (lanes) {
        case 32: return launch_rows<32>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms);
        case 16: return launch_rows<16>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms);
        case 8: return launch_rows<8>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms);
        case 4: return launch_rows<4>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms);
        case 2: return launch_rows<2>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms);
        default: return launch_rows<1>(kind, grad, d_x, n, nx32, d_f, d_g, stream, num_sms);
    }
}

namespace
{
__global__ void lj_reciprocal_kernel(const double *__restrict__ d, uint64_t n, double *__restrict__ inv,
                                     double *__restrict__ cube)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        double r, s;
        dev::lj_rcp_cube(d[i], r, s);
        inv[i] = r;
        cube[i] = s;
    }
}
} // namespace

// The Lennard-Jones pair loops' 1/d and 1/d^3 on host values (self-test).
int run_lj_reciprocal(pgx_context *ctx, const double *d, uint64_t n, double *inv, double *cube)
{
    if (n == 0) return PGX_OK;
    const size_t b = (n * sizeof(double) + 255u) & ~size_t(255);
    PGX_TRY(ctx->s_points.ensure(3u * b));
    double *dd = ctx->s_points.as<double>();
    double *dinv = reinterpret_cast<double *>(ctx->s_points.as<char>() + b);
    double *dcube = reinterpret_cast<double *>(ctx->s_points.as<char>() + 2u * b);
    cudaStream_t s = ctx->stream;
    PGX_CUDA(cudaMemcpyAsync(dd, d, n * sizeof(double), cudaMemcpyHostToDevice, s));
    const int grid = static_cast<int>(std::min<uint64_t>((n + 255u) / 256u, static_cast<uint64_t>(ctx->num_sms) * 8u));
    lj_reciprocal_kernel<<<grid, 256, 0, s>>>(dd, n, dinv, dcube);
    PGX_CUDA(cudaGetLastError());
    PGX_CUDA(cudaMemcpyAsync(inv, dinv, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (cube) PGX_CUDA(cudaMemcpyAsync(cube, dcube, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    PGX_CUDA(cudaStreamSynchronize(s));
    return PGX_OK;
}

} // namespace pgx

