// FP64 pipe throughput probe: the denominator of the FP64 roofline of the
// fitness kernels (the measured peaks cover HBM and bf16 only).
// Eight independent DFMA chains per thread keep the pipe busy; every SM runs
// several resident blocks.
#include "pgx_internal.cuh"

namespace pgx
{
namespace
{

__global__ void __launch_bounds__(256) dfma_probe_kernel(double *out, int iters, double a, double b)
{
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    if (s == 12345.678) out[blockIdx.x] = s; // never true; keeps the chains live
}

} // namespace
} // namespace pgx

using namespace pgx;

extern "C" int pgx_measure_fp64_peak(pgx_context *ctx, double *gflops)
{
    PGX_CHECK(ctx != nullptr && gflops != nullptr, PGX_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> g(ctx->lock);
    PGX_TRY(use_device(ctx));
    const int blocks = ctx->num_sms * 8, threads = 256, iters = 8192;
    PGX_TRY(ctx->d_out.ensure(static_cast<size_t>(blocks) * sizeof(double)));
    cudaEvent_t e0, e1;
    PGX_CUDA(cudaEventCreate(&e0));
    PGX_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 6; ++rep) {
        PGX_CUDA(cudaEventRecord(e0, ctx->stream));
        dfma_probe_kernel<<<blocks, threads, 0, ctx->stream>>>(ctx->d_out.as<double>(), iters, 0.9999999, 1e-7);
        PGX_CUDA(cudaGetLastError());
        PGX_CUDA(cudaEventRecord(e1, ctx->stream));
        PGX_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        PGX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->launches += 6;
    const double flops = 2.0 * 8.0 * iters * static_cast<double>(blocks) * threads;
    *gflops = flops / (best * 1e-3) / 1e9;
    return PGX_OK;
}
