// calibrate.cu -- measured integer-ALU peak used as the roofline of the
// motion-search kernel: the dp4a (4 byte products + accumulate) issue rate of
// the whole GPU, timed with CUDA events on the context stream.
#include "vppgpu_internal.cuh"

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_dp4a_peak(unsigned seed, int iters, unsigned* sink)
{
    unsigned a = seed ^ threadIdx.x, b = seed * 2654435761u + blockIdx.x;
    unsigned acc[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) acc[c] = c + threadIdx.x;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) acc[c] = __dp4a(a + c, b, acc[c]);
#pragma unroll
        for (int c = 0; c < kChains; c++) acc[c] = __dp4a(b, a - c, acc[c]);
    }
    unsigned r = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) r ^= acc[c];
    if (r == 0x12345678u) sink[0] = r;  // keep the work observable
}

}  // namespace

extern "C" {

// Not part of the vpp interface: measures the dp4a rate (instructions per
// second over the whole device) against which the full-search table kernel is reported.
int vppgpu_calibrate_dp4a(vppgpu_ctx* ctx, double* dp4a_per_second)
{
    if (!ctx || !dp4a_per_second) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    unsigned* sink = nullptr;
    VPP_CUDA(cudaMallocAsync((void**)&sink, sizeof(unsigned), ctx->stream));
    cudaEvent_t e0, e1;
    VPP_CUDA(cudaEventCreate(&e0));
    VPP_CUDA(cudaEventCreate(&e1));
    const int blocks = ctx->sm_count * 8, threads = 256, iters = 4096;
    k_dp4a_peak<<<blocks, threads, 0, ctx->stream>>>(1u, 64, sink);  // warm-up
    cudaEventRecord(e0, ctx->stream);
    k_dp4a_peak<<<blocks, threads, 0, ctx->stream>>>(2u, iters, sink);
    cudaEventRecord(e1, ctx->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(sink, ctx->stream);
    if (e != cudaSuccess) return vppgpu::cuda_status(e);
    ctx->launches += 2;
    double n = (double)blocks * threads * iters * 2.0 * kChains;
    *dp4a_per_second = n / (ms * 1e-3);
    return VPPGPU_OK;
}

}  // extern "C"
