// context.cu -- device/stream binding, status strings and launch accounting
// for the vppgpu C ABI.
#include <stdlib.h>

#include "vppgpu_internal.cuh"

namespace vppgpu {

int cuda_status(cudaError_t e)
{
    if (e == cudaErrorMemoryAllocation) return VPPGPU_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice || e == cudaErrorNoKernelImageForDevice ||
        e == cudaErrorInsufficientDriver)
        return VPPGPU_ERR_NO_DEVICE;
    return VPPGPU_ERR_CUDA;
}

int bind(vppgpu_ctx* ctx)
{
    if (!ctx) return VPPGPU_ERR_INVALID_ARG;
    VPP_CUDA(cudaSetDevice(ctx->device));
    return VPPGPU_OK;
}

}  // namespace vppgpu

extern "C" {

const char* vppgpu_status_string(int s)
{
    switch (s) {
    case VPPGPU_OK: return "ok";
    case VPPGPU_ERR_INVALID_ARG: return "invalid argument";
    case VPPGPU_ERR_CUDA: return "CUDA runtime error";
    case VPPGPU_ERR_OUT_OF_MEMORY: return "out of memory";
    case VPPGPU_ERR_PIXEL_RANGE: return "luma sample outside 0..255";
    case VPPGPU_ERR_TIMEOUT: return "device-side wait gave up";
    case VPPGPU_ERR_UNSUPPORTED: return "unsupported configuration";
    case VPPGPU_ERR_NOT_READY: return "handle not ready";
    case VPPGPU_ERR_NO_DEVICE: return "no usable CUDA device";
    default: return "unknown status";
    }
}

int vppgpu_ctx_create(int device, vppgpu_ctx** out)
{
    if (!out) return VPPGPU_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev <= 0) return VPPGPU_ERR_NO_DEVICE;
    if (device < 0 || device >= ndev) return VPPGPU_ERR_INVALID_ARG;
    VPP_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    VPP_CUDA(cudaGetDeviceProperties(&prop, device));
    // The kernels are built for sm_103a only.
    if (prop.major != 10 || prop.minor != 3) return VPPGPU_ERR_NO_DEVICE;
    vppgpu_ctx* c = (vppgpu_ctx*)calloc(1, sizeof(vppgpu_ctx));
    if (!c) return VPPGPU_ERR_OUT_OF_MEMORY;
    c->device = device;
    c->sm_count = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        free(c);
        return VPPGPU_ERR_CUDA;
    }
    c->stream = c->own_stream;
    *out = c;
    return VPPGPU_OK;
}

int vppgpu_ctx_destroy(vppgpu_ctx* ctx)
{
    if (!ctx) return VPPGPU_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->own_stream);
    free(ctx);
    return VPPGPU_OK;
}

int vppgpu_ctx_set_stream(vppgpu_ctx* ctx, void* s)
{
    if (!ctx) return VPPGPU_ERR_INVALID_ARG;
    ctx->stream = s ? (cudaStream_t)s : ctx->own_stream;
    return VPPGPU_OK;
}

int vppgpu_ctx_get_stream(vppgpu_ctx* ctx, void** s)
{
    if (!ctx || !s) return VPPGPU_ERR_INVALID_ARG;
    *s = (void*)ctx->stream;
    return VPPGPU_OK;
}

int vppgpu_ctx_synchronize(vppgpu_ctx* ctx)
{
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    VPP_CUDA(cudaStreamSynchronize(ctx->stream));
    return VPPGPU_OK;
}

int vppgpu_ctx_launch_count(vppgpu_ctx* ctx, unsigned long long* count)
{
    if (!ctx || !count) return VPPGPU_ERR_INVALID_ARG;
    *count = ctx->launches;
    return VPPGPU_OK;
}

}  // extern "C"
