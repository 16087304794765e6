// vppgpu_internal.cuh -- shared host/device definitions of the GB300 encoder
// hot path (context, status handling, launch accounting, small device helpers).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/vppgpu.h"

struct vppgpu_ctx {
    int device;
    int sm_count;
    cudaStream_t own_stream;
    cudaStream_t stream;  // own_stream or a caller-provided stream
    unsigned long long launches;
};

namespace vppgpu {

// Map a CUDA error to a status; keeps the first error message for debugging.
int cuda_status(cudaError_t e);

#define VPP_CUDA(call)                                 \
    do {                                               \
        cudaError_t _e = (call);                       \
        if (_e != cudaSuccess) return vppgpu::cuda_status(_e); \
    } while (0)

#define VPP_CHECK_LAUNCH(ctx)                                   \
    do {                                                        \
        cudaError_t _e = cudaGetLastError();                    \
        if (_e != cudaSuccess) return vppgpu::cuda_status(_e);  \
        (ctx)->launches++;                                      \
    } while (0)

// Bind the context's device on the calling thread.
int bind(vppgpu_ctx* ctx);

static inline unsigned int blocks_for(long long n, int threads)
{
    return (unsigned int)((n + threads - 1) / threads);
}

}  // namespace vppgpu

// ---- device helpers ------------------------------------------------------
__device__ __forceinline__ int clip255(int x) { return min(max(x, 0), 255); }
