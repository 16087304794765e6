// mc.cu -- MotionCompensatorH264ImplStd and the block add / subtract helpers
// on sm_103a.
//
// Reference: MotionCompensatorH264ImplStd::Compensate(pMotionList)
// (src/CodecUtils/MotionCompensatorH264ImplStd.cpp:323-473).  The reference
// copies the 4:2:0 reference frame into edge-extended temporaries and, block
// by block, overwrites the frame with the block each vector points at: luma
// 16x16 by OverlayMem2Dv2::QuarterRead at the quarter-pel vector, chroma 8x8
// by OverlayMem2Dv2::EighthRead at the same vector in eighth-pel units
// (bilinear, (z + 32) >> 6).  A zero vector leaves its block as it is.
//
// GB300 design: the frame is first copied to a stream-ordered temporary (the
// reference's temporaries; it makes compensation in place possible), then
// one thread per output sample computes its value from the temporary.  The
// edge extension is a clamp of the sample coordinates, which gives the
// extended border's values for every vector within the reference's range.
// Luma half-pel samples are computed on the fly (6-tap, and j from the
// unrounded vertical taps), the two samples of a quarter position averaged
// as QuarterRead does.  Only full macroblock rows are compensated (the
// reference reads vectors past the end of its list for a partial bottom
// row); rows below keep the reference samples.
//
// The add-with-clip and subtract helpers (Add16x16WithClip255 /
// Add8x8WithClip255, Sub16x16 / Sub8x8, OverlayMem2Dv2.cpp:1195-1426) are
// elementwise over whole planes, 8 samples per thread with 16-byte accesses.
#include <cstdint>
#include <new>

#include "me_common.cuh"

namespace {

struct Plane {
    const short* p;
    int w, h;
    __device__ __forceinline__ int at(int x, int y) const
    {
        x = x < 0 ? 0 : (x >= w ? w - 1 : x);
        y = y < 0 ? 0 : (y >= h ? h - 1 : y);
        return __ldg(p + (size_t)y * w + x);
    }
    __device__ __forceinline__ int tap_h(int x, int y) const  // unrounded horizontal 6-tap between x and x+1
    {
        return at(x - 2, y) - 5 * at(x - 1, y) + 20 * at(x, y) + 20 * at(x + 1, y) - 5 * at(x + 2, y) + at(x + 3, y);
    }
    __device__ __forceinline__ int tap_v(int x, int y) const
    {
        return at(x, y - 2) - 5 * at(x, y - 1) + 20 * at(x, y) + 20 * at(x, y + 1) - 5 * at(x, y + 2) + at(x, y + 3);
    }
    __device__ __forceinline__ int b(int x, int y) const { return clip255((tap_h(x, y) + 16) >> 5); }
    __device__ __forceinline__ int hh(int x, int y) const { return clip255((tap_v(x, y) + 16) >> 5); }
    __device__ __forceinline__ int j(int x, int y) const
    {
        const int s = tap_v(x - 2, y) - 5 * tap_v(x - 1, y) + 20 * tap_v(x, y) + 20 * tap_v(x + 1, y) -
                      5 * tap_v(x + 2, y) + tap_v(x + 3, y);
        return clip255((s + 512) >> 10);
    }
};

// One sample of QuarterRead at full-pel (x, y) with fraction (fx, fy) in 0..3
// (a negative offset already folded into (x, y)): the full-pel sample, one of
// the half-pel samples b, h, j, or the rounded mean of two of them.
__device__ int qpel_sample(const Plane& P, int x, int y, int fx, int fy)
{
    switch (fx | (fy << 2)) {
    case 0: return P.at(x, y);
    case 2: return P.b(x, y);
    case 8: return P.hh(x, y);
    case 10: return P.j(x, y);
    case 1: return (P.at(x, y) + P.b(x, y) + 1) >> 1;
    case 3: return (P.at(x + 1, y) + P.b(x, y) + 1) >> 1;
    case 4: return (P.at(x, y) + P.hh(x, y) + 1) >> 1;
    case 12: return (P.at(x, y + 1) + P.hh(x, y) + 1) >> 1;
    case 6: return (P.j(x, y) + P.b(x, y) + 1) >> 1;
    case 14: return (P.j(x, y) + P.b(x, y + 1) + 1) >> 1;
    case 9: return (P.j(x, y) + P.hh(x, y) + 1) >> 1;
    case 11: return (P.j(x, y) + P.hh(x + 1, y) + 1) >> 1;
    case 5: return (P.b(x, y) + P.hh(x, y) + 1) >> 1;
    case 7: return (P.b(x, y) + P.hh(x + 1, y) + 1) >> 1;
    case 13: return (P.hh(x, y) + P.b(x, y + 1) + 1) >> 1;
    default: return (P.hh(x + 1, y) + P.b(x, y + 1) + 1) >> 1;
    }
}

__global__ void __launch_bounds__(256) k_mc_luma(Plane ref, const int* __restrict__ mv, int cols, int rows,
                                                short* __restrict__ out)
{
    const long long n = (long long)ref.w * ref.h;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(i / ref.w), x = (int)(i - (long long)y * ref.w);
        int v = __ldg(ref.p + i);
        if (y < 16 * rows) {
            const int k = (y >> 4) * cols + (x >> 4);
            const int m = __ldg(mv + k), mvx = vppgpu::mv_x(m), mvy = vppgpu::mv_y(m);
            if (mvx | mvy) {
                // C quotient and remainder, a negative remainder folded as QuarterRead does
                const int qx = mvx % 4, qy = mvy % 4;
                const int ox = x + mvx / 4 + (qx < 0 ? -1 : 0), oy = y + mvy / 4 + (qy < 0 ? -1 : 0);
                v = qpel_sample(ref, ox, oy, qx < 0 ? qx + 4 : qx, qy < 0 ? qy + 4 : qy);
            }
        }
        out[i] = (short)v;
    }
}

// Both chroma planes: EighthRead at the vector in eighth-pel units.
__global__ void __launch_bounds__(256) k_mc_chroma(Plane u, Plane v, const int* __restrict__ mv, int cols, int rows,
                                                  short* __restrict__ out_u, short* __restrict__ out_v)
{
    const long long n = (long long)u.w * u.h;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 2 * n;
         i += (long long)gridDim.x * blockDim.x) {
        const bool second = i >= n;
        const long long o = second ? i - n : i;
        const Plane& P = second ? v : u;
        const int y = (int)(o / P.w), x = (int)(o - (long long)y * P.w);
        int s = __ldg(P.p + o);
        if (y < 8 * rows) {
            const int k = (y >> 3) * cols + (x >> 3);
            const int m = __ldg(mv + k), mvx = vppgpu::mv_x(m), mvy = vppgpu::mv_y(m);
            if (mvx | mvy) {
                const int ex = mvx % 8, ey = mvy % 8;
                const int cx = x + mvx / 8 + (ex < 0 ? -1 : 0), cy = y + mvy / 8 + (ey < 0 ? -1 : 0);
                const int fx = ex < 0 ? ex + 8 : ex, fy = ey < 0 ? ey + 8 : ey;
                if (fx | fy) {
                    const int z = (8 - fx) * (8 - fy) * P.at(cx, cy) + fx * (8 - fy) * P.at(cx + 1, cy) +
                                  (8 - fx) * fy * P.at(cx, cy + 1) + fx * fy * P.at(cx + 1, cy + 1);
                    s = (z + 32) >> 6;
                } else {
                    s = P.at(cx, cy);
                }
            }
        }
        (second ? out_v : out_u)[o] = (short)s;
    }
}

// a = clip255(a + b) or a -= b, 8 samples per thread (16-byte accesses), the tail one by one.
template <bool kAdd>
__global__ void __launch_bounds__(256) k_plane_op(short* __restrict__ a, const short* __restrict__ b, long long n)
{
    const long long n8 = n >> 3;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n8; i += stride) {
        uint4 va = reinterpret_cast<const uint4*>(a)[i];
        const uint4 vb = __ldg(reinterpret_cast<const uint4*>(b) + i);
        short* sa = reinterpret_cast<short*>(&va);
        const short* sb = reinterpret_cast<const short*>(&vb);
#pragma unroll
        for (int t = 0; t < 8; t++) {
            const int r = kAdd ? sa[t] + sb[t] : sa[t] - sb[t];
            sa[t] = (short)(kAdd ? (r < 0 ? 0 : (r > 255 ? 255 : r)) : r);
        }
        reinterpret_cast<uint4*>(a)[i] = va;
    }
    for (long long i = 8 * n8 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
        const int r = kAdd ? a[i] + b[i] : a[i] - b[i];
        a[i] = (short)(kAdd ? (r < 0 ? 0 : (r > 255 ? 255 : r)) : r);
    }
}

int grid_for(vppgpu_ctx* ctx, long long work)
{
    long long g = (work + 255) / 256;
    const long long cap = (long long)ctx->sm_count * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

struct vppgpu_mc {
    vppgpu_ctx* ctx;
    int W, H, range;
    short* d_tmp;  // the reference before compensation (Y, U, V)
    short* d_io;   // staging of the host entry point
    int* d_mv;
};

extern "C" {

int vppgpu_mc_create(vppgpu_ctx* ctx, int width, int height, int range, vppgpu_mc** out)
{
    if (!ctx || !out || width < 16 || height < 16 || (width % 16) || (height % 2) || range < 0)
        return VPPGPU_ERR_INVALID_ARG;
    *out = nullptr;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    vppgpu_mc* mc = new (std::nothrow) vppgpu_mc();
    if (!mc) return VPPGPU_ERR_OUT_OF_MEMORY;
    mc->ctx = ctx;
    mc->W = width;
    mc->H = height;
    mc->range = range;
    const size_t frame = (size_t)width * height * 3 / 2;
    const size_t nmb = (size_t)(width / 16) * (height / 16);
    if (cudaMalloc((void**)&mc->d_tmp, frame * sizeof(short)) != cudaSuccess ||
        cudaMalloc((void**)&mc->d_io, frame * sizeof(short)) != cudaSuccess ||
        cudaMalloc((void**)&mc->d_mv, (nmb ? nmb : 1) * sizeof(int)) != cudaSuccess) {
        cudaFree(mc->d_tmp);
        cudaFree(mc->d_io);
        delete mc;
        return VPPGPU_ERR_OUT_OF_MEMORY;
    }
    *out = mc;
    return VPPGPU_OK;
}

int vppgpu_mc_destroy(vppgpu_mc* mc)
{
    if (!mc) return VPPGPU_ERR_INVALID_ARG;
    cudaSetDevice(mc->ctx->device);
    cudaStreamSynchronize(mc->ctx->stream);
    cudaFree(mc->d_tmp);
    cudaFree(mc->d_io);
    cudaFree(mc->d_mv);
    delete mc;
    return VPPGPU_OK;
}

int vppgpu_mc_compensate_device(vppgpu_mc* mc, const short* d_ref_yuv, const short* d_mv, short* d_out_yuv)
{
    if (!mc || !d_ref_yuv || !d_mv || !d_out_yuv) return VPPGPU_ERR_INVALID_ARG;
    if (((uintptr_t)d_mv & 3) || ((uintptr_t)d_out_yuv & 1) || ((uintptr_t)d_ref_yuv & 1))
        return VPPGPU_ERR_INVALID_ARG;
    vppgpu_ctx* ctx = mc->ctx;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    const int W = mc->W, H = mc->H, cw = W / 2, ch = H / 2, cols = W / 16, rows = H / 16;
    const size_t ny = (size_t)W * H, nc = (size_t)cw * ch;
    VPP_CUDA(cudaMemcpyAsync(mc->d_tmp, d_ref_yuv, (ny + 2 * nc) * sizeof(short), cudaMemcpyDeviceToDevice,
                             ctx->stream));
    k_mc_luma<<<grid_for(ctx, (long long)ny), 256, 0, ctx->stream>>>(Plane{mc->d_tmp, W, H}, (const int*)d_mv, cols,
                                                                      rows, d_out_yuv);
    VPP_CHECK_LAUNCH(ctx);
    k_mc_chroma<<<grid_for(ctx, 2 * (long long)nc), 256, 0, ctx->stream>>>(
        Plane{mc->d_tmp + ny, cw, ch}, Plane{mc->d_tmp + ny + nc, cw, ch}, (const int*)d_mv, cols, rows,
        d_out_yuv + ny, d_out_yuv + ny + nc);
    VPP_CHECK_LAUNCH(ctx);
    ctx->launches += 2;
    return VPPGPU_OK;
}

int vppgpu_mc_compensate(vppgpu_mc* mc, short* yuv, const short* mv)
{
    if (!mc || !yuv || !mv) return VPPGPU_ERR_INVALID_ARG;
    vppgpu_ctx* ctx = mc->ctx;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    const size_t frame = (size_t)mc->W * mc->H * 3 / 2, nmb = (size_t)(mc->W / 16) * (mc->H / 16);
    VPP_CUDA(cudaMemcpyAsync(mc->d_io, yuv, frame * sizeof(short), cudaMemcpyHostToDevice, ctx->stream));
    VPP_CUDA(cudaMemcpyAsync(mc->d_mv, mv, nmb * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    if ((rc = vppgpu_mc_compensate_device(mc, mc->d_io, (const short*)mc->d_mv, mc->d_io))) return rc;
    VPP_CUDA(cudaMemcpyAsync(yuv, mc->d_io, frame * sizeof(short), cudaMemcpyDeviceToHost, ctx->stream));
    VPP_CUDA(cudaStreamSynchronize(ctx->stream));
    return VPPGPU_OK;
}

static int plane_op(vppgpu_ctx* ctx, short* d_a, const short* d_b, long long n, bool add)
{
    if (!ctx || !d_a || !d_b || n < 0 || ((uintptr_t)d_a & 15) || ((uintptr_t)d_b & 15)) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    if (n == 0) return VPPGPU_OK;
    const int g = grid_for(ctx, (n + 7) / 8);
    if (add)
        k_plane_op<true><<<g, 256, 0, ctx->stream>>>(d_a, d_b, n);
    else
        k_plane_op<false><<<g, 256, 0, ctx->stream>>>(d_a, d_b, n);
    VPP_CHECK_LAUNCH(ctx);
    ctx->launches++;
    return VPPGPU_OK;
}

int vppgpu_add_clip255_device(vppgpu_ctx* ctx, short* d_a, const short* d_b, long long n)
{
    return plane_op(ctx, d_a, d_b, n, true);
}

int vppgpu_sub_device(vppgpu_ctx* ctx, short* d_a, const short* d_b, long long n)
{
    return plane_op(ctx, d_a, d_b, n, false);
}

}  // extern "C"
