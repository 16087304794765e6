// colour.cu -- packed BGR24 -> planar YUV 4:2:0 (short planes) for sm_103a.
//
//   fixed point: FastFixedPointRGB24toYUV420Converter::Convert
//                (src/ImageUtils/FastFixedPointRGB24toYUV420Converter.cpp:94-169)
//   real:        RealRGB24toYUV420Converter::{NonFlip,Flip}Convert
//                (src/ImageUtils/RealRGB24toYUV420Converter.cpp:83-242)
//   real impl2:  RealRGB24toYUV420ConverterImpl2 (…ConverterImpl2.cpp:104-262)
//
// HBM-bound: 3 B in and 3 B out (Y + quarter-size U, V as int16) per pixel.
// The fixed-point kernel gives each thread four horizontally adjacent 2x2
// pixel blocks, so a row of its input is three aligned 8-byte loads and its
// luma output one 16-byte store.  The double kernels round after every
// operation (__dmul_rn/__dadd_rn) exactly like the reference's
// left-to-right evaluation with no FMA contraction.
#include "vppgpu_internal.cuh"

namespace {

// (int)(0.5 + c * 8192) as the reference's static_cast does (…FixedPoint….cpp:65-74).
struct FixedCoefs {
    int c[9];
};

FixedCoefs make_fixed()
{
    const double k[9] = {0.299, 0.587, 0.114, -0.147, -0.289, 0.436, 0.615, -0.515, -0.100};
    FixedCoefs f;
    for (int i = 0; i < 9; i++) f.c[i] = (int)(0.5 + k[i] * (double)(2 << 12));
    return f;
}

__device__ __forceinline__ int clamp_s8(int x) { return min(max(x, -128), 127); }

__device__ __forceinline__ void fixed_pixel(const FixedCoefs& k, int b, int g, int r, int& y, int& u, int& v)
{
    y = clip255((k.c[0] * r + k.c[1] * g + k.c[2] * b) >> 13);
    u += k.c[3] * r + k.c[4] * g + k.c[5] * b;
    v += k.c[6] * r + k.c[7] * g + k.c[8] * b;
}

__device__ __forceinline__ int fixed_chroma(int acc, int chr_off)
{
    int t = acc >> 13;
    t += t < 0 ? -2 : 2;
    return chr_off + clamp_s8(t >> 2);
}

__device__ __forceinline__ unsigned pack2(int a, int b) { return (unsigned)(a & 0xffff) | ((unsigned)b << 16); }

// Four 2x2 blocks per thread (8 pixels of two rows); width % 8 == 0.
__global__ void __launch_bounds__(256) k_rgb_fixed_x8(const unsigned char* __restrict__ bgr, int w, int h,
                                                     int chr_off, FixedCoefs k, short* __restrict__ py,
                                                     short* __restrict__ pu, short* __restrict__ pv)
{
    size_t fpix = (size_t)w * h;
    const unsigned char* src = bgr + blockIdx.y * fpix * 3;
    short* Y = py + blockIdx.y * fpix;
    short* U = pu + blockIdx.y * (fpix / 4);
    short* V = pv + blockIdx.y * (fpix / 4);
    int groups_x = w >> 3, rows2 = h >> 1;
    long long ngroups = (long long)groups_x * rows2;
    for (long long gi = blockIdx.x * (long long)blockDim.x + threadIdx.x; gi < ngroups;
         gi += (long long)gridDim.x * blockDim.x) {
        int yb = (int)(gi / groups_x), gx = (int)(gi - (long long)yb * groups_x);
        int x0 = gx * 8, y0 = 2 * yb;
        unsigned char px[2][24];
#pragma unroll
        for (int rr = 0; rr < 2; rr++) {
            const uint2* s = reinterpret_cast<const uint2*>(src + ((size_t)(y0 + rr) * w + x0) * 3);
            uint2 a = s[0], b = s[1], c = s[2];
            unsigned wds[6] = {a.x, a.y, b.x, b.y, c.x, c.y};
#pragma unroll
            for (int i = 0; i < 24; i++) px[rr][i] = (unsigned char)(wds[i >> 2] >> (8 * (i & 3)));
        }
        int yv[2][8], uo[4], vo[4];
#pragma unroll
        for (int blk = 0; blk < 4; blk++) {
            int u = 0, v = 0;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                int rr = q >> 1, cc = 2 * blk + (q & 1);
                fixed_pixel(k, px[rr][3 * cc], px[rr][3 * cc + 1], px[rr][3 * cc + 2], yv[rr][cc], u, v);
            }
            uo[blk] = fixed_chroma(u, chr_off);
            vo[blk] = fixed_chroma(v, chr_off);
        }
#pragma unroll
        for (int rr = 0; rr < 2; rr++) {
            uint4 o;
            o.x = pack2(yv[rr][0], yv[rr][1]);
            o.y = pack2(yv[rr][2], yv[rr][3]);
            o.z = pack2(yv[rr][4], yv[rr][5]);
            o.w = pack2(yv[rr][6], yv[rr][7]);
            *reinterpret_cast<uint4*>(Y + (size_t)(y0 + rr) * w + x0) = o;
        }
        size_t co = (size_t)yb * (w >> 1) + (x0 >> 1);
        *reinterpret_cast<uint2*>(U + co) = make_uint2(pack2(uo[0], uo[1]), pack2(uo[2], uo[3]));
        *reinterpret_cast<uint2*>(V + co) = make_uint2(pack2(vo[0], vo[1]), pack2(vo[2], vo[3]));
    }
}

// Generic fixed-point path: one 2x2 block per thread (any even width).
__global__ void __launch_bounds__(256) k_rgb_fixed(const unsigned char* __restrict__ bgr, int w, int h,
                                                  int chr_off, FixedCoefs k, short* __restrict__ py,
                                                  short* __restrict__ pu, short* __restrict__ pv)
{
    size_t fpix = (size_t)w * h;
    const unsigned char* src = bgr + blockIdx.y * fpix * 3;
    short* Y = py + blockIdx.y * fpix;
    short* U = pu + blockIdx.y * (fpix / 4);
    short* V = pv + blockIdx.y * (fpix / 4);
    int xb_n = w >> 1, yb_n = h >> 1;
    long long n = (long long)xb_n * yb_n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int yb = (int)(i / xb_n), xb = (int)(i - (long long)yb * xb_n);
        int u = 0, v = 0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int yy = 2 * yb + (q >> 1), xx = 2 * xb + (q & 1);
            const unsigned char* t = src + ((size_t)yy * w + xx) * 3;
            int yv;
            fixed_pixel(k, t[0], t[1], t[2], yv, u, v);
            Y[(size_t)yy * w + xx] = (short)yv;
        }
        U[(size_t)yb * xb_n + xb] = (short)fixed_chroma(u, chr_off);
        V[(size_t)yb * xb_n + xb] = (short)fixed_chroma(v, chr_off);
    }
}

// Real converters: IEEE double, one rounding per operation, left to right.
__device__ __forceinline__ double lin3(double k0, double k1, double k2, double r, double g, double b)
{
    return __dadd_rn(__dadd_rn(__dmul_rn(k0, r), __dmul_rn(k1, g)), __dmul_rn(k2, b));
}

__global__ void __launch_bounds__(256) k_rgb_real(const unsigned char* __restrict__ bgr, int w, int h, int chr_off,
                                                 int flip, int impl2, short* __restrict__ py,
                                                 short* __restrict__ pu, short* __restrict__ pv)
{
    const double K00 = 0.299, K01 = 0.587, K02 = 0.114;
    const double K10 = -0.147, K11 = -0.289, K12 = 0.436;
    const double K20 = 0.615, K21 = -0.515, K22 = -0.100;
    size_t fpix = (size_t)w * h;
    const unsigned char* src = bgr + blockIdx.y * fpix * 3;
    short* Y = py + blockIdx.y * fpix;
    short* U = pu + blockIdx.y * (fpix / 4);
    short* V = pv + blockIdx.y * (fpix / 4);
    int xb_n = w >> 1, yb_n = h >> 1;
    long long n = (long long)xb_n * yb_n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int yb = (int)(i / xb_n), xb = (int)(i - (long long)yb * xb_n);
        double u = 0.0, v = 0.0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int yy = 2 * yb + (q >> 1), xx = 2 * xb + (q & 1);
            int sy = flip ? (h - 1 - yy) : yy;
            const unsigned char* t = src + ((size_t)sy * w + xx) * 3;
            double b = (double)t[0], g = (double)t[1], r = (double)t[2];
            double yl = __dadd_rn(__dadd_rn(__dadd_rn(0.5, __dmul_rn(K00, r)), __dmul_rn(K01, g)), __dmul_rn(K02, b));
            Y[(size_t)yy * w + xx] = (short)clip255(__double2int_rz(yl));
            double uu = lin3(K10, K11, K12, r, g, b);
            double vv = lin3(K20, K21, K22, r, g, b);
            if (q == 0) {
                u = uu;
                v = vv;
            } else {
                u = __dadd_rn(u, uu);
                v = __dadd_rn(v, vv);
            }
        }
        int iu, iv;
        if (!impl2) {
            iu = __double2int_rz(u);
            iv = __double2int_rz(v);
            iu += iu < 0 ? -2 : 2;
            iv += iv < 0 ? -2 : 2;
            iu /= 4;
            iv /= 4;
        } else {
            double au = __ddiv_rn(u, 4.0), av = __ddiv_rn(v, 4.0);
            au = u < 0.0 ? __dsub_rn(au, 0.5) : __dadd_rn(au, 0.5);
            av = v < 0.0 ? __dsub_rn(av, 0.5) : __dadd_rn(av, 0.5);
            iu = __double2int_rz(au);
            iv = __double2int_rz(av);
        }
        U[(size_t)yb * xb_n + xb] = (short)(chr_off + clamp_s8(iu));
        V[(size_t)yb * xb_n + xb] = (short)(chr_off + clamp_s8(iv));
    }
}

int launch(vppgpu_ctx* ctx, int kind, const unsigned char* bgr, int nframes, int w, int h, int chr_off,
           int flip, short* y, short* u, short* v)
{
    long long per = (long long)(w >> 1) * (h >> 1);
    if (kind == VPPGPU_RGB_FIXED_POINT && (w & 7) == 0) {
        long long groups = per / 4;
        int gx = (int)((groups + 255) / 256);
        if (gx > 4096) gx = 4096;
        k_rgb_fixed_x8<<<dim3(gx, nframes), 256, 0, ctx->stream>>>(bgr, w, h, chr_off, make_fixed(), y, u, v);
    } else if (kind == VPPGPU_RGB_FIXED_POINT) {
        int gx = (int)((per + 255) / 256);
        if (gx > 4096) gx = 4096;
        k_rgb_fixed<<<dim3(gx, nframes), 256, 0, ctx->stream>>>(bgr, w, h, chr_off, make_fixed(), y, u, v);
    } else {
        int gx = (int)((per + 255) / 256);
        if (gx > 4096) gx = 4096;
        k_rgb_real<<<dim3(gx, nframes), 256, 0, ctx->stream>>>(bgr, w, h, chr_off, flip != 0,
                                                               kind == VPPGPU_RGB_REAL_IMPL2, y, u, v);
    }
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

int check(vppgpu_ctx* ctx, int kind, const void* bgr, int w, int h, const void* y, const void* u, const void* v)
{
    if (!ctx || !bgr || !y || !u || !v || w < 2 || h < 2 || (w & 1) || (h & 1)) return VPPGPU_ERR_INVALID_ARG;
    if (kind < VPPGPU_RGB_FIXED_POINT || kind > VPPGPU_RGB_REAL_IMPL2) return VPPGPU_ERR_INVALID_ARG;
    return VPPGPU_OK;
}

}  // namespace

extern "C" {

int vppgpu_rgb24_to_yuv420_device(vppgpu_ctx* ctx, int kind, const unsigned char* d_bgr, int w, int h,
                                  int chr_off, int flip, short* d_y, short* d_u, short* d_v)
{
    int rc = check(ctx, kind, d_bgr, w, h, d_y, d_u, d_v);
    if (rc) return rc;
    if ((rc = vppgpu::bind(ctx))) return rc;
    return launch(ctx, kind, d_bgr, 1, w, h, chr_off, flip, d_y, d_u, d_v);
}

int vppgpu_rgb24_to_yuv420_frames_device(vppgpu_ctx* ctx, int kind, const unsigned char* d_bgr, int nframes,
                                         int w, int h, int chr_off, int flip, short* d_y, short* d_u,
                                         short* d_v)
{
    int rc = check(ctx, kind, d_bgr, w, h, d_y, d_u, d_v);
    if (rc) return rc;
    if (nframes < 1 || nframes > 65535) return VPPGPU_ERR_INVALID_ARG;
    if ((rc = vppgpu::bind(ctx))) return rc;
    return launch(ctx, kind, d_bgr, nframes, w, h, chr_off, flip, d_y, d_u, d_v);
}

int vppgpu_rgb24_to_yuv420(vppgpu_ctx* ctx, int kind, const unsigned char* bgr, int w, int h, int chr_off,
                           int flip, short* y, short* u, short* v)
{
    int rc = check(ctx, kind, bgr, w, h, y, u, v);
    if (rc) return rc;
    if ((rc = vppgpu::bind(ctx))) return rc;
    size_t nin = (size_t)w * h * 3, ny = (size_t)w * h * 2, nc = (size_t)(w / 2) * (h / 2) * 2;
    unsigned char* d = nullptr;
    // 16-byte aligned sub-buffers
    size_t o_y = (nin + 255) & ~(size_t)255, o_u = o_y + ((ny + 255) & ~(size_t)255),
           o_v = o_u + ((nc + 255) & ~(size_t)255), tot = o_v + nc;
    VPP_CUDA(cudaMallocAsync((void**)&d, tot, ctx->stream));
    cudaError_t e = cudaMemcpyAsync(d, bgr, nin, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        rc = launch(ctx, kind, d, 1, w, h, chr_off, flip, (short*)(d + o_y), (short*)(d + o_u), (short*)(d + o_v));
        if (rc == VPPGPU_OK) e = cudaMemcpyAsync(y, d + o_y, ny, cudaMemcpyDeviceToHost, ctx->stream);
        if (rc == VPPGPU_OK && e == cudaSuccess) e = cudaMemcpyAsync(u, d + o_u, nc, cudaMemcpyDeviceToHost, ctx->stream);
        if (rc == VPPGPU_OK && e == cudaSuccess) e = cudaMemcpyAsync(v, d + o_v, nc, cudaMemcpyDeviceToHost, ctx->stream);
    }
    cudaFreeAsync(d, ctx->stream);
    cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
    if (rc) return rc;
    if (e != cudaSuccess) return vppgpu::cuda_status(e);
    if (e2 != cudaSuccess) return vppgpu::cuda_status(e2);
    return VPPGPU_OK;
}

}  // extern "C"
