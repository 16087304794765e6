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
// GB300 design: for compensation in place the frame is first copied to a
// stream-ordered temporary (the reference's temporaries), else read as it is;
// the output is computed from it in one launch, one warp per macroblock
// (luma window and the half-pel lattices its fraction reads in shared
// memory, then both chroma blocks).  The edge extension is a clamp of the sample coordinates,
// which gives the extended border's values for every vector within the
// reference's range.  Only full macroblock rows are compensated (the
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
};

constexpr int kMcWarps = 4;  // macroblocks per CTA, one warp each

struct McLattice {
    short win[22][24];     // luma window, 2 samples of margin on each side of the 17x17 the block reads
    int th[22][16];        // unrounded horizontal 6-tap between window columns x+2 and x+3 (j cases only)
    short cwin[2][9][10];  // the 9x9 chroma windows (U, V)
};

// the six-tap (1, -5, 20, 20, -5, 1) over samples s apart
template <int kS, typename T>
__device__ __forceinline__ int tap6(const T* p)
{
    return p[0] - 5 * p[kS] + 20 * p[2 * kS] + 20 * p[3 * kS] - 5 * p[4 * kS] + p[5 * kS];
}

// QuarterRead per quarter case cs = fx | fy << 2: one sample, or the
// rounded average of two, from G (full-pel), b (horizontal half: 6-tap over a
// window row), h (vertical half: 6-tap down a window column) and j (centre:
// 6-tap down th).  Each entry: kind and offset of the first and the second
// term (kind 4: none), offsets in window samples from the output sample's
// row base &win[Y][X] (G(dx, dy) at (dy + 2) * 24 + dx + 2, b(dy) at
// (dy + 2) * 24, h(dx) at dx + 2).
enum : int { kTermG = 0, kTermB = 1, kTermH = 2, kTermJ = 3, kTermNone = 4 };
__constant__ int4 c_quarter_terms[16] = {
    {kTermG, 50, kTermNone, 0},  // 0: G
    {kTermG, 50, kTermB, 48},    // 1: (G + b) / 2
    {kTermB, 48, kTermNone, 0},  // 2: b
    {kTermG, 51, kTermB, 48},    // 3: (G(x+1) + b) / 2
    {kTermG, 50, kTermH, 2},     // 4: (G + h) / 2
    {kTermB, 48, kTermH, 2},     // 5: (b + h) / 2
    {kTermJ, 0, kTermB, 48},     // 6: (j + b) / 2
    {kTermB, 48, kTermH, 3},     // 7: (b + h(x+1)) / 2
    {kTermH, 2, kTermNone, 0},   // 8: h
    {kTermJ, 0, kTermH, 2},      // 9: (j + h) / 2
    {kTermJ, 0, kTermNone, 0},   // 10: j
    {kTermJ, 0, kTermH, 3},      // 11: (j + h(x+1)) / 2
    {kTermG, 74, kTermH, 2},     // 12: (G(y+1) + h) / 2
    {kTermH, 2, kTermB, 72},     // 13: (h + b(y+1)) / 2
    {kTermJ, 0, kTermB, 72},     // 14: (j + b(y+1)) / 2
    {kTermH, 3, kTermB, 72},     // 15: (h(x+1) + b(y+1)) / 2
};

// The 256 luma samples of quarter case cs, lane (X = lane & 15,
// Y = lane >> 4 + 2t): one compact loop per term kind (the kind is
// warp-uniform), every shared access a constant offset from the lane's base.
__device__ __forceinline__ void mc_luma_quarter(const McLattice& L, int cs, int lane, short* __restrict__ dst,
                                                int stride)
{
    const int X = lane & 15, Y0 = lane >> 4;
    const int4 tm = c_quarter_terms[cs];
    const int nterm = tm.z == kTermNone ? 1 : 2;
    int acc[8];
#pragma unroll
    for (int t = 0; t < 8; t++) acc[t] = 0;
#pragma unroll 1
    for (int e = 0; e < nterm; e++) {
        const int kind = e ? tm.z : tm.x;
        if (kind == kTermJ) {
            const int* tb = &L.th[Y0][X];
#pragma unroll
            for (int t = 0; t < 8; t++) acc[t] += clip255((tap6<16>(tb + 32 * t) + 512) >> 10);
            continue;
        }
        const short* w = &L.win[Y0][X] + (e ? tm.w : tm.y);
        if (kind == kTermG) {
#pragma unroll
            for (int t = 0; t < 8; t++) acc[t] += w[48 * t];
        } else if (kind == kTermB) {
#pragma unroll
            for (int t = 0; t < 8; t++) acc[t] += clip255((tap6<1>(w + 48 * t) + 16) >> 5);
        } else {
#pragma unroll
            for (int t = 0; t < 8; t++) acc[t] += clip255((tap6<24>(w + 48 * t) + 16) >> 5);
        }
    }
#pragma unroll
    for (int t = 0; t < 8; t++)
        dst[(size_t)(Y0 + 2 * t) * stride + X] = (short)(nterm == 1 ? acc[t] : (acc[t] + 1) >> 1);
}

// EighthRead of the two 8x8 chroma blocks at the vector in eighth-pel units,
// from 9x9 windows staged one column per lane (U lanes 0-8, V lanes 16-24).
__device__ __forceinline__ void mc_chroma_blocks(McLattice& L, const Plane& U, const Plane& V, int mvx, int mvy,
                                                 int bx, int by, int lane, short* __restrict__ ou,
                                                 short* __restrict__ ov)
{
    const int ex = mvx % 8, ey = mvy % 8;
    const int dx = mvx / 8 + (ex < 0 ? -1 : 0), dy = mvy / 8 + (ey < 0 ? -1 : 0);
    const int fx = ex < 0 ? ex + 8 : ex, fy = ey < 0 ? ey + 8 : ey;
    const int pl = lane >> 4, c = lane & 15;
    if (c < 9) {
        const Plane& P = pl ? V : U;
        int x = bx + dx + c;
        x = x < 0 ? 0 : (x >= P.w ? P.w - 1 : x);
        int q[9];
#pragma unroll
        for (int r = 0; r < 9; r++) {
            int y = by + dy + r;
            y = y < 0 ? 0 : (y >= P.h ? P.h - 1 : y);
            q[r] = __ldg(P.p + (size_t)y * P.w + x);
        }
#pragma unroll
        for (int r = 0; r < 9; r++) L.cwin[pl][r][c] = (short)q[r];
    }
    __syncwarp();
    const int w00 = (8 - fx) * (8 - fy), w10 = fx * (8 - fy), w01 = (8 - fx) * fy, w11 = fx * fy;
    const int x = lane & 7, y0 = lane >> 3;
#pragma unroll
    for (int t = 0; t < 4; t++) {  // t: U rows 0-3, U rows 4-7, V rows 0-3, V rows 4-7
        const int y = y0 + 4 * (t & 1);
        const short* p = &L.cwin[t >> 1][y][x];
        const int s = (w00 * p[0] + w10 * p[1] + w01 * p[10] + w11 * p[11] + 32) >> 6;
        (t < 2 ? ou : ov)[(size_t)(by + y) * U.w + bx + x] = (short)s;
    }
}

// One warp per macroblock: its 16x16 luma block and its two 8x8 chroma
// blocks.  Luma stages the 22x22 reference window around the vector's
// full-pel position (one column per lane, rows clamped only at the frame
// edge), the j cases also the horizontal 6-taps, then computes the quarter
// samples of its case from the term table.  Warp-synchronous: no block barrier.
__global__ void __launch_bounds__(32 * kMcWarps, 12) k_mc_frame(Plane ry, Plane ru, Plane rv,
                                                               const int* __restrict__ mv, int cols, int nmb,
                                                               short* __restrict__ oy, short* __restrict__ ou,
                                                               short* __restrict__ ov)
{
    __shared__ McLattice lat_s[kMcWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int k = blockIdx.x * kMcWarps + w;
    if (k >= nmb) return;  // whole warps only
    McLattice& L = lat_s[w];
    const int n = (k % cols) * 16, m = (k / cols) * 16;
    const int v = __ldg(mv + k), mvx = vppgpu::mv_x(v), mvy = vppgpu::mv_y(v);
    mc_chroma_blocks(L, ru, rv, mvx, mvy, n >> 1, m >> 1, lane, ou, ov);
    short* dst = oy + (size_t)m * ry.w + n;
    if (!(mvx | mvy)) {  // a zero vector keeps the block
        const short* src = ry.p + (size_t)m * ry.w + n;
        int q[8];
#pragma unroll
        for (int t = 0; t < 8; t++) q[t] = __ldg(src + (size_t)(2 * t + (lane >> 4)) * ry.w + (lane & 15));
#pragma unroll
        for (int t = 0; t < 8; t++) dst[(size_t)(2 * t + (lane >> 4)) * ry.w + (lane & 15)] = (short)q[t];
        return;
    }
    // C quotient and remainder, a negative remainder folded as QuarterRead does
    const int qx = mvx % 4, qy = mvy % 4;
    const int ox = n + mvx / 4 + (qx < 0 ? -1 : 0) - 2, oy0 = m + mvy / 4 + (qy < 0 ? -1 : 0) - 2;
    const int cs = (qx < 0 ? qx + 4 : qx) | ((qy < 0 ? qy + 4 : qy) << 2);
    if (lane < 22) {
        int x = ox + lane;
        x = x < 0 ? 0 : (x >= ry.w ? ry.w - 1 : x);
        const bool inside = oy0 >= 0 && oy0 + 22 <= ry.h;
#pragma unroll
        for (int h0 = 0; h0 < 22; h0 += 11) {  // two halves of 11 rows in flight
            int q[11];
            if (inside) {
                const short* p = ry.p + (size_t)(oy0 + h0) * ry.w + x;
#pragma unroll
                for (int r = 0; r < 11; r++) q[r] = __ldg(p + (size_t)r * ry.w);
            } else {
#pragma unroll
                for (int r = 0; r < 11; r++) q[r] = ry.at(x, oy0 + h0 + r);
            }
#pragma unroll
            for (int r = 0; r < 11; r++) L.win[h0 + r][lane] = (short)q[r];
        }
    }
    __syncwarp();
    if (cs == 6 || cs == 9 || cs == 10 || cs == 11 || cs == 14) {  // the cases that read j
        const int c = lane & 15, r0 = lane >> 4;
#pragma unroll
        for (int t = 0; t < 11; t++) L.th[r0 + 2 * t][c] = tap6<1>(&L.win[r0 + 2 * t][c]);
        __syncwarp();
    }
    mc_luma_quarter(L, cs, lane, dst, ry.w);
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
    // read from the frame itself unless the output overlaps it (then from a copy, as the reference does)
    const size_t frame = ny + 2 * nc;
    const short* src = d_ref_yuv;
    if (d_out_yuv < d_ref_yuv + frame && d_ref_yuv < d_out_yuv + frame) {
        VPP_CUDA(cudaMemcpyAsync(mc->d_tmp, d_ref_yuv, frame * sizeof(short), cudaMemcpyDeviceToDevice, ctx->stream));
        src = mc->d_tmp;
    }
    if (cols * rows > 0) {
        k_mc_frame<<<(cols * rows + kMcWarps - 1) / kMcWarps, 32 * kMcWarps, 0, ctx->stream>>>(
            Plane{src, W, H}, Plane{src + ny, cw, ch}, Plane{src + ny + nc, cw, ch}, (const int*)d_mv, cols,
            cols * rows, d_out_yuv, d_out_yuv + ny, d_out_yuv + ny + nc);
        VPP_CHECK_LAUNCH(ctx);
        ctx->launches++;
    }
    if (16 * rows < H) {  // rows below the last whole macroblock row keep the reference samples
        VPP_CUDA(cudaMemcpyAsync(d_out_yuv + (size_t)16 * rows * W, src + (size_t)16 * rows * W,
                                 (size_t)(H - 16 * rows) * W * sizeof(short), cudaMemcpyDeviceToDevice, ctx->stream));
        for (int p = 0; p < 2; p++) {
            const size_t o = ny + p * nc + (size_t)8 * rows * cw;
            VPP_CUDA(cudaMemcpyAsync(d_out_yuv + o, src + o, (size_t)(ch - 8 * rows) * cw * sizeof(short),
                                     cudaMemcpyDeviceToDevice, ctx->stream));
        }
    }
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
