// transform.cu -- H.264 4x4 forward integer transform + quantisation and
// dequantisation + inverse transform for sm_103a.
//
// Bit-exact with FastForward4x4ITImpl1/Impl2 / FastForward4x4On16x16ITImpl1
// (src/CodecUtils/FastForward4x4ITImpl1.cpp:100-201, FastForward4x4On16x16ITImpl1.cpp:457-757)
// and FastInverse4x4ITImpl1 / FastInverse4x4On16x16ITImpl1
// (src/CodecUtils/FastInverse4x4ITImpl1.cpp:119-244, FastInverse4x4On16x16ITImpl1.cpp:120-361):
// every intermediate the reference stores to a `short` is truncated to 16
// bits here at the same point.
//
// Also the DC Hadamard transforms of the Intra16x16 luma DC block (4x4) and
// the chroma DC block (2x2), FastForward/InverseDC4x4ITImpl1 and
// FastForward/InverseDC2x2ITImpl1.
//
// The work is HBM-bound (32 B read, 32 B written per block and pass), so the
// kernels are one thread per 4x4 block with each row moved as one 8-byte
// access; a warp covers 32 horizontally adjacent blocks, i.e. 256 contiguous
// bytes per row access.
#include "vppgpu_internal.cuh"

namespace {

// Quantiser multiplication factors MF[qp%6][class] and dequantiser scales
// V[qp%6][class]; class 0 = (even row, even col), 1 = (odd, odd), 2 = mixed
// (FastForward4x4ITImpl1.cpp:57-73, FastInverse4x4ITImpl1.cpp:60-74).
__constant__ int c_fwd_mf[6][3] = {{13107, 5243, 8066}, {11916, 4660, 7490}, {10082, 4194, 6554},
                                   {9362, 3647, 5825},  {8192, 3355, 5243},  {7282, 2893, 4559}};
__constant__ int c_inv_v[6][3] = {{10, 16, 13}, {11, 18, 14}, {13, 20, 16},
                                  {14, 23, 18}, {16, 25, 20}, {18, 29, 23}};

__host__ __device__ constexpr int pos_class(int pos)
{
    return (((pos >> 2) & 1) == 0 && (pos & 1) == 0) ? 0 : ((((pos >> 2) & 1) && (pos & 1)) ? 1 : 2);
}

struct FwdParams {
    int qm, f, sh;
};

struct InvParams {
    int weight[16];  // SetScale() weights (16 = flat)
    int qm, q, f, right, left;
};

FwdParams make_fwd(int qp, int intra)
{
    FwdParams p;
    int qe = qp / 6;
    p.qm = qp % 6;
    p.sh = 15 + qe;
    p.f = intra ? (1 << (15 + qe)) / 3 : (1 << (15 + qe)) / 6;
    return p;
}

InvParams make_inv(int qp, const int* weight16)
{
    InvParams p;
    int qe = qp / 6;
    for (int i = 0; i < 16; i++) p.weight[i] = weight16 ? weight16[i] : 16;
    p.qm = qp % 6;
    p.q = qp;
    p.f = qe <= 3 ? (1 << (3 - qe)) : 0;
    p.right = 4 - qe;
    p.left = qe - 4;
    return p;
}

__device__ __forceinline__ int s16(int x) { return (int)(short)x; }

__device__ __forceinline__ int quant(int x, int mf, const FwdParams& p)
{
    // sign-magnitude rounding: negative inputs are negated, never shifted
    return x < 0 ? s16(-(((-x) * mf + p.f) >> p.sh)) : s16((x * mf + p.f) >> p.sh);
}

// Forward transform of one block held as 16 ints (row-major), modes 0/1/2.
__device__ __forceinline__ void fwd_block(int* b, int mode, const FwdParams& p)
{
    if (mode == 2) {
#pragma unroll
        for (int i = 0; i < 16; i++) b[i] = quant(b[i], c_fwd_mf[p.qm][pos_class(i)], p);
        return;
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
        int* q = b + 4 * r;
        int s0 = q[0] + q[3], s3 = q[0] - q[3], s1 = q[1] + q[2], s2 = q[1] - q[2];
        q[0] = s16(s0 + s1);
        q[2] = s16(s0 - s1);
        q[1] = s16(s2 + (s3 << 1));
        q[3] = s16(s3 - (s2 << 1));
    }
#pragma unroll
    for (int c = 0; c < 4; c++) {
        int s0 = b[c] + b[12 + c], s3 = b[c] - b[12 + c];
        int s1 = b[4 + c] + b[8 + c], s2 = b[4 + c] - b[8 + c];
        int y0 = s0 + s1, y1 = s2 + (s3 << 1), y2 = s0 - s1, y3 = s3 - (s2 << 1);
        if (mode == 0) {
            b[c] = quant(y0, c_fwd_mf[p.qm][pos_class(c)], p);
            b[4 + c] = quant(y1, c_fwd_mf[p.qm][pos_class(4 + c)], p);
            b[8 + c] = quant(y2, c_fwd_mf[p.qm][pos_class(8 + c)], p);
            b[12 + c] = quant(y3, c_fwd_mf[p.qm][pos_class(12 + c)], p);
        } else {
            b[c] = s16(y0);
            b[4 + c] = s16(y1);
            b[8 + c] = s16(y2);
            b[12 + c] = s16(y3);
        }
    }
}

__device__ __forceinline__ int dequant(int x, int pos, const InvParams& p)
{
    int v = x * (c_inv_v[p.qm][pos_class(pos)] * p.weight[pos]);
    return p.q < 24 ? (v + p.f) >> p.right : v << p.left;
}

__device__ __forceinline__ void inv_1d(int x0, int x1, int x2, int x3, int& y0, int& y1, int& y2, int& y3)
{
    int s0 = x0 + x2, s1 = x0 - x2, s2 = (x1 >> 1) - x3, s3 = x1 + (x3 >> 1);
    y0 = s0 + s3;
    y1 = s1 + s2;
    y2 = s1 - s2;
    y3 = s0 - s3;
}

// Inverse of one block: mode 2 = dequant only; modes 0/1 with the pass order
// of FastInverse4x4ITImpl1 (rows first) or the On16x16 variant (cols first).
__device__ __forceinline__ void inv_block(int* b, int mode, int cols_first, const InvParams& p)
{
    if (mode == 2) {
#pragma unroll
        for (int i = 0; i < 16; i++) b[i] = s16(dequant(b[i], i, p));
        return;
    }
    if (mode == 0) {
#pragma unroll
        for (int i = 0; i < 16; i++) b[i] = dequant(b[i], i, p);
    }
    int y0, y1, y2, y3;
    if (!cols_first) {
#pragma unroll
        for (int r = 0; r < 4; r++) {
            int* q = b + 4 * r;
            inv_1d(q[0], q[1], q[2], q[3], y0, y1, y2, y3);
            q[0] = s16(y0); q[1] = s16(y1); q[2] = s16(y2); q[3] = s16(y3);
        }
#pragma unroll
        for (int c = 0; c < 4; c++) {
            inv_1d(b[c], b[4 + c], b[8 + c], b[12 + c], y0, y1, y2, y3);
            b[c] = s16((y0 + 32) >> 6); b[4 + c] = s16((y1 + 32) >> 6);
            b[8 + c] = s16((y2 + 32) >> 6); b[12 + c] = s16((y3 + 32) >> 6);
        }
    } else {
#pragma unroll
        for (int c = 0; c < 4; c++) {
            inv_1d(b[c], b[4 + c], b[8 + c], b[12 + c], y0, y1, y2, y3);
            b[c] = s16(y0); b[4 + c] = s16(y1); b[8 + c] = s16(y2); b[12 + c] = s16(y3);
        }
#pragma unroll
        for (int r = 0; r < 4; r++) {
            int* q = b + 4 * r;
            inv_1d(q[0], q[1], q[2], q[3], y0, y1, y2, y3);
            q[0] = s16((y0 + 32) >> 6); q[1] = s16((y1 + 32) >> 6);
            q[2] = s16((y2 + 32) >> 6); q[3] = s16((y3 + 32) >> 6);
        }
    }
}

// ---- block addressing ----------------------------------------------------
// Returns the element offset of block `blk`'s top-left sample and its row
// stride for the two unit layouts.
__device__ __forceinline__ long long block_origin(long long blk, int layout, int& rs)
{
    if (layout == VPPGPU_LAYOUT_BLOCKS) {
        rs = 4;
        return blk * 16;
    }
    rs = 16;  // 16x16 raster macroblock: 16 blocks per unit
    long long mb = blk >> 4;
    int bi = (int)(blk & 15);
    return mb * 256 + (bi >> 2) * 64 + (bi & 3) * 4;
}

__device__ __forceinline__ void load_rows(const short* p, int rs, int* b)
{
#pragma unroll
    for (int r = 0; r < 4; r++) {
        uint2 v = *reinterpret_cast<const uint2*>(p + (size_t)r * rs);
        b[4 * r + 0] = (int)(short)(v.x & 0xffff);
        b[4 * r + 1] = (int)(short)(v.x >> 16);
        b[4 * r + 2] = (int)(short)(v.y & 0xffff);
        b[4 * r + 3] = (int)(short)(v.y >> 16);
    }
}

__device__ __forceinline__ void store_rows(short* p, int rs, const int* b)
{
#pragma unroll
    for (int r = 0; r < 4; r++) {
        uint2 v;
        v.x = (unsigned)(b[4 * r + 0] & 0xffff) | ((unsigned)b[4 * r + 1] << 16);
        v.y = (unsigned)(b[4 * r + 2] & 0xffff) | ((unsigned)b[4 * r + 3] << 16);
        *reinterpret_cast<uint2*>(p + (size_t)r * rs) = v;
    }
}

__global__ void __launch_bounds__(256) k_fwd_units(short* __restrict__ data, long long nblocks, int layout,
                                                   int mode, FwdParams p)
{
    for (long long blk = blockIdx.x * (long long)blockDim.x + threadIdx.x; blk < nblocks;
         blk += (long long)gridDim.x * blockDim.x) {
        int rs;
        short* q = data + block_origin(blk, layout, rs);
        int b[16];
        load_rows(q, rs, b);
        fwd_block(b, mode, p);
        store_rows(q, rs, b);
    }
}

__global__ void __launch_bounds__(256) k_inv_units(short* __restrict__ data, long long nblocks, int layout,
                                                   int mode, InvParams p)
{
    int cols_first = layout == VPPGPU_LAYOUT_MB16;
    for (long long blk = blockIdx.x * (long long)blockDim.x + threadIdx.x; blk < nblocks;
         blk += (long long)gridDim.x * blockDim.x) {
        int rs;
        short* q = data + block_origin(blk, layout, rs);
        int b[16];
        load_rows(q, rs, b);
        inv_block(b, mode, cols_first, p);
        store_rows(q, rs, b);
    }
}

}  // namespace

// ---- fused plane round trip (also used by the batched/served forms) -------
namespace vppgpu {

// Same layout as vppgpu_tq_job (include/vppgpu.h).
struct TqJob {
    const short* res;
    short* lev;
    short* rec;
    int width, height, stride;
    int qp, intra;
};
static_assert(sizeof(TqJob) == sizeof(vppgpu_tq_job), "TqJob must mirror vppgpu_tq_job");

}  // namespace vppgpu

namespace {

// Per-plane constants of the fused round trip, computed once per thread:
// the quantiser factors of the three position classes, its rounding and
// shift, the dequantiser scales V[qp%6][class] and the post-scale.  The
// SetScale() weights stay in the kernel's parameter space: the dequantised
// coefficient is x * V[class] * weight[pos] (the same bits as x * (V * w)).
struct RtConsts {
    int mf0, mf1, mf2, f, sh;
    int v0, v1, v2, df, right, left;
    bool small_q;  // qp < 24: rounded right shift, else left shift
};

__device__ __forceinline__ RtConsts rt_consts(int qp, int intra)
{
    RtConsts c;
    const int qe = qp / 6, qm = qp % 6;
    c.mf0 = c_fwd_mf[qm][0];
    c.mf1 = c_fwd_mf[qm][1];
    c.mf2 = c_fwd_mf[qm][2];
    c.sh = 15 + qe;
    c.f = intra ? (1 << (15 + qe)) / 3 : (1 << (15 + qe)) / 6;
    c.v0 = c_inv_v[qm][0];
    c.v1 = c_inv_v[qm][1];
    c.v2 = c_inv_v[qm][2];
    c.df = qe <= 3 ? (1 << (3 - qe)) : 0;
    c.right = 4 - qe;
    c.left = qe - 4;
    c.small_q = qp < 24;
    return c;
}

__device__ __forceinline__ int rt_quant(int x, int mf, const RtConsts& c)
{
    const int q = ((x < 0 ? -x : x) * mf + c.f) >> c.sh;
    return s16(x < 0 ? -q : q);
}

// Forward transform + quantisation (mode 0) of fwd_block, then the
// dequantisation + inverse of inv_block (mode 0, pass order kColsFirst),
// with the constants in registers; the levels are stored in between.
template <bool kColsFirst>
__device__ __forceinline__ void roundtrip_block(const short* res, short* lev, short* rec, int stride,
                                               const RtConsts& c, const int* weight)
{
    int b[16];
    load_rows(res, stride, b);
#pragma unroll
    for (int r = 0; r < 4; r++) {
        int* q = b + 4 * r;
        const int s0 = q[0] + q[3], s3 = q[0] - q[3], s1 = q[1] + q[2], s2 = q[1] - q[2];
        q[0] = s16(s0 + s1);
        q[2] = s16(s0 - s1);
        q[1] = s16(s2 + (s3 << 1));
        q[3] = s16(s3 - (s2 << 1));
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int s0 = b[k] + b[12 + k], s3 = b[k] - b[12 + k], s1 = b[4 + k] + b[8 + k], s2 = b[4 + k] - b[8 + k];
        // classes: even row & even col 0, odd & odd 1, mixed 2
        const int mf_even = (k & 1) ? c.mf2 : c.mf0, mf_odd = (k & 1) ? c.mf1 : c.mf2;
        b[k] = rt_quant(s0 + s1, mf_even, c);
        b[4 + k] = rt_quant(s2 + (s3 << 1), mf_odd, c);
        b[8 + k] = rt_quant(s0 - s1, mf_even, c);
        b[12 + k] = rt_quant(s3 - (s2 << 1), mf_odd, c);
    }
    store_rows(lev, stride, b);
#pragma unroll
    for (int i = 0; i < 16; i++) {
        const int cls = pos_class(i);
        const int v = b[i] * (cls == 0 ? c.v0 : (cls == 1 ? c.v1 : c.v2)) * weight[i];
        b[i] = c.small_q ? (v + c.df) >> c.right : v << c.left;
    }
    int y0, y1, y2, y3;
    if constexpr (!kColsFirst) {
#pragma unroll
        for (int r = 0; r < 4; r++) {
            int* q = b + 4 * r;
            inv_1d(q[0], q[1], q[2], q[3], y0, y1, y2, y3);
            q[0] = s16(y0); q[1] = s16(y1); q[2] = s16(y2); q[3] = s16(y3);
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            inv_1d(b[k], b[4 + k], b[8 + k], b[12 + k], y0, y1, y2, y3);
            b[k] = s16((y0 + 32) >> 6); b[4 + k] = s16((y1 + 32) >> 6);
            b[8 + k] = s16((y2 + 32) >> 6); b[12 + k] = s16((y3 + 32) >> 6);
        }
    } else {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            inv_1d(b[k], b[4 + k], b[8 + k], b[12 + k], y0, y1, y2, y3);
            b[k] = s16(y0); b[4 + k] = s16(y1); b[8 + k] = s16(y2); b[12 + k] = s16(y3);
        }
#pragma unroll
        for (int r = 0; r < 4; r++) {
            int* q = b + 4 * r;
            inv_1d(q[0], q[1], q[2], q[3], y0, y1, y2, y3);
            q[0] = s16((y0 + 32) >> 6); q[1] = s16((y1 + 32) >> 6);
            q[2] = s16((y2 + 32) >> 6); q[3] = s16((y3 + 32) >> 6);
        }
    }
    store_rows(rec, stride, b);
}

// One plane: rows of 4x4 blocks strided over the CTAs that serve the plane,
// the blocks of a row over the CTA's threads (8-byte row accesses, 256
// contiguous bytes per warp and row).  No index division.
template <bool kColsFirst>
__device__ __forceinline__ void roundtrip_plane(const vppgpu::TqJob& j, const int* weight, int row0, int rstep)
{
    const RtConsts c = rt_consts(j.qp, j.intra);
    const int bw = j.width >> 2, bh = j.height >> 2;
    for (int by = row0; by < bh; by += rstep) {
        const size_t row = (size_t)by * 4 * j.stride;
        for (int bx = threadIdx.x; bx < bw; bx += blockDim.x) {
            const size_t off = row + (size_t)bx * 4;
            roundtrip_block<kColsFirst>(j.res + off, j.lev + off, j.rec + off, j.stride, c, weight);
        }
    }
}

struct Weights {
    int w[16];
};

// blockIdx.y selects the plane; blockIdx.x strides over its rows of blocks.
// Up to 256 CTAs per plane, so a CTA holds one or two rows of a 1080p or 4K
// plane and the kernel's tail is one short CTA.
template <bool kColsFirst>
__global__ void __launch_bounds__(256, 6) k_tq_roundtrip(const vppgpu::TqJob* __restrict__ jobs, Weights wt)
{
    const vppgpu::TqJob j = jobs[blockIdx.y];
    roundtrip_plane<kColsFirst>(j, wt.w, blockIdx.x, gridDim.x);
}

template <bool kColsFirst>
__global__ void __launch_bounds__(256, 6) k_tq_roundtrip_single(vppgpu::TqJob j, Weights wt)
{
    roundtrip_plane<kColsFirst>(j, wt.w, blockIdx.x, gridDim.x);
}

// ---- DC Hadamard transforms (Intra16x16 luma DC 4x4, chroma DC 2x2) --------
// FastForwardDC4x4ITImpl1 / FastInverseDC4x4ITImpl1 and FastForwardDC2x2ITImpl1
// / FastInverseDC2x2ITImpl1 (src/CodecUtils/FastForwardDC4x4ITImpl1.cpp:101-196,
// FastInverseDC4x4ITImpl1.cpp:111-202, FastForwardDC2x2ITImpl1.cpp:100-164,
// FastInverseDC2x2ITImpl1.cpp:110-157): one thread per block, the block moved
// with 16-byte (4x4) or 8-byte (2x2) accesses when the array allows it.
struct DcParams {
    int mode, q, qe;
    int na, f, sh;  // forward: NormAdjust[qp%6], 2 * (2^(15+qe) / 3), 16 + qe
    int ls[16];     // inverse: NormAdjust[qp%6] * weight[pos]
};

DcParams make_dc(int size, int mode, int qp, const int* weight)
{
    static const int fwd_na[6] = {13107, 11916, 10082, 9362, 8192, 7282};
    static const int inv_na[6] = {10, 11, 13, 14, 16, 18};
    DcParams p;
    p.mode = mode;
    p.q = qp;
    p.qe = qp / 6;
    p.na = fwd_na[qp % 6];
    p.f = 2 * ((1 << (15 + p.qe)) / 3);
    p.sh = 16 + p.qe;
    for (int i = 0; i < 16; i++) p.ls[i] = i < size * size ? inv_na[qp % 6] * (weight ? weight[i] : 16) : 0;
    return p;
}

__device__ __forceinline__ int dc_quant(int x, const DcParams& p)
{
    return x < 0 ? s16(-(((-x) * p.na + p.f) >> p.sh)) : s16((x * p.na + p.f) >> p.sh);
}

__device__ __forceinline__ int shl(int x, int s) { return (int)((unsigned)x << s); }

// inverse 4x4 post-scale: qp < 36 rounds at 2^(5-qe) and shifts right by 6-qe, else shifts left by qe-6
__device__ __forceinline__ int dc4_scale(int x, int ls, const DcParams& p)
{
    const int v = x * ls;
    return p.q < 36 ? s16((v + (1 << (5 - p.qe))) >> (6 - p.qe)) : s16(shl(v, p.qe - 6));
}

__device__ __forceinline__ void fwd_dc4(int* b, const DcParams& p)
{
    if (p.mode == 2) {
#pragma unroll
        for (int i = 0; i < 16; i++) b[i] = dc_quant(b[i], p);
        return;
    }
#pragma unroll
    for (int r = 0; r < 16; r += 4) {  // rows, each stored as short
        const int a = b[r] + b[r + 3], d = b[r] - b[r + 3], c = b[r + 1] + b[r + 2], e = b[r + 1] - b[r + 2];
        b[r] = s16(a + c);
        b[r + 2] = s16(a - c);
        b[r + 1] = s16(e + d);
        b[r + 3] = s16(d - e);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {  // columns, halved, then quantised (mode 0)
        const int a = b[k] + b[k + 12], d = b[k] - b[k + 12], c = b[k + 4] + b[k + 8], e = b[k + 4] - b[k + 8];
        const int y0 = (a + c) >> 1, y2 = (a - c) >> 1, y1 = (e + d) >> 1, y3 = (d - e) >> 1;
        b[k] = p.mode == 0 ? dc_quant(y0, p) : s16(y0);
        b[k + 4] = p.mode == 0 ? dc_quant(y1, p) : s16(y1);
        b[k + 8] = p.mode == 0 ? dc_quant(y2, p) : s16(y2);
        b[k + 12] = p.mode == 0 ? dc_quant(y3, p) : s16(y3);
    }
}

__device__ __forceinline__ void inv_dc4(int* b, const DcParams& p)
{
    if (p.mode == 2) {
#pragma unroll
        for (int i = 0; i < 16; i++) b[i] = dc4_scale(b[i], p.ls[i], p);
        return;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {  // columns, each stored as short
        const int s0 = b[k] + b[8 + k], s1 = b[k] - b[8 + k], s2 = b[4 + k] - b[12 + k], s3 = b[4 + k] + b[12 + k];
        b[k] = s16(s0 + s3);
        b[12 + k] = s16(s0 - s3);
        b[4 + k] = s16(s1 + s2);
        b[8 + k] = s16(s1 - s2);
    }
#pragma unroll
    for (int r = 0; r < 16; r += 4) {  // rows, post-scaled (mode 0)
        const int s0 = b[r] + b[2 + r], s1 = b[r] - b[2 + r], s2 = b[1 + r] - b[3 + r], s3 = b[1 + r] + b[3 + r];
        if (p.mode == 0) {
            const int y0 = dc4_scale(s0 + s3, p.ls[r], p), y1 = dc4_scale(s1 + s2, p.ls[r + 1], p);
            const int y2 = dc4_scale(s1 - s2, p.ls[r + 2], p), y3 = dc4_scale(s0 - s3, p.ls[r + 3], p);
            b[r] = y0;
            b[r + 1] = y1;
            b[r + 2] = y2;
            b[r + 3] = y3;
        } else {
            b[r] = s16(s0 + s3);
            b[r + 3] = s16(s0 - s3);
            b[r + 1] = s16(s1 + s2);
            b[r + 2] = s16(s1 - s2);
        }
    }
}

__device__ __forceinline__ void fwd_dc2(int* b, const DcParams& p)
{
    if (p.mode == 2) {
#pragma unroll
        for (int i = 0; i < 4; i++) b[i] = dc_quant(b[i], p);
        return;
    }
    const int s0 = b[0] + b[1], s2 = b[0] - b[1], s1 = b[2] + b[3], s3 = b[2] - b[3];
    const int y0 = s0 + s1, y2 = s0 - s1, y1 = s2 + s3, y3 = s2 - s3;
    b[0] = p.mode == 0 ? dc_quant(y0, p) : s16(y0);
    b[1] = p.mode == 0 ? dc_quant(y1, p) : s16(y1);
    b[2] = p.mode == 0 ? dc_quant(y2, p) : s16(y2);
    b[3] = p.mode == 0 ? dc_quant(y3, p) : s16(y3);
}

// inverse 2x2 post-scale: (x * levelScale << qe) >> 5
__device__ __forceinline__ void inv_dc2(int* b, const DcParams& p)
{
    if (p.mode == 2) {
#pragma unroll
        for (int i = 0; i < 4; i++) b[i] = s16(shl(b[i] * p.ls[i], p.qe) >> 5);
        return;
    }
    const int s0 = b[0] + b[1], s2 = b[0] - b[1], s1 = b[2] + b[3], s3 = b[2] - b[3];
    if (p.mode == 0) {
        const int x0 = (s0 + s1) * p.ls[0], x1 = (s2 + s3) * p.ls[1], x2 = (s0 - s1) * p.ls[2],
                  x3 = (s2 - s3) * p.ls[3];
        b[0] = s16(shl(x0, p.qe) >> 5);
        b[1] = s16(shl(x1, p.qe) >> 5);
        b[2] = s16(shl(x2, p.qe) >> 5);
        b[3] = s16(shl(x3, p.qe) >> 5);
    } else {
        b[0] = s16(s0 + s1);
        b[2] = s16(s0 - s1);
        b[1] = s16(s2 + s3);
        b[3] = s16(s2 - s3);
    }
}

template <int kN>
__device__ __forceinline__ void load_unit(const short* q, bool vec, int* b)
{
    auto lo = [](unsigned w) { return (int)(short)(w & 0xffff); };
    auto hi = [](unsigned w) { return (int)(short)(w >> 16); };
    if (vec) {
        if constexpr (kN == 16) {
#pragma unroll
            for (int h = 0; h < 16; h += 8) {
                const uint4 v = *reinterpret_cast<const uint4*>(q + h);
                b[h] = lo(v.x), b[h + 1] = hi(v.x), b[h + 2] = lo(v.y), b[h + 3] = hi(v.y);
                b[h + 4] = lo(v.z), b[h + 5] = hi(v.z), b[h + 6] = lo(v.w), b[h + 7] = hi(v.w);
            }
        } else {
            const uint2 v = *reinterpret_cast<const uint2*>(q);
            b[0] = lo(v.x), b[1] = hi(v.x), b[2] = lo(v.y), b[3] = hi(v.y);
        }
    } else {
#pragma unroll
        for (int i = 0; i < kN; i++) b[i] = q[i];
    }
}

template <int kN>
__device__ __forceinline__ void store_unit(short* q, bool vec, const int* b)
{
    auto pk = [&](int i) { return (unsigned)(b[i] & 0xffff) | ((unsigned)b[i + 1] << 16); };
    if (vec) {
        if constexpr (kN == 16) {
#pragma unroll
            for (int h = 0; h < 16; h += 8)
                *reinterpret_cast<uint4*>(q + h) = make_uint4(pk(h), pk(h + 2), pk(h + 4), pk(h + 6));
        } else {
            *reinterpret_cast<uint2*>(q) = make_uint2(pk(0), pk(2));
        }
    } else {
#pragma unroll
        for (int i = 0; i < kN; i++) q[i] = (short)b[i];
    }
}

template <int kSize, bool kFwd>
__global__ void __launch_bounds__(256) k_dc_units(short* __restrict__ data, long long nunits, bool vec, DcParams p)
{
    constexpr int kN = kSize * kSize;
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < nunits;
         u += (long long)gridDim.x * blockDim.x) {
        short* q = data + u * kN;
        int b[kN];
        load_unit<kN>(q, vec, b);
        if constexpr (kSize == 4) {
            if constexpr (kFwd) fwd_dc4(b, p);
            else inv_dc4(b, p);
        } else {
            if constexpr (kFwd) fwd_dc2(b, p);
            else inv_dc2(b, p);
        }
        store_unit<kN>(q, vec, b);
    }
}

int grid_for(vppgpu_ctx* ctx, long long nblocks)
{
    long long want = (nblocks + 255) / 256;
    long long cap = (long long)ctx->sm_count * 8;
    return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

int check_common(vppgpu_ctx* ctx, const void* p, long long nunits, int layout, int mode, int qp)
{
    if (!ctx || !p || nunits < 0) return VPPGPU_ERR_INVALID_ARG;
    if (layout != VPPGPU_LAYOUT_BLOCKS && layout != VPPGPU_LAYOUT_MB16) return VPPGPU_ERR_INVALID_ARG;
    if (mode < 0 || mode > 2 || qp < 0 || qp > 51) return VPPGPU_ERR_INVALID_ARG;
    return VPPGPU_OK;
}

}  // namespace

namespace vppgpu {

int launch_tq_jobs(vppgpu_ctx* ctx, const TqJob* d_jobs, int njobs, int inv_order, const int* weight16)
{
    Weights wt;
    for (int i = 0; i < 16; i++) wt.w[i] = weight16 ? weight16[i] : 16;
    const dim3 grid(256, njobs);
    if (inv_order == VPPGPU_INV_COLS_FIRST)
        k_tq_roundtrip<true><<<grid, 256, 0, ctx->stream>>>(d_jobs, wt);
    else
        k_tq_roundtrip<false><<<grid, 256, 0, ctx->stream>>>(d_jobs, wt);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

}  // namespace vppgpu

extern "C" {

int vppgpu_fwd4x4_device(vppgpu_ctx* ctx, short* d, long long nunits, int layout, int mode, int qp, int intra)
{
    int rc = check_common(ctx, d, nunits, layout, mode, qp);
    if (rc) return rc;
    if ((rc = vppgpu::bind(ctx))) return rc;
    long long nblocks = layout == VPPGPU_LAYOUT_BLOCKS ? nunits : nunits * 16;
    if (nblocks == 0) return VPPGPU_OK;
    k_fwd_units<<<grid_for(ctx, nblocks), 256, 0, ctx->stream>>>(d, nblocks, layout, mode,
                                                                   make_fwd(qp, intra != 0));
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

int vppgpu_inv4x4_device(vppgpu_ctx* ctx, short* d, long long nunits, int layout, int mode, int qp,
                         const int* weight16)
{
    int rc = check_common(ctx, d, nunits, layout, mode, qp);
    if (rc) return rc;
    if ((rc = vppgpu::bind(ctx))) return rc;
    long long nblocks = layout == VPPGPU_LAYOUT_BLOCKS ? nunits : nunits * 16;
    if (nblocks == 0) return VPPGPU_OK;
    k_inv_units<<<grid_for(ctx, nblocks), 256, 0, ctx->stream>>>(d, nblocks, layout, mode,
                                                                   make_inv(qp, weight16));
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

static int host_units(vppgpu_ctx* ctx, short* data, long long nunits, int layout, bool fwd, int mode, int qp,
                      int intra, const int* weight16)
{
    int rc = check_common(ctx, data, nunits, layout, mode, qp);
    if (rc) return rc;
    if ((rc = vppgpu::bind(ctx))) return rc;
    size_t bytes = (size_t)nunits * (layout == VPPGPU_LAYOUT_BLOCKS ? 32 : 512);
    if (bytes == 0) return VPPGPU_OK;
    short* d = nullptr;
    VPP_CUDA(cudaMallocAsync((void**)&d, bytes, ctx->stream));
    cudaError_t e = cudaMemcpyAsync(d, data, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        rc = fwd ? vppgpu_fwd4x4_device(ctx, d, nunits, layout, mode, qp, intra)
                 : vppgpu_inv4x4_device(ctx, d, nunits, layout, mode, qp, weight16);
        if (rc == VPPGPU_OK) e = cudaMemcpyAsync(data, d, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    }
    cudaFreeAsync(d, ctx->stream);
    cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
    if (rc) return rc;
    if (e != cudaSuccess) return vppgpu::cuda_status(e);
    if (e2 != cudaSuccess) return vppgpu::cuda_status(e2);
    return VPPGPU_OK;
}

int vppgpu_fwd4x4(vppgpu_ctx* ctx, short* data, long long nunits, int layout, int mode, int qp, int intra)
{
    return host_units(ctx, data, nunits, layout, true, mode, qp, intra, nullptr);
}

int vppgpu_inv4x4(vppgpu_ctx* ctx, short* data, long long nunits, int layout, int mode, int qp,
                  const int* weight16)
{
    return host_units(ctx, data, nunits, layout, false, mode, qp, 0, weight16);
}

int vppgpu_tq_roundtrip_plane_device(vppgpu_ctx* ctx, const short* res, short* lev, short* rec, int width,
                                     int height, int stride, int qp, int intra, int inv_order,
                                     const int* weight16)
{
    if (!ctx || !res || !lev || !rec || width <= 0 || height <= 0 || (width & 3) || (height & 3) ||
        stride < width || (stride & 3) || qp < 0 || qp > 51 ||
        (inv_order != VPPGPU_INV_ROWS_FIRST && inv_order != VPPGPU_INV_COLS_FIRST))
        return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    vppgpu::TqJob j{res, lev, rec, width, height, stride, qp, intra != 0};
    Weights wt;
    for (int i = 0; i < 16; i++) wt.w[i] = weight16 ? weight16[i] : 16;
    const int rows = height >> 2, g = rows < 2 * 8 * ctx->sm_count ? rows : 2 * 8 * ctx->sm_count;
    if (inv_order == VPPGPU_INV_COLS_FIRST)
        k_tq_roundtrip_single<true><<<g, 256, 0, ctx->stream>>>(j, wt);
    else
        k_tq_roundtrip_single<false><<<g, 256, 0, ctx->stream>>>(j, wt);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

int vppgpu_tq_roundtrip_plane(vppgpu_ctx* ctx, const short* residual, short* levels, short* recon, int width,
                              int height, int stride, int qp, int intra, int inv_order, const int* weight16)
{
    if (!ctx || !residual || !levels || !recon || width <= 0 || height <= 0 || stride < width)
        return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    size_t bytes = (size_t)stride * height * sizeof(short);
    short* d = nullptr;
    VPP_CUDA(cudaMallocAsync((void**)&d, 3 * bytes, ctx->stream));
    cudaError_t e = cudaMemcpyAsync(d, residual, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        short* dl = d + (size_t)stride * height;
        short* dr = dl + (size_t)stride * height;
        rc = vppgpu_tq_roundtrip_plane_device(ctx, d, dl, dr, width, height, stride, qp, intra, inv_order,
                                              weight16);
        if (rc == VPPGPU_OK) e = cudaMemcpyAsync(levels, dl, bytes, cudaMemcpyDeviceToHost, ctx->stream);
        if (rc == VPPGPU_OK && e == cudaSuccess)
            e = cudaMemcpyAsync(recon, dr, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    }
    cudaFreeAsync(d, ctx->stream);
    cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
    if (rc) return rc;
    if (e != cudaSuccess) return vppgpu::cuda_status(e);
    if (e2 != cudaSuccess) return vppgpu::cuda_status(e2);
    return VPPGPU_OK;
}

int vppgpu_tq_roundtrip_planes_device(vppgpu_ctx* ctx, const vppgpu_tq_job* d_jobs, int njobs, int inv_order,
                                      const int* weight16)
{
    if (!ctx || !d_jobs || njobs < 1 || njobs > 65535 ||
        (inv_order != VPPGPU_INV_ROWS_FIRST && inv_order != VPPGPU_INV_COLS_FIRST))
        return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    return vppgpu::launch_tq_jobs(ctx, reinterpret_cast<const vppgpu::TqJob*>(d_jobs), njobs, inv_order, weight16);
}

static int dc_device(vppgpu_ctx* ctx, short* d, long long nunits, int size, bool forward, int mode, int qp,
                     const int* weight)
{
    if (!ctx || nunits < 0 || (nunits > 0 && !d) || (size != 2 && size != 4) || mode < 0 || mode > 2 || qp < 0 ||
        qp > 51)
        return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    if (nunits == 0) return VPPGPU_OK;
    const bool vec = ((uintptr_t)d & (size == 4 ? 15 : 7)) == 0;
    const DcParams p = make_dc(size, mode, qp, forward ? nullptr : weight);
    const int g = grid_for(ctx, nunits);
    if (size == 4 && forward) k_dc_units<4, true><<<g, 256, 0, ctx->stream>>>(d, nunits, vec, p);
    else if (size == 4) k_dc_units<4, false><<<g, 256, 0, ctx->stream>>>(d, nunits, vec, p);
    else if (forward) k_dc_units<2, true><<<g, 256, 0, ctx->stream>>>(d, nunits, vec, p);
    else k_dc_units<2, false><<<g, 256, 0, ctx->stream>>>(d, nunits, vec, p);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

static int dc_host(vppgpu_ctx* ctx, short* data, long long nunits, int size, bool forward, int mode, int qp,
                   const int* weight)
{
    if (!ctx || nunits < 0 || (nunits > 0 && !data) || (size != 2 && size != 4) || mode < 0 || mode > 2 || qp < 0 ||
        qp > 51)
        return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    const size_t bytes = (size_t)nunits * size * size * sizeof(short);
    if (bytes == 0) return VPPGPU_OK;
    short* d = nullptr;
    VPP_CUDA(cudaMallocAsync((void**)&d, bytes, ctx->stream));
    cudaError_t e = cudaMemcpyAsync(d, data, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        rc = dc_device(ctx, d, nunits, size, forward, mode, qp, weight);
        if (rc == VPPGPU_OK) e = cudaMemcpyAsync(data, d, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    }
    cudaFreeAsync(d, ctx->stream);
    cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
    if (rc) return rc;
    if (e != cudaSuccess) return vppgpu::cuda_status(e);
    if (e2 != cudaSuccess) return vppgpu::cuda_status(e2);
    return VPPGPU_OK;
}

int vppgpu_fwd_dc_device(vppgpu_ctx* ctx, short* d_data, long long nunits, int size, int mode, int qp)
{
    return dc_device(ctx, d_data, nunits, size, true, mode, qp, nullptr);
}

int vppgpu_inv_dc_device(vppgpu_ctx* ctx, short* d_data, long long nunits, int size, int mode, int qp,
                         const int* weight)
{
    return dc_device(ctx, d_data, nunits, size, false, mode, qp, weight);
}

int vppgpu_fwd_dc(vppgpu_ctx* ctx, short* data, long long nunits, int size, int mode, int qp)
{
    return dc_host(ctx, data, nunits, size, true, mode, qp, nullptr);
}

int vppgpu_inv_dc(vppgpu_ctx* ctx, short* data, long long nunits, int size, int mode, int qp, const int* weight)
{
    return dc_host(ctx, data, nunits, size, false, mode, qp, weight);
}

int vppgpu_dc_quantise_value(short val, int qp)
{
    if (qp < 0 || qp > 51) return 0;
    const DcParams p = make_dc(4, 0, qp, nullptr);
    const int x = (int)val;
    return x < 0 ? (int)(short)(-(((-x) * p.na + p.f) >> p.sh)) : (int)(short)((x * p.na + p.f) >> p.sh);
}

int vppgpu_quantise_value(short val, int pos, int qp, int intra)
{
    static const int mf[6][3] = {{13107, 5243, 8066}, {11916, 4660, 7490}, {10082, 4194, 6554},
                                 {9362, 3647, 5825},  {8192, 3355, 5243},  {7282, 2893, 4559}};
    if (pos < 0 || pos > 15 || qp < 0 || qp > 51) return 0;
    int qe = qp / 6;
    int f = intra ? (1 << (15 + qe)) / 3 : (1 << (15 + qe)) / 6;
    int m = mf[qp % 6][pos_class(pos)];
    int x = (int)val;
    return x < 0 ? (int)(short)(-(((-x) * m + f) >> (15 + qe))) : (int)(short)((x * m + f) >> (15 + qe));
}

}  // extern "C"
