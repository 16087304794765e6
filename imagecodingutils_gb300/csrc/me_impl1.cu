// me_impl1.cu -- MotionEstimatorImpl1::Estimate
// (src/CodecUtils/MotionEstimatorImpl1.cpp:275-395) on the GPU.
//
// A full search of [-R, R-1]^2 full pels by SSD per block (16x16 or 8x8), the
// OverlayMem2Dv2::HalfRead half-pel refinement (OverlayMem2Dv2.cpp:452-596)
// over the neighbours GetHalfPelSearchStruct allows at the range's extremes
// (MotionEstimatorImpl1.cpp:445-515), and a weighted choice between the winner
// and the zero vector (:356-378).  There is no predictor, so every block is
// independent: one warp per block, its search window (rows and columns
// -R-1 .. R+B of the padded reference) and template staged in shared memory,
// one lane per candidate.  The reference's raster scan keeps the first
// strictly smaller distortion, i.e. the smallest (distortion, raster index)
// pair below the zero vector's distortion: a warp argmin on that pair.
#include "me_full_common.cuh"

namespace vppgpu {
namespace {

constexpr int kMaxRange = 32;
constexpr int kWinStride = 112;                    // 15 alignment bytes + 2R + 16 + 2, rounded to 16
constexpr int kWinRows = 2 * kMaxRange + 16 + 2;   // 82
constexpr int kWinBytes = kWinStride * kWinRows;
constexpr int kSlot = kWinBytes + 16 + 256;        // window, five-word overrun, template (16 rows of 16 bytes)
constexpr int kWarps = 4;

struct Impl1Args {
    FullArgs f;       // planes, job, control
    int bw, bh;       // block size
    int bcols, nblk;  // blocks per row, blocks
    int range;        // R, full pels
};

// Eight or sixteen window bytes of row p (any alignment) against the
// template row: SSD of one block row by one lane.
template <int BW>
__device__ __forceinline__ unsigned row_sd(const unsigned char* p, const unsigned* t, unsigned acc)
{
    const unsigned* w = reinterpret_cast<const unsigned*>(reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)3);
    const unsigned sh = (unsigned)(reinterpret_cast<uintptr_t>(p) & 3) * 8;
#pragma unroll
    for (int q = 0; q < BW / 4; q++) {
        const unsigned d = __vabsdiffu4(__funnelshift_r(w[q], w[q + 1], sh), t[q]);
        acc = __dp4a(d, d, acc);
    }
    return acc;
}

// H.263 half-pel samples of four bytes (OverlayMem2Dv2::HalfRead) from the
// samples a (the block's), b (beside it), c (below or above it) and d (both):
// the rounded mean of a and its one neighbour on the horizontal or vertical
// lines, (a + b + c + d + 2) / 4 on the diagonals, evaluated in 16-bit lanes.
__device__ __forceinline__ unsigned half4(unsigned a, unsigned b, unsigned c, unsigned d, int hx, int hy)
{
    if (!hy) return __vavgu4(a, b);
    if (!hx) return __vavgu4(a, c);
    const unsigned m = 0x00ff00ffu;
    const unsigned lo = (a & m) + (b & m) + (c & m) + (d & m) + 0x00020002u;
    const unsigned hi = ((a >> 8) & m) + ((b >> 8) & m) + ((c >> 8) & m) + ((d >> 8) & m) + 0x00020002u;
    return ((lo >> 2) & m) | (((hi >> 2) & m) << 8);
}

// Four bytes at any offset of a shared-memory row.
__device__ __forceinline__ unsigned word_at(const unsigned char* p)
{
    const unsigned* w = reinterpret_cast<const unsigned*>(reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)3);
    const unsigned sh = (unsigned)(reinterpret_cast<uintptr_t>(p) & 3) * 8;
    return __funnelshift_r(w[0], w[1], sh);
}

// GetHalfPelSearchStruct (MotionEstimatorImpl1.cpp:445-515): candidate k of
// the half-pel neighbours left inside the range at (x, y), in the reference's
// order; their number.
__device__ __forceinline__ int half_position(int x, int y, int range, int k, int* hx, int* hy)
{
    const bool r = x == range - 1, l = x == -range, b = y == range - 1, t = y == -range;
    // packed {x+1, y+1} per entry, two bits each
    auto pick = [&](unsigned tab, int len) {
        if (k < len) {
            *hx = (int)((tab >> (4 * k)) & 3u) - 1;
            *hy = (int)((tab >> (4 * k + 2)) & 3u) - 1;
        }
        return len;
    };
    if (!(r || l || b || t)) return pick(0xa9864210u, 8);  // MEI1_HalfPos
    if (!r && !l && !b && t) return pick(0xa9864u, 5);     // top edge
    if (!r && !l && b && !t) return pick(0x64210u, 5);     // bottom edge
    if (!r && l && !b && !t) return pick(0xa9621u, 5);     // left edge
    if (r && !l && !b && !t) return pick(0x98410u, 5);     // right edge
    if (!r && l && !b && t) return pick(0xa96u, 3);        // top-left
    if (r && !l && !b && t) return pick(0x984u, 3);        // top-right
    if (!r && l && b && !t) return pick(0x621u, 3);        // bottom-left
    if (r && !l && b && !t) return pick(0x410u, 3);        // bottom-right
    return pick(0xa9864210u, 8);
}

template <int BW, int BH>
__global__ void __launch_bounds__(32 * kWarps) k_impl1(Impl1Args g)
{
    __shared__ __align__(16) unsigned char smem[kWarps][kSlot];
    const FullArgs& a = g.f;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int k = blockIdx.x * kWarps + wid;
    if (k >= g.nblk) return;
    if (*((volatile int*)&a.ctrl->status) & ST_PIXEL_RANGE) return;
    unsigned char* win = smem[wid];
    unsigned* tmpl = reinterpret_cast<unsigned*>(win + kWinBytes + 16);
    const int R = g.range;
    const int n = (k % g.bcols) * BW, m = (k / g.bcols) * BH;
    // window: padded-reference rows m-R-1 .., columns from the 16-byte boundary at or left of n-R-1
    const int px = n - R - 1 + PAD, x0 = px & ~15, ox = px - x0;
    const unsigned char* src = a.refp + (size_t)(m - R - 1 + PAD) * a.rstride + x0;
    const int rows = 2 * R + BH + 2, vecs = (ox + 2 * R + BW + 2 + 15) / 16;  // the columns the search reads
    for (int v = lane; v < rows * vecs; v += 32) {
        const int r = v / vecs, c = v - r * vecs;
        *reinterpret_cast<uint4*>(win + r * kWinStride + 16 * c) =
            __ldg(reinterpret_cast<const uint4*>(src + (size_t)r * a.rstride + 16 * c));
    }
    if (lane < BH) {
        const unsigned char* s = a.src8 + (size_t)(m + lane) * a.W + n;
        if (BW == 16) *reinterpret_cast<uint4*>(tmpl + 4 * lane) = __ldg(reinterpret_cast<const uint4*>(s));
        else *reinterpret_cast<uint2*>(tmpl + 4 * lane) = __ldg(reinterpret_cast<const uint2*>(s));
    }
    __syncwarp();
    // block at offset (x, y) starts at window (ox + R + 1 + x, R + 1 + y)
    const unsigned char* base = win + (R + 1) * kWinStride + ox + R + 1;
    auto block_sd = [&](int x, int y) {
        unsigned acc = 0;
        const unsigned char* p = base + y * kWinStride + x;
#pragma unroll 4
        for (int r = 0; r < BH; r++) acc = row_sd<BW>(p + r * kWinStride, tmpl + 4 * r, acc);
        return (int)acc;
    };
    // full search: lane-strided raster candidates, the smallest (distortion, index)
    const int side = 2 * R, ncand = side * side;
    int best_d = 0x7fffffff, best_c = 0x7fffffff;
    for (int c = lane; c < ncand; c += 32) {
        const int d = block_sd(c % side - R, c / side - R);
        if (d < best_d) {  // a lane's candidates rise in index: strict keeps its first minimum
            best_d = d;
            best_c = c;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const int od = __shfl_xor_sync(0xffffffffu, best_d, o), oc = __shfl_xor_sync(0xffffffffu, best_c, o);
        if (od < best_d || (od == best_d && oc < best_c)) {
            best_d = od;
            best_c = oc;
        }
    }
    const int zero = block_sd(0, 0);  // every lane, the same value
    int min = zero, mx = 0, my = 0;
    if (best_d < zero) {
        min = best_d;
        mx = best_c % side - R;
        my = best_c / side - R;
    }
    // half pel: lane k takes neighbour k, then the reference's order of strict improvements
    int hx = 0, hy = 0;
    const int np = half_position(mx, my, R, lane, &hx, &hy);
    int hd = 0;
    if (lane < np) {
        const unsigned char* p = base + my * kWinStride + mx;
        unsigned acc = 0;
        for (int r = 0; r < BH; r++) {
            const unsigned char* q = p + r * kWinStride;
            const unsigned char* qv = q + hy * kWinStride;
#pragma unroll
            for (int w = 0; w < BW / 4; w++) {
                const unsigned s = half4(word_at(q + 4 * w), word_at(q + 4 * w + hx), word_at(qv + 4 * w),
                                         word_at(qv + 4 * w + hx), hx, hy);
                const unsigned d = __vabsdiffu4(s, tmpl[4 * r + w]);
                acc = __dp4a(d, d, acc);
            }
        }
        hd = (int)acc;
    }
    int hmx = 0, hmy = 0, last = -1;
    while (true) {
        const unsigned b = __ballot_sync(0xffffffffu, lane < np && lane > last && hd < min);
        if (!b) break;
        const int f = __ffs(b) - 1;
        min = __shfl_sync(0xffffffffu, hd, f);
        hmx = __shfl_sync(0xffffffffu, hx, f);
        hmy = __shfl_sync(0xffffffffu, hy, f);
        last = f;
    }
    if (lane == 0) {
        int mvx = 2 * mx + hmx, mvy = 2 * my + hmy;
        // the weighted choice against the zero vector (:356-378)
        const int diff = zero - min, mag = mvx * mvx + mvy * mvy;
        const int weight = ((diff >> 2) < mag) + (zero < 512) + (diff * 10 < min);
        int d = min;
        if (!(min < zero && weight < 2)) {
            mvx = mvy = 0;
            d = zero;
        }
        // the reference stores the vector as chars
        a.job->out_mv[k] = pack_mv((int)(signed char)mvx, (int)(signed char)mvy);
        if (a.job->out_dist) a.job->out_dist[k] = d;
        atomicAdd((unsigned long long*)&a.ctrl->total, (unsigned long long)d);
    }
}

__global__ void k_impl1_average(Impl1Args g)
{
    const FullArgs& a = g.f;
    if (*((volatile int*)&a.ctrl->status) & ST_PIXEL_RANGE) return;
    a.ctrl->count = g.nblk;
    if (a.job->out_avg) *a.job->out_avg = a.ctrl->total / g.nblk;  // every block, as the reference divides
}

}  // namespace

int impl1_launch(vppgpu_ctx* ctx, const FullArgs& args, int bw, int bh, int range)
{
    if (range < 1 || range > kMaxRange) return VPPGPU_ERR_UNSUPPORTED;
    Impl1Args g;
    g.f = args;
    g.bw = bw;
    g.bh = bh;
    g.bcols = args.W / bw;
    g.nblk = g.bcols * (args.H / bh);
    g.range = range;
    int rc = full_planes_launch(ctx, args);
    if (rc) return rc;
    const int grid = (g.nblk + kWarps - 1) / kWarps;
    if (bw == 16 && bh == 16) k_impl1<16, 16><<<grid, 32 * kWarps, 0, ctx->stream>>>(g);
    else if (bw == 8 && bh == 8) k_impl1<8, 8><<<grid, 32 * kWarps, 0, ctx->stream>>>(g);
    else return VPPGPU_ERR_UNSUPPORTED;
    VPP_CHECK_LAUNCH(ctx);
    k_impl1_average<<<1, 1, 0, ctx->stream>>>(g);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

}  // namespace vppgpu
