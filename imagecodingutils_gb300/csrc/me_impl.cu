// me_impl.cu -- MotionEstimatorImpl1::Estimate
// (src/CodecUtils/MotionEstimatorImpl1.cpp:275-395) and MotionEstimatorImpl2::Estimate
// (src/CodecUtils/MotionEstimatorImpl2.cpp:505-826) on the GPU.
//
// A full search of [-R, R-1]^2 full pels by SSD per block (16x16 or 8x8), the
// OverlayMem2Dv2::HalfRead half-pel refinement (OverlayMem2Dv2.cpp:452-596)
// over the neighbours GetHalfPelSearchStruct allows at the range's extremes
// (MotionEstimatorImpl1.cpp:445-515), and a weighted choice between the winner
// and the zero vector (:356-378).  There is no predictor, so every block is
// independent: one warp per block, its search window (rows and columns
// -R-1 .. R+B of the padded reference) and template staged in shared memory,
// one lane per candidate column.  The reference's raster scan keeps the first
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
    // full search, the smallest (distortion, raster index): lane l takes the candidate columns
    // x = -R + l (+ 32) and eight candidate rows at a time.  SSD = A^2 + B^2 - 2 sum(ab): the cross
    // terms one dp4a per four pixels, B^2 of each candidate from the energies of its window rows,
    // A^2 once per block.  Each window row is aligned once for the lane's column (funnel shifts)
    // into a ring of eight rows, its energy added to the candidates that cover it; template row r
    // then scores the eight candidates of rows y .. y+7 against ring rows y+r .. y+r+7.  Rows and
    // columns past the range are scored from bytes inside the slot and dropped.
    const int side = 2 * R;
    constexpr int WPR = BW / 4;  // words per block row
    unsigned a2u = 0u;
#pragma unroll
    for (int r = 0; r < BH; r++)
#pragma unroll
        for (int w = 0; w < WPR; w++) a2u = __dp4a(tmpl[4 * r + w], tmpl[4 * r + w], a2u);
    const int a2 = (int)a2u;
    int best_d = 0x7fffffff, best_c = 0x7fffffff;
    for (int xc = 0; xc < side; xc += 32) {
        const int x = xc + lane - R;
        const unsigned char* col = base + x;
        const unsigned* wp = reinterpret_cast<const unsigned*>(reinterpret_cast<uintptr_t>(col) & ~(uintptr_t)3);
        const unsigned sh = (unsigned)(reinterpret_cast<uintptr_t>(col) & 3) * 8;
        constexpr int kStrideW = kWinStride / 4;
        for (int yc = 0; yc < side; yc += 8) {
            const int y0 = yc - R;
            unsigned al[8][WPR], acc[8], en[8];
            // window row y0 + row at the lane's column into dst; its energy to the candidates on it
            auto load_row = [&](unsigned* dst, int row) {
                const unsigned* q = wp + (y0 + row) * kStrideW;
                unsigned e = 0u;
#pragma unroll
                for (int i = 0; i < WPR; i++) {
                    dst[i] = __funnelshift_r(q[i], q[i + 1], sh);
                    e = __dp4a(dst[i], dst[i], e);
                }
#pragma unroll
                for (int i = 0; i < 8; i++)
                    if (i <= row && row - i < BH) en[i] += e;
            };
#pragma unroll
            for (int i = 0; i < 8; i++) acc[i] = en[i] = 0u;
#pragma unroll
            for (int i = 0; i < 8; i++) load_row(al[i], i);
#pragma unroll
            for (int r0 = 0; r0 < BH; r0 += 8) {
#pragma unroll
                for (int ru = 0; ru < 8; ru++) {
                    const int r = r0 + ru;
                    unsigned t[WPR];
#pragma unroll
                    for (int i = 0; i < WPR; i++) t[i] = tmpl[4 * r + i];
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        const unsigned* B = al[(i + ru) % 8];
                        unsigned c = acc[i];
#pragma unroll
                        for (int w = 0; w < WPR; w++) c = __dp4a(t[w], B[w], c);
                        acc[i] = c;
                    }
                    if (r < BH - 1) load_row(al[ru], r + 8);  // row r is done: the ring takes row r + 8
                }
            }
            if (x < R) {
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    const int c = (yc + i) * side + (x + R), d = a2 + (int)en[i] - 2 * (int)acc[i];
                    if (yc + i < side && (d < best_d || (d == best_d && c < best_c))) {
                        best_d = d;
                        best_c = c;
                    }
                }
            }
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

// ---------------------------------------------------------------------------
// MotionEstimatorImpl2: a SAD pyramid, 16x16 blocks.  Level planes (2:1
// decimations, OverlayMem2Dv2::Half (a+b+c+d+2)>>2, of the picture and of
// level 1) with edge replication, as the reference extends each level after
// decimating it.
constexpr int kPad1 = 24, kPad2 = 12;  // >= range/2 + 1 and range/4 + 1 for ranges up to 32, plus a row word

struct Impl2Args {
    FullArgs f;
    unsigned char* r1;  // padded level-1 reference, stride s1
    unsigned char* r2;  // padded level-2 reference, stride s2
    unsigned char* i1;  // level-1 input, w1 x h1
    unsigned char* i2;  // level-2 input, w2 x h2
    int w1, h1, w2, h2, s1, s2;
    int range, mode;    // full pels; 1 two levels, 2 three levels
};

__device__ __forceinline__ int half4px(const unsigned char* p, int stride)
{
    return (p[0] + p[1] + p[stride] + p[stride + 1] + 2) >> 2;
}

// Level planes from the byte-packed picture (args.f.src8) and the padded
// level-0 reference (args.f.refp): level 1 of both, then level 2 as the
// decimation of level 1 (each level-1 value recomputed from level 0).
__global__ void __launch_bounds__(256) k_impl2_levels(Impl2Args g)
{
    const FullArgs& a = g.f;
    if (*((volatile int*)&a.ctrl->status) & ST_PIXEL_RANGE) return;
    const int P1 = g.w1 + 2 * kPad1, Q1 = g.h1 + 2 * kPad1, P2 = g.w2 + 2 * kPad2, Q2 = g.h2 + 2 * kPad2;
    const long long n1 = (long long)P1 * Q1, n2 = (long long)P2 * Q2;
    const unsigned char* r0 = a.refp + (size_t)PAD * a.rstride + PAD;  // picture origin of level 0
    auto l1ref = [&](int x, int y) { return half4px(r0 + (size_t)(2 * y) * a.rstride + 2 * x, a.rstride); };
    auto l1in = [&](int x, int y) { return half4px(a.src8 + (size_t)(2 * y) * a.W + 2 * x, a.W); };
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n1 + n2 + (long long)g.w1 * g.h1 +
                                                                             (long long)g.w2 * g.h2;
         t += (long long)gridDim.x * blockDim.x) {
        if (t < n1) {  // padded level-1 reference: edge replication of level 1
            const int x = min(max((int)(t % P1) - kPad1, 0), g.w1 - 1), y = min(max((int)(t / P1) - kPad1, 0), g.h1 - 1);
            g.r1[(size_t)(t / P1) * g.s1 + t % P1] = (unsigned char)l1ref(x, y);
        } else if (t < n1 + n2) {  // padded level-2 reference
            const long long u = t - n1;
            const int x = min(max((int)(u % P2) - kPad2, 0), g.w2 - 1), y = min(max((int)(u / P2) - kPad2, 0), g.h2 - 1);
            const int v = (l1ref(2 * x, 2 * y) + l1ref(2 * x + 1, 2 * y) + l1ref(2 * x, 2 * y + 1) +
                           l1ref(2 * x + 1, 2 * y + 1) + 2) >> 2;
            g.r2[(size_t)(u / P2) * g.s2 + u % P2] = (unsigned char)v;
        } else if (t < n1 + n2 + (long long)g.w1 * g.h1) {  // level-1 input
            const long long u = t - n1 - n2;
            g.i1[u] = (unsigned char)l1in((int)(u % g.w1), (int)(u / g.w1));
        } else {  // level-2 input
            const long long u = t - n1 - n2 - (long long)g.w1 * g.h1;
            const int x = (int)(u % g.w2), y = (int)(u / g.w2);
            g.i2[u] = (unsigned char)((l1in(2 * x, 2 * y) + l1in(2 * x + 1, 2 * y) + l1in(2 * x, 2 * y + 1) +
                                       l1in(2 * x + 1, 2 * y + 1) + 2) >> 2);
        }
    }
}

// SAD of an n x n block of a global plane (any alignment) against a template
// held as n rows of n/4 words in shared memory, by one lane.
template <int N>
__device__ __forceinline__ int lane_sad(const unsigned char* p, int stride, const unsigned* t)
{
    const unsigned sh = (unsigned)(reinterpret_cast<uintptr_t>(p) & 3) * 8;
    const unsigned* w = reinterpret_cast<const unsigned*>(reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)3);
    unsigned acc = 0;
#pragma unroll 4
    for (int r = 0; r < N; r++) {
        const unsigned* q = reinterpret_cast<const unsigned*>(reinterpret_cast<const unsigned char*>(w) +
                                                              (size_t)r * stride);
        unsigned prev = __ldg(q);
#pragma unroll
        for (int k = 0; k < N / 4; k++) {
            const unsigned nxt = __ldg(q + k + 1);
            acc = __vsadu4(__funnelshift_r(prev, nxt, sh), t[r * (N / 4) + k]) + acc;
            prev = nxt;
        }
    }
    return (int)acc;
}

// One level of MotionEstimatorImpl2 (:585-743), one warp: the centre's SAD,
// then candidates (j, i) in [-r, r]^2 \ (0, 0) in raster order, lane per
// candidate; a candidate is taken when below the running minimum, or equal
// to it and its vector (centre + offset) not farther from the origin than the
// running best's (a ballot walk applies them in order).
template <int N>
__device__ __forceinline__ int impl2_level(const unsigned char* at, int stride, const unsigned* tmpl, int cx, int cy,
                                           int r, int lane, int* rx, int* ry)
{
    int min = lane_sad<N>(at + (ptrdiff_t)cy * stride + cx, stride, tmpl);
    int bx = 0, by = 0;
    const int side = 2 * r + 1, total = side * side;
    for (int base = 0; base < total; base += 32) {
        const int c = base + lane, i = c / side - r, j = c % side - r;
        const bool v = c < total && (i || j);
        const int d = v ? lane_sad<N>(at + (ptrdiff_t)(cy + i) * stride + cx + j, stride, tmpl) : 0;
        const int nd = (cy + i) * (cy + i) + (cx + j) * (cx + j);
        int last = -1;
        while (true) {
            const int bd = (cy + by) * (cy + by) + (cx + bx) * (cx + bx);
            const unsigned m = __ballot_sync(0xffffffffu, v && lane > last && (d < min || (d == min && nd <= bd)));
            if (!m) break;
            const int f = __ffs(m) - 1;
            min = __shfl_sync(0xffffffffu, d, f);
            bx = __shfl_sync(0xffffffffu, j, f);
            by = __shfl_sync(0xffffffffu, i, f);
            last = f;
        }
    }
    *rx = bx;
    *ry = by;
    return min;
}

__device__ __forceinline__ int impl2_clamp(int v, int range)
{
    if (v + 2 >= range) return range - 1 - 2;
    if (v - 2 < -range) return -(range - 2);
    return v;
}

__global__ void __launch_bounds__(128) k_impl2(Impl2Args g)
{
    __shared__ unsigned tmpl[4][64 + 16 + 4];  // level-0, level-1, level-2 templates per warp
    const FullArgs& a = g.f;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int cols = a.W / 16, nmb = cols * (a.H / 16);
    const int k = blockIdx.x * 4 + wid;
    if (k >= nmb) return;
    if (*((volatile int*)&a.ctrl->status) & ST_PIXEL_RANGE) return;
    const int n = (k % cols) * 16, m = (k / cols) * 16;
    unsigned* t0 = tmpl[wid];
    unsigned* t1 = t0 + 64;
    unsigned* t2 = t1 + 16;
    if (lane < 16) *reinterpret_cast<uint4*>(t0 + 4 * lane) =
        __ldg(reinterpret_cast<const uint4*>(a.src8 + (size_t)(m + lane) * a.W + n));
    else if (lane < 24) *reinterpret_cast<uint2*>(t1 + 2 * (lane - 16)) =
        __ldg(reinterpret_cast<const uint2*>(g.i1 + (size_t)(m / 2 + lane - 16) * g.w1 + n / 2));
    else if (lane < 28) t2[lane - 24] = __ldg(reinterpret_cast<const unsigned*>(g.i2 + (size_t)(m / 4 + lane - 24) * g.w2 + n / 4));
    __syncwarp();
    const int R = g.range, r1 = R / 2, r2 = r1 / 2;
    const unsigned char* at0 = a.refp + (size_t)(m + PAD) * a.rstride + n + PAD;
    const int zero = lane_sad<16>(at0, a.rstride, t0);
    int mx = 0, my = 0, rx, ry;
    if (g.mode == 2) {  // level 2: the full range (:585-631)
        const unsigned char* at2 = g.r2 + (size_t)(m / 4 + kPad2) * g.s2 + n / 4 + kPad2;
        impl2_level<4>(at2, g.s2, t2, 0, 0, r2, lane, &rx, &ry);
        mx = impl2_clamp(2 * rx, r1);
        my = impl2_clamp(2 * ry, r1);
    }
    // level 1: the full range, or +-2 around the level-2 result (:648-684)
    const unsigned char* at1 = g.r1 + (size_t)(m / 2 + kPad1) * g.s1 + n / 2 + kPad1;
    impl2_level<8>(at1, g.s1, t1, mx, my, g.mode == 2 ? 2 : r1, lane, &rx, &ry);
    mx = impl2_clamp((mx + rx) * 2, R);
    my = impl2_clamp((my + ry) * 2, R);
    // level 0: +-2 (:697-729)
    int min = impl2_level<16>(at0, a.rstride, t0, mx, my, 2, lane, &rx, &ry);
    mx += rx;
    my += ry;
    // half pel: HalfRead at the neighbours the range leaves, SAD, strict improvement (:731-746)
    int hx = 0, hy = 0;
    const int np = half_position(mx, my, R, lane, &hx, &hy);
    int hd = 0;
    if (lane < np) {
        const unsigned char* p = at0 + (ptrdiff_t)my * a.rstride + mx;
        unsigned acc = 0;
        for (int r = 0; r < 16; r++) {
            const unsigned char* q = p + (size_t)r * a.rstride;
            const unsigned char* qv = q + (ptrdiff_t)hy * a.rstride;
            for (int w = 0; w < 4; w++) {
                auto word = [](const unsigned char* b) {
                    return (unsigned)b[0] | ((unsigned)b[1] << 8) | ((unsigned)b[2] << 16) | ((unsigned)b[3] << 24);
                };
                const unsigned s = half4(word(q + 4 * w), word(q + 4 * w + hx), word(qv + 4 * w),
                                         word(qv + 4 * w + hx), hx, hy);
                acc = __vsadu4(s, t0[4 * r + w]) + acc;
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
        // the weighted choice against the zero vector (:752-774)
        const int diff = zero - min, mag = mvx * mvx + mvy * mvy;
        const int weight = ((diff >> 1) < mag) + (zero < 26) + (diff * 7 < min);
        int d = min;
        if (!(min < zero && weight < 2)) {
            mvx = mvy = 0;
            d = zero;
        }
        a.job->out_mv[k] = pack_mv((int)(signed char)mvx, (int)(signed char)mvy);
        if (a.job->out_dist) a.job->out_dist[k] = d;
        atomicAdd((unsigned long long*)&a.ctrl->total, (unsigned long long)d);
    }
}

__global__ void k_impl2_average(Impl2Args g)
{
    const FullArgs& a = g.f;
    if (*((volatile int*)&a.ctrl->status) & ST_PIXEL_RANGE) return;
    const int nmb = (a.W / 16) * (a.H / 16);
    a.ctrl->count = nmb;
    if (a.job->out_avg) *a.job->out_avg = a.ctrl->total / nmb;
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

size_t impl2_scratch_bytes(int W, int H)
{
    const int w1 = W / 2, h1 = H / 2, w2 = w1 / 2, h2 = h1 / 2;
    const size_t s1 = (size_t)((w1 + 2 * kPad1 + 15) & ~15), s2 = (size_t)((w2 + 2 * kPad2 + 15) & ~15);
    return s1 * (h1 + 2 * kPad1) + s2 * (h2 + 2 * kPad2) + (size_t)w1 * h1 + (size_t)w2 * h2 + 64;
}

int impl2_launch(vppgpu_ctx* ctx, const FullArgs& args, unsigned char* scratch, int range, int mode)
{
    if (range < 4 || range > kMaxRange) return VPPGPU_ERR_UNSUPPORTED;
    Impl2Args g;
    g.f = args;
    g.w1 = args.W / 2;
    g.h1 = args.H / 2;
    g.w2 = g.w1 / 2;
    g.h2 = g.h1 / 2;
    g.s1 = (g.w1 + 2 * kPad1 + 15) & ~15;
    g.s2 = (g.w2 + 2 * kPad2 + 15) & ~15;
    g.r1 = scratch;
    g.r2 = g.r1 + (size_t)g.s1 * (g.h1 + 2 * kPad1);
    g.i1 = g.r2 + (size_t)g.s2 * (g.h2 + 2 * kPad2);
    g.i2 = g.i1 + (size_t)g.w1 * g.h1;
    g.range = range;
    g.mode = mode;
    int rc = full_planes_launch(ctx, args);
    if (rc) return rc;
    const long long work = (long long)(g.w1 + 2 * kPad1) * (g.h1 + 2 * kPad1) +
                           (long long)(g.w2 + 2 * kPad2) * (g.h2 + 2 * kPad2) + (long long)g.w1 * g.h1 +
                           (long long)g.w2 * g.h2;
    const long long blocks = (work + 255) / 256;
    k_impl2_levels<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, ctx->stream>>>(g);
    VPP_CHECK_LAUNCH(ctx);
    const int nmb = (args.W / 16) * (args.H / 16);
    k_impl2<<<(nmb + 3) / 4, 128, 0, ctx->stream>>>(g);
    VPP_CHECK_LAUNCH(ctx);
    k_impl2_average<<<1, 1, 0, ctx->stream>>>(g);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

}  // namespace vppgpu
