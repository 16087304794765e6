// me_cross_search.cuh -- MotionEstimatorH264ImplCross on the full-search
// estimator's planes, one warp per macroblock.
//
// Reference: MotionEstimatorH264ImplCross::Estimate
// (src/CodecUtils/MotionEstimatorH264ImplCross.cpp:354-649).  Its distortion
// is the SSD over 64 points of MEH264IC_OptimalPath (:89-98, _pathLength 64),
// compared during the search by OverlayMem2Dv2::Tsd16x16PartialPathLessThan
// with batches of 16 (OverlayMem2Dv2.cpp:2449-2493): after each batch the
// final distortion is predicted as Dp * 4 / batches-done and the first
// prediction above the running minimum is returned.  The full-pel search is
// a cross of step mRng/2, mRng/4, .., 1 around the running winner (ties to
// the point not farther from the rounded prediction), the sub-pel passes use
// the full-search estimator's window (the same LoadHalfQuartPelWindow /
// LoadQuartPelWindow / QuarterRead), GetBestVector has lambda 0.9 and norm 64.
//
// GB300 layout: lane l holds row l/2, columns 8*(l&1)..+7 of the macroblock
// as packed bytes (the planes of the full-search estimator); per-lane byte
// masks select the path points of each batch, so one candidate is two
// absolute-difference words, four masked dp4a and four warp reductions.
#pragma once

#include "me_full_common.cuh"
#include "me_mrc_search.cuh"

namespace vppgpu {
namespace cross {

constexpr int EST_CROSS = 3;
constexpr int PATH_NORM = 64;

// The first 64 points {x, y} of MEH264IC_OptimalPath.
constexpr signed char kPath[64][2] = {
    {5, 10}, {13, 5}, {2, 1},   {13, 14}, {1, 14},  {9, 1},   {1, 6},   {15, 9},  {8, 13},  {14, 2},  {7, 4},
    {10, 8}, {4, 15}, {0, 10},  {0, 3},   {5, 0},   {12, 11}, {4, 7},   {12, 0},  {10, 14}, {3, 12},  {10, 5},
    {15, 13}, {4, 3}, {7, 8},   {14, 7},  {6, 13},  {11, 3},  {2, 9},   {9, 10},  {15, 1},  {7, 2},   {3, 5},
    {8, 15}, {1, 12}, {8, 6},   {0, 1},   {12, 9},  {14, 15}, {15, 4},  {11, 12}, {6, 6},   {7, 11},  {0, 7},
    {14, 11}, {7, 0}, {2, 15},  {12, 7},  {2, 3},   {4, 9},   {12, 2},  {9, 3},   {12, 13}, {3, 0},   {5, 14},
    {5, 4},  {0, 13}, {8, 9},   {2, 11},  {11, 15}, {10, 1},  {2, 7},   {15, 6},  {9, 12}};

// Byte masks of each lane's 8 samples per batch of 16 path points.
struct alignas(16) PathMasks {
    unsigned m[32][4][2];
};

constexpr PathMasks make_path_masks()
{
    PathMasks t{};
    for (int p = 0; p < 64; p++) {
        const int x = kPath[p][0], y = kPath[p][1], lane = 2 * y + (x >> 3), b = x & 7;
        t.m[lane][p >> 4][b >> 2] |= 0xffu << (8 * (b & 3));
    }
    return t;
}

static __device__ const PathMasks c_path_masks = make_path_masks();

struct LaneMasks {
    uint2 b[4];
};

__device__ __forceinline__ LaneMasks lane_masks(int lane)
{
    const uint4* p = reinterpret_cast<const uint4*>(c_path_masks.m[lane]);
    const uint4 lo = __ldg(p), hi = __ldg(p + 1);
    LaneMasks r;
    r.b[0] = make_uint2(lo.x, lo.y);
    r.b[1] = make_uint2(lo.z, lo.w);
    r.b[2] = make_uint2(hi.x, hi.y);
    r.b[3] = make_uint2(hi.z, hi.w);
    return r;
}

// Warp-wide path SSD of each batch for this lane's samples cur / cand.
__device__ __forceinline__ void batch_sums(uint2 cur, uint2 cand, const LaneMasks& mk, int* s)
{
    const unsigned d0 = __vabsdiffu4(cur.x, cand.x), d1 = __vabsdiffu4(cur.y, cand.y);
#pragma unroll
    for (int b = 0; b < 4; b++)
        s[b] = (int)__reduce_add_sync(0xffffffffu, __dp4a(d0 & mk.b[b].x, d0, __dp4a(d1 & mk.b[b].y, d1, 0u)));
}

// Tsd16x16PartialPathLessThan(…, min, 16) from the batch sums.
__device__ __forceinline__ int path_less_than(const int* s, int min)
{
    const int d0 = s[0], d1 = d0 + s[1], d2 = d1 + s[2], d3 = d2 + s[3];
    const int e0 = d0 * 4, e1 = d1 * 2, e2 = (d2 * 4) / 3;
    return e0 > min ? e0 : (e1 > min ? e1 : (e2 > min ? e2 : d3));
}

// Full-pel plane samples of this lane at block origin (x0, y0).
__device__ __forceinline__ uint2 gplane8(const FullArgs& a, int x0, int y0, int lane)
{
    return full::load8(a.refp + (size_t)(y0 + (lane >> 1) + PAD) * a.rstride + (x0 + 8 * (lane & 1) + PAD));
}

struct CrossResult {
    int mvx, mvy, min_d, zero_d;
    bool tie;
};

// The search of macroblock (n, m); an exact tie of the full-pel cross is
// decided by skip(cx, cy, nx, ny) (true keeps the current winner (cx, cy)
// against the point (nx, ny)).  mode 0 quarter, 1 half, 2 full pel.  One
// warp; the result is warp-uniform.
template <typename Skip>
__device__ __forceinline__ CrossResult cross_search_with(const FullArgs& a, int n, int m, Skip&& skip, int lane)
{
    constexpr int CX[4] = {-1, 1, 0, 0}, CY[4] = {0, 0, -1, 1};  // MEH264IC_CrossPos
    const LaneMasks mk = lane_masks(lane);
    const uint2 cur = full::load_cur8(a, n, m, lane);
    int s[4];
    batch_sums(cur, gplane8(a, n, m, lane), mk, s);
    const int zd = s[0] + s[1] + s[2] + s[3];  // Tsd16x16PartialPath at the zero vector
    int min_d = zd, mx = 0, my = 0;
    bool tie = false;
    int xl, xr, yu, yd;
    full::full_range(n, m, a.W, a.H, a.motion_range, xl, xr, yu, yd);
    for (int step = (a.motion_range / 4) / 2; step > 0; step /= 2) {
        int sums[4][4];
        bool valid[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int i = step * CY[c], j = step * CX[c];
            valid[c] = !(i + my < yu || i + my > yd || j + mx < xl || j + mx > xr);
            if (valid[c]) batch_sums(cur, gplane8(a, n + mx + j, m + my + i, lane), mk, sums[c]);
        }
        int rmx = 0, rmy = 0;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            if (!valid[c]) continue;
            const int i = step * CY[c], j = step * CX[c];
            const int d = path_less_than(sums[c], min_d);
            if (d > min_d) continue;
            if (d == min_d) {
                tie = true;
                if (skip(mx + rmx, my + rmy, mx + j, my + i)) continue;
            }
            min_d = d;
            rmx = j;
            rmy = i;
        }
        mx += rmx;
        my += rmy;
    }
    int mvx = 4 * mx, mvy = 4 * my;
    if (a.mode != 2) {
        // the full-search estimator's sub-pel window around (n + mx, m + my)
        constexpr int SX[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
        constexpr int SY[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
        constexpr int AY[8] = {-2, -2, -2, 0, 0, 0, 2, 2}, AX[8] = {-2, 0, 0, -2, 2, -2, 0, 0};
        constexpr int BY[8] = {0, 0, 0, 0, 0, 2, 0, 0}, BX[8] = {0, 0, 2, 0, 0, 0, 0, 2};
        const int x0 = n + mx, y0 = m + my;
        int sub[8][4];
#pragma unroll
        for (int k = 0; k < 8; k++)
            batch_sums(cur, full::load8(full::even_block(a, x0, y0, 2 * SY[k], 2 * SX[k], lane)), mk, sub[k]);
        int hmx = 0, hmy = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int d = path_less_than(sub[k], min_d);
            if (d < min_d) {
                min_d = d;
                hmx = 2 * SX[k];
                hmy = 2 * SY[k];
            }
        }
        int qmx = hmx, qmy = hmy;
        if (a.mode != 1) {
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const uint2 va = full::load8(full::even_block(a, x0, y0, hmy + AY[k], hmx + AX[k], lane));
                const uint2 vb = full::load8(full::even_block(a, x0, y0, hmy + BY[k], hmx + BX[k], lane));
                batch_sums(cur, make_uint2(__vavgu4(va.x, vb.x), __vavgu4(va.y, vb.y)), mk, sub[k]);
            }
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int d = path_less_than(sub[k], min_d);
                if (d < min_d) {
                    min_d = d;
                    qmx = hmx + SX[k];
                    qmy = hmy + SY[k];
                }
            }
        }
        mvx += qmx;
        mvy += qmy;
    }
    return CrossResult{mvx, mvy, min_d, zd, tie};
}

// The search at rounded prediction (prx, pry): a tie keeps the current
// winner when it is nearer (MotionEstimatorH264ImplCross.cpp:446-456).
static __device__ __noinline__ CrossResult cross_search(const FullArgs& a, int n, int m, int prx, int pry, int lane)
{
    return cross_search_with(
        a, n, m,
        [prx, pry](int cx, int cy, int nx, int ny) {
            return (cx - prx) * (cx - prx) + (cy - pry) * (cy - pry) < (nx - prx) * (nx - prx) + (ny - pry) * (ny - pry);
        },
        lane);
}

// Tie tree run `run` of a tie macroblock (the tree of the Ver2 estimator,
// mrc::V2TieRun, at level 0): its t-th tie (t < 3) takes the point by bit t
// of run; the two vectors compared and the result are recorded.
static __device__ __noinline__ void cross_search_run(const FullArgs& a, int n, int m, int run, mrc::V2TieRun* rec,
                                                      int lane)
{
    int t = 0, geo[mrc::V2_TIE_BITS] = {0, 0, 0};
    const CrossResult r = cross_search_with(
        a, n, m,
        [&](int cx, int cy, int nx, int ny) {
            const bool take = t < mrc::V2_TIE_BITS ? ((run >> t) & 1) : true;
            if (t < mrc::V2_TIE_BITS)
                geo[t] = (cx & 0xff) | ((cy & 0xff) << 8) | ((nx & 0xff) << 16) | ((ny & 0xff) << 24);
            t++;
            return !take;
        },
        lane);
    if (lane == 0) {
        for (int e = 0; e < mrc::V2_TIE_BITS; e++) rec->geo[e] = geo[e];
        rec->lvl = 0;  // every tie at full pel
        rec->nev = t;
        rec->mv = pack_mv(r.mvx, r.mvy);
        rec->min_d = r.min_d;
    }
}

// Tsd16x16PartialPath at the prediction (QuarterRead's sixteen cases).
__device__ __forceinline__ int path_pred_distortion(const FullArgs& a, int n, int m, const full::PredGeom& g, int lane)
{
    const LaneMasks mk = lane_masks(lane);
    const uint2 cur = full::load_cur8(a, n, m, lane), cand = full::qpel_block8(a, g.ox, g.oy, g.fx, g.fy, lane);
    const unsigned d0 = __vabsdiffu4(cur.x, cand.x), d1 = __vabsdiffu4(cur.y, cand.y);
    const unsigned m0 = mk.b[0].x | mk.b[1].x | mk.b[2].x | mk.b[3].x;
    const unsigned m1 = mk.b[0].y | mk.b[1].y | mk.b[2].y | mk.b[3].y;
    return (int)__reduce_add_sync(0xffffffffu, __dp4a(d0 & m0, d0, __dp4a(d1 & m1, d1, 0u)));
}

}  // namespace cross
}  // namespace vppgpu
