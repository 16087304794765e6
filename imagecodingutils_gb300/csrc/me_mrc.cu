// me_mrc.cu -- MotionEstimatorH264ImplMultiresCross on sm_103a.
//
// Reference: MotionEstimatorH264ImplMultiresCross::Estimate
// (src/CodecUtils/MotionEstimatorH264ImplMultiresCross.cpp:525-1019).  No
// motion-vector predictor: every macroblock is independent.  Per MB: a cross
// search at level 2 (quarter resolution, mode 2), a +-2 full search (mode 2)
// or a cross search (mode 1) at level 1, a +-2 full search at level 0, the
// half- and quarter-pel stages in the estimator's own 88x88 window, and the
// accept-or-zero heuristic.  Levels 1 and 2 use PartialLessThan (16 phases on
// the stride-4 lattice, reject when 16*D_p > p*min), which is not
// decision-neutral and is reproduced phase by phase.
//
// The reference reads its extended-boundary level copies (borders 19 / 9 / 5)
// through overlays whose origins are clamped (OverlayExtMem2Dv2::SetOrigin)
// and, for the sub-pel window, past the overlay edge as flat row-major memory
// (a column beyond the row continues on the next row).  The device copies
// keep exactly that flat geometry, so the same addresses hold the same
// samples; a read outside a copy sets an error instead of reading.
//
// GB300 design
//   k_mrc_level0   input luma to bytes (0..255 check) and the border-19
//                  reference copy.
//   k_mrc_level1   2:1 decimations (OverlayMem2Dv2::Half) of input and
//                  reference, the border-9 reference copy.
//   k_mrc_level2   the second decimation (mode 2), border-5 copy.
//   k_mrc_search   one warp per macroblock.  Candidate distortions are warp
//                  reductions laid out by phase (lane pair = one phase), so
//                  the 16 phase prefix sums are a shuffle scan; candidates
//                  are tested in the reference's order against the running
//                  minimum.  The sub-pel window's lattice (G, h, b,
//                  j at 22x22 points, with the window's unwritten and
//                  unscaled edge samples) is built per warp in shared memory.
#include "me_full_common.cuh"
#include "me_internal.h"

namespace vppgpu {
namespace {

constexpr int MRC_NOISE_FLOOR = 512;

// Phase order of the partial distortion (OverlayMem2Dv2.cpp:79-80), p = 1..16.
__constant__ int kPhaseRow[17] = {0, 0, 2, 0, 2, 1, 3, 1, 3, 0, 2, 1, 3, 0, 2, 1, 3};
__constant__ int kPhaseCol[17] = {0, 0, 2, 2, 0, 1, 3, 3, 1, 1, 3, 0, 2, 3, 1, 2, 0};

struct Buf {
    const unsigned char* p;
    int w, h;  // flat row-major geometry
};

struct MrcArgs {
    int W, H, cols, nmb, rows_all, mode, motion_range;
    Buf in0, in1, in2, e0, e1, e2;
    const unsigned char* incl;
    int* out_mv;
    int* out_dist;
    long long* out_avg;
    MeCtrl* ctrl;
};

// Overlay origin (OverlayMem2Dv2::SetOrigin / OverlayExtMem2Dv2::SetOrigin):
// buffer coordinates of block (x, y), clamped so that the block fits.
struct Org {
    int x, y;
};
__device__ __forceinline__ Org origin(const Buf& b, int bw, int bh, int eb, int x, int y)
{
    x += eb;
    y += eb;
    x = x < 0 ? 0 : (x > b.w - bw ? b.w - bw : x);
    y = y < 0 ? 0 : (y > b.h - bh ? b.h - bh : y);
    return Org{x, y};
}

// Flat read, as the reference addresses its buffers.
__device__ __forceinline__ int rd(const Buf& b, int r, int c, bool& bad)
{
    const long long f = (long long)r * b.w + c;
    if (f < 0 || f >= (long long)b.w * b.h) {
        bad = true;
        return 0;
    }
    return __ldg(b.p + f);
}

// GetMotionRange of the multi-resolution estimators (…MultiresCross.cpp:1195-1262).
struct Level {
    int boundary, width, height, vec_range;
};
__device__ __forceinline__ void mr_range(const Level& L, int xpos, int ypos, int xoff, int yoff, int range, int& xl,
                                         int& xr, int& yu, int& yd)
{
    const int x = xpos + xoff, y = ypos + yoff, vr = L.vec_range;
    const int xlr = (xoff - range > -vr) ? range : (vr - 1) + xoff;
    const int xrr = (xoff + range < vr) ? range : (vr - 1) - xoff;
    const int yur = (yoff - range > -vr) ? range : (vr - 1) + yoff;
    const int ydr = (yoff + range < vr) ? range : (vr - 1) - yoff;
    xl = (x - xlr >= -L.boundary) ? -xlr : -(x + L.boundary);
    xr = (x + xrr < L.width) ? xrr : L.width - x;
    yu = (y - yur >= -L.boundary) ? -yur : -(y + L.boundary);
    yd = (y + ydr < L.height) ? ydr : L.height - y;
}

// ---------------------------------------------------------------------------
// Partial distortion of an n x n block (n = 8 or 16): lane pair 2(p-1),
// 2(p-1)+1 holds phase p; `part` is this lane's share of that phase.  Returns
// PartialLessThan's value against `min`: 16*D_p at the first phase p with
// 16*D_p > p*min (shifts wrap as the reference's int arithmetic), else D.
__device__ __forceinline__ int partial_value(int part, int min, int lane)
{
    int v = part + __shfl_xor_sync(0xffffffffu, part, 1);  // the phase sum
#pragma unroll
    for (int o = 2; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    const int p = (lane >> 1) + 1;
    const int s = (int)((unsigned)v << 4);
    const unsigned rej = __ballot_sync(0xffffffffu, (lane & 1) == 0 && s > p * min);
    if (rej) return __shfl_sync(0xffffffffu, s, __ffs(rej) - 1);
    return __shfl_sync(0xffffffffu, v, 31);
}

// This lane's samples of phase p (lane pair), half h = lane & 1: rows
// phase_row + 4*(2h + i), i < n/8; columns phase_col + 4*j, j < n/4.
template <int N>
__device__ __forceinline__ void phase_coords(int lane, int& r0, int& c0)
{
    const int p = (lane >> 1) + 1;
    r0 = kPhaseRow[p] + 4 * (N / 8) * (lane & 1);
    c0 = kPhaseCol[p];
}

// Full n x n SSD of two overlays, one warp (lane per column/row chunk).
__device__ __forceinline__ int full_ssd(const Buf& a, Org oa, const Buf& b, Org ob, int n, int lane, bool& bad)
{
    int acc = 0;
    for (int i = lane; i < n * n; i += 32) {
        const int r = i / n, c = i - r * n;
        const int d = rd(a, oa.y + r, oa.x + c, bad) - rd(b, ob.y + r, ob.x + c, bad);
        acc += d * d;
    }
    return warp_sum(acc);
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_mrc_level0(const short* __restrict__ src16, const short* __restrict__ ref16,
                                                   int W, int H, unsigned char* __restrict__ in0,
                                                   unsigned char* __restrict__ e0, int* status)
{
    const int EW = W + 38, EH = H + 38;
    const long long n_in = (long long)W * H, n_e = (long long)EW * EH;
    bool bad = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_in + n_e;
         i += (long long)gridDim.x * blockDim.x) {
        if (i < n_in) {
            const int v = src16[i];
            bad |= (v < 0) | (v > 255);
            in0[i] = (unsigned char)(v & 0xff);
        } else {
            const long long j = i - n_in;
            const int y = (int)(j / EW), x = (int)(j - (long long)y * EW);
            const int sy = min(max(y - 19, 0), H - 1), sx = min(max(x - 19, 0), W - 1);
            const int v = ref16[(size_t)sy * W + sx];
            bad |= (v < 0) | (v > 255);
            e0[j] = (unsigned char)(v & 0xff);
        }
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(status, ST_PIXEL_RANGE);
}

// 2:1 decimation (OverlayMem2Dv2::Half, OverlayMem2Dv2.cpp:3018-3033) of a
// w x h plane at (x, y).
template <typename T>
__device__ __forceinline__ int half_at(const T* p, int w, int x, int y)
{
    const T* q = p + (size_t)(2 * y) * w + 2 * x;
    return ((int)q[0] + q[1] + q[w] + q[w + 1] + 2) >> 2;
}

__global__ void __launch_bounds__(256) k_mrc_level1(const short* __restrict__ src16, const short* __restrict__ ref16,
                                                   int W, int H, unsigned char* __restrict__ in1,
                                                   unsigned char* __restrict__ e1)
{
    const int w1 = W / 2, h1 = H / 2, EW = w1 + 18, EH = h1 + 18;
    const long long n_in = (long long)w1 * h1, n_e = (long long)EW * EH;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_in + n_e;
         i += (long long)gridDim.x * blockDim.x) {
        if (i < n_in) {
            const int y = (int)(i / w1), x = (int)(i - (long long)y * w1);
            in1[i] = (unsigned char)half_at(src16, W, x, y);
        } else {
            const long long j = i - n_in;
            const int y = (int)(j / EW), x = (int)(j - (long long)y * EW);
            e1[j] = (unsigned char)half_at(ref16, W, min(max(x - 9, 0), w1 - 1), min(max(y - 9, 0), h1 - 1));
        }
    }
}

__global__ void __launch_bounds__(256) k_mrc_level2(const unsigned char* __restrict__ in1,
                                                   const unsigned char* __restrict__ e1, int W, int H,
                                                   unsigned char* __restrict__ in2, unsigned char* __restrict__ e2)
{
    const int w1 = W / 2, h1 = H / 2, w2 = w1 / 2, h2 = h1 / 2, EW = w2 + 10, EH = h2 + 10, EW1 = w1 + 18;
    const long long n_in = (long long)w2 * h2, n_e = (long long)EW * EH;
    const unsigned char* r1 = e1 + 9 * (size_t)EW1 + 9;  // level-1 reference inside its border-9 copy
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_in + n_e;
         i += (long long)gridDim.x * blockDim.x) {
        if (i < n_in) {
            const int y = (int)(i / w2), x = (int)(i - (long long)y * w2);
            in2[i] = (unsigned char)half_at(in1, w1, x, y);
        } else {
            const long long j = i - n_in;
            const int y = (int)(j / EW), x = (int)(j - (long long)y * EW);
            e2[j] = (unsigned char)half_at(r1, EW1, min(max(x - 5, 0), w2 - 1), min(max(y - 5, 0), h2 - 1));
        }
    }
}

// ---------------------------------------------------------------------------
// The sub-pel window as a lattice of 22 x 22 full-pel points (fr, fc), each
// with the four even quarter samples G (0,0), h (2,0), b (0,2), j (2,2)
// (LoadHalfQuartPelWindow, …MultiresCross.cpp:1281-1349): raw h for rows 2..18
// over all columns, raw b for all rows over columns 2..18, j from the raw h,
// then h, b scaled and G copied for rows and columns 2..18 only; every other
// sample is never written (0).
struct Lattice {
    short g[22][22], h[22][22], b[22][22], j[22][22];
};

__device__ __forceinline__ int lat(const Lattice& L, int qr, int qc)
{
    const int fr = qr >> 2, fc = qc >> 2;
    if ((qr & 3) == 0) return (qc & 3) == 0 ? L.g[fr][fc] : L.b[fr][fc];
    return (qc & 3) == 0 ? L.h[fr][fc] : L.j[fr][fc];
}

template <bool kVer2>
__device__ void build_lattice(Lattice& L, const Buf& e0, Org o, int lane, bool& bad)
{
    for (int i = lane; i < 22 * 22; i += 32) {
        const int fr = i / 22, fc = i - fr * 22;
        L.g[fr][fc] = 0;
        L.h[fr][fc] = 0;
        L.b[fr][fc] = 0;
        L.j[fr][fc] = 0;
    }
    __syncwarp();
    for (int i = lane; i < 17 * 22; i += 32) {  // raw h: rows 2..18, all columns
        const int fr = 2 + i / 22, fc = i % 22;
        const int rr = o.y + fr - 3, cc = o.x + fc - 3;
        L.h[fr][fc] = (short)tap6(rd(e0, rr - 2, cc, bad), rd(e0, rr - 1, cc, bad), rd(e0, rr, cc, bad),
                                  rd(e0, rr + 1, cc, bad), rd(e0, rr + 2, cc, bad), rd(e0, rr + 3, cc, bad));
    }
    for (int i = lane; i < 22 * 17; i += 32) {  // raw b: all rows, columns 2..18
        const int fr = i / 17, fc = 2 + i % 17;
        const int rr = o.y + fr - 3, cc = o.x + fc - 3;
        L.b[fr][fc] = (short)tap6(rd(e0, rr, cc - 2, bad), rd(e0, rr, cc - 1, bad), rd(e0, rr, cc, bad),
                                  rd(e0, rr, cc + 1, bad), rd(e0, rr, cc + 2, bad), rd(e0, rr, cc + 3, bad));
    }
    __syncwarp();
    for (int i = lane; i < 17 * 17; i += 32) {  // j from the raw h (columns fc-2 .. fc+3)
        const int fr = 2 + i / 17, fc = 2 + i % 17;
        const short* hr = L.h[fr];
        const int v = ((int)hr[fc - 2] - 5 * hr[fc - 1] + 20 * hr[fc] + 20 * hr[fc + 1] - 5 * hr[fc + 2] + hr[fc + 3] +
                       512) >> 10;
        L.j[fr][fc] = (short)clip255(v);
    }
    __syncwarp();
    for (int i = lane; i < 17 * 17; i += 32) {  // scale h and b, copy G: rows and columns 2..18
        const int fr = 2 + i / 17, fc = 2 + i % 17;
        L.h[fr][fc] = (short)clip255((L.h[fr][fc] + 16) >> 5);
        L.b[fr][fc] = (short)clip255((L.b[fr][fc] + 16) >> 5);
        L.g[fr][fc] = (short)rd(e0, o.y + fr - 3, o.x + fc - 3, bad);
    }
    if (kVer2 && lane < 18) {
        // Ver2 completes column and row 19 (…MultiresCrossVer2.cpp:2075-2093):
        // scaled h and G at column 19 of rows 2..18, scaled b and G at row 19
        // of columns 2..18, G at (19, 19)
        if (lane < 17) {
            const int f = 2 + lane;
            L.h[f][19] = (short)clip255((L.h[f][19] + 16) >> 5);
            L.g[f][19] = (short)rd(e0, o.y + f - 3, o.x + 16, bad);
            L.b[19][f] = (short)clip255((L.b[19][f] + 16) >> 5);
            L.g[19][f] = (short)rd(e0, o.y + 16, o.x + f - 3, bad);
        } else {
            L.g[19][19] = (short)rd(e0, o.y + 16, o.x + 16, bad);
        }
    }
    __syncwarp();
}

// Quarter sample at offset (sy, sx) around the even point (qr, qc), the
// assignments of LoadQuartPelWindow (…MultiresCross.cpp:1365-1389).
__device__ __forceinline__ int quarter(const Lattice& L, int qr, int qc, int sy, int sx)
{
    int a, b;
    if (sy < 0) {
        a = lat(L, qr - 2, sx < 0 ? qc - 2 : qc);
        b = sx > 0 ? lat(L, qr, qc + 2) : lat(L, qr, qc);
    } else if (sy == 0) {
        a = lat(L, qr, qc + (sx < 0 ? -2 : 2));
        b = lat(L, qr, qc);
    } else {
        a = sx < 0 ? lat(L, qr, qc - 2) : lat(L, qr + 2, qc);
        b = sx > 0 ? lat(L, qr, qc + 2) : (sx < 0 ? lat(L, qr + 2, qc) : lat(L, qr, qc));
    }
    return (a + b + 1) >> 1;
}

// ---------------------------------------------------------------------------
struct MbSearch {
    int zero_d, min_d, mvx, mvy;
    bool tie;  // an integer stage met a candidate equal to its running minimum
};

// Tie rule of the integer stages: an equal distortion replaces the current
// best (offset (rmx, rmy) from the centre (mx, my)) unless the candidate at
// (j, i) is farther from (px, py): (0, 0) for MultiresCross
// (…MultiresCross.cpp:741-746, 794, 857), the level's rounded prediction for
// Ver2 (…MultiresCrossVer2.cpp:778-786, 834-842, 906-914).
__device__ __forceinline__ bool farther(int mx, int my, int rmx, int rmy, int j, int i, int px, int py)
{
    const int cx = mx + rmx - px, cy = my + rmy - py, nx = mx + j - px, ny = my + i - py;
    return (cy * cy + cx * cx) - (ny * ny + nx * nx) < 0;
}

// The search of one macroblock, one warp, from the zero vector to the
// quarter-pel winner (…MultiresCross.cpp:612-941; …MultiresCrossVer2.cpp:643-992).
// kVer2: ties towards pl = {level-2 x, y, level-1 x, y, level-0 rounded x, y}
// of the prediction and the completed sub-pel window.
template <bool kVer2>
__device__ MbSearch search_mb(const MrcArgs& a, Lattice& LT, int mbr, int mbc, const int* pl, int lane, bool& bad)
{
    const int m = 16 * mbr, n = 16 * mbc, p = 8 * mbr, q = 8 * mbc, kk = 4 * mbr, ll = 4 * mbc;
    const int w1 = a.W / 2, h1 = a.H / 2, w2 = w1 / 2, h2 = h1 / 2;
    const int l1_range = a.motion_range / 8, l2_range = l1_range / 2;
    const int lcl_l1_range = a.mode == 2 ? 2 : l1_range;
    const Level L0{16, a.W, a.H, a.motion_range / 4}, L1{8, w1, h1, l1_range}, L2{4, w2, h2, l2_range};
    constexpr int CRX[4] = {-1, 1, 0, 0}, CRY[4] = {0, 0, -1, 1};
    constexpr int SX[8] = {-1, 0, 1, -1, 1, -1, 0, 1}, SY[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
    MbSearch out;
    out.tie = false;

    const Org oin0 = origin(a.in0, 16, 16, 0, n, m);
    out.zero_d = full_ssd(a.in0, oin0, a.e0, origin(a.e0, 16, 16, 19, n, m), 16, lane, bad);
    int mx = 0, my = 0, rmx = 0, rmy = 0, xl, xr, yu, yd;

    if (a.mode == 2) {  // level 2 cross search (…MultiresCross.cpp:639-697)
        const Org oin2 = origin(a.in2, 4, 4, 0, ll, kk);
        int min2 = full_ssd(a.in2, oin2, a.e2, origin(a.e2, 4, 4, 5, ll, kk), 4, lane, bad);
        mr_range(L2, ll, kk, 0, 0, l2_range - 1, xl, xr, yu, yd);
        for (int s = l2_range / 2; s > 0; s /= 2) {
            rmx = rmy = 0;
            for (int c = 0; c < 4; c++) {
                const int i = s * CRY[c], j = s * CRX[c];
                if (i + my < yu || i + my > yd || j + mx < xl || j + mx > xr) continue;
                // Tsd4x4LessThan stops early only on a sum already above min: a full SSD decides the same
                const int d = full_ssd(a.in2, oin2, a.e2, origin(a.e2, 4, 4, 5, j + ll + mx, i + kk + my), 4, lane, bad);
                if (d > min2) continue;
                if (d == min2) {
                    out.tie = true;
                    // MultiresCross compares the centre with the offset (…MultiresCross.cpp:673-679)
                    if (kVer2 ? farther(mx, my, rmx, rmy, j, i, pl[0], pl[1]) : (my * my + mx * mx) - (i * i + j * j) < 0)
                        continue;
                }
                min2 = d;
                rmx = j;
                rmy = i;
            }
            mx += rmx;
            my += rmy;
        }
        mx <<= 1;
        my <<= 1;
    }

    // level 1 (…MultiresCross.cpp:699-816): input samples of this lane's phase share, kept
    const int p1x = kVer2 ? pl[2] : 0, p1y = kVer2 ? pl[3] : 0;
    const Org oin1 = origin(a.in1, 8, 8, 0, q, p);
    int r1, c1;
    phase_coords<8>(lane, r1, c1);
    int cur1[2];
#pragma unroll
    for (int j = 0; j < 2; j++) cur1[j] = rd(a.in1, oin1.y + r1, oin1.x + c1 + 4 * j, bad);
    auto part8 = [&](Org o) {
        int acc = 0;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int d = cur1[j] - rd(a.e1, o.y + r1, o.x + c1 + 4 * j, bad);
            acc += d * d;
        }
        return acc;
    };
    int min1 = full_ssd(a.in1, oin1, a.e1, origin(a.e1, 8, 8, 9, mx + q, my + p), 8, lane, bad);
    rmx = rmy = 0;
    auto consider1 = [&](int i, int j) {
        const int d = partial_value(part8(origin(a.e1, 8, 8, 9, j + mx + q, i + my + p)), min1, lane);
        if (d > min1) return;
        if (d == min1) {
            out.tie = true;
            if (farther(mx, my, rmx, rmy, j, i, p1x, p1y)) return;
        }
        min1 = d;
        rmx = j;
        rmy = i;
    };
    if (a.mode == 2) {
        mr_range(L1, q, p, mx, my, lcl_l1_range, xl, xr, yu, yd);
        for (int i = yu; i <= yd; i++)
            for (int j = xl; j <= xr; j++)
                if (i || j) consider1(i, j);
    } else {
        for (int s = l1_range / 2; s > 0; s /= 2) {
            mr_range(L1, q, p, mx, my, lcl_l1_range - 1, xl, xr, yu, yd);
            rmx = rmy = 0;
            for (int c = 0; c < 4; c++) {
                const int i = s * CRY[c], j = s * CRX[c];
                if (i + my < yu || i + my > yd || j + mx < xl || j + mx > xr) continue;
                consider1(i, j);
            }
            mx += rmx;
            my += rmy;
        }
    }
    // the last level-1 refinement is added once more (…MultiresCross.cpp:815-816)
    mx = (mx + rmx) * 2;
    my = (my + rmy) * 2;

    // level 0 +-2 refinement (…MultiresCross.cpp:819-873)
    const int p0x = kVer2 ? pl[4] : 0, p0y = kVer2 ? pl[5] : 0;
    int r0, c0;
    phase_coords<16>(lane, r0, c0);
    int cur0[8];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) cur0[4 * i + j] = rd(a.in0, oin0.y + r0 + 4 * i, oin0.x + c0 + 4 * j, bad);
    auto part16 = [&](Org o) {
        int acc = 0;
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int d = cur0[4 * i + j] - rd(a.e0, o.y + r0 + 4 * i, o.x + c0 + 4 * j, bad);
                acc += d * d;
            }
        return acc;
    };
    int min_d = full_ssd(a.in0, oin0, a.e0, origin(a.e0, 16, 16, 19, n + mx, m + my), 16, lane, bad);
    rmx = rmy = 0;
    mr_range(L0, n, m, mx, my, 2, xl, xr, yu, yd);
    for (int i = yu; i <= yd; i++)
        for (int j = xl; j <= xr; j++) {
            if (!(i || j)) continue;
            const int d = partial_value(part16(origin(a.e0, 16, 16, 19, n + mx + j, m + my + i)), min_d, lane);
            if (d > min_d) continue;
            if (d == min_d) {
                out.tie = true;
                if (farther(mx, my, rmx, rmy, j, i, p0x, p0y)) continue;
            }
            min_d = d;
            rmx = j;
            rmy = i;
        }
    mx += rmx;
    my += rmy;
    int mvx = mx * 4, mvy = my * 4;

    // half then quarter pel in the estimator's window (…MultiresCross.cpp:875-941), strict improvements
    build_lattice<kVer2>(LT, a.e0, origin(a.e0, 16, 16, 19, n + mx, m + my), lane, bad);
    int hmx = 0, hmy = 0;
    for (int c = 0; c < 8; c++) {
        const int qx = 2 * SX[c], qy = 2 * SY[c];
        int acc = 0;
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int d = cur0[4 * i + j] - lat(LT, 12 + qy + 4 * (r0 + 4 * i), 12 + qx + 4 * (c0 + 4 * j));
                acc += d * d;
            }
        const int d = partial_value(acc, min_d, lane);
        if (d < min_d) {
            min_d = d;
            hmx = qx;
            hmy = qy;
        }
    }
    int qmx = hmx, qmy = hmy;
    for (int c = 0; c < 8; c++) {
        int acc = 0;
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int d = cur0[4 * i + j] -
                              quarter(LT, 12 + hmy + 4 * (r0 + 4 * i), 12 + hmx + 4 * (c0 + 4 * j), SY[c], SX[c]);
                acc += d * d;
            }
        const int d = partial_value(acc, min_d, lane);
        if (d < min_d) {
            min_d = d;
            qmx = hmx + SX[c];
            qmy = hmy + SY[c];
        }
    }
    __syncwarp();  // the lattice is reused by this warp's next search
    out.min_d = min_d;
    out.mvx = mvx + qmx;
    out.mvy = mvy + qmy;
    return out;
}

__global__ void __launch_bounds__(256) k_mrc_search(MrcArgs a)
{
    __shared__ Lattice lattice[8];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int k = blockIdx.x * 8 + wib;
    if (k >= a.cols * a.rows_all) return;
    bool bad = false;
    const int mbr = k / a.cols, mbc = k - mbr * a.cols;
    const int vec_pos = k < a.nmb ? k : a.nmb;
    const MbSearch r = search_mb<false>(a, lattice[wib], mbr, mbc, nullptr, lane, bad);
    int mvx = r.mvx, mvy = r.mvy;

    // accept-or-zero heuristic (…MultiresCross.cpp:943-999)
    int weight = 0;
    const int diff0 = r.zero_d - r.min_d, mag = mvx * mvx + mvy * mvy;
    if (diff0 < mag) weight++;
    if (r.zero_d < MRC_NOISE_FLOOR) weight++;
    if (diff0 * 10 < r.min_d) weight++;
    int chosen;
    if (r.min_d < r.zero_d && weight < 2) {
        chosen = r.min_d;
    } else {
        mvx = mvy = 0;
        chosen = r.zero_d;
    }
    const bool do_it = a.incl ? (vec_pos < a.nmb ? a.incl[vec_pos] != 0 : false) : true;
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
        if (bad) atomicOr(&a.ctrl->status, ST_OUT_OF_BOUNDS);
        if (vec_pos < a.nmb) {
            a.out_mv[vec_pos] = pack_mv(mvx, mvy);
            if (a.out_dist) a.out_dist[vec_pos] = chosen;
        }
        if (do_it) {
            atomicAdd(reinterpret_cast<unsigned long long*>(&a.ctrl->total), (unsigned long long)(long long)chosen);
            atomicAdd(&a.ctrl->count, 1);
        }
    }
}

__global__ void k_mrc_average(long long* out_avg, MeCtrl* ctrl)
{
    const long long t = ctrl->total;
    const int c = ctrl->count;
    if (out_avg) *out_avg = c ? t / c : 0;
}

// ---------------------------------------------------------------------------
// MultiresCrossVer2 (…MultiresCrossVer2.cpp:537-1151).  The search depends on
// the median prediction only through its tie rules, so every macroblock is
// searched once with the prediction (0, 0) and remembers whether a tie
// occurred; the result is the search at any prediction unless it did.  The
// rest is a function of the prediction (distortion at the prediction through
// the half-pel planes, GetBestVector with lambda 0.9) and the predictions form
// the raster-order DAG of the full-search estimator: relaxation sweeps reach
// its unique fixed point on most frames; otherwise a ticket-ordered dataflow
// pass replays the exact order.
constexpr int kV2Empty = 0x7fffffff;

struct V2Args {
    MrcArgs m;
    FullArgs f;        // byte input, padded reference and half-pel planes (distortion at the prediction)
    int4* spec;        // per MB {searched vector at prediction (0,0), its distortion, zero-vector distortion, flags}
    int* final_mv;
    int* final_dist;
    int* pred_used;    // prediction of the last evaluation, kV2Empty before the first
    int* changed;      // MBs whose vector changed, per sweep
    int* done;         // dataflow pass: MB final
    const int* slice;
    long long spin_limit;
};

constexpr int V2_TIE = 1;

__global__ void __launch_bounds__(256) k_v2_search(V2Args a)
{
    __shared__ Lattice lattice[8];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int k = blockIdx.x * 8 + wib;
    if (k >= a.m.nmb) return;
    bool bad = false;
    const int mbr = k / a.m.cols, mbc = k - mbr * a.m.cols;
    const int zero6[6] = {0, 0, 0, 0, 0, 0};
    const MbSearch r = search_mb<true>(a.m, lattice[wib], mbr, mbc, zero6, lane, bad);
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
        if (bad) atomicOr(&a.m.ctrl->status, ST_OUT_OF_BOUNDS);
        const int flags = (r.tie ? V2_TIE : 0) | neighbour_mask(a.slice, k, a.m.cols, a.m.nmb / a.m.cols);
        a.spec[k] = make_int4(pack_mv(r.mvx, r.mvy), r.min_d, r.zero_d, flags);
        a.final_mv[k] = pack_mv(r.mvx, r.mvy);
        a.pred_used[k] = kV2Empty;
    }
}

// Final vector and distortion of macroblock k at prediction (px, py), one warp.
__device__ void v2_evaluate(const V2Args& a, Lattice& LT, int k, int px, int py, int lane, int* fmv, int* fd,
                            bool& bad)
{
    const int4 s = __ldg(a.spec + k);
    const int mbr = k / a.m.cols, mbc = k - mbr * a.m.cols, n = 16 * mbc, m = 16 * mbr;
    int mvx = mv_x(s.x), mvy = mv_y(s.x), md = s.y;
    const int p0x = round_pred(px), p0y = round_pred(py);
    if ((s.w & V2_TIE) && (p0x | p0y)) {  // the searched result holds for prediction levels (0, 0) only
        const int pl[6] = {p0x / 2 / 2, p0y / 2 / 2, p0x / 2, p0y / 2, p0x, p0y};
        const MbSearch r = search_mb<true>(a.m, LT, mbr, mbc, pl, lane, bad);
        mvx = r.mvx;
        mvy = r.mvy;
        md = r.min_d;
    }
    // pred-vector check and GetBestVector (…MultiresCrossVer2.cpp:1008-1064)
    const full::PredGeom g = full::pred_geom(n, m, a.m.W, a.m.H, px, py);
    const int pd = full::plane_pred_distortion(a.f, n, m, g, lane);
    const int pos = best_of3_fast(mvx, mvy, md, g.pcx, g.pcy, pd, s.z, 0.9, g.pcx, g.pcy);
    *fmv = pos == 0 ? pack_mv(mvx, mvy) : (pos == 1 ? pack_mv(g.pcx, g.pcy) : 0);
    *fd = pos == 0 ? md : (pos == 1 ? pd : s.z);
}

// Relaxation sweep s: every MB (s = 0) or those whose prediction moved.  A
// sweep that changes nothing leaves the fixed point; later sweeps exit.
__global__ void __launch_bounds__(256) k_v2_sweep(V2Args a, int s)
{
    __shared__ Lattice lattice[8];
    if (s > 0 && __ldcg(a.changed + s - 1) == 0) return;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int k = blockIdx.x * 8 + wib;
    if (k >= a.m.nmb) return;
    const int av = __ldg(&a.spec[k].w);
    int px, py;
    median_pred(a.final_mv, av, k, a.m.cols, &px, &py);
    const int key = pack_mv(px, py);
    if (s > 0 && key == __ldcg(a.pred_used + k)) return;
    bool bad = false;
    int fmv, fd;
    v2_evaluate(a, lattice[wib], k, px, py, lane, &fmv, &fd, bad);
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
        if (bad) atomicOr(&a.m.ctrl->status, ST_OUT_OF_BOUNDS);
        a.pred_used[k] = key;
        a.final_dist[k] = fd;
        if (fmv != __ldcg(a.final_mv + k)) {
            a.final_mv[k] = fmv;
            atomicAdd(a.changed + s, 1);
        }
    }
}

// Lane 0: wait until MB j is final (bounded).
__device__ __forceinline__ void v2_wait(const V2Args& a, int j)
{
    long long spins = 0;
    while (ld_acquire(a.done + j) == 0) {
        if (++spins > a.spin_limit) {
            atomicOr(&a.m.ctrl->status, ST_TIMEOUT);
            return;
        }
        __nanosleep(32);
    }
}

// Exact raster order when the sweeps did not converge: warps take MBs in
// raster order from a ticket counter and wait for the neighbours the
// prediction reads; every earlier ticket is held by a running warp, so the
// waits end.  An MB whose prediction equals the one of its last evaluation
// keeps that result.
__global__ void __launch_bounds__(256) k_v2_wave(V2Args a, int last_sweep)
{
    __shared__ Lattice lattice[8];
    if (__ldcg(a.changed + last_sweep) == 0) return;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int cols = a.m.cols;
    for (;;) {
        int k = 0;
        if (lane == 0) k = atomicAdd(&a.m.ctrl->ticket, 1);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= a.m.nmb) return;
        const int av = __ldg(&a.spec[k].w);
        int px = 0, py = 0;
        if (lane == 0) {
            if (av & AV_A) v2_wait(a, k - 1);
            if (av & AV_B) v2_wait(a, k - cols);
            if (av & AV_C) v2_wait(a, k - cols + 1);
            else if (av & AV_D) v2_wait(a, k - cols - 1);
            median_pred(a.final_mv, av, k, cols, &px, &py);
        }
        px = __shfl_sync(0xffffffffu, px, 0);
        py = __shfl_sync(0xffffffffu, py, 0);
        const int key = pack_mv(px, py);
        if (key != __ldcg(a.pred_used + k)) {
            bool bad = false;
            int fmv, fd;
            v2_evaluate(a, lattice[wib], k, px, py, lane, &fmv, &fd, bad);
            bad = __any_sync(0xffffffffu, bad);
            if (lane == 0) {
                if (bad) atomicOr(&a.m.ctrl->status, ST_OUT_OF_BOUNDS);
                a.pred_used[k] = key;
                a.final_dist[k] = fd;
                a.final_mv[k] = fmv;
            }
        }
        __syncwarp();
        if (lane == 0) st_release(a.done + k, 1);
    }
}

__global__ void __launch_bounds__(256) k_v2_outputs(V2Args a, int sweeps)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) {  // sweeps to the fixed point, or 1000 + sweeps when the dataflow pass ran
        int s = 0;
        while (s < sweeps && __ldcg(a.changed + s) != 0) s++;
        a.m.ctrl->sweeps = s < sweeps ? s + 1 : 1000 + sweeps;
        a.m.ctrl->converged = s < sweeps;
    }
    bool inc = false;
    int d = 0;
    if (k < a.m.nmb) {
        const int v = __ldcg(a.final_mv + k);
        d = __ldcg(a.final_dist + k);
        a.m.out_mv[k] = v;
        if (a.m.out_dist) a.m.out_dist[k] = d;
        inc = a.m.incl && a.m.incl[k];
    }
    // avgDistortion counts included MBs only; none without pDistortionIncluded (…:1053-1062)
    const unsigned mask = __ballot_sync(0xffffffffu, inc);
    long long sum = inc ? d : 0;
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0 && mask) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&a.m.ctrl->total), (unsigned long long)sum);
        atomicAdd(&a.m.ctrl->count, __popc(mask));
    }
}

}  // namespace

size_t mrc_scratch_bytes(int W, int H)
{
    const size_t w1 = W / 2, h1 = H / 2, w2 = w1 / 2, h2 = h1 / 2;
    return (size_t)W * H + (size_t)(W + 38) * (H + 38) + w1 * h1 + (w1 + 18) * (h1 + 18) + w2 * h2 +
           (w2 + 10) * (h2 + 10) + 64;
}

namespace {

MrcArgs mrc_args(int W, int H, int motion_range, int mode, unsigned char* scratch)
{
    const int w1 = W / 2, h1 = H / 2, w2 = w1 / 2, h2 = h1 / 2;
    if (mode == 0) mode = (W * H > 40000) ? 2 : 1;  // SetMode(0) (…MultiresCross.cpp:501-513)
    MrcArgs a;
    a.W = W;
    a.H = H;
    a.cols = W / 16;
    a.nmb = a.cols * (H / 16);
    a.rows_all = (H + 15) / 16;
    a.mode = mode;
    a.motion_range = motion_range;
    unsigned char* p = scratch;
    unsigned char* in0 = p;
    p += (size_t)W * H;
    unsigned char* e0 = p;
    p += (size_t)(W + 38) * (H + 38);
    unsigned char* in1 = p;
    p += (size_t)w1 * h1;
    unsigned char* e1 = p;
    p += (size_t)(w1 + 18) * (h1 + 18);
    unsigned char* in2 = p;
    p += (size_t)w2 * h2;
    unsigned char* e2 = p;
    a.in0 = Buf{in0, W, H};
    a.e0 = Buf{e0, W + 38, H + 38};
    a.in1 = Buf{in1, w1, h1};
    a.e1 = Buf{e1, w1 + 18, h1 + 18};
    a.in2 = Buf{in2, w2, h2};
    a.e2 = Buf{e2, w2 + 10, h2 + 10};
    a.incl = nullptr;
    a.out_mv = nullptr;
    a.out_dist = nullptr;
    a.out_avg = nullptr;
    a.ctrl = nullptr;
    return a;
}

int levels_launch(vppgpu_ctx* ctx, const MrcArgs& a, const short* d_src16, const short* d_ref16)
{
    const int W = a.W, H = a.H, w1 = W / 2, h1 = H / 2, w2 = w1 / 2, h2 = h1 / 2;
    const int cap = ctx->sm_count * 8;
    auto grid = [&](long long work) {
        long long g = (work + 255) / 256;
        return (int)(g < cap ? g : cap);
    };
    k_mrc_level0<<<grid((long long)W * H + (long long)(W + 38) * (H + 38)), 256, 0, ctx->stream>>>(
        d_src16, d_ref16, W, H, (unsigned char*)a.in0.p, (unsigned char*)a.e0.p, &a.ctrl->status);
    VPP_CHECK_LAUNCH(ctx);
    k_mrc_level1<<<grid((long long)w1 * h1 + (long long)(w1 + 18) * (h1 + 18)), 256, 0, ctx->stream>>>(
        d_src16, d_ref16, W, H, (unsigned char*)a.in1.p, (unsigned char*)a.e1.p);
    VPP_CHECK_LAUNCH(ctx);
    if (a.mode == 2) {
        k_mrc_level2<<<grid((long long)w2 * h2 + (long long)(w2 + 10) * (h2 + 10)), 256, 0, ctx->stream>>>(
            a.in1.p, a.e1.p, W, H, (unsigned char*)a.in2.p, (unsigned char*)a.e2.p);
        VPP_CHECK_LAUNCH(ctx);
    }
    return VPPGPU_OK;
}

}  // namespace

int mrc_launch(vppgpu_ctx* ctx, int W, int H, int motion_range, int mode, const short* d_src16, const short* d_ref16,
               unsigned char* scratch, const unsigned char* incl, int* out_mv, int* out_dist, long long* out_avg,
               MeCtrl* ctrl)
{
    MrcArgs a = mrc_args(W, H, motion_range, mode, scratch);
    a.incl = incl;
    a.out_mv = out_mv;
    a.out_dist = out_dist;
    a.out_avg = out_avg;
    a.ctrl = ctrl;
    int rc = levels_launch(ctx, a, d_src16, d_ref16);
    if (rc) return rc;
    const int warps = a.cols * a.rows_all;
    k_mrc_search<<<(warps + 7) / 8, 256, 0, ctx->stream>>>(a);
    VPP_CHECK_LAUNCH(ctx);
    k_mrc_average<<<1, 1, 0, ctx->stream>>>(out_avg, ctrl);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

int mrc2_launch(vppgpu_ctx* ctx, int mode, const V2State& st, const FullArgs& planes, const short* d_src16,
                const short* d_ref16, const unsigned char* incl, const int* slice, int* out_mv, int* out_dist,
                long long* out_avg)
{
    V2Args a;
    a.m = mrc_args(planes.W, planes.H, planes.motion_range, mode, st.scratch);
    a.m.incl = incl;
    a.m.out_mv = out_mv;
    a.m.out_dist = out_dist;
    a.m.out_avg = out_avg;
    a.m.ctrl = planes.ctrl;
    a.f = planes;
    a.spec = st.spec;
    a.final_mv = st.final_mv;
    a.final_dist = st.final_dist;
    a.pred_used = st.pred_used;
    a.changed = st.changed;
    a.done = st.done;
    a.slice = slice;
    a.spin_limit = planes.spin_limit;
    int rc = full_planes_launch(ctx, planes);
    if (rc) return rc;
    if ((rc = levels_launch(ctx, a.m, d_src16, d_ref16))) return rc;
    const int nmb = a.m.nmb, blocks = (nmb + 7) / 8;
    const int sweeps = st.sweeps < 1 ? 1 : (st.sweeps > V2_SWEEPS ? V2_SWEEPS : st.sweeps);
    VPP_CUDA(cudaMemsetAsync(st.changed, 0, sizeof(int) * V2_SWEEPS, ctx->stream));
    VPP_CUDA(cudaMemsetAsync(st.done, 0, sizeof(int) * (size_t)nmb, ctx->stream));
    k_v2_search<<<blocks, 256, 0, ctx->stream>>>(a);
    VPP_CHECK_LAUNCH(ctx);
    for (int s = 0; s < sweeps; s++) {
        k_v2_sweep<<<blocks, 256, 0, ctx->stream>>>(a, s);
        VPP_CHECK_LAUNCH(ctx);
    }
    k_v2_wave<<<ctx->sm_count * 4, 256, 0, ctx->stream>>>(a, sweeps - 1);
    VPP_CHECK_LAUNCH(ctx);
    k_v2_outputs<<<(nmb + 255) / 256, 256, 0, ctx->stream>>>(a, sweeps);
    VPP_CHECK_LAUNCH(ctx);
    k_mrc_average<<<1, 1, 0, ctx->stream>>>(out_avg, planes.ctrl);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

}  // namespace vppgpu
