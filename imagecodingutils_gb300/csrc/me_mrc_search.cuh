// me_mrc_search.cuh -- the macroblock search of the multi-resolution H.264
// estimators, shared by MotionEstimatorH264ImplMultiresCross and
// MotionEstimatorH264ImplMultiresCrossVer2 (me_mrc.cu) and by the
// prediction-dependent resolve (me_full_resolve.cu), which searches a
// Ver2 macroblock again when a tie makes its search depend on the prediction.
//
// The reference reads its extended-boundary level copies (borders 19 / 9 / 5)
// through overlays whose origins are clamped (OverlayExtMem2Dv2::SetOrigin)
// and, for the sub-pel window, past the overlay edge as flat row-major memory
// (a column beyond the row continues on the next row).  The device copies
// keep exactly that flat geometry, so the same addresses hold the same
// samples; a read outside a copy sets an error instead of reading.
#pragma once

#include "me_common.cuh"
#include "me_internal.h"

namespace vppgpu {
namespace mrc {
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
    double lambda;  // MultiresCrossVer2's Lagrangian overload: its lambda
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
    // level copies hold fewer than 2^31 samples; reads stay within a few rows of a
    // copy, so the flat index cannot overflow and a negative one compares as huge
    const unsigned f = (unsigned)(r * b.w + c);
    if (f >= (unsigned)(b.w * b.h)) {
        bad = true;
        return 0;
    }
    return __ldg(b.p + f);
}

// A read inside a block that origin() placed in its buffer (every row and column of the block lies
// within the copy, as the clamp guarantees): no check needed.
__device__ __forceinline__ int rdb(const Buf& b, int r, int c) { return __ldg(b.p + (size_t)r * b.w + c); }

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

// Full n x n SSD of two overlays placed by origin(), one warp (lane per column/row chunk).
__device__ __forceinline__ int full_ssd(const Buf& a, Org oa, const Buf& b, Org ob, int n, int lane, bool& bad)
{
    (void)bad;  // both blocks lie inside their copies
    int acc = 0;
    for (int i = lane; i < n * n; i += 32) {
        const int r = i / n, c = i - r * n;
        const int d = rdb(a, oa.y + r, oa.x + c) - rdb(b, ob.y + r, ob.x + c);
        acc += d * d;
    }
    return warp_sum(acc);
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
constexpr int TIE_L2 = 1, TIE_L1 = 2, TIE_L0 = 4;


// A search decides ties only with the prediction's vectors at the levels
// where its own trajectory met them, so a search made for prediction
// (ex, ey) whose trajectory tied at levels `tie` has the same trajectory, and
// result, for every prediction with the same vectors at those levels.
__device__ __forceinline__ int level_pred(int est, int p, int lvl);
__device__ __forceinline__ bool search_reusable(int est, int tie, int ex, int ey, int px, int py)
{
    for (int l = 0; l < 3; l++)
        if ((tie & (TIE_L0 >> l)) &&
            (level_pred(est, ex, l) != level_pred(est, px, l) || level_pred(est, ey, l) != level_pred(est, py, l)))
            return false;
    return true;
}

struct MbSearch {
    int zero_d, min_d, mvx, mvy;
    int tie;  // integer stages that met a candidate equal to their running minimum: TIE_L2 | TIE_L1 | TIE_L0
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
// kVer2: the completed sub-pel window.  skip(level, mx, my, rmx, rmy, j, i)
// decides an exact tie at an integer level: true keeps the current best
// (offset (rmx, rmy) from the centre (mx, my)), false takes the candidate at
// offset (j, i).  It is called with the same arguments in every lane.
template <bool kVer2, typename Skip, bool kH263 = false>
__device__ MbSearch search_mb_with(const MrcArgs& a, Lattice& LT, int mbr, int mbc, Skip&& skip, int lane, bool& bad)
{
    const int m = 16 * mbr, n = 16 * mbc, p = 8 * mbr, q = 8 * mbc, kk = 4 * mbr, ll = 4 * mbc;
    const int w1 = a.W / 2, h1 = a.H / 2, w2 = w1 / 2, h2 = h1 / 2;
    const int l1_range = a.motion_range / 8, l2_range = l1_range / 2;
    const int lcl_l1_range = a.mode == 2 ? 2 : l1_range;
    const Level L0{16, a.W, a.H, a.motion_range / 4}, L1{8, w1, h1, l1_range}, L2{4, w2, h2, l2_range};
    constexpr int CRX[4] = {-1, 1, 0, 0}, CRY[4] = {0, 0, -1, 1};
    constexpr int SX[8] = {-1, 0, 1, -1, 1, -1, 0, 1}, SY[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
    MbSearch out;
    out.tie = 0;

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
                    out.tie |= TIE_L2;
                    if (skip(2, mx, my, rmx, rmy, j, i)) continue;
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
    const Org oin1 = origin(a.in1, 8, 8, 0, q, p);
    int r1, c1;
    phase_coords<8>(lane, r1, c1);
    int cur1[2];
#pragma unroll
    for (int j = 0; j < 2; j++) cur1[j] = rdb(a.in1, oin1.y + r1, oin1.x + c1 + 4 * j);
    auto part8 = [&](Org o) {
        int acc = 0;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int d = cur1[j] - rdb(a.e1, o.y + r1, o.x + c1 + 4 * j);
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
            out.tie |= TIE_L1;
            if (skip(1, mx, my, rmx, rmy, j, i)) return;
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
    int r0, c0;
    phase_coords<16>(lane, r0, c0);
    int cur0[8];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) cur0[4 * i + j] = rdb(a.in0, oin0.y + r0 + 4 * i, oin0.x + c0 + 4 * j);
    auto part16 = [&](Org o) {
        int acc = 0;
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int d = cur0[4 * i + j] - rdb(a.e0, o.y + r0 + 4 * i, o.x + c0 + 4 * j);
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
                out.tie |= TIE_L0;
                if (skip(0, mx, my, rmx, rmy, j, i)) continue;
            }
            min_d = d;
            rmx = j;
            rmy = i;
        }
    mx += rmx;
    my += rmy;
    if constexpr (kH263) {
        // MotionEstimatorH263ImplMultiresCross (…H263ImplMultiresCross.cpp:885-940): the best of the
        // four diagonal half-pel corners, then the two points beside the winning corner (the full cross
        // if no corner won), each an OverlayMem2Dv2::HalfRead block (bilinear, +2 >> 2 diagonal, +1 >> 1
        // linear; the left neighbour for -1) of the level-0 reference, strict improvements; half pels.
        // Every sample read lies within 17 of the picture, where the border-19 copy holds the same edge
        // replication as the reference's border-17 one.
        constexpr int CX4[4] = {-1, 1, -1, 1}, CY4[4] = {-1, -1, 1, 1};
        constexpr int RX[4][2] = {{0, -1}, {0, 1}, {0, -1}, {0, 1}}, RY[4][2] = {{-1, 0}, {-1, 0}, {1, 0}, {1, 0}};
        const Org o = origin(a.e0, 16, 16, 19, n + mx, m + my);
        auto half_part = [&](int hx, int hy) {
            int acc = 0;
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int r = o.y + r0 + 4 * i, c = o.x + c0 + 4 * j + (hx < 0 ? -1 : 0);
                    int v;
                    if (hx && hy)
                        v = (rd(a.e0, r, c, bad) + rd(a.e0, r + hy, c, bad) + rd(a.e0, r, c + 1, bad) +
                             rd(a.e0, r + hy, c + 1, bad) + 2) >> 2;
                    else if (hx)
                        v = (rd(a.e0, r, c, bad) + rd(a.e0, r, c + 1, bad) + 1) >> 1;
                    else
                        v = (rd(a.e0, r, c, bad) + rd(a.e0, r + hy, c, bad) + 1) >> 1;
                    const int d = cur0[4 * i + j] - v;
                    acc += d * d;
                }
            return acc;
        };
        int hmx = 0, hmy = 0, best_corner = 0;
        for (int k = 0; k < 4; k++) {
            const int d = partial_value(half_part(CX4[k], CY4[k]), min_d, lane);
            if (d < min_d) {
                best_corner = k;
                min_d = d;
                hmx = CX4[k];
                hmy = CY4[k];
            }
        }
        const bool won = hmx || hmy;
        for (int k = 0; k < (won ? 2 : 4); k++) {
            const int hx = won ? RX[best_corner][k] : CRX[k], hy = won ? RY[best_corner][k] : CRY[k];
            const int d = partial_value(half_part(hx, hy), min_d, lane);
            if (d < min_d) {
                min_d = d;
                hmx = hx;
                hmy = hy;
            }
        }
        out.min_d = min_d;
        out.mvx = 2 * mx + hmx;
        out.mvy = 2 * my + hmy;
        return out;
    }
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

// The search of MotionEstimatorH264ImplMultires (…Multires.cpp:644-906): full
// searches at level 2 (+-(range/16 - 1)) and level 1 (+-2 after level 2, else
// +-range/8), +-2 at level 0, half and quarter pel in the MultiresCross-style
// window; LessThan distortions, which decide exactly as full SSDs do.  The
// warp scores candidates in raster order: level 0 and 1 one candidate at a
// time, each lane holding a fixed share of the input block; level 2 (4x4)
// two at a time, one per half-warp.
template <typename Skip>
__device__ MbSearch search_mr_with(const MrcArgs& a, Lattice& LT, int mbr, int mbc, Skip&& skip, int lane, bool& bad)
{
    const int m = 16 * mbr, n = 16 * mbc, p = 8 * mbr, q = 8 * mbc, kk = 4 * mbr, ll = 4 * mbc;
    const int w1 = a.W / 2, h1 = a.H / 2, w2 = w1 / 2, h2 = h1 / 2;
    const int l1_range = a.motion_range / 8, l2_range = l1_range / 2;
    const int lcl_l1_range = a.mode == 2 ? 2 : l1_range;
    const Level L0{16, a.W, a.H, a.motion_range / 4}, L1{8, w1, h1, l1_range}, L2{4, w2, h2, l2_range};
    constexpr int SX[8] = {-1, 0, 1, -1, 1, -1, 0, 1}, SY[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
    MbSearch out;
    out.tie = 0;
    const Org oin0 = origin(a.in0, 16, 16, 0, n, m);
    out.zero_d = full_ssd(a.in0, oin0, a.e0, origin(a.e0, 16, 16, 19, n, m), 16, lane, bad);
    int mx = 0, my = 0, xl, xr, yu, yd;

    if (a.mode == 2) {  // level 2 full search around (0, 0) (…Multires.cpp:667-731)
        // 8 candidates of a row at a time, 4 lanes each (one block row per lane)
        const Org oin2 = origin(a.in2, 4, 4, 0, ll, kk);
        const int sub = lane >> 2, br = lane & 3;
        int cur2[4];
#pragma unroll
        for (int c = 0; c < 4; c++) cur2[c] = rdb(a.in2, oin2.y + br, oin2.x + c);
        int min2 = full_ssd(a.in2, oin2, a.e2, origin(a.e2, 4, 4, 5, ll, kk), 4, lane, bad);
        mr_range(L2, ll, kk, 0, 0, l2_range - 1, xl, xr, yu, yd);
        for (int i = yu; i <= yd; i++)
            for (int j0 = xl; j0 <= xr; j0 += 8) {
                int d = 0;
                if (j0 + sub <= xr) {
                    const Org o = origin(a.e2, 4, 4, 5, ll + j0 + sub, kk + i);
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        const int e = cur2[c] - rdb(a.e2, o.y + br, o.x + c);
                        d += e * e;
                    }
                }
                d += __shfl_xor_sync(0xffffffffu, d, 1);
                d += __shfl_xor_sync(0xffffffffu, d, 2);
                const int nj = xr - j0 + 1 < 8 ? xr - j0 + 1 : 8;
                for (int t = 0; t < nj; t++) {
                    const int j = j0 + t, dt = __shfl_sync(0xffffffffu, d, 4 * t);
                    if (!(i || j) || dt > min2) continue;
                    if (dt == min2) {
                        out.tie |= TIE_L2;
                        if (skip(2, 0, 0, mx, my, j, i)) continue;
                    }
                    min2 = dt;
                    mx = j;
                    my = i;
                }
            }
        mx <<= 1;
        my <<= 1;
    }

    // level 1 around (mx, my) (…Multires.cpp:735-790): this lane's 2 samples of the 8x8 block
    const Org oin1 = origin(a.in1, 8, 8, 0, q, p);
    int r1, c1;
    phase_coords<8>(lane, r1, c1);
    int cur1[2];
#pragma unroll
    for (int j = 0; j < 2; j++) cur1[j] = rdb(a.in1, oin1.y + r1, oin1.x + c1 + 4 * j);
    int min1 = full_ssd(a.in1, oin1, a.e1, origin(a.e1, 8, 8, 9, mx + q, my + p), 8, lane, bad);
    int rmx = 0, rmy = 0;
    mr_range(L1, q, p, mx, my, lcl_l1_range, xl, xr, yu, yd);
    for (int i = yu; i <= yd; i++)
        for (int j = xl; j <= xr; j++) {
            if (!(i || j)) continue;
            const Org o = origin(a.e1, 8, 8, 9, j + mx + q, i + my + p);
            int acc = 0;
#pragma unroll
            for (int t = 0; t < 2; t++) {
                const int e = cur1[t] - rdb(a.e1, o.y + r1, o.x + c1 + 4 * t);
                acc += e * e;
            }
            const int d = warp_sum(acc);
            if (d > min1) continue;
            if (d == min1) {
                out.tie |= TIE_L1;
                if (skip(1, mx, my, rmx, rmy, j, i)) continue;
            }
            min1 = d;
            rmx = j;
            rmy = i;
        }
    mx = (mx + rmx) * 2;
    my = (my + rmy) * 2;

    // level 0 +-2 (…Multires.cpp:792-849): this lane's 8 samples of the 16x16 block
    int r0, c0;
    phase_coords<16>(lane, r0, c0);
    int cur0[8];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) cur0[4 * i + j] = rdb(a.in0, oin0.y + r0 + 4 * i, oin0.x + c0 + 4 * j);
    auto ssd16 = [&](Org o) {
        int acc = 0;
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int e = cur0[4 * i + j] - rdb(a.e0, o.y + r0 + 4 * i, o.x + c0 + 4 * j);
                acc += e * e;
            }
        return warp_sum(acc);
    };
    int min_d = ssd16(origin(a.e0, 16, 16, 19, n + mx, m + my));
    rmx = rmy = 0;
    mr_range(L0, n, m, mx, my, 2, xl, xr, yu, yd);
    for (int i = yu; i <= yd; i++)
        for (int j = xl; j <= xr; j++) {
            if (!(i || j)) continue;
            const int d = ssd16(origin(a.e0, 16, 16, 19, n + mx + j, m + my + i));
            if (d > min_d) continue;
            if (d == min_d) {
                out.tie |= TIE_L0;
                if (skip(0, mx, my, rmx, rmy, j, i)) continue;
            }
            min_d = d;
            rmx = j;
            rmy = i;
        }
    mx += rmx;
    my += rmy;
    int mvx = mx * 4, mvy = my * 4;

    // half then quarter pel (…Multires.cpp:851-917), strict improvements, full distortions
    build_lattice<false>(LT, a.e0, origin(a.e0, 16, 16, 19, n + mx, m + my), lane, bad);
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
        const int d = warp_sum(acc);
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
        const int d = warp_sum(acc);
        if (d < min_d) {
            min_d = d;
            qmx = hmx + SX[c];
            qmy = hmy + SY[c];
        }
    }
    __syncwarp();
    out.min_d = min_d;
    out.mvx = mvx + qmx;
    out.mvy = mvy + qmy;
    return out;
}

// ---------------------------------------------------------------------------
// MultiresCrossVer2::Estimate(long*, void* lambda): every search level keeps
// its improvements in a five-slot list (Fifo(5) of include/GeneralUtils/Fifo.h,
// newest in slot 0; the first item after a reset fills every slot) and ends
// with GetBestVector over it.  Lane i < 5 of the searching warp holds slot i.
struct Fifo5 {
    int x, y, d;
    __device__ __forceinline__ void reset(int vx, int vy, int vd)
    {
        x = vx;
        y = vy;
        d = vd;
    }
    __device__ __forceinline__ void push(int vx, int vy, int vd, int lane)
    {
        x = __shfl_up_sync(0xffffffffu, x, 1);
        y = __shfl_up_sync(0xffffffffu, y, 1);
        d = __shfl_up_sync(0xffffffffu, d, 1);
        if (lane == 0) {
            x = vx;
            y = vy;
            d = vd;
        }
    }
};

// GetBestVector (include/CodecUtils/MotionEstimatorH264ImplMultiresCrossVer2.h:168-197):
// cost D/norm + lambda*sqrt(|v - ref|^2) in IEEE double, one rounding per
// operation as the reference's expression; slot 0 is costed at the current
// vector (mx, my) with lambda * 2^(level+2) / 16, slots 1..4 with the raw
// lambda; the slots in order, strict improvement.  Lanes 0..4 cost their slot
// at once.  Sets (mx, my) and returns the winning slot's distortion.
__device__ __forceinline__ int fifo_best(const Fifo5& f, double lambda, double norm, int level, int xr, int yr,
                                         int& mx, int& my, int lane)
{
    const double l = lane == 0 ? __ddiv_rn(__dmul_rn(lambda, (double)(1 << (level + 2))), 16.0) : lambda;
    const int vx = lane == 0 ? mx : f.x, vy = lane == 0 ? my : f.y;
    const double m2 = (double)((vx - xr) * (vx - xr) + (vy - yr) * (vy - yr));
    const double c = __dadd_rn(__ddiv_rn((double)f.d, norm), __dmul_rn(l, __dsqrt_rn(m2)));
    double best = __shfl_sync(0xffffffffu, c, 0);
    int bi = 0;
#pragma unroll
    for (int i = 1; i < 5; i++) {
        const double ci = __shfl_sync(0xffffffffu, c, i);
        if (ci < best) {
            best = ci;
            bi = i;
        }
    }
    const int nx = __shfl_sync(0xffffffffu, f.x, bi), ny = __shfl_sync(0xffffffffu, f.y, bi);
    if (bi) {
        mx = nx;
        my = ny;
    }
    return __shfl_sync(0xffffffffu, f.d, bi);
}

constexpr int TIE_ALL = TIE_L2 | TIE_L1 | TIE_L0;

// The search of the Lagrangian overload (…MultiresCrossVer2.cpp:1237-1676),
// one warp: the Ver2 search with GetBestVector towards the prediction's
// vector of each level (pl[2l], pl[2l+1]: level l's x, y, level 0 rounded;
// norms 16, 64, 256 at levels 2, 1, 0), at the end of the sub-pel stages towards the clamped
// quarter-pel prediction (pcx, pcy).  Unlike Estimate(long*), the cross mode
// adds its last level-1 refinement once only (…:1434-1499), and level 0
// continues from the list's choice.  Every result depends on the prediction:
// tie = TIE_ALL.
__device__ MbSearch search_lambda(const MrcArgs& a, Lattice& LT, int mbr, int mbc, const int* pl, int pcx, int pcy,
                                  int lane, bool& bad)
{
    const int m = 16 * mbr, n = 16 * mbc, p = 8 * mbr, q = 8 * mbc, kk = 4 * mbr, ll = 4 * mbc;
    const int w1 = a.W / 2, h1 = a.H / 2, w2 = w1 / 2, h2 = h1 / 2;
    const int l1_range = a.motion_range / 8, l2_range = l1_range / 2;
    const int lcl_l1_range = a.mode == 2 ? 2 : l1_range;
    const Level L0{16, a.W, a.H, a.motion_range / 4}, L1{8, w1, h1, l1_range}, L2{4, w2, h2, l2_range};
    constexpr int CRX[4] = {-1, 1, 0, 0}, CRY[4] = {0, 0, -1, 1};
    constexpr int SX[8] = {-1, 0, 1, -1, 1, -1, 0, 1}, SY[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
    const double lam = a.lambda;
    MbSearch out;
    out.tie = TIE_ALL;
    Fifo5 f;

    const Org oin0 = origin(a.in0, 16, 16, 0, n, m);
    out.zero_d = full_ssd(a.in0, oin0, a.e0, origin(a.e0, 16, 16, 19, n, m), 16, lane, bad);
    int mx = 0, my = 0, rmx = 0, rmy = 0, xl, xr, yu, yd;

    if (a.mode == 2) {  // level 2 cross search (…:1287-1370)
        const Org oin2 = origin(a.in2, 4, 4, 0, ll, kk);
        int min2 = full_ssd(a.in2, oin2, a.e2, origin(a.e2, 4, 4, 5, ll, kk), 4, lane, bad);
        f.reset(0, 0, min2);
        mr_range(L2, ll, kk, 0, 0, l2_range - 1, xl, xr, yu, yd);
        for (int s = l2_range / 2; s > 0; s /= 2) {
            rmx = rmy = 0;
            for (int c = 0; c < 4; c++) {
                const int i = s * CRY[c], j = s * CRX[c];
                if (i + my < yu || i + my > yd || j + mx < xl || j + mx > xr) continue;
                // Tsd4x4LessThan stops early only on a sum already above min: a full SSD decides the same
                const int d = full_ssd(a.in2, oin2, a.e2, origin(a.e2, 4, 4, 5, j + ll + mx, i + kk + my), 4, lane, bad);
                if (d > min2) continue;
                if (d == min2 && farther(mx, my, rmx, rmy, j, i, pl[4], pl[5])) continue;
                min2 = d;
                rmx = j;
                rmy = i;
                f.push(j + mx, i + my, d, lane);
            }
            mx += rmx;
            my += rmy;
        }
        fifo_best(f, lam, 16.0, 2, pl[4], pl[5], mx, my, lane);
        mx <<= 1;
        my <<= 1;
    }

    // level 1 (…:1374-1502): input samples of this lane's phase share, kept
    const Org oin1 = origin(a.in1, 8, 8, 0, q, p);
    int r1, c1;
    phase_coords<8>(lane, r1, c1);
    int cur1[2];
#pragma unroll
    for (int j = 0; j < 2; j++) cur1[j] = rdb(a.in1, oin1.y + r1, oin1.x + c1 + 4 * j);
    auto part8 = [&](Org o) {
        int acc = 0;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int d = cur1[j] - rdb(a.e1, o.y + r1, o.x + c1 + 4 * j);
            acc += d * d;
        }
        return acc;
    };
    int min1 = full_ssd(a.in1, oin1, a.e1, origin(a.e1, 8, 8, 9, mx + q, my + p), 8, lane, bad);
    f.reset(mx, my, min1);
    rmx = rmy = 0;
    auto consider1 = [&](int i, int j) {
        const int d = partial_value(part8(origin(a.e1, 8, 8, 9, j + mx + q, i + my + p)), min1, lane);
        if (d > min1) return;
        if (d == min1 && farther(mx, my, rmx, rmy, j, i, pl[2], pl[3])) return;
        min1 = d;
        rmx = j;
        rmy = i;
        f.push(j + mx, i + my, d, lane);
    };
    if (a.mode == 2) {
        mr_range(L1, q, p, mx, my, lcl_l1_range, xl, xr, yu, yd);
        for (int i = yu; i <= yd; i++)
            for (int j = xl; j <= xr; j++)
                if (i || j) consider1(i, j);
        mx += rmx;
        my += rmy;
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
    fifo_best(f, lam, 64.0, 1, pl[2], pl[3], mx, my, lane);
    mx <<= 1;
    my <<= 1;

    // level 0 +-2 refinement (…:1503-1574)
    int r0, c0;
    phase_coords<16>(lane, r0, c0);
    int cur0[8];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) cur0[4 * i + j] = rdb(a.in0, oin0.y + r0 + 4 * i, oin0.x + c0 + 4 * j);
    auto part16 = [&](Org o) {
        int acc = 0;
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int d = cur0[4 * i + j] - rdb(a.e0, o.y + r0 + 4 * i, o.x + c0 + 4 * j);
                acc += d * d;
            }
        return acc;
    };
    int min_d = out.zero_d;
    if (mx || my) min_d = full_ssd(a.in0, oin0, a.e0, origin(a.e0, 16, 16, 19, n + mx, m + my), 16, lane, bad);
    f.reset(mx, my, min_d);
    rmx = rmy = 0;
    mr_range(L0, n, m, mx, my, 2, xl, xr, yu, yd);
    for (int i = yu; i <= yd; i++)
        for (int j = xl; j <= xr; j++) {
            if (!(i || j)) continue;
            const int d = partial_value(part16(origin(a.e0, 16, 16, 19, n + mx + j, m + my + i)), min_d, lane);
            if (d > min_d) continue;
            if (d == min_d && farther(mx, my, rmx, rmy, j, i, pl[0], pl[1])) continue;
            min_d = d;
            rmx = j;
            rmy = i;
            f.push(j + mx, i + my, d, lane);
        }
    mx += rmx;
    my += rmy;
    min_d = fifo_best(f, lam, 256.0, 0, pl[0], pl[1], mx, my, lane);

    // half then quarter pel in Ver2's window (…:1575-1662), strict improvements
    int mvx = mx * 4, mvy = my * 4;
    f.reset(mvx, mvy, min_d);
    build_lattice<true>(LT, a.e0, origin(a.e0, 16, 16, 19, n + mx, m + my), lane, bad);
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
            f.push(qx + mvx, qy + mvy, d, lane);
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
            f.push(qmx + mvx, qmy + mvy, d, lane);
        }
    }
    __syncwarp();  // the lattice is reused by this warp's next search
    mvx += qmx;
    mvy += qmy;
    // towards the clamped quarter-pel prediction (…:1664-1677)
    out.min_d = fifo_best(f, lam, 256.0, 2, pcx, pcy, mvx, mvy, lane);
    out.mvx = mvx;
    out.mvy = mvy;
    return out;
}

// MultiresCross's tie rules: at level 2 the centre against the offset
// (…MultiresCross.cpp:673-679), elsewhere distances from (0, 0) (…:741-746, 857).
template <bool kH263 = false>
__device__ __forceinline__ MbSearch search_mb_mrc(const MrcArgs& a, Lattice& LT, int mbr, int mbc, int lane,
                                                  bool& bad)
{
    auto skip = [](int lvl, int mx, int my, int rmx, int rmy, int j, int i) {
        return lvl == 2 ? (my * my + mx * mx) - (i * i + j * j) < 0 : farther(mx, my, rmx, rmy, j, i, 0, 0);
    };
    return search_mb_with<false, decltype(skip)&, kH263>(a, LT, mbr, mbc, skip, lane, bad);
}

// The prediction's vector at a pyramid level (quarter-pel component p):
// Ver2 rounds to level 0 and halves (…MultiresCrossVer2.cpp:627-642),
// Multires rounds to every level (…Multires.cpp:646-655).
constexpr int EST_VER2 = 1, EST_MULTIRES = 2, EST_V2_LAMBDA = 4;
__device__ __forceinline__ int level_pred(int est, int p, int lvl)
{
    if (est == EST_MULTIRES) {
        const int h = 2 << lvl;  // 2, 4, 8
        return p < 0 ? (p - h) / (2 * h) : (p + h) / (2 * h);
    }
    int v = p < 0 ? (p - 2) / 4 : (p + 2) / 4;
    for (int l = 0; l < lvl; l++) v /= 2;
    return v;
}

// Search of a predictor estimator (est) with ties decided by the distances
// from prediction (px, py) at each level.
template <int kEst>
__device__ __forceinline__ MbSearch search_pred(const MrcArgs& a, Lattice& LT, int mbr, int mbc, int px, int py,
                                                int lane, bool& bad)
{
    int pl[6];
    for (int l = 0; l < 3; l++) {
        pl[2 * l] = level_pred(kEst, px, l);
        pl[2 * l + 1] = level_pred(kEst, py, l);
    }
    if constexpr (kEst == EST_V2_LAMBDA) {
        // the prediction clamped to one macroblock outside the picture (…MultiresCrossVer2.cpp:1664-1675)
        const int n = 16 * mbc, m = 16 * mbr;
        int px0 = px / 4, py0 = py / 4;
        if (px0 + n > a.W) px0 = 16;
        if (px0 + n < -16) px0 = -16;
        if (py0 + m > a.H) py0 = 16;
        if (py0 + m < -16) py0 = -16;
        return search_lambda(a, LT, mbr, mbc, pl, 4 * px0 + px % 4, 4 * py0 + py % 4, lane, bad);
    }
    auto skip = [&pl](int lvl, int mx, int my, int rmx, int rmy, int j, int i) {
        return farther(mx, my, rmx, rmy, j, i, pl[2 * lvl], pl[2 * lvl + 1]);
    };
    if constexpr (kEst == EST_MULTIRES) return search_mr_with(a, LT, mbr, mbc, skip, lane, bad);
    else return search_mb_with<true>(a, LT, mbr, mbc, skip, lane, bad);
}

// Tie tree of a Ver2 macroblock: run r of eight decides its t-th tie (t < 3)
// by bit t of r (1 takes the candidate) and records the tie's level and the
// two vectors compared, current (cx, cy) and candidate (nx, ny) in level
// units, so that the decision for any prediction follows from them; runs
// sharing their low t bits share their first t ties.
constexpr int V2_TIE_RUNS = 8, V2_TIE_BITS = 3;
struct V2TieRun {
    int geo[V2_TIE_BITS];  // bytes: cx, cy, nx, ny (signed)
    int lvl;               // 2 bits per tie
    int nev;               // ties met (> V2_TIE_BITS: the tree is too deep)
    int mv;                // packed quarter-pel result
    int min_d;
    int pad;
};

template <int kEst>
__device__ __forceinline__ MbSearch search_run(const MrcArgs& a, Lattice& LT, int mbr, int mbc, int run,
                                               V2TieRun* rec, int lane, bool& bad)
{
    int t = 0, lvls = 0, geo[V2_TIE_BITS] = {0, 0, 0};
    bool wide = false;
    auto skip = [&](int lvl, int mx, int my, int rmx, int rmy, int j, int i) {
        const int cx = mx + rmx, cy = my + rmy, nx = mx + j, ny = my + i;
        const bool take = t < V2_TIE_BITS ? ((run >> t) & 1) : true;
        if (t < V2_TIE_BITS) {
            wide |= (unsigned)(cx + 128) > 255u || (unsigned)(cy + 128) > 255u || (unsigned)(nx + 128) > 255u ||
                    (unsigned)(ny + 128) > 255u;
            geo[t] = (cx & 0xff) | ((cy & 0xff) << 8) | ((nx & 0xff) << 16) | ((ny & 0xff) << 24);
            lvls |= lvl << (2 * t);
        }
        t++;
        return !take;
    };
    MbSearch r;
    if constexpr (kEst == EST_MULTIRES) r = search_mr_with(a, LT, mbr, mbc, skip, lane, bad);
    else r = search_mb_with<true>(a, LT, mbr, mbc, skip, lane, bad);
    if (lane == 0) {
        for (int e = 0; e < V2_TIE_BITS; e++) rec->geo[e] = geo[e];
        rec->lvl = lvls;
        rec->nev = wide ? 1000 : t;
        rec->mv = pack_mv(r.mvx, r.mvy);
        rec->min_d = r.min_d;
    }
    return r;
}

// The searched vector and distortion of a tie MB for prediction (px, py)
// from its tie tree; false when the tree is too deep.
__device__ __forceinline__ bool tie_tree_result(int est, const V2TieRun* runs, int ppx, int ppy, int* mv, int* min_d)
{
    int run = 0;
    for (int t = 0; t < V2_TIE_BITS; t++) {
        const V2TieRun& r = runs[run];
        const int nev = __ldcg(&r.nev);
        if (t >= nev) break;
        const int g = __ldcg(&r.geo[t]), lvl = (__ldcg(&r.lvl) >> (2 * t)) & 3;
        const int cx = (signed char)(g & 0xff), cy = (signed char)((g >> 8) & 0xff);
        const int nx = (signed char)((g >> 16) & 0xff), ny = (signed char)(g >> 24);
        const int px = level_pred(est, ppx, lvl), py = level_pred(est, ppy, lvl);
        const bool skip = (cy - py) * (cy - py) + (cx - px) * (cx - px) < (ny - py) * (ny - py) + (nx - px) * (nx - px);
        run |= (skip ? 0 : 1) << t;
    }
    const V2TieRun& r = runs[run];
    if (__ldcg(&r.nev) > V2_TIE_BITS) return false;
    *mv = __ldcg(&r.mv);
    *min_d = __ldcg(&r.min_d);
    return true;
}

}  // namespace
}  // namespace mrc
}  // namespace vppgpu
