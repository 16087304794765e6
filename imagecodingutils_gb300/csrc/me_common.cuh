// me_common.cuh -- device building blocks shared by the motion estimators:
// padded-reference geometry, the H.264 sub-pel samplers, warp-level 16x16
// distortion, the median predictor and the Lagrangian vector pick.
#pragma once

#include "vppgpu_internal.cuh"

namespace vppgpu {

// Padded 8-bit reference: every plane is stored with PAD samples of edge
// replication on each side (OverlayExtMem2Dv2::FillBoundary,
// src/ImageUtils/OverlayExtMem2Dv2.cpp:153-211, is a coordinate clamp).  48
// covers the +-31 search window, the 3-sample 6-tap margin of the sub-pel
// stages and the 16-sample macroblock overhang the reference allows.
constexpr int PAD = 48;

struct Plane8 {
    const unsigned char* p;  // top-left of the padded buffer
    int stride;              // bytes per padded row (multiple of 16)
    __device__ __forceinline__ const unsigned char* at(int x, int y) const
    {
        return p + (size_t)(y + PAD) * stride + (x + PAD);
    }
};

// Status bits written by device code.
constexpr int ST_PIXEL_RANGE = 1;
constexpr int ST_TIMEOUT = 2;

__device__ __forceinline__ int pack_mv(int x, int y) { return (int)((unsigned)(x & 0xffff) | ((unsigned)y << 16)); }
__device__ __forceinline__ int mv_x(int p) { return (int)(short)(p & 0xffff); }
__device__ __forceinline__ int mv_y(int p) { return p >> 16; }

__device__ __forceinline__ int tap6(int a, int b, int c, int d, int e, int f)
{
    return a - 5 * b + 20 * c + 20 * d - 5 * e + f;
}

// ---------------------------------------------------------------------------
// Sub-pel refinement of the full-pel winner, one warp.
//
// MotionEstimatorH264ImplFull::LoadHalfQuartPelWindow / LoadQuartPelWindow /
// QuarterRead (src/CodecUtils/MotionEstimatorH264ImplFull.cpp:1095-1255) and
// the two candidate passes of Estimate (Full.cpp:452-517): eight half-pel
// neighbours (6-tap b/h/j, clipped), then eight quarter-pel neighbours of the
// half-pel winner, each the rounded mean of two lattice samples, strict
// improvement in MEH264IF_SubPos order (Full.cpp:77-81).
// ---------------------------------------------------------------------------
struct SubpelScratch {
    unsigned char patch[22][24];  // full-pel samples at fy,fx in [-3,18]
    int rawv[17][22];             // unrounded vertical 6-tap, fy in [-1,15], fx in [-3,18]
    unsigned char hp[17][18];     // h (vertical half) fy in [-1,15], fx in [-1,16]
    unsigned char bp[18][17];     // b (horizontal half) fy in [-1,16], fx in [-1,15]
    unsigned char jp[17][17];     // j (centre half) fy,fx in [-1,15]
};

__device__ __constant__ static const signed char kSubX[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
__device__ __constant__ static const signed char kSubY[8] = {-1, -1, -1, 0, 0, 1, 1, 1};

// Lattice sample at even quarter coordinates (qy, qx) relative to the origin.
__device__ __forceinline__ int lattice(const SubpelScratch& s, int qy, int qx)
{
    int fy = qy >> 2, fx = qx >> 2;
    int ry = qy & 3, rx = qx & 3;
    if (ry == 0) return rx == 0 ? s.patch[fy + 3][fx + 3] : s.bp[fy + 1][fx + 1];
    return rx == 0 ? s.hp[fy + 1][fx + 1] : s.jp[fy + 1][fx + 1];
}

// Quarter sample at (cy+sy, cx+sx) around the even point (cy, cx), with the
// neighbour pairs of LoadQuartPelWindow (Full.cpp:1207-1220).
__device__ __forceinline__ int quarter_sample(const SubpelScratch& s, int cy, int cx, int sy, int sx)
{
    int a, b;
    if (sy < 0) {
        a = lattice(s, cy - 2, sx < 0 ? cx - 2 : cx);
        b = sx > 0 ? lattice(s, cy, cx + 2) : lattice(s, cy, cx);
    } else if (sy == 0) {
        a = lattice(s, cy, cx + (sx < 0 ? -2 : 2));
        b = lattice(s, cy, cx);
    } else {
        a = sx < 0 ? lattice(s, cy, cx - 2) : lattice(s, cy + 2, cx);
        b = sx > 0 ? lattice(s, cy, cx + 2) : (sx < 0 ? lattice(s, cy + 2, cx) : lattice(s, cy, cx));
    }
    return (a + b + 1) >> 1;
}

__device__ __forceinline__ int warp_sum(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Build the half-pel planes from s.patch (already filled, __syncwarp'd).
__device__ __forceinline__ void subpel_planes(SubpelScratch& s, int lane)
{
    for (int i = lane; i < 17 * 22; i += 32) {
        int r = i / 22, c = i - r * 22;  // fy = r-1, fx = c-3 ; patch row fy+3 = r+2
        s.rawv[r][c] = tap6(s.patch[r][c], s.patch[r + 1][c], s.patch[r + 2][c], s.patch[r + 3][c],
                            s.patch[r + 4][c], s.patch[r + 5][c]);
    }
    for (int i = lane; i < 18 * 17; i += 32) {
        int r = i / 17, c = i - r * 17;  // fy = r-1, fx = c-1 ; patch row fy+3 = r+2, cols fx+1.. = c..
        const unsigned char* q = &s.patch[r + 2][c];
        s.bp[r][c] = (unsigned char)clip255((tap6(q[0], q[1], q[2], q[3], q[4], q[5]) + 16) >> 5);
    }
    __syncwarp();
    for (int i = lane; i < 17 * 18; i += 32) {
        int r = i / 18, c = i - r * 18;  // fy = r-1, fx = c-1 -> rawv col fx+3 = c+2
        s.hp[r][c] = (unsigned char)clip255((s.rawv[r][c + 2] + 16) >> 5);
    }
    for (int i = lane; i < 17 * 17; i += 32) {
        int r = i / 17, c = i - r * 17;  // fx = c-1 -> rawv cols fx+1..fx+6 = c..c+5
        const int* q = &s.rawv[r][c];
        s.jp[r][c] = (unsigned char)clip255((tap6(q[0], q[1], q[2], q[3], q[4], q[5]) + 512) >> 10);
    }
    __syncwarp();
}

// cur: 16x16 input block (row stride 16).  Enters with the full-pel minimum
// in *min_d; leaves with the refined minimum and quarter offsets (qmx, qmy).
// kLean: loops kept rolled, for callers where registers matter more than
// speed (the rare tie rescans inside the prediction-dependent kernels).
template <bool kLean = false>
__device__ __forceinline__ void subpel_refine_warp(SubpelScratch& s, const unsigned char* cur, int lane, int* min_d,
                                                   int* qmx, int* qmy)
{
    subpel_planes(s, lane);
    int best = *min_d, hmx = 0, hmy = 0;
    // lane handles pixels lane + 32*t, t = 0..7
#pragma unroll(kLean ? 1 : 8)
    for (int k = 0; k < 8; k++) {
        int qx = 2 * kSubX[k], qy = 2 * kSubY[k];
        int acc = 0;
#pragma unroll(kLean ? 1 : 8)
        for (int t = 0; t < 8; t++) {
            int px = lane + 32 * t, r = px >> 4, c = px & 15;
            int d = (int)cur[px] - lattice(s, 4 * r + qy, 4 * c + qx);
            acc += d * d;
        }
        acc = warp_sum(acc);
        if (acc < best) {
            best = acc;
            hmx = qx;
            hmy = qy;
        }
    }
    int bx = hmx, by = hmy;
#pragma unroll(kLean ? 1 : 8)
    for (int k = 0; k < 8; k++) {
        int sx = kSubX[k], sy = kSubY[k];
        int acc = 0;
#pragma unroll(kLean ? 1 : 8)
        for (int t = 0; t < 8; t++) {
            int px = lane + 32 * t, r = px >> 4, c = px & 15;
            int d = (int)cur[px] - quarter_sample(s, 4 * r + hmy, 4 * c + hmx, sy, sx);
            acc += d * d;
        }
        acc = warp_sum(acc);
        if (acc < best) {
            best = acc;
            bx = hmx + sx;
            by = hmy + sy;
        }
    }
    *min_d = best;
    *qmx = bx;
    *qmy = by;
}

// ---------------------------------------------------------------------------
// OverlayMem2Dv2::QuarterRead + Tsd16x16 (src/ImageUtils/OverlayMem2Dv2.cpp:704-1052,
// 1623-1700) at a quarter-pel vector, one warp.  `patch` holds full-pel
// samples at fy,fx in [-3,18] around the full-pel position of the vector
// (row stride 24); (fx, fy) are the fractional parts 0..3 after negative
// offsets are folded into the full-pel position.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int pG(const unsigned char (*p)[24], int y, int x) { return p[y + 3][x + 3]; }
__device__ __forceinline__ int pB(const unsigned char (*p)[24], int y, int x)
{
    const unsigned char* q = &p[y + 3][x + 1];
    return clip255((tap6(q[0], q[1], q[2], q[3], q[4], q[5]) + 16) >> 5);
}
__device__ __forceinline__ int pHraw(const unsigned char (*p)[24], int y, int x)
{
    return tap6(p[y + 1][x + 3], p[y + 2][x + 3], p[y + 3][x + 3], p[y + 4][x + 3], p[y + 5][x + 3], p[y + 6][x + 3]);
}
__device__ __forceinline__ int pH(const unsigned char (*p)[24], int y, int x) { return clip255((pHraw(p, y, x) + 16) >> 5); }
__device__ __forceinline__ int pJ(const unsigned char (*p)[24], int y, int x)
{
    int s = tap6(pHraw(p, y, x - 2), pHraw(p, y, x - 1), pHraw(p, y, x), pHraw(p, y, x + 1), pHraw(p, y, x + 2),
                 pHraw(p, y, x + 3));
    return clip255((s + 512) >> 10);
}

__device__ __forceinline__ int qread_sample(const unsigned char (*p)[24], int y, int x, int fx, int fy)
{
    switch (fx | (fy << 2)) {
    case 0: return pG(p, y, x);
    case 2: return pB(p, y, x);
    case 8: return pH(p, y, x);
    case 10: return pJ(p, y, x);
    case 1: return (pG(p, y, x) + pB(p, y, x) + 1) >> 1;
    case 3: return (pG(p, y, x + 1) + pB(p, y, x) + 1) >> 1;
    case 4: return (pG(p, y, x) + pH(p, y, x) + 1) >> 1;
    case 12: return (pG(p, y + 1, x) + pH(p, y, x) + 1) >> 1;
    case 6: return (pJ(p, y, x) + pB(p, y, x) + 1) >> 1;
    case 14: return (pJ(p, y, x) + pB(p, y + 1, x) + 1) >> 1;
    case 9: return (pJ(p, y, x) + pH(p, y, x) + 1) >> 1;
    case 11: return (pJ(p, y, x) + pH(p, y, x + 1) + 1) >> 1;
    case 5: return (pB(p, y, x) + pH(p, y, x) + 1) >> 1;
    case 7: return (pB(p, y, x) + pH(p, y, x + 1) + 1) >> 1;
    case 13: return (pH(p, y, x) + pB(p, y + 1, x) + 1) >> 1;
    default: return (pH(p, y, x + 1) + pB(p, y + 1, x) + 1) >> 1;
    }
}

// Squared distortion of `cur` against the quarter-pel block whose folded
// full-pel origin is the patch centre.
__device__ __forceinline__ int qread_ssd_warp(const unsigned char (*patch)[24], const unsigned char* cur, int fx,
                                              int fy, int lane)
{
    int acc = 0;
#pragma unroll 2
    for (int t = 0; t < 8; t++) {
        int px = lane + 32 * t, r = px >> 4, c = px & 15;
        int d = (int)cur[px] - qread_sample(patch, r, c, fx, fy);
        acc += d * d;
    }
    return warp_sum(acc);
}

// Planar form of the same distortion: the half-pel planes the fractional
// case needs are computed once into per-warp scratch (b: 17x16, h: 16x17,
// j from 16x21 unrounded vertical taps), then every pixel is a lookup or a
// rounded mean of two lookups -- about 20x fewer taps than per-pixel j.
struct PdScratch {
    unsigned char patch[22][24];
    int rawv[16][21];
    unsigned char b[17][16];
    unsigned char h[16][17];
    unsigned char j[16][16];
};

__device__ __forceinline__ int pd_planar_warp(PdScratch& s, const unsigned char* cur, int fx, int fy, int lane)
{
    const int sel = fx | (fy << 2);
    // which planes: b for x-half and the b-based quarter cases, h likewise, j for the centre cases
    const bool need_b = sel == 2 || sel == 1 || sel == 3 || sel == 6 || sel == 14 || sel == 5 || sel == 7 ||
                        sel == 13 || sel == 15;
    const bool need_h = sel == 8 || sel == 4 || sel == 12 || sel == 9 || sel == 11 || sel == 5 || sel == 7 ||
                        sel == 13 || sel == 15;
    const bool need_j = sel == 10 || sel == 6 || sel == 14 || sel == 9 || sel == 11;
    if (need_b)
        for (int i = lane; i < 17 * 16; i += 32) {
            int r = i >> 4, c = i & 15;  // b at (r, c): row r, cols c-2..c+3 -> patch [r+3][c+1..c+6]
            const unsigned char* q = &s.patch[r + 3][c + 1];
            s.b[r][c] = (unsigned char)clip255((tap6(q[0], q[1], q[2], q[3], q[4], q[5]) + 16) >> 5);
        }
    if (need_h)
        for (int i = lane; i < 16 * 17; i += 32) {
            int r = i / 17, c = i - r * 17;  // h at (r, c): rows r-2..r+3 -> patch [r+1..r+6][c+3]
            s.h[r][c] = (unsigned char)clip255((tap6(s.patch[r + 1][c + 3], s.patch[r + 2][c + 3], s.patch[r + 3][c + 3],
                                                     s.patch[r + 4][c + 3], s.patch[r + 5][c + 3], s.patch[r + 6][c + 3]) +
                                                16) >> 5);
        }
    if (need_j) {
        for (int i = lane; i < 16 * 21; i += 32) {
            int r = i / 21, c = i - r * 21;  // vertical taps at col c-2 -> patch col c+1
            s.rawv[r][c] = tap6(s.patch[r + 1][c + 1], s.patch[r + 2][c + 1], s.patch[r + 3][c + 1], s.patch[r + 4][c + 1],
                                s.patch[r + 5][c + 1], s.patch[r + 6][c + 1]);
        }
        __syncwarp();
        for (int i = lane; i < 256; i += 32) {
            int r = i >> 4, c = i & 15;
            const int* q = &s.rawv[r][c];  // cols c-2..c+3
            s.j[r][c] = (unsigned char)clip255((tap6(q[0], q[1], q[2], q[3], q[4], q[5]) + 512) >> 10);
        }
    }
    __syncwarp();
    // each case reads one plane sample or the rounded mean of two; the case
    // is uniform across the warp, so pick base pointers and strides once
    const unsigned char* G0 = &s.patch[3][3];
    const unsigned char *p1 = G0, *p2 = G0;
    int st1 = 24, st2 = 24;
    bool two = true;
    switch (sel) {
    case 0: two = false; break;
    case 2: p1 = &s.b[0][0]; st1 = 16; two = false; break;                   // b
    case 8: p1 = &s.h[0][0]; st1 = 17; two = false; break;                   // h
    case 10: p1 = &s.j[0][0]; st1 = 16; two = false; break;                  // j
    case 1: p2 = &s.b[0][0]; st2 = 16; break;                                // a = (G + b)
    case 3: p1 = G0 + 1; p2 = &s.b[0][0]; st2 = 16; break;                   // c = (G[x+1] + b)
    case 4: p2 = &s.h[0][0]; st2 = 17; break;                                // d = (G + h)
    case 12: p1 = G0 + 24; p2 = &s.h[0][0]; st2 = 17; break;                 // n = (G[y+1] + h)
    case 6: p1 = &s.j[0][0]; st1 = 16; p2 = &s.b[0][0]; st2 = 16; break;     // f = (j + b)
    case 14: p1 = &s.j[0][0]; st1 = 16; p2 = &s.b[1][0]; st2 = 16; break;    // q = (j + b[y+1])
    case 9: p1 = &s.j[0][0]; st1 = 16; p2 = &s.h[0][0]; st2 = 17; break;     // i = (j + h)
    case 11: p1 = &s.j[0][0]; st1 = 16; p2 = &s.h[0][1]; st2 = 17; break;    // k = (j + h[x+1])
    case 5: p1 = &s.b[0][0]; st1 = 16; p2 = &s.h[0][0]; st2 = 17; break;     // e = (b + h)
    case 7: p1 = &s.b[0][0]; st1 = 16; p2 = &s.h[0][1]; st2 = 17; break;     // g = (b + h[x+1])
    case 13: p1 = &s.h[0][0]; st1 = 17; p2 = &s.b[1][0]; st2 = 16; break;    // p = (h + b[y+1])
    default: p1 = &s.h[0][1]; st1 = 17; p2 = &s.b[1][0]; st2 = 16; break;    // r = (h[x+1] + b[y+1])
    }
    int acc = 0;
#pragma unroll
    for (int t = 0; t < 8; t++) {
        int px = lane + 32 * t, r = px >> 4, c = px & 15;
        int v = p1[r * st1 + c];
        if (two) v = (v + p2[r * st2 + c] + 1) >> 1;
        int d = (int)cur[px] - v;
        acc += d * d;
    }
    return warp_sum(acc);
}

// Copy a 22x22 full-pel patch (rows/cols -3..18 around (x, y)) from a padded plane.
__device__ __forceinline__ void load_patch22(unsigned char (*dst)[24], const Plane8& pl, int x, int y, int lane)
{
    unsigned char v[16];
#pragma unroll
    for (int t = 0; t < 16; t++) {  // all loads in flight before any store
        int i = lane + 32 * t;
        int r = i / 22, c = i - r * 22;
        v[t] = i < 22 * 22 ? __ldg(pl.at(x - 3 + c, y - 3 + r)) : 0;
    }
#pragma unroll
    for (int t = 0; t < 16; t++) {
        int i = lane + 32 * t;
        if (i < 22 * 22) dst[i / 22][i % 22] = v[t];
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------
// Median prediction (MacroBlockH264::GetMbMotionMedianPred,
// src/CodecUtils/MacroBlockH264.cpp:757-816; Median :923-936) from the
// current vectors of the left (A), above (B), above-right (C, else
// above-left D) neighbours; unavailable neighbours count as (0,0) and with
// neither B nor C both take A.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int median3(int x, int y, int z)
{
    int lo = y - z < 0 ? y : z, hi = y - z < 0 ? z : y;
    lo = x < lo ? x : lo;
    hi = x > hi ? x : hi;
    return x + y + z - lo - hi;
}

// Neighbour availability bits kept in the per-macroblock flags (position
// and slice membership, MacroBlockH264::Initialise, MacroBlockH264.cpp:319-).
constexpr int AV_A = 1 << 1;   // left
constexpr int AV_B = 1 << 2;   // above
constexpr int AV_C = 1 << 3;   // above-right
constexpr int AV_D = 1 << 4;   // above-left

__device__ __forceinline__ int neighbour_mask(const int* slice, int k, int cols, int rows)
{
    int r = k / cols, c = k - r * cols;
    int sk = slice ? slice[k] : 0;
    auto ok = [&](int rr, int cc) { return rr >= 0 && rr < rows && cc >= 0 && cc < cols && (!slice || slice[rr * cols + cc] == sk); };
    return (ok(r, c - 1) ? AV_A : 0) | (ok(r - 1, c) ? AV_B : 0) | (ok(r - 1, c + 1) ? AV_C : 0) |
           (ok(r - 1, c - 1) ? AV_D : 0);
}

// Median of the packed neighbour vectors under the availability mask.
__device__ __forceinline__ void median_from(int av, int A, int B, int C, int D, int* px, int* py)
{
    if (!(av & AV_A)) A = 0;
    if (!(av & AV_B)) B = 0;
    if (av & AV_C) {
    } else if (av & AV_D) {
        C = D;
    } else {
        C = 0;
    }
    if (!(av & AV_B) && !(av & AV_C)) B = C = A;
    *px = median3(mv_x(A), mv_x(B), mv_x(C));
    *py = median3(mv_y(A), mv_y(B), mv_y(C));
}

// Same median on packed vectors (x in the low, y in the high signed 16-bit
// half): per-half min/max, the packed result equals pack_mv(px, py).
__device__ __forceinline__ int median_packed(int av, int A, int B, int C, int D)
{
    if (!(av & AV_A)) A = 0;
    if (!(av & AV_B)) B = 0;
    C = (av & AV_C) ? C : ((av & AV_D) ? D : 0);
    if (!(av & AV_B) && !(av & AV_C)) B = C = A;
    const unsigned a = (unsigned)A, b = (unsigned)B, c = (unsigned)C;
    return (int)__vmaxs2(__vmins2(a, b), __vmins2(__vmaxs2(a, b), c));
}

// From the current vectors in global memory (L2, bypassing L1: other SMs update them).
__device__ __forceinline__ void median_pred(const int* final_mv, int av, int k, int cols, int* px, int* py)
{
    int A = (av & AV_A) ? __ldcg(final_mv + k - 1) : 0;
    int B = (av & AV_B) ? __ldcg(final_mv + k - cols) : 0;
    int C = (av & AV_C) ? __ldcg(final_mv + k - cols + 1) : 0;
    int D = (!(av & AV_C) && (av & AV_D)) ? __ldcg(final_mv + k - cols - 1) : 0;
    median_from(av, A, B, C, D, px, py);
}

// Nearest full-pel prediction with C division (Full.cpp:368-380).
__device__ __forceinline__ int round_pred(int p) { return p < 0 ? (p - 2) / 4 : (p + 2) / 4; }

// GetBestVector over the Fifo slots (best, pred, zero, zero, zero)
// (include/CodecUtils/MotionEstimatorH264ImplFull.h:140-168): cost =
// D/norm + lambda*sqrt(|v-ref|^2) in IEEE double, one rounding per
// operation, strict improvement.  Returns the winning slot 0..2.
static __device__ __noinline__ int best_of3(int bx, int by, int bd, int px, int py, int pd, int zd, double lambda,
                                        double norm, int xref, int yref)
{
    auto cost = [&](int x, int y, int d) {
        double m = (double)((x - xref) * (x - xref) + (y - yref) * (y - yref));
        return __dadd_rn(__ddiv_rn((double)d, norm), __dmul_rn(lambda, __dsqrt_rn(m)));
    };
    double c0 = cost(bx, by, bd);
    int pos = 0;
    double c1 = cost(px, py, pd);
    if (c1 < c0) {
        c0 = c1;
        pos = 1;
    }
    double c2 = cost(0, 0, zd);
    if (c2 < c0) pos = 2;
    return pos;
}

// Same decision without FP64 in the common cases.  Two costs with the same
// sqrt argument differ only in D/norm, and D/256 is exact; with |lambda| <
// 2^20 every sum stays below 2^40, where costs 1/256 apart never round
// together, so their double order is the order of the integers D.  This
// covers the most frequent near-tie, the prediction slot against a searched
// vector equal to it.  Other pairs compare in float: each float cost is
// within a few ulp of the exact real value and the double costs within 2^-50
// relative, so when a pair differs by more than 2^-18 relative both orderings
// agree with the exact one; closer pairs take the double path.
__device__ __forceinline__ int best_of3_fast(int bx, int by, int bd, int px, int py, int pd, int zd, double lambda,
                                             int xref, int yref)
{
    const int m0 = (bx - xref) * (bx - xref) + (by - yref) * (by - yref);
    const int m1 = (px - xref) * (px - xref) + (py - yref) * (py - yref);
    const int m2 = xref * xref + yref * yref;
    const float lf = (float)lambda, inv = 1.0f / 256.0f;
    const float c0 = (float)bd * inv + lf * sqrtf((float)m0);
    const float c1 = (float)pd * inv + lf * sqrtf((float)m1);
    const float c2 = (float)zd * inv + lf * sqrtf((float)m2);
    bool slow = false;
    const bool small_lambda = fabs(lambda) < 1048576.0;
    // strict "cost a < cost b" in the double arithmetic of best_of3
    auto less = [&](int da, int ma, float ca, int db, int mb, float cb) {
        if (ma == mb && small_lambda) return da < db;
        if (fabsf(ca - cb) <= 4e-6f * fmaxf(fabsf(ca), fabsf(cb)) + 1e-30f) slow = true;
        return ca < cb;
    };
    int pos = less(pd, m1, c1, bd, m0, c0) ? 1 : 0;
    const bool z = pos == 0 ? less(zd, m2, c2, bd, m0, c0) : less(zd, m2, c2, pd, m1, c1);
    if (slow) return best_of3(bx, by, bd, px, py, pd, zd, lambda, 256.0, xref, yref);
    return z ? 2 : pos;
}

// ---------------------------------------------------------------------------
// Grid-wide barrier for cooperative launches with a bounded wait: a block
// that waits longer than `limit` polls sets ST_TIMEOUT and leaves.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool grid_sync(unsigned* bar, int* status, unsigned nblocks, long long limit)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = bar + 1;
        unsigned gen = *vgen;
        __threadfence();
        unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == nblocks - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long it = 0;
            while (*vgen == gen) {
                __nanosleep(100);
                if (++it > limit) {
                    atomicOr(status, ST_TIMEOUT);
                    break;
                }
                if (*((volatile int*)status) & ST_TIMEOUT) break;
            }
        }
        __threadfence();
    }
    __syncthreads();
    return (*((volatile int*)status) & ST_TIMEOUT) == 0;
}

}  // namespace vppgpu
