/*
 * oracle_me_impl.c -- TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * Restatement of MotionEstimatorImpl1::Estimate
 * (src/CodecUtils/MotionEstimatorImpl1.cpp:275-395): a full search of
 * [-range, range-1]^2 full pels by SSD, the OverlayMem2Dv2::HalfRead half-pel
 * refinement (OverlayMem2Dv2.cpp:452-596) over the neighbours GetHalfPelSearchStruct
 * allows (MotionEstimatorImpl1.cpp:445-515), and a weighted choice between the
 * winner and the zero vector.  No predictor: every block is independent.
 */
#include <stdlib.h>
#include "oracle_internal.h"

/* MEI1_HalfPos and the edge variants (MotionEstimatorImpl1.cpp:43-97), {x, y}. */
static const signed char HP_ALL[8][2] = {{-1, -1}, {0, -1}, {1, -1}, {-1, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1}};
static const signed char HP_TL[3][2] = {{1, 0}, {0, 1}, {1, 1}};
static const signed char HP_TR[3][2] = {{-1, 0}, {-1, 1}, {0, 1}};
static const signed char HP_BL[3][2] = {{0, -1}, {1, -1}, {1, 0}};
static const signed char HP_BR[3][2] = {{-1, -1}, {0, -1}, {-1, 0}};
static const signed char HP_L[5][2] = {{0, -1}, {1, -1}, {1, 0}, {0, 1}, {1, 1}};
static const signed char HP_R[5][2] = {{-1, -1}, {0, -1}, {-1, 0}, {-1, 1}, {0, 1}};
static const signed char HP_T[5][2] = {{-1, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1}};
static const signed char HP_B[5][2] = {{-1, -1}, {0, -1}, {1, -1}, {-1, 0}, {1, 0}};

/* GetHalfPelSearchStruct (MotionEstimatorImpl1.cpp:445-515): the half-pel
 * neighbours left inside the range at its extremes. */
static int half_positions(int x, int y, int range, const signed char (**pos)[2])
{
    const int r = x == range - 1, l = x == -range, b = y == range - 1, t = y == -range;
    if (!(r || l || b || t)) { *pos = HP_ALL; return 8; }
    if (!r && !l && !b && t) { *pos = HP_T; return 5; }
    if (!r && !l && b && !t) { *pos = HP_B; return 5; }
    if (!r && l && !b && !t) { *pos = HP_L; return 5; }
    if (r && !l && !b && !t) { *pos = HP_R; return 5; }
    if (!r && l && !b && t) { *pos = HP_TL; return 3; }
    if (r && !l && !b && t) { *pos = HP_TR; return 3; }
    if (!r && l && b && !t) { *pos = HP_BL; return 3; }
    if (r && !l && b && !t) { *pos = HP_BR; return 3; }
    *pos = HP_ALL;
    return 8;
}

static int blk_sd(const short* a, int as, const short* b, int bs, int bw, int bh)
{
    int acc = 0;
    for (int r = 0; r < bh; r++)
        for (int c = 0; c < bw; c++) {
            const int d = a[(size_t)r * as + c] - b[(size_t)r * bs + c];
            acc += d * d;
        }
    return acc;
}

/* OverlayMem2Dv2::HalfRead at half-pel offset (hx, hy) in -1..1 of the block at
 * p: rounded means of two (linear) or four (diagonal) full-pel samples. */
static void half_read(const short* p, int ps, int bw, int bh, int hx, int hy, short* dst)
{
    for (int r = 0; r < bh; r++)
        for (int c = 0; c < bw; c++) {
            const short* q = p + (size_t)r * ps + c;
            int v;
            if (hx && hy) v = (q[0] + q[hx] + q[(ptrdiff_t)hy * ps] + q[(ptrdiff_t)hy * ps + hx] + 2) / 4;
            else if (hx || hy) v = (q[0] + q[(ptrdiff_t)hy * ps + hx] + 1) / 2;
            else v = q[0];
            dst[r * bw + c] = (short)v;
        }
}

int vo_me_impl1(const short* src, const short* ref, int w, int h, int bw, int bh, int range, short* mv_out,
                int* mb_dist, long* avg_dist)
{
    if (!src || !ref || !mv_out || bw < 2 || bh < 1 || bw > 16 || bh > 16 || (bw & 1) || w % bw || h % bh ||
        range < 1 || range > 63)
        return -1;
    const int B = range + 1, es = w + 2 * B;
    short* e = vo_ext_alloc(ref, w, h, B);
    if (!e) return -2;
    const int cols = w / bw, nmb = cols * (h / bh);
    long total = 0;
    short blk[256];
    for (int k = 0; k < nmb; k++) {
        const int n = (k % cols) * bw, m = (k / cols) * bh;
        const short* in = src + (size_t)m * w + n;
        const short* at = e + (size_t)(m + B) * es + n + B;  /* block (n, m) of the extended reference */
        const int zero = blk_sd(in, w, at, es, bw, bh);
        int min = zero, mx = 0, my = 0;
        for (int y = -range; y < range; y++)
            for (int x = -range; x < range; x++) {
                const int d = blk_sd(in, w, at + (ptrdiff_t)y * es + x, es, bw, bh);
                if (d < min) { min = d; mx = x; my = y; }
            }
        const signed char(*pos)[2];
        const int np = half_positions(mx, my, range, &pos);
        int hmx = 0, hmy = 0;
        for (int i = 0; i < np; i++) {
            half_read(at + (ptrdiff_t)my * es + mx, es, bw, bh, pos[i][0], pos[i][1], blk);
            const int d = blk_sd(in, w, blk, bw, bw, bh);
            if (d < min) { min = d; hmx = pos[i][0]; hmy = pos[i][1]; }
        }
        int mvx = 2 * mx + hmx, mvy = 2 * my + hmy;
        /* the weighted choice against the zero vector (MotionEstimatorImpl1.cpp:356-378) */
        const int diff = zero - min, mag = mvx * mvx + mvy * mvy;
        const int weight = ((diff >> 2) < mag) + (zero < 512) + (diff * 10 < min);
        int d;
        if (min < zero && weight < 2) {
            d = min;
        } else {
            mvx = mvy = 0;
            d = zero;
        }
        total += d;
        if (mb_dist) mb_dist[k] = d;
        mv_out[2 * k] = (short)(signed char)mvx; /* the SimpleMotionVectorList holds chars */
        mv_out[2 * k + 1] = (short)(signed char)mvy;
    }
    if (avg_dist) *avg_dist = total / nmb;
    free(e);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* MotionEstimatorImpl2                                                      */
/* ------------------------------------------------------------------------ */
static int blk_ad(const short* a, int as, const short* b, int bs, int n)
{
    int acc = 0;
    for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) acc += abs(a[(size_t)r * as + c] - b[(size_t)r * bs + c]);
    return acc;
}

/* One level's search of MotionEstimatorImpl2 (MotionEstimatorImpl2.cpp:585-743):
 * candidates (j, i) in [-r, r]^2 around the centre (cx, cy) in raster order,
 * (0, 0) skipped; a candidate is taken when its SAD is below the running
 * minimum, or equal to it and its vector (centre + offset) not farther from
 * the origin than the running best.  Returns the minimum; *rx, *ry the offset. */
static int impl2_level(const short* in, int ins, const short* at, int es, int n, int cx, int cy, int r, int* rx,
                       int* ry)
{
    int min = blk_ad(in, ins, at + (ptrdiff_t)cy * es + cx, es, n), bx = 0, by = 0;
    for (int i = -r; i <= r; i++)
        for (int j = -r; j <= r; j++) {
            if (!(i || j)) continue;
            const int d = blk_ad(in, ins, at + (ptrdiff_t)(cy + i) * es + cx + j, es, n);
            if (d > min) continue;
            if (d == min) {
                const int dist = ((cy + by) * (cy + by) + (cx + bx) * (cx + bx)) - ((cy + i) * (cy + i) + (cx + j) * (cx + j));
                if (dist < 0) continue;
            }
            min = d;
            bx = j;
            by = i;
        }
    *rx = bx;
    *ry = by;
    return min;
}

/* The clamp between levels (MotionEstimatorImpl2.cpp:638-645, 686-695): the
 * centre keeps a +-2 refinement inside [-range, range-1]. */
static int impl2_clamp(int v, int range)
{
    if (v + 2 >= range) return range - 1 - 2;
    if (v - 2 < -range) return -(range - 2);
    return v;
}

int vo_me_impl2(const short* src, const short* ref, int w, int h, int range, int mode, short* mv_out, int* mb_dist,
                long* avg_dist)
{
    if (!src || !ref || !mv_out || w % 16 || h % 16 || w < 16 || h < 16 || range < 4 || range > 63) return -1;
    if (mode == 0) mode = (w * h > 40000) ? 2 : 1;  /* SetMode(0), MotionEstimatorImpl2.cpp:481-493 */
    const int w1 = w / 2, h1 = h / 2, w2 = w1 / 2, h2 = h1 / 2;
    const int r1 = range / 2, r2 = r1 / 2;
    const int B0 = range + 1, B1 = r1 + 1, B2 = r2 + 1;
    short* ref1 = (short*)malloc(sizeof(short) * (size_t)w1 * h1);
    short* ref2 = (short*)malloc(sizeof(short) * (size_t)w2 * h2);
    short* in1 = (short*)malloc(sizeof(short) * (size_t)w1 * h1);
    short* in2 = (short*)malloc(sizeof(short) * (size_t)w2 * h2);
    if (!ref1 || !ref2 || !in1 || !in2) {
        free(ref1); free(ref2); free(in1); free(in2);
        return -2;
    }
    vo_half(ref, w, h, ref1);
    vo_half(ref1, w1, h1, ref2);
    vo_half(src, w, h, in1);
    vo_half(in1, w1, h1, in2);
    short* e0 = vo_ext_alloc(ref, w, h, B0);
    short* e1 = vo_ext_alloc(ref1, w1, h1, B1);
    short* e2 = vo_ext_alloc(ref2, w2, h2, B2);
    if (!e0 || !e1 || !e2) {
        free(ref1); free(ref2); free(in1); free(in2); free(e0); free(e1); free(e2);
        return -2;
    }
    const int es0 = w + 2 * B0, es1 = w1 + 2 * B1, es2 = w2 + 2 * B2;
    const int cols = w / 16, nmb = cols * (h / 16);
    long total = 0;
    short blk[256];
    for (int k = 0; k < nmb; k++) {
        const int n = (k % cols) * 16, m = (k / cols) * 16;
        const short* in = src + (size_t)m * w + n;
        const short* at0 = e0 + (size_t)(m + B0) * es0 + n + B0;
        const int zero = blk_ad(in, w, at0, es0, 16);
        int mx = 0, my = 0, rx, ry;
        if (mode == 2) {  /* level 2: the full range (:585-631) */
            const short* at2 = e2 + (size_t)(m / 4 + B2) * es2 + n / 4 + B2;
            impl2_level(in2 + (size_t)(m / 4) * w2 + n / 4, w2, at2, es2, 4, 0, 0, r2, &rx, &ry);
            mx = impl2_clamp(2 * rx, r1);
            my = impl2_clamp(2 * ry, r1);
        }
        /* level 1: the full range, or +-2 around the level-2 result (:648-684) */
        const short* at1 = e1 + (size_t)(m / 2 + B1) * es1 + n / 2 + B1;
        impl2_level(in1 + (size_t)(m / 2) * w1 + n / 2, w1, at1, es1, 8, mx, my, mode == 2 ? 2 : r1, &rx, &ry);
        mx = impl2_clamp((mx + rx) * 2, range);
        my = impl2_clamp((my + ry) * 2, range);
        /* level 0: +-2 (:697-729) */
        int min = impl2_level(in, w, at0, es0, 16, mx, my, 2, &rx, &ry);
        mx += rx;
        my += ry;
        /* half pel: HalfRead at the neighbours the range leaves, strict improvement (:731-746) */
        const signed char(*pos)[2];
        const int np = half_positions(mx, my, range, &pos);
        int hmx = 0, hmy = 0;
        for (int i = 0; i < np; i++) {
            half_read(at0 + (ptrdiff_t)my * es0 + mx, es0, 16, 16, pos[i][0], pos[i][1], blk);
            const int d = blk_ad(in, w, blk, 16, 16);
            if (d < min) { min = d; hmx = pos[i][0]; hmy = pos[i][1]; }
        }
        int mvx = 2 * mx + hmx, mvy = 2 * my + hmy;
        /* the weighted choice against the zero vector (:752-774) */
        const int diff = zero - min, mag = mvx * mvx + mvy * mvy;
        const int weight = ((diff >> 1) < mag) + (zero < 26) + (diff * 7 < min);
        int d;
        if (min < zero && weight < 2) {
            d = min;
        } else {
            mvx = mvy = 0;
            d = zero;
        }
        total += d;
        if (mb_dist) mb_dist[k] = d;
        mv_out[2 * k] = (short)(signed char)mvx;
        mv_out[2 * k + 1] = (short)(signed char)mvy;
    }
    if (avg_dist) *avg_dist = total / nmb;
    free(ref1); free(ref2); free(in1); free(in2); free(e0); free(e1); free(e2);
    return 0;
}
