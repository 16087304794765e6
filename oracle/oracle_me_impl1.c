/*
 * oracle_me_impl1.c -- TEST INFRASTRUCTURE ONLY (CPU oracle).
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
