/*
 * oracle_overlay.c -- TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * Restates the OverlayMem2Dv2 / OverlayExtMem2Dv2 primitives the motion
 * estimators use: edge-replicated boundary extension, clamped block origins,
 * squared / absolute block distortion (plain, early-exit and the 16-phase
 * partial form), the H.264 6-tap half-pel and bilinear quarter-pel read, and
 * 2:1 decimation.  Each function cites the reference lines it follows.
 */
#include <stdlib.h>
#include <string.h>
#include "oracle_internal.h"

/* OverlayExtMem2Dv2::ExtendBoundary + FillBoundary
 * (src/ImageUtils/OverlayExtMem2Dv2.cpp:120-211): the centre is the source
 * plane, every boundary sample repeats the nearest edge sample (corners repeat
 * the corner sample).  That is exactly a coordinate clamp. */
short* vo_ext_alloc(const short* plane, int w, int h, int border)
{
    int ew = w + 2 * border, eh = h + 2 * border;
    short* e = (short*)malloc(sizeof(short) * (size_t)ew * (size_t)eh);
    if (!e) return NULL;
    vo_ext_fill(e, plane, w, h, border);
    return e;
}

void vo_ext_fill(short* e, const short* plane, int w, int h, int border)
{
    int ew = w + 2 * border, eh = h + 2 * border;
    for (int y = 0; y < eh; y++) {
        int sy = y - border;
        if (sy < 0) sy = 0;
        if (sy > h - 1) sy = h - 1;
        const short* srow = plane + (size_t)sy * w;
        short* drow = e + (size_t)y * ew;
        for (int x = 0; x < ew; x++) {
            int sx = x - border;
            if (sx < 0) sx = 0;
            if (sx > w - 1) sx = w - 1;
            drow[x] = srow[sx];
        }
    }
}

/* OverlayMem2Dv2::SetOrigin (OverlayMem2Dv2.cpp:202-216): clamp the block
 * origin so the block stays inside the source. */
int vo_clamp_origin(int v, int src_len, int blk_len)
{
    if (v < 0) return 0;
    if (v > src_len - blk_len) return src_len - blk_len;
    return v;
}

/* OverlayMem2Dv2::Tsd16x16 (OverlayMem2Dv2.cpp:1623-1700). */
int vo_tsd16(const short* a, int as, const short* b, int bs)
{
    int acc = 0;
    for (int r = 0; r < 16; r++) {
        const short* pa = a + (size_t)r * as;
        const short* pb = b + (size_t)r * bs;
        for (int c = 0; c < 16; c++) {
            int d = (int)pa[c] - (int)pb[c];
            acc += d * d;
        }
    }
    return acc;
}

/* OverlayMem2Dv2::Tsd16x16LessThan (OverlayMem2Dv2.cpp:1923-1983): the running
 * sum is compared with `min` after every 4 columns and returned early once it
 * exceeds it.  The early value is only ever compared against `min`, so the
 * accept decision equals that of the full sum. */
int vo_tsd16_lt(const short* a, int as, const short* b, int bs, int min)
{
    int acc = 0;
    for (int r = 0; r < 16; r++) {
        const short* pa = a + (size_t)r * as;
        const short* pb = b + (size_t)r * bs;
        for (int c = 0; c < 16; c += 4) {
            for (int k = 0; k < 4; k++) {
                int d = (int)pa[c + k] - (int)pb[c + k];
                acc += d * d;
            }
            if (acc > min) return acc;
        }
    }
    return acc;
}

/* OverlayMem2Dv2::Tad16x16 (OverlayMem2Dv2.cpp:2655-2730): sum of |a-b|. */
int vo_tad16(const short* a, int as, const short* b, int bs)
{
    int acc = 0;
    for (int r = 0; r < 16; r++) {
        const short* pa = a + (size_t)r * as;
        const short* pb = b + (size_t)r * bs;
        for (int c = 0; c < 16; c++) {
            int d = (int)pa[c] - (int)pb[c];
            acc += d < 0 ? -d : d;
        }
    }
    return acc;
}

/* OverlayMem2Dv2::Tad16x16LessThan (OverlayMem2Dv2.cpp:2889-2960): the running
 * sum is tested against `min` after every sample (decision-neutral, as for
 * the squared form). */
int vo_tad16_lt(const short* a, int as, const short* b, int bs, int min)
{
    int acc = 0;
    for (int r = 0; r < 16; r++) {
        const short* pa = a + (size_t)r * as;
        const short* pb = b + (size_t)r * bs;
        for (int c = 0; c < 16; c++) {
            int d = (int)pa[c] - (int)pb[c];
            acc += d < 0 ? -d : d;
            if (acc > min) return acc;
        }
    }
    return acc;
}

/* Generic square distortion of an n x n block (Tsd4x4 / Tsd8x8,
 * OverlayMem2Dv2.cpp:1523-1622). */
int vo_tsd_n(const short* a, int as, const short* b, int bs, int n)
{
    int acc = 0;
    for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) {
            int d = (int)a[(size_t)r * as + c] - (int)b[(size_t)r * bs + c];
            acc += d * d;
        }
    return acc;
}

/* Phase order of the partial-distortion lattice (OverlayMem2Dv2.cpp:79-80):
 * phase p (1..16) visits the samples at (Tp[p] + 4i, Sp[p] + 4j). */
const int vo_phase_col[17] = {0, 0, 2, 2, 0, 1, 3, 3, 1, 1, 3, 0, 2, 3, 1, 2, 0};
const int vo_phase_row[17] = {0, 0, 2, 0, 2, 1, 3, 1, 3, 0, 2, 1, 3, 0, 2, 1, 3};

/* Tsd16x16PartialLessThan / Tsd8x8PartialLessThan (OverlayMem2Dv2.cpp:1886-1913,
 * 1993-2020) for an n x n block (n = 8 or 16): accumulate the phases in order
 * and reject as soon as 16 * D_p > p * min, returning 16 * D_p; otherwise
 * return the full sum.  Not decision-neutral: a candidate whose full sum is
 * below `min` can still be rejected by an early phase. */
int vo_tsd_partial_lt(const short* a, int as, const short* b, int bs, int n, int min)
{
    int dp = 0;
    for (int p = 1; p <= 16; p++) {
        int pr = vo_phase_row[p], pc = vo_phase_col[p];
        int pd = 0;
        for (int i = 0; i < n; i += 4)
            for (int j = 0; j < n; j += 4) {
                int d = (int)a[(size_t)(pr + i) * as + pc + j] - (int)b[(size_t)(pr + i) * bs + pc + j];
                pd += d * d;
            }
        dp += pd;
        if ((dp << 4) > p * min) return dp << 4;
    }
    return dp;
}

/* Tsd4x4LessThan (OverlayMem2Dv2.cpp:1739-1790): early exit checked after
 * each of the first three samples of a row and at the end of each row. */
int vo_tsd4_lt(const short* a, int as, const short* b, int bs, int min)
{
    int acc = 0;
    for (int r = 0; r < 4; r++) {
        for (int c = 0; c < 4; c++) {
            int d = (int)a[(size_t)r * as + c] - (int)b[(size_t)r * bs + c];
            acc += d * d;
            if (c < 3 && acc > min) return acc;
        }
    }
    return acc;
}

static inline int clip255(int x) { return x < 0 ? 0 : (x > 255 ? 255 : x); }

/* Unscaled 6-tap (1,-5,20,20,-5,1) through p[-2*st] .. p[3*st]
 * (OverlayMem2Dv2.cpp:92-94). */
static inline int tap6(const short* p, int st)
{
    return (int)p[-2 * st] - 5 * (int)p[-st] + 20 * (int)p[0] + 20 * (int)p[st]
           - 5 * (int)p[2 * st] + (int)p[3 * st];
}

/* Half-pel samples of an extended plane `e` (row stride es) at full-pel
 * position (x, y): b = right of (x,y), h = below, j = centre
 * (OverlayMem2Dv2.cpp:96-98, clipped as at every use in QuarterRead). */
int vo_hp_b(const short* e, int es, int x, int y)
{
    return clip255((tap6(e + (size_t)y * es + x, 1) + 16) >> 5);
}
int vo_hp_h(const short* e, int es, int x, int y)
{
    return clip255((tap6(e + (size_t)y * es + x, es) + 16) >> 5);
}
int vo_hp_j(const short* e, int es, int x, int y)
{
    int v[6];
    for (int k = -2; k <= 3; k++) v[k + 2] = tap6(e + (size_t)y * es + x + k, es);
    int s = v[0] - 5 * v[1] + 20 * v[2] + 20 * v[3] - 5 * v[4] + v[5];
    return clip255((s + 512) >> 10);
}

/* One sample of OverlayMem2Dv2::QuarterRead (OverlayMem2Dv2.cpp:704-1052) at
 * full-pel (x, y) of the extended plane with fractional part (fx, fy) in 0..3
 * (negative offsets are already folded into (x, y) by the caller). */
int vo_qpel_sample(const short* e, int es, int x, int y, int fx, int fy)
{
    int G = (int)e[(size_t)y * es + x];
    switch (fx | (fy << 2)) {
    case 0:  return G;
    case 2:  return vo_hp_b(e, es, x, y);                                          /* b */
    case 8:  return vo_hp_h(e, es, x, y);                                          /* h */
    case 10: return vo_hp_j(e, es, x, y);                                          /* j */
    case 1:  return (G + vo_hp_b(e, es, x, y) + 1) >> 1;                            /* a */
    case 3:  return ((int)e[(size_t)y * es + x + 1] + vo_hp_b(e, es, x, y) + 1) >> 1;  /* c */
    case 4:  return (G + vo_hp_h(e, es, x, y) + 1) >> 1;                            /* d */
    case 12: return ((int)e[(size_t)(y + 1) * es + x] + vo_hp_h(e, es, x, y) + 1) >> 1; /* n */
    case 6:  return (vo_hp_j(e, es, x, y) + vo_hp_b(e, es, x, y) + 1) >> 1;          /* f */
    case 14: return (vo_hp_j(e, es, x, y) + vo_hp_b(e, es, x, y + 1) + 1) >> 1;      /* q */
    case 9:  return (vo_hp_j(e, es, x, y) + vo_hp_h(e, es, x, y) + 1) >> 1;          /* i */
    case 11: return (vo_hp_j(e, es, x, y) + vo_hp_h(e, es, x + 1, y) + 1) >> 1;      /* k */
    case 5:  return (vo_hp_b(e, es, x, y) + vo_hp_h(e, es, x, y) + 1) >> 1;          /* e */
    case 7:  return (vo_hp_b(e, es, x, y) + vo_hp_h(e, es, x + 1, y) + 1) >> 1;      /* g */
    case 13: return (vo_hp_h(e, es, x, y) + vo_hp_b(e, es, x, y + 1) + 1) >> 1;      /* p */
    default: return (vo_hp_h(e, es, x + 1, y) + vo_hp_b(e, es, x, y + 1) + 1) >> 1;  /* r (15) */
    }
}

/* QuarterRead of a 16x16 block whose (already clamped) origin is (ox, oy) in
 * the extended plane, with quarter offsets (qx, qy) in -3..3. */
void vo_qread16_ext(const short* e, int es, int ox, int oy, int qx, int qy, short* dst)
{
    int fullx = 0, fracx = qx, fully = 0, fracy = qy;
    if (qx < 0) { fullx = -1; fracx = 4 + qx; }
    if (qy < 0) { fully = -1; fracy = 4 + qy; }
    for (int r = 0; r < 16; r++)
        for (int c = 0; c < 16; c++)
            dst[r * 16 + c] = (short)vo_qpel_sample(e, es, ox + c + fullx, oy + r + fully, fracx, fracy);
}

void vo_quarter_read16(const short* plane, int w, int h, int x, int y, int qx, int qy, short* dst)
{
    const int B = 24;
    short* e = vo_ext_alloc(plane, w, h, B);
    if (!e) return;
    vo_qread16_ext(e, w + 2 * B, x + B, y + B, qx, qy, dst);
    free(e);
}

/* OverlayMem2Dv2::Half (OverlayMem2Dv2.cpp:3018-3033). */
void vo_half(const short* src, int w, int h, short* dst)
{
    int hw = w / 2;
    for (int m = 0, y = 0; m < h; m += 2, y++)
        for (int n = 0, x = 0; n < w; n += 2, x++) {
            const short* p = src + (size_t)m * w + n;
            dst[(size_t)y * hw + x] = (short)(((int)p[0] + p[1] + p[w] + p[w + 1] + 2) >> 2);
        }
}
