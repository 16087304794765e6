/*
 * oracle_mc.c -- TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * Restatement of MotionCompensatorH264ImplStd (src/CodecUtils/
 * MotionCompensatorH264ImplStd.cpp) and the block add/subtract helpers of
 * OverlayMem2Dv2 used around it.
 *
 * Compensate(pMotionList) (…ImplStd.cpp:323-357) copies the reference into
 * edge-extended temporaries (PrepareForSingleVectorMode, :360-402; luma
 * border range + 1 + 4, chroma border range/2 + 4) and, macroblock by
 * macroblock in raster order, overwrites the reference with the block the
 * vector points at (:410-473): luma 16x16 by QuarterRead at the quarter-pel
 * vector (a copy for a full-pel one), chroma 8x8 of U and V by EighthRead at
 * the same vector in eighth-pel units (OverlayMem2Dv2.cpp:1063-1114: bilinear
 * weights (8-x)(8-y), x(8-y), (8-x)y, xy, (z + 32) >> 6, a negative fraction
 * taken from the sample to the left / above).  A zero vector leaves the block
 * as it is.  Only full macroblock rows are compensated: for a partial bottom
 * row the reference reads vectors past the end of its list.
 */
#include <stdlib.h>
#include <string.h>
#include "oracle_internal.h"

static int eighth_sample(const short* e, int es, int x, int y, int fx, int fy)
{
    const short* p = e + (size_t)y * es + x;
    const int z = (8 - fx) * (8 - fy) * p[0] + fx * (8 - fy) * p[1] + (8 - fx) * fy * p[es] + fx * fy * p[es + 1];
    return (z + 32) >> 6;
}

int vo_mc_compensate(short* yuv, int w, int h, int range, const short* mv)
{
    if (!yuv || !mv || w < 16 || h < 16 || (w % 16) != 0 || range < 0) return -1;
    const int cw = w / 2, ch = h / 2, lb = range + 1 + 4, cb = range / 2 + 4;
    short* Y = yuv;
    short* U = yuv + (size_t)w * h;
    short* V = U + (size_t)cw * ch;
    short* eY = vo_ext_alloc(Y, w, h, lb);
    short* eU = vo_ext_alloc(U, cw, ch, cb);
    short* eV = vo_ext_alloc(V, cw, ch, cb);
    if (!eY || !eU || !eV) {
        free(eY);
        free(eU);
        free(eV);
        return -2;
    }
    const int les = w + 2 * lb, ces = cw + 2 * cb, cols = w / 16, rows = h / 16;
    short blk[256];
    for (int k = 0; k < cols * rows; k++) {
        const int n = (k % cols) * 16, m = (k / cols) * 16;
        const int mvx = mv[2 * k], mvy = mv[2 * k + 1];
        if (!mvx && !mvy) continue;
        /* luma: full-pel part by C division, the C remainder to QuarterRead */
        const int qx = mvx % 4, qy = mvy % 4, fx = mvx / 4, fy = mvy / 4;
        vo_qread16_ext(eY, les, n + fx + lb, m + fy + lb, qx, qy, blk);
        for (int r = 0; r < 16; r++) memcpy(Y + (size_t)(m + r) * w + n, blk + 16 * r, 32);
        /* chroma: eighth-pel */
        const int ex = mvx % 8, ey = mvy % 8, cx = n / 2 + mvx / 8, cy = m / 2 + mvy / 8;
        const int ox = ex < 0 ? -1 : 0, oy = ey < 0 ? -1 : 0, frx = ex < 0 ? ex + 8 : ex, fry = ey < 0 ? ey + 8 : ey;
        for (int pl = 0; pl < 2; pl++) {
            const short* e = pl ? eV : eU;
            short* d = pl ? V : U;
            for (int r = 0; r < 8; r++)
                for (int c = 0; c < 8; c++) {
                    const int x = cx + c + cb, y = cy + r + cb;
                    d[(size_t)(m / 2 + r) * cw + n / 2 + c] =
                        (short)((frx || fry) ? eighth_sample(e, ces, x + ox, y + oy, frx, fry) : e[(size_t)y * ces + x]);
                }
        }
    }
    free(eY);
    free(eU);
    free(eV);
    return 0;
}

/* OverlayMem2Dv2::Add16x16WithClip255 / Add8x8WithClip255 (OverlayMem2Dv2.cpp:1343-1426)
 * over n samples: a = clip255(a + b). */
void vo_add_clip255(short* a, const short* b, long long n)
{
    for (long long i = 0; i < n; i++) {
        const int v = a[i] + b[i];
        a[i] = (short)(v < 0 ? 0 : (v > 255 ? 255 : v));
    }
}

/* OverlayMem2Dv2::Sub16x16 / Sub8x8 (OverlayMem2Dv2.cpp:1195-1240) over n samples: a -= b. */
void vo_sub(short* a, const short* b, long long n)
{
    for (long long i = 0; i < n; i++) a[i] = (short)(a[i] - b[i]);
}
