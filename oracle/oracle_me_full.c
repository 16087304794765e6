/*
 * oracle_me_full.c -- TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * Restatement of MotionEstimatorH264ImplFull::Estimate
 * (src/CodecUtils/MotionEstimatorH264ImplFull.cpp:330-613) and the median
 * predictor it drives (H264MotionVectorPredictorImpl1 over MacroBlockH264).
 * Build without FMA contraction (-ffp-contract=off): GetBestVector is IEEE
 * double arithmetic and must be evaluated one rounded operation at a time.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle_internal.h"

#define MB 16
#define EXT_BORDER (MB + 3) /* macroblock + MEH264IF_PADDING (Full.cpp:71,244) */

int vo_num_mbs(int w, int h) { return (w / MB) * (h / MB); }

/* ------------------------------------------------------------------------ */
/* Median predictor                                                          */
/* ------------------------------------------------------------------------ */

/* MacroBlockH264::Median (MacroBlockH264.cpp:923-936). */
int vo_median3(int x, int y, int z)
{
    int lo, hi;
    if (y - z < 0) { lo = y; hi = z; } else { lo = z; hi = y; }
    if (x < lo) lo = x;
    if (x > hi) hi = x;
    return x + y + z - lo - hi;
}

int vo_pred_init(vo_pred_state* st, int cols, int rows, const int* slice)
{
    st->cols = cols;
    st->rows = rows;
    st->slice = slice;
    st->mvx = (int*)calloc((size_t)cols * rows, sizeof(int));
    st->mvy = (int*)calloc((size_t)cols * rows, sizeof(int));
    return (st->mvx && st->mvy) ? 0 : -1;
}

void vo_pred_free(vo_pred_state* st)
{
    free(st->mvx);
    free(st->mvy);
    st->mvx = st->mvy = NULL;
}

static int nb_avail(const vo_pred_state* st, int k, int r, int c)
{
    if (r < 0 || c < 0 || c >= st->cols) return -1;
    int n = r * st->cols + c;
    if (st->slice && st->slice[n] != st->slice[k]) return -1;
    return n;
}

/* MacroBlockH264::GetMbMotionMedianPred (MacroBlockH264.cpp:757-816): A = left,
 * B = above, C = above-right (D = above-left when C is missing); a missing
 * neighbour contributes (0,0); with neither B nor C, B and C take A.  Every
 * neighbour of a macroblock precedes it in raster order, so within one
 * Estimate() call it has already been given its final vector and is inter. */
void vo_pred_get(const vo_pred_state* st, int k, int* px, int* py)
{
    int r = k / st->cols, c = k % st->cols;
    int a = nb_avail(st, k, r, c - 1);
    int b = nb_avail(st, k, r - 1, c);
    int cc = nb_avail(st, k, r - 1, c + 1);
    int ax = 0, ay = 0, bx = 0, by = 0, cx = 0, cy = 0;
    if (a >= 0) { ax = st->mvx[a]; ay = st->mvy[a]; }
    if (b >= 0) { bx = st->mvx[b]; by = st->mvy[b]; }
    if (cc >= 0) { cx = st->mvx[cc]; cy = st->mvy[cc]; }
    else {
        int d = nb_avail(st, k, r - 1, c - 1);
        if (d >= 0) { cx = st->mvx[d]; cy = st->mvy[d]; }
    }
    if (b < 0 && cc < 0) { bx = cx = ax; by = cy = ay; }
    *px = vo_median3(ax, bx, cx);
    *py = vo_median3(ay, by, cy);
}

/* H264MotionVectorPredictorImpl1::Set16x16MotionVector (…Impl1.h:103-111). */
void vo_pred_set(vo_pred_state* st, int k, int mvx, int mvy)
{
    st->mvx[k] = mvx;
    st->mvy[k] = mvy;
}

/* GetBestVector over the Fifo contents (Full.h:140-168): cost = D/norm +
 * lambda*sqrt(|v-ref|^2), strict improvement, scanning from slot 0. */
int vo_best_vector5(const int* xs, const int* ys, const int* ds, double lambda, double norm,
                    int xref, int yref)
{
    int pos = 0;
    double mag = (double)((xs[0] - xref) * (xs[0] - xref) + (ys[0] - yref) * (ys[0] - yref));
    double cost = ((double)ds[0] / norm) + (lambda * sqrt(mag));
    for (int i = 1; i < 5; i++) {
        double m = (double)((xs[i] - xref) * (xs[i] - xref) + (ys[i] - yref) * (ys[i] - yref));
        double c = ((double)ds[i] / norm) + (lambda * sqrt(m));
        if (c < cost) { cost = c; pos = i; }
    }
    return pos;
}

/* ------------------------------------------------------------------------ */
/* Search range                                                              */
/* ------------------------------------------------------------------------ */

/* MotionEstimatorH264ImplFull::GetMotionRange with zero offset
 * (Full.cpp:1029-1081): the vector magnitude is limited to vecRange-1 and the
 * block may reach at most `MB` pels outside the picture. */
static void full_range(int x, int y, int w, int h, int motion_range, int range,
                       int* xl, int* xr, int* yu, int* yd)
{
    const int boundary = EXT_BORDER - 3;
    int vec_range = motion_range / 4;
    int lr = (-range > -vec_range) ? range : vec_range - 1;
    int rr = (range < vec_range) ? range : vec_range - 1;
    *xl = (x - lr >= -boundary) ? -lr : -(x + boundary);
    *xr = (x + rr < w) ? rr : w - x;
    *yu = (y - lr >= -boundary) ? -lr : -(y + boundary);
    *yd = (y + rr < h) ? rr : h - y;
}

/* ------------------------------------------------------------------------ */
/* Sub-pel window                                                            */
/* ------------------------------------------------------------------------ */
/* LoadHalfQuartPelWindow / LoadQuartPelWindow / QuarterRead of the window
 * (Full.cpp:1095-1255), restated with explicit sample planes.  Coordinates
 * are in quarter pels relative to the best full-pel block origin (ox, oy) of
 * the extended reference.  Even positions hold G (full), h (vertical half),
 * b (horizontal half) and j (centre half) samples, computed once per
 * macroblock as the reference's window is; odd positions around the winning
 * half-pel point are rounded averages of two even neighbours. */
typedef struct {
    const short* e;
    int es, ox, oy;
    short h[17][18]; /* fy in [-1,15], fx in [-1,16] */
    short b[18][17]; /* fy in [-1,16], fx in [-1,15] */
    short j[17][17]; /* fy,fx in [-1,15] */
} subpel_win;

static void win_load(subpel_win* w, const short* e, int es, int ox, int oy)
{
    w->e = e;
    w->es = es;
    w->ox = ox;
    w->oy = oy;
    for (int fy = -1; fy <= 15; fy++)
        for (int fx = -1; fx <= 16; fx++) w->h[fy + 1][fx + 1] = (short)vo_hp_h(e, es, ox + fx, oy + fy);
    for (int fy = -1; fy <= 16; fy++)
        for (int fx = -1; fx <= 15; fx++) w->b[fy + 1][fx + 1] = (short)vo_hp_b(e, es, ox + fx, oy + fy);
    for (int fy = -1; fy <= 15; fy++)
        for (int fx = -1; fx <= 15; fx++) w->j[fy + 1][fx + 1] = (short)vo_hp_j(e, es, ox + fx, oy + fy);
}

static int floordiv4(int v) { return v >= 0 ? v / 4 : -((-v + 3) / 4); }

static int win_even(const subpel_win* w, int qy, int qx)
{
    int fy = floordiv4(qy), fx = floordiv4(qx);
    int ry = qy - 4 * fy, rx = qx - 4 * fx;
    if (ry == 0 && rx == 0) return w->e[(size_t)(w->oy + fy) * w->es + w->ox + fx];
    if (ry == 2 && rx == 0) return w->h[fy + 1][fx + 1];
    if (ry == 0 && rx == 2) return w->b[fy + 1][fx + 1];
    return w->j[fy + 1][fx + 1];
}

/* Quarter sample at offset (sy, sx) in -1..1 around the even point (cy, cx),
 * following the eight assignments of LoadQuartPelWindow (Full.cpp:1207-1220). */
static int win_quarter(const subpel_win* w, int cy, int cx, int sy, int sx)
{
    int a, b;
    if (sy < 0) {
        if (sx < 0) { a = win_even(w, cy - 2, cx - 2); b = win_even(w, cy, cx); }
        else if (sx == 0) { a = win_even(w, cy - 2, cx); b = win_even(w, cy, cx); }
        else { a = win_even(w, cy - 2, cx); b = win_even(w, cy, cx + 2); }
    } else if (sy == 0) {
        if (sx < 0) { a = win_even(w, cy, cx - 2); b = win_even(w, cy, cx); }
        else { a = win_even(w, cy, cx + 2); b = win_even(w, cy, cx); }
    } else {
        if (sx < 0) { a = win_even(w, cy, cx - 2); b = win_even(w, cy + 2, cx); }
        else if (sx == 0) { a = win_even(w, cy + 2, cx); b = win_even(w, cy, cx); }
        else { a = win_even(w, cy + 2, cx); b = win_even(w, cy, cx + 2); }
    }
    return (a + b + 1) >> 1;
}

/* Neighbour order of the sub-pel passes (MEH264IF_SubPos, Full.cpp:77-81). */
static const int SUB_X[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
static const int SUB_Y[8] = {-1, -1, -1, 0, 0, 1, 1, 1};

/* Half-pel pass then quarter-pel pass around the full-pel winner at ext
 * origin (ox, oy) (Full.cpp:452-517).  *min_d enters as the full-pel minimum
 * and leaves as the refined one; returns the quarter-pel refinement.
 * quarter == 0: the half-pel pass only (a half-pel SetMode). */
static void subpel_refine(const short* in, int ins, const short* e, int es, int ox, int oy, int quarter,
                          int* min_d, int* qmx, int* qmy)
{
    subpel_win w;
    win_load(&w, e, es, ox, oy);
    short blk[256];
    int hmx = 0, hmy = 0, best = *min_d;
    for (int k = 0; k < 8; k++) {
        int qx = 2 * SUB_X[k], qy = 2 * SUB_Y[k];
        for (int r = 0; r < 16; r++)
            for (int c = 0; c < 16; c++)
                blk[r * 16 + c] = (short)win_even(&w, 4 * r + qy, 4 * c + qx);
        int d = vo_tsd16_lt(in, ins, blk, 16, best);
        if (d < best) { best = d; hmx = qx; hmy = qy; }
    }
    int bx = hmx, by = hmy;
    for (int k = 0; quarter && k < 8; k++) {
        for (int r = 0; r < 16; r++)
            for (int c = 0; c < 16; c++)
                blk[r * 16 + c] = (short)win_quarter(&w, 4 * r + hmy, 4 * c + hmx, SUB_Y[k], SUB_X[k]);
        int d = vo_tsd16_lt(in, ins, blk, 16, best);
        if (d < best) { best = d; bx = hmx + SUB_X[k]; by = hmy + SUB_Y[k]; }
    }
    *min_d = best;
    *qmx = bx;
    *qmy = by;
}

/* ------------------------------------------------------------------------ */
/* Integer-pel scan                                                          */
/* ------------------------------------------------------------------------ */
/* Full.cpp:394-446: raster scan of the range; (0,0) is the start point; a
 * candidate is skipped when, shifted by the current best vector, it would
 * leave the range; ties go to the candidate nearer the rounded prediction. */
static int int_scan(const short* in, int ins, const short* e, int es, int w, int h,
                    int n, int m, int motion_range, int metric, int prx, int pry,
                    int* zero_d, int* bx, int* by)
{
    int xl, xr, yu, yd;
    int eox = vo_clamp_origin(n + EXT_BORDER, w + 2 * EXT_BORDER, MB);
    int eoy = vo_clamp_origin(m + EXT_BORDER, h + 2 * EXT_BORDER, MB);
    const short* blk0 = e + (size_t)eoy * es + eox;
    int zd = metric ? vo_tad16(in, ins, blk0, es) : vo_tsd16(in, ins, blk0, es);
    int min_d = zd, mx = 0, my = 0;
    full_range(n, m, w, h, motion_range, motion_range / 4, &xl, &xr, &yu, &yd);
    for (int i = yu; i <= yd; i++) {
        for (int j = xl; j <= xr; j++) {
            if (i == 0 && j == 0) continue;
            if (i + my < yu || i + my > yd || j + mx < xl || j + mx > xr) continue;
            int ox = vo_clamp_origin(n + j + EXT_BORDER, w + 2 * EXT_BORDER, MB);
            int oy = vo_clamp_origin(m + i + EXT_BORDER, h + 2 * EXT_BORDER, MB);
            const short* cand = e + (size_t)oy * es + ox;
            int d = metric ? vo_tad16_lt(in, ins, cand, es, min_d) : vo_tsd16_lt(in, ins, cand, es, min_d);
            if (d > min_d) continue;
            if (d == min_d) {
                int cxo = mx - prx, cyo = my - pry, nxo = j - prx, nyo = i - pry;
                if ((cyo * cyo + cxo * cxo) - (nyo * nyo + nxo * nxo) < 0) continue;
            }
            min_d = d;
            mx = j;
            my = i;
        }
    }
    *zero_d = zd;
    *bx = mx;
    *by = my;
    return min_d;
}

/* Nearest full-pel prediction, C integer division (Full.cpp:368-380). */
static int round_pred(int p) { return p < 0 ? (p - 2) / 4 : (p + 2) / 4; }

int vo_me_full_detail(const short* src, const short* ref, int w, int h, int motion_range,
                      const unsigned char* dist_incl, const int* slice,
                      short* mv_out, int* mb_dist, long* avg_dist,
                      int* int_mv, int* sub_mv, int* min_dv, int* zero_dv,
                      int* pred_mv, int* pred_dv)
{
    if (!src || !ref || !mv_out || w < MB || h < MB || (w % MB) != 0 || motion_range < 4)
        return -1;
    int cols = w / MB, rows = h / MB, nmb = cols * rows;
    int es = w + 2 * EXT_BORDER;
    short* e = vo_ext_alloc(ref, w, h, EXT_BORDER);
    vo_pred_state ps;
    if (!e || vo_pred_init(&ps, cols, rows, slice) != 0) {
        free(e);
        vo_pred_free(&ps);
        return -2;
    }
    long total = 0;
    int included = 0;
    for (int k = 0; k < nmb; k++) {
        int n = (k % cols) * MB, m = (k / cols) * MB;
        const short* in = src + (size_t)vo_clamp_origin(m, h, MB) * w + vo_clamp_origin(n, w, MB);

        int px, py;
        vo_pred_get(&ps, k, &px, &py);
        int pxq = px % 4, pyq = py % 4, px0 = px / 4, py0 = py / 4;

        int zd, mx, my;
        int min_d = int_scan(in, w, e, es, w, h, n, m, motion_range, 0,
                             round_pred(px), round_pred(py), &zd, &mx, &my);
        if (int_mv) { int_mv[2 * k] = mx; int_mv[2 * k + 1] = my; }

        int ox = vo_clamp_origin(n + mx + EXT_BORDER, es, MB);
        int oy = vo_clamp_origin(m + my + EXT_BORDER, h + 2 * EXT_BORDER, MB);
        int qmx, qmy;
        subpel_refine(in, w, e, es, ox, oy, 1, &min_d, &qmx, &qmy);
        int mvx = 4 * mx + qmx, mvy = 4 * my + qmy;
        if (sub_mv) { sub_mv[2 * k] = mvx; sub_mv[2 * k + 1] = mvy; }
        if (min_dv) min_dv[k] = min_d;
        if (zero_dv) zero_dv[k] = zd;

        /* Prediction clamped to one macroblock outside the picture (Full.cpp:532-541). */
        if (px0 + n > w) px0 = MB;
        if (px0 + n < -MB) px0 = -MB;
        if (py0 + m > h) py0 = MB;
        if (py0 + m < -MB) py0 = -MB;
        px = 4 * px0 + pxq;
        py = 4 * py0 + pyq;
        int pox = vo_clamp_origin(px0 + n + EXT_BORDER, es, MB);
        int poy = vo_clamp_origin(py0 + m + EXT_BORDER, h + 2 * EXT_BORDER, MB);
        int pd;
        if (pxq || pyq) {
            short blk[256];
            vo_qread16_ext(e, es, pox, poy, pxq, pyq, blk);
            pd = vo_tsd16(in, w, blk, 16);
        } else {
            pd = vo_tsd16(in, w, e + (size_t)poy * es + pox, es);
        }
        if (pred_mv) { pred_mv[2 * k] = px; pred_mv[2 * k + 1] = py; }
        if (pred_dv) pred_dv[k] = pd;

        /* Fifo after pushing zero, pred, best (Full.cpp:573-576; Fifo.h:74-94). */
        int xs[5] = {mvx, px, 0, 0, 0}, ys[5] = {mvy, py, 0, 0, 0}, ds[5] = {min_d, pd, zd, zd, zd};
        int pos = vo_best_vector5(xs, ys, ds, 1.05, 256.0, px, py);
        mvx = xs[pos];
        mvy = ys[pos];
        if (dist_incl && dist_incl[k]) {
            included++;
            total += ds[pos];
        }
        if (mb_dist) mb_dist[k] = ds[pos];
        mv_out[2 * k] = (short)mvx;
        mv_out[2 * k + 1] = (short)mvy;
        vo_pred_set(&ps, k, mvx, mvy);
    }
    if (avg_dist) *avg_dist = included ? total / included : 0;
    vo_pred_free(&ps);
    free(e);
    return 0;
}

int vo_me_full(const short* src, const short* ref, int w, int h, int motion_range,
               const unsigned char* dist_incl, const int* slice,
               short* mv_out, int* mb_dist, long* avg_dist)
{
    return vo_me_full_detail(src, ref, w, h, motion_range, dist_incl, slice, mv_out, mb_dist,
                             avg_dist, NULL, NULL, NULL, NULL, NULL, NULL);
}

int vo_me_full_intpel(const short* src, const short* ref, int w, int h, int motion_range,
                      int metric, short* mv_out, int* mb_dist)
{
    if (!src || !ref || !mv_out || w < MB || h < MB || (w % MB) != 0 || motion_range < 4)
        return -1;
    int cols = w / MB, rows = h / MB, nmb = cols * rows;
    int es = w + 2 * EXT_BORDER;
    short* e = vo_ext_alloc(ref, w, h, EXT_BORDER);
    vo_pred_state ps;
    if (!e || vo_pred_init(&ps, cols, rows, NULL) != 0) {
        free(e);
        vo_pred_free(&ps);
        return -2;
    }
    for (int k = 0; k < nmb; k++) {
        int n = (k % cols) * MB, m = (k / cols) * MB;
        const short* in = src + (size_t)vo_clamp_origin(m, h, MB) * w + vo_clamp_origin(n, w, MB);
        int px, py, zd, mx, my;
        vo_pred_get(&ps, k, &px, &py);
        int d = int_scan(in, w, e, es, w, h, n, m, motion_range, metric,
                         round_pred(px), round_pred(py), &zd, &mx, &my);
        mv_out[2 * k] = (short)(4 * mx);
        mv_out[2 * k + 1] = (short)(4 * my);
        if (mb_dist) mb_dist[k] = d;
        vo_pred_set(&ps, k, 4 * mx, 4 * my);
    }
    vo_pred_free(&ps);
    free(e);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* MotionEstimatorH264ImplCross                                              */
/* ------------------------------------------------------------------------ */
/* The first 64 points of MotionEstimatorH264ImplCross::MEH264IC_OptimalPath
 * (MotionEstimatorH264ImplCross.cpp:89-98), {x, y} within the macroblock:
 * the distortion of this estimator is the SSD over these points only
 * (_pathLength = 64, MotionEstimatorH264ImplCross.cpp:226). */
static const signed char CROSS_PATH[64][2] = {
    {5, 10}, {13, 5}, {2, 1},   {13, 14}, {1, 14},  {9, 1},   {1, 6},   {15, 9},  {8, 13},  {14, 2},  {7, 4},
    {10, 8}, {4, 15}, {0, 10},  {0, 3},   {5, 0},   {12, 11}, {4, 7},   {12, 0},  {10, 14}, {3, 12},  {10, 5},
    {15, 13}, {4, 3}, {7, 8},   {14, 7},  {6, 13},  {11, 3},  {2, 9},   {9, 10},  {15, 1},  {7, 2},   {3, 5},
    {8, 15}, {1, 12}, {8, 6},   {0, 1},   {12, 9},  {14, 15}, {15, 4},  {11, 12}, {6, 6},   {7, 11},  {0, 7},
    {14, 11}, {7, 0}, {2, 15},  {12, 7},  {2, 3},   {4, 9},   {12, 2},  {9, 3},   {12, 13}, {3, 0},   {5, 14},
    {5, 4},  {0, 13}, {8, 9},   {2, 11},  {11, 15}, {10, 1},  {2, 7},   {15, 6},  {9, 12}};

/* OverlayMem2Dv2::Tsd16x16PartialPath over the 64 path points (OverlayMem2Dv2.cpp:2495-2517). */
static int cross_path_sd(const short* a, int as, const short* b, int bs)
{
    int d = 0;
    for (int p = 0; p < 64; p++) {
        const int x = CROSS_PATH[p][0], y = CROSS_PATH[p][1];
        const int e = a[(size_t)y * as + x] - b[(size_t)y * bs + x];
        d += e * e;
    }
    return d;
}

/* OverlayMem2Dv2::Tsd16x16PartialPathLessThan with batch length 16
 * (OverlayMem2Dv2.cpp:2449-2493): after each batch of 16 path points the
 * final distortion is predicted as Dp * 4 / batches-done; the first
 * prediction above `min` is returned (early exit), else the full 64-point SSD. */
static int cross_path_lt(const short* a, int as, const short* b, int bs, int min)
{
    int dp = 0, expected = 0;
    for (int batch = 0; batch < 4 && expected <= min; batch++) {
        for (int p = 16 * batch; p < 16 * batch + 16; p++) {
            const int x = CROSS_PATH[p][0], y = CROSS_PATH[p][1];
            const int e = a[(size_t)y * as + x] - b[(size_t)y * bs + x];
            dp += e * e;
        }
        expected = (dp * 4) / (batch + 1);
    }
    return expected;
}

/* The half-pel then quarter-pel passes of MotionEstimatorH264ImplCross::Estimate
 * (MotionEstimatorH264ImplCross.cpp:492-560): the window of the full-search
 * estimator (the same LoadHalfQuartPelWindow / LoadQuartPelWindow /
 * QuarterRead), candidates compared with the path LessThan, strict
 * improvement; mode 1 stops after the half-pel pass. */
static void cross_subpel(const short* in, int ins, const short* e, int es, int ox, int oy, int mode, int* min_d,
                         int* qmx, int* qmy)
{
    subpel_win w;
    win_load(&w, e, es, ox, oy);
    short blk[256];
    int hmx = 0, hmy = 0, best = *min_d;
    for (int k = 0; k < 8; k++) {
        int qx = 2 * SUB_X[k], qy = 2 * SUB_Y[k];
        for (int r = 0; r < 16; r++)
            for (int c = 0; c < 16; c++) blk[r * 16 + c] = (short)win_even(&w, 4 * r + qy, 4 * c + qx);
        int d = cross_path_lt(in, ins, blk, 16, best);
        if (d < best) { best = d; hmx = qx; hmy = qy; }
    }
    int bx = hmx, by = hmy;
    if (mode != 1) {
        for (int k = 0; k < 8; k++) {
            for (int r = 0; r < 16; r++)
                for (int c = 0; c < 16; c++)
                    blk[r * 16 + c] = (short)win_quarter(&w, 4 * r + hmy, 4 * c + hmx, SUB_Y[k], SUB_X[k]);
            int d = cross_path_lt(in, ins, blk, 16, best);
            if (d < best) { best = d; bx = hmx + SUB_X[k]; by = hmy + SUB_Y[k]; }
        }
    }
    *min_d = best;
    *qmx = bx;
    *qmy = by;
}

/* Cross positions in test order (MEH264IC_CrossPos, MotionEstimatorH264ImplCross.cpp:83-87). */
static const int CROSS_X[4] = {-1, 1, 0, 0};
static const int CROSS_Y[4] = {0, 0, -1, 1};

/* MotionEstimatorH264ImplCross::Estimate (MotionEstimatorH264ImplCross.cpp:354-649):
 * a full-pel cross search with steps mRng/2, mRng/4, .., 1 (mRng = motion
 * range in pels) around the running winner, the four cross points tested in
 * order against the step's running best (ties to the point not farther from
 * the rounded prediction), the sub-pel passes, then GetBestVector of (best,
 * prediction, zero) with lambda 0.9 and norm 64.  mode 0 quarter, 1 half,
 * 2 full pel.  A partial bottom macroblock row is not computed (its vectors
 * are dropped by the reference). */
int vo_me_cross(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                const unsigned char* dist_incl, const int* slice, short* mv_out, int* mb_dist, long* avg_dist,
                int* tie_out)
{
    if (!src || !ref || !mv_out || w < MB || h < MB || (w % MB) != 0 || motion_range < 4) return -1;
    int cols = w / MB, rows = h / MB, nmb = cols * rows;
    int es = w + 2 * EXT_BORDER;
    short* e = vo_ext_alloc(ref, w, h, EXT_BORDER);
    vo_pred_state ps;
    if (!e || vo_pred_init(&ps, cols, rows, slice) != 0) {
        free(e);
        vo_pred_free(&ps);
        return -2;
    }
    const int mrng = motion_range / 4;
    long total = 0;
    int included = 0;
    for (int k = 0; k < nmb; k++) {
        int n = (k % cols) * MB, m = (k / cols) * MB;
        const short* in = src + (size_t)m * w + n;
        int px, py;
        vo_pred_get(&ps, k, &px, &py);
        const int pxq = px % 4, pyq = py % 4;
        int px0 = px / 4, py0 = py / 4;
        const int prx = round_pred(px), pry = round_pred(py);

        const int eox = n + EXT_BORDER, eoy = m + EXT_BORDER;
        const int zd = cross_path_sd(in, w, e + (size_t)eoy * es + eox, es);
        int min_d = zd, mx = 0, my = 0, tie = 0;
        int xl, xr, yu, yd;
        full_range(n, m, w, h, motion_range, mrng, &xl, &xr, &yu, &yd);
        for (int step = mrng / 2; step > 0; step /= 2) {
            int rmx = 0, rmy = 0;
            for (int c = 0; c < 4; c++) {
                const int i = step * CROSS_Y[c], j = step * CROSS_X[c];
                if (i + my < yu || i + my > yd || j + mx < xl || j + mx > xr) continue;
                const short* cand = e + (size_t)(eoy + my + i) * es + eox + mx + j;
                const int d = cross_path_lt(in, w, cand, es, min_d);
                if (d > min_d) continue;
                if (d == min_d) {
                    tie = 1;
                    const int cxo = mx + rmx - prx, cyo = my + rmy - pry, nxo = mx + j - prx, nyo = my + i - pry;
                    if ((cyo * cyo + cxo * cxo) - (nyo * nyo + nxo * nxo) < 0) continue;
                }
                min_d = d;
                rmx = j;
                rmy = i;
            }
            mx += rmx;
            my += rmy;
        }
        int mvx = 4 * mx, mvy = 4 * my;
        if (mode != 2) {
            int qmx, qmy;
            cross_subpel(in, w, e, es, eox + mx, eoy + my, mode, &min_d, &qmx, &qmy);
            mvx += qmx;
            mvy += qmy;
        }
        /* prediction clamped to one macroblock outside the picture (MotionEstimatorH264ImplCross.cpp:574-583) */
        if (px0 + n > w) px0 = MB;
        if (px0 + n < -MB) px0 = -MB;
        if (py0 + m > h) py0 = MB;
        if (py0 + m < -MB) py0 = -MB;
        px = 4 * px0 + pxq;
        py = 4 * py0 + pyq;
        const int pox = vo_clamp_origin(px0 + n + EXT_BORDER, es, MB);
        const int poy = vo_clamp_origin(py0 + m + EXT_BORDER, h + 2 * EXT_BORDER, MB);
        int pd;
        if (pxq || pyq) {
            short blk[256];
            vo_qread16_ext(e, es, pox, poy, pxq, pyq, blk);
            pd = cross_path_sd(in, w, blk, 16);
        } else {
            pd = cross_path_sd(in, w, e + (size_t)poy * es + pox, es);
        }
        int xs[5] = {mvx, px, 0, 0, 0}, ys[5] = {mvy, py, 0, 0, 0}, ds[5] = {min_d, pd, zd, zd, zd};
        int pos = vo_best_vector5(xs, ys, ds, 0.9, 64.0, px, py);
        mvx = xs[pos];
        mvy = ys[pos];
        if (dist_incl && dist_incl[k]) {
            included++;
            total += ds[pos];
        }
        if (mb_dist) mb_dist[k] = ds[pos];
        if (tie_out) tie_out[k] = tie;
        mv_out[2 * k] = (short)mvx;
        mv_out[2 * k + 1] = (short)mvy;
        vo_pred_set(&ps, k, mvx, mvy);
    }
    if (avg_dist) *avg_dist = included ? total / included : 0;
    vo_pred_free(&ps);
    free(e);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* MotionEstimatorH264ImplUMHS                                               */
/* ------------------------------------------------------------------------ */
/* Pattern tables of MotionEstimatorH264ImplUMHS.cpp:82-122, {x, y} offsets in
 * the order the reference tests them. */
static const signed char UMHS_5X5[24][2] = {
    {-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1}, {0, -2}, {-2, 0}, {2, 0}, {0, 2},
    {-1, -2}, {1, -2}, {-2, -1}, {2, -1}, {-2, 1}, {2, 1}, {-1, 2}, {1, 2}, {-2, -2}, {2, -2}, {-2, 2}, {2, 2}};
static const signed char UMHS_CROSS[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
static const signed char UMHS_HEX[16][2] = {{-4, 0}, {4, 0},  {-4, 1}, {4, 1},  {-4, -1}, {4, -1}, {-4, 2}, {4, 2},
                                            {-4, -2}, {4, -2}, {-2, 3}, {2, 3}, {-2, -3}, {2, -3}, {0, 4},  {0, -4}};
static const signed char UMHS_EXTHEX[6][2] = {{-2, 0}, {-1, -2}, {1, -2}, {2, 0}, {1, 2}, {-1, 2}};

/* MEH264IUMHS_COST (MotionEstimatorH264ImplUMHS.cpp:179): D/256 plus 1.05 x the
 * Euclidean distance to the reference vector, in double, truncated to int. */
static int umhs_cost(int d, int x, int y, int xr, int yr)
{
    const double mag = sqrt((double)((x - xr) * (x - xr) + (y - yr) * (y - yr)));
    return (int)(((double)d / 256.0) + (1.05 * mag));
}

/* MacroBlockH264::GetMbMotionMedianPred with the distortion output
 * (MacroBlockH264.cpp:818-915): the median vector of A, B, C (D for a missing
 * C; B and C take A when both are missing), and the smaller of the
 * distortions attached to each median component: among the neighbours whose
 * component equals the median, A first, then B and C if smaller.  The y
 * component compares C's x component with the median (MacroBlockH264.cpp:898),
 * kept as it is. */
static void umhs_pred_get(const vo_pred_state* st, const int* dist, int k, int* px, int* py, int* pd)
{
    int r = k / st->cols, c = k % st->cols;
    int a = nb_avail(st, k, r, c - 1);
    int b = nb_avail(st, k, r - 1, c);
    int cc = nb_avail(st, k, r - 1, c + 1);
    int ax = 0, ay = 0, ad = 0, bx = 0, by = 0, bd = 0, cx = 0, cy = 0, cd = 0;
    if (a >= 0) { ax = st->mvx[a]; ay = st->mvy[a]; ad = dist[a]; }
    if (b >= 0) { bx = st->mvx[b]; by = st->mvy[b]; bd = dist[b]; }
    if (cc >= 0) { cx = st->mvx[cc]; cy = st->mvy[cc]; cd = dist[cc]; }
    else {
        int d = nb_avail(st, k, r - 1, c - 1);
        if (d >= 0) { cx = st->mvx[d]; cy = st->mvy[d]; cd = dist[d]; }
    }
    if (b < 0 && cc < 0) { bx = cx = ax; by = cy = ay; bd = cd = ad; }
    const int x = vo_median3(ax, bx, cx), y = vo_median3(ay, by, cy);
    int xd = ad;
    if (x == bx && bd < xd) xd = bd;
    if (x == cx && cd < xd) xd = cd;
    int yd = ad;
    if (y == by && bd < yd) yd = bd;
    if (y == cx && cd < yd) yd = cd;
    *px = x;
    *py = y;
    *pd = yd < xd ? yd : xd;
}

/* State of one macroblock's UMHS search: the running best (its distortion
 * and cost), the pattern centre and the refinement offset from it. */
typedef struct {
    const short* in;
    int ins;
    const short* e;
    int es, w, h, n, m;
    int xl, xr, yu, yd;
    int px0, py0;  /* full-pel prediction after truncation: the cost reference */
    int mx, my, rmx, rmy, min_d, min_cost;
} umhs_search;

static int umhs_sd(const umhs_search* s, int x, int y)
{
    const int ox = vo_clamp_origin(s->n + x + EXT_BORDER, s->es, MB);
    const int oy = vo_clamp_origin(s->m + y + EXT_BORDER, s->h + 2 * EXT_BORDER, MB);
    return vo_tsd16(s->in, s->ins, s->e + (size_t)oy * s->es + ox, s->es);
}

/* One candidate offset (j, i) from the centre, as every pattern loop of
 * MotionEstimatorH264ImplUMHS::Estimate tests it: inside the range, D not
 * above the running minimum (Tsd16x16LessThan decides as the full SSD), then
 * a strictly lower cost. */
static void umhs_probe(umhs_search* s, int j, int i)
{
    if (i + s->my < s->yu || i + s->my > s->yd || j + s->mx < s->xl || j + s->mx > s->xr) return;
    const int ox = vo_clamp_origin(s->n + s->mx + j + EXT_BORDER, s->es, MB);
    const int oy = vo_clamp_origin(s->m + s->my + i + EXT_BORDER, s->h + 2 * EXT_BORDER, MB);
    const int d = vo_tsd16_lt(s->in, s->ins, s->e + (size_t)oy * s->es + ox, s->es, s->min_d);
    if (d > s->min_d) return;
    const int cost = umhs_cost(d, s->mx + j, s->my + i, s->px0, s->py0);
    if (cost < s->min_cost) {
        s->min_d = d;
        s->min_cost = cost;
        s->rmx = j;
        s->rmy = i;
    }
}

/* MotionEstimatorH264ImplUMHS::Estimate (MotionEstimatorH264ImplUMHS.cpp:446-945).
 * Per macroblock in raster order: the median prediction with its distortion,
 * truncated to one macroblock outside the picture; starting points at the
 * prediction, zero and the previous frame's co-located vector; early exits on
 * absolute and prediction-relative thresholds; the unsymmetrical cross, 5x5,
 * multi-hexagon, extended hexagon and diamond patterns; the half / quarter
 * passes of the full-search window; the prediction check at quarter-pel
 * costs.  The chosen vector and its distortion feed later predictions. */
int vo_me_umhs(const short* src, const short* ref, int w, int h, int motion_range, int mode,
               const unsigned char* dist_incl, const int* slice, const short* prev_mv,
               const unsigned char* prev_intra, short* mv_out, int* mb_dist, long* avg_dist)
{
    if (!src || !ref || !mv_out || w < MB || h < MB || (w % MB) != 0 || motion_range < 4) return -1;
    int cols = w / MB, rows = h / MB, nmb = cols * rows;
    int es = w + 2 * EXT_BORDER;
    short* e = vo_ext_alloc(ref, w, h, EXT_BORDER);
    int* dist = (int*)calloc((size_t)nmb, sizeof(int));
    vo_pred_state ps;
    if (!e || !dist || vo_pred_init(&ps, cols, rows, slice) != 0) {
        free(e);
        free(dist);
        vo_pred_free(&ps);
        return -2;
    }
    /* A previous-frame vector is a starting point whose block the reference
     * reads through its clamped extended-reference overlay; should it win,
     * the sub-pel window around it is read unclamped.  Vectors whose block
     * origin leaves [-16, w] x [-16, h] (what a previous estimate never gives)
     * would make it read outside its buffers: refused. */
    for (int k = 0; prev_mv && k < nmb; k++) {
        const int x = (k % cols) * MB + prev_mv[2 * k] / 4, y = (k / cols) * MB + prev_mv[2 * k + 1] / 4;
        if (!(prev_intra && prev_intra[k]) && (x < -MB || x > w || y < -MB || y > h)) {
            free(e);
            free(dist);
            vo_pred_free(&ps);
            return -3;
        }
    }
    const int mrng = motion_range / 4;
    long total = 0;
    int included = 0;
    for (int k = 0; k < nmb; k++) {
        umhs_search s;
        s.n = (k % cols) * MB;
        s.m = (k / cols) * MB;
        s.in = src + (size_t)s.m * w + s.n;
        s.ins = w;
        s.e = e;
        s.es = es;
        s.w = w;
        s.h = h;
        int px, py, pred_d;
        umhs_pred_get(&ps, dist, k, &px, &py, &pred_d);
        const int pxq = px % 4, pyq = py % 4;
        int px0 = px / 4, py0 = py / 4;
        const int opx0 = px0, opy0 = py0;
        if (px0 + s.n > w) px0 = MB;
        if (px0 + s.n < -MB) px0 = -MB;
        if (py0 + s.m > h) py0 = MB;
        if (py0 + s.m < -MB) py0 = -MB;
        const int truncated = opx0 != px0 || opy0 != py0;
        s.px0 = px0;
        s.py0 = py0;
        full_range(s.n, s.m, w, h, motion_range, mrng, &s.xl, &s.xr, &s.yu, &s.yd);

        /* starting points (:489-571) */
        int pred_vd = umhs_sd(&s, px0, py0);
        s.min_d = pred_vd;
        s.mx = px0;
        s.my = py0;
        s.min_cost = pred_vd / 256;
        if (px0 || py0) {
            const int zd = umhs_sd(&s, 0, 0);
            const int zc = umhs_cost(zd, 0, 0, px0, py0);
            if (zc < s.min_cost) { s.min_d = zd; s.min_cost = zc; s.mx = 0; s.my = 0; }
        }
        if (!(prev_intra && prev_intra[k])) {
            const int pvx0 = prev_mv ? prev_mv[2 * k] / 4 : 0, pvy0 = prev_mv ? prev_mv[2 * k + 1] / 4 : 0;
            if ((pvx0 || pvy0) && pvx0 != px0 && pvy0 != py0) {
                const int vd = umhs_sd(&s, pvx0, pvy0);
                const int vc = umhs_cost(vd, pvx0, pvy0, px0, py0);
                if (vc < s.min_cost) { s.min_d = vd; s.min_cost = vc; s.mx = pvx0; s.my = pvy0; }
            }
        }
        int prior;
        if (s.min_d < 1000) goto diamond;
        if (s.min_d < 4000 || (s.min_d == pred_vd && s.min_d < pred_d * 12 / 10 && s.min_d > pred_d * 8 / 10))
            goto hexagon;

        /* unsymmetrical cross, vertical reach below half the range (:573-623) */
        s.rmx = s.rmy = 0;
        prior = s.min_d;
        for (int wgt = 1; wgt < 16; wgt += 2)
            for (int x = 0; x < 4; x++) {
                const int i = wgt * UMHS_CROSS[x][1], j = wgt * UMHS_CROSS[x][0];
                if (i < mrng / 2 && i > -mrng / 2) umhs_probe(&s, j, i);
            }
        s.mx += s.rmx;
        s.my += s.rmy;
        if (s.min_d < 1000) goto diamond;
        if (s.min_d < 2000 ||
            (s.min_d < prior * 9 / 10 && (s.rmx || s.rmy) && abs(s.rmx) <= 3 && abs(s.rmy) <= 3))
            goto hexagon;

        /* 5x5 without the points the cross already tested (:625-656) */
        {
            const int crx = s.rmx, cry = s.rmy;
            s.rmx = s.rmy = 0;
            for (int x = 0; x < 24; x++) {
                const int j = UMHS_5X5[x][0], i = UMHS_5X5[x][1];
                const int tested = (crx || cry) && ((cry == 0 && (j == 2 || j == -2)) || (crx == 0 && (i == 2 || i == -2)));
                if (!tested) umhs_probe(&s, j, i);
            }
        }
        /* the centre stays at the cross winner on this exit (:658-662) */
        if (s.min_d < 1000) goto diamond;

        /* multi-hexagon from the cross winner; the 5x5 offset stays a candidate (:664-702) */
        prior = s.min_d;
        for (int wgt = 1; wgt < 4; wgt++) {
            for (int x = 0; x < 16; x++) umhs_probe(&s, wgt * UMHS_HEX[x][0], wgt * UMHS_HEX[x][1]);
            if ((s.rmx || s.rmy) && (s.min_d < 2000 || s.min_d < prior / 5)) break;
        }
        s.mx += s.rmx;
        s.my += s.rmy;

    hexagon: /* extended hexagon until the centre wins (:705-736) */
        do {
            s.rmx = s.rmy = 0;
            for (int x = 0; x < 6; x++) umhs_probe(&s, UMHS_EXTHEX[x][0], UMHS_EXTHEX[x][1]);
            s.mx += s.rmx;
            s.my += s.rmy;
        } while (s.rmx || s.rmy);

    diamond: /* small diamond until the centre wins (:739-769) */
        do {
            s.rmx = s.rmy = 0;
            for (int x = 0; x < 4; x++) umhs_probe(&s, UMHS_CROSS[x][0], UMHS_CROSS[x][1]);
            s.mx += s.rmx;
            s.my += s.rmy;
        } while (s.rmx || s.rmy);

        /* half / quarter passes (:790-867) */
        int min_d = s.min_d;
        int mvx = 4 * s.mx, mvy = 4 * s.my;
        if (mode != 2) {
            const int ox = vo_clamp_origin(s.n + s.mx + EXT_BORDER, es, MB);
            const int oy = vo_clamp_origin(s.m + s.my + EXT_BORDER, h + 2 * EXT_BORDER, MB);
            int qmx, qmy;
            subpel_refine(s.in, w, e, es, ox, oy, mode != 1, &min_d, &qmx, &qmy);
            mvx += qmx;
            mvy += qmy;
        }

        /* the prediction at quarter pel against the winner (:869-908) */
        const int rpx = 4 * px0 + pxq, rpy = 4 * py0 + pyq;
        if (pxq || pyq) {
            short blk[256];
            const int pox = vo_clamp_origin(px0 + s.n + EXT_BORDER, es, MB);
            const int poy = vo_clamp_origin(py0 + s.m + EXT_BORDER, h + 2 * EXT_BORDER, MB);
            vo_qread16_ext(e, es, pox, poy, pxq, pyq, blk);
            pred_vd = vo_tsd16(s.in, w, blk, 16);
        } else if (truncated) {
            pred_vd = umhs_sd(&s, px0, py0);
        }
        if (umhs_cost(pred_vd, rpx, rpy, px, py) <= umhs_cost(min_d, mvx, mvy, px, py)) {
            min_d = pred_vd;
            mvx = rpx;
            mvy = rpy;
        }
        if (dist_incl && dist_incl[k]) {
            included++;
            total += min_d;
        }
        if (mb_dist) mb_dist[k] = min_d;
        mv_out[2 * k] = (short)mvx;
        mv_out[2 * k + 1] = (short)mvy;
        vo_pred_set(&ps, k, mvx, mvy);
        dist[k] = min_d;
    }
    if (avg_dist) *avg_dist = included ? total / included : 0;
    vo_pred_free(&ps);
    free(dist);
    free(e);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* MotionEstimatorH264ImplFHS                                                */
/* ------------------------------------------------------------------------ */
/* Points 64..79 of the path MotionEstimatorH264ImplFHS::Td16x16OptimalPathLessThan
 * reads (MotionEstimatorH264ImplFHS.cpp:1685-1785, {x, y}); points 0..63 are
 * CROSS_PATH. */
static const signed char FHS_PATH_TAIL[16][2] = {{5, 2},  {5, 12}, {1, 4},  {11, 5}, {13, 8},  {9, 7},
                                                 {13, 3}, {5, 8},  {10, 11}, {6, 15}, {13, 10}, {8, 4},
                                                 {3, 10}, {13, 1}, {1, 8},  {14, 0}};
static void fhs_path_point(int p, int* x, int* y)
{
    if (p < 64) {
        *x = CROSS_PATH[p][0];
        *y = CROSS_PATH[p][1];
    } else {
        *x = FHS_PATH_TAIL[p - 64][0];
        *y = FHS_PATH_TAIL[p - 64][1];
    }
}

/* Td16x16OptimalPathLessThan (MotionEstimatorH264ImplFHS.cpp:1685-1790): squared
 * differences along the first 80 path points; after 32, 40, 48, 56, 64 and 72 of
 * them the whole block's distortion is extrapolated as D * 256 / N and returned
 * once it exceeds min; after 80 the extrapolation is returned. */
static int fhs_path_lt(const short* a, int as, const short* b, int bs, int min)
{
    int d = 0;
    for (int p = 0; p < 80; p++) {
        int x, y;
        fhs_path_point(p, &x, &y);
        const int e = a[(size_t)y * as + x] - b[(size_t)y * bs + x];
        d += e * e;
        const int n = p + 1;
        if (n >= 32 && n < 80 && (n % 8) == 0) {
            const int v = d * 256 / n;
            if (v > min) return v;
        }
    }
    return d * 256 / 80;
}

/* MEH264IFHS_COST (MotionEstimatorH264ImplFHS.cpp:222): (D + 269 * (int)sqrt(s)) >> 8,
 * all integer but the square root, truncated. */
static int fhs_cost(int d, int x, int y, int xr, int yr)
{
    const int s = (x - xr) * (x - xr) + (y - yr) * (y - yr);
    return (d + 269 * (int)sqrt((double)s)) >> 8;
}

/* One macroblock's FHS state: the running best and the pattern centre. */
typedef struct {
    const short* in;
    const short* e;
    int es, w, h, n, m;
    int xl, xr, yu, yd, px0, py0;
    int mx, my, rmx, rmy, min_d, min_cost;
} fhs_search;

static const short* fhs_block(const fhs_search* s, int x, int y)
{
    const int ox = vo_clamp_origin(s->n + x + EXT_BORDER, s->es, MB);
    const int oy = vo_clamp_origin(s->m + y + EXT_BORDER, s->h + 2 * EXT_BORDER, MB);
    return s->e + (size_t)oy * s->es + ox;
}

/* A pattern candidate (UMHS-style loop body of FHS.cpp:690-738, :758-780, :792-818):
 * in range, its path distortion not above the running minimum, a strictly lower cost. */
static void fhs_probe(fhs_search* s, int j, int i)
{
    if (i + s->my < s->yu || i + s->my > s->yd || j + s->mx < s->xl || j + s->mx > s->xr) return;
    const int d = fhs_path_lt(s->in, s->w, fhs_block(s, s->mx + j, s->my + i), s->es, s->min_d);
    if (d > s->min_d) return;
    const int cost = fhs_cost(d, s->mx + j, s->my + i, s->px0, s->py0);
    if (cost < s->min_cost) {
        s->min_d = d;
        s->min_cost = cost;
        s->rmx = j;
        s->rmy = i;
    }
}

/* SSD of the block at quarter-pel offset (qx, qy) from the full-pel origin
 * (ox, oy) of the extended reference: the H.264 samples the reference's
 * half-pel cache and QuarterRead hold there. */
static int fhs_sub_sd(const fhs_search* s, int ox, int oy, int qx, int qy)
{
    short blk[256];
    vo_qread16_ext(s->e, s->es, ox, oy, qx, qy, blk);
    return vo_tsd16(s->in, s->w, blk, 16);
}

/* HalfPelEstimate (MotionEstimatorH264ImplFHS.cpp:1109-1200): the two "h"
 * offsets, then the two "b", then the four "j", strict improvement, leaving
 * after a stage whose minimum is below 1000.  Returns the minimum and the
 * half-pel offset; *h_exit says it left after the "h" stage. */
static int fhs_half(const fhs_search* s, int ox, int oy, int min, int* hx, int* hy, int* h_exit)
{
    static const int HX[8] = {0, 0, -1, 1, -1, 1, -1, 1}, HY[8] = {-1, 1, 0, 0, -1, -1, 1, 1};
    int lcl = min;
    *hx = *hy = 0;
    *h_exit = 0;
    for (int k = 0; k < 8; k++) {
        const int d = fhs_sub_sd(s, ox, oy, 2 * HX[k], 2 * HY[k]);
        if (d < lcl) {
            lcl = d;
            *hx = HX[k];
            *hy = HY[k];
        }
        if ((k == 1 || k == 3) && lcl < 1000) {
            *h_exit = k == 1;
            break;
        }
    }
    return lcl;
}

/* QuarterPelEstimate (MotionEstimatorH264ImplFHS.cpp:1213-1480): the half-pel
 * stage, then the eight quarter offsets around its winner, strict improvement,
 * leaving at a minimum below 1000.  The returned offset is the last quarter-pel
 * improvement only: a half-pel winner without one returns (0, 0) with the
 * half-pel distortion, as the reference does.
 *
 * When the half-pel stage leaves after its "h" stage without an improvement
 * (the full-pel minimum was already below 1000), the reference's quarter pass
 * reads "b" and "j" samples its cache holds from earlier macroblocks.  That
 * history is not reproduced: the samples of this macroblock are used, and
 * *stale counts the occurrence so that pinned cases can assert there is none. */
static int fhs_quarter(const fhs_search* s, int ox, int oy, int min, int* qx, int* qy, int* stale)
{
    int hx, hy, h_exit;
    const int half = fhs_half(s, ox, oy, min, &hx, &hy, &h_exit);
    int lcl = min;
    *qx = *qy = 0;
    if (half < min) {
        lcl = half;
        if (half < 1000) return lcl;
    }
    if (h_exit) (*stale)++;
    for (int k = 0; k < 8; k++) {
        const int qox = 2 * hx + SUB_X[k], qoy = 2 * hy + SUB_Y[k];
        const int d = fhs_sub_sd(s, ox, oy, qox, qoy);
        if (d < lcl) {
            lcl = d;
            *qx = qox;
            *qy = qoy;
            if (d < 1000) break;
        }
    }
    return lcl;
}

/* MotionEstimatorH264ImplFHS::Estimate (MotionEstimatorH264ImplFHS.cpp:497-900).
 * Per macroblock in raster order: the median prediction with its distortion,
 * truncated to one macroblock outside the picture (its quarter-pel part then
 * dropped); the prediction's full SSD at quarter pel and the zero vector's path
 * distortion as starting points, each ending the search below 1000; the
 * four-scale hexagon, one extended-hexagon and one diamond pass on path
 * distortions with integer costs; the half / quarter stages; the prediction
 * check, whose costs compare quarter-pel vectors with the full-pel prediction
 * as the reference does.  The previous-frame starting point is disabled in the
 * reference (:627-673). */
int vo_me_fhs(const short* src, const short* ref, int w, int h, int motion_range, int mode,
              const unsigned char* dist_incl, const int* slice, short* mv_out, int* mb_dist, long* avg_dist,
              int* stale_out)
{
    if (!src || !ref || !mv_out || w < MB || h < MB || (w % MB) != 0 || motion_range < 4) return -1;
    int cols = w / MB, rows = h / MB, nmb = cols * rows;
    int es = w + 2 * EXT_BORDER;
    short* e = vo_ext_alloc(ref, w, h, EXT_BORDER);
    int* dist = (int*)calloc((size_t)nmb, sizeof(int));
    vo_pred_state ps;
    if (!e || !dist || vo_pred_init(&ps, cols, rows, slice) != 0) {
        free(e);
        free(dist);
        vo_pred_free(&ps);
        return -2;
    }
    long total = 0;
    int included = 0, stale = 0;
    for (int k = 0; k < nmb; k++) {
        fhs_search s;
        s.n = (k % cols) * MB;
        s.m = (k / cols) * MB;
        s.in = src + (size_t)s.m * w + s.n;
        s.e = e;
        s.es = es;
        s.w = w;
        s.h = h;
        int px, py, pred_d;
        umhs_pred_get(&ps, dist, k, &px, &py, &pred_d);
        int pxq = px % 4, pyq = py % 4;
        int px0 = px / 4, py0 = py / 4;
        const int opx0 = px0, opy0 = py0;
        if (px0 + s.n > w) px0 = MB;
        if (px0 + s.n < -MB) px0 = -MB;
        if (py0 + s.m > h) py0 = MB;
        if (py0 + s.m < -MB) py0 = -MB;
        if (opx0 != px0 || opy0 != py0) pxq = pyq = 0;  /* (:549-550) */
        const int rpx = 4 * px0 + pxq, rpy = 4 * py0 + pyq;
        s.px0 = px0;
        s.py0 = py0;
        full_range(s.n, s.m, w, h, motion_range, motion_range / 4, &s.xl, &s.xr, &s.yu, &s.yd);
        int mvx, mvy;

        /* the prediction at quarter pel (:555-597) */
        const int pox = vo_clamp_origin(px0 + s.n + EXT_BORDER, es, MB);
        const int poy = vo_clamp_origin(py0 + s.m + EXT_BORDER, h + 2 * EXT_BORDER, MB);
        const int pred_vd = fhs_sub_sd(&s, pox, poy, pxq, pyq);
        s.min_d = pred_vd;
        s.mx = px0;
        s.my = py0;
        s.min_cost = pred_vd / 256;
        if (pred_vd < 1000) {
            mvx = rpx;
            mvy = rpy;
            goto done;
        }
        /* zero (:599-625) */
        if (rpx || rpy) {
            const int zd = fhs_path_lt(s.in, w, fhs_block(&s, 0, 0), es, s.min_d);
            if (zd < s.min_d) {
                const int zc = fhs_cost(zd, 0, 0, px0, py0);
                if (zc < s.min_cost) { s.min_d = zd; s.min_cost = zc; s.mx = 0; s.my = 0; }
                if (zd < 1000) {
                    mvx = 0;
                    mvy = 0;
                    goto done;
                }
            }
        }
        if (s.min_d < 1000) goto diamond;
        if (s.min_d < 4000 || (s.min_d == pred_vd && s.min_d < pred_d * 12 / 10 && s.min_d > pred_d * 8 / 10))
            goto hexagon;
        /* four hexagon scales (:684-748) */
        s.rmx = s.rmy = 0;
        for (int wgt = 1; wgt <= 4; wgt++)
            for (int x = 0; x < 16; x++) fhs_probe(&s, wgt * UMHS_HEX[x][0], wgt * UMHS_HEX[x][1]);  /* MEH264IFHS_HexPos, the UMHS table */
        s.mx += s.rmx;
        s.my += s.rmy;
    hexagon: /* one extended-hexagon pass (:751-784) */
        s.rmx = s.rmy = 0;
        for (int x = 0; x < 6; x++) fhs_probe(&s, UMHS_EXTHEX[x][0], UMHS_EXTHEX[x][1]);
        s.mx += s.rmx;
        s.my += s.rmy;
    diamond: /* one diamond pass (:786-820) */
        s.rmx = s.rmy = 0;
        for (int x = 0; x < 4; x++) fhs_probe(&s, UMHS_CROSS[x][0], UMHS_CROSS[x][1]);
        s.mx += s.rmx;
        s.my += s.rmy;
        /* half / quarter stages (:822-856) */
        mvx = 4 * s.mx;
        mvy = 4 * s.my;
        {
            const int ox = vo_clamp_origin(s.n + s.mx + EXT_BORDER, es, MB);
            const int oy = vo_clamp_origin(s.m + s.my + EXT_BORDER, h + 2 * EXT_BORDER, MB);
            if (mode == 0) {
                int qx, qy;
                const int nm = fhs_quarter(&s, ox, oy, s.min_d, &qx, &qy, &stale);
                if (nm < s.min_d) { s.min_d = nm; mvx += qx; mvy += qy; }
            } else if (mode == 1) {
                int hx, hy, h_exit;
                const int nm = fhs_half(&s, ox, oy, s.min_d, &hx, &hy, &h_exit);
                if (nm < s.min_d) { s.min_d = nm; mvx += 2 * hx; mvy += 2 * hy; }
            }
        }
        /* the prediction check (:858-867) */
        if (fhs_cost(pred_vd, rpx, rpy, px0, py0) <= fhs_cost(s.min_d, mvx, mvy, px0, py0)) {
            s.min_d = pred_vd;
            mvx = rpx;
            mvy = rpy;
        }
    done: /* (:869-890) */
        if (dist_incl && dist_incl[k]) {
            included++;
            total += s.min_d;
        }
        if (mb_dist) mb_dist[k] = s.min_d;
        mv_out[2 * k] = (short)mvx;
        mv_out[2 * k + 1] = (short)mvy;
        vo_pred_set(&ps, k, mvx, mvy);
        dist[k] = s.min_d;
    }
    if (avg_dist) *avg_dist = included ? total / included : 0;
    if (stale_out) *stale_out = stale;
    vo_pred_free(&ps);
    free(dist);
    free(e);
    return 0;
}
