/*
 * oracle_me_multires.c -- TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * Restatement of the multi-resolution H.264 estimators:
 *   MotionEstimatorH264ImplMultiresCross::Estimate
 *     (src/CodecUtils/MotionEstimatorH264ImplMultiresCross.cpp:525-1019)
 *   MotionEstimatorH264ImplMultiresCrossVer2::Estimate(long*)
 *     (src/CodecUtils/MotionEstimatorH264ImplMultiresCrossVer2.cpp:537-1151)
 *   MotionEstimatorH264ImplMultiresCrossVer2::Estimate(long*, void* lambda)
 *     (src/CodecUtils/MotionEstimatorH264ImplMultiresCrossVer2.cpp:1162-1742)
 *   MotionEstimatorH264ImplMultires::Estimate
 *     (src/CodecUtils/MotionEstimatorH264ImplMultires.cpp:557-1024)
 *
 * The reference works on extended-boundary copies of each pyramid level
 * (borders 19 / 9 / 5 samples for levels 0 / 1 / 2), addresses them through
 * row-pointer overlays whose origins are clamped (OverlayExtMem2Dv2::SetOrigin,
 * src/ImageUtils/OverlayExtMem2Dv2.cpp:86-101) and reads beyond an overlay
 * without checks.  The oracle keeps the same flat buffers and origin clamps
 * and aborts (returns an error) if a read would leave a buffer, so that the
 * restatement is exact wherever the reference itself is defined.
 *
 * The half-pel window of MultiresCross (…MultiresCross.cpp:1281-1349) does
 * not write the full-pel samples of its last column and row, nor scale the
 * last h column / b row (the full-search estimator and Ver2 do, Full.cpp:1162-1180,
 * …MultiresCrossVer2.cpp:2075-2093).
 * Those never-written samples are taken as 0, the content of the window
 * buffer when its allocation is fresh zeroed memory; the unscaled edge
 * samples are reproduced as they are.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle_internal.h"

typedef struct {
    short* mem;
    int w, h;
} mr_buf;

typedef struct {
    const mr_buf* b;
    int bw, bh;  /* block (overlay) dimensions */
    int x, y;    /* origin in buffer coordinates */
    int ebx, eby; /* extended border for OverlayExtMem2Dv2 origins (0 for plain overlays) */
} mr_ov;

static int g_mr_fault;

static inline int mr_read(const mr_buf* b, int r, int c)
{
    long long f = (long long)r * b->w + c;
    if (f < 0 || f >= (long long)b->w * b->h) {
        g_mr_fault = 1;
        return 0;
    }
    return b->mem[f];
}

/* OverlayMem2Dv2::SetOrigin / OverlayExtMem2Dv2::SetOrigin. */
static void ov_origin(mr_ov* o, int x, int y)
{
    x += o->ebx;
    y += o->eby;
    if (x < 0) x = 0;
    else if (x > o->b->w - o->bw) x = o->b->w - o->bw;
    if (y < 0) y = 0;
    else if (y > o->b->h - o->bh) y = o->b->h - o->bh;
    o->x = x;
    o->y = y;
}

static inline int ov_px(const mr_ov* o, int r, int c) { return mr_read(o->b, o->y + r, o->x + c); }

/* Tsd4x4 / Tsd8x8 / Tsd16x16 (OverlayMem2Dv2.cpp:1523-1700). */
static int ov_tsd(const mr_ov* a, const mr_ov* b, int n)
{
    int acc = 0;
    for (int r = 0; r < n; r++)
        for (int c = 0; c < n; c++) {
            int d = ov_px(a, r, c) - ov_px(b, r, c);
            acc += d * d;
        }
    return acc;
}

/* Tsd4x4LessThan (OverlayMem2Dv2.cpp:1739-1790). */
static int ov_tsd4_lt(const mr_ov* a, const mr_ov* b, int min)
{
    int acc = 0;
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            int d = ov_px(a, r, c) - ov_px(b, r, c);
            acc += d * d;
            if (c < 3 && acc > min) return acc;
        }
    return acc;
}

/* Tsd8x8PartialLessThan / Tsd16x16PartialLessThan (OverlayMem2Dv2.cpp:1886-1913, 1993-2020). */
static int ov_tsd_partial_lt(const mr_ov* a, const mr_ov* b, int n, int min)
{
    int dp = 0;
    for (int p = 1; p <= 16; p++) {
        int pd = 0;
        for (int i = 0; i < n; i += 4)
            for (int j = 0; j < n; j += 4) {
                int d = ov_px(a, vo_phase_row[p] + i, vo_phase_col[p] + j) - ov_px(b, vo_phase_row[p] + i, vo_phase_col[p] + j);
                pd += d * d;
            }
        dp += pd;
        if ((dp << 4) > p * min) return dp << 4;
    }
    return dp;
}

/* Same partial test against a plain 16x16 block (the sub-pel candidates). */
static int blk_tsd16_partial_lt(const mr_ov* a, const short* blk, int min)
{
    int dp = 0;
    for (int p = 1; p <= 16; p++) {
        int pd = 0;
        for (int i = 0; i < 16; i += 4)
            for (int j = 0; j < 16; j += 4) {
                int r = vo_phase_row[p] + i, c = vo_phase_col[p] + j;
                int d = ov_px(a, r, c) - blk[r * 16 + c];
                pd += d * d;
            }
        dp += pd;
        if ((dp << 4) > p * min) return dp << 4;
    }
    return dp;
}

static int mr_buf_ext(mr_buf* e, const short* plane, int w, int h, int border)
{
    e->w = w + 2 * border;
    e->h = h + 2 * border;
    e->mem = vo_ext_alloc(plane, w, h, border);
    return e->mem ? 0 : -1;
}

/* Ranged GetMotionRange of the multi-resolution estimators
 * (…MultiresCross.cpp:1195-1262): vector limits from vecRange of the level,
 * then the block may reach `boundary` samples outside the level's picture. */
typedef struct {
    int boundary, width, height, vec_range;
} mr_level;

static void mr_range(const mr_level* L, int xpos, int ypos, int xoff, int yoff, int range,
                     int* xl, int* xr, int* yu, int* yd)
{
    int x = xpos + xoff, y = ypos + yoff;
    int vr = L->vec_range;
    int xlr = (xoff - range > -vr) ? range : (vr - 1) + xoff;
    int xrr = (xoff + range < vr) ? range : (vr - 1) - xoff;
    int yur = (yoff - range > -vr) ? range : (vr - 1) + yoff;
    int ydr = (yoff + range < vr) ? range : (vr - 1) - yoff;
    *xl = (x - xlr >= -L->boundary) ? -xlr : -(x + L->boundary);
    *xr = (x + xrr < L->width) ? xrr : L->width - x;
    *yu = (y - yur >= -L->boundary) ? -yur : -(y + L->boundary);
    *yd = (y + ydr < L->height) ? ydr : L->height - y;
}

/* ---- the 88x88 quarter-pel window ------------------------------------- */
#define WIN 88
typedef struct {
    short w[WIN][WIN];
} mr_window;

static inline int clip255i(int x) { return x < 0 ? 0 : (x > 255 ? 255 : x); }

/* MotionEstimatorH264ImplMultiresCross::LoadHalfQuartPelWindow (…:1281-1349):
 * raw h over rows 2..18 x all 22 columns, raw b over all 22 rows x columns
 * 2..18, j from the raw h, then h/b scaled and G copied over columns and rows
 * 2..18 only. */
static void mr_load_half_window(mr_window* W, const mr_ov* ref, int ver2)
{
    const int rx = ref->x, ry = ref->y;
    for (int fr = 2; fr < 19; fr++)
        for (int fc = 0; fc < 22; fc++) {
            int rr = ry + fr - 3, cc = rx + fc - 3;
            int h = mr_read(ref->b, rr - 2, cc) - 5 * mr_read(ref->b, rr - 1, cc) + 20 * mr_read(ref->b, rr, cc) +
                    20 * mr_read(ref->b, rr + 1, cc) - 5 * mr_read(ref->b, rr + 2, cc) + mr_read(ref->b, rr + 3, cc);
            W->w[4 * fr + 2][4 * fc] = (short)h;
        }
    for (int fr = 0; fr < 22; fr++)
        for (int fc = 2; fc < 19; fc++) {
            int rr = ry + fr - 3, cc = rx + fc - 3;
            int b = mr_read(ref->b, rr, cc - 2) - 5 * mr_read(ref->b, rr, cc - 1) + 20 * mr_read(ref->b, rr, cc) +
                    20 * mr_read(ref->b, rr, cc + 1) - 5 * mr_read(ref->b, rr, cc + 2) + mr_read(ref->b, rr, cc + 3);
            W->w[4 * fr][4 * fc + 2] = (short)b;
        }
    for (int fr = 2; fr < 19; fr++)
        for (int fc = 2; fc < 19; fc++) {
            int qr = 4 * fr + 2, qc = 4 * fc + 2;
            int j = ((int)W->w[qr][qc - 10] - 5 * W->w[qr][qc - 6] + 20 * W->w[qr][qc - 2] + 20 * W->w[qr][qc + 2] -
                     5 * W->w[qr][qc + 6] + W->w[qr][qc + 10] + 512) >> 10;
            W->w[qr][qc] = (short)clip255i(j);
        }
    for (int fr = 2; fr < 19; fr++)
        for (int fc = 2; fc < 19; fc++) {
            int qr = 4 * fr, qc = 4 * fc;
            W->w[qr + 2][qc] = (short)clip255i((W->w[qr + 2][qc] + 16) >> 5);
            W->w[qr][qc + 2] = (short)clip255i((W->w[qr][qc + 2] + 16) >> 5);
            W->w[qr][qc] = (short)mr_read(ref->b, ry + fr - 3, rx + fc - 3);
        }
    if (ver2) {
        /* Ver2 also completes column and row 19: scaled h and G at column 19
         * of rows 2..18, scaled b and G at row 19 of columns 2..18, and G at
         * (19, 19) (…MultiresCrossVer2.cpp:2075-2093) */
        for (int fr = 2; fr < 19; fr++) {
            W->w[4 * fr + 2][76] = (short)clip255i((W->w[4 * fr + 2][76] + 16) >> 5);
            W->w[4 * fr][76] = (short)mr_read(ref->b, ry + fr - 3, rx + 16);
        }
        for (int fc = 2; fc < 19; fc++) {
            W->w[76][4 * fc + 2] = (short)clip255i((W->w[76][4 * fc + 2] + 16) >> 5);
            W->w[76][4 * fc] = (short)mr_read(ref->b, ry + 16, rx + fc - 3);
        }
        W->w[76][76] = (short)mr_read(ref->b, ry + 16, rx + 16);
    }
}

/* LoadQuartPelWindow (…MultiresCross.cpp:1365-1389): the eight quarter
 * samples around every point of the winning half-pel grid. */
static void mr_load_quarter_window(mr_window* W, int hx, int hy)
{
    for (int fr = 0; fr < 16; fr++)
        for (int fc = 0; fc < 16; fc++) {
            int qr = 12 + hy + 4 * fr, qc = 12 + hx + 4 * fc;
            short (*w)[WIN] = W->w;
            w[qr - 1][qc - 1] = (short)((w[qr - 2][qc - 2] + w[qr][qc] + 1) >> 1);
            w[qr - 1][qc] = (short)((w[qr - 2][qc] + w[qr][qc] + 1) >> 1);
            w[qr - 1][qc + 1] = (short)((w[qr - 2][qc] + w[qr][qc + 2] + 1) >> 1);
            w[qr][qc - 1] = (short)((w[qr][qc - 2] + w[qr][qc] + 1) >> 1);
            w[qr][qc + 1] = (short)((w[qr][qc + 2] + w[qr][qc] + 1) >> 1);
            w[qr + 1][qc - 1] = (short)((w[qr][qc - 2] + w[qr + 2][qc] + 1) >> 1);
            w[qr + 1][qc] = (short)((w[qr + 2][qc] + w[qr][qc] + 1) >> 1);
            w[qr + 1][qc + 1] = (short)((w[qr + 2][qc] + w[qr][qc + 2] + 1) >> 1);
        }
}

static void mr_window_read(const mr_window* W, int qx, int qy, short* blk)
{
    for (int r = 0; r < 16; r++)
        for (int c = 0; c < 16; c++) blk[r * 16 + c] = W->w[12 + qy + 4 * r][12 + qx + 4 * c];
}

static const int SUBX[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
static const int SUBY[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
static const int CRX[4] = {-1, 1, 0, 0};
static const int CRY[4] = {0, 0, -1, 1};

#define MRC_NOISE_FLOOR 512

/* ------------------------------------------------------------------------ */
/* The pyramid one estimate works on. */
typedef struct {
    int w, h, cols, nmb, rows_all, mode, l1_range, l2_range, lcl_l1_range;
    mr_buf in0, in1, in2, r1, r2, e0, e1, e2;
    mr_level L0, L1, L2;
    mr_window* win;
    int h263; /* MotionEstimatorH263ImplMultiresCross: half-pel stage by HalfRead, its accept rule */
    int tie_plus_y; /* MotionEstimatorH263ImplMultiresCrossVer2: the candidate's y distance adds the prediction */
} mr_ctx;

/* OverlayMem2Dv2::HalfRead at half-pel offset (hx, hy) in -1..1 of the
 * block at overlay o (OverlayMem2Dv2.cpp:452-530, the unrolled branch that is
 * compiled): bilinear means with +2 >> 2 (diagonal) or +1 >> 1 rounding; the
 * left neighbour for hx = -1, the right one for hx = 1. */
static void mr_half_read(const mr_ov* o, int hx, int hy, short* blk)
{
    for (int r = 0; r < 16; r++)
        for (int col = 0; col < 16; col++) {
            const int c0 = hx < 0 ? col - 1 : col;
            int v;
            if (hx && hy)
                v = (ov_px(o, r, c0) + ov_px(o, r + hy, c0) + ov_px(o, r, c0 + 1) + ov_px(o, r + hy, c0 + 1) + 2) / 4;
            else if (hx)
                v = (ov_px(o, r, c0) + ov_px(o, r, c0 + 1) + 1) / 2;
            else
                v = (ov_px(o, r, col) + ov_px(o, r + hy, col) + 1) / 2;
            blk[r * 16 + col] = (short)v;
        }
}

static void mr_ctx_free(mr_ctx* c)
{
    free(c->in1.mem);
    free(c->r1.mem);
    free(c->in2.mem);
    free(c->r2.mem);
    free(c->e0.mem);
    free(c->e1.mem);
    free(c->e2.mem);
    free(c->win);
}

/* Level copies as Estimate builds them before its macroblock loop
 * (…MultiresCross.cpp:539-601; …MultiresCrossVer2.cpp:552-611). */
static int mr_ctx_init_h(mr_ctx* c, const short* src, const short* ref, int w, int h, int motion_range, int mode,
                         int h263);
static int mr_ctx_init(mr_ctx* c, const short* src, const short* ref, int w, int h, int motion_range, int mode)
{
    return mr_ctx_init_h(c, src, ref, w, h, motion_range, mode, 0);
}

/* h263: MotionEstimatorH263ImplMultiresCross::Create (…H263ImplMultiresCross.cpp:160-300): the motion
 * range is in half pels (level 0 vecRange motionRange/2, level 1 motionRange/4: the H.264 estimator's
 * ranges at twice the value) and the level-0 reference is extended by 16 + 1 samples. */
static int mr_ctx_init_h(mr_ctx* c, const short* src, const short* ref, int w, int h, int motion_range, int mode,
                         int h263)
{
    memset(c, 0, sizeof(*c));
    c->h263 = h263;
    if (h263) motion_range *= 2;
    c->w = w;
    c->h = h;
    c->cols = w / 16;
    c->nmb = c->cols * (h / 16);
    c->rows_all = (h + 15) / 16;
    const int w1 = w / 2, h1 = h / 2, w2 = w1 / 2, h2 = h1 / 2;
    c->l1_range = motion_range / 8;
    c->l2_range = c->l1_range / 2;
    if (mode == 0) mode = (w * h > 40000) ? 2 : 1; /* SetMode(0) (…MultiresCross.cpp:501-513) */
    c->mode = mode;
    c->lcl_l1_range = (mode == 2) ? 2 : c->l1_range;
    c->in0.mem = (short*)src;
    c->in0.w = w;
    c->in0.h = h;
    c->in1.w = c->r1.w = w1;
    c->in1.h = c->r1.h = h1;
    c->in2.w = c->r2.w = w2;
    c->in2.h = c->r2.h = h2;
    c->in1.mem = (short*)malloc(sizeof(short) * (size_t)w1 * h1);
    c->r1.mem = (short*)malloc(sizeof(short) * (size_t)w1 * h1);
    c->in2.mem = (short*)malloc(sizeof(short) * (size_t)w2 * h2 + 2);
    c->r2.mem = (short*)malloc(sizeof(short) * (size_t)w2 * h2 + 2);
    c->win = (mr_window*)calloc(1, sizeof(mr_window));
    if (!c->in1.mem || !c->r1.mem || !c->in2.mem || !c->r2.mem || !c->win) return -2;
    vo_half(ref, w, h, c->r1.mem);
    vo_half(src, w, h, c->in1.mem);
    if (mode == 2) {
        vo_half(c->r1.mem, w1, h1, c->r2.mem);
        vo_half(c->in1.mem, w1, h1, c->in2.mem);
    }
    if (mr_buf_ext(&c->e0, ref, w, h, h263 ? 17 : 19) || mr_buf_ext(&c->e1, c->r1.mem, w1, h1, 9) ||
        (mode == 2 && mr_buf_ext(&c->e2, c->r2.mem, w2, h2, 5)))
        return -2;
    c->L0 = (mr_level){16, w, h, motion_range / 4};
    c->L1 = (mr_level){8, w1, h1, c->l1_range};
    c->L2 = (mr_level){4, w2, h2, c->l2_range};
    return 0;
}

/* Tie rule of the integer stages: an equal distortion replaces the current
 * best (offset (rmx, rmy) from the centre (mx, my)) unless the candidate at
 * (j, i) is farther from the reference point (px, py): MultiresCross measures
 * from (0, 0) (…MultiresCross.cpp:741-746, 794, 857), MultiresCrossVer2 from
 * the rounded prediction of the level (…MultiresCrossVer2.cpp:778-786,
 * 834-842, 906-914). */
static inline int mr_farther(int mx, int my, int rmx, int rmy, int j, int i, int px, int py)
{
    const int cx = mx + rmx - px, cy = my + rmy - py, nx = mx + j - px, ny = my + i - py;
    return (cy * cy + cx * cx) - (ny * ny + nx * nx) < 0;
}

/* MotionEstimatorH263ImplMultiresCrossVer2's tie rule (…H263ImplMultiresCrossVer2.cpp:714-721, 787-794,
 * 844-851, 912-919): the candidate's y distance is taken as my + i + predY, with the prediction's y added
 * where the current best's subtracts it. */
static inline int mr_farther_v2(const mr_ctx* c, int mx, int my, int rmx, int rmy, int j, int i, int px, int py)
{
    if (!c->tie_plus_y) return mr_farther(mx, my, rmx, rmy, j, i, px, py);
    const int cx = mx + rmx - px, cy = my + rmy - py, nx = mx + j - px, ny = my + i + py;
    return (cy * cy + cx * cx) - (ny * ny + nx * nx) < 0;
}

/* Result of the search of one macroblock. */
typedef struct {
    int zero_d, min_d, mvx, mvy;
    int tie; /* integer stages that met a candidate equal to their running minimum: 1 level 2, 2 level 1, 4 level 0 */
} mr_result;

/* The search of macroblock (mbr, mbc) of both estimators, from the zero
 * vector to the quarter-pel winner (…MultiresCross.cpp:612-941;
 * …MultiresCrossVer2.cpp:643-992).  pred == NULL: MultiresCross's tie rules;
 * else Ver2's, pred = {level-2 x, y, level-1 x, y, level-0 rounded x, y}. */
static void mr_search_mb(mr_ctx* c, int mbr, int mbc, const int* pred, mr_result* out)
{
    const int m = 16 * mbr, n = 16 * mbc, p = 8 * mbr, q = 8 * mbc, kk = 4 * mbr, ll = 4 * mbc;
    const int b0 = c->h263 ? 17 : 19;
    mr_ov oin0 = {&c->in0, 16, 16, 0, 0, 0, 0}, oin1 = {&c->in1, 8, 8, 0, 0, 0, 0}, oin2 = {&c->in2, 4, 4, 0, 0, 0, 0};
    mr_ov oe0 = {&c->e0, 16, 16, 0, 0, b0, b0}, oe1 = {&c->e1, 8, 8, 0, 0, 9, 9}, oe2 = {&c->e2, 4, 4, 0, 0, 5, 5};
    int mx = 0, my = 0, rmx = 0, rmy = 0, hmx = 0, hmy = 0, qmx, qmy, xl, xr, yu, yd, tie = 0;
    short blk[256];
    ov_origin(&oin0, n, m);
    ov_origin(&oe0, n, m);
    const int zero_d = ov_tsd(&oin0, &oe0, 16);
    int min_d;

    if (c->mode == 2) { /* level 2 cross search (…MultiresCross.cpp:639-697) */
        ov_origin(&oin2, ll, kk);
        ov_origin(&oe2, ll, kk);
        int min2 = ov_tsd(&oin2, &oe2, 4);
        mr_range(&c->L2, ll, kk, 0, 0, c->l2_range - 1, &xl, &xr, &yu, &yd);
        for (int s = c->l2_range / 2; s > 0; s /= 2) {
            rmx = rmy = 0;
            for (int k = 0; k < 4; k++) {
                int i = s * CRY[k], j = s * CRX[k];
                if (i + my < yu || i + my > yd || j + mx < xl || j + mx > xr) continue;
                ov_origin(&oe2, j + ll + mx, i + kk + my);
                int d = ov_tsd4_lt(&oin2, &oe2, min2);
                if (d > min2) continue;
                if (d == min2) {
                    tie |= 1;
                    /* MultiresCross compares the centre with the offset (…:673-679) */
                    if (pred ? mr_farther_v2(c, mx, my, rmx, rmy, j, i, pred[0], pred[1])
                             : (my * my + mx * mx) - (i * i + j * j) < 0)
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

    /* level 1 (…MultiresCross.cpp:699-816) */
    const int p1x = pred ? pred[2] : 0, p1y = pred ? pred[3] : 0;
    ov_origin(&oin1, q, p);
    ov_origin(&oe1, mx + q, my + p);
    int min1 = ov_tsd(&oin1, &oe1, 8);
    rmx = rmy = 0;
    if (c->mode == 2) {
        mr_range(&c->L1, q, p, mx, my, c->lcl_l1_range, &xl, &xr, &yu, &yd);
        for (int i = yu; i <= yd; i++)
            for (int j = xl; j <= xr; j++) {
                if (!(i || j)) continue;
                ov_origin(&oe1, j + mx + q, i + my + p);
                int d = ov_tsd_partial_lt(&oin1, &oe1, 8, min1);
                if (d > min1) continue;
                if (d == min1) {
                    tie |= 2;
                    if (mr_farther_v2(c, mx, my, rmx, rmy, j, i, p1x, p1y)) continue;
                }
                min1 = d;
                rmx = j;
                rmy = i;
            }
    } else {
        for (int s = c->l1_range / 2; s > 0; s /= 2) {
            mr_range(&c->L1, q, p, mx, my, c->lcl_l1_range - 1, &xl, &xr, &yu, &yd);
            rmx = rmy = 0;
            for (int k = 0; k < 4; k++) {
                int i = s * CRY[k], j = s * CRX[k];
                if (i + my < yu || i + my > yd || j + mx < xl || j + mx > xr) continue;
                ov_origin(&oe1, j + mx + q, i + my + p);
                int d = ov_tsd_partial_lt(&oin1, &oe1, 8, min1);
                if (d > min1) continue;
                if (d == min1) {
                    tie |= 2;
                    if (mr_farther_v2(c, mx, my, rmx, rmy, j, i, p1x, p1y)) continue;
                }
                min1 = d;
                rmx = j;
                rmy = i;
            }
            mx += rmx;
            my += rmy;
        }
    }
    /* the last level-1 refinement is added once more here in the cross mode
     * (…MultiresCross.cpp:815-816) */
    mx = (mx + rmx) * 2;
    my = (my + rmy) * 2;

    /* level 0 +-2 refinement (…MultiresCross.cpp:819-873) */
    const int p0x = pred ? pred[4] : 0, p0y = pred ? pred[5] : 0;
    ov_origin(&oe0, n + mx, m + my);
    min_d = ov_tsd(&oin0, &oe0, 16);
    rmx = rmy = 0;
    mr_range(&c->L0, n, m, mx, my, 2, &xl, &xr, &yu, &yd);
    for (int i = yu; i <= yd; i++)
        for (int j = xl; j <= xr; j++) {
            if (!(i || j)) continue;
            ov_origin(&oe0, n + mx + j, m + my + i);
            int d = ov_tsd_partial_lt(&oin0, &oe0, 16, min_d);
            if (d > min_d) continue;
            if (d == min_d) {
                tie |= 4;
                if (mr_farther_v2(c, mx, my, rmx, rmy, j, i, p0x, p0y)) continue;
            }
            min_d = d;
            rmx = j;
            rmy = i;
        }
    mx += rmx;
    my += rmy;
    if (c->h263) {
        /* half pel (…H263ImplMultiresCross.cpp:885-940): the best of the four diagonal corners, then the
         * two half-pel points beside the winning corner (or the full cross if no corner won), each an
         * OverlayMem2Dv2::HalfRead block, strict improvements; vector in half pels */
        static const int CORNER[4][2] = {{-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
        static const int REFINED[4][2][2] = {{{0, -1}, {-1, 0}}, {{0, -1}, {1, 0}}, {{0, 1}, {-1, 0}}, {{0, 1}, {1, 0}}};
        static const int CROSS[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
        ov_origin(&oe0, n + mx, m + my);
        int best_corner = 0;
        for (int k = 0; k < 4; k++) {
            mr_half_read(&oe0, CORNER[k][0], CORNER[k][1], blk);
            int d = blk_tsd16_partial_lt(&oin0, blk, min_d);
            if (d < min_d) { best_corner = k; min_d = d; hmx = CORNER[k][0]; hmy = CORNER[k][1]; }
        }
        const int won = hmx || hmy;
        for (int k = 0; k < (won ? 2 : 4); k++) {
            const int hx = won ? REFINED[best_corner][k][0] : CROSS[k][0];
            const int hy = won ? REFINED[best_corner][k][1] : CROSS[k][1];
            mr_half_read(&oe0, hx, hy, blk);
            int d = blk_tsd16_partial_lt(&oin0, blk, min_d);
            if (d < min_d) { min_d = d; hmx = hx; hmy = hy; }
        }
        out->zero_d = zero_d;
        out->min_d = min_d;
        out->mvx = 2 * mx + hmx;
        out->mvy = 2 * my + hmy;
        out->tie = tie;
        return;
    }
    int mvx = mx << 2, mvy = my << 2;

    /* half then quarter pel (…MultiresCross.cpp:875-941), strict improvements */
    ov_origin(&oe0, n + mx, m + my);
    mr_load_half_window(c->win, &oe0, pred != NULL);
    for (int k = 0; k < 8; k++) {
        int qx = 2 * SUBX[k], qy = 2 * SUBY[k];
        mr_window_read(c->win, qx, qy, blk);
        int d = blk_tsd16_partial_lt(&oin0, blk, min_d);
        if (d < min_d) { min_d = d; hmx = qx; hmy = qy; }
    }
    qmx = hmx;
    qmy = hmy;
    mr_load_quarter_window(c->win, hmx, hmy);
    for (int k = 0; k < 8; k++) {
        int qx = hmx + SUBX[k], qy = hmy + SUBY[k];
        mr_window_read(c->win, qx, qy, blk);
        int d = blk_tsd16_partial_lt(&oin0, blk, min_d);
        if (d < min_d) { min_d = d; qmx = qx; qmy = qy; }
    }
    out->zero_d = zero_d;
    out->min_d = min_d;
    out->mvx = mvx + qmx;
    out->mvy = mvy + qmy;
    out->tie = tie;
}

/* The candidate lists of the Lagrangian overload: Fifo(5) of doubles
 * (include/GeneralUtils/Fifo.h), the newest item at 0.  AddFirstIn on an
 * empty list fills every slot with the item; GetLength is always 5. */
typedef struct {
    int x[5], y[5], d[5];
} mr_fifo;

static void fifo_reset(mr_fifo* f, int x, int y, int d)
{
    for (int i = 0; i < 5; i++) {
        f->x[i] = x;
        f->y[i] = y;
        f->d[i] = d;
    }
}

static void fifo_push(mr_fifo* f, int x, int y, int d)
{
    for (int i = 4; i > 0; i--) {
        f->x[i] = f->x[i - 1];
        f->y[i] = f->y[i - 1];
        f->d[i] = f->d[i - 1];
    }
    f->x[0] = x;
    f->y[0] = y;
    f->d[0] = d;
}

/* GetBestVector (include/CodecUtils/MotionEstimatorH264ImplMultiresCrossVer2.h:168-197):
 * cost D/norm + lambda*|v - ref| over the five slots; slot 0 is costed at the
 * current vector (*mx, *my) with lambda * 2^(level+2) / 16, the others with the
 * raw lambda; strict improvement.  Returns the slot and sets (*mx, *my). */
static int fifo_best(const mr_fifo* f, double lambda, double norm, int level, int xref, int yref, int* mx, int* my)
{
    const double lcl = (lambda * (double)(1 << (level + 2))) / 16.0;
    int pos = 0;
    const double mag = (double)((*mx - xref) * (*mx - xref) + (*my - yref) * (*my - yref));
    double cost = ((double)f->d[0] / norm) + (lcl * sqrt(mag));
    for (int i = 1; i < 5; i++) {
        const double m = (double)((f->x[i] - xref) * (f->x[i] - xref) + (f->y[i] - yref) * (f->y[i] - yref));
        const double c = ((double)f->d[i] / norm) + (lambda * sqrt(m));
        if (c < cost) {
            *mx = f->x[i];
            *my = f->y[i];
            cost = c;
            pos = i;
        }
    }
    return pos;
}

/* The search of MotionEstimatorH264ImplMultiresCrossVer2::Estimate(long*, void* lambda)
 * (src/CodecUtils/MotionEstimatorH264ImplMultiresCrossVer2.cpp:1237-1676): the
 * Ver2 search whose every level ends with GetBestVector over the last five
 * improvements of that level (level 2: norm 16, level 1: 64, level 0: 256,
 * sub-pel: 256 at level weight 2), each towards the prediction's vector of the
 * level.  Unlike Estimate(long*), the cross mode's level 1 adds its last
 * refinement once only (…:1434-1499).  pl = {level-2 x, y, level-1 x, y,
 * level-0 rounded x, y}; (pcx, pcy) the clamped quarter-pel prediction. */
static void mr_search_mb_lambda(mr_ctx* c, int mbr, int mbc, const int* pl, int pcx, int pcy, double lambda,
                                mr_result* out)
{
    const int m = 16 * mbr, n = 16 * mbc, p = 8 * mbr, q = 8 * mbc, kk = 4 * mbr, ll = 4 * mbc;
    mr_ov oin0 = {&c->in0, 16, 16, 0, 0, 0, 0}, oin1 = {&c->in1, 8, 8, 0, 0, 0, 0}, oin2 = {&c->in2, 4, 4, 0, 0, 0, 0};
    mr_ov oe0 = {&c->e0, 16, 16, 0, 0, 19, 19}, oe1 = {&c->e1, 8, 8, 0, 0, 9, 9}, oe2 = {&c->e2, 4, 4, 0, 0, 5, 5};
    int mx = 0, my = 0, rmx = 0, rmy = 0, hmx = 0, hmy = 0, qmx, qmy, xl, xr, yu, yd;
    mr_fifo f;
    short blk[256];
    ov_origin(&oin0, n, m);
    ov_origin(&oe0, n, m);
    const int zero_d = ov_tsd(&oin0, &oe0, 16);

    if (c->mode == 2) { /* level 2 cross search (…:1287-1370) */
        ov_origin(&oin2, ll, kk);
        ov_origin(&oe2, ll, kk);
        int min2 = ov_tsd(&oin2, &oe2, 4);
        fifo_reset(&f, 0, 0, min2);
        mr_range(&c->L2, ll, kk, 0, 0, c->l2_range - 1, &xl, &xr, &yu, &yd);
        for (int s = c->l2_range / 2; s > 0; s /= 2) {
            rmx = rmy = 0;
            for (int k = 0; k < 4; k++) {
                int i = s * CRY[k], j = s * CRX[k];
                if (i + my < yu || i + my > yd || j + mx < xl || j + mx > xr) continue;
                ov_origin(&oe2, j + ll + mx, i + kk + my);
                int d = ov_tsd4_lt(&oin2, &oe2, min2);
                if (d > min2) continue;
                if (d == min2 && mr_farther(mx, my, rmx, rmy, j, i, pl[0], pl[1])) continue;
                min2 = d;
                rmx = j;
                rmy = i;
                fifo_push(&f, j + mx, i + my, d);
            }
            mx += rmx;
            my += rmy;
        }
        fifo_best(&f, lambda, 16.0, 2, pl[0], pl[1], &mx, &my);
        mx <<= 1;
        my <<= 1;
    }

    /* level 1 (…:1374-1502) */
    ov_origin(&oin1, q, p);
    ov_origin(&oe1, mx + q, my + p);
    int min1 = ov_tsd(&oin1, &oe1, 8);
    fifo_reset(&f, mx, my, min1);
    rmx = rmy = 0;
    if (c->mode == 2) {
        mr_range(&c->L1, q, p, mx, my, c->lcl_l1_range, &xl, &xr, &yu, &yd);
        for (int i = yu; i <= yd; i++)
            for (int j = xl; j <= xr; j++) {
                if (!(i || j)) continue;
                ov_origin(&oe1, j + mx + q, i + my + p);
                int d = ov_tsd_partial_lt(&oin1, &oe1, 8, min1);
                if (d > min1) continue;
                if (d == min1 && mr_farther(mx, my, rmx, rmy, j, i, pl[2], pl[3])) continue;
                min1 = d;
                rmx = j;
                rmy = i;
                fifo_push(&f, j + mx, i + my, d);
            }
        mx += rmx;
        my += rmy;
    } else {
        for (int s = c->l1_range / 2; s > 0; s /= 2) {
            mr_range(&c->L1, q, p, mx, my, c->lcl_l1_range - 1, &xl, &xr, &yu, &yd);
            rmx = rmy = 0;
            for (int k = 0; k < 4; k++) {
                int i = s * CRY[k], j = s * CRX[k];
                if (i + my < yu || i + my > yd || j + mx < xl || j + mx > xr) continue;
                ov_origin(&oe1, j + mx + q, i + my + p);
                int d = ov_tsd_partial_lt(&oin1, &oe1, 8, min1);
                if (d > min1) continue;
                if (d == min1 && mr_farther(mx, my, rmx, rmy, j, i, pl[2], pl[3])) continue;
                min1 = d;
                rmx = j;
                rmy = i;
                fifo_push(&f, j + mx, i + my, d);
            }
            mx += rmx;
            my += rmy;
        }
    }
    fifo_best(&f, lambda, 64.0, 1, pl[2], pl[3], &mx, &my);
    mx <<= 1;
    my <<= 1;

    /* level 0 +-2 refinement (…:1503-1574) */
    int min_d = zero_d;
    if (mx || my) {
        ov_origin(&oe0, n + mx, m + my);
        min_d = ov_tsd(&oin0, &oe0, 16);
    }
    fifo_reset(&f, mx, my, min_d);
    rmx = rmy = 0;
    mr_range(&c->L0, n, m, mx, my, 2, &xl, &xr, &yu, &yd);
    for (int i = yu; i <= yd; i++)
        for (int j = xl; j <= xr; j++) {
            if (!(i || j)) continue;
            ov_origin(&oe0, n + mx + j, m + my + i);
            int d = ov_tsd_partial_lt(&oin0, &oe0, 16, min_d);
            if (d > min_d) continue;
            if (d == min_d && mr_farther(mx, my, rmx, rmy, j, i, pl[4], pl[5])) continue;
            min_d = d;
            rmx = j;
            rmy = i;
            fifo_push(&f, j + mx, i + my, d);
        }
    mx += rmx;
    my += rmy;
    min_d = f.d[fifo_best(&f, lambda, 256.0, 0, pl[4], pl[5], &mx, &my)];

    /* half then quarter pel in Ver2's window (…:1575-1662), strict improvements */
    int mvx = mx << 2, mvy = my << 2;
    fifo_reset(&f, mvx, mvy, min_d);
    ov_origin(&oe0, n + mx, m + my);
    mr_load_half_window(c->win, &oe0, 1);
    for (int k = 0; k < 8; k++) {
        int qx = 2 * SUBX[k], qy = 2 * SUBY[k];
        mr_window_read(c->win, qx, qy, blk);
        int d = blk_tsd16_partial_lt(&oin0, blk, min_d);
        if (d < min_d) {
            min_d = d;
            hmx = qx;
            hmy = qy;
            fifo_push(&f, qx + mvx, qy + mvy, d);
        }
    }
    qmx = hmx;
    qmy = hmy;
    mr_load_quarter_window(c->win, hmx, hmy);
    for (int k = 0; k < 8; k++) {
        int qx = hmx + SUBX[k], qy = hmy + SUBY[k];
        mr_window_read(c->win, qx, qy, blk);
        int d = blk_tsd16_partial_lt(&oin0, blk, min_d);
        if (d < min_d) {
            min_d = d;
            qmx = qx;
            qmy = qy;
            fifo_push(&f, qx + mvx, qy + mvy, d);
        }
    }
    mvx += qmx;
    mvy += qmy;
    /* towards the clamped quarter-pel prediction (…:1664-1677) */
    min_d = f.d[fifo_best(&f, lambda, 256.0, 2, pcx, pcy, &mvx, &mvy)];
    out->zero_d = zero_d;
    out->min_d = min_d;
    out->mvx = mvx;
    out->mvy = mvy;
    out->tie = 0;
}

static int me_multires_cross_any(int h263, const short* src, const short* ref, int w, int h, int motion_range,
                                 int mode, const unsigned char* dist_incl, short* mv_out, int* mb_dist, long* avg_dist);

int vo_me_multires_cross(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                         const unsigned char* dist_incl, short* mv_out, int* mb_dist, long* avg_dist)
{
    return me_multires_cross_any(0, src, ref, w, h, motion_range, mode, dist_incl, mv_out, mb_dist, avg_dist);
}

/* MotionEstimatorH263ImplMultiresCross::Estimate
 * (src/CodecUtils/MotionEstimatorH263ImplMultiresCross.cpp:531-1010): the
 * H.264 estimator's levels and level-0 refinement at its doubled range, the
 * HalfRead half-pel stage, vectors in half pels and the accept rule with
 * (zero - min) >> 2 against |v|^2. */
int vo_me_h263_multires_cross(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                              const unsigned char* dist_incl, short* mv_out, int* mb_dist, long* avg_dist)
{
    return me_multires_cross_any(1, src, ref, w, h, motion_range, mode, dist_incl, mv_out, mb_dist, avg_dist);
}

static int me_multires_cross_any(int h263, const short* src, const short* ref, int w, int h, int motion_range,
                                 int mode, const unsigned char* dist_incl, short* mv_out, int* mb_dist, long* avg_dist)
{
    if (!src || !ref || !mv_out || w < 16 || h < 16 || (w % 16) != 0) return -1;
    g_mr_fault = 0;
    mr_ctx c;
    int rc = mr_ctx_init_h(&c, src, ref, w, h, motion_range, mode, h263);
    if (rc == 0) {
        long total = 0;
        int included = 0;
        for (int mbr = 0; mbr < c.rows_all; mbr++)
            for (int mbc = 0; mbc < c.cols; mbc++) {
                const int vec_pos = mbr * c.cols + mbc < c.nmb ? mbr * c.cols + mbc : c.nmb;
                mr_result r;
                mr_search_mb(&c, mbr, mbc, NULL, &r);
                int mvx = r.mvx, mvy = r.mvy;
                /* accept-or-zero heuristic (…MultiresCross.cpp:943-999) */
                int weight = 0, diff0 = r.zero_d - r.min_d, mag = mvx * mvx + mvy * mvy;
                if (h263 ? (diff0 >> 2) < mag : diff0 < mag) weight++;
                if (r.zero_d < MRC_NOISE_FLOOR) weight++;
                if (diff0 * 10 < r.min_d) weight++;
                int do_it = dist_incl ? (vec_pos < c.nmb ? dist_incl[vec_pos] != 0 : 0) : 1;
                int chosen;
                if (r.min_d < r.zero_d && weight < 2) {
                    chosen = r.min_d;
                } else {
                    mvx = mvy = 0;
                    chosen = r.zero_d;
                }
                if (do_it) {
                    included++;
                    total += chosen;
                }
                if (vec_pos < c.nmb) {
                    mv_out[2 * vec_pos] = (short)mvx;
                    mv_out[2 * vec_pos + 1] = (short)mvy;
                    if (mb_dist) mb_dist[vec_pos] = chosen;
                }
            }
        if (avg_dist) *avg_dist = included ? total / included : 0;
        if (g_mr_fault) rc = -3;
    }
    mr_ctx_free(&c);
    return rc;
}

/* H263MotionVectorPredictorImpl1::Get16x16Prediction (src/CodecUtils/H263MotionVectorPredictorImpl1.cpp:72-128)
 * over the vectors written so far: in the top row the left neighbour (0 at the left edge), else the
 * componentwise median of left, above and above-right, each 0 beyond the left or right edge. */
static void h263_pred(const short* mv, int cols, int blk, int* px, int* py)
{
    const int mby = blk / cols, mbx = blk % cols;
    int a[2] = {0, 0}, b[2], c[2] = {0, 0};
    if (mbx > 0) {
        a[0] = mv[2 * (mby * cols + mbx - 1)];
        a[1] = mv[2 * (mby * cols + mbx - 1) + 1];
    }
    if (mby < 1) {
        *px = a[0];
        *py = a[1];
        return;
    }
    b[0] = mv[2 * ((mby - 1) * cols + mbx)];
    b[1] = mv[2 * ((mby - 1) * cols + mbx) + 1];
    if (mbx + 1 < cols) {
        c[0] = mv[2 * ((mby - 1) * cols + mbx + 1)];
        c[1] = mv[2 * ((mby - 1) * cols + mbx + 1) + 1];
    }
    int out[2];
    for (int k = 0; k < 2; k++) {
        int lo = b[k] < c[k] ? b[k] : c[k], hi = b[k] < c[k] ? c[k] : b[k];
        if (a[k] < lo) lo = a[k];
        if (a[k] > hi) hi = a[k];
        out[k] = a[k] + b[k] + c[k] - lo - hi;
    }
    *px = out[0];
    *py = out[1];
}

/* MotionEstimatorH263ImplMultiresCrossVer2::Estimate
 * (src/CodecUtils/MotionEstimatorH263ImplMultiresCrossVer2.cpp:537-1151): the H.263 MultiresCross
 * search with ties decided towards the prediction of each level (half-pel prediction rounded away
 * from zero to full pels, then halved per level, :622-639) by the rule of mr_farther_v2; then the
 * distortion at the prediction clamped to one macroblock outside the picture (HalfRead for its half
 * components, :1012-1050) competes with the zero vector's, and the accept rule of MultiresCross picks
 * the searched vector or the better of the two (:1052-1142).  The prediction of a partial bottom row
 * is that of index N_MB (vecPos stops there); its results only enter the average. */
int vo_me_h263_multires_cross_ver2(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                                   const unsigned char* dist_incl, short* mv_out, int* mb_dist, long* avg_dist)
{
    if (!src || !ref || !mv_out || w < 16 || h < 16 || (w % 16) != 0) return -1;
    g_mr_fault = 0;
    mr_ctx c;
    int rc = mr_ctx_init_h(&c, src, ref, w, h, motion_range, mode, 1);
    c.tie_plus_y = 1;
    if (rc == 0) {
        long total = 0;
        int included = 0;
        short blk[256];
        for (int mbr = 0; mbr < c.rows_all; mbr++)
            for (int mbc = 0; mbc < c.cols; mbc++) {
                const int vec_pos = mbr * c.cols + mbc < c.nmb ? mbr * c.cols + mbc : c.nmb;
                const int n = 16 * mbc, m = 16 * mbr;
                int px, py;
                h263_pred(mv_out, c.cols, vec_pos, &px, &py);
                const int pxh = px % 2, pyh = py % 2;
                int px0 = px / 2, py0 = py / 2;
                const int px0r = px < 0 ? (px - 1) / 2 : (px + 1) / 2, py0r = py < 0 ? (py - 1) / 2 : (py + 1) / 2;
                const int pl[6] = {px0r / 2 / 2, py0r / 2 / 2, px0r / 2, py0r / 2, px0r, py0r};
                mr_result r;
                mr_search_mb(&c, mbr, mbc, pl, &r);
                int mvx = r.mvx, mvy = r.mvy;
                if (px0 + n > w) px0 = 16;
                if (px0 + n < -16) px0 = -16;
                if (py0 + m > h) py0 = 16;
                if (py0 + m < -16) py0 = -16;
                const int pvx = 2 * px0 + pxh, pvy = 2 * py0 + pyh;
                mr_ov oin0 = {&c.in0, 16, 16, 0, 0, 0, 0}, oe0 = {&c.e0, 16, 16, 0, 0, 17, 17};
                ov_origin(&oin0, n, m);
                ov_origin(&oe0, px0 + n, py0 + m);
                int pred_d;
                if (pxh || pyh) {
                    mr_half_read(&oe0, pxh, pyh, blk);
                    pred_d = 0;
                    for (int i = 0; i < 256; i++) {
                        const int d = ov_px(&oin0, i / 16, i % 16) - blk[i];
                        pred_d += d * d;
                    }
                } else {
                    pred_d = ov_tsd(&oin0, &oe0, 16);
                }
                int zx = pvx, zy = pvy, zd = pred_d;
                if (r.zero_d < zd) {
                    zd = r.zero_d;
                    zx = zy = 0;
                }
                int weight = 0, diff0 = zd - r.min_d, mag = mvx * mvx + mvy * mvy;
                if ((diff0 >> 2) < mag) weight++;
                if (zd < MRC_NOISE_FLOOR) weight++;
                if (diff0 * 10 < r.min_d) weight++;
                int do_it = dist_incl ? (vec_pos < c.nmb ? dist_incl[vec_pos] != 0 : 0) : 1;
                int chosen;
                if (r.min_d < zd && weight < 2) {
                    chosen = r.min_d;
                } else {
                    mvx = zx;
                    mvy = zy;
                    chosen = zd;
                }
                if (do_it) {
                    included++;
                    total += chosen;
                }
                if (vec_pos < c.nmb) {
                    mv_out[2 * vec_pos] = (short)mvx;
                    mv_out[2 * vec_pos + 1] = (short)mvy;
                    if (mb_dist) mb_dist[vec_pos] = chosen;
                }
            }
        if (avg_dist) *avg_dist = included ? total / included : 0;
        if (g_mr_fault) rc = -3;
    }
    mr_ctx_free(&c);
    return rc;
}

/* The search of MotionEstimatorH264ImplMultires::Estimate
 * (src/CodecUtils/MotionEstimatorH264ImplMultires.cpp:644-917) for macroblock
 * (mbr, mbc): full searches at level 2 (around (0, 0)) and level 1 (around
 * the level-2 winner), +-2 at level 0, then half and quarter pel in the
 * MultiresCross-style window.  Its LessThan distortions (…:701, 764, 822, 873,
 * 899) stop early only on a sum above the running minimum, so full SSDs give
 * the same decisions.  Ties are measured from the prediction rounded to each
 * level, pl = {level-2 x, y, level-1 x, y, level-0 x, y} (…:646-655). */
static void mr_search_mb_multires(mr_ctx* c, int mbr, int mbc, const int* pl, mr_result* out)
{
    const int m = 16 * mbr, n = 16 * mbc, p = 8 * mbr, q = 8 * mbc, kk = 4 * mbr, ll = 4 * mbc;
    mr_ov oin0 = {&c->in0, 16, 16, 0, 0, 0, 0}, oin1 = {&c->in1, 8, 8, 0, 0, 0, 0}, oin2 = {&c->in2, 4, 4, 0, 0, 0, 0};
    mr_ov oe0 = {&c->e0, 16, 16, 0, 0, 19, 19}, oe1 = {&c->e1, 8, 8, 0, 0, 9, 9}, oe2 = {&c->e2, 4, 4, 0, 0, 5, 5};
    int mx = 0, my = 0, rmx = 0, rmy = 0, hmx = 0, hmy = 0, qmx, qmy, xl, xr, yu, yd, tie = 0;
    short blk[256];
    ov_origin(&oin0, n, m);
    ov_origin(&oe0, n, m);
    const int zero_d = ov_tsd(&oin0, &oe0, 16);

    if (c->mode == 2) { /* level 2 full search (…:667-731) */
        ov_origin(&oin2, ll, kk);
        ov_origin(&oe2, ll, kk);
        int min2 = ov_tsd(&oin2, &oe2, 4);
        mr_range(&c->L2, ll, kk, 0, 0, c->l2_range - 1, &xl, &xr, &yu, &yd);
        for (int i = yu; i <= yd; i++)
            for (int j = xl; j <= xr; j++) {
                if (!(i || j)) continue;
                ov_origin(&oe2, ll + j, kk + i);
                int d = ov_tsd(&oin2, &oe2, 4);
                if (d > min2) continue;
                if (d == min2) {
                    tie |= 1;
                    if (mr_farther(0, 0, mx, my, j, i, pl[0], pl[1])) continue;
                }
                min2 = d;
                mx = j;
                my = i;
            }
        mx <<= 1;
        my <<= 1;
    }

    /* level 1 around (mx, my) (…:735-790) */
    ov_origin(&oin1, q, p);
    ov_origin(&oe1, mx + q, my + p);
    int min1 = ov_tsd(&oin1, &oe1, 8);
    mr_range(&c->L1, q, p, mx, my, c->lcl_l1_range, &xl, &xr, &yu, &yd);
    for (int i = yu; i <= yd; i++)
        for (int j = xl; j <= xr; j++) {
            if (!(i || j)) continue;
            ov_origin(&oe1, j + mx + q, i + my + p);
            int d = ov_tsd(&oin1, &oe1, 8);
            if (d > min1) continue;
            if (d == min1) {
                tie |= 2;
                if (mr_farther(mx, my, rmx, rmy, j, i, pl[2], pl[3])) continue;
            }
            min1 = d;
            rmx = j;
            rmy = i;
        }
    mx = (mx + rmx) * 2;
    my = (my + rmy) * 2;

    /* level 0 +-2 (…:792-849) */
    ov_origin(&oe0, n + mx, m + my);
    int min_d = ov_tsd(&oin0, &oe0, 16);
    rmx = rmy = 0;
    mr_range(&c->L0, n, m, mx, my, 2, &xl, &xr, &yu, &yd);
    for (int i = yu; i <= yd; i++)
        for (int j = xl; j <= xr; j++) {
            if (!(i || j)) continue;
            ov_origin(&oe0, n + mx + j, m + my + i);
            int d = ov_tsd(&oin0, &oe0, 16);
            if (d > min_d) continue;
            if (d == min_d) {
                tie |= 4;
                if (mr_farther(mx, my, rmx, rmy, j, i, pl[4], pl[5])) continue;
            }
            min_d = d;
            rmx = j;
            rmy = i;
        }
    mx += rmx;
    my += rmy;
    int mvx = mx << 2, mvy = my << 2;

    /* half then quarter pel (…:851-917), strict improvements */
    ov_origin(&oe0, n + mx, m + my);
    mr_load_half_window(c->win, &oe0, 0);
    for (int k = 0; k < 8; k++) {
        int qx = 2 * SUBX[k], qy = 2 * SUBY[k];
        mr_window_read(c->win, qx, qy, blk);
        int d = vo_tsd16(oin0.b->mem + (size_t)oin0.y * oin0.b->w + oin0.x, oin0.b->w, blk, 16);
        if (d < min_d) { min_d = d; hmx = qx; hmy = qy; }
    }
    qmx = hmx;
    qmy = hmy;
    mr_load_quarter_window(c->win, hmx, hmy);
    for (int k = 0; k < 8; k++) {
        int qx = hmx + SUBX[k], qy = hmy + SUBY[k];
        mr_window_read(c->win, qx, qy, blk);
        int d = vo_tsd16(oin0.b->mem + (size_t)oin0.y * oin0.b->w + oin0.x, oin0.b->w, blk, 16);
        if (d < min_d) { min_d = d; qmx = qx; qmy = qy; }
    }
    out->zero_d = zero_d;
    out->min_d = min_d;
    out->mvx = mvx + qmx;
    out->mvy = mvy + qmy;
    out->tie = tie;
}

/* MotionEstimatorH264ImplMultiresCrossVer2::Estimate(long*)
 * (src/CodecUtils/MotionEstimatorH264ImplMultiresCrossVer2.cpp:537-1151): the
 * MultiresCross search with ties resolved towards the rounded median
 * prediction of each level (…:627-642), then the pred-vector check and the
 * Lagrangian choice among {search winner, prediction, zero} with lambda 0.9
 * (…:1008-1064; GetBestVector at level 2 weighs every item with lambda,
 * MultiresCrossVer2.h:168-197).  Only full macroblock rows are estimated: the
 * reference drops the partial bottom row's vectors (…:1137) and asks the
 * predictor for an index past its array for it.  tie_out (nullable): per MB,
 * the integer stages that met an equal distortion (1 level 2, 2 level 1,
 * 4 level 0; the search then depends on the prediction). */
static int me_multires_pred(int multires, const short* src, const short* ref, int w, int h, int motion_range,
                            int mode, const unsigned char* dist_incl, const int* slice, short* mv_out, int* mb_dist,
                            long* avg_dist, int* tie_out, const double* lambda)
{
    if (!src || !ref || !mv_out || w < 16 || h < 16 || (w % 16) != 0) return -1;
    g_mr_fault = 0;
    mr_ctx c;
    vo_pred_state ps;
    const int rows = h / 16;
    int rc = mr_ctx_init(&c, src, ref, w, h, motion_range, mode);
    if (rc == 0 && vo_pred_init(&ps, c.cols, rows, slice) != 0) {
        vo_pred_free(&ps);
        rc = -2;
    }
    if (rc == 0) {
        const int es = w + 38;
        long total = 0;
        int included = 0;
        for (int k = 0; k < c.nmb; k++) {
            const int mbr = k / c.cols, mbc = k % c.cols, n = 16 * mbc, m = 16 * mbr;
            int px, py;
            vo_pred_get(&ps, k, &px, &py);
            const int pxq = px % 4, pyq = py % 4;
            int px0 = px / 4, py0 = py / 4;
            const int px0r = px < 0 ? (px - 2) / 4 : (px + 2) / 4, py0r = py < 0 ? (py - 2) / 4 : (py + 2) / 4;
            mr_result r;
            if (lambda) {
                /* the clamped prediction of the last two GetBestVector calls (…:1664-1675) */
                int cx0 = px0, cy0 = py0;
                if (cx0 + n > w) cx0 = 16;
                if (cx0 + n < -16) cx0 = -16;
                if (cy0 + m > h) cy0 = 16;
                if (cy0 + m < -16) cy0 = -16;
                const int pl[6] = {px0r / 2 / 2, py0r / 2 / 2, px0r / 2, py0r / 2, px0r, py0r};
                mr_search_mb_lambda(&c, mbr, mbc, pl, 4 * cx0 + pxq, 4 * cy0 + pyq, *lambda, &r);
            } else if (multires) {
                /* Multires rounds to every level (…Multires.cpp:646-655) */
                const int pl[6] = {px < 0 ? (px - 8) / 16 : (px + 8) / 16, py < 0 ? (py - 8) / 16 : (py + 8) / 16,
                                   px < 0 ? (px - 4) / 8 : (px + 4) / 8,   py < 0 ? (py - 4) / 8 : (py + 4) / 8,
                                   px0r, py0r};
                mr_search_mb_multires(&c, mbr, mbc, pl, &r);
            } else {
                const int pl[6] = {px0r / 2 / 2, py0r / 2 / 2, px0r / 2, py0r / 2, px0r, py0r};
                mr_search_mb(&c, mbr, mbc, pl, &r);
            }
            if (tie_out) tie_out[k] = r.tie;

            /* pred-vector check, clamped to one macroblock outside (…:1008-1045) */
            if (px0 + n > w) px0 = 16;
            if (px0 + n < -16) px0 = -16;
            if (py0 + m > h) py0 = 16;
            if (py0 + m < -16) py0 = -16;
            px = 4 * px0 + pxq;
            py = 4 * py0 + pyq;
            const int pox = vo_clamp_origin(px0 + n + 19, es, 16), poy = vo_clamp_origin(py0 + m + 19, h + 38, 16);
            const short* in = src + (size_t)m * w + n;
            int pd;
            if (pxq || pyq) {
                short blk[256];
                vo_qread16_ext(c.e0.mem, es, pox, poy, pxq, pyq, blk);
                pd = vo_tsd16(in, w, blk, 16);
            } else {
                pd = vo_tsd16(in, w, c.e0.mem + (size_t)poy * es + pox, es);
            }
            /* Fifo after pushing zero, pred, best (…:1047-1050) */
            int xs[5] = {r.mvx, px, 0, 0, 0}, ys[5] = {r.mvy, py, 0, 0, 0};
            int ds[5] = {r.min_d, pd, r.zero_d, r.zero_d, r.zero_d};
            const int pos = vo_best_vector5(xs, ys, ds, lambda ? *lambda : (multires ? 1.1 : 0.9), 256.0, px, py);
            if (dist_incl && dist_incl[k]) {
                included++;
                total += ds[pos];
            }
            if (mb_dist) mb_dist[k] = ds[pos];
            mv_out[2 * k] = (short)xs[pos];
            mv_out[2 * k + 1] = (short)ys[pos];
            vo_pred_set(&ps, k, xs[pos], ys[pos]);
        }
        if (avg_dist) *avg_dist = included ? total / included : 0;
        vo_pred_free(&ps);
        if (g_mr_fault) rc = -3;
    }
    mr_ctx_free(&c);
    return rc;
}

int vo_me_multires_cross_v2(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                            const unsigned char* dist_incl, const int* slice, short* mv_out, int* mb_dist,
                            long* avg_dist, int* tie_out)
{
    return me_multires_pred(0, src, ref, w, h, motion_range, mode, dist_incl, slice, mv_out, mb_dist, avg_dist,
                            tie_out, NULL);
}

/* MotionEstimatorH264ImplMultiresCrossVer2::Estimate(long*, void* lambda)
 * (src/CodecUtils/MotionEstimatorH264ImplMultiresCrossVer2.cpp:1162-1742): the
 * search above with GetBestVector at every level, then the pred-vector check
 * and the final GetBestVector (…:1704-1710) with the given lambda.  Full
 * macroblock rows only, as for Estimate(long*). */
int vo_me_multires_cross_v2_lambda(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                                   double lambda, const unsigned char* dist_incl, const int* slice, short* mv_out,
                                   int* mb_dist, long* avg_dist)
{
    return me_multires_pred(0, src, ref, w, h, motion_range, mode, dist_incl, slice, mv_out, mb_dist, avg_dist, NULL,
                            &lambda);
}

/* MotionEstimatorH264ImplMultires::Estimate (src/CodecUtils/MotionEstimatorH264ImplMultires.cpp:557-1024):
 * the search above with the prediction rounded to each level, the pred-vector
 * check and GetBestVector with lambda 1.1 (…:958).  Full macroblock rows only,
 * as for Ver2. */
int vo_me_multires(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                   const unsigned char* dist_incl, const int* slice, short* mv_out, int* mb_dist, long* avg_dist,
                   int* tie_out)
{
    return me_multires_pred(1, src, ref, w, h, motion_range, mode, dist_incl, slice, mv_out, mb_dist, avg_dist,
                            tie_out, NULL);
}
