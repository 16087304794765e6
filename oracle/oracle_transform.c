/*
 * oracle_transform.c -- TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * Restatement of the H.264 4x4 forward integer transform with quantisation
 * (FastForward4x4ITImpl1 / Impl2 / FastForward4x4On16x16ITImpl1) and the
 * dequantisation + inverse transform (FastInverse4x4ITImpl1,
 * FastInverse4x4On16x16ITImpl1).  Every intermediate is stored to a `short`
 * at the same points as the reference, so int16 wrap-around is reproduced.
 */
#include "oracle_internal.h"

/* Multiplication factors MF[qp%6][class] and the position -> class map
 * (FastForward4x4ITImpl1.cpp:57-73). */
static const int FWD_MF[6][3] = {
    {13107, 5243, 8066}, {11916, 4660, 7490}, {10082, 4194, 6554},
    {9362, 3647, 5825},  {8192, 3355, 5243},  {7282, 2893, 4559}};
/* Dequantisation scales V[qp%6][class] (FastInverse4x4ITImpl1.cpp:60-67). */
static const int INV_V[6][3] = {
    {10, 16, 13}, {11, 18, 14}, {13, 20, 16}, {14, 23, 18}, {16, 25, 20}, {18, 29, 23}};
/* Class of coefficient position 4*row+col: 0 = (even,even), 1 = (odd,odd), 2 = mixed. */
static int pos_class(int row, int col)
{
    int ro = row & 1, co = col & 1;
    if (!ro && !co) return 0;
    if (ro && co) return 1;
    return 2;
}

/* Forward quantiser of one coefficient: sign-magnitude, (|x|*MF + f) >> (15+qp/6),
 * f = 2^(15+qp/6)/3 intra or /6 inter (FastForward4x4ITImpl1.cpp:130-160, 269-278). */
static short fwd_quant(int x, int mf, int f, int sh)
{
    if (x < 0) return (short)(-((((-x) * mf) + f) >> sh));
    return (short)(((x * mf) + f) >> sh);
}

/* Apply the forward transform to one 4x4 block addressed as p[r*rs + c]. */
static void fwd_block(short* p, int rs, int mode, int qm, int f, int sh)
{
    if (mode == 2) { /* quantisation only */
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++)
                p[r * rs + c] = fwd_quant(p[r * rs + c], FWD_MF[qm][pos_class(r, c)], f, sh);
        return;
    }
    /* Rows: even/odd butterflies, stored as short (FastForward4x4ITImpl1.cpp:110-124). */
    for (int r = 0; r < 4; r++) {
        short* q = p + r * rs;
        int s0 = (int)q[0] + q[3], s3 = (int)q[0] - q[3];
        int s1 = (int)q[1] + q[2], s2 = (int)q[1] - q[2];
        q[0] = (short)(s0 + s1);
        q[2] = (short)(s0 - s1);
        q[1] = (short)(s2 + (s3 << 1));
        q[3] = (short)(s3 - (s2 << 1));
    }
    /* Columns (and quantisation in mode 0) (FastForward4x4ITImpl1.cpp:127-182). */
    for (int c = 0; c < 4; c++) {
        int s0 = (int)p[c] + p[3 * rs + c], s3 = (int)p[c] - p[3 * rs + c];
        int s1 = (int)p[rs + c] + p[2 * rs + c], s2 = (int)p[rs + c] - p[2 * rs + c];
        int y[4] = {s0 + s1, s2 + (s3 << 1), s0 - s1, s3 - (s2 << 1)};
        for (int r = 0; r < 4; r++) {
            if (mode == 0)
                p[r * rs + c] = fwd_quant(y[r], FWD_MF[qm][pos_class(r, c)], f, sh);
            else
                p[r * rs + c] = (short)y[r];
        }
    }
}

void vo_fwd4x4(short* data, int nunits, int layout, int mode, int qp, int intra)
{
    int qm = qp % 6, qe = qp / 6;
    int f = intra ? (1 << (15 + qe)) / 3 : (1 << (15 + qe)) / 6;
    int sh = 15 + qe;
    for (int u = 0; u < nunits; u++) {
        if (layout == 0) {
            fwd_block(data + (size_t)u * 16, 4, mode, qm, f, sh);
        } else {
            short* mb = data + (size_t)u * 256;
            for (int br = 0; br < 4; br++)
                for (int bc = 0; bc < 4; bc++)
                    fwd_block(mb + br * 64 + bc * 4, 16, mode, qm, f, sh);
        }
    }
}

typedef struct {
    int level[16]; /* V * weight per position */
    int q, f, right, left;
} inv_params;

/* FastInverse4x4ITImpl1 constructor / SetParameter / SetScale
 * (FastInverse4x4ITImpl1.cpp:83-110, 251-303). */
static void inv_setup(inv_params* ip, int qp, const int* weight)
{
    int qm = qp % 6, qe = qp / 6;
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++)
            ip->level[4 * r + c] = INV_V[qm][pos_class(r, c)] * (weight ? weight[4 * r + c] : 16);
    ip->q = qp;
    ip->f = (qe <= 3) ? (1 << (3 - qe)) : 0;
    ip->right = 4 - qe;
    ip->left = qe - 4;
}

static int dequant(int x, const inv_params* ip, int pos)
{
    int v = x * ip->level[pos];
    return ip->q < 24 ? (v + ip->f) >> ip->right : v << ip->left;
}

/* 1-D inverse butterfly of (x0,x1,x2,x3) -> (y0..y3). */
static void inv_1d(int x0, int x1, int x2, int x3, int* y)
{
    int s0 = x0 + x2, s1 = x0 - x2;
    int s2 = (x1 >> 1) - x3, s3 = x1 + (x3 >> 1);
    y[0] = s0 + s3;
    y[1] = s1 + s2;
    y[2] = s1 - s2;
    y[3] = s0 - s3;
}

/* Row-first inverse (FastInverse4x4ITImpl1::InverseTransform, .cpp:119-236):
 * dequantise in the row pass (mode 0), store short, then columns with
 * (x + 32) >> 6. */
static void inv_block_rows_first(short* p, int rs, int mode, const inv_params* ip)
{
    int y[4];
    for (int r = 0; r < 4; r++) {
        short* q = p + r * rs;
        int x[4];
        for (int c = 0; c < 4; c++) x[c] = (mode == 0) ? dequant(q[c], ip, 4 * r + c) : (int)q[c];
        inv_1d(x[0], x[1], x[2], x[3], y);
        for (int c = 0; c < 4; c++) q[c] = (short)y[c];
    }
    for (int c = 0; c < 4; c++) {
        inv_1d(p[c], p[rs + c], p[2 * rs + c], p[3 * rs + c], y);
        for (int r = 0; r < 4; r++) p[r * rs + c] = (short)((y[r] + 32) >> 6);
    }
}

/* Column-first inverse (FastInverse4x4On16x16ITImpl1::InverseTransform,
 * .cpp:120-361): dequantise in the column pass (mode 0), store short, then
 * rows with (x + 32) >> 6. */
static void inv_block_cols_first(short* p, int rs, int mode, const inv_params* ip)
{
    int y[4];
    for (int c = 0; c < 4; c++) {
        int x[4];
        for (int r = 0; r < 4; r++) x[r] = (mode == 0) ? dequant(p[r * rs + c], ip, 4 * r + c) : (int)p[r * rs + c];
        inv_1d(x[0], x[1], x[2], x[3], y);
        for (int r = 0; r < 4; r++) p[r * rs + c] = (short)y[r];
    }
    for (int r = 0; r < 4; r++) {
        short* q = p + r * rs;
        inv_1d(q[0], q[1], q[2], q[3], y);
        for (int c = 0; c < 4; c++) q[c] = (short)((y[c] + 32) >> 6);
    }
}

static void dequant_block(short* p, int rs, const inv_params* ip)
{
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) p[r * rs + c] = (short)dequant(p[r * rs + c], ip, 4 * r + c);
}

void vo_inv4x4(short* data, int nunits, int layout, int mode, int qp, const int* weight_scale16)
{
    inv_params ip;
    inv_setup(&ip, qp, weight_scale16);
    for (int u = 0; u < nunits; u++) {
        if (layout == 0) {
            short* b = data + (size_t)u * 16;
            if (mode == 2) dequant_block(b, 4, &ip);
            else inv_block_rows_first(b, 4, mode, &ip);
        } else {
            short* mb = data + (size_t)u * 256;
            for (int br = 0; br < 4; br++)
                for (int bc = 0; bc < 4; bc++) {
                    short* b = mb + br * 64 + bc * 4;
                    if (mode == 2) dequant_block(b, 16, &ip);
                    else inv_block_cols_first(b, 16, mode, &ip);
                }
        }
    }
}

/* FastForward4x4ITImpl2::QuantiseValue (FastForward4x4ITImpl2.cpp:640-683). */
int vo_quantise_value(short val, int pos, int qp, int intra)
{
    int qm = qp % 6, qe = qp / 6;
    int f = intra ? (1 << (15 + qe)) / 3 : (1 << (15 + qe)) / 6;
    int mf = FWD_MF[qm][pos_class(pos / 4, pos % 4)];
    return (int)fwd_quant((int)val, mf, f, 15 + qe);
}
