/*
 * oracle_dc.c -- TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * Restatement of the H.264 DC Hadamard transforms with their quantisers:
 * FastForwardDC4x4ITImpl1 / FastInverseDC4x4ITImpl1 (the Intra16x16 luma DC
 * block) and FastForwardDC2x2ITImpl1 / FastInverseDC2x2ITImpl1 (the chroma DC
 * block).  Every intermediate the reference stores to a `short` is
 * truncated to 16 bits at the same point, so int16 wrap-around is
 * reproduced.  Units are contiguous 16-short (4x4) or 4-short (2x2) blocks,
 * one Transform(void*) / InverseTransform(void*) call each.
 */
#include "oracle_internal.h"

/* Forward scale NormAdjust[qp%6] (FastForwardDC4x4ITImpl1.cpp:63-71, the
 * same table in FastForwardDC2x2ITImpl1.cpp:62-70) and inverse
 * NormAdjust[qp%6] (FastInverseDC4x4ITImpl1.cpp:61-69,
 * FastInverseDC2x2ITImpl1.cpp:61-69). */
static const int DC_FWD_NA[6] = {13107, 11916, 10082, 9362, 8192, 7282};
static const int DC_INV_NA[6] = {10, 11, 13, 14, 16, 18};

/* x << s on the two's complement bits (the reference shifts negative ints). */
static int shl(int x, int s) { return (int)((unsigned)x << s); }

/* Sign-magnitude quantiser with f = 2 * (2^(15+qp/6) / 3) and shift
 * 16 + qp/6 (FastForwardDC4x4ITImpl1.cpp:78-88, 101-196). */
static short dc_quant(int x, int qp)
{
    const int qe = qp / 6, na = DC_FWD_NA[qp % 6];
    const int f = 2 * ((1 << (15 + qe)) / 3), sh = 16 + qe;
    if (x < 0) return (short)(-((((-x) * na) + f) >> sh));
    return (short)(((x * na) + f) >> sh);
}

/* FastForwardDC4x4ITImpl1::Transform(void*) (FastForwardDC4x4ITImpl1.cpp:101-196):
 * rows first (stored as short), then columns with >> 1 and, in mode 0, the
 * quantiser; mode 2 quantises only. */
static void fwd_dc4x4(short* b, int mode, int qp)
{
    if (mode == 2) {
        for (int i = 0; i < 16; i++) b[i] = dc_quant(b[i], qp);
        return;
    }
    for (int r = 0; r < 16; r += 4) {
        const int a = b[r] + b[r + 3], d = b[r] - b[r + 3];
        const int c = b[r + 1] + b[r + 2], e = b[r + 1] - b[r + 2];
        b[r] = (short)(a + c);
        b[r + 2] = (short)(a - c);
        b[r + 1] = (short)(e + d);
        b[r + 3] = (short)(d - e);
    }
    for (int k = 0; k < 4; k++) {
        const int a = b[k] + b[k + 12], d = b[k] - b[k + 12];
        const int c = b[k + 4] + b[k + 8], e = b[k + 4] - b[k + 8];
        const int y0 = (a + c) >> 1, y2 = (a - c) >> 1, y1 = (e + d) >> 1, y3 = (d - e) >> 1;
        if (mode == 0) {
            b[k] = dc_quant(y0, qp);
            b[k + 8] = dc_quant(y2, qp);
            b[k + 4] = dc_quant(y1, qp);
            b[k + 12] = dc_quant(y3, qp);
        } else {
            b[k] = (short)y0;
            b[k + 8] = (short)y2;
            b[k + 4] = (short)y1;
            b[k + 12] = (short)y3;
        }
    }
}

/* FastForwardDC2x2ITImpl1::Transform(void*) (FastForwardDC2x2ITImpl1.cpp:100-164). */
static void fwd_dc2x2(short* b, int mode, int qp)
{
    if (mode == 2) {
        for (int i = 0; i < 4; i++) b[i] = dc_quant(b[i], qp);
        return;
    }
    const int s0 = b[0] + b[1], s2 = b[0] - b[1], s1 = b[2] + b[3], s3 = b[2] - b[3];
    const int y0 = s0 + s1, y2 = s0 - s1, y1 = s2 + s3, y3 = s2 - s3;
    if (mode == 0) {
        b[0] = dc_quant(y0, qp);
        b[2] = dc_quant(y2, qp);
        b[1] = dc_quant(y1, qp);
        b[3] = dc_quant(y3, qp);
    } else {
        b[0] = (short)y0;
        b[2] = (short)y2;
        b[1] = (short)y1;
        b[3] = (short)y3;
    }
}

/* Inverse 4x4 post-scale of one coefficient x * levelScale: qp < 36 rounds
 * (x + 2^(5-qp/6)) >> (6-qp/6), else << (qp/6-6)
 * (FastInverseDC4x4ITImpl1.cpp:76-98, 111-202). */
static short dc4_scale(int x, int ls, int qp)
{
    const int qe = qp / 6;
    const int v = x * ls;
    if (qp < 36) return (short)((v + (1 << (5 - qe))) >> (6 - qe));
    return (short)shl(v, qe - 6);
}

/* FastInverseDC4x4ITImpl1::InverseTransform(void*) (FastInverseDC4x4ITImpl1.cpp:111-202):
 * columns first (stored as short), then rows with the post-scale in mode 0;
 * mode 2 post-scales only.  levelScale[pos] = NormAdjust[qp%6] * weight[pos]. */
static void inv_dc4x4(short* b, int mode, int qp, const int* weight)
{
    int ls[16];
    for (int i = 0; i < 16; i++) ls[i] = DC_INV_NA[qp % 6] * (weight ? weight[i] : 16);
    if (mode == 2) {
        for (int i = 0; i < 16; i++) b[i] = dc4_scale(b[i], ls[i], qp);
        return;
    }
    for (int k = 0; k < 4; k++) {
        const int s0 = b[k] + b[8 + k], s1 = b[k] - b[8 + k];
        const int s2 = b[4 + k] - b[12 + k], s3 = b[4 + k] + b[12 + k];
        b[k] = (short)(s0 + s3);
        b[12 + k] = (short)(s0 - s3);
        b[4 + k] = (short)(s1 + s2);
        b[8 + k] = (short)(s1 - s2);
    }
    for (int r = 0; r < 16; r += 4) {
        const int s0 = b[r] + b[2 + r], s1 = b[r] - b[2 + r];
        const int s2 = b[1 + r] - b[3 + r], s3 = b[1 + r] + b[3 + r];
        if (mode == 0) {
            const short y0 = dc4_scale(s0 + s3, ls[r], qp), y3 = dc4_scale(s0 - s3, ls[r + 3], qp);
            const short y1 = dc4_scale(s1 + s2, ls[r + 1], qp), y2 = dc4_scale(s1 - s2, ls[r + 2], qp);
            b[r] = y0;
            b[r + 1] = y1;
            b[r + 2] = y2;
            b[r + 3] = y3;
        } else {
            b[r] = (short)(s0 + s3);
            b[r + 3] = (short)(s0 - s3);
            b[r + 1] = (short)(s1 + s2);
            b[r + 2] = (short)(s1 - s2);
        }
    }
}

/* FastInverseDC2x2ITImpl1::InverseTransform(void*) (FastInverseDC2x2ITImpl1.cpp:110-157):
 * post-scale (x * levelScale << qp/6) >> 5. */
static void inv_dc2x2(short* b, int mode, int qp, const int* weight)
{
    int ls[4];
    const int qe = qp / 6;
    for (int i = 0; i < 4; i++) ls[i] = DC_INV_NA[qp % 6] * (weight ? weight[i] : 16);
    if (mode == 2) {
        for (int i = 0; i < 4; i++) b[i] = (short)(shl(b[i] * ls[i], qe) >> 5);
        return;
    }
    const int s0 = b[0] + b[1], s2 = b[0] - b[1], s1 = b[2] + b[3], s3 = b[2] - b[3];
    if (mode == 0) {
        const int x0 = (s0 + s1) * ls[0], x2 = (s0 - s1) * ls[2];
        const int x1 = (s2 + s3) * ls[1], x3 = (s2 - s3) * ls[3];
        b[0] = (short)(shl(x0, qe) >> 5);
        b[1] = (short)(shl(x1, qe) >> 5);
        b[2] = (short)(shl(x2, qe) >> 5);
        b[3] = (short)(shl(x3, qe) >> 5);
    } else {
        b[0] = (short)(s0 + s1);
        b[2] = (short)(s0 - s1);
        b[1] = (short)(s2 + s3);
        b[3] = (short)(s2 - s3);
    }
}

void vo_fwd_dc(short* data, int nunits, int size, int mode, int qp)
{
    const int unit = size * size;
    for (int u = 0; u < nunits; u++) {
        if (size == 4) fwd_dc4x4(data + (size_t)u * unit, mode, qp);
        else fwd_dc2x2(data + (size_t)u * unit, mode, qp);
    }
}

void vo_inv_dc(short* data, int nunits, int size, int mode, int qp, const int* weight)
{
    const int unit = size * size;
    for (int u = 0; u < nunits; u++) {
        if (size == 4) inv_dc4x4(data + (size_t)u * unit, mode, qp, weight);
        else inv_dc2x2(data + (size_t)u * unit, mode, qp, weight);
    }
}

/* FastForwardDC4x4ITImpl1::QuantiseValue (FastForwardDC4x4ITImpl1.cpp:268-283). */
int vo_dc_quantise_value(short val, int qp) { return dc_quant(val, qp); }
