/*
 * oracle_colour.c -- TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * Restatement of the packed BGR24 -> planar YUV 4:2:0 converters:
 *   kind 0: FastFixedPointRGB24toYUV420Converter::Convert
 *           (src/ImageUtils/FastFixedPointRGB24toYUV420Converter.cpp:94-169)
 *   kind 1: RealRGB24toYUV420Converter::{NonFlip,Flip}Convert
 *           (src/ImageUtils/RealRGB24toYUV420Converter.cpp:83-242)
 *   kind 2: RealRGB24toYUV420ConverterImpl2 (src/ImageUtils/RealRGB24toYUV420ConverterImpl2.cpp:104-262)
 * The double variants must be built without FMA contraction.
 */
#include "oracle_internal.h"

/* BT.601-style analysis matrix used by all three converters. */
#define K00 0.299
#define K01 0.587
#define K02 0.114
#define K10 -0.147
#define K11 -0.289
#define K12 0.436
#define K20 0.615
#define K21 -0.515
#define K22 -0.100

static inline int clamp_u8(int x) { return x < 0 ? 0 : (x > 255 ? 255 : x); }
static inline int clamp_s8(int x) { return x < -128 ? -128 : (x > 127 ? 127 : x); }

/* Fixed-point coefficients: (int)(0.5 + c * (2 << 12)), truncation toward zero
 * for negative c exactly as the static_cast in the reference (…FixedPoint….cpp:65-74). */
static int fx_coef(double c) { return (int)(0.5 + c * (double)(2 << 12)); }

static void convert_fixed(const unsigned char* src, int w, int h, int chr_off, short* py, short* pu, short* pv)
{
    const int c00 = fx_coef(K00), c01 = fx_coef(K01), c02 = fx_coef(K02);
    const int c10 = fx_coef(K10), c11 = fx_coef(K11), c12 = fx_coef(K12);
    const int c20 = fx_coef(K20), c21 = fx_coef(K21), c22 = fx_coef(K22);
    const int sh = 13;
    int xb_n = w >> 1, yb_n = h >> 1;
    for (int yb = 0; yb < yb_n; yb++)
        for (int xb = 0; xb < xb_n; xb++) {
            int u = 0, v = 0;
            for (int k = 0; k < 4; k++) {
                int yy = 2 * yb + (k >> 1), xx = 2 * xb + (k & 1);
                const unsigned char* t = src + ((size_t)yy * w + xx) * 3;
                int b = t[0], g = t[1], r = t[2];
                py[(size_t)yy * w + xx] = (short)clamp_u8((c00 * r + c01 * g + c02 * b) >> sh);
                u += c10 * r + c11 * g + c12 * b;
                v += c20 * r + c21 * g + c22 * b;
            }
            int iu = u >> sh, iv = v >> sh;
            iu += (iu < 0) ? -2 : 2;
            iv += (iv < 0) ? -2 : 2;
            size_t co = (size_t)yb * xb_n + xb;
            pu[co] = (short)(chr_off + clamp_s8(iu >> 2));
            pv[co] = (short)(chr_off + clamp_s8(iv >> 2));
        }
}

/* Real converters.  Luma: (int)(0.5 + k0*r + k1*g + k2*b) evaluated left to
 * right.  Chroma: the per-pixel sums k0*r + k1*g + k2*b accumulated over the
 * 2x2 block in raster order, then rounded per variant. */
static void convert_real(const unsigned char* src, int w, int h, int chr_off, int flip, int impl2,
                         short* py, short* pu, short* pv)
{
    int xb_n = w >> 1, yb_n = h >> 1;
    for (int yb = 0; yb < yb_n; yb++)
        for (int xb = 0; xb < xb_n; xb++) {
            double u = 0.0, v = 0.0;
            for (int k = 0; k < 4; k++) {
                int dy = k >> 1, xx = 2 * xb + (k & 1);
                int yy = 2 * yb + dy;
                int sy = flip ? (h - 1 - yy) : yy;
                const unsigned char* t = src + ((size_t)sy * w + xx) * 3;
                double b = (double)t[0], g = (double)t[1], r = (double)t[2];
                py[(size_t)yy * w + xx] = (short)clamp_u8((int)(0.5 + K00 * r + K01 * g + K02 * b));
                double uu = K10 * r + K11 * g + K12 * b;
                double vv = K20 * r + K21 * g + K22 * b;
                if (k == 0) { u = uu; v = vv; }
                else { u += uu; v += vv; }
            }
            int iu, iv;
            if (!impl2) {
                /* (int) truncation, +-2, then /4 truncating (RealRGB24…Converter.cpp:226-239). */
                iu = (int)u;
                iv = (int)v;
                iu += (iu < 0) ? -2 : 2;
                iv += (iv < 0) ? -2 : 2;
                iu = iu / 4;
                iv = iv / 4;
            } else {
                /* Average first, then +-0.5 and truncate (…ConverterImpl2.cpp). */
                double au = u / 4.0, av = v / 4.0;
                iu = (int)(au < 0.0 ? au - 0.5 : au + 0.5);
                iv = (int)(av < 0.0 ? av - 0.5 : av + 0.5);
            }
            size_t co = (size_t)yb * xb_n + xb;
            pu[co] = (short)(chr_off + clamp_s8(iu));
            pv[co] = (short)(chr_off + clamp_s8(iv));
        }
}

int vo_rgb24_to_yuv420(int kind, const unsigned char* bgr, int w, int h, int chr_off, int flip,
                       short* y, short* u, short* v)
{
    if (!bgr || !y || !u || !v || w < 2 || h < 2) return -1;
    if (kind == 0) convert_fixed(bgr, w, h, chr_off, y, u, v);
    else if (kind == 1) convert_real(bgr, w, h, chr_off, flip, 0, y, u, v);
    else if (kind == 2) convert_real(bgr, w, h, chr_off, flip, 1, y, u, v);
    else return -1;
    return 0;
}
