/*
 * oracle_yuv2rgb.c -- TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * Restatement of the floating-point planar YUV 4:2:0 (short planes) ->
 * packed B,G,R byte converters:
 *   kind 0  RealYUV420toRGB24Converter
 *           (src/ImageUtils/RealYUV420toRGB24Converter.cpp:66-352):
 *           Convert = flip ? InvertConvert : rotate ? RotateConvert : NonRotateConvert
 *           (include/ImageUtils/RealYUV420toRGB24Converter.h:58-68).
 *           InvertConvert and NonRotateConvert take the luma as an unsigned
 *           char and u, v as signed chars of (sample + chrOff);
 *           RotateConvert takes them as (double)sample and sample - 128.
 *   kind 1  RealYUV420toRGB24ConverterImpl2 and ...Impl2Ver16
 *           (RealYUV420toRGB24ConverterImpl2.cpp:94-368): Convert = flip ?
 *           FlipConvert : rotate ? RotateConvert : NonRotateConvert, luma as
 *           is, u, v = sample - 128 on every path.
 *   kind 2  RealYUV420toRGB24CCIR601Converter and ...Ver16
 *           (RealYUV420toRGB24CCIR601Converter.cpp:59-241): rotate ?
 *           RotateConvert : NonRotateConvert (no flip), luma - 16, u, v - 128,
 *           U0 = 2.033.
 * Every pixel: b = (int)(lum + (U0*u + 0.5)), g = (int)(lum + (U1*u + V1*v
 * + 0.5)), r = (int)(lum + (V0*v + 0.5)) in double, evaluated left to right
 * (the Makefile builds with -ffp-contract=off), clipped to 0..255.  Output
 * layouts: rows top-down (NonRotate), bottom-up (Invert / Flip), or the
 * transpose (Rotate: pixel (x, y) at byte 3 * (x * height + y)).
 */
#include "oracle_internal.h"

static unsigned char clip_u8(int x) { return (unsigned char)(x > 255 ? 255 : (x < 0 ? 0 : x)); }

void vo_yuv420_to_rgb24(int kind, const short* py, const short* pu, const short* pv, int w, int h, int chr_off,
                        int rotate, int flip, unsigned char* rgb)
{
    const double U0 = kind == 2 ? 2.033 : 2.032, U1 = -0.394, V1 = -0.581, V0 = 1.140;
    /* 0 top-down, 1 transpose, 2 bottom-up */
    const int layout = (kind != 2 && flip) ? 2 : (rotate ? 1 : 0);
    const int byte_casts = kind == 0 && layout != 1;  /* Real: Invert / NonRotate */
    for (int y = 0; y < h; y += 2) {
        for (int x = 0; x < w; x += 2) {
            const int c = (y >> 1) * (w >> 1) + (x >> 1);
            double u, v;
            if (byte_casts) {
                u = (double)(signed char)(int)((double)pu[c] + chr_off);
                v = (double)(signed char)(int)((double)pv[c] + chr_off);
            } else {
                u = (double)(pu[c] - 128);
                v = (double)(pv[c] - 128);
            }
            const double cc = (U0 * u) + 0.5;
            const double cb = (U1 * u) + (V1 * v) + 0.5;
            const double ca = (V0 * v) + 0.5;
            for (int dy = 0; dy < 2; dy++)
                for (int dx = 0; dx < 2; dx++) {
                    const int px = x + dx, pyy = y + dy;
                    const int s = py[(size_t)pyy * w + px];
                    double lum;
                    if (byte_casts) lum = (double)(unsigned char)s;
                    else lum = (double)(kind == 2 ? s - 16 : s);
                    size_t o;
                    if (layout == 1) o = ((size_t)px * h + pyy) * 3;
                    else if (layout == 2) o = ((size_t)(h - 1 - pyy) * w + px) * 3;
                    else o = ((size_t)pyy * w + px) * 3;
                    rgb[o] = clip_u8((int)(lum + cc));
                    rgb[o + 1] = clip_u8((int)(lum + cb));
                    rgb[o + 2] = clip_u8((int)(lum + ca));
                }
        }
    }
}
