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
 *
 * The 6-bit converters (6-bit samples, scaled to 8 bits on the way):
 *   kind 3  Fast6BitYUV420toRGB24Converter
 *           (src/ImageUtils/Fast6BitYUV420toRGB24Converter.cpp:47-245):
 *           integers, lum = Y << 2, cc = (u << 3) + (u >> 3) - 260,
 *           cb = -u - (u >> 1) - (u >> 4) - (v << 1) - (v >> 2) - (v >> 4) + 124,
 *           ca = (v << 2) + (v >> 1) + (v >> 4) - 146 on the raw samples;
 *           rotate ? RotateConvert : NonRotateConvert.
 *   kind 4  Real6BitYUV420toRGB24Converter
 *           (src/ImageUtils/Real6BitYUV420toRGB24Converter.cpp:53-246): the
 *           Real arithmetic on lum = Y << 2, u = (U << 2) - 128,
 *           v = (V << 2) - 128; rotate ? RotateConvert : NonRotateConvert.
 * vo_yuv420_to_rgb24_zoom: Fast6BitYUV420toRGB24ZoomConverter
 * (src/ImageUtils/Fast6BitYUV420toRGB24ZoomConverter.cpp:48-230).
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

/* kinds 3 and 4: one 2x2 block of the 6-bit converters */
void vo_yuv420_to_rgb24_6bit(int kind, const short* py, const short* pu, const short* pv, int w, int h, int rotate,
                             unsigned char* rgb)
{
    for (int y = 0; y < h; y += 2) {
        for (int x = 0; x < w; x += 2) {
            const int c = (y >> 1) * (w >> 1) + (x >> 1);
            const int su = pu[c], sv = pv[c];
            int cc = 0, cb = 0, ca = 0;
            double dc = 0.0, db = 0.0, da = 0.0;
            if (kind == 3) {
                cc = (su << 3) + (su >> 3) - 260;
                cb = -su - (su >> 1) - (su >> 4) - (sv << 1) - (sv >> 2) - (sv >> 4) + 124;
                ca = (sv << 2) + (sv >> 1) + (sv >> 4) - 146;
            } else {
                const double u = (double)((su << 2) - 128), v = (double)((sv << 2) - 128);
                dc = (2.032 * u) + 0.5;
                db = (-0.394 * u) + (-0.581 * v) + 0.5;
                da = (1.140 * v) + 0.5;
            }
            for (int dy = 0; dy < 2; dy++)
                for (int dx = 0; dx < 2; dx++) {
                    const int px = x + dx, pyy = y + dy;
                    const int l = py[(size_t)pyy * w + px] << 2;
                    const size_t o = rotate ? ((size_t)px * h + pyy) * 3 : ((size_t)pyy * w + px) * 3;
                    if (kind == 3) {
                        rgb[o] = clip_u8(l + cc);
                        rgb[o + 1] = clip_u8(l + cb);
                        rgb[o + 2] = clip_u8(l + ca);
                    } else {
                        const double lum = (double)l;
                        rgb[o] = clip_u8((int)(lum + dc));
                        rgb[o + 1] = clip_u8((int)(lum + db));
                        rgb[o + 2] = clip_u8((int)(lum + da));
                    }
                }
        }
    }
}

/* Fast6BitYUV420toRGB24ZoomConverter::NonRotateConvert: output pixel (x, y)
 * reads source position ((int)(scale * x + 0.5), (int)(scale * y + 0.5)) in
 * double, weights its 3x3 neighbourhood (edge-clamped) plus 7 more of the
 * centre (16 in all, then >> 2: /16 and 6 -> 8 bits); the chroma of each
 * 2x2 output block is the same weighting at the block's first luma position
 * halved, with the shift-based terms of the reference ("divide by 16 built
 * in").  Output sizes must be even (the reference writes rows and columns in
 * pairs) and the centres in range (its centre reads are unclamped):
 * returns -1 otherwise. */
int vo_yuv420_to_rgb24_zoom(const short* py, const short* pu, const short* pv, int w, int h, int ow, int oh,
                            unsigned char* rgb)
{
    if (ow < 2 || oh < 2 || (ow & 1) || (oh & 1)) return -1;
    const double sx = (double)w / (double)ow, sy = (double)h / (double)oh;
    const int cw = w >> 1, chh = h >> 1;
    if ((int)((sx * (double)(ow - 1)) + 0.5) >= w || (int)((sy * (double)(oh - 1)) + 0.5) >= h) return -1;
    for (int y = 0; y < oh; y += 2) {
        const int ly0 = (int)((sy * (double)y) + 0.5), ly1 = (int)((sy * (double)(y + 1)) + 0.5);
        const int uy = ly0 >> 1;
        for (int x = 0; x < ow; x += 2) {
            const int lx0 = (int)((sx * (double)x) + 0.5), lx1 = (int)((sx * (double)(x + 1)) + 0.5);
            const int ux = lx0 >> 1;
            int u = 7 * pu[uy * cw + ux], v = 7 * pv[uy * cw + ux];
            for (int i = -1; i <= 1; i++) {
                int r = uy + i;
                r = r < 0 ? 0 : (r >= chh ? chh - 1 : r);
                for (int j = -1; j <= 1; j++) {
                    int c = ux + j;
                    c = c < 0 ? 0 : (c >= cw ? cw - 1 : c);
                    u += pu[r * cw + c];
                    v += pv[r * cw + c];
                }
            }
            const int cc = (u >> 1) - 256;
            const int cb = -(u >> 3) + (u >> 5) - (v >> 3) - (v >> 6) + 120;
            const int ca = (v >> 2) + (v >> 5) - 144;
            for (int dy = 0; dy < 2; dy++)
                for (int dx = 0; dx < 2; dx++) {
                    const int ly = dy ? ly1 : ly0, lx = dx ? lx1 : lx0;
                    int l = 7 * py[ly * w + lx];
                    for (int i = -1; i <= 1; i++) {
                        int r = ly + i;
                        r = r < 0 ? 0 : (r >= h ? h - 1 : r);
                        for (int j = -1; j <= 1; j++) {
                            int c = lx + j;
                            c = c < 0 ? 0 : (c >= w ? w - 1 : c);
                            l += py[r * w + c];
                        }
                    }
                    l >>= 2;
                    const size_t o = ((size_t)(y + dy) * ow + (x + dx)) * 3;
                    rgb[o] = clip_u8(l + cc);
                    rgb[o + 1] = clip_u8(l + cb);
                    rgb[o + 2] = clip_u8(l + ca);
                }
        }
    }
    return 0;
}
