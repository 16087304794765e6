// yuv2rgb.cu -- planar YUV 4:2:0 (short planes) -> packed B,G,R bytes for
// sm_103a, bit-exact with the reference's double-precision converters:
//
//   kind 0  RealYUV420toRGB24Converter (src/ImageUtils/RealYUV420toRGB24Converter.cpp:66-352)
//   kind 1  RealYUV420toRGB24ConverterImpl2 / ...Impl2Ver16 (RealYUV420toRGB24ConverterImpl2.cpp:94-368)
//   kind 2  RealYUV420toRGB24CCIR601Converter / ...Ver16 (RealYUV420toRGB24CCIR601Converter.cpp:59-241)
//   kind 3  Fast6BitYUV420toRGB24Converter (src/ImageUtils/Fast6BitYUV420toRGB24Converter.cpp:47-245):
//           6-bit samples, integer shift-and-add terms
//   kind 4  Real6BitYUV420toRGB24Converter (src/ImageUtils/Real6BitYUV420toRGB24Converter.cpp:53-246):
//           the kind 0 double terms on 6-bit samples scaled by 4
//   zoom    Fast6BitYUV420toRGB24ZoomConverter (src/ImageUtils/Fast6BitYUV420toRGB24ZoomConverter.cpp:48-230)
//
// Each pixel is b = (int)(lum + (U0*u + 0.5)), g = (int)(lum + (U1*u + V1*v
// + 0.5)), r = (int)(lum + (V0*v + 0.5)) in double, clipped to 0..255, with
// U0 = 2.032 (2.033 for CCIR601), U1 = -0.394, V1 = -0.581, V0 = 1.140.
//
// GB300 design: the exact value of every term is a rational in thousandths,
// N / 1000 with N = 1000 * coefficient * u + ... + 500.  Where N is not a
// multiple of 1000 its fractional part is at least 0.001 from an integer,
// far beyond the double rounding error (< 1e-10 for any short input), so
// (int)(lum + term) clipped is clip(lum + floor(N / 1000)) in integers.
// Where N is a multiple of 1000 (no u for b with U0 = 2.032, six v values of
// 0..255 for r, about one (u, v) pair in a thousand for g) the double term
// is evaluated once per 2x2 block in IEEE double, operation by operation as
// the reference does (__dmul_rn / __dadd_rn, no contraction), and how far it
// falls below the integer decides, per pixel in integers, whether the
// reference's sum truncates one lower.  The kernel stays HBM-bound: 3 B read
// (luma and quarter-size chroma as int16) and 3 B written per pixel.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "vppgpu_internal.cuh"

namespace {

struct YuvParams {
    int w, h;
    int six_bit;     // Real6Bit: samples scaled by 4 (luma << 2, chroma << 2 then - 128)
    int byte_casts;  // Real Invert / NonRotate: luma as unsigned char, chroma as signed char of (sample + chr_off)
    int chr_off;
    int luma_off;    // 16 for CCIR601
    int a0;          // U0 in thousandths
    double U0;
    // below_limit of the b term for u = -128..127 and of the r term for v = -128..127
    int lim_b[256], lim_r[256];
};

// floor(n / 1000) and whether 1000 divides n, for |n| < 2^27 (every term of
// short inputs: |2033 u| + |581 v| + 500 < 9e7): one unsigned division of
// the biased numerator by a constant.
__device__ __forceinline__ int floordiv1000(int n, bool& exact)
{
    constexpr int kBias = 1 << 17;  // multiples of 1000 added: n + 1000 * kBias > 0
    const unsigned b = (unsigned)(n + 1000 * kBias);
    const unsigned q = b / 1000u;
    exact = b - q * 1000u == 0u;
    return (int)q - kBias;
}

// Where the exact term is an integer m, the double term c may lie just
// below it: c = m - d.  Then (int)(lum + c) is K = lum + m when the double
// nearest to K - d is K, else K - 1 (for K >= 1; K <= 0 clips to 0 either
// way).  The double just below an integer K >= 1 is 2^(floor(log2(K-1)) - 52)
// away, and ties round to K (its significand is even), so the result is
// K - 1 exactly for 1 <= K <= 2^t with t = ceil(log2 d) + 53.  Returns that
// bound 2^t (0 when c >= m: the result is K).  d = m - c is exact
// (Sterbenz), and normal.
__device__ __forceinline__ int below_limit(double c, int m)
{
    const double d = __dsub_rn((double)m, c);
    if (!(d > 0.0)) return 0;
    const long long bits = __double_as_longlong(d);
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;
    const int t = ((bits & 0xfffffffffffffLL) ? e + 1 : e) + 53;
    return t >= 31 ? 0x7fffffff : (t < 0 ? 0 : (1 << t));
}

// The three terms of one 2x2 block: floor(N / 1000), and for the terms whose
// exact value is an integer the bound of below_limit (FP64 once per block,
// in the reference's operation order).
struct Terms {
    int qb, qg, qr;
    int lb, lg, lr;
};

__device__ __forceinline__ Terms block_terms(int su, int sv, const YuvParams& p)
{
    if (p.six_bit) {  // (s << 2) - 128 is the plain path's s - 128 of 4s
        su *= 4;
        sv *= 4;
    }
    int u, v;
    if (p.byte_casts) {
        u = (signed char)(su + p.chr_off);
        v = (signed char)(sv + p.chr_off);
    } else {
        u = su - 128;
        v = sv - 128;
    }
    const int nb = p.a0 * u + 500, ng = -394 * u - 581 * v + 500, nr = 1140 * v + 500;
    Terms t;
    bool xb, xg, xr;
    t.qb = floordiv1000(nb, xb);
    t.qg = floordiv1000(ng, xg);
    t.qr = floordiv1000(nr, xr);
    t.lb = t.lg = t.lr = 0;
    if (xb)
        t.lb = (unsigned)(u + 128) < 256u ? p.lim_b[u + 128]
                                          : below_limit(__dadd_rn(__dmul_rn(p.U0, (double)u), 0.5), t.qb);
    if (xg)
        t.lg = below_limit(__dadd_rn(__dadd_rn(__dmul_rn(-0.394, (double)u), __dmul_rn(-0.581, (double)v)), 0.5),
                           t.qg);
    if (xr)
        t.lr = (unsigned)(v + 128) < 256u ? p.lim_r[v + 128]
                                          : below_limit(__dadd_rn(__dmul_rn(1.140, (double)v), 0.5), t.qr);
    return t;
}

__device__ __forceinline__ int luma(int s, const YuvParams& p)
{
    return p.byte_casts ? (int)(unsigned char)s : (p.six_bit ? 4 * s : s - p.luma_off);
}

__device__ __forceinline__ int chan(int l, int q, int lim)
{
    const int k = l + q;
    return clip255(k - ((unsigned)(k - 1) < (unsigned)lim ? 1 : 0));  // 1 <= k <= lim
}

// b, g, r of one pixel packed in the low 24 bits; kExact: some term of the
// block needs below_limit's correction
template <bool kExact = true>
__device__ __forceinline__ unsigned pixel(int s, const Terms& t, const YuvParams& p)
{
    const int l = luma(s, p);
    if constexpr (!kExact)
        return (unsigned)clip255(l + t.qb) | ((unsigned)clip255(l + t.qg) << 8) | ((unsigned)clip255(l + t.qr) << 16);
    return (unsigned)chan(l, t.qb, t.lb) | ((unsigned)chan(l, t.qg, t.lg) << 8) | ((unsigned)chan(l, t.qr, t.lr) << 16);
}

// Rows layout (NonRotate, or bottom-up with kFlip), four 2x2 blocks per
// thread: two 16-byte luma loads, 8-byte chroma loads, three 8-byte stores
// per output row.  Needs width % 8 == 0 and aligned planes.
template <bool kFlip>
__global__ void __launch_bounds__(256) k_yuv_rgb_x8(const short* __restrict__ Y, const short* __restrict__ U,
                                                    const short* __restrict__ V, YuvParams p,
                                                    unsigned char* __restrict__ rgb)
{
    const int f = blockIdx.y;
    const int gpr = p.w >> 3, groups = gpr * (p.h >> 1);
    const short* y0 = Y + (size_t)f * p.w * p.h;
    const short* u0 = U + (size_t)f * (p.w >> 1) * (p.h >> 1);
    const short* v0 = V + (size_t)f * (p.w >> 1) * (p.h >> 1);
    unsigned char* o0 = rgb + (size_t)f * p.w * p.h * 3;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < groups; g += gridDim.x * blockDim.x) {
        const int qy = g / gpr, gx = g - qy * gpr, x = gx * 8, y = 2 * qy;
        const uint4 ya = __ldg(reinterpret_cast<const uint4*>(y0 + (size_t)y * p.w + x));
        const uint4 yb = __ldg(reinterpret_cast<const uint4*>(y0 + (size_t)(y + 1) * p.w + x));
        const uint2 uu = __ldg(reinterpret_cast<const uint2*>(u0 + (size_t)qy * (p.w >> 1) + 4 * gx));
        const uint2 vv = __ldg(reinterpret_cast<const uint2*>(v0 + (size_t)qy * (p.w >> 1) + 4 * gx));
        const short* sa = reinterpret_cast<const short*>(&ya);
        const short* sb = reinterpret_cast<const short*>(&yb);
        const short* su = reinterpret_cast<const short*>(&uu);
        const short* sv = reinterpret_cast<const short*>(&vv);
        unsigned ra[8], rb[8];
        Terms tk[4];
        int lims = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            tk[k] = block_terms(su[k], sv[k], p);
            lims |= tk[k].lb | tk[k].lg | tk[k].lr;
        }
        if (__any_sync(__activemask(), lims != 0)) {  // a block of the warp needs the correction
#pragma unroll
            for (int k = 0; k < 4; k++) {
                ra[2 * k] = pixel<true>(sa[2 * k], tk[k], p);
                ra[2 * k + 1] = pixel<true>(sa[2 * k + 1], tk[k], p);
                rb[2 * k] = pixel<true>(sb[2 * k], tk[k], p);
                rb[2 * k + 1] = pixel<true>(sb[2 * k + 1], tk[k], p);
            }
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                ra[2 * k] = pixel<false>(sa[2 * k], tk[k], p);
                ra[2 * k + 1] = pixel<false>(sa[2 * k + 1], tk[k], p);
                rb[2 * k] = pixel<false>(sb[2 * k], tk[k], p);
                rb[2 * k + 1] = pixel<false>(sb[2 * k + 1], tk[k], p);
            }
        }
        // 8 pixels x 3 bytes = six little-endian words per row
        auto pack = [](const unsigned* q, unsigned* w) {
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const unsigned a = q[4 * i], b = q[4 * i + 1], c = q[4 * i + 2], d = q[4 * i + 3];
                w[3 * i] = a | (b << 24);
                w[3 * i + 1] = (b >> 8) | (c << 16);
                w[3 * i + 2] = (c >> 16) | (d << 8);
            }
        };
        unsigned wa[6], wb[6];
        pack(ra, wa);
        pack(rb, wb);
        const int ya_out = kFlip ? p.h - 1 - y : y, yb_out = kFlip ? p.h - 2 - y : y + 1;
        uint2* da = reinterpret_cast<uint2*>(o0 + ((size_t)ya_out * p.w + x) * 3);
        uint2* db = reinterpret_cast<uint2*>(o0 + ((size_t)yb_out * p.w + x) * 3);
#pragma unroll
        for (int i = 0; i < 3; i++) {
            da[i] = make_uint2(wa[2 * i], wa[2 * i + 1]);
            db[i] = make_uint2(wb[2 * i], wb[2 * i + 1]);
        }
    }
}

// Any even width, any layout: one 2x2 block per thread, byte stores.
// layout 0 rows top-down, 1 transpose (pixel (x, y) at 3 * (x * h + y);
// consecutive threads walk down a column so the stores stay contiguous),
// 2 rows bottom-up.
__global__ void __launch_bounds__(256) k_yuv_rgb(const short* __restrict__ Y, const short* __restrict__ U,
                                                 const short* __restrict__ V, YuvParams p, int layout,
                                                 unsigned char* __restrict__ rgb)
{
    const int f = blockIdx.y;
    const int cw = p.w >> 1, ch = p.h >> 1, blocks = cw * ch;
    const short* y0 = Y + (size_t)f * p.w * p.h;
    const short* u0 = U + (size_t)f * cw * ch;
    const short* v0 = V + (size_t)f * cw * ch;
    unsigned char* o0 = rgb + (size_t)f * p.w * p.h * 3;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < blocks; k += gridDim.x * blockDim.x) {
        int qx, qy;
        if (layout == 1) {
            qx = k / ch;
            qy = k - qx * ch;
        } else {
            qy = k / cw;
            qx = k - qy * cw;
        }
        const int c = qy * cw + qx;
        const Terms t = block_terms(__ldg(u0 + c), __ldg(v0 + c), p);
#pragma unroll
        for (int dy = 0; dy < 2; dy++)
#pragma unroll
            for (int dx = 0; dx < 2; dx++) {
                const int px = 2 * qx + dx, py = 2 * qy + dy;
                const unsigned q = pixel(__ldg(y0 + (size_t)py * p.w + px), t, p);
                size_t o;
                if (layout == 1) o = ((size_t)px * p.h + py) * 3;
                else if (layout == 2) o = ((size_t)(p.h - 1 - py) * p.w + px) * 3;
                else o = ((size_t)py * p.w + px) * 3;
                o0[o] = (unsigned char)q;
                o0[o + 1] = (unsigned char)(q >> 8);
                o0[o + 2] = (unsigned char)(q >> 16);
            }
    }
}

// Real6Bit for samples beyond +-16000 (where the thousandths of a term no
// longer fit floordiv1000's range): the reference's double arithmetic per
// pixel, operation by operation.
__device__ __forceinline__ unsigned pixel_real6_fp64(int s, int su, int sv)
{
    const double u = (double)(4 * su - 128), v = (double)(4 * sv - 128), lum = (double)(4 * s);
    const double cc = __dadd_rn(__dmul_rn(2.032, u), 0.5);
    const double cb = __dadd_rn(__dadd_rn(__dmul_rn(-0.394, u), __dmul_rn(-0.581, v)), 0.5);
    const double ca = __dadd_rn(__dmul_rn(1.140, v), 0.5);
    return (unsigned)clip255(__double2int_rz(__dadd_rn(lum, cc))) |
           ((unsigned)clip255(__double2int_rz(__dadd_rn(lum, cb))) << 8) |
           ((unsigned)clip255(__double2int_rz(__dadd_rn(lum, ca))) << 16);
}

// The 6-bit converters, one 2x2 block per thread, rows (layout 0) or the
// transpose (layout 1: pixel (x, y) at 3 * (x * h + y)).  kReal: kind 4
// through the exact-integer terms (block_terms with six_bit), else kind 3's
// integer terms on the raw samples (arithmetic shifts, as the reference's
// int shifts on gcc).
template <bool kReal>
__global__ void __launch_bounds__(256) k_yuv_rgb_6bit(const short* __restrict__ Y, const short* __restrict__ U,
                                                      const short* __restrict__ V, YuvParams p, int layout,
                                                      unsigned char* __restrict__ rgb)
{
    const int f = blockIdx.y;
    const int cw = p.w >> 1, ch = p.h >> 1, blocks = cw * ch;
    const short* y0 = Y + (size_t)f * p.w * p.h;
    const short* u0 = U + (size_t)f * cw * ch;
    const short* v0 = V + (size_t)f * cw * ch;
    unsigned char* o0 = rgb + (size_t)f * p.w * p.h * 3;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < blocks; k += gridDim.x * blockDim.x) {
        int qx, qy;
        if (layout == 1) {
            qx = k / ch;
            qy = k - qx * ch;
        } else {
            qy = k / cw;
            qx = k - qy * cw;
        }
        const int c = qy * cw + qx;
        const int su = __ldg(u0 + c), sv = __ldg(v0 + c);
        const bool big = kReal && (su < -16000 || su > 16000 || sv < -16000 || sv > 16000);
        Terms t{};
        int cc = 0, cb = 0, ca = 0;
        if (kReal) {
            if (!big) t = block_terms(su, sv, p);
        } else {
            cc = (su << 3) + (su >> 3) - 260;
            cb = -su - (su >> 1) - (su >> 4) - (sv << 1) - (sv >> 2) - (sv >> 4) + 124;
            ca = (sv << 2) + (sv >> 1) + (sv >> 4) - 146;
        }
#pragma unroll
        for (int dy = 0; dy < 2; dy++)
#pragma unroll
            for (int dx = 0; dx < 2; dx++) {
                const int px = 2 * qx + dx, py = 2 * qy + dy;
                const int s = __ldg(y0 + (size_t)py * p.w + px);
                unsigned q;
                if (!kReal) {
                    const int l = s << 2;
                    q = (unsigned)clip255(l + cc) | ((unsigned)clip255(l + cb) << 8) | ((unsigned)clip255(l + ca) << 16);
                } else {
                    q = big ? pixel_real6_fp64(s, su, sv) : pixel(s, t, p);
                }
                const size_t o = layout == 1 ? ((size_t)px * p.h + py) * 3 : ((size_t)py * p.w + px) * 3;
                o0[o] = (unsigned char)q;
                o0[o + 1] = (unsigned char)(q >> 8);
                o0[o + 2] = (unsigned char)(q >> 16);
            }
    }
}

// Fast6BitYUV420toRGB24ZoomConverter, one 2x2 output block per thread: the
// source positions (int)(scale * x + 0.5) in IEEE double, each output luma
// 7 x its centre plus its edge-clamped 3x3 neighbourhood, >> 2 (/16 and 6 ->
// 8 bits); the block's chroma the same weighting at the first position
// halved, with the reference's shift terms.  The host has checked that the
// centres stay inside the planes.
struct ZoomParams {
    int w, h, ow, oh;
    double sx, sy;  // w / ow, h / oh
};

__device__ __forceinline__ int zoom_pos(double scale, int i)
{
    return __double2int_rz(__dadd_rn(__dmul_rn(scale, (double)i), 0.5));
}

__device__ __forceinline__ int weighted16(const short* __restrict__ pl, int w, int h, int cx, int cy)
{
    int acc = 7 * (int)__ldg(pl + (size_t)cy * w + cx);
#pragma unroll
    for (int i = -1; i <= 1; i++) {
        const int r = min(max(cy + i, 0), h - 1);
#pragma unroll
        for (int j = -1; j <= 1; j++) acc += __ldg(pl + (size_t)r * w + min(max(cx + j, 0), w - 1));
    }
    return acc;
}

__global__ void __launch_bounds__(256) k_yuv_rgb_zoom(const short* __restrict__ Y, const short* __restrict__ U,
                                                      const short* __restrict__ V, ZoomParams z,
                                                      unsigned char* __restrict__ rgb)
{
    const int bw = z.ow >> 1, blocks = bw * (z.oh >> 1);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < blocks; k += gridDim.x * blockDim.x) {
        const int by = k / bw, x = 2 * (k - by * bw), y = 2 * by;
        const int ly[2] = {zoom_pos(z.sy, y), zoom_pos(z.sy, y + 1)};
        const int lx[2] = {zoom_pos(z.sx, x), zoom_pos(z.sx, x + 1)};
        const int u = weighted16(U, z.w >> 1, z.h >> 1, lx[0] >> 1, ly[0] >> 1);
        const int v = weighted16(V, z.w >> 1, z.h >> 1, lx[0] >> 1, ly[0] >> 1);
        const int cc = (u >> 1) - 256;
        const int cb = -(u >> 3) + (u >> 5) - (v >> 3) - (v >> 6) + 120;
        const int ca = (v >> 2) + (v >> 5) - 144;
#pragma unroll
        for (int dy = 0; dy < 2; dy++)
#pragma unroll
            for (int dx = 0; dx < 2; dx++) {
                const int l = weighted16(Y, z.w, z.h, lx[dx], ly[dy]) >> 2;
                unsigned char* o = rgb + ((size_t)(y + dy) * z.ow + x + dx) * 3;
                o[0] = (unsigned char)clip255(l + cc);
                o[1] = (unsigned char)clip255(l + cb);
                o[2] = (unsigned char)clip255(l + ca);
            }
    }
}

// below_limit on the host for the tabulated terms: the same IEEE double
// operations (volatile intermediates: no multiply-add contraction).
int host_below_limit(double coef, int x)
{
    volatile double prod = coef * (double)x;
    volatile double c = prod + 0.5;
    const long long n = (long long)llround(coef * 1000.0) * x + 500;  // the exact term in thousandths
    if (n % 1000) return 0;  // not an integer: the kernel never reads the entry
    const int m = (int)(n / 1000);
    volatile double d = (double)m - c;
    if (!(d > 0.0)) return 0;
    long long bits;
    const double dd = d;
    memcpy(&bits, &dd, sizeof bits);
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;
    const int t = ((bits & 0xfffffffffffffLL) ? e + 1 : e) + 53;
    return t >= 31 ? 0x7fffffff : (t < 0 ? 0 : (1 << t));
}

int check(vppgpu_ctx* ctx, int kind, const void* y, const void* u, const void* v, int w, int h, const void* rgb)
{
    if (!ctx || !y || !u || !v || !rgb || w < 2 || h < 2 || (w & 1) || (h & 1)) return VPPGPU_ERR_INVALID_ARG;
    if (kind < VPPGPU_YUV_REAL || kind > VPPGPU_YUV_REAL_6BIT) return VPPGPU_ERR_INVALID_ARG;
    if ((long long)w * h * 3 > 0x7fffffffLL) return VPPGPU_ERR_INVALID_ARG;
    return VPPGPU_OK;
}

int launch(vppgpu_ctx* ctx, int kind, const short* y, const short* u, const short* v, int nframes, int w, int h,
           int chr_off, int rotate, int flip, unsigned char* rgb)
{
    // Convert(): Real and Impl2 flip first, then rotate; CCIR601 and the 6-bit converters have no flip
    const bool six = kind == VPPGPU_YUV_FAST_6BIT || kind == VPPGPU_YUV_REAL_6BIT;
    const int layout = (kind != VPPGPU_YUV_CCIR601 && !six && flip) ? 2 : (rotate ? 1 : 0);
    YuvParams p;
    p.w = w;
    p.h = h;
    p.six_bit = kind == VPPGPU_YUV_REAL_6BIT;
    p.byte_casts = kind == VPPGPU_YUV_REAL && layout != 1;
    p.chr_off = chr_off;
    p.luma_off = kind == VPPGPU_YUV_CCIR601 ? 16 : 0;
    p.a0 = kind == VPPGPU_YUV_CCIR601 ? 2033 : 2032;
    p.U0 = kind == VPPGPU_YUV_CCIR601 ? 2.033 : 2.032;
    for (int i = 0; i < 256; i++) {
        p.lim_b[i] = host_below_limit(p.U0, i - 128);
        p.lim_r[i] = host_below_limit(1.140, i - 128);
    }
    if (six) {  // a 2x2 block per thread
        long long gx = ((long long)(w >> 1) * (h >> 1) + 255) / 256;
        if (gx > 4096) gx = 4096;
        const dim3 grid((unsigned)gx, nframes);
        if (kind == VPPGPU_YUV_REAL_6BIT)
            k_yuv_rgb_6bit<true><<<grid, 256, 0, ctx->stream>>>(y, u, v, p, layout, rgb);
        else
            k_yuv_rgb_6bit<false><<<grid, 256, 0, ctx->stream>>>(y, u, v, p, layout, rgb);
        VPP_CHECK_LAUNCH(ctx);
        return VPPGPU_OK;
    }
    const bool vec = layout != 1 && (w & 7) == 0 && ((uintptr_t)y & 15) == 0 && ((uintptr_t)u & 7) == 0 &&
                     ((uintptr_t)v & 7) == 0 && ((uintptr_t)rgb & 7) == 0;
    const long long work = vec ? (long long)(w >> 3) * (h >> 1) : (long long)(w >> 1) * (h >> 1);
    long long gx = (work + 255) / 256;
    if (gx > 4096) gx = 4096;
    const dim3 grid((unsigned)gx, nframes);
    if (vec && layout == 2)
        k_yuv_rgb_x8<true><<<grid, 256, 0, ctx->stream>>>(y, u, v, p, rgb);
    else if (vec)
        k_yuv_rgb_x8<false><<<grid, 256, 0, ctx->stream>>>(y, u, v, p, rgb);
    else
        k_yuv_rgb<<<grid, 256, 0, ctx->stream>>>(y, u, v, p, layout, rgb);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

// The zoom converter's sizes: even outputs, and source positions that stay
// inside the planes (the reference reads its centres unclamped: beyond them,
// e.g. for a 2x zoom, it reads outside its buffers).
int zoom_params(int w, int h, int ow, int oh, ZoomParams* z)
{
    if (w < 2 || h < 2 || (w & 1) || (h & 1) || ow < 2 || oh < 2 || (ow & 1) || (oh & 1))
        return VPPGPU_ERR_INVALID_ARG;
    if ((long long)ow * oh * 3 > 0x7fffffffLL || (long long)w * h > 0x7fffffffLL) return VPPGPU_ERR_INVALID_ARG;
    z->w = w;
    z->h = h;
    z->ow = ow;
    z->oh = oh;
    z->sx = (double)w / (double)ow;
    z->sy = (double)h / (double)oh;
    volatile double px = z->sx * (double)(ow - 1), py = z->sy * (double)(oh - 1);
    volatile double qx = px + 0.5, qy = py + 0.5;
    if ((int)qx >= w || (int)qy >= h) return VPPGPU_ERR_UNSUPPORTED;
    return VPPGPU_OK;
}

int zoom_launch(vppgpu_ctx* ctx, const ZoomParams& z, const short* y, const short* u, const short* v,
                unsigned char* rgb)
{
    long long gx = ((long long)(z.ow >> 1) * (z.oh >> 1) + 255) / 256;
    if (gx > 4096) gx = 4096;
    k_yuv_rgb_zoom<<<(unsigned)gx, 256, 0, ctx->stream>>>(y, u, v, z, rgb);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

}  // namespace

extern "C" {

int vppgpu_yuv420_to_rgb24_zoom_device(vppgpu_ctx* ctx, const short* d_y, const short* d_u, const short* d_v,
                                       int width, int height, int out_width, int out_height, unsigned char* d_rgb)
{
    if (!ctx || !d_y || !d_u || !d_v || !d_rgb) return VPPGPU_ERR_INVALID_ARG;
    ZoomParams z;
    int rc = zoom_params(width, height, out_width, out_height, &z);
    if (rc) return rc;
    if ((rc = vppgpu::bind(ctx))) return rc;
    return zoom_launch(ctx, z, d_y, d_u, d_v, d_rgb);
}

int vppgpu_yuv420_to_rgb24_zoom(vppgpu_ctx* ctx, const short* y, const short* u, const short* v, int width,
                                int height, int out_width, int out_height, unsigned char* rgb)
{
    if (!ctx || !y || !u || !v || !rgb) return VPPGPU_ERR_INVALID_ARG;
    ZoomParams z;
    int rc = zoom_params(width, height, out_width, out_height, &z);
    if (rc) return rc;
    if ((rc = vppgpu::bind(ctx))) return rc;
    const size_t ny = (size_t)width * height * 2, nc = (size_t)(width / 2) * (height / 2) * 2,
                 nout = (size_t)out_width * out_height * 3;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t o_u = up(ny), o_v = o_u + up(nc), o_rgb = o_v + up(nc), tot = o_rgb + nout;
    unsigned char* d = nullptr;
    VPP_CUDA(cudaMallocAsync((void**)&d, tot, ctx->stream));
    cudaError_t e = cudaMemcpyAsync(d, y, ny, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d + o_u, u, nc, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d + o_v, v, nc, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        rc = zoom_launch(ctx, z, (const short*)d, (const short*)(d + o_u), (const short*)(d + o_v), d + o_rgb);
        if (rc == VPPGPU_OK) e = cudaMemcpyAsync(rgb, d + o_rgb, nout, cudaMemcpyDeviceToHost, ctx->stream);
    }
    cudaFreeAsync(d, ctx->stream);
    cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
    if (rc) return rc;
    if (e != cudaSuccess) return vppgpu::cuda_status(e);
    if (e2 != cudaSuccess) return vppgpu::cuda_status(e2);
    return VPPGPU_OK;
}

int vppgpu_yuv420_to_rgb24_device(vppgpu_ctx* ctx, int kind, const short* d_y, const short* d_u, const short* d_v,
                                  int width, int height, int chr_off, int rotate, int flip, unsigned char* d_rgb)
{
    int rc = check(ctx, kind, d_y, d_u, d_v, width, height, d_rgb);
    if (rc) return rc;
    if ((rc = vppgpu::bind(ctx))) return rc;
    return launch(ctx, kind, d_y, d_u, d_v, 1, width, height, chr_off, rotate, flip, d_rgb);
}

int vppgpu_yuv420_to_rgb24_frames_device(vppgpu_ctx* ctx, int kind, const short* d_y, const short* d_u,
                                         const short* d_v, int nframes, int width, int height, int chr_off,
                                         int rotate, int flip, unsigned char* d_rgb)
{
    int rc = check(ctx, kind, d_y, d_u, d_v, width, height, d_rgb);
    if (rc) return rc;
    if (nframes < 1 || nframes > 65535) return VPPGPU_ERR_INVALID_ARG;
    if ((rc = vppgpu::bind(ctx))) return rc;
    return launch(ctx, kind, d_y, d_u, d_v, nframes, width, height, chr_off, rotate, flip, d_rgb);
}

int vppgpu_yuv420_to_rgb24(vppgpu_ctx* ctx, int kind, const short* y, const short* u, const short* v, int width,
                           int height, int chr_off, int rotate, int flip, unsigned char* rgb)
{
    int rc = check(ctx, kind, y, u, v, width, height, rgb);
    if (rc) return rc;
    if ((rc = vppgpu::bind(ctx))) return rc;
    const size_t ny = (size_t)width * height * 2, nc = (size_t)(width / 2) * (height / 2) * 2,
                 nout = (size_t)width * height * 3;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t o_u = up(ny), o_v = o_u + up(nc), o_rgb = o_v + up(nc), tot = o_rgb + nout;
    unsigned char* d = nullptr;
    VPP_CUDA(cudaMallocAsync((void**)&d, tot, ctx->stream));
    cudaError_t e = cudaMemcpyAsync(d, y, ny, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d + o_u, u, nc, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d + o_v, v, nc, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) {
        rc = launch(ctx, kind, (const short*)d, (const short*)(d + o_u), (const short*)(d + o_v), 1, width, height,
                    chr_off, rotate, flip, d + o_rgb);
        if (rc == VPPGPU_OK) e = cudaMemcpyAsync(rgb, d + o_rgb, nout, cudaMemcpyDeviceToHost, ctx->stream);
    }
    cudaFreeAsync(d, ctx->stream);
    cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
    if (rc) return rc;
    if (e != cudaSuccess) return vppgpu::cuda_status(e);
    if (e2 != cudaSuccess) return vppgpu::cuda_status(e2);
    return VPPGPU_OK;
}

}  // extern "C"
