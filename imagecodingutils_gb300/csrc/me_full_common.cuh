// me_full_common.cuh -- pieces shared by the full-search kernels (search,
// resolve, wavefront): table geometry, the search range of
// MotionEstimatorH264ImplFull::GetMotionRange and the sequential scan replay.
#pragma once

#include "me_common.cuh"
#include "me_internal.h"

namespace vppgpu {
namespace full {

constexpr int RMAX = 31;       // table geometry: i in [-31,31] -> ii = i+31, j -> jj = j+32
constexpr int WROWS = 78;      // window rows m-31 .. m+46 (candidate rows -31..31, plus 15)
constexpr int WSTRIDE = 80;    // window cols n-32 .. n+47 (candidate cols -32..31, plus 15; 16-aligned)
constexpr int H2STRIDE = 81;   // odd stride: conflict-free column walks
constexpr int TAB = 64;        // SSD table is TAB x TAB ints
constexpr int FLAG_TIE = 1;   // the scan met an exact tie: its result may depend on the prediction
constexpr int FLAG_DEEP = 32; // ... and more ties than the tie tree holds: rescan the kept table

// Tie tree of a FLAG_TIE macroblock.  The prediction enters the integer
// search only through exact ties (Full.cpp:424-441): tie e is decided by
// whether the new candidate is not farther from the rounded prediction than
// the running best.  Run p of the tree is the scan with tie e decided by bit
// e of p; it keeps the geometry of its ties and its result after the sub-pel
// stage, so the result for any prediction is a walk down the runs: decide
// tie 0 with run 0's geometry, tie 1 with the geometry of the run that made
// decision 0, and so on.  Stored in the unused last row of the MB's table.
constexpr int TIE_DEPTH = 3;
constexpr int TIE_RUNS = 1 << TIE_DEPTH;
struct TieRun {
    int ev[TIE_DEPTH];  // per tie: running best (x, y), candidate (x, y) as signed bytes
    int nev;            // ties met (<= TIE_DEPTH), -1 for more
    int qmv;            // packed quarter-pel vector after sub-pel refinement
    int qmin;           // its distortion
};
constexpr int TIE_ROW = 63;  // table row (ii = 2*RMAX + 1) free for the tree
static_assert(sizeof(TieRun) * TIE_RUNS <= 64 * sizeof(int), "tie tree exceeds one table row");


// GetMotionRange with zero offset (Full.cpp:1029-1081).
__device__ __forceinline__ void full_range(int n, int m, int W, int H, int motion_range, int& xl, int& xr, int& yu,
                                           int& yd)
{
    // Estimate asks for range = vecRange = motion_range/4 with zero offset, so
    // both vector limits resolve to vecRange - 1 (Full.cpp:1046-1061).
    int vr = motion_range / 4;
    int lr = vr - 1, rr = vr - 1;
    const int boundary = 16;
    xl = (n - lr >= -boundary) ? -lr : -(n + boundary);
    xr = (n + rr < W) ? rr : W - n;
    yu = (m - lr >= -boundary) ? -lr : -(m + boundary);
    yd = (m + rr < H) ? rr : H - m;
}

// Sequential raster replay of the integer search over tab (ii = i+31,
// jj = j+32), one warp.  prx/pry: rounded prediction used at ties.  Returns
// the winner and sets *tie when any exact tie was decided.
//
// Column 0 of the table (jj = 0, outside every range) holds each row's
// minimum over the searched columns.  A row whose minimum is above the
// running minimum cannot accept any candidate (acceptance needs d <= min and
// the minimum only falls), and neither can a row that the skip rule puts out
// of range (Full.cpp:410: row offset plus the running best's row outside
// [yu, yd]), so only the rows that can are visited, found with a ballot over
// the row minima.  On the 1080p pan sequence this visits ~8 rows per
// macroblock instead of ~38.
//
// kForced: instead of the distance rule, exact tie e (in scan order) takes
// bit e of `path`; the geometry of the first TIE_DEPTH ties goes to ev[] and
// their count to *nev (-1 when there were more).
template <bool kForced, int kBatch = 1, typename TabT>
__device__ __forceinline__ void scan_table_t(const TabT& tab, int xl, int xr, int yu, int yd, int prx, int pry,
                                             int path, int lane, int* omx, int* omy, int* omin, int* tie, int* nev,
                                             int* ev)
{
    int ne = 0;
    constexpr int kNone = 0x7fffffff;  // above any 16x16 SSD
    int minD = tab(RMAX, RMAX + 1), mx = 0, my = 0, t = 0;
    const int rm0 = yu + lane <= yd ? tab(yu + lane + RMAX, 0) : kNone;
    const int rm1 = yu + lane + 32 <= yd ? tab(yu + lane + 32 + RMAX, 0) : kNone;
    int done = 0;  // rows yu .. yu+done-1 are behind the scan
    while (true) {
        // the next kBatch rows that can accept, read together: a row needs its
        // minimum at or below the running minimum, and its row offset added to
        // the running best must stay in range (the skip rule applies to every
        // candidate of the row alike, and the best only moves on an acceptance)
        const int r0 = yu + lane + my, r1 = r0 + 32;
        unsigned m0 = __ballot_sync(0xffffffffu, rm0 <= minD && lane >= done && r0 >= yu && r0 <= yd);
        unsigned m1 = __ballot_sync(0xffffffffu, rm1 <= minD && lane + 32 >= done && r1 >= yu && r1 <= yd);
        if (!m0 && !m1) break;
        int offs[kBatch];
        int vals[kBatch][2];
        const int my_batch = my;
#pragma unroll
        for (int q = 0; q < kBatch; q++) {
            int off = -1;
            if (m0) {
                off = __ffs(m0) - 1;
                m0 &= m0 - 1;
            } else if (m1) {
                off = 32 + __ffs(m1) - 1;
                m1 &= m1 - 1;
            }
            offs[q] = off;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int i = yu + off, j = xl + 32 * h + lane;
                const bool valid = off >= 0 && j <= xr && !(i == 0 && j == 0);
                vals[q][h] = valid ? tab(i + RMAX, j + RMAX + 1) : kNone;
            }
        }
#pragma unroll
        for (int q = 0; q < kBatch; q++) {
            const int off = offs[q];
            if (off < 0) break;
            // an acceptance that moved the best to another row changes which rows are in
            // range: the rows after it are found again by the next ballot
            if (q > 0 && my != my_batch) break;
            done = off + 1;
            const int rmin = __shfl_sync(0xffffffffu, off < 32 ? rm0 : rm1, off & 31);
            if (rmin > minD) continue;  // the minimum fell below this row's within the batch
            const int i = yu + off;
            int v[2] = {vals[q][0], vals[q][1]};
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int base = xl + 32 * h;
                if (base > xr) break;
                const int j = base + lane;
                const int d = v[h];
                unsigned pending = 0xffffffffu;
                while (true) {
                    bool ok = d != kNone && d <= minD && (i + my >= yu) && (i + my <= yd) && (j + mx >= xl) &&
                              (j + mx <= xr);
                    unsigned m = __ballot_sync(0xffffffffu, ok) & pending;
                    if (!m) break;
                    int f = __ffs(m) - 1;
                    int df = __shfl_sync(0xffffffffu, d, f);
                    int jf = base + f;
                    bool accept = true;
                    if (df == minD) {
                        t = 1;
                        if (kForced) {
                            const int g = (mx & 0xff) | ((my & 0xff) << 8) | ((jf & 0xff) << 16) | ((i & 0xff) << 24);
                            if (ne == 0) ev[0] = g;
                            if (ne == 1) ev[1] = g;
                            if (ne == 2) ev[2] = g;
                            accept = ne < TIE_DEPTH ? ((path >> ne) & 1) != 0 : true;
                            ne++;
                        } else {
                            int cx = mx - prx, cy = my - pry, nx = jf - prx, ny = i - pry;
                            accept = (cy * cy + cx * cx) - (ny * ny + nx * nx) >= 0;
                        }
                    }
                    if (accept) {
                        minD = df;
                        mx = jf;
                        my = i;
                    }
                    pending &= ~((2u << f) - 1u);
                    if (f == 31) break;
                }
            }
        }
    }
    *omx = mx;
    *omy = my;
    *omin = minD;
    *tie = t;
    if (kForced) *nev = ne <= TIE_DEPTH ? ne : -1;
}

template <typename TabT>
__device__ __forceinline__ void scan_table(const TabT& tab, int xl, int xr, int yu, int yd, int prx, int pry,
                                           int lane, int* omx, int* omy, int* omin, int* tie)
{
    scan_table_t<false, TabT::kBatch>(tab, xl, xr, yu, yd, prx, pry, 0, lane, omx, omy, omin, tie, nullptr, nullptr);
}

// Row minima of the searched columns into column 0 (see scan_table), one
// warp per row.
__device__ __forceinline__ void table_row_minima(int (*tab)[TAB], int xl, int xr, int yu, int yd, int warp,
                                                 int nwarps, int lane)
{
    for (int i = yu + warp; i <= yd; i += nwarps) {
        int* row = tab[i + RMAX];
        const int j0 = xl + lane, j1 = xl + 32 + lane;
        int v = j0 <= xr ? row[j0 + RMAX + 1] : 0x7fffffff;
        if (j1 <= xr) v = min(v, row[j1 + RMAX + 1]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
        __syncwarp();
        if (lane == 0) row[0] = v;
    }
}

struct SmemTab {
    static constexpr int kBatch = 1;
    const int (*t)[TAB];
    __device__ int operator()(int r, int c) const { return t[r][c]; }
};
struct GlobalTab {
    static constexpr int kBatch = 4;  // rows per round trip
    const int* t;
    __device__ int operator()(int r, int c) const { return __ldcg(t + r * TAB + c); }
};

// Eight consecutive bytes from any address: three aligned words and two
// funnel shifts (little endian).
__device__ __forceinline__ uint2 load8(const unsigned char* p)
{
    const uintptr_t u = reinterpret_cast<uintptr_t>(p);
    const unsigned* w = reinterpret_cast<const unsigned*>(u & ~(uintptr_t)3);
    const unsigned sh = (unsigned)(u & 3) * 8;
    const unsigned w0 = __ldg(w), w1 = __ldg(w + 1), w2 = __ldg(w + 2);
    return make_uint2(__funnelshift_r(w0, w1, sh), __funnelshift_r(w1, w2, sh));
}

// Sum of squared byte differences of 8 samples.
__device__ __forceinline__ int ssd8(uint2 a, uint2 b)
{
    const unsigned d0 = __vabsdiffu4(a.x, b.x), d1 = __vabsdiffu4(a.y, b.y);
    return (int)__dp4a(d0, d0, __dp4a(d1, d1, 0u));
}

// This lane's 8 samples (row lane/2, columns 8*(lane&1)..+7 of the 16x16
// block) of the even quarter-pel lattice at quarter offset (qy, qx) from the
// full-pel block origin (x0, y0): the full-pel plane, b (x half), h (y half)
// or j (centre) at a whole-sample shift, which is what the sub-pel window of
// LoadHalfQuartPelWindow (Full.cpp:1095-1182) holds at those offsets.
__device__ __forceinline__ const unsigned char* even_block(const FullArgs& a, int x0, int y0, int qy, int qx, int lane)
{
    const int ry = qy & 3, rx = qx & 3;
    const unsigned char* pl = ry == 0 ? (rx == 0 ? a.refp : a.hpel)
                                      : (rx == 0 ? a.hpel + a.plane_size : a.hpel + 2 * a.plane_size);
    return pl + (size_t)(y0 + (qy >> 2) + (lane >> 1) + PAD) * a.rstride + (x0 + (qx >> 2) + 8 * (lane & 1) + PAD);
}

// Half-pel then quarter-pel refinement around the full-pel winner at
// (x0, y0) (Full.cpp:452-517), one warp, samples from the frame's planes:
// eight half-pel neighbours in MEH264IF_SubPos order, then eight quarter-pel
// neighbours of the half-pel winner, each the rounded mean of the two
// lattice samples LoadQuartPelWindow pairs (Full.cpp:1207-1220); strict
// improvement.  cur: this lane's 8 input samples.  quarter false: the
// half-pel pass only (a half-pel SetMode).
__device__ __forceinline__ void subpel_refine_planes(const FullArgs& a, int x0, int y0, uint2 cur, int lane, int* min_d,
                                                     int* qmx, int* qmy, bool quarter = true)
{
    constexpr int SX[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
    constexpr int SY[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
    // quarter pass: lattice offsets (dy, dx) of the two averaged samples
    constexpr int AY[8] = {-2, -2, -2, 0, 0, 0, 2, 2}, AX[8] = {-2, 0, 0, -2, 2, -2, 0, 0};
    constexpr int BY[8] = {0, 0, 0, 0, 0, 2, 0, 0}, BX[8] = {0, 0, 2, 0, 0, 0, 0, 2};
    int part[8];
#pragma unroll
    for (int k = 0; k < 8; k++) part[k] = ssd8(cur, load8(even_block(a, x0, y0, 2 * SY[k], 2 * SX[k], lane)));
    int best = *min_d, hmx = 0, hmy = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int acc = warp_sum(part[k]);
        if (acc < best) {
            best = acc;
            hmx = 2 * SX[k];
            hmy = 2 * SY[k];
        }
    }
    if (!quarter) {
        *min_d = best;
        *qmx = hmx;
        *qmy = hmy;
        return;
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const uint2 va = load8(even_block(a, x0, y0, hmy + AY[k], hmx + AX[k], lane));
        const uint2 vb = load8(even_block(a, x0, y0, hmy + BY[k], hmx + BX[k], lane));
        part[k] = ssd8(cur, make_uint2(__vavgu4(va.x, vb.x), __vavgu4(va.y, vb.y)));
    }
    int bx = hmx, by = hmy;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int acc = warp_sum(part[k]);
        if (acc < best) {
            best = acc;
            bx = hmx + SX[k];
            by = hmy + SY[k];
        }
    }
    *min_d = best;
    *qmx = bx;
    *qmy = by;
}

// This lane's 8 input samples of macroblock (n, m).
__device__ __forceinline__ uint2 load_cur8(const FullArgs& a, int n, int m, int lane)
{
    return __ldg(reinterpret_cast<const uint2*>(a.src8 + (size_t)(m + (lane >> 1)) * a.W + n + 8 * (lane & 1)));
}

// Prediction clamped to one macroblock outside the picture (Full.cpp:532-541)
// and the folded full-pel origin / fraction of its QuarterRead.
struct PredGeom {
    int pcx, pcy, ox, oy, fx, fy;
};

__device__ __forceinline__ PredGeom pred_geom(int n, int m, int W, int H, int px, int py)
{
    int pxq = px % 4, pyq = py % 4, px0 = px / 4, py0 = py / 4;
    if (px0 + n > W) px0 = 16;
    if (px0 + n < -16) px0 = -16;
    if (py0 + m > H) py0 = 16;
    if (py0 + m < -16) py0 = -16;
    PredGeom g;
    g.pcx = 4 * px0 + pxq;
    g.pcy = 4 * py0 + pyq;
    g.fx = pxq < 0 ? pxq + 4 : pxq;
    g.fy = pyq < 0 ? pyq + 4 : pyq;
    g.ox = n + px0 + (pxq < 0 ? -1 : 0);
    g.oy = m + py0 + (pyq < 0 ? -1 : 0);
    return g;
}

// Distortion at the prediction, one warp: QuarterRead's sixteen cases
// (OverlayMem2Dv2::QuarterRead) as one sample of the full-pel, b, h or j
// plane, or the rounded mean of two.  Lane l covers row l/2, columns
// 8*(l&1) .. +7; squared differences with dp4a on per-byte |differences|.
// This lane's 8 quarter-pel samples (row lane/2, columns 8*(lane&1)..+7) of
// the 16x16 block at full-pel origin (ox, oy) and fraction (fx, fy) in 0..3.
__device__ __forceinline__ uint2 qpel_block8(const FullArgs& a, int ox, int oy, int fx, int fy, int lane)
{
    const int r = lane >> 1, c0 = (lane & 1) * 8, st = a.rstride;
    const size_t o = (size_t)(oy + r + PAD) * st + (size_t)(ox + c0 + PAD);
    const unsigned char* G = a.refp;
    const unsigned char* Bp = a.hpel;
    const unsigned char* Hp = a.hpel + a.plane_size;
    const unsigned char* Jp = a.hpel + 2 * a.plane_size;
    const unsigned char *p1 = G + o, *p2 = G + o;
    bool two = true;
    switch (fx | (fy << 2)) {
    case 0: two = false; break;                          // G
    case 2: p1 = Bp + o; two = false; break;             // b
    case 8: p1 = Hp + o; two = false; break;             // h
    case 10: p1 = Jp + o; two = false; break;            // j
    case 1: p2 = Bp + o; break;                          // a = (G + b)
    case 3: p1 = G + o + 1; p2 = Bp + o; break;          // c = (G[x+1] + b)
    case 4: p2 = Hp + o; break;                          // d = (G + h)
    case 12: p1 = G + o + st; p2 = Hp + o; break;        // n = (G[y+1] + h)
    case 6: p1 = Jp + o; p2 = Bp + o; break;             // f = (j + b)
    case 14: p1 = Jp + o; p2 = Bp + o + st; break;       // q = (j + b[y+1])
    case 9: p1 = Jp + o; p2 = Hp + o; break;             // i = (j + h)
    case 11: p1 = Jp + o; p2 = Hp + o + 1; break;        // k = (j + h[x+1])
    case 5: p1 = Bp + o; p2 = Hp + o; break;             // e = (b + h)
    case 7: p1 = Bp + o; p2 = Hp + o + 1; break;         // g = (b + h[x+1])
    case 13: p1 = Hp + o; p2 = Bp + o + st; break;       // p = (h + b[y+1])
    default: p1 = Hp + o + 1; p2 = Bp + o + st; break;   // r = (h[x+1] + b[y+1])
    }
    uint2 v = load8(p1);
    if (two) {
        const uint2 w = load8(p2);
        v.x = __vavgu4(v.x, w.x);  // (p + q + 1) >> 1 per byte
        v.y = __vavgu4(v.y, w.y);
    }
    return v;
}

__device__ __forceinline__ int plane_pred_distortion(const FullArgs& a, int n, int m, const PredGeom& g, int lane)
{
    return warp_sum(ssd8(load_cur8(a, n, m, lane), qpel_block8(a, g.ox, g.oy, g.fx, g.fy, lane)));
}

}  // namespace full
}  // namespace vppgpu
