// me_umhs.cu -- MotionEstimatorH264ImplUMHS::Estimate
// (src/CodecUtils/MotionEstimatorH264ImplUMHS.cpp:446-945) and
// MotionEstimatorH264ImplFHS::Estimate (src/CodecUtils/MotionEstimatorH264ImplFHS.cpp:497-900)
// on the GPU.  Both search from the median prediction and share everything
// but the search itself (the kernels are templates on it).
//
// The estimator searches from the median prediction: starting points at the
// prediction, zero and the previous frame's co-located vector; early exits on
// absolute thresholds and on the prediction's distortion; an unsymmetrical
// cross, a 5x5 square, a three-scale 16-point hexagon, then extended-hexagon
// and diamond descents; the half / quarter passes of the full-search window;
// a last comparison with the prediction at quarter-pel costs.  Every search
// depends on its prediction, and the prediction (vector and distortion,
// MacroBlockH264.cpp:818-915) on the left, above and above-right (else
// above-left) final results: a function over the raster-order DAG.
//
//   k_umhs_sweep  relaxation: every macroblock at the prediction of its
//                 neighbours' current states, one warp each, results kept as
//                 records (the search depends on the prediction's distortion
//                 only through one early-exit test, so a record holds for
//                 every distortion that decides that test alike).  A sweep
//                 that changes no state is the DAG's unique fixed point: the
//                 sequential result.
//   k_umhs_wave   otherwise the exact raster result by dataflow: warps take
//                 macroblocks in anti-diagonal order (c + 2r) from a ticket
//                 counter, wait (bounded) for the neighbours' published
//                 states, and take a record for the prediction or search.
//                 Every dependency holds a lower ticket, taken by a running
//                 warp, so the pass cannot deadlock.
//   k_umhs_outputs vectors, distortions and the included average.
#include "me_full_common.cuh"

namespace vppgpu {
namespace {
using namespace full;

constexpr unsigned long long kPending = ~0ull;
constexpr int kNoPdTest = -1;  // record outcome word: the prediction's distortion took no part

__device__ __forceinline__ unsigned long long state_word(int mv, int d)
{
    return (unsigned long long)(unsigned)mv | ((unsigned long long)(unsigned)d << 32);
}
__device__ __forceinline__ int state_mv(unsigned long long s) { return (int)(unsigned)(s & 0xffffffffull); }
__device__ __forceinline__ int state_d(unsigned long long s) { return (int)(unsigned)(s >> 32); }

// A published state is one 64-bit word holding all a reader needs (vector and
// distortion), so the dataflow pass publishes and polls with relaxed
// device-scope accesses: no other data is ordered by them.
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// MEH264IUMHS_COST (MotionEstimatorH264ImplUMHS.cpp:179): (int)(D/256.0 +
// 1.05 * sqrt((double)s)) for a squared distance s.  D/256 splits exactly into
// its integer part and a fraction; the rest is evaluated in float (error
// below 1e-3 over the ranges met here) and only a fractional part within
// 0.002 of an integer takes the IEEE double path, one rounding per operation
// as the reference (built without contraction) evaluates it.
__device__ __noinline__ int cost_double(int d, int s)
{
    return (int)__dadd_rn(__ddiv_rn((double)d, 256.0), __dmul_rn(1.05, __dsqrt_rn((double)s)));
}
__device__ __forceinline__ int umhs_cost(int d, int s)
{
    if (s == 0) return d >> 8;
    const float w = (float)(d & 255) * (1.0f / 256.0f) + 1.05f * __fsqrt_rn((float)s);
    const float fl = floorf(w);
    const float fr = w - fl;
    if (fr > 0.002f && fr < 0.998f) return (d >> 8) + (int)fl;
    return cost_double(d, s);
}

// This lane's 8-sample part of the SSD of the block at full-pel origin
// (x0, y0) (Tsd16x16; Tsd16x16LessThan decides as the full sum).
__device__ __forceinline__ int sd_part(const FullArgs& a, int x0, int y0, uint2 cur, int lane)
{
    const unsigned char* p = a.refp + (size_t)(y0 + (lane >> 1) + PAD) * a.rstride + (x0 + 8 * (lane & 1) + PAD);
    return ssd8(cur, load8(p));
}

// The search window of one macroblock in shared memory: rows m-31 .. m+46,
// columns n-32 .. n+47 of the padded reference (every candidate of a +-31
// range; 16-byte aligned rows, filled with 16-byte loads), and the
// macroblock's own 16x16 samples.
constexpr int kWinRows = 78, kWinStride = 80;
constexpr int kWinBytes = kWinRows * kWinStride;
// per-warp slot: the window, 16 bytes the last row's five-word reads may
// touch, and the 256-byte template
constexpr int kWinSlot = kWinBytes + 16 + 256;

__device__ __forceinline__ void window_fill(const FullArgs& a, int n, int m, unsigned char* win, int lane)
{
    const unsigned char* src = a.refp + (size_t)(m - 31 + PAD) * a.rstride + (n - 32 + PAD);
    constexpr int kVecs = kWinBytes / 16;  // 5 per row
    for (int v = lane; v < kVecs; v += 32) {
        const int r = v / 5, c = v - 5 * r;
        *reinterpret_cast<uint4*>(win + r * kWinStride + 16 * c) =
            __ldg(reinterpret_cast<const uint4*>(src + (size_t)r * a.rstride + 16 * c));
    }
    if (lane < 16)
        *reinterpret_cast<uint4*>(win + kWinBytes + 16 + 16 * lane) =
            __ldg(reinterpret_cast<const uint4*>(a.src8 + (size_t)(m + lane) * a.W + n));
    __syncwarp();
}

// SSD of the whole 16x16 block at offset (x, y) from the macroblock, by one
// lane: per row five window words, funnel-shifted to the block's 16 bytes,
// against the template row (a broadcast read), |a-b| per byte and dp4a.
__device__ __forceinline__ int lane_ssd(const unsigned char* win, int x, int y)
{
    const unsigned char* p = win + (31 + y) * kWinStride + 32 + x;
    const uint4* t = reinterpret_cast<const uint4*>(win + kWinBytes + 16);
    const unsigned* w = reinterpret_cast<const unsigned*>(reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)3);
    const unsigned sh = (unsigned)(reinterpret_cast<uintptr_t>(p) & 3) * 8;
    unsigned acc = 0;
#pragma unroll 2
    for (int r = 0; r < 16; r++) {
        const unsigned* q = w + r * (kWinStride / 4);
        const unsigned w0 = q[0], w1 = q[1], w2 = q[2], w3 = q[3], w4 = q[4];
        const uint4 tr = t[r];
        const unsigned d0 = __vabsdiffu4(__funnelshift_r(w0, w1, sh), tr.x);
        const unsigned d1 = __vabsdiffu4(__funnelshift_r(w1, w2, sh), tr.y);
        const unsigned d2 = __vabsdiffu4(__funnelshift_r(w2, w3, sh), tr.z);
        const unsigned d3 = __vabsdiffu4(__funnelshift_r(w3, w4, sh), tr.w);
        acc = __dp4a(d0, d0, __dp4a(d1, d1, __dp4a(d2, d2, __dp4a(d3, d3, acc))));
    }
    return (int)acc;
}

// One macroblock's search state; every lane of the warp holds the same copy.
struct Search {
    int n, m, xl, xr, yu, yd, px0, py0;
    int mx, my, rmx, rmy, min_d, min_cost;
};

// Search patterns of MotionEstimatorH264ImplUMHS.cpp:82-122, as the steps of
// the search's state machine.
enum Pattern { P_CROSS, P_SQ5, P_HEX, P_EXTHEX, P_DIAMOND, P_DONE };

// Offset (j, i) of candidate c of a pattern, in the reference's test order,
// and whether the pattern tests it at all.  The tables are packed four bits
// per coordinate (value + 4).
__device__ __forceinline__ bool pattern_offset(int kind, int c, int w, int crx, int cry, int mrng, int& j, int& i)
{
    auto nib = [](unsigned long long t, int e) { return (int)((t >> (4 * e)) & 15ull) - 4; };
    switch (kind) {
    case P_CROSS: {  // MEH264IUMHS_CrossPos at scales 1, 3, .., 15, vertical reach below half the range
        const int s = 2 * (c >> 2) + 1, dir = c & 3;
        j = dir == 0 ? -s : (dir == 1 ? s : 0);
        i = dir == 2 ? -s : (dir == 3 ? s : 0);
        return c < 32 && i < mrng / 2 && i > -mrng / 2;
    }
    case P_SQ5: {  // MEH264IUMHS_5x5Pos without the points the cross tested (:632-633)
        if (c >= 24) return false;
        j = c < 16 ? nib(0x6253462453534453ull, c) : nib(0x62625362ull, c - 16);
        i = c < 16 ? nib(0x3322644255335344ull, c) : nib(0x66226655ull, c - 16);
        return !((crx || cry) && ((cry == 0 && (j == 2 || j == -2)) || (crx == 0 && (i == 2 || i == -2))));
    }
    case P_HEX:  // MEH264IUMHS_HexPos at scale w
        if (c >= 16) return false;
        j = w * nib(0x4462628080808080ull, c);
        i = w * nib(0x0811772266335544ull, c);
        return true;
    case P_EXTHEX:  // MEH264IUMHS_ExtHexPos
        if (c >= 6) return false;
        j = nib(0x356532ull, c);
        i = nib(0x664224ull, c);
        return true;
    default:  // P_DIAMOND: MEH264IUMHS_CrossPos at scale 1
        j = c == 0 ? -1 : (c == 1 ? 1 : 0);
        i = c == 2 ? -1 : (c == 3 ? 1 : 0);
        return c < 4;
    }
}

// One pattern step: lane c takes candidate c (in range, D <= the running
// minimum and a strictly lower cost make it the best offset: each pattern
// loop of UMHS.cpp:590-767), computes its SSD and cost, then a ballot walk
// applies the acceptances in the reference's order -- a candidate the walk
// passes was rejected by the state the reference had when it reached it,
// since the state only changes on an acceptance.
__device__ __forceinline__ void probe(Search& s, int kind, int w, int crx, int cry, int mrng, const unsigned char* win,
                                      int lane)
{
    int j = 0, i = 0;
    bool v = pattern_offset(kind, lane, w, crx, cry, mrng, j, i);
    v = v && i + s.my >= s.yu && i + s.my <= s.yd && j + s.mx >= s.xl && j + s.mx <= s.xr;
    int d = 0, cost = 0;
    if (v) {
        d = lane_ssd(win, s.mx + j, s.my + i);
        const int dx = s.mx + j - s.px0, dy = s.my + i - s.py0;
        cost = umhs_cost(d, dx * dx + dy * dy);
    }
    int last = -1;
    while (true) {
        const unsigned m = __ballot_sync(0xffffffffu, v && lane > last && d <= s.min_d && cost < s.min_cost);
        if (!m) break;
        const int f = __ffs(m) - 1;
        s.min_d = __shfl_sync(0xffffffffu, d, f);
        s.min_cost = __shfl_sync(0xffffffffu, cost, f);
        s.rmx = __shfl_sync(0xffffffffu, j, f);
        s.rmy = __shfl_sync(0xffffffffu, i, f);
        last = f;
    }
}

// MotionEstimatorH264ImplUMHS::Estimate for macroblock k at prediction
// (px, py) with distortion pd, one warp.  Returns the record {prediction,
// outcome word, vector, distortion}; the outcome word says whether the
// prediction's distortion decided the first early exit (UMHS.cpp:573-579)
// and how: (start minimum << 1) | taken, else kNoPdTest.  The reference's
// gotos between its pattern stages are a state machine over one probe.
__device__ __noinline__ int4 umhs_evaluate(const UmhsArgs& u, int k, int px, int py, int pd, int lane, int* bad,
                                           unsigned char* win)
{
    const FullArgs& a = u.f;
    Search s;
    s.n = (k % a.cols) * 16;
    s.m = (k / a.cols) * 16;
    const uint2 cur = load_cur8(a, s.n, s.m, lane);
    const int mrng = a.motion_range / 4;
    // the prediction truncated to one macroblock outside the picture (:506-515)
    int px0 = px / 4, py0 = py / 4;
    if (px0 + s.n > a.W) px0 = 16;
    if (px0 + s.n < -16) px0 = -16;
    if (py0 + s.m > a.H) py0 = 16;
    if (py0 + s.m < -16) py0 = -16;
    s.px0 = px0;
    s.py0 = py0;
    full_range(s.n, s.m, a.W, a.H, a.motion_range, s.xl, s.xr, s.yu, s.yd);

    // starting points: prediction, zero, previous frame (:517-571)
    const int pv = __ldg(u.prev + k);
    const int pvx = mv_x(pv), pvy = mv_y(pv);
    const bool use_zero = px0 || py0;
    const bool use_prev = (pvx || pvy) && pvx != px0 && pvy != py0;
    const int p0 = sd_part(a, s.n + px0, s.m + py0, cur, lane);
    const int p1 = use_zero ? sd_part(a, s.n, s.m, cur, lane) : 0;
    const int p2 = use_prev ? sd_part(a, s.n + pvx, s.m + pvy, cur, lane) : 0;
    window_fill(a, s.n, s.m, win, lane);  // the patterns read their candidates from here
    const int pred_vd = warp_sum(p0);
    s.min_d = pred_vd;
    s.mx = px0;
    s.my = py0;
    s.min_cost = pred_vd / 256;
    if (use_zero) {
        const int zd = warp_sum(p1);
        const int zc = umhs_cost(zd, px0 * px0 + py0 * py0);
        if (zc < s.min_cost) {
            s.min_d = zd;
            s.min_cost = zc;
            s.mx = s.my = 0;
        }
    }
    if (use_prev) {
        const int vd = warp_sum(p2);
        const int vc = umhs_cost(vd, (pvx - px0) * (pvx - px0) + (pvy - py0) * (pvy - py0));
        if (vc < s.min_cost) {
            s.min_d = vd;
            s.min_cost = vc;
            s.mx = pvx;
            s.my = pvy;
        }
    }
    int outcome = kNoPdTest;
    const int d0 = s.min_d;
    int st;  // first early exit (:573-579)
    if (d0 < 1000) {
        st = P_DIAMOND;
    } else if (d0 < 4000) {
        st = P_EXTHEX;
    } else {
        bool taken = false;
        if (d0 == pred_vd) {
            taken = d0 < pd * 12 / 10 && d0 > pd * 8 / 10;
            outcome = (d0 << 1) | (taken ? 1 : 0);
        }
        st = taken ? P_EXTHEX : P_CROSS;
    }
    // each step lowers the integer cost or moves to the next stage: a bound far above any search
    constexpr int kMaxSteps = 1 << 14;
    int w = 1, prior = 0, crx = 0, cry = 0, steps = 0;
    while (st != P_DONE && steps++ < kMaxSteps) {
        if (st == P_CROSS) {  // unsymmetrical cross (:581-616)
            s.rmx = s.rmy = 0;
            prior = s.min_d;
        } else if (st == P_SQ5) {  // 5x5 around the cross winner (:625-656)
            crx = s.rmx;
            cry = s.rmy;
            s.rmx = s.rmy = 0;
        } else if (st == P_HEX) {  // hexagon scales 1..3 around the cross winner, the 5x5 offset kept (:664-702)
            if (w == 1) prior = s.min_d;
        } else {  // extended hexagon (:705-736) and diamond (:739-769) until the centre wins
            s.rmx = s.rmy = 0;
        }
        probe(s, st, w, crx, cry, mrng, win, lane);
        switch (st) {
        case P_CROSS:
            s.mx += s.rmx;
            s.my += s.rmy;
            if (s.min_d < 1000) st = P_DIAMOND;
            else if (s.min_d < 2000 ||
                     (s.min_d < prior * 9 / 10 && (s.rmx || s.rmy) && abs(s.rmx) <= 3 && abs(s.rmy) <= 3))
                st = P_EXTHEX;
            else st = P_SQ5;
            break;
        case P_SQ5:  // on this exit the centre stays at the cross winner (:658-662)
            if (s.min_d < 1000) st = P_DIAMOND;
            else {
                st = P_HEX;
                w = 1;
            }
            break;
        case P_HEX:
            if (((s.rmx || s.rmy) && (s.min_d < 2000 || s.min_d < prior / 5)) || w == 3) {
                s.mx += s.rmx;
                s.my += s.rmy;
                st = P_EXTHEX;
            } else {
                w++;
            }
            break;
        case P_EXTHEX:
            s.mx += s.rmx;
            s.my += s.rmy;
            if (!(s.rmx || s.rmy)) st = P_DIAMOND;
            break;
        default:
            s.mx += s.rmx;
            s.my += s.rmy;
            if (!(s.rmx || s.rmy)) st = P_DONE;
            break;
        }
    }
    if (st != P_DONE) *bad = 1;
    // half / quarter passes of the full-search window (:790-867)
    int min_d = s.min_d;
    int mvx = 4 * s.mx, mvy = 4 * s.my;
    if (a.mode != 2) {
        int qmx, qmy;
        subpel_refine_planes(a, s.n + s.mx, s.m + s.my, cur, lane, &min_d, &qmx, &qmy, a.mode != 1);
        mvx += qmx;
        mvy += qmy;
    }
    // the prediction at quarter pel against the winner, ties to the prediction (:869-908)
    const PredGeom g = pred_geom(s.n, s.m, a.W, a.H, px, py);
    const int pq = (g.fx | g.fy) ? plane_pred_distortion(a, s.n, s.m, g, lane) : pred_vd;
    const int cp = umhs_cost(pq, (g.pcx - px) * (g.pcx - px) + (g.pcy - py) * (g.pcy - py));
    const int cw = umhs_cost(min_d, (mvx - px) * (mvx - px) + (mvy - py) * (mvy - py));
    if (cp <= cw) {
        min_d = pq;
        mvx = g.pcx;
        mvy = g.pcy;
    }
    return make_int4(pack_mv(px, py), outcome, pack_mv(mvx, mvy), min_d);
}

// ---------------------------------------------------------------------------
// MotionEstimatorH264ImplFHS (src/CodecUtils/MotionEstimatorH264ImplFHS.cpp:497-900)
// ---------------------------------------------------------------------------

// Exact floor(sqrt(s)): what (int)std::sqrt(int) gives for the integers met here.
__device__ __forceinline__ int isqrt_floor(int s)
{
    int r = (int)__fsqrt_rn((float)s);
    while (r * r > s) r--;
    while ((r + 1) * (r + 1) <= s) r++;
    return r;
}

// MEH264IFHS_COST (MotionEstimatorH264ImplFHS.cpp:222): (D + 269 * (int)sqrt(s)) >> 8.
__device__ __forceinline__ int fhs_cost(int d, int s) { return (d + 269 * isqrt_floor(s)) >> 8; }

// Td16x16OptimalPathLessThan (MotionEstimatorH264ImplFHS.cpp:1685-1790) by one
// lane for the block at offset (x, y): squared differences along the first 80
// path points, the whole block's distortion extrapolated as D * 256 / N after
// 32, 40, .., 72 points (returned at once above the running minimum) and after
// 80 (returned).  The reference accepts a candidate iff no extrapolation
// exceeds the minimum and the last does not either: *worst is the largest
// extrapolation, *last the value returned when none exceeds.
__device__ __forceinline__ void lane_path(const unsigned char* win, int x, int y, int* worst, int* last)
{
    constexpr signed char P[80][2] = {
        {5, 10},  {13, 5},  {2, 1},   {13, 14}, {1, 14},  {9, 1},   {1, 6},   {15, 9},  {8, 13},  {14, 2},
        {7, 4},   {10, 8},  {4, 15},  {0, 10},  {0, 3},   {5, 0},   {12, 11}, {4, 7},   {12, 0},  {10, 14},
        {3, 12},  {10, 5},  {15, 13}, {4, 3},   {7, 8},   {14, 7},  {6, 13},  {11, 3},  {2, 9},   {9, 10},
        {15, 1},  {7, 2},   {3, 5},   {8, 15},  {1, 12},  {8, 6},   {0, 1},   {12, 9},  {14, 15}, {15, 4},
        {11, 12}, {6, 6},   {7, 11},  {0, 7},   {14, 11}, {7, 0},   {2, 15},  {12, 7},  {2, 3},   {4, 9},
        {12, 2},  {9, 3},   {12, 13}, {3, 0},   {5, 14},  {5, 4},   {0, 13},  {8, 9},   {2, 11},  {11, 15},
        {10, 1},  {2, 7},   {15, 6},  {9, 12},  {5, 2},   {5, 12},  {1, 4},   {11, 5},  {13, 8},  {9, 7},
        {13, 3},  {5, 8},   {10, 11}, {6, 15},  {13, 10}, {8, 4},   {3, 10},  {13, 1},  {1, 8},   {14, 0}};
    const unsigned char* b = win + (31 + y) * kWinStride + 32 + x;
    const unsigned char* t = win + kWinBytes + 16;
    int d = 0, w = 0;
#pragma unroll
    for (int p = 0; p < 80; p++) {
        const int e = (int)b[P[p][1] * kWinStride + P[p][0]] - (int)t[P[p][1] * 16 + P[p][0]];
        d += e * e;
        if (p + 1 >= 32 && p + 1 < 80 && ((p + 1) & 7) == 0) w = max(w, d * 256 / (p + 1));
    }
    *last = d * 256 / 80;
    *worst = max(w, *last);
}

// One FHS pattern pass (the loops of FHS.cpp:688-818): lane c takes candidate
// c, in range, its path distortion accepted at the running minimum and a
// strictly lower integer cost; the acceptances are applied in order by a
// ballot walk as in probe().
__device__ __forceinline__ void fhs_probe(Search& s, int kind, int w, const unsigned char* win, int lane)
{
    int j = 0, i = 0;
    bool v = pattern_offset(kind, lane, w, 0, 0, 1 << 20, j, i);
    v = v && i + s.my >= s.yu && i + s.my <= s.yd && j + s.mx >= s.xl && j + s.mx <= s.xr;
    int worst = 0, d = 0, cost = 0;
    if (v) {
        lane_path(win, s.mx + j, s.my + i, &worst, &d);
        const int dx = s.mx + j - s.px0, dy = s.my + i - s.py0;
        cost = fhs_cost(d, dx * dx + dy * dy);
    }
    int last = -1;
    while (true) {
        const unsigned m = __ballot_sync(0xffffffffu, v && lane > last && worst <= s.min_d && cost < s.min_cost);
        if (!m) break;
        const int f = __ffs(m) - 1;
        s.min_d = __shfl_sync(0xffffffffu, d, f);
        s.min_cost = __shfl_sync(0xffffffffu, cost, f);
        s.rmx = __shfl_sync(0xffffffffu, j, f);
        s.rmy = __shfl_sync(0xffffffffu, i, f);
        last = f;
    }
}

// SSD of the block at quarter-pel offset (qx, qy) from full-pel origin
// (x0, y0), one warp: the H.264 samples of the half-pel planes (the values
// FHS's half-pel cache and QuarterRead hold).
__device__ __forceinline__ int fhs_sub_sd(const FullArgs& a, int x0, int y0, int qx, int qy, uint2 cur, int lane)
{
    const int fx = qx & 3, fy = qy & 3;
    return warp_sum(ssd8(cur, qpel_block8(a, x0 + (qx >> 2), y0 + (qy >> 2), fx, fy, lane)));
}

// HalfPelEstimate (FHS.cpp:1109-1200): the two "h" offsets, the two "b", the
// four "j", strict improvement, leaving after a stage whose minimum is below
// 1000.  *h_exit: it left after the "h" stage.
__device__ __forceinline__ int fhs_half(const FullArgs& a, int x0, int y0, int min, uint2 cur, int lane, int* hx,
                                        int* hy, bool* h_exit)
{
    constexpr int HX[8] = {0, 0, -1, 1, -1, 1, -1, 1}, HY[8] = {-1, 1, 0, 0, -1, -1, 1, 1};
    int part[8];
#pragma unroll
    for (int k = 0; k < 8; k++)
        part[k] = ssd8(cur, load8(even_block(a, x0, y0, 2 * HY[k], 2 * HX[k], lane)));
    int lcl = min;
    *hx = *hy = 0;
    *h_exit = false;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int d = warp_sum(part[k]);
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

// QuarterPelEstimate (FHS.cpp:1213-1480): the half-pel stage, then the eight
// quarter offsets around its winner in MEH264IFHS_SubPos order, strict
// improvement, leaving at a minimum below 1000.  The offset returned is the
// last quarter-pel improvement only (a half-pel winner without one comes back
// as (0, 0) with its distortion), as the reference does.  Where the half-pel
// stage left after "h" with nothing better, the reference's quarter pass reads
// "b" / "j" cache samples of earlier macroblocks; this macroblock's samples
// are used instead, and the event is counted (MeCtrl::ntie).
__device__ __forceinline__ int fhs_quarter(const FullArgs& a, int x0, int y0, int min, uint2 cur, int lane, int* qx,
                                           int* qy)
{
    constexpr int SX[8] = {-1, 0, 1, -1, 1, -1, 0, 1}, SY[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
    int hx, hy;
    bool h_exit;
    const int half = fhs_half(a, x0, y0, min, cur, lane, &hx, &hy, &h_exit);
    int lcl = min;
    *qx = *qy = 0;
    if (half < min) {
        lcl = half;
        if (half < 1000) return lcl;
    }
    if (h_exit && lane == 0) atomicAdd(&a.ctrl->ntie, 1);
    for (int k = 0; k < 8; k++) {
        const int ox = 2 * hx + SX[k], oy = 2 * hy + SY[k];
        const int d = fhs_sub_sd(a, x0, y0, ox, oy, cur, lane);
        if (d < lcl) {
            lcl = d;
            *qx = ox;
            *qy = oy;
            if (d < 1000) break;
        }
    }
    return lcl;
}

// MotionEstimatorH264ImplFHS::Estimate for macroblock k at prediction (px, py)
// with distortion pd, one warp; the record as umhs_evaluate returns it.
__device__ __noinline__ int4 fhs_evaluate(const UmhsArgs& u, int k, int px, int py, int pd, int lane, int* bad,
                                          unsigned char* win)
{
    const FullArgs& a = u.f;
    Search s;
    s.n = (k % a.cols) * 16;
    s.m = (k / a.cols) * 16;
    const uint2 cur = load_cur8(a, s.n, s.m, lane);
    // the prediction truncated to one macroblock outside the picture, its
    // quarter-pel part dropped then (:540-560)
    int pxq = px % 4, pyq = py % 4, px0 = px / 4, py0 = py / 4;
    const int opx0 = px0, opy0 = py0;
    if (px0 + s.n > a.W) px0 = 16;
    if (px0 + s.n < -16) px0 = -16;
    if (py0 + s.m > a.H) py0 = 16;
    if (py0 + s.m < -16) py0 = -16;
    if (opx0 != px0 || opy0 != py0) pxq = pyq = 0;
    const int rpx = 4 * px0 + pxq, rpy = 4 * py0 + pyq;
    s.px0 = px0;
    s.py0 = py0;
    full_range(s.n, s.m, a.W, a.H, a.motion_range, s.xl, s.xr, s.yu, s.yd);
    // the prediction's full SSD at quarter pel (:562-597)
    const int pq = ssd8(cur, qpel_block8(a, s.n + px0 + (pxq < 0 ? -1 : 0), s.m + py0 + (pyq < 0 ? -1 : 0), pxq & 3,
                                         pyq & 3, lane));
    window_fill(a, s.n, s.m, win, lane);
    const int pred_vd = warp_sum(pq);
    s.min_d = pred_vd;
    s.mx = px0;
    s.my = py0;
    s.min_cost = pred_vd >> 8;
    if (pred_vd < 1000) return make_int4(pack_mv(px, py), kNoPdTest, pack_mv(rpx, rpy), pred_vd);
    // zero (:599-625)
    if (rpx || rpy) {
        int worst = 0, zd = 0;
        if (lane == 0) lane_path(win, 0, 0, &worst, &zd);
        worst = __shfl_sync(0xffffffffu, worst, 0);
        zd = __shfl_sync(0xffffffffu, zd, 0);
        if (worst <= s.min_d && zd < s.min_d) {
            const int zc = fhs_cost(zd, px0 * px0 + py0 * py0);
            if (zc < s.min_cost) {
                s.min_d = zd;
                s.min_cost = zc;
                s.mx = s.my = 0;
            }
            if (zd < 1000) return make_int4(pack_mv(px, py), kNoPdTest, 0, s.min_d);
        }
    }
    // first early exit (:681-683)
    int outcome = kNoPdTest;
    const int d0 = s.min_d;
    int st;
    if (d0 < 1000) {
        st = P_DIAMOND;
    } else if (d0 < 4000) {
        st = P_EXTHEX;
    } else {
        bool taken = false;
        if (d0 == pred_vd) {
            taken = d0 < pd * 12 / 10 && d0 > pd * 8 / 10;
            outcome = (d0 << 1) | (taken ? 1 : 0);
        }
        st = taken ? P_EXTHEX : P_HEX;
    }
    if (st == P_HEX) {  // four hexagon scales, no early exit (:684-748)
        s.rmx = s.rmy = 0;
        for (int w = 1; w <= 4; w++) fhs_probe(s, P_HEX, w, win, lane);
        s.mx += s.rmx;
        s.my += s.rmy;
        st = P_EXTHEX;
    }
    if (st == P_EXTHEX) {  // one extended-hexagon pass (:751-784)
        s.rmx = s.rmy = 0;
        fhs_probe(s, P_EXTHEX, 1, win, lane);
        s.mx += s.rmx;
        s.my += s.rmy;
    }
    {  // one diamond pass (:786-820)
        s.rmx = s.rmy = 0;
        fhs_probe(s, P_DIAMOND, 1, win, lane);
        s.mx += s.rmx;
        s.my += s.rmy;
    }
    // half / quarter stages (:822-856)
    int mvx = 4 * s.mx, mvy = 4 * s.my;
    if (a.mode == 0) {
        int qx, qy;
        const int nm = fhs_quarter(a, s.n + s.mx, s.m + s.my, s.min_d, cur, lane, &qx, &qy);
        if (nm < s.min_d) {
            s.min_d = nm;
            mvx += qx;
            mvy += qy;
        }
    } else if (a.mode == 1) {
        int hx, hy;
        bool h_exit;
        const int nm = fhs_half(a, s.n + s.mx, s.m + s.my, s.min_d, cur, lane, &hx, &hy, &h_exit);
        if (nm < s.min_d) {
            s.min_d = nm;
            mvx += 2 * hx;
            mvy += 2 * hy;
        }
    }
    // the prediction check; the costs compare quarter-pel vectors with the
    // full-pel prediction, as the reference does (:858-867)
    const int cp = fhs_cost(pred_vd, (rpx - px0) * (rpx - px0) + (rpy - py0) * (rpy - py0));
    const int cw = fhs_cost(s.min_d, (mvx - px0) * (mvx - px0) + (mvy - py0) * (mvy - py0));
    if (cp <= cw) {
        s.min_d = pred_vd;
        mvx = rpx;
        mvy = rpy;
    }
    (void)bad;
    return make_int4(pack_mv(px, py), outcome, pack_mv(mvx, mvy), s.min_d);
}

// The estimator's evaluation: UMHS or FHS.
template <bool kFhs>
__device__ __forceinline__ int4 evaluate(const UmhsArgs& u, int k, int px, int py, int pd, int lane, int* bad,
                                         unsigned char* win)
{
    if constexpr (kFhs) return fhs_evaluate(u, k, px, py, pd, lane, bad, win);
    else return umhs_evaluate(u, k, px, py, pd, lane, bad, win);
}

// Whether a record made at the prediction's vector holds for distortion pd.
__device__ __forceinline__ bool record_holds(int outcome, int pd)
{
    if (outcome == kNoPdTest) return true;
    const int d0 = outcome >> 1;
    const bool taken = d0 < pd * 12 / 10 && d0 > pd * 8 / 10;
    return taken == ((outcome & 1) != 0);
}

// MacroBlockH264::GetMbMotionMedianPred with distortion (MacroBlockH264.cpp:818-915)
// from the neighbours' state words: the median vector, and the smaller of the
// distortions attached to its components (the y component compares C's x
// component, MacroBlockH264.cpp:898, as the reference does).
__device__ __forceinline__ void median_with_distortion(int av, unsigned long long A, unsigned long long B,
                                                       unsigned long long C, int* px, int* py, int* pd)
{
    if (!(av & AV_A)) A = 0;
    if (!(av & AV_B)) B = 0;
    if (!(av & (AV_C | AV_D))) C = 0;
    if (!(av & AV_B) && !(av & AV_C)) B = C = A;
    const int ax = mv_x(state_mv(A)), ay = mv_y(state_mv(A)), ad = state_d(A);
    const int bx = mv_x(state_mv(B)), by = mv_y(state_mv(B)), bd = state_d(B);
    const int cx = mv_x(state_mv(C)), cy = mv_y(state_mv(C)), cd = state_d(C);
    const int x = median3(ax, bx, cx), y = median3(ay, by, cy);
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

// Lanes 0..UMHS_RECORDS-1 each hold one record of the macroblock: the result
// for prediction (px, py, pd), if one holds.
__device__ __forceinline__ bool record_lookup(int4 e, int px, int py, int pd, int* mv, int* d)
{
    const unsigned hit = __ballot_sync(0xffffffffu, e.x == pack_mv(px, py) && e.w >= 0 && record_holds(e.y, pd));
    if (!hit) return false;
    const int f = __ffs(hit) - 1;
    *mv = __shfl_sync(0xffffffffu, e.z, f);
    *d = __shfl_sync(0xffffffffu, e.w, f);
    return true;
}

__device__ __forceinline__ int4 empty_record() { return make_int4(0, 0, 0, -1); }

// One relaxation sweep: every macroblock (a warp each, grid-stride) at the
// prediction of its neighbours' current states.  Sweep 0 starts from the
// handle's previous estimate's final states (zero after creation): the fixed
// point does not depend on where the relaxation starts, and consecutive frames
// start close to it.  Skipped once an earlier sweep changed nothing.
template <bool kFhs>
__global__ void __launch_bounds__(128) k_umhs_sweep(UmhsArgs u, int sweep)
{
    __shared__ __align__(16) unsigned char wins[4][kWinSlot];
    const FullArgs& a = u.f;
    if (sweep > 0 && __ldcg(a.changed + sweep - 1) == 0) {
        return;  // the fixed point: this sweep's counter stays 0, so the next sweeps return too
    }
    const int lane = threadIdx.x & 31;
    const int rows = a.nmb / a.cols;
    const int* slice = a.job->slice;
    int changed = 0, evals = 0;
    for (int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < a.nmb; k += (gridDim.x * blockDim.x) >> 5) {
        const int av = neighbour_mask(slice, k, a.cols, rows);
        unsigned long long v = 0;
        {
            int nb = -1;
            if (lane == 0 && (av & AV_A)) nb = k - 1;
            if (lane == 1 && (av & AV_B)) nb = k - a.cols;
            if (lane == 2) nb = (av & AV_C) ? k - a.cols + 1 : ((av & AV_D) ? k - a.cols - 1 : -1);
            if (nb >= 0) v = __ldcg(u.state + nb);
        }
        int px, py, pd;
        median_with_distortion(av, __shfl_sync(0xffffffffu, v, 0), __shfl_sync(0xffffffffu, v, 1),
                               __shfl_sync(0xffffffffu, v, 2), &px, &py, &pd);
        int4* rec = u.rec + (size_t)k * UMHS_RECORDS;
        const int4 e = (sweep > 0 && lane < UMHS_RECORDS) ? __ldcg(rec + lane) : empty_record();
        int mv, d;
        if (!record_lookup(e, px, py, pd, &mv, &d)) {
            int bad = 0;
            const int4 r = evaluate<kFhs>(u, k, px, py, pd, lane, &bad, wins[threadIdx.x >> 5]);
            if (bad && lane == 0) atomicOr(&a.ctrl->status, ST_OUT_OF_BOUNDS);
            mv = r.z;
            d = r.w;
            evals++;
            if (sweep == 0) {
                if (lane < UMHS_RECORDS) __stcg(rec + lane, lane == 0 ? r : empty_record());
            } else if (lane == 0) {
                __stcg(rec + sweep % UMHS_RECORDS, r);
            }
        }
        const unsigned long long ns = state_word(mv, d);
        if (lane == 0) {
            if (sweep == 0 || __ldcg(u.state + k) != ns) changed++;
            __stcg(u.state + k, ns);
        }
        __syncwarp();
    }
    if (lane == 0) {
        if (changed) atomicAdd(a.changed + sweep, changed);
        if (evals) {
            atomicAdd(&a.ctrl->relax_miss, evals);
            atomicAdd(a.changed + UMHS_EVALS + sweep, evals);
        }
    }
}

// Whether a relaxation sweep reached the fixed point.
__device__ __forceinline__ bool relaxed(const UmhsArgs& u)
{
    for (int s = 1; s < u.sweeps; s++)
        if (*((volatile const int*)u.f.changed + s) == 0) return true;
    return false;
}

// Which exact pass decides a frame the relaxation left unsettled: the one-CTA
// diagonal pass when the last sweep had to search few macroblocks (few record
// misses to come: cheap steps matter), else the dataflow pass over all SMs
// (many misses: parallel searches matter).  The diagonal pass hands the rest
// of the frame to the dataflow pass when its misses exceed a budget.
__device__ __forceinline__ bool diagonal_pass(const UmhsArgs& u)
{
    return *((volatile const int*)u.f.changed + UMHS_EVALS + u.sweeps - 1) <= u.diag_limit;
}
constexpr int kDiagMissBudget = 48;

// The exact raster result in one CTA: lane l of warp w owns row 32w + l and
// at step t takes column t - 2r, so a step is an anti-diagonal c + 2r = t,
// whose predictions read only earlier steps: the row's own previous result
// (a register) and the row above's last three (a four-slot ring per row in
// shared memory; the slot the row above writes in step t is none of the
// three read).  One block barrier per step, no waits.  A record gives the
// result for the prediction; the lanes that find none are searched by their
// warp, one after another.
template <bool kFhs>
__global__ void __launch_bounds__(512) k_umhs_diag(UmhsArgs u)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const FullArgs& a = u.f;
    if (relaxed(u) || !diagonal_pass(u)) return;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int cols = a.cols, rows = a.nmb / cols;
    unsigned char* win = smem + (size_t)wid * kWinSlot;
    unsigned long long* ring = reinterpret_cast<unsigned long long*>(smem + (size_t)nw * kWinSlot);
    __shared__ int s_misses;
    const int r = wid * 32 + lane;
    const bool row_ok = r < rows;
    const int* slice = a.job->slice;
    unsigned long long left = 0;
    if (threadIdx.x == 0) s_misses = 0;
    __syncthreads();
    int4 nxt[UMHS_RECORDS];
#pragma unroll
    for (int e = 0; e < UMHS_RECORDS; e++) nxt[e] = empty_record();
    if (row_ok && r == 0)
#pragma unroll
        for (int e = 0; e < UMHS_RECORDS; e++) nxt[e] = __ldcg(u.rec + e);
    int misses = 0;
    const int steps = cols + 2 * (rows - 1);
    for (int t = 0; t < steps; t++) {
        const int c = t - 2 * r;
        const bool act = row_ok && c >= 0 && c < cols;
        int4 cur[UMHS_RECORDS];
#pragma unroll
        for (int e = 0; e < UMHS_RECORDS; e++) cur[e] = nxt[e];
        if (row_ok && c + 1 >= 0 && c + 1 < cols)  // next step's records, loaded during this one
#pragma unroll
            for (int e = 0; e < UMHS_RECORDS; e++) nxt[e] = __ldcg(u.rec + ((size_t)r * cols + c + 1) * UMHS_RECORDS + e);
        const int k = r * cols + c;
        int px = 0, py = 0, pd = 0, mv = 0, d = 0;
        bool hit = false;
        if (act) {
            const int av = neighbour_mask(slice, k, cols, rows);
            const unsigned long long* above = ring + (size_t)(r - 1) * 4;
            const unsigned long long B = (av & AV_B) ? above[c & 3] : 0;
            const unsigned long long C =
                (av & AV_C) ? above[(c + 1) & 3] : ((av & AV_D) ? above[(c - 1) & 3] : 0);
            median_with_distortion(av, left, B, C, &px, &py, &pd);
#pragma unroll
            for (int e = 0; e < UMHS_RECORDS; e++)
                if (!hit && cur[e].w >= 0 && cur[e].x == pack_mv(px, py) && record_holds(cur[e].y, pd)) {
                    hit = true;
                    mv = cur[e].z;
                    d = cur[e].w;
                }
        }
        unsigned miss = __ballot_sync(0xffffffffu, act && !hit);
        while (miss) {
            const int f = __ffs(miss) - 1;
            miss &= miss - 1;
            int bad = 0;
            const int4 rr = evaluate<kFhs>(u, __shfl_sync(0xffffffffu, k, f), __shfl_sync(0xffffffffu, px, f),
                                          __shfl_sync(0xffffffffu, py, f), __shfl_sync(0xffffffffu, pd, f), lane,
                                          &bad, win);
            if (bad && lane == 0) atomicOr(&a.ctrl->status, ST_OUT_OF_BOUNDS);
            if (lane == f) {
                mv = rr.z;
                d = rr.w;
            }
            misses++;
        }
        if (act) {
            const unsigned long long st = state_word(mv, d);
            left = st;
            ring[(size_t)r * 4 + (c & 3)] = st;
            __stcg(u.wave + k, st);
        }
        if (lane == 0 && misses) atomicAdd(&s_misses, misses);
        if (lane == 0 && misses) atomicAdd(&a.ctrl->wave_miss, misses);
        misses = 0;
        __syncthreads();
        // every macroblock of diagonals 0..t is published: past the budget the
        // dataflow pass takes the rest
        if (s_misses > kDiagMissBudget) return;
    }
    if (threadIdx.x == 0) a.ctrl->converged = 2;  // the diagonal pass decided the whole frame
}

// The exact raster result by dataflow over the anti-diagonal order.  A warp
// takes the next ticket, prefetches the macroblock's records, waits for its
// neighbours' published states (lanes 0..2, bounded, giving up at once when
// another warp gave up), then takes the record for its prediction or
// searches, and publishes its state with release semantics.
template <bool kFhs>
__global__ void __launch_bounds__(128) k_umhs_wave(UmhsArgs u)
{
    __shared__ __align__(16) unsigned char wins[4][kWinSlot];
    const FullArgs& a = u.f;
    if (relaxed(u) || *((volatile int*)&a.ctrl->converged) == 2) return;
    const int lane = threadIdx.x & 31;
    const int rows = a.nmb / a.cols;
    const int* slice = a.job->slice;
    volatile int* status = &a.ctrl->status;
    int misses = 0;
    while (true) {
        int t = 0;
        if (lane == 0) t = atomicAdd(&a.ctrl->ticket, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= a.nmb) break;
        const int k = __ldg(u.order + t);
        if (__ldcg(u.wave + k) != kPending) continue;  // decided by the diagonal pass before it handed over
        const int av = neighbour_mask(slice, k, a.cols, rows);
        const int4 e = lane < UMHS_RECORDS ? __ldcg(u.rec + (size_t)k * UMHS_RECORDS + lane) : empty_record();
        int nb = -1;
        if (lane == 0 && (av & AV_A)) nb = k - 1;
        if (lane == 1 && (av & AV_B)) nb = k - a.cols;
        if (lane == 2) nb = (av & AV_C) ? k - a.cols + 1 : ((av & AV_D) ? k - a.cols - 1 : -1);
        unsigned long long v = 0;
        if (nb >= 0) {
            long long it = 0;
            while ((v = ld_relaxed_u64(u.wave + nb)) == kPending) {
                if ((++it & 63) == 0 && ((*status & ST_TIMEOUT) || it > a.spin_limit)) {
                    atomicOr(&a.ctrl->status, ST_TIMEOUT);
                    v = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        int px, py, pd;
        median_with_distortion(av, __shfl_sync(0xffffffffu, v, 0), __shfl_sync(0xffffffffu, v, 1),
                               __shfl_sync(0xffffffffu, v, 2), &px, &py, &pd);
        int mv, d;
        if (!record_lookup(e, px, py, pd, &mv, &d)) {
            int bad = 0;
            const int4 r = evaluate<kFhs>(u, k, px, py, pd, lane, &bad, wins[threadIdx.x >> 5]);
            if (bad && lane == 0) atomicOr(&a.ctrl->status, ST_OUT_OF_BOUNDS);
            mv = r.z;
            d = r.w;
            misses++;
        }
        if (lane == 0) st_relaxed_u64(u.wave + k, state_word(mv, d));
        __syncwarp();
    }
    if (lane == 0 && misses) atomicAdd(&a.ctrl->wave_miss, misses);
}

// Outputs: the relaxed state or the exact pass's, vectors, distortions and
// the included sums (UMHS.cpp:910-935); the final states stay as the next
// estimate's starting point.
__global__ void __launch_bounds__(256) k_umhs_outputs(UmhsArgs u)
{
    const FullArgs& a = u.f;
    if (*((volatile int*)&a.ctrl->status) & ST_TIMEOUT) return;
    const bool rel = relaxed(u);
    long long tot = 0;
    int cnt = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.nmb; k += gridDim.x * blockDim.x) {
        const unsigned long long s = rel ? __ldcg(u.state + k) : __ldcg(u.wave + k);
        if (!rel) __stcg(u.state + k, s);
        const int d = state_d(s);
        a.job->out_mv[k] = state_mv(s);
        if (a.job->out_dist) a.job->out_dist[k] = d;
        if (a.job->incl && a.job->incl[k]) {
            tot += d;
            cnt++;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        tot += __shfl_xor_sync(0xffffffffu, tot, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0 && cnt) {
        atomicAdd((unsigned long long*)&a.ctrl->total, (unsigned long long)tot);
        atomicAdd(&a.ctrl->count, cnt);
    }
}

__global__ void k_umhs_average(UmhsArgs u)
{
    const FullArgs& a = u.f;
    if (*((volatile int*)&a.ctrl->status) & ST_TIMEOUT) return;
    // sweeps to the fixed point, or 1000 + the sweeps run when the dataflow pass decided
    int used = 1000 + u.sweeps;
    for (int s = 1; s < u.sweeps; s++)
        if (__ldcg(a.changed + s) == 0) {
            used = s;
            break;
        }
    a.ctrl->sweeps = used;
    const long long t = a.ctrl->total;
    const int c = a.ctrl->count;
    if (a.job->out_avg) *a.job->out_avg = c ? t / c : 0;
}

}  // namespace

size_t umhs_diag_smem(int rows) { return (size_t)((rows + 31) / 32) * kWinSlot + (size_t)rows * 4 * 8; }

int umhs_prepare()
{
    // the largest frame: 8192 / 16 = 512 macroblock rows, 16 warps
    VPP_CUDA(cudaFuncSetAttribute(k_umhs_diag<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)umhs_diag_smem(512)));
    VPP_CUDA(cudaFuncSetAttribute(k_umhs_diag<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)umhs_diag_smem(512)));
    return VPPGPU_OK;
}

int umhs_launch(vppgpu_ctx* ctx, const UmhsArgs& u, int wave_grid)
{
    int rc = full_planes_launch(ctx, u.f);
    if (rc) return rc;
    const int sweep_grid = (u.f.nmb + 3) / 4;
    for (int s = 0; s < u.sweeps; s++) {
        if (u.fhs) k_umhs_sweep<true><<<sweep_grid, 128, 0, ctx->stream>>>(u, s);
        else k_umhs_sweep<false><<<sweep_grid, 128, 0, ctx->stream>>>(u, s);
        VPP_CHECK_LAUNCH(ctx);
    }
    VPP_CUDA(cudaMemsetAsync(u.wave, 0xff, sizeof(unsigned long long) * (size_t)u.f.nmb, ctx->stream));
    const int rows = u.f.nmb / u.f.cols, nw = (rows + 31) / 32;
    if (u.fhs) k_umhs_diag<true><<<1, nw * 32, umhs_diag_smem(rows), ctx->stream>>>(u);
    else k_umhs_diag<false><<<1, nw * 32, umhs_diag_smem(rows), ctx->stream>>>(u);
    VPP_CHECK_LAUNCH(ctx);
    if (u.fhs) k_umhs_wave<true><<<wave_grid, 128, 0, ctx->stream>>>(u);
    else k_umhs_wave<false><<<wave_grid, 128, 0, ctx->stream>>>(u);
    VPP_CHECK_LAUNCH(ctx);
    k_umhs_outputs<<<(u.f.nmb + 255) / 256, 256, 0, ctx->stream>>>(u);
    VPP_CHECK_LAUNCH(ctx);
    k_umhs_average<<<1, 1, 0, ctx->stream>>>(u);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

}  // namespace vppgpu
