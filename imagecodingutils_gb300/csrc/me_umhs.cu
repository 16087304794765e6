// me_umhs.cu -- MotionEstimatorH264ImplUMHS::Estimate
// (src/CodecUtils/MotionEstimatorH264ImplUMHS.cpp:446-945) on the GPU.
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

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
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

// Pattern tables of MotionEstimatorH264ImplUMHS.cpp:82-122 ({x, y} offsets in
// the reference's test order).
__constant__ signed char kSq5[24][2] = {{-1, 0},  {1, 0},  {0, -1}, {0, 1},  {-1, -1}, {1, -1}, {-1, 1}, {1, 1},
                                        {0, -2},  {-2, 0}, {2, 0},  {0, 2},  {-1, -2}, {1, -2}, {-2, -1}, {2, -1},
                                        {-2, 1},  {2, 1},  {-1, 2}, {1, 2},  {-2, -2}, {2, -2}, {-2, 2}, {2, 2}};
__constant__ signed char kCross[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
__constant__ signed char kHex[16][2] = {{-4, 0},  {4, 0},  {-4, 1}, {4, 1},  {-4, -1}, {4, -1}, {-4, 2}, {4, 2},
                                        {-4, -2}, {4, -2}, {-2, 3}, {2, 3}, {-2, -3}, {2, -3}, {0, 4},  {0, -4}};
__constant__ signed char kExtHex[6][2] = {{-2, 0}, {-1, -2}, {1, -2}, {2, 0}, {1, 2}, {-1, 2}};

// One macroblock's search state; every lane of the warp holds the same copy.
struct Search {
    int n, m, xl, xr, yu, yd, px0, py0;
    int mx, my, rmx, rmy, min_d, min_cost;
};

// Candidates c = 0..K-1 at offsets off(c) = (j, i, tested) from the centre,
// in the reference's order: a candidate in range with D <= the running
// minimum and a strictly lower cost becomes the best offset (each pattern
// loop of UMHS.cpp:590-767).  The K distortions are summed together (lane c
// keeps candidate c's sum and its cost), then a ballot walk applies the
// acceptances in order: a candidate the walk passes was rejected by the state
// the reference had when it reached it, since the state only changes on an
// acceptance.
template <int K, typename Off>
__device__ __forceinline__ void probe(const FullArgs& a, Search& s, uint2 cur, int lane, Off off)
{
    static_assert(K <= 32, "one candidate per lane");
    int myd = 0, myj = 0, myi = 0;
    bool myv = false;
#pragma unroll
    for (int c = 0; c < K; c++) {
        int j, i;
        bool v = off(c, j, i);
        v = v && i + s.my >= s.yu && i + s.my <= s.yd && j + s.mx >= s.xl && j + s.mx <= s.xr;
        const int part = v ? sd_part(a, s.n + s.mx + j, s.m + s.my + i, cur, lane) : 0;
        const int sum = warp_sum(part);
        if (lane == c) {
            myd = sum;
            myj = j;
            myi = i;
            myv = v;
        }
    }
    const int dx = s.mx + myj - s.px0, dy = s.my + myi - s.py0;
    const int mycost = myv ? umhs_cost(myd, dx * dx + dy * dy) : 0;
    int last = -1;
    while (true) {
        const unsigned m = __ballot_sync(0xffffffffu, myv && lane > last && myd <= s.min_d && mycost < s.min_cost);
        if (!m) break;
        const int f = __ffs(m) - 1;
        s.min_d = __shfl_sync(0xffffffffu, myd, f);
        s.min_cost = __shfl_sync(0xffffffffu, mycost, f);
        s.rmx = __shfl_sync(0xffffffffu, myj, f);
        s.rmy = __shfl_sync(0xffffffffu, myi, f);
        last = f;
    }
}

// MotionEstimatorH264ImplUMHS::Estimate for macroblock k at prediction
// (px, py) with distortion pd, one warp.  Returns the record {prediction,
// outcome word, vector, distortion}; the outcome word says whether the
// prediction's distortion decided the first early exit (UMHS.cpp:573-579)
// and how: (start minimum << 1) | taken, else kNoPdTest.
__device__ __noinline__ int4 umhs_evaluate(const UmhsArgs& u, int k, int px, int py, int pd, int lane, int* bad)
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
    // 0: diamond, 1: extended hexagon, 2: the full descent
    int entry;
    if (d0 < 1000) {
        entry = 0;
    } else if (d0 < 4000) {
        entry = 1;
    } else {
        bool taken = false;
        if (d0 == pred_vd) {
            taken = d0 < pd * 12 / 10 && d0 > pd * 8 / 10;
            outcome = (d0 << 1) | (taken ? 1 : 0);
        }
        entry = taken ? 1 : 2;
    }
    if (entry == 2) {
        // unsymmetrical cross, 8 scales x 4 points, vertical reach below half the range (:581-616)
        s.rmx = s.rmy = 0;
        int prior = s.min_d;
        probe<32>(a, s, cur, lane, [&](int c, int& j, int& i) {
            const int w = 2 * (c >> 2) + 1;
            j = w * kCross[c & 3][0];
            i = w * kCross[c & 3][1];
            return i < mrng / 2 && i > -mrng / 2;
        });
        s.mx += s.rmx;
        s.my += s.rmy;
        if (s.min_d < 1000) {
            entry = 0;
        } else if (s.min_d < 2000 ||
                   (s.min_d < prior * 9 / 10 && (s.rmx || s.rmy) && abs(s.rmx) <= 3 && abs(s.rmy) <= 3)) {
            entry = 1;
        } else {
            // 5x5 without the points the cross tested (:625-656)
            const int crx = s.rmx, cry = s.rmy;
            s.rmx = s.rmy = 0;
            probe<24>(a, s, cur, lane, [&](int c, int& j, int& i) {
                j = kSq5[c][0];
                i = kSq5[c][1];
                return !((crx || cry) && ((cry == 0 && (j == 2 || j == -2)) || (crx == 0 && (i == 2 || i == -2))));
            });
            if (s.min_d < 1000) {
                entry = 0;  // the centre stays at the cross winner (:658-662)
            } else {
                // three hexagon scales around the cross winner, the 5x5 offset still a candidate (:664-702)
                prior = s.min_d;
                for (int w = 1; w < 4; w++) {
                    probe<16>(a, s, cur, lane, [&](int c, int& j, int& i) {
                        j = w * kHex[c][0];
                        i = w * kHex[c][1];
                        return true;
                    });
                    if ((s.rmx || s.rmy) && (s.min_d < 2000 || s.min_d < prior / 5)) break;
                }
                s.mx += s.rmx;
                s.my += s.rmy;
                entry = 1;
            }
        }
    }
    // each step of the descents lowers the integer cost: at most a few hundred steps
    constexpr int kMaxSteps = 1 << 14;
    if (entry == 1) {  // extended hexagon until the centre wins (:705-736)
        int it = 0;
        do {
            s.rmx = s.rmy = 0;
            probe<6>(a, s, cur, lane, [&](int c, int& j, int& i) {
                j = kExtHex[c][0];
                i = kExtHex[c][1];
                return true;
            });
            s.mx += s.rmx;
            s.my += s.rmy;
        } while ((s.rmx || s.rmy) && ++it < kMaxSteps);
        if (it >= kMaxSteps) *bad = 1;
    }
    {  // diamond until the centre wins (:739-769)
        int it = 0;
        do {
            s.rmx = s.rmy = 0;
            probe<4>(a, s, cur, lane, [&](int c, int& j, int& i) {
                j = kCross[c][0];
                i = kCross[c][1];
                return true;
            });
            s.mx += s.rmx;
            s.my += s.rmy;
        } while ((s.rmx || s.rmy) && ++it < kMaxSteps);
        if (it >= kMaxSteps) *bad = 1;
    }
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
// prediction of its neighbours' current states (all zero in sweep 0).
// Skipped once an earlier sweep changed nothing.
__global__ void __launch_bounds__(256) k_umhs_sweep(UmhsArgs u, int sweep)
{
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
        if (sweep > 0) {
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
            const int4 r = umhs_evaluate(u, k, px, py, pd, lane, &bad);
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
        if (evals) atomicAdd(&a.ctrl->relax_miss, evals);
    }
}

// Whether a relaxation sweep reached the fixed point.
__device__ __forceinline__ bool relaxed(const UmhsArgs& u)
{
    for (int s = 1; s < u.sweeps; s++)
        if (*((volatile const int*)u.f.changed + s) == 0) return true;
    return false;
}

// The exact raster result by dataflow over the anti-diagonal order.  A warp
// takes the next ticket, prefetches the macroblock's records, waits for its
// neighbours' published states (lanes 0..2, bounded, giving up at once when
// another warp gave up), then takes the record for its prediction or
// searches, and publishes its state with release semantics.
__global__ void __launch_bounds__(128) k_umhs_wave(UmhsArgs u)
{
    const FullArgs& a = u.f;
    if (relaxed(u)) return;
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
        const int av = neighbour_mask(slice, k, a.cols, rows);
        const int4 e = lane < UMHS_RECORDS ? __ldcg(u.rec + (size_t)k * UMHS_RECORDS + lane) : empty_record();
        int nb = -1;
        if (lane == 0 && (av & AV_A)) nb = k - 1;
        if (lane == 1 && (av & AV_B)) nb = k - a.cols;
        if (lane == 2) nb = (av & AV_C) ? k - a.cols + 1 : ((av & AV_D) ? k - a.cols - 1 : -1);
        unsigned long long v = 0;
        if (nb >= 0) {
            long long it = 0;
            while ((v = ld_acquire_u64(u.wave + nb)) == kPending) {
                if ((++it & 63) == 0 && ((*status & ST_TIMEOUT) || it > a.spin_limit)) {
                    atomicOr(&a.ctrl->status, ST_TIMEOUT);
                    v = 0;
                    break;
                }
            }
        }
        int px, py, pd;
        median_with_distortion(av, __shfl_sync(0xffffffffu, v, 0), __shfl_sync(0xffffffffu, v, 1),
                               __shfl_sync(0xffffffffu, v, 2), &px, &py, &pd);
        int mv, d;
        if (!record_lookup(e, px, py, pd, &mv, &d)) {
            int bad = 0;
            const int4 r = umhs_evaluate(u, k, px, py, pd, lane, &bad);
            if (bad && lane == 0) atomicOr(&a.ctrl->status, ST_OUT_OF_BOUNDS);
            mv = r.z;
            d = r.w;
            misses++;
        }
        if (lane == 0) st_release_u64(u.wave + k, state_word(mv, d));
        __syncwarp();
    }
    if (lane == 0 && misses) atomicAdd(&a.ctrl->wave_miss, misses);
}

// Outputs: the relaxed state or the dataflow pass's, vectors, distortions and
// the included sums (UMHS.cpp:910-935).
__global__ void __launch_bounds__(256) k_umhs_outputs(UmhsArgs u)
{
    const FullArgs& a = u.f;
    if (*((volatile int*)&a.ctrl->status) & ST_TIMEOUT) return;
    const bool rel = relaxed(u);
    long long tot = 0;
    int cnt = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.nmb; k += gridDim.x * blockDim.x) {
        const unsigned long long s = rel ? __ldcg(u.state + k) : __ldcg(u.wave + k);
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

int umhs_launch(vppgpu_ctx* ctx, const UmhsArgs& u, int wave_grid)
{
    int rc = full_planes_launch(ctx, u.f);
    if (rc) return rc;
    const int sweep_grid = (u.f.nmb + 7) / 8;
    for (int s = 0; s < u.sweeps; s++) {
        k_umhs_sweep<<<sweep_grid, 256, 0, ctx->stream>>>(u, s);
        VPP_CHECK_LAUNCH(ctx);
    }
    VPP_CUDA(cudaMemsetAsync(u.wave, 0xff, sizeof(unsigned long long) * (size_t)u.f.nmb, ctx->stream));
    k_umhs_wave<<<wave_grid, 128, 0, ctx->stream>>>(u);
    VPP_CHECK_LAUNCH(ctx);
    k_umhs_outputs<<<(u.f.nmb + 255) / 256, 256, 0, ctx->stream>>>(u);
    VPP_CHECK_LAUNCH(ctx);
    k_umhs_average<<<1, 1, 0, ctx->stream>>>(u);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

}  // namespace vppgpu
