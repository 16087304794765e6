// me_mrc.cu -- MotionEstimatorH264ImplMultiresCross on sm_103a.
//
// Reference: MotionEstimatorH264ImplMultiresCross::Estimate
// (src/CodecUtils/MotionEstimatorH264ImplMultiresCross.cpp:525-1019).  No
// motion-vector predictor: every macroblock is independent.  Per MB: a cross
// search at level 2 (quarter resolution, mode 2), a +-2 full search (mode 2)
// or a cross search (mode 1) at level 1, a +-2 full search at level 0, the
// half- and quarter-pel stages in the estimator's own 88x88 window, and the
// accept-or-zero heuristic.  Levels 1 and 2 use PartialLessThan (16 phases on
// the stride-4 lattice, reject when 16*D_p > p*min), which is not
// decision-neutral and is reproduced phase by phase.
//
// The reference reads its extended-boundary level copies (borders 19 / 9 / 5)
// through overlays whose origins are clamped (OverlayExtMem2Dv2::SetOrigin)
// and, for the sub-pel window, past the overlay edge as flat row-major memory
// (a column beyond the row continues on the next row).  The device copies
// keep exactly that flat geometry, so the same addresses hold the same
// samples; a read outside a copy sets an error instead of reading.
//
// GB300 design
//   k_mrc_level0   input luma to bytes (0..255 check) and the border-19
//                  reference copy.
//   k_mrc_level1   2:1 decimations (OverlayMem2Dv2::Half) of input and
//                  reference, the border-9 reference copy.
//   k_mrc_level2   the second decimation (mode 2), border-5 copy.
//   k_mrc_search   one warp per macroblock.  Candidate distortions are warp
//                  reductions laid out by phase (lane pair = one phase), so
//                  the 16 phase prefix sums are a shuffle scan; candidates
//                  are tested in the reference's order against the running
//                  minimum.  The sub-pel window's lattice (G, h, b,
//                  j at 22x22 points, with the window's unwritten and
//                  unscaled edge samples) is built per warp in shared memory.
//
// The same file holds the searches of the predictor multi-resolution estimators at prediction
// (0, 0) with their tie trees (MultiresCrossVer2, Multires; their resolve is me_full_resolve.cu),
// and MotionEstimatorH263ImplMultiresCrossVer2 whole (k_v263_*: search, tie trees, relaxation
// sweeps over work lists, the one-CTA exact pass, outputs).
#include "me_full_common.cuh"
#include "me_mrc_search.cuh"

namespace vppgpu {
namespace {

using namespace mrc;

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_mrc_level0(const short* __restrict__ src16, const short* __restrict__ ref16,
                                                   int W, int H, unsigned char* __restrict__ in0,
                                                   unsigned char* __restrict__ e0, int* status)
{
    const int EW = W + 38, EH = H + 38;
    const long long n_in = (long long)W * H, n_e = (long long)EW * EH;
    bool bad = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_in + n_e;
         i += (long long)gridDim.x * blockDim.x) {
        if (i < n_in) {
            const int v = src16[i];
            bad |= (v < 0) | (v > 255);
            in0[i] = (unsigned char)(v & 0xff);
        } else {
            const long long j = i - n_in;
            const int y = (int)(j / EW), x = (int)(j - (long long)y * EW);
            const int sy = min(max(y - 19, 0), H - 1), sx = min(max(x - 19, 0), W - 1);
            const int v = ref16[(size_t)sy * W + sx];
            bad |= (v < 0) | (v > 255);
            e0[j] = (unsigned char)(v & 0xff);
        }
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(status, ST_PIXEL_RANGE);
}

// 2:1 decimation (OverlayMem2Dv2::Half, OverlayMem2Dv2.cpp:3018-3033) of a
// w x h plane at (x, y).
template <typename T>
__device__ __forceinline__ int half_at(const T* p, int w, int x, int y)
{
    const T* q = p + (size_t)(2 * y) * w + 2 * x;
    return ((int)q[0] + q[1] + q[w] + q[w + 1] + 2) >> 2;
}

__global__ void __launch_bounds__(256) k_mrc_level1(const short* __restrict__ src16, const short* __restrict__ ref16,
                                                   int W, int H, unsigned char* __restrict__ in1,
                                                   unsigned char* __restrict__ e1)
{
    const int w1 = W / 2, h1 = H / 2, EW = w1 + 18, EH = h1 + 18;
    const long long n_in = (long long)w1 * h1, n_e = (long long)EW * EH;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_in + n_e;
         i += (long long)gridDim.x * blockDim.x) {
        if (i < n_in) {
            const int y = (int)(i / w1), x = (int)(i - (long long)y * w1);
            in1[i] = (unsigned char)half_at(src16, W, x, y);
        } else {
            const long long j = i - n_in;
            const int y = (int)(j / EW), x = (int)(j - (long long)y * EW);
            e1[j] = (unsigned char)half_at(ref16, W, min(max(x - 9, 0), w1 - 1), min(max(y - 9, 0), h1 - 1));
        }
    }
}

__global__ void __launch_bounds__(256) k_mrc_level2(const unsigned char* __restrict__ in1,
                                                   const unsigned char* __restrict__ e1, int W, int H,
                                                   unsigned char* __restrict__ in2, unsigned char* __restrict__ e2)
{
    const int w1 = W / 2, h1 = H / 2, w2 = w1 / 2, h2 = h1 / 2, EW = w2 + 10, EH = h2 + 10, EW1 = w1 + 18;
    const long long n_in = (long long)w2 * h2, n_e = (long long)EW * EH;
    const unsigned char* r1 = e1 + 9 * (size_t)EW1 + 9;  // level-1 reference inside its border-9 copy
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_in + n_e;
         i += (long long)gridDim.x * blockDim.x) {
        if (i < n_in) {
            const int y = (int)(i / w2), x = (int)(i - (long long)y * w2);
            in2[i] = (unsigned char)half_at(in1, w1, x, y);
        } else {
            const long long j = i - n_in;
            const int y = (int)(j / EW), x = (int)(j - (long long)y * EW);
            e2[j] = (unsigned char)half_at(r1, EW1, min(max(x - 5, 0), w2 - 1), min(max(y - 5, 0), h2 - 1));
        }
    }
}

// kH263: MotionEstimatorH263ImplMultiresCross (…H263ImplMultiresCross.cpp:531-1010), whose motion
// range (doubled into a.motion_range by the caller) and vectors are in half pels.
template <bool kH263>
__global__ void __launch_bounds__(256) k_mrc_search(MrcArgs a)
{
    extern __shared__ Lattice lattice[];  // one per warp
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int k = blockIdx.x * (blockDim.x >> 5) + wib;
    if (k >= a.cols * a.rows_all) return;
    bool bad = false;
    const int mbr = k / a.cols, mbc = k - mbr * a.cols;
    const int vec_pos = k < a.nmb ? k : a.nmb;
    const MbSearch r = search_mb_mrc<kH263>(a, lattice[wib], mbr, mbc, lane, bad);
    int mvx = r.mvx, mvy = r.mvy;

    // accept-or-zero heuristic (…MultiresCross.cpp:943-999; …H263ImplMultiresCross.cpp:960-999: (diff >> 2))
    int weight = 0;
    const int diff0 = r.zero_d - r.min_d, mag = mvx * mvx + mvy * mvy;
    if (kH263 ? (diff0 >> 2) < mag : diff0 < mag) weight++;
    if (r.zero_d < MRC_NOISE_FLOOR) weight++;
    if (diff0 * 10 < r.min_d) weight++;
    int chosen;
    if (r.min_d < r.zero_d && weight < 2) {
        chosen = r.min_d;
    } else {
        mvx = mvy = 0;
        chosen = r.zero_d;
    }
    const bool do_it = a.incl ? (vec_pos < a.nmb ? a.incl[vec_pos] != 0 : false) : true;
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
        if (bad) atomicOr(&a.ctrl->status, ST_OUT_OF_BOUNDS);
        if (vec_pos < a.nmb) {
            a.out_mv[vec_pos] = pack_mv(mvx, mvy);
            if (a.out_dist) a.out_dist[vec_pos] = chosen;
        }
        if (do_it) {
            atomicAdd(reinterpret_cast<unsigned long long*>(&a.ctrl->total), (unsigned long long)(long long)chosen);
            atomicAdd(&a.ctrl->count, 1);
        }
    }
}

__global__ void k_mrc_average(long long* out_avg, MeCtrl* ctrl)
{
    const long long t = ctrl->total;
    const int c = ctrl->count;
    if (out_avg) *out_avg = c ? t / c : 0;
}

// ---------------------------------------------------------------------------
// The predictor estimators, MultiresCrossVer2 (…MultiresCrossVer2.cpp:537-1151)
// and Multires (…Multires.cpp:557-1024).  Their searches depend on the median
// prediction only through tie rules, so every macroblock is searched once at
// prediction (0, 0) and remembers whether a tie occurred: the result then
// holds for any prediction unless it did, and for those MBs eight runs with
// the first three ties decided both ways (the tie tree) give it for any
// prediction.  What follows is a function of the prediction (distortion at
// the prediction through the half-pel planes, GetBestVector) over the
// raster-order DAG of predictions, the same as the full-search estimator's,
// and is resolved by its kernels (me_full_resolve.cu).
template <int kEst>
__global__ void __launch_bounds__(256) k_pred_search(MrcArgs m, FullArgs f)
{
    __shared__ Lattice lattice[8];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int k = blockIdx.x * 8 + wib;
    if (k >= f.nmb) return;
    bool bad = false;
    const MbSearch r = search_pred<kEst>(m, lattice[wib], k / f.cols, k % f.cols, 0, 0, lane, bad);
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
        if (bad) atomicOr(&f.ctrl->status, ST_OUT_OF_BOUNDS);
        if (r.tie) f.tie_list[atomicAdd(&f.ctrl->ntie, 1)] = k;
        const int flags = (r.tie ? full::FLAG_TIE : 0) | neighbour_mask(f.job->slice, k, f.cols, f.nmb / f.cols);
        const int v = pack_mv(r.mvx, r.mvy);
        f.spec4[k] = make_int4(v, r.min_d, r.zero_d, flags);
        f.final_mv[k] = v;
    }
    // searches of a tie MB at other predictions: this one (prediction (0, 0)) and empty slots
    if (r.tie && lane < V2_SEARCH_CACHE)
        f.search_cache[(size_t)k * V2_SEARCH_CACHE + lane] =
            lane == 0 ? make_int4(0, pack_mv(r.mvx, r.mvy), r.min_d, r.tie) : make_int4(0, 0, 0, -1);
}

// The tie tree of every MB whose search met a tie: warp r of a block makes
// run r (its first three ties decided by the bits of r).
template <int kEst>
__global__ void __launch_bounds__(V2_TIE_RUNS * 32) k_pred_tietree(MrcArgs m, FullArgs f)
{
    __shared__ Lattice lattice[V2_TIE_RUNS];
    const int lane = threadIdx.x & 31, run = threadIdx.x >> 5;
    const int ntie = __ldcg(&f.ctrl->ntie);
    V2TieRun* runs = static_cast<V2TieRun*>(f.tie_runs);
    for (int i = blockIdx.x; i < ntie; i += gridDim.x) {
        const int k = __ldcg(f.tie_list + i);
        bool bad = false;
        search_run<kEst>(m, lattice[run], k / f.cols, k % f.cols, run, runs + (size_t)k * V2_TIE_RUNS + run, lane,
                         bad);
        if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&f.ctrl->status, ST_OUT_OF_BOUNDS);
    }
}

__global__ void k_set_mrc(MrcArgs* dst, MrcArgs v) { *dst = v; }

// ---------------------------------------------------------------------------
// MotionEstimatorH263ImplMultiresCrossVer2 (…H263ImplMultiresCrossVer2.cpp:537-1151).  Its search is
// the H.263 MultiresCross search with ties decided towards the prediction of each level, and what
// follows the search (the distortion at the clamped prediction against the zero vector's, the
// accept rule) is a function of the prediction, which H263MotionVectorPredictorImpl1 takes from the
// vectors written so far: a DAG in raster order, as for the H.264 predictor estimators.  Every
// macroblock is searched at prediction (0, 0); a search whose ties never involved a level where the
// prediction differs from zero holds for every prediction, and for the others a tie tree answers for
// any prediction.  Relaxation sweeps then evaluate the macroblocks at the prediction their
// neighbours' current vectors give (results kept as records keyed by the prediction) until a sweep
// changes nothing, which is the unique fixed point of the DAG and so the sequential result;
// otherwise a one-CTA pass over the anti-diagonals decides the frame exactly.
constexpr int kV2Rec = H263V2_RECORDS;   // records per macroblock: {prediction, vector, distortion, 0}
constexpr int kV2Empty = 0x7f7f7f7f;     // no half-pel vector packs to this (memset byte 0x7f)

struct V263 {
    MrcArgs m;
    int4* s0;           // per MB: searched vector at prediction (0, 0), its distortion, zero-vector distortion, ties
    int* state;         // per MB: relaxation's current vector (packed half pels)
    int* wave;          // per MB: the exact pass's vector
    int4* rec;          // kV2Rec per MB
    int* changed;       // vectors changed per sweep, then (from kListLen) each sweep's work-list length
    int* lists;         // two work lists of nmb macroblocks (sweeps alternate), then nmb queue marks
    int* tie_list;      // macroblocks whose search at (0, 0) met a tie
    V2TieRun* runs;     // V2_TIE_RUNS per macroblock: the tie trees of those
    int sweeps;
};

// H263MotionVectorPredictorImpl1::Get16x16Prediction (…H263MotionVectorPredictorImpl1.cpp:72-128) from
// the left (a), above (b) and above-right (c) vectors, each 0 beyond the picture's side: the left one
// in the top row, else the componentwise median.
__device__ __forceinline__ int h263_median(bool top, int a, int b, int c)
{
    if (top) return a;
    return pack_mv(median3(mv_x(a), mv_x(b), mv_x(c)), median3(mv_y(a), mv_y(b), mv_y(c)));
}

// The prediction's vector at each level (…H263ImplMultiresCrossVer2.cpp:624-639): half pels rounded
// away from zero to full pels, halved per level by truncation; pl[2l], pl[2l+1] for level l.
__device__ __forceinline__ void h263_levels(int px, int py, int* pl)
{
    const int x0 = px < 0 ? (px - 1) / 2 : (px + 1) / 2, y0 = py < 0 ? (py - 1) / 2 : (py + 1) / 2;
    pl[0] = x0;
    pl[1] = y0;
    pl[2] = x0 / 2;
    pl[3] = y0 / 2;
    pl[4] = x0 / 2 / 2;
    pl[5] = y0 / 2 / 2;
}

// The search with the estimator's tie rule (…:714-721, 787-794, 844-851, 912-919): the current best
// is kept when the candidate is farther from the level's prediction, the candidate's y distance being
// taken as my + i + predY (the prediction added where the current best's subtracts it).
__device__ __forceinline__ MbSearch h263v2_search(const MrcArgs& a, Lattice& lt, int mbr, int mbc, const int* pl,
                                                  int lane, bool& bad)
{
    auto skip = [pl](int lvl, int mx, int my, int rmx, int rmy, int j, int i) {
        const int px = pl[2 * lvl], py = pl[2 * lvl + 1];
        const int cx = mx + rmx - px, cy = my + rmy - py, nx = mx + j - px, ny = my + i + py;
        return (cy * cy + cx * cx) - (ny * ny + nx * nx) < 0;
    };
    return search_mb_with<false, decltype(skip)&, true>(a, lt, mbr, mbc, skip, lane, bad);
}

// Distortion at the prediction (…:1012-1050): its full-pel part clamped to one macroblock outside the
// picture, OverlayMem2Dv2::HalfRead for its half-pel part, against the input block; one warp, eight
// samples (a row half) per lane.  Within the border-19 copy, which the clamp guarantees except for a
// partial bottom row's block pushed to the copy's last rows, the samples are packed words: HalfRead
// as byte means (half4), the squares by __vabsdiffu4 and dp4a.  Otherwise every sample is a checked
// flat read, as the reference reads past its copy there.  *pv: the clamped half-pel vector.
__device__ int h263v2_pred_d(const MrcArgs& a, int mbr, int mbc, int px, int py, int lane, bool& bad, int* pv)
{
    const int n = 16 * mbc, m = 16 * mbr;
    const int hx = px % 2, hy = py % 2;
    int x0 = px / 2, y0 = py / 2;
    if (x0 + n > a.W) x0 = 16;
    if (x0 + n < -16) x0 = -16;
    if (y0 + m > a.H) y0 = 16;
    if (y0 + m < -16) y0 = -16;
    *pv = pack_mv(2 * x0 + hx, 2 * y0 + hy);
    const Org oi = origin(a.in0, 16, 16, 0, n, m), oe = origin(a.e0, 16, 16, 19, x0 + n, y0 + m);
    const int r = oe.y + (lane >> 1), ri = oi.y + (lane >> 1), cb = (lane & 1) * 8;
    int acc = 0;
    const bool inside = oe.y + (hy < 0 ? -1 : 0) >= 0 && oe.y + 15 + (hy > 0 ? 1 : 0) < a.e0.h && oe.x >= 1 &&
                        oe.x + 17 < a.e0.w;  // warp-uniform
    if (inside) {
        const unsigned char* q = a.e0.p + (size_t)r * a.e0.w + oe.x + cb;
        const unsigned char* qv = q + hy * a.e0.w;
        const uint2 in = __ldg(reinterpret_cast<const uint2*>(a.in0.p + (size_t)ri * a.in0.w + oi.x + cb));
        unsigned u = 0u;
#pragma unroll
        for (int w = 0; w < 2; w++) {
            const unsigned s = (hx || hy) ? half4(word_at(q + 4 * w), word_at(q + 4 * w + hx), word_at(qv + 4 * w),
                                                  word_at(qv + 4 * w + hx), hx, hy)
                                          : word_at(q + 4 * w);
            const unsigned d = __vabsdiffu4(s, w ? in.y : in.x);
            u = __dp4a(d, d, u);
        }
        acc = (int)u;
    } else {
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int c = oe.x + cb + j + (hx < 0 ? -1 : 0);
            int v;
            if (hx && hy)
                v = (rd(a.e0, r, c, bad) + rd(a.e0, r + hy, c, bad) + rd(a.e0, r, c + 1, bad) +
                     rd(a.e0, r + hy, c + 1, bad) + 2) >> 2;
            else if (hx)
                v = (rd(a.e0, r, c, bad) + rd(a.e0, r, c + 1, bad) + 1) >> 1;
            else if (hy)
                v = (rd(a.e0, r, c, bad) + rd(a.e0, r + hy, c, bad) + 1) >> 1;
            else
                v = rd(a.e0, r, c, bad);
            const int d = rd(a.in0, ri, oi.x + cb + j, bad) - v;
            acc += d * d;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

// The choice (…:1052-1142): the better of the clamped prediction and the zero vector (the zero vector on
// a strictly smaller distortion) against the searched vector by MultiresCross's accept rule with
// (zero - min) >> 2.  Returns {vector, distortion}.
__device__ __forceinline__ int2 h263v2_choose(const MbSearch& s, int pv, int pred_d)
{
    int zv = pv, zd = pred_d;
    if (s.zero_d < zd) {
        zd = s.zero_d;
        zv = 0;
    }
    const int diff0 = zd - s.min_d, mag = s.mvx * s.mvx + s.mvy * s.mvy;
    int weight = 0;
    if ((diff0 >> 2) < mag) weight++;
    if (zd < MRC_NOISE_FLOOR) weight++;
    if (diff0 * 10 < s.min_d) weight++;
    if (s.min_d < zd && weight < 2) return make_int2(pack_mv(s.mvx, s.mvy), s.min_d);
    return make_int2(zv, zd);
}

// Tie tree of a macroblock (V2TieRun, as the H.264 Ver2 trees): run `run` of eight decides its t-th tie
// (t < 3) by bit t of run (1 takes the candidate) and records the tie's level and the two vectors
// compared, current (cx, cy) and candidate (nx, ny) in level units.
__device__ void h263v2_run(const MrcArgs& a, Lattice& lt, int mbr, int mbc, int run, V2TieRun* rec, int lane,
                           bool& bad)
{
    int t = 0, lvls = 0, geo[V2_TIE_BITS] = {0, 0, 0};
    bool wide = false;
    auto skip = [&](int lvl, int mx, int my, int rmx, int rmy, int j, int i) {
        const int cx = mx + rmx, cy = my + rmy, nx = mx + j, ny = my + i;
        const bool take = t < V2_TIE_BITS ? ((run >> t) & 1) : true;
        if (t < V2_TIE_BITS) {
            wide |= (unsigned)(cx + 128) > 255u || (unsigned)(cy + 128) > 255u || (unsigned)(nx + 128) > 255u ||
                    (unsigned)(ny + 128) > 255u;
            geo[t] = (cx & 0xff) | ((cy & 0xff) << 8) | ((nx & 0xff) << 16) | ((ny & 0xff) << 24);
            lvls |= lvl << (2 * t);
        }
        t++;
        return !take;
    };
    const MbSearch r = search_mb_with<false, decltype(skip)&, true>(a, lt, mbr, mbc, skip, lane, bad);
    if (lane == 0) {
        for (int e = 0; e < V2_TIE_BITS; e++) rec->geo[e] = geo[e];
        rec->lvl = lvls;
        rec->nev = wide ? 1000 : t;
        rec->mv = pack_mv(r.mvx, r.mvy);
        rec->min_d = r.min_d;
    }
}

// The searched vector and distortion for level predictions pl from a tie tree (the estimator's
// y-sum rule at every recorded tie); false when the tree is too deep.  Lane i < 8 loads run i, so the
// walk costs one round trip.  One warp.
__device__ __forceinline__ bool h263v2_tree(const V2TieRun* runs, const int* pl, int lane, int* mv, int* min_d)
{
    static_assert(kV2Rec == 4, "rec_slot picks one of 4");
    static_assert(sizeof(V2TieRun) == 32, "two 16-byte words per run");
    int4 a = make_int4(0, 0, 0, 0), b = make_int4(0, 0, 0, 0);  // {geo0, geo1, geo2, lvl}, {nev, mv, min_d, -}
    if (lane < V2_TIE_RUNS) {
        const int4* w = reinterpret_cast<const int4*>(runs + lane);
        a = __ldcg(w);
        b = __ldcg(w + 1);
    }
    int run = 0;
    for (int t = 0; t < V2_TIE_BITS; t++) {
        if (t >= __shfl_sync(0xffffffffu, b.x, run)) break;
        const int g = __shfl_sync(0xffffffffu, t == 0 ? a.x : (t == 1 ? a.y : a.z), run);
        const int lvl = (__shfl_sync(0xffffffffu, a.w, run) >> (2 * t)) & 3;
        const int cx = (signed char)(g & 0xff), cy = (signed char)((g >> 8) & 0xff);
        const int nx = (signed char)((g >> 16) & 0xff), ny = (signed char)(g >> 24);
        const int px = pl[2 * lvl], py = pl[2 * lvl + 1];
        const bool skip = (cy - py) * (cy - py) + (cx - px) * (cx - px) < (ny + py) * (ny + py) + (nx - px) * (nx - px);
        run |= (skip ? 0 : 1) << t;
    }
    if (__shfl_sync(0xffffffffu, b.x, run) > V2_TIE_BITS) return false;
    *mv = __shfl_sync(0xffffffffu, b.y, run);
    *min_d = __shfl_sync(0xffffffffu, b.z, run);
    return true;
}

__device__ __forceinline__ unsigned rec_slot(int p) { return ((unsigned)p * 2654435761u) >> 30; }

// Vector and distortion of macroblock k (row mbr, column mbc) at prediction p given its search at
// (0, 0), s0: that search where its ties do not involve the prediction, else the tie tree's answer,
// else a search at p; then the choice, recorded.  One warp.  ghost: a macroblock of a partial bottom
// row (not recorded).
__device__ int2 h263v2_compute(const V263& v, Lattice& lt, int k, int mbr, int mbc, int p, int4 s0, bool ghost,
                               int lane, bool& bad, int& misses, int& searches)
{
    const int px = mv_x(p), py = mv_y(p);
    int pl[6];
    h263_levels(px, py, pl);
    MbSearch s;
    s.mvx = mv_x(s0.x);
    s.mvy = mv_y(s0.x);
    s.min_d = s0.y;
    s.zero_d = s0.z;
    s.tie = s0.w;
    bool reuse = true;
    for (int l = 0; l < 3; l++)
        if ((s.tie & (TIE_L0 >> l)) && (pl[2 * l] || pl[2 * l + 1])) reuse = false;
    if (!reuse) {
        int tmv, td;
        if (h263v2_tree(v.runs + (size_t)k * V2_TIE_RUNS, pl, lane, &tmv, &td)) {
            s.mvx = mv_x(tmv);
            s.mvy = mv_y(tmv);
            s.min_d = td;
        } else {
            s = h263v2_search(v.m, lt, mbr, mbc, pl, lane, bad);
            searches++;
        }
    }
    misses++;
    int pv;
    const int pd = h263v2_pred_d(v.m, mbr, mbc, px, py, lane, bad, &pv);
    const int2 r = h263v2_choose(s, pv, pd);
    if (!ghost && lane == 0) v.rec[(size_t)k * kV2Rec + rec_slot(p)] = make_int4(p, r.x, r.y, 0);
    return r;
}

// The same from the macroblock's record when it holds prediction p (its records and its search at
// (0, 0) are loaded together).
__device__ int2 h263v2_eval(const V263& v, Lattice& lt, int k, int mbr, int mbc, int p, bool ghost, int lane,
                            bool& bad, int& misses, int& searches)
{
    const int4 s0 = __ldcg(v.s0 + k);
    if (!ghost) {
        const int4 e = lane < kV2Rec ? __ldcg(v.rec + (size_t)k * kV2Rec + lane) : make_int4(kV2Empty, 0, 0, 0);
        const unsigned hit = __ballot_sync(0xffffffffu, e.x == p);
        if (hit) {
            const int f = __ffs(hit) - 1;
            return make_int2(__shfl_sync(0xffffffffu, e.y, f), __shfl_sync(0xffffffffu, e.z, f));
        }
    }
    return h263v2_compute(v, lt, k, mbr, mbc, p, s0, ghost, lane, bad, misses, searches);
}

// Prediction of macroblock k from the vector words s, read by ld (left, above, above-right).
template <typename Ld>
__device__ __forceinline__ int h263v2_pred(int k, int cols, Ld&& ld)
{
    const int r = k / cols, c = k - r * cols;
    const int a = c > 0 ? ld(k - 1) : 0;
    if (r == 0) return a;
    return h263_median(false, a, ld(k - cols), c + 1 < cols ? ld(k - cols + 1) : 0);
}

// The search at prediction (0, 0) of every macroblock (a partial bottom row's too) and its choice
// there: the first state.
__global__ void __launch_bounds__(256) k_v263_search(V263 v)
{
    __shared__ Lattice lt;  // never touched by the H.263 search (no sub-pel lattice)
    const int lane = threadIdx.x & 31, k = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (k >= v.m.cols * v.m.rows_all) return;
    bool bad = false;
    const int pl[6] = {0, 0, 0, 0, 0, 0};
    const int mbr = k / v.m.cols, mbc = k - mbr * v.m.cols;
    const MbSearch s = h263v2_search(v.m, lt, mbr, mbc, pl, lane, bad);
    const int2 r = h263v2_choose(s, 0, s.zero_d);  // at (0, 0) the prediction's distortion is the zero vector's
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
        if (bad) atomicOr(&v.m.ctrl->status, ST_OUT_OF_BOUNDS);
        v.s0[k] = make_int4(pack_mv(s.mvx, s.mvy), s.min_d, s.zero_d, s.tie);
        if (s.tie) v.tie_list[atomicAdd(&v.m.ctrl->tie_mbs, 1)] = k;
        if (k < v.m.nmb) {
            v.state[k] = r.x;
            v.rec[(size_t)k * kV2Rec + rec_slot(0)] = make_int4(0, r.x, r.y, 0);
        }
    }
}

// The tie trees of the macroblocks whose search met a tie: warp r of a block makes run r.
__global__ void __launch_bounds__(V2_TIE_RUNS * 32) k_v263_tietree(V263 v)
{
    __shared__ Lattice lt;
    const int lane = threadIdx.x & 31, run = threadIdx.x >> 5;
    const int n = __ldcg(&v.m.ctrl->tie_mbs);
    bool bad = false;
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        const int k = __ldcg(v.tie_list + i), mbr = k / v.m.cols;
        h263v2_run(v.m, lt, mbr, k - mbr * v.m.cols, run, v.runs + (size_t)k * V2_TIE_RUNS + run, lane, bad);
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&v.m.ctrl->status, ST_OUT_OF_BOUNDS);
}

constexpr int kListLen = 64;  // offset of the work-list lengths in V263::changed (after the change counts)
static_assert(H263V2_SWEEPS <= kListLen, "change counts and list lengths must not overlap");

// One relaxation sweep over the macroblocks whose prediction may have moved: every macroblock in the
// first sweep, then those a vector change of the previous sweep reaches (its right, below-left and
// below neighbours, queued once each), each at the prediction of the current vectors (updated in
// place).  A sweep in which nothing changed leaves every macroblock evaluated at its current
// prediction: the fixed point.  A sweep after one that changed nothing returns at once.
__global__ void __launch_bounds__(256) k_v263_sweep(V263 v, int sweep)
{
    __shared__ Lattice lt;
    if (sweep > 0 && __ldcg(v.changed + sweep - 1) == 0) return;
    const int lane = threadIdx.x & 31, cols = v.m.cols, rows = v.m.nmb / cols;
    const int n = sweep == 0 ? v.m.nmb : __ldcg(v.changed + kListLen + sweep - 1);
    const int* in = v.lists + (size_t)((sweep - 1) & 1) * v.m.nmb;
    int* out = v.lists + (size_t)(sweep & 1) * v.m.nmb;
    int* mark = v.lists + 2 * (size_t)v.m.nmb;
    int changed = 0, evals = 0, misses = 0, searches = 0;
    bool bad = false;
    for (int i = blockIdx.x * 8 + (threadIdx.x >> 5); i < n; i += gridDim.x * 8) {
        const int k = sweep == 0 ? i : __ldcg(in + i);
        const int p = h263v2_pred(k, cols, [&](int j) { return __ldcg(v.state + j); });
        const int mbr = k / cols, mbc = k - mbr * cols;
        const int2 r = h263v2_eval(v, lt, k, mbr, mbc, p, false, lane, bad, misses, searches);
        evals++;
        if (lane == 0 && r.x != __ldcg(v.state + k)) {
            __stcg(v.state + k, r.x);
            changed++;
            const int nb[3] = {mbc + 1 < cols ? k + 1 : -1, (mbr + 1 < rows && mbc > 0) ? k + cols - 1 : -1,
                               mbr + 1 < rows ? k + cols : -1};
            for (int e = 0; e < 3; e++)
                if (nb[e] >= 0 && atomicExch(mark + nb[e], sweep) != sweep)
                    out[atomicAdd(v.changed + kListLen + sweep, 1)] = nb[e];
        }
    }
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
        if (bad) atomicOr(&v.m.ctrl->status, ST_OUT_OF_BOUNDS);
        if (changed) atomicAdd(v.changed + sweep, changed);
        atomicAdd(&v.m.ctrl->relax_evals, evals);
        if (misses) atomicAdd(&v.m.ctrl->relax_miss, misses);
        if (searches) atomicAdd(&v.m.ctrl->ntie, searches);
    }
}

__device__ __forceinline__ bool v263_relaxed(const V263& v)
{
    return v.sweeps > 0 && __ldcg(v.changed + v.sweeps - 1) == 0;
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// The exact result in one CTA: thread r owns macroblock row r and at step t takes column t - 2r, so a
// step is an anti-diagonal c + 2r = t whose predictions read only earlier steps: the row's previous
// vector (a register) and the row above's last vectors (a four-slot ring per row in shared memory; the
// slot row r writes in step t is none of the two row r + 1 reads then).  Each row's records and search
// at (0, 0) arrive by cp.async kDiagDepth - 1 steps ahead; a record gives the result for the
// prediction and is published at once; the macroblocks that find none are listed in shared memory
// and evaluated by every warp of the CTA, one macroblock per warp.  One block barrier per step, three
// when a step has misses; no waits.
constexpr int kDiagThreads = 512;  // rows of at most 512 macroblocks (pictures up to 8192 lines)
constexpr int kDiagDepth = 4;      // steps of records in flight per row
constexpr int kDiagPre = kV2Rec + 1;  // 16-byte words per row and step: the records, then the search at (0, 0)
__host__ __device__ constexpr size_t diag_smem(int rows)
{
    return 16 * ((size_t)rows * kDiagDepth * kDiagPre + (size_t)rows + 1) + sizeof(int) * 7 * (size_t)rows;
}
__global__ void __launch_bounds__(kDiagThreads, 1) k_v263_diag(V263 v)
{
    extern __shared__ __align__(16) int4 dsm4[];  // prefetch slots, search-at-(0, 0) list, then the int arrays
    __shared__ Lattice lt;
    __shared__ int s_nmiss[2];
    if (v263_relaxed(v)) return;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int cols = v.m.cols, rows = v.m.nmb / cols;
    int4* pre = dsm4;                                                  // rows x kDiagDepth x kDiagPre
    int4* miss_s0 = pre + (size_t)rows * kDiagDepth * kDiagPre;        // rows (+1 spare)
    int* ring = reinterpret_cast<int*>(miss_s0 + rows + 1);            // 4 per row
    int* miss_k = ring + 4 * rows;
    int* miss_p = miss_k + rows;
    int* miss_v = miss_p + rows;
    const int r = threadIdx.x;
    const bool row_ok = r < rows;
    int4* mine = pre + (size_t)(row_ok ? r : 0) * kDiagDepth * kDiagPre;
    auto issue = [&](int t) {  // the records and search of this row's macroblock of step t
        const int c = t - 2 * r;
        if (row_ok && c >= 0 && c < cols) {
            const size_t k = (size_t)r * cols + c;
            int4* slot = mine + (t % kDiagDepth) * kDiagPre;
#pragma unroll
            for (int e = 0; e < kV2Rec; e++) cp_async16(slot + e, v.rec + k * kV2Rec + e);
            cp_async16(slot + kV2Rec, v.s0 + k);
        }
        cp_async_commit();
    };
    if (threadIdx.x < 2) s_nmiss[threadIdx.x] = 0;
    for (int t = 0; t < kDiagDepth - 1; t++) issue(t);
    __syncthreads();
    int left = 0, misses = 0, searches = 0;
    bool bad = false;
    const int steps = cols + 2 * (rows - 1);
    for (int t = 0; t < steps; t++) {
        issue(t + kDiagDepth - 1);
        cp_async_wait<kDiagDepth - 1>();  // this thread's copies of step t have landed
        const int c = t - 2 * r;
        const bool act = row_ok && c >= 0 && c < cols;
        const int k = r * cols + c;
        int mv = 0, slot = -1;
        if (act) {
            const int4* cur = mine + (t % kDiagDepth) * kDiagPre;
            const int b = r > 0 ? ring[(r - 1) * 4 + (c & 3)] : 0;
            const int cc = (r > 0 && c + 1 < cols) ? ring[(r - 1) * 4 + ((c + 1) & 3)] : 0;
            const int p = h263_median(r == 0, c > 0 ? left : 0, b, cc);
            bool hit = false;
#pragma unroll
            for (int e = 0; e < kV2Rec; e++) {
                const int4 rec = cur[e];
                if (!hit && rec.x == p) {
                    hit = true;
                    mv = rec.y;
                }
            }
            if (hit) {  // published now: no row reads this slot in this step
                left = mv;
                ring[r * 4 + (c & 3)] = mv;
                __stcg(v.wave + k, mv);
            } else {
                slot = atomicAdd(&s_nmiss[t & 1], 1);
                miss_k[slot] = k;
                miss_p[slot] = p;
                miss_s0[slot] = cur[kV2Rec];
            }
        }
        // the next step's counter: last read in step t-1 before that step's last barrier (or it is
        // zero already), first incremented after this step's first barrier
        if (threadIdx.x == 0) s_nmiss[(t + 1) & 1] = 0;
        __syncthreads();
        const int n = s_nmiss[t & 1];
        if (n) {  // the misses, one warp each; then their rows publish and the step ends
            for (int i = wid; i < n; i += nw) {
                const int kk = miss_k[i], mbr = kk / cols;
                const int2 res = h263v2_compute(v, lt, kk, mbr, kk - mbr * cols, miss_p[i], miss_s0[i], false, lane,
                                                bad, misses, searches);
                if (lane == 0) miss_v[i] = res.x;
            }
            __syncthreads();
            if (slot >= 0) {
                mv = miss_v[slot];
                left = mv;
                ring[r * 4 + (c & 3)] = mv;
                __stcg(v.wave + k, mv);
            }
            __syncthreads();
        }
    }
    cp_async_wait<0>();
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
        if (bad) atomicOr(&v.m.ctrl->status, ST_OUT_OF_BOUNDS);
        if (misses) atomicAdd(&v.m.ctrl->wave_miss, misses);
        if (searches) atomicAdd(&v.m.ctrl->ntie, searches);
    }
}

// Outputs: every macroblock's vector and distortion at its final prediction (a record), the
// macroblocks of a partial bottom row evaluated at the prediction of list position N_MB (vecPos stops
// there, …:1137-1143) for the average only, and the included sums (all macroblocks when
// pDistortionIncluded is NULL, …:1095-1101).
__global__ void __launch_bounds__(256) k_v263_outputs(V263 v)
{
    __shared__ Lattice lt;
    if (*((volatile int*)&v.m.ctrl->status) & ST_TIMEOUT) return;
    const int* fin = v263_relaxed(v) ? v.state : v.wave;
    const int lane = threadIdx.x & 31, cols = v.m.cols, nmb = v.m.nmb;
    const int k = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (k >= cols * v.m.rows_all) return;
    const bool ghost = k >= nmb;
    if (ghost && v.m.incl) return;  // pDistortionIncluded[N_MB] is past its end: not included
    bool bad = false;
    int p;
    if (ghost) {
        const int top = nmb - cols;  // H263MotionVectorPredictorImpl1 at blk = N_MB: row N_MB / cols, column 0
        p = top < 0 ? 0 : h263_median(false, 0, __ldcg(fin + top), cols > 1 ? __ldcg(fin + top + 1) : 0);
    } else {
        p = h263v2_pred(k, cols, [&](int i) { return __ldcg(fin + i); });
    }
    const int mbr = k / cols;
    int misses = 0, searches = 0;
    const int2 r = h263v2_eval(v, lt, k, mbr, k - mbr * cols, p, ghost, lane, bad, misses, searches);
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
        if (bad) atomicOr(&v.m.ctrl->status, ST_OUT_OF_BOUNDS);
        if (!ghost) {
            v.m.out_mv[k] = r.x;
            if (v.m.out_dist) v.m.out_dist[k] = r.y;
        }
        if (ghost || !v.m.incl || v.m.incl[k]) {
            atomicAdd(reinterpret_cast<unsigned long long*>(&v.m.ctrl->total), (unsigned long long)(long long)r.y);
            atomicAdd(&v.m.ctrl->count, 1);
        }
        if (k == 0) {  // sweeps to the fixed point, or 1000 + the sweeps run when the exact pass decided
            int used = 1000 + v.sweeps;
            for (int s = 0; s < v.sweeps; s++)
                if (__ldcg(v.changed + s) == 0) {
                    used = s + 1;
                    break;
                }
            v.m.ctrl->sweeps = used;
        }
    }
}

}  // namespace

size_t mrc_scratch_bytes(int W, int H)
{
    const size_t w1 = W / 2, h1 = H / 2, w2 = w1 / 2, h2 = h1 / 2;
    return (size_t)W * H + (size_t)(W + 38) * (H + 38) + w1 * h1 + (w1 + 18) * (h1 + 18) + w2 * h2 +
           (w2 + 10) * (h2 + 10) + 64;
}

namespace {

MrcArgs mrc_args(int W, int H, int motion_range, int mode, unsigned char* scratch)
{
    const int w1 = W / 2, h1 = H / 2, w2 = w1 / 2, h2 = h1 / 2;
    if (mode == 0) mode = (W * H > 40000) ? 2 : 1;  // SetMode(0) (…MultiresCross.cpp:501-513)
    MrcArgs a;
    a.W = W;
    a.H = H;
    a.cols = W / 16;
    a.nmb = a.cols * (H / 16);
    a.rows_all = (H + 15) / 16;
    a.mode = mode;
    a.motion_range = motion_range;
    a.lambda = 0.0;
    unsigned char* p = scratch;
    unsigned char* in0 = p;
    p += (size_t)W * H;
    unsigned char* e0 = p;
    p += (size_t)(W + 38) * (H + 38);
    unsigned char* in1 = p;
    p += (size_t)w1 * h1;
    unsigned char* e1 = p;
    p += (size_t)(w1 + 18) * (h1 + 18);
    unsigned char* in2 = p;
    p += (size_t)w2 * h2;
    unsigned char* e2 = p;
    a.in0 = Buf{in0, W, H};
    a.e0 = Buf{e0, W + 38, H + 38};
    a.in1 = Buf{in1, w1, h1};
    a.e1 = Buf{e1, w1 + 18, h1 + 18};
    a.in2 = Buf{in2, w2, h2};
    a.e2 = Buf{e2, w2 + 10, h2 + 10};
    a.incl = nullptr;
    a.out_mv = nullptr;
    a.out_dist = nullptr;
    a.out_avg = nullptr;
    a.ctrl = nullptr;
    return a;
}

int levels_launch(vppgpu_ctx* ctx, const MrcArgs& a, const short* d_src16, const short* d_ref16)
{
    const int W = a.W, H = a.H, w1 = W / 2, h1 = H / 2, w2 = w1 / 2, h2 = h1 / 2;
    const int cap = ctx->sm_count * 8;
    auto grid = [&](long long work) {
        long long g = (work + 255) / 256;
        return (int)(g < cap ? g : cap);
    };
    k_mrc_level0<<<grid((long long)W * H + (long long)(W + 38) * (H + 38)), 256, 0, ctx->stream>>>(
        d_src16, d_ref16, W, H, (unsigned char*)a.in0.p, (unsigned char*)a.e0.p, &a.ctrl->status);
    VPP_CHECK_LAUNCH(ctx);
    k_mrc_level1<<<grid((long long)w1 * h1 + (long long)(w1 + 18) * (h1 + 18)), 256, 0, ctx->stream>>>(
        d_src16, d_ref16, W, H, (unsigned char*)a.in1.p, (unsigned char*)a.e1.p);
    VPP_CHECK_LAUNCH(ctx);
    if (a.mode == 2) {
        k_mrc_level2<<<grid((long long)w2 * h2 + (long long)(w2 + 10) * (h2 + 10)), 256, 0, ctx->stream>>>(
            a.in1.p, a.e1.p, W, H, (unsigned char*)a.in2.p, (unsigned char*)a.e2.p);
        VPP_CHECK_LAUNCH(ctx);
    }
    return VPPGPU_OK;
}

}  // namespace

int mrc_launch(vppgpu_ctx* ctx, int W, int H, int motion_range, int mode, const short* d_src16, const short* d_ref16,
               unsigned char* scratch, const unsigned char* incl, int* out_mv, int* out_dist, long long* out_avg,
               MeCtrl* ctrl, int warps, bool h263)
{
    MrcArgs a = mrc_args(W, H, h263 ? 2 * motion_range : motion_range, mode, scratch);
    a.incl = incl;
    a.out_mv = out_mv;
    a.out_dist = out_dist;
    a.out_avg = out_avg;
    a.ctrl = ctrl;
    int rc = levels_launch(ctx, a, d_src16, d_ref16);
    if (rc) return rc;
    const int mbs = a.cols * a.rows_all, wpb = (warps == 2 || warps == 4) ? warps : 8;
    if (h263)
        k_mrc_search<true><<<(mbs + wpb - 1) / wpb, 32 * wpb, wpb * sizeof(Lattice), ctx->stream>>>(a);
    else
        k_mrc_search<false><<<(mbs + wpb - 1) / wpb, 32 * wpb, wpb * sizeof(Lattice), ctx->stream>>>(a);
    VPP_CHECK_LAUNCH(ctx);
    k_mrc_average<<<1, 1, 0, ctx->stream>>>(out_avg, ctrl);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

size_t mrc_args_bytes() { return sizeof(MrcArgs); }
size_t mrc_lattice_bytes() { return sizeof(Lattice); }
size_t mrc_tie_runs_bytes() { return sizeof(V2TieRun) * V2_TIE_RUNS; }

int mrc2_launch(vppgpu_ctx* ctx, int est, int mode, unsigned char* scratch, const FullArgs& args,
                const short* d_src16, const short* d_ref16)
{
    MrcArgs m = mrc_args(args.W, args.H, args.motion_range, mode, scratch);
    m.ctrl = args.ctrl;
    m.lambda = args.lambda;
    k_set_mrc<<<1, 1, 0, ctx->stream>>>((MrcArgs*)args.mrc, m);  // for the searches at a prediction
    VPP_CHECK_LAUNCH(ctx);
    int rc = full_planes_launch(ctx, args);
    if (rc) return rc;
    if ((rc = levels_launch(ctx, m, d_src16, d_ref16))) return rc;
    if (est == EST_MULTIRES) {
        k_pred_search<EST_MULTIRES><<<(args.nmb + 7) / 8, 256, 0, ctx->stream>>>(m, args);
        VPP_CHECK_LAUNCH(ctx);
        k_pred_tietree<EST_MULTIRES><<<ctx->sm_count * 2, V2_TIE_RUNS * 32, 0, ctx->stream>>>(m, args);
    } else if (est == EST_V2_LAMBDA) {
        // every MB depends on its prediction: the search at (0, 0) seeds the resolve, no tie trees
        k_pred_search<EST_V2_LAMBDA><<<(args.nmb + 7) / 8, 256, 0, ctx->stream>>>(m, args);
    } else {
        k_pred_search<EST_VER2><<<(args.nmb + 7) / 8, 256, 0, ctx->stream>>>(m, args);
        VPP_CHECK_LAUNCH(ctx);
        k_pred_tietree<EST_VER2><<<ctx->sm_count * 2, V2_TIE_RUNS * 32, 0, ctx->stream>>>(m, args);
    }
    VPP_CHECK_LAUNCH(ctx);
    return full_resolve_launch(ctx, args, 0, est);
}

int h263v2_prepare()
{
    VPP_CUDA(cudaFuncSetAttribute(k_v263_diag, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)diag_smem(kDiagThreads)));
    return VPPGPU_OK;
}

int h263v2_launch(vppgpu_ctx* ctx, const H263V2Job& j)
{
    MrcArgs m = mrc_args(j.W, j.H, 2 * j.motion_range, j.mode, j.scratch);
    m.incl = j.incl;
    m.out_mv = j.out_mv;
    m.out_dist = j.out_dist;
    m.out_avg = j.out_avg;
    m.ctrl = j.ctrl;
    int rc = levels_launch(ctx, m, j.src16, j.ref16);
    if (rc) return rc;
    V263 v;
    v.m = m;
    v.s0 = j.s0;
    v.state = j.state;
    v.wave = j.wave;
    v.rec = j.rec;
    v.changed = j.changed;
    v.lists = j.lists;
    v.tie_list = j.tie_list;
    v.runs = static_cast<V2TieRun*>(j.tie_runs);
    v.sweeps = j.sweeps;
    VPP_CUDA(cudaMemsetAsync(j.rec, 0x7f, sizeof(int4) * kV2Rec * (size_t)m.nmb, ctx->stream));
    VPP_CUDA(cudaMemsetAsync(j.changed, 0, sizeof(int) * (size_t)(kListLen + H263V2_SWEEPS), ctx->stream));
    VPP_CUDA(cudaMemsetAsync(j.lists + 2 * (size_t)m.nmb, 0xff, sizeof(int) * (size_t)m.nmb, ctx->stream));
    // later sweeps walk short work lists: a grid of a few CTAs per SM strides over them
    const int blocks = min((m.nmb + 7) / 8, 4 * ctx->sm_count);
    k_v263_search<<<(m.cols * m.rows_all + 7) / 8, 256, 0, ctx->stream>>>(v);
    VPP_CHECK_LAUNCH(ctx);
    k_v263_tietree<<<j.tree_grid, V2_TIE_RUNS * 32, 0, ctx->stream>>>(v);
    VPP_CHECK_LAUNCH(ctx);
    for (int s = 0; s < j.sweeps; s++) {
        k_v263_sweep<<<blocks, 256, 0, ctx->stream>>>(v, s);
        VPP_CHECK_LAUNCH(ctx);
    }
    k_v263_diag<<<1, kDiagThreads, diag_smem(m.nmb / m.cols), ctx->stream>>>(v);
    VPP_CHECK_LAUNCH(ctx);
    k_v263_outputs<<<(m.cols * m.rows_all + 7) / 8, 256, 0, ctx->stream>>>(v);
    VPP_CHECK_LAUNCH(ctx);
    k_mrc_average<<<1, 1, 0, ctx->stream>>>(j.out_avg, j.ctrl);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

}  // namespace vppgpu
