// me_full_resolve.cu -- prediction-dependent tail of MotionEstimatorH264ImplFull.
//
// After the search every macroblock has its prediction-independent results
// (sub-pel vector and distortion, zero-vector distortion).  What is left is a
// function of the median prediction (Full.cpp:368-380 rounding, 401-446 tie
// rescan, 532-590 prediction distortion and GetBestVector), and the
// prediction depends on the left / above / above-right (else above-left)
// neighbours' final vectors: a DAG in raster order.
//
// Every evaluation of a macroblock at a prediction is kept as a record
// {prediction, distortion at it, final vector, final distortion} in a small
// per-MB cache, so a later visit with the same prediction is a lookup.  The
// distortion at a prediction reads the frame's precomputed half-pel planes
// (two byte loads per sample at most).
//
//   k_full_sweep0      every MB at once, prediction from the current vectors
//                      (initially the searched ones).
//   k_full_relax_sweep up to FullArgs::relax_sweeps launches, each re-evaluating the
//                      MBs whose prediction moved.  A sweep without change
//                      is the unique fixed point of the DAG, i.e. the
//                      sequential result; most frames stop here
//                      (k_full_relax_outcome writes their outputs).
//                      Otherwise (long copy chains: the prediction wins and
//                      is copied along rows and columns) k_full_relax_outcome
//                      builds a dictionary of the frame's dominant vectors.
//   k_full_precompute  records of every MB at every dictionary vector.
//   k_full_wave        one CTA replays the exact sequential order, pipelined
//                      by rows: warp w owns rows w, w+32, ...; a row advances
//                      one MB per step once the row above has finished the
//                      MB above-right, signalled through shared-memory
//                      progress counters.  A step is a median, a key match
//                      against the MB's records (prefetched with cp.async)
//                      and, on a miss only, a full evaluation by the warp.
#include "me_cross_search.cuh"
#include "me_full_common.cuh"
#include "me_mrc_search.cuh"

namespace vppgpu {
namespace {
using namespace full;

constexpr int kEmpty = 0x7fffffff;  // no vector packs to this (|y| < 32767 quarter pels)
constexpr int kCacheRelax = 1;      // entries 1..3 round robin in relaxation
constexpr int kCacheDict = 4;       // entries 4..11 dictionary
constexpr int kCacheClosure = 12;   // entries 12..31 neighbour closure
constexpr int kSetMax = 6;          // possible final vectors kept per neighbour

__device__ __forceinline__ int4 empty_record() { return make_int4(kEmpty, 0, 0, 0); }

// Walk a tie tree held one word per lane (t0: words 0..31, t1: 32..): the
// outcome of the scan for rounded prediction (prx, pry).
__device__ __forceinline__ void tree_pick(int t0, int t1, int prx, int pry, int* mvx, int* mvy, int* minD)
{
    constexpr int RW = sizeof(TieRun) / sizeof(int);
    auto get = [&](int idx) {
        const int v0 = __shfl_sync(0xffffffffu, t0, idx & 31), v1 = __shfl_sync(0xffffffffu, t1, idx & 31);
        return idx < 32 ? v0 : v1;
    };
    int path = 0;
    for (int e = 0; e < TIE_DEPTH; e++) {
        if (e >= get(path * RW + TIE_DEPTH)) break;
        const int g = get(path * RW + e);
        const int cx = (int)(signed char)(g & 0xff) - prx, cy = (int)(signed char)((g >> 8) & 0xff) - pry;
        const int nx = (int)(signed char)((g >> 16) & 0xff) - prx, ny = (int)(signed char)((g >> 24) & 0xff) - pry;
        if ((cy * cy + cx * cx) - (ny * ny + nx * nx) >= 0) path |= 1 << e;
    }
    const int q = get(path * RW + TIE_DEPTH + 1);
    *mvx = mv_x(q);
    *mvy = mv_y(q);
    *minD = get(path * RW + TIE_DEPTH + 2);
}

// Exact-tie macroblocks: the integer scan depends on the rounded prediction.
// Walk the tie tree the search kernel kept (one load per lane), or, for the
// rare macroblock with more ties than the tree holds, replay the scan from
// the kept table and redo the sub-pel stage if the full-pel winner moved.
// Kept out of line.
__device__ __noinline__ void tie_path(const FullArgs& a, int k, int px, int py, int flags, int lane, int* mvx,
                                      int* mvy, int* minD)
{
    int prx = round_pred(px), pry = round_pred(py);
    if (prx == 0 && pry == 0) return;  // the search kernel already decided ties with (0,0)
    const int* tab = a.tables + (size_t)k * TAB * TAB;
    if (!(flags & FLAG_DEEP)) {
        constexpr int TW = TIE_RUNS * (int)(sizeof(TieRun) / sizeof(int));
        const int* tree = tab + TIE_ROW * TAB;
        const int t0 = __ldcg(tree + lane);
        const int t1 = lane < TW - 32 ? __ldcg(tree + 32 + lane) : 0;
        tree_pick(t0, t1, prx, pry, mvx, mvy, minD);
        return;
    }
    const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
    int xl, xr, yu, yd, mx, my, md, tie;
    full_range(n, m, a.W, a.H, a.motion_range, xl, xr, yu, yd);
    scan_table(GlobalTab{tab}, xl, xr, yu, yd, prx, pry, lane, &mx, &my, &md, &tie);
    int imv = a.spec_imv[k];
    if (mx != mv_x(imv) || my != mv_y(imv)) {
        if (a.intpel) {  // the integer-pel stage ends at the full-pel winner
            *mvx = 4 * mx;
            *mvy = 4 * my;
            *minD = md;
            return;
        }
        int qmx, qmy;
        subpel_refine_planes(a, n + mx, m + my, load_cur8(a, n, m, lane), lane, &md, &qmx, &qmy);
        *mvx = 4 * mx + qmx;
        *mvy = 4 * my + qmy;
        *minD = md;
    }
}

// Warp-level record lookup: lanes 0..KCACHE-1 each hold one record.
__device__ __forceinline__ bool cache_probe(const int4* c, int key, int lane, int4* rec)
{
    int4 e = lane < KCACHE ? __ldcg(c + lane) : empty_record();
    unsigned hit = __ballot_sync(0xffffffffu, e.x == key);
    if (!hit) return false;
    const int f = __ffs(hit) - 1;
    rec->x = key;
    rec->y = __shfl_sync(0xffffffffu, e.y, f);
    rec->z = __shfl_sync(0xffffffffu, e.z, f);
    rec->w = __shfl_sync(0xffffffffu, e.w, f);
    return true;
}

// The predictor multi-resolution estimators (kEst 1 Ver2, 2 Multires): the
// searched vector and distortion of tie MB k at prediction (px, py): from its
// tie tree, else a kept search whose tie decisions agree, else a new search
// (kept in slots 1..3; slot 0 holds the search at prediction (0, 0)).  One warp.
template <int kEst>
__device__ __noinline__ void pred_search_at(const FullArgs& a, int k, int px, int py, int lane, int* mvx, int* mvy,
                                            int* minD, mrc::Lattice* lt)
{
    if constexpr (kEst == cross::EST_CROSS) {
        // Cross: the tie tree, else a search at the rounded prediction (the
        // only way the prediction enters, MotionEstimatorH264ImplCross.cpp:393-405),
        // cached by it
        int tv, td;
        if (mrc::tie_tree_result(cross::EST_CROSS, static_cast<const mrc::V2TieRun*>(a.tie_runs) +
                                                       (size_t)k * mrc::V2_TIE_RUNS,
                                 px, py, &tv, &td)) {
            *mvx = mv_x(tv);
            *mvy = mv_y(tv);
            *minD = td;
            return;
        }
        const int key = pack_mv(round_pred(px), round_pred(py));
        int4* sc = a.search_cache + (size_t)k * V2_SEARCH_CACHE;
        const int4 e = lane < V2_SEARCH_CACHE ? __ldcg(sc + lane) : make_int4(0, 0, 0, -1);
        const unsigned hit = __ballot_sync(0xffffffffu, e.w >= 0 && e.x == key);
        if (hit) {
            const int f = __ffs(hit) - 1;
            const int v = __shfl_sync(0xffffffffu, e.y, f);
            *mvx = mv_x(v);
            *mvy = mv_y(v);
            *minD = __shfl_sync(0xffffffffu, e.z, f);
            return;
        }
        const cross::CrossResult r =
            cross::cross_search(a, (k % a.cols) * 16, (k / a.cols) * 16, round_pred(px), round_pred(py), lane);
        *mvx = r.mvx;
        *mvy = r.mvy;
        *minD = r.min_d;
        const unsigned slot = 1 + ((unsigned)key * 2654435761u >> 30) % (V2_SEARCH_CACHE - 1);
        if (lane == 0) __stcg(sc + slot, make_int4(key, pack_mv(r.mvx, r.mvy), r.min_d, 1));
        __syncwarp();
        return;
    }
    int tv, td;
    // the Lagrangian overload's search depends on the whole prediction: no tie tree, kept searches by
    // their exact prediction
    if (kEst != mrc::EST_V2_LAMBDA &&
        mrc::tie_tree_result(kEst, static_cast<const mrc::V2TieRun*>(a.tie_runs) + (size_t)k * mrc::V2_TIE_RUNS, px,
                             py, &tv, &td)) {
        *mvx = mv_x(tv);
        *mvy = mv_y(tv);
        *minD = td;
        return;
    }
    int4* sc = a.search_cache + (size_t)k * V2_SEARCH_CACHE;
    const int4 e = lane < V2_SEARCH_CACHE ? __ldcg(sc + lane) : make_int4(0, 0, 0, -1);
    const unsigned hit = __ballot_sync(0xffffffffu, e.w >= 0 && (kEst == mrc::EST_V2_LAMBDA
                                                                     ? e.x == pack_mv(px, py)
                                                                     : mrc::search_reusable(kEst, e.w, mv_x(e.x),
                                                                                            mv_y(e.x), px, py)));
    if (hit) {
        const int f = __ffs(hit) - 1;
        const int v = __shfl_sync(0xffffffffu, e.y, f);
        *mvx = mv_x(v);
        *mvy = mv_y(v);
        *minD = __shfl_sync(0xffffffffu, e.z, f);
        return;
    }
    bool bad = false;
    const mrc::MrcArgs& m = *static_cast<const mrc::MrcArgs*>(a.mrc);
    mrc::Lattice& LT = lt ? *lt : static_cast<mrc::Lattice*>(a.lattice)[k];
    const mrc::MbSearch r = mrc::search_pred<kEst>(m, LT, k / a.cols, k % a.cols, px, py, lane, bad);
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&a.ctrl->status, ST_OUT_OF_BOUNDS);
    *mvx = r.mvx;
    *mvy = r.mvy;
    *minD = r.min_d;
    const unsigned slot = 1 + ((unsigned)pack_mv(px, py) * 2654435761u >> 30) % (V2_SEARCH_CACHE - 1);
    if (lane == 0) __stcg(sc + slot, make_int4(pack_mv(px, py), pack_mv(r.mvx, r.mvy), r.min_d, r.tie));
    __syncwarp();
}

// Per-warp shared sub-pel lattices for the predictor estimators' searches at
// a prediction (8 warps per block); none for the full-search estimator.  The
// wavefront, which evaluates rarely, uses the per-MB scratch in global memory.
template <int kEst>
struct LatticeSlots {
    __device__ static mrc::Lattice* get(int warp)
    {
        __shared__ mrc::Lattice slots[8];
        return &slots[warp];
    }
};
template <>
struct LatticeSlots<0> {
    __device__ static mrc::Lattice* get(int) { return nullptr; }
};
template <>
struct LatticeSlots<cross::EST_CROSS> {
    __device__ static mrc::Lattice* get(int) { return nullptr; }
};

// Full evaluation of MB k for raw prediction (px, py), one warp: the record
// {prediction, distortion at it, final vector, final distortion}.  kEst 0:
// MotionEstimatorH264ImplFull, a tie MB's scan from its table / tie tree;
// kEst 1: MotionEstimatorH264ImplMultiresCrossVer2, whose searched result
// (at prediction (0, 0)) holds for any prediction unless the search met a
// tie; for such an MB the search at the prediction's level vectors
// (…MultiresCrossVer2.cpp:627-642) comes from pred_search_at.  kEst 2:
// MotionEstimatorH264ImplMultires, the same with its own search.  kEst 3:
// MotionEstimatorH264ImplCross, the same with its search at the rounded
// prediction, the 64-point path distortion and norm 64.  kEst 4: Ver2's
// Lagrangian overload (…MultiresCrossVer2.cpp:1162-1742), every MB searched at
// its prediction (mrc::search_lambda), the final choice with the caller's
// lambda.
template <int kEst>
__device__ __noinline__ int4 evaluate(const FullArgs& a, int k, int px, int py, int lane, mrc::Lattice* lt = nullptr)
{
    const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
    const PredGeom g = pred_geom(n, m, a.W, a.H, px, py);
    const int4 sp = a.spec4[k];  // loads of spec and planes are independent: one round trip
    int pd;
    if constexpr (kEst == cross::EST_CROSS) pd = cross::path_pred_distortion(a, n, m, g, lane);
    else pd = plane_pred_distortion(a, n, m, g, lane);
    int mvx = mv_x(sp.x), mvy = mv_y(sp.x), minD = sp.y;
    const int zd = sp.z;
    if constexpr (kEst == 0) {
        if ((sp.w & FLAG_TIE) && (round_pred(px) != 0 || round_pred(py) != 0))
            tie_path(a, k, px, py, sp.w, lane, &mvx, &mvy, &minD);
    } else {
        if (sp.w & FLAG_TIE) pred_search_at<kEst>(a, k, px, py, lane, &mvx, &mvy, &minD, lt);
    }
    const int pos = best_of3_fast(mvx, mvy, minD, g.pcx, g.pcy, pd, zd, a.lambda, g.pcx, g.pcy,
                                  kEst == cross::EST_CROSS ? cross::PATH_NORM : 256);
    int4 rec;
    rec.x = pack_mv(px, py);
    rec.y = pd;
    if (pos == 0) {
        rec.z = pack_mv(mvx, mvy);
        rec.w = minD;
    } else if (pos == 1) {
        rec.z = pack_mv(g.pcx, g.pcy);
        rec.w = pd;
    } else {
        rec.z = pack_mv(0, 0);
        rec.w = zd;
    }
    return rec;
}

// ---------------------------------------------------------------------------
template <int kEst>
__global__ void __launch_bounds__(256, 4) k_full_sweep0(FullArgs a)
{
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int k = blockIdx.x * 8 + wib;
    if (k >= a.nmb) return;
    int px, py;
    median_pred(a.final_mv, a.spec4[k].w, k, a.cols, &px, &py);
    const int4 rec = evaluate<kEst>(a, k, px, py, lane, LatticeSlots<kEst>::get(wib));
    if (lane < KCACHE) __stcg(a.cache + (size_t)k * KCACHE + lane, lane == 0 ? rec : empty_record());
    if (lane == 0) {
        a.pred_used[k] = rec.x;
        a.final_dist[k] = rec.w;
        __stcg(a.final_mv + k, rec.z);
    }
}

// ---------------------------------------------------------------------------
// The MBs whose median prediction reads MB k (left of the right neighbour,
// above of the MB below, above-right of the MB below-left, above-left of the
// MB below-right), set in a bitmap of one bit per MB.
__device__ __forceinline__ void mark_dependents(const FullArgs& a, int k, unsigned* bits)
{
    const int cols = a.cols, rows = a.nmb / cols, r = k / cols, c = k - r * cols;
    auto set = [&](int j) { atomicOr(bits + (j >> 5), 1u << (j & 31)); };
    if (c + 1 < cols) set(k + 1);
    if (r + 1 < rows) {
        set(k + cols);
        if (c > 0) set(k + cols - 1);
        if (c + 1 < cols) set(k + cols + 1);
    }
}

// State of the relaxation before sweep `upto` from the change counts of sweeps
// 1 .. upto-1: s > 0 when sweep s changed nothing (the fixed point), -1 when
// more than a few MBs still change and the counts stopped falling fast enough
// to reach zero within `limit` sweeps (they fall about geometrically while
// copy chains shorten; a ratio above 7/8, or a projection past the limit,
// gives up to the wavefront), 0 while
// the sweeps go on.  The sweep kernels and the outcome kernel evaluate the
// same counts with this one function, so they agree.
__device__ __forceinline__ int relax_status(const int* changed, int upto, int limit)
{
    int prev = 0;
    for (int s = 1; s < upto; s++) {
        const int c = *((const volatile int*)&changed[s]);
        if (c == 0) return s;
        if (s >= 3 && c > 32) {  // a few changes settle within a sweep or two: never give up on them
            const float r = (float)c / (float)prev;
            if (r >= 0.875f) return -1;
            if ((float)s + logf((float)c + 1.0f) / -logf(r) > (float)limit + 1.0f) return -1;
        }
        prev = c;
    }
    return 0;
}

constexpr int kHist = 4096;  // dictionary histogram slots
struct RelaxSmem {
    union {
        struct {
            int keys[kHist];
            int counts[kHist];
        } hist;
    } u;
    long long red_total[8];
    int red_count[8];
    int red_key[8];
    int red_val[8];
};

// One relaxation sweep: lane per MB (MBs gwarp + lane*nwarps ...) to find the
// MBs whose prediction moved, then the warp on each.  Skipped once an earlier
// sweep changed no vector (the fixed point is reached).
template <int kEst>
__global__ void __launch_bounds__(256, 4) k_full_relax_sweep(FullArgs a, int sweep, int mark)
{
    if (relax_status(a.changed, sweep, a.relax_sweeps) != 0) return;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gwarp = blockIdx.x * 8 + wib, nwarps = gridDim.x * 8;
    int changed = 0;
    for (int base = gwarp; base < a.nmb; base += 32 * nwarps) {
        const int k = base + lane * nwarps;
        int px = 0, py = 0, key = 0;
        bool moved = false;
        if (k < a.nmb) {
            median_pred(a.final_mv, __ldcg(&a.spec4[k].w), k, a.cols, &px, &py);
            key = pack_mv(px, py);
            moved = __ldcg(a.pred_used + k) != key;
        }
        unsigned todo = __ballot_sync(0xffffffffu, moved);
        while (todo) {
            const int f = __ffs(todo) - 1;
            todo &= todo - 1;
            const int kk = base + f * nwarps, fkey = __shfl_sync(0xffffffffu, key, f);
            const int fx = __shfl_sync(0xffffffffu, px, f), fy = __shfl_sync(0xffffffffu, py, f);
            int4* cache = a.cache + (size_t)kk * KCACHE;
            int4 rec;
            const bool hit = cache_probe(cache, fkey, lane, &rec);
            if (!hit) rec = evaluate<kEst>(a, kk, fx, fy, lane, LatticeSlots<kEst>::get(wib));
            if (lane == 0) {
                atomicAdd(&a.ctrl->relax_evals, 1);
                if (!hit) {
                    atomicAdd(&a.ctrl->relax_miss, 1);
                    __stcg(cache + kCacheRelax + (sweep % 3), rec);
                }
                __stcg(a.pred_used + kk, fkey);
                a.final_dist[kk] = rec.w;
                if (__ldcg(a.final_mv + kk) != rec.z) {
                    __stcg(a.final_mv + kk, rec.z);
                    changed++;
                    if (mark) mark_dependents(a, kk, a.dirty);
                }
            }
            __syncwarp();
        }
    }
    if (lane == 0 && changed) atomicAdd(&a.changed[sweep], changed);
}

// The remaining sweeps (3 ..) by one block: only the MBs whose prediction
// inputs changed in the previous sweep (dependents of changed MBs, kept as
// bitmaps in shared memory) are visited, 32 warps at a time, with a block
// barrier between sweeps.  A frame that settled in the grid sweeps costs one
// short launch here instead of a grid launch per remaining sweep.
template <int kEst>
__global__ void __launch_bounds__(1024, 1) k_full_relax_tail(FullArgs a, int first)
{
    extern __shared__ unsigned tail_bits[];  // current and next dirty sets, one bit per MB
    __shared__ int s_changed;
    if (relax_status(a.changed, first, a.relax_sweeps) != 0) return;
    const int words = (a.nmb + 31) >> 5;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned* cur = tail_bits;
    unsigned* nxt = tail_bits + words;
    for (int i = threadIdx.x; i < words; i += blockDim.x) {
        cur[i] = __ldcg(a.dirty + i);
        nxt[i] = 0u;
    }
    __syncthreads();
    for (int sweep = first; sweep <= a.relax_sweeps; sweep++) {
        if (threadIdx.x == 0) s_changed = 0;
        __syncthreads();
        int changes = 0;
        for (int w = wib; w < words; w += nw) {
            unsigned bits = cur[w];
            while (bits) {
                const int k = 32 * w + __ffs(bits) - 1;
                bits &= bits - 1;
                int px, py;
                median_pred(a.final_mv, __ldcg(&a.spec4[k].w), k, a.cols, &px, &py);
                const int key = pack_mv(px, py);
                if (__ldcg(a.pred_used + k) == key) continue;
                int4* cache = a.cache + (size_t)k * KCACHE;
                int4 rec;
                const bool hit = cache_probe(cache, key, lane, &rec);
                if (!hit) rec = evaluate<kEst>(a, k, px, py, lane, nullptr);
                if (lane == 0) {
                    atomicAdd(&a.ctrl->relax_evals, 1);
                    if (!hit) {
                        atomicAdd(&a.ctrl->relax_miss, 1);
                        __stcg(cache + kCacheRelax + (sweep % 3), rec);
                    }
                    __stcg(a.pred_used + k, key);
                    a.final_dist[k] = rec.w;
                    if (__ldcg(a.final_mv + k) != rec.z) {
                        __stcg(a.final_mv + k, rec.z);
                        changes++;
                        mark_dependents(a, k, nxt);
                    }
                }
                __syncwarp();
            }
        }
        if (lane == 0 && changes) atomicAdd(&s_changed, changes);
        __syncthreads();
        for (int i = threadIdx.x; i < words; i += blockDim.x) cur[i] = 0u;
        if (threadIdx.x == 0) a.changed[sweep] = s_changed;
        __syncthreads();
        unsigned* t = cur;
        cur = nxt;
        nxt = t;
        if (relax_status(a.changed, sweep + 1, a.relax_sweeps) != 0) break;
    }
}

// After the sweeps: a sweep that changed nothing means the vectors are the
// sequential result -- every block writes its MBs' outputs and adds their
// included distortions; otherwise block 0 finds the frame's dominant vectors
// for the wavefront's records.
__global__ void __launch_bounds__(256) k_full_relax_outcome(FullArgs a)
{
    __shared__ RelaxSmem S;
    const int status = relax_status(a.changed, a.relax_sweeps + 1, a.relax_sweeps);
    const int sweeps = status > 0 ? status : 0;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    if (sweeps) {
        long long tot = 0;
        int cnt = 0;
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.nmb; k += gridDim.x * blockDim.x) {
            const int fmv = __ldcg(a.final_mv + k);
            a.job->out_mv[k] = fmv;
            const int d = a.final_dist[k];
            if (a.job->out_dist) a.job->out_dist[k] = d;
            if (a.job->incl && a.job->incl[k]) {
                tot += d;
                cnt++;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        if (lane == 0 && cnt) {
            atomicAdd(reinterpret_cast<unsigned long long*>(&a.ctrl->total), (unsigned long long)tot);
            atomicAdd(&a.ctrl->count, cnt);
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            a.ctrl->sweeps = sweeps;
            a.ctrl->converged = 1;
        }
        return;
    }
    if (blockIdx.x != 0) return;
    for (int i = threadIdx.x; i < kHist; i += blockDim.x) {
        S.u.hist.keys[i] = kEmpty;
        S.u.hist.counts[i] = 0;
    }
    __syncthreads();
    for (int base = 0; base < a.nmb; base += 8 * blockDim.x) {  // uniform trip count: every lane shuffles
        const int k0 = base + threadIdx.x;
        int vals[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {  // eight loads in flight per thread
            const int k = k0 + u * blockDim.x;
            vals[u] = k < a.nmb ? __ldcg(a.final_mv + k) : kEmpty;
        }
#pragma unroll
        for (int u = 0; u < 8; u++) {
            // one insert per distinct vector of the warp (a pan makes most vectors equal:
            // per-lane atomics on one slot would serialise)
            const int v = vals[u];
            const unsigned same = __match_any_sync(0xffffffffu, v);
            if (v == kEmpty || (__ffs(same) - 1) != (int)(threadIdx.x & 31)) continue;
            // counts only steer which records are precomputed: a vector that finds
            // no slot within a few probes (frames with thousands of distinct
            // vectors) is left out
            unsigned h = ((unsigned)v * 2654435761u) >> 20;  // 12 bits
            for (int probe = 0; probe < 8; probe++) {
                int slot = (h + probe) & (kHist - 1);
                int prev = atomicCAS(&S.u.hist.keys[slot], kEmpty, v);
                if (prev == kEmpty || prev == v) {
                    atomicAdd(&S.u.hist.counts[slot], __popc(same));
                    break;
                }
            }
        }
    }
    __syncthreads();
    for (int d = 0; d < NDICT; d++) {
        int best_c = 0, best_k = kEmpty;
        for (int i = threadIdx.x; i < kHist; i += blockDim.x)
            if (S.u.hist.counts[i] > best_c) {
                best_c = S.u.hist.counts[i];
                best_k = i;
            }
        for (int o = 16; o > 0; o >>= 1) {
            int oc = __shfl_xor_sync(0xffffffffu, best_c, o), ok2 = __shfl_xor_sync(0xffffffffu, best_k, o);
            if (oc > best_c || (oc == best_c && ok2 < best_k)) {
                best_c = oc;
                best_k = ok2;
            }
        }
        if (lane == 0) {
            S.red_val[wib] = best_c;
            S.red_key[wib] = best_k;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int bc = 0, bk = kEmpty;
            for (int w = 0; w < 8; w++)
                if (S.red_val[w] > bc || (S.red_val[w] == bc && S.red_key[w] < bk)) {
                    bc = S.red_val[w];
                    bk = S.red_key[w];
                }
            a.dict[d] = bc > 0 ? S.u.hist.keys[bk] : kEmpty;
            if (bc > 0) S.u.hist.counts[bk] = 0;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) a.ctrl->sweeps = a.relax_sweeps;
}

// ---------------------------------------------------------------------------
// One warp per MB: records at every dictionary vector the MB's cache lacks.
template <int kEst>
__global__ void __launch_bounds__(256, 2) k_full_precompute(FullArgs a)
{
    if (*((volatile int*)&a.ctrl->converged)) return;
    __shared__ int dict[NDICT];
    if (threadIdx.x < NDICT) dict[threadIdx.x] = a.dict[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (int k = blockIdx.x * 8 + wib; k < a.nmb; k += gridDim.x * 8) {
        int4* cache = a.cache + (size_t)k * KCACHE;
        const int4 mine = __ldcg(cache + lane);
        for (int d = 0; d < NDICT; d++) {
            const int v = dict[d];
            if (v == kEmpty || __any_sync(0xffffffffu, mine.x == v)) continue;
            const int4 rec = evaluate<kEst>(a, k, mv_x(v), mv_y(v), lane, LatticeSlots<kEst>::get(wib));
            if (lane == 0) __stcg(cache + kCacheDict + d, rec);
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------------------
// Neighbour closure, one warp per MB.  The prediction of MB k is the median
// of the final vectors of A, B and C (or D); each of those is one of a few
// values: its current vector, its searched vector, zero, or the outcome of
// one of its records.  Medians of those per-neighbour sets, taken in order of
// plausibility (index sum), that MB k has no record for yet become records
// 12..31, evaluated here.  Then MB k's wavefront record is written.
// Wavefront record hashing: a prediction whose halves fit in signed 11 bits
// encodes to 22 bits; two distinct buckets of 4 per encoding.
__device__ __forceinline__ bool wave_encode(int key, unsigned* e)
{
    const int x = mv_x(key), y = mv_y(key);
    *e = (unsigned)(x & 0x7ff) | ((unsigned)(y & 0x7ff) << 11);
    return (unsigned)(x + 1024) < 2048u && (unsigned)(y + 1024) < 2048u;
}
__device__ __forceinline__ void wave_buckets(unsigned e, int* h1, int* h2)
{
    *h1 = (int)((e * 0x9e3779b1u) >> 28);
    *h2 = *h1 ^ (1 + (int)((e * 0xc2b2ae3du) >> 29));  // differs from h1
}

// Index triples (ia, ib, ic) < kSetMax^3 by index sum, then lexicographic,
// packed as ia | ib << 3 | ic << 6.
constexpr int kCombos = kSetMax * kSetMax * kSetMax;
struct ClosureOrder {
    short v[kCombos];
};
constexpr ClosureOrder make_closure_order()
{
    ClosureOrder o{};
    int n = 0;
    for (int sum = 0; sum <= 3 * (kSetMax - 1); sum++)
        for (int ia = 0; ia < kSetMax; ia++)
            for (int ib = 0; ib < kSetMax; ib++) {
                const int ic = sum - ia - ib;
                if (ic >= 0 && ic < kSetMax) o.v[n++] = (short)(ia | (ib << 3) | (ic << 6));
            }
    return o;
}
__constant__ const ClosureOrder kClosureOrder = make_closure_order();

struct ClosureSmem {
    unsigned tab[8][64];
    int cnt[8][16];
    int set[8][3][kSetMax];
    int nset[8][3];
    int fresh[8][KCACHE - kCacheClosure];
};

// Ordered, de-duplicated possible final vectors of MB x into set[0..n).
__device__ __forceinline__ int neighbour_set(const FullArgs& a, int x, int lane, int* set)
{
    int v = kEmpty;
    if (lane == 0) v = __ldcg(a.final_mv + x);
    else if (lane == 1) v = __ldcg(&a.spec4[x].x);
    else if (lane == 2) v = 0;
    else if (lane < 3 + kCacheClosure) {
        const int4 r = __ldcg(a.cache + (size_t)x * KCACHE + (lane - 3));
        if (r.x != kEmpty) v = r.z;
    }
    const bool valid = v != kEmpty;
    const unsigned vm = __ballot_sync(0xffffffffu, valid);
    const unsigned same = __match_any_sync(0xffffffffu, v);
    const bool keep = valid && (__ffs(same) - 1) == lane;
    const unsigned km = __ballot_sync(0xffffffffu, keep);
    const int rank = __popc(km & ((1u << lane) - 1u));
    if (keep && rank < kSetMax) set[rank] = v;
    (void)vm;
    __syncwarp();
    return min(__popc(km), kSetMax);
}

template <int kEst>
__global__ void __launch_bounds__(256, kEst == 0 ? 3 : 2) k_full_closure(FullArgs a)
{
    if (*((volatile int*)&a.ctrl->converged)) return;
    __shared__ ClosureSmem S;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int cols = a.cols, rows = a.nmb / cols;
    for (int k = blockIdx.x * 8 + wib; k < a.nmb; k += gridDim.x * 8) {
        int4* cache = a.cache + (size_t)k * KCACHE;
        int4 mine = __ldcg(cache + lane);
        const int av = __ldcg(&a.spec4[k].w);
        // neighbour sets (an unavailable neighbour contributes zero, as in the median)
        const int r = k / cols, c = k - r * cols;
        (void)rows;
        const int nb[3] = {(av & AV_A) ? k - 1 : -1, (av & AV_B) ? k - cols : -1,
                           (av & AV_C) ? k - cols + 1 : ((av & AV_D) ? k - cols - 1 : -1)};
        for (int s = 0; s < 3; s++) {
            if (nb[s] >= 0) {
                const int n = neighbour_set(a, nb[s], lane, S.set[wib][s]);
                if (lane == 0) S.nset[wib][s] = n;
            } else if (lane == 0) {
                S.set[wib][s][0] = 0;
                S.nset[wib][s] = 1;
            }
        }
        __syncwarp();
        if (!(av & AV_B) && !(av & AV_C)) {
            // neither above nor above-right: B and C take A (median_from)
            for (int i = lane; i < kSetMax; i += 32) S.set[wib][1][i] = S.set[wib][2][i] = S.set[wib][0][i];
            if (lane == 0) S.nset[wib][1] = S.nset[wib][2] = S.nset[wib][0];
            __syncwarp();
        }
        const int nA = S.nset[wib][0], nB = S.nset[wib][1], nC = S.nset[wib][2];
        // combinations by index sum, 32 at a time
        int fresh = 0;
        for (int base = 0; base < kCombos && fresh < KCACHE - kCacheClosure; base += 32) {
            const int idx = base + lane;
            int ia = 0, ib = 0, ic = 0;
            bool ok = false;
            if (idx < kCombos) {
                const int code = kClosureOrder.v[idx];
                ia = code & 7;
                ib = (code >> 3) & 7;
                ic = (code >> 6) & 7;
                ok = ia < nA && ib < nB && ic < nC;
            }
            if (!__any_sync(0xffffffffu, ok)) continue;
            int key = kEmpty;
            if (ok) {
                const int A = S.set[wib][0][ia], B = S.set[wib][1][ib], C = S.set[wib][2][ic];
                key = pack_mv(median3(mv_x(A), mv_x(B), mv_x(C)), median3(mv_y(A), mv_y(B), mv_y(C)));
            }
            // new: not among the MB's records (including those added so far), first of its kind in the batch
            bool dup = !ok;
            for (int e = 0; e < KCACHE; e++) dup |= __shfl_sync(0xffffffffu, mine.x, e) == key;
            const unsigned same = __match_any_sync(0xffffffffu, key);
            const bool take = !dup && (__ffs(same) - 1) == lane;
            const unsigned tm = __ballot_sync(0xffffffffu, take);
            const int slot = fresh + __popc(tm & ((1u << lane) - 1u));
            if (take && slot < KCACHE - kCacheClosure) S.fresh[wib][slot] = key;
            __syncwarp();
            const int added = min(__popc(tm), KCACHE - kCacheClosure - fresh);
            if (lane >= kCacheClosure + fresh && lane < kCacheClosure + fresh + added)
                mine.x = S.fresh[wib][lane - kCacheClosure];
            fresh += added;
            __syncwarp();
        }
        // evaluate the new records
        for (int i = 0; i < fresh; i++) {
            const int key = S.fresh[wib][i];
            const int4 rec = evaluate<kEst>(a, k, mv_x(key), mv_y(key), lane, LatticeSlots<kEst>::get(wib));
            if (lane == kCacheClosure + i) mine = rec;
        }
        if (lane >= kCacheClosure) {
            if (lane < kCacheClosure + fresh) __stcg(cache + lane, mine);
        }
        // the wavefront record: entries hashed into 16 buckets of 4, each to
        // the emptier of its two buckets, in slot order (a record that does not
        // fit, or whose outcome is a clamped prediction, is left out: the
        // wavefront then evaluates that prediction itself)
        const int spec = __ldcg(&a.spec4[k].x);
        unsigned entry = 0xffffffffu;
        int h1 = 0, h2 = 0;
        if (mine.x != kEmpty) {
            const int code = mine.z == spec ? 0 : (mine.z == mine.x ? 1 : (mine.z == 0 ? 2 : 3));
            unsigned e;
            if (code < 3 && wave_encode(mine.x, &e)) {
                entry = e | ((unsigned)code << 22);
                wave_buckets(e, &h1, &h2);
            }
        }
        unsigned* tab = S.tab[wib];
        int* cnt = S.cnt[wib];
        tab[lane] = 0xffffffffu;
        tab[lane + 32] = 0xffffffffu;
        if (lane < 16) cnt[lane] = 0;
        __syncwarp();
        for (int i = 0; i < 32; i++) {
            if (lane == i && entry != 0xffffffffu) {
                const int c1 = cnt[h1], c2 = cnt[h2];
                const int b = c1 <= c2 ? h1 : h2, cb = c1 <= c2 ? c1 : c2;
                if (cb < 4) {
                    tab[4 * b + cb] = entry;
                    cnt[b] = cb + 1;
                }
            }
            __syncwarp();
        }
        WaveRec* wr = a.wave_rec + wave_rec_index(cols, r, c);
        reinterpret_cast<uint2*>(wr->slot)[lane] = make_uint2(tab[2 * lane], tab[2 * lane + 1]);
        if (lane == 0) {
            wr->spec = spec;
            wr->av = av;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Exact order, one CTA per group of up to WAVE_WARPS bands of 32 rows.
// Lane l of warp w owns row 32(band0+w) + l and handles column t - 2l at step
// t: its left neighbour is its own previous output, above / above-right /
// above-left are lane l-1's outputs of steps t-2, t-1 and t-3 (shuffles), so
// a warp advances 32 rows in lock step with no synchronisation.  Lane 0 takes
// the row above from warp w-1's lane 31 through shared memory, where each
// vector is its own flag (the array starts as kEmpty, which no vector packs
// to), or, for the first band of a launch, from the vectors the previous
// launch stored.  The 32 wavefront records of a step are contiguous (diagonal
// layout) and arrive by one bulk copy, kRing-1 steps ahead.  A step is a
// median, 32 key compares and, only for a lane whose prediction is in none of
// its records, a full evaluation by the whole warp.
constexpr int kWaveMaxWarps = WAVE_WARPS;
constexpr unsigned kWaveStepBytes = 32 * sizeof(WaveRec);

template <int kChunk, int kEst>
__global__ void __launch_bounds__(kWaveMaxWarps * 32, 1) k_full_wave(FullArgs a, int band0, int last)
{
    if (*((volatile int*)&a.ctrl->converged)) return;
    extern __shared__ __align__(16) unsigned char wave_smem[];
    const int cols = a.cols, rows = a.nmb / a.cols, nw = blockDim.x >> 5;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // per warp: two buffers of kChunk steps (32 records a step), a barrier each
    WaveRec* ring = reinterpret_cast<WaveRec*>(wave_smem);                                // [nw][2][kChunk][32]
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(ring + nw * 2 * kChunk * 32);  // [nw][2]
    volatile int* edge = reinterpret_cast<int*>(bars + nw * 2);                           // [nw][cols]
    __shared__ int abort_flag;
    for (int i = threadIdx.x; i < nw * cols; i += blockDim.x) edge[i] = kEmpty;
    if (threadIdx.x < nw * 2) mbar_init(bars + threadIdx.x, 1);
    if (threadIdx.x == 0) abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    __syncthreads();

    const int band = band0 + w;
    const int r = 32 * band + lane;
    const bool row_ok = r < rows;
    const int lanes_used = min(32, rows - 32 * band);
    const int nsteps = cols + 2 * (lanes_used - 1);
    const int nchunks = (nsteps + kChunk - 1) / kChunk;
    const WaveRec* src = a.wave_rec + (size_t)band * (cols + 62) * 32;  // step t: src[32t .. 32t+31]
    WaveRec* mybuf = ring + w * 2 * kChunk * 32;
    unsigned long long* mybars = bars + w * 2;
    const volatile int* above = edge + (w - 1) * cols;                 // lane 0 of warps > 0
    const int* above_g = a.final_mv + (size_t)(32 * band - 1) * cols;  // lane 0 of warp 0 when band0 > 0

    auto issue = [&](int ci) {  // chunk ci into buffer ci & 1 (lane 0)
        const int steps = min(kChunk, nsteps - ci * kChunk);
        const unsigned bytes = (unsigned)steps * kWaveStepBytes;
        mbar_expect_tx(mybars + (ci & 1), bytes);
        bulk_load(mybuf + (ci & 1) * kChunk * 32, src + (size_t)ci * kChunk * 32, bytes, mybars + (ci & 1));
    };
    if (lane == 0) {
        issue(0);
        if (nchunks > 1) issue(1);
    }
    int issued = min(2, nchunks), consumed = 0;  // chunks of this warp
    // o1: this lane's output of step t-1 (its left neighbour at step t); s1, s2, s3: lane l-1's outputs of
    // steps t-1, t-2, t-3 (above-right, above, above-left at step t), received one shuffle per step
    int o1 = 0, s1 = 0, s2 = 0, s3 = 0;
    int pb = 0, pc = 0;          // lane 0: row above at columns c-1 and c (previous step's B and C)
    int misses = 0;
    bool stop = false;
    for (int t = 0; t < nsteps; t++) {
        const int ci = t / kChunk, ti = t - ci * kChunk;
        if (ti == 0) {
            long long it = 0;
            while (!mbar_try_wait(mybars + (ci & 1), (unsigned)(ci >> 1) & 1u))
                if (++it > a.spin_limit) {
                    stop = true;
                    break;
                }
            // a wait that ran out here, or lane 0's wait on the row above in the last chunk
            if (__any_sync(0xffffffffu, stop || *((volatile int*)&abort_flag))) {
                if (lane == 0) {
                    abort_flag = 1;
                    atomicOr(&a.ctrl->status, ST_TIMEOUT);
                }
                break;
            }
            consumed = ci + 1;
            // the other buffer held chunk ci-1, finished: refill it with chunk ci+1
            if (ci >= 1 && ci + 1 < nchunks) {
                if (lane == 0) issue(ci + 1);
                issued++;
            }
        }
        const int c = t - 2 * lane;
        const bool active = row_ok && c >= 0 && c < cols;
        const WaveRec& rec = mybuf[((ci & 1) * kChunk + ti) * 32 + lane];
        int B = s2, C = s1, D = s3;
        if (w > 0) {
            if (lane == 0 && active) {
                // warp w-1's lane 31 stores the row above: only column c+1 is new.  A wait that runs
                // out leaves this step's neighbours as they are (indices do not depend on them) and
                // ends the warp at the next chunk boundary.
                if (c == 0) {
                    long long it = 0;
                    while ((pc = above[0]) == kEmpty)
                        if (++it > a.spin_limit || *((volatile int*)&abort_flag)) {
                            stop = true;
                            abort_flag = 1;
                            break;
                        }
                    pb = 0;
                }
                int nc = 0;
                if (c + 1 < cols) {
                    long long it = 0;
                    while ((nc = above[c + 1]) == kEmpty)
                        if (++it > a.spin_limit || *((volatile int*)&abort_flag)) {
                            stop = true;
                            abort_flag = 1;
                            break;
                        }
                }
                D = pb;
                B = pc;
                C = nc;
                pb = pc;
                pc = nc;
            }
        } else if (band0 > 0 && lane == 0 && active) {
            B = __ldcg(above_g + c);
            C = c + 1 < cols ? __ldcg(above_g + c + 1) : 0;
            D = c >= 1 ? __ldcg(above_g + c - 1) : 0;
        }
        // the record lookup, straight-line in every lane (an inactive lane's record slot holds data of
        // some step, its result is not stored)
        const int key = median_packed(rec.av, o1, B, C, D);
        unsigned e;
        const bool inr = wave_encode(key, &e);
        int h1, h2;
        wave_buckets(e, &h1, &h2);
        const uint4 b1 = reinterpret_cast<const uint4*>(rec.slot)[h1];
        const uint4 b2 = reinterpret_cast<const uint4*>(rec.slot)[h2];
        // a table holds each prediction once: the matching entry's code + 1, else 0
        const unsigned m = 0xff3fffffu;
        auto code1 = [&](unsigned v) { return (v & m) == e ? ((v >> 22) & 3u) + 1u : 0u; };
        const unsigned k1 = max(max(code1(b1.x), code1(b1.y)), max(code1(b1.z), code1(b1.w)));
        const unsigned k2 = max(max(code1(b2.x), code1(b2.y)), max(code1(b2.z), code1(b2.w)));
        const unsigned k = max(k1, k2);
        const bool hit = inr && k != 0u;
        int out = k == 1u ? rec.spec : (k == 2u ? key : 0);
        unsigned miss = __ballot_sync(0xffffffffu, active && !hit);
        if (miss) {
            misses += __popc(miss);
            do {
                const int f = __ffs(miss) - 1;
                miss &= miss - 1;
                const int fkey = __shfl_sync(0xffffffffu, key, f);
                const int fk = (32 * band + f) * cols + (t - 2 * f);
                int4 rv;
                if constexpr (kEst == mrc::EST_V2_LAMBDA) {
                    // a full search per miss: first the MB's records of this estimate (their final
                    // vectors are searched ones, which the wavefront table leaves out)
                    const int4 cr = __ldcg(a.cache + (size_t)fk * KCACHE + lane);
                    const unsigned ch = __ballot_sync(0xffffffffu, cr.x == fkey);
                    if (ch) {
                        const int src = __ffs(ch) - 1;
                        rv = make_int4(fkey, 0, __shfl_sync(0xffffffffu, cr.z, src),
                                       __shfl_sync(0xffffffffu, cr.w, src));
                    } else {
                        rv = evaluate<kEst>(a, fk, mv_x(fkey), mv_y(fkey), lane);
                    }
                } else {
                    rv = evaluate<kEst>(a, fk, mv_x(fkey), mv_y(fkey), lane);
                }
                if (lane == f) {
                    out = rv.z;
                    a.final_mv[fk] = rv.z;
                    a.final_dist[fk] = rv.w;
                }
            } while (miss);
        }
        if (active) {
            a.wave_choice[r * cols + c] = hit ? key : kEmpty;
            if (lane == 31) {
                edge[w * cols + c] = out;
                a.final_mv[r * cols + c] = out;  // the next launch's first band reads this row
            }
        }
        o1 = out;
        s3 = s2;
        s2 = s1;
        s1 = __shfl_up_sync(0xffffffffu, out, 1);
    }
    // copies still in flight after an abort land before the CTA leaves; a
    // drain that gives up (only after a timeout) is reported as one too
    for (int ci = consumed; ci < issued; ci++) {
        long long it = 0;
        while (!mbar_try_wait(mybars + (ci & 1), (unsigned)(ci >> 1) & 1u))
            if (++it > a.spin_limit) {
                atomicOr(&a.ctrl->status, ST_TIMEOUT);
                break;
            }
    }
    if (lane == 0 && misses) atomicAdd(&a.ctrl->wave_miss, misses);
    __syncthreads();
    if (threadIdx.x == 0 && !abort_flag && last) a.ctrl->sweeps = a.relax_sweeps + 1000;
}

// Outputs of a wavefront-resolved frame, one thread per MB: the record each
// MB took (or the vector and distortion the wavefront evaluated), and the
// included-distortion average (Full.cpp:581-611).
__global__ void __launch_bounds__(256) k_full_wave_outputs(FullArgs a)
{
    if (*((volatile int*)&a.ctrl->converged) || (*((volatile int*)&a.ctrl->status) & ST_TIMEOUT)) return;
    long long tot = 0;
    int cnt = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.nmb; k += gridDim.x * blockDim.x) {
        const int key = a.wave_choice[k];
        int fmv = 0, d = 0;
        if (key != kEmpty) {
            const int4* cache = a.cache + (size_t)k * KCACHE;
            for (int e = 0; e < KCACHE; e++) {
                const int4 rec = __ldcg(cache + e);
                if (rec.x == key) {
                    fmv = rec.z;
                    d = rec.w;
                    break;
                }
            }
        } else {
            fmv = a.final_mv[k];
            d = a.final_dist[k];
        }
        a.final_mv[k] = fmv;
        a.final_dist[k] = d;
        a.job->out_mv[k] = fmv;
        if (a.job->out_dist) a.job->out_dist[k] = d;
        if (a.job->incl && a.job->incl[k]) {
            tot += d;
            cnt++;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        tot += __shfl_xor_sync(0xffffffffu, tot, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0 && cnt) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&a.ctrl->total), (unsigned long long)tot);
        atomicAdd(&a.ctrl->count, cnt);
    }
}

// The included-distortion average, once every output block has added its sums.
__global__ void k_full_average(FullArgs a)
{
    if (*((volatile int*)&a.ctrl->status) & ST_TIMEOUT) return;
    const long long t = a.ctrl->total;
    const int c = a.ctrl->count;
    if (a.job->out_avg) *a.job->out_avg = c ? t / c : 0;
}

// The integer-pel SAD stage's tail.  The prediction enters only the exact-tie
// decisions of the scan (MotionEstimatorH264ImplFull.cpp:424-441), so every
// macroblock without a tie already holds its final vector.  One CTA walks the
// anti-diagonals t = c + 2r: the median prediction of (r, c) reads (r, c-1),
// (r-1, c-1), (r-1, c) and (r-1, c+1), all on earlier diagonals, so a
// diagonal's tie macroblocks settle together (warp each: tie tree walk, or a
// rescan of the kept table), with a block barrier between diagonals.  Then the
// outputs and the included-distortion average (Full.cpp:581-607).
constexpr int kSadWaveWords = 64;   // one bit per diagonal: 2048 >= cols + 2 rows - 1 at 8192 x 8192
constexpr int kSadSmemMbs = 16384;  // final vectors kept in shared memory up to this many macroblocks

size_t sad_resolve_smem(int nmb)
{
    const size_t words = (size_t)(nmb + 31) / 32;
    return 4 * (words + (nmb <= kSadSmemMbs ? (size_t)nmb : 0));
}

__global__ void __launch_bounds__(1024, 1) k_sad_resolve(FullArgs a)
{
    extern __shared__ unsigned s_dyn[];  // tie bit per macroblock, then (local) the final vectors
    __shared__ long long s_tot;
    __shared__ int s_cnt;
    __shared__ unsigned s_wave[kSadWaveWords];  // diagonals holding a tie macroblock
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int cols = a.cols, rows = a.nmb / cols, words = (a.nmb + 31) >> 5;
    const int ntie = *((volatile int*)&a.ctrl->ntie);
    const int waves = cols + 2 * (rows - 1);
    const bool every = waves > 32 * kSadWaveWords;
    const bool local = a.nmb <= kSadSmemMbs;
    unsigned* s_tie = s_dyn;
    int* s_fin = reinterpret_cast<int*>(s_dyn + words);
    if (threadIdx.x == 0) {
        s_tot = 0;
        s_cnt = 0;
    }
    for (int i = threadIdx.x; i < kSadWaveWords; i += blockDim.x) s_wave[i] = 0u;
    for (int i = threadIdx.x; i < words; i += blockDim.x) s_tie[i] = 0u;
    if (local)
        for (int k = threadIdx.x; k < a.nmb; k += blockDim.x) s_fin[k] = __ldcg(a.final_mv + k);
    __syncthreads();
    for (int i = threadIdx.x; i < ntie; i += blockDim.x) {
        const int k = a.tie_list[i], r = k / cols, t = k - r * cols + 2 * r;
        atomicOr(&s_tie[k >> 5], 1u << (k & 31));
        if (!every) atomicOr(&s_wave[t >> 5], 1u << (t & 31));
    }
    __syncthreads();
    if (ntie > 0) {
        constexpr int TW = TIE_RUNS * (int)(sizeof(TieRun) / sizeof(int));
        for (int t = 0; t < waves; t++) {
            if (!every && !((s_wave[t >> 5] >> (t & 31)) & 1u)) continue;  // block-uniform: no tie on it
            const int r_lo = max(0, (t - cols + 2) / 2), r_hi = min(rows - 1, t / 2);
            for (int r = r_lo + wib; r <= r_hi; r += nw) {
                const int k = r * cols + (t - 2 * r);
                if (!((s_tie[k >> 5] >> (k & 31)) & 1u)) continue;
                // the record and the tie tree do not depend on the prediction: one round trip for both
                const int* tree = a.tables + (size_t)k * TAB * TAB + TIE_ROW * TAB;
                const int4 sp = __ldcg(a.spec4 + k);
                const int t0 = __ldcg(tree + lane);
                const int t1 = lane < TW - 32 ? __ldcg(tree + 32 + lane) : 0;
                int px, py;
                if (local) {
                    const int av = sp.w;
                    const int A = (av & AV_A) ? s_fin[k - 1] : 0;
                    const int B = (av & AV_B) ? s_fin[k - cols] : 0;
                    const int C = (av & AV_C) ? s_fin[k - cols + 1] : 0;
                    const int D = (!(av & AV_C) && (av & AV_D)) ? s_fin[k - cols - 1] : 0;
                    median_from(av, A, B, C, D, &px, &py);
                } else {
                    median_pred(a.final_mv, sp.w, k, cols, &px, &py);
                }
                int mvx = mv_x(sp.x), mvy = mv_y(sp.x), md = sp.y;
                if (round_pred(px) != 0 || round_pred(py) != 0) {  // (0, 0): the scan already decided
                    if (!(sp.w & FLAG_DEEP)) tree_pick(t0, t1, round_pred(px), round_pred(py), &mvx, &mvy, &md);
                    else tie_path(a, k, px, py, sp.w, lane, &mvx, &mvy, &md);
                }
                if (lane == 0) {
                    const int v = pack_mv(mvx, mvy);
                    if (local) s_fin[k] = v;
                    __stcg(a.final_mv + k, v);
                    __stcg(a.final_dist + k, md);
                }
            }
            __syncthreads();
        }
    }
    __syncthreads();
    long long tot = 0;
    int cnt = 0;
    for (int k = threadIdx.x; k < a.nmb; k += blockDim.x) {
        const bool tie = (s_tie[k >> 5] >> (k & 31)) & 1u;
        const int fmv = local ? s_fin[k] : __ldcg(a.final_mv + k);
        const int d = tie ? __ldcg(a.final_dist + k) : __ldcg(&a.spec4[k].y);
        a.job->out_mv[k] = fmv;
        if (a.job->out_dist) a.job->out_dist[k] = d;
        if (a.job->incl && a.job->incl[k]) {
            tot += d;
            cnt++;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        tot += __shfl_xor_sync(0xffffffffu, tot, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if (lane == 0 && cnt) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&s_tot), (unsigned long long)tot);
        atomicAdd(&s_cnt, cnt);
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // the host reads the sums, device callers the average
        a.ctrl->total = s_tot;
        a.ctrl->count = s_cnt;
        if (a.job->out_avg) *a.job->out_avg = s_cnt ? s_tot / s_cnt : 0;
    }
}

// Motion-compensated luma residual (MotionCompensatorH264ImplStd::Compensate,
// MotionCompensatorH264ImplStd.cpp:413-431: QuarterRead of the reference at
// the vector, a copy for full-pel vectors; then OverlayMem2Dv2::Sub16x16):
// one warp per macroblock, samples from the estimate's planes.
__global__ void __launch_bounds__(256) k_full_residual(FullArgs a, const int* __restrict__ mv, short* __restrict__ res)
{
    const int lane = threadIdx.x & 31;
    const int k = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (k >= a.nmb) return;
    const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
    const int v = mv[k], mvx = mv_x(v), mvy = mv_y(v);
    const int qx = mvx % 4, qy = mvy % 4;  // C remainders, folded as QuarterRead does
    const int fx = qx < 0 ? qx + 4 : qx, fy = qy < 0 ? qy + 4 : qy;
    const int ox = n + mvx / 4 + (qx < 0 ? -1 : 0), oy = m + mvy / 4 + (qy < 0 ? -1 : 0);
    short* dst = res + (size_t)(m + (lane >> 1)) * a.W + n + 8 * (lane & 1);
    // a prediction more than 32 samples outside the picture would leave the
    // padded planes: flagged, residual zero
    if (ox < -32 || oy < -32 || ox > a.W + 16 || oy > a.H + 16) {
        *reinterpret_cast<uint4*>(dst) = make_uint4(0, 0, 0, 0);
        if (lane == 0) atomicOr(&a.ctrl->status, ST_OUT_OF_BOUNDS);
        return;
    }
    const uint2 p = qpel_block8(a, ox, oy, fx, fy, lane);
    const uint2 c = load_cur8(a, n, m, lane);
    short vals[8];
#pragma unroll
    for (int b = 0; b < 4; b++) {
        vals[b] = (short)((int)((c.x >> (8 * b)) & 0xff) - (int)((p.x >> (8 * b)) & 0xff));
        vals[4 + b] = (short)((int)((c.y >> (8 * b)) & 0xff) - (int)((p.y >> (8 * b)) & 0xff));
    }
    *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(vals);
}

size_t wave_smem_bytes(int nw, int cols, int chunk)
{
    return (size_t)kWaveStepBytes * nw * 2 * chunk + sizeof(unsigned long long) * nw * 2 + sizeof(int) * (size_t)nw * cols;
}

constexpr int kWaveMaxCols = 512;  // 8192 / 16

}  // namespace

int full_resolve_prepare(vppgpu_ctx* ctx, int* resolve_cap)
{
    *resolve_cap = ctx->sm_count * 8;
    // dirty bitmaps of the largest picture (8192 x 8192)
    const int tail_smem = 2 * (512 * 512 / 32) * (int)sizeof(unsigned);
    VPP_CUDA(cudaFuncSetAttribute(k_full_relax_tail<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, tail_smem));
    VPP_CUDA(cudaFuncSetAttribute(k_full_relax_tail<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, tail_smem));
    VPP_CUDA(cudaFuncSetAttribute(k_full_relax_tail<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, tail_smem));
    VPP_CUDA(cudaFuncSetAttribute(k_full_relax_tail<mrc::EST_V2_LAMBDA>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  tail_smem));
    VPP_CUDA(cudaFuncSetAttribute(k_full_relax_tail<cross::EST_CROSS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  tail_smem));
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<4, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(3, kWaveMaxCols, 4)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<2, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(kWaveMaxWarps, kWaveMaxCols, 2)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<4, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(3, kWaveMaxCols, 4)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<2, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(kWaveMaxWarps, kWaveMaxCols, 2)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<4, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(3, kWaveMaxCols, 4)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<2, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(kWaveMaxWarps, kWaveMaxCols, 2)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<4, mrc::EST_V2_LAMBDA>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(3, kWaveMaxCols, 4)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<2, mrc::EST_V2_LAMBDA>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(kWaveMaxWarps, kWaveMaxCols, 2)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<4, cross::EST_CROSS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(3, kWaveMaxCols, 4)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<2, cross::EST_CROSS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(kWaveMaxWarps, kWaveMaxCols, 2)));
    // the SAD resolve's largest dynamic shared memory: the local final vectors
    // end at kSadSmemMbs macroblocks (larger pictures keep only the tie bits)
    VPP_CUDA(cudaFuncSetAttribute(k_sad_resolve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sad_resolve_smem(kSadSmemMbs)));
    return VPPGPU_OK;
}

namespace {

template <int kEst>
int resolve_launch(vppgpu_ctx* ctx, const FullArgs& args)
{
    const int rows = args.nmb / args.cols, nbands = (rows + 31) / 32;
    if (args.cols > kWaveMaxCols) return VPPGPU_ERR_UNSUPPORTED;
    k_full_sweep0<kEst><<<(args.nmb + 7) / 8, 256, 0, ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    {
        // many warps, few MBs each: a sweep's latency is its busiest warp's evaluations
        const int want = (args.nmb + 7) / 8, cap = ctx->sm_count * args.relax_blocks_per_sm;
        const int blocks = want < cap ? want : cap;
        // the first sweeps over every MB, the rest (if any) over the dirty sets by one block
        const int grid_sweeps = args.relax_sweeps < args.grid_sweeps ? args.relax_sweeps : args.grid_sweeps;
        const bool tail = args.relax_sweeps > grid_sweeps;
        for (int sweep = 1; sweep <= grid_sweeps; sweep++) {
            k_full_relax_sweep<kEst><<<blocks, 256, 0, ctx->stream>>>(args, sweep, tail && sweep == grid_sweeps);
            VPP_CHECK_LAUNCH(ctx);
        }
        if (tail) {
            const size_t words = (size_t)(args.nmb + 31) / 32;
            k_full_relax_tail<kEst><<<1, 1024, 2 * words * sizeof(unsigned), ctx->stream>>>(args, grid_sweeps + 1);
            VPP_CHECK_LAUNCH(ctx);
        }
        const int ob = (args.nmb + 255) / 256, ocap = ctx->sm_count * 4;
        k_full_relax_outcome<<<ob < ocap ? ob : ocap, 256, 0, ctx->stream>>>(args);
        VPP_CHECK_LAUNCH(ctx);
    }
    {
        const int blocks = (args.nmb + 7) / 8, cap = ctx->sm_count * 8, grid = blocks < cap ? blocks : cap;
        k_full_precompute<kEst><<<grid, 256, 0, ctx->stream>>>(args);
        VPP_CHECK_LAUNCH(ctx);
        k_full_closure<kEst><<<grid, 256, 0, ctx->stream>>>(args);
        VPP_CHECK_LAUNCH(ctx);
    }
    for (int b0 = 0; b0 < nbands; b0 += kWaveMaxWarps) {
        const int nw = nbands - b0 < kWaveMaxWarps ? nbands - b0 : kWaveMaxWarps;
        const int last = b0 + nw == nbands;
        if (nw <= 3)
            k_full_wave<4, kEst><<<1, nw * 32, wave_smem_bytes(nw, args.cols, 4), ctx->stream>>>(args, b0, last);
        else
            k_full_wave<2, kEst><<<1, nw * 32, wave_smem_bytes(nw, args.cols, 2), ctx->stream>>>(args, b0, last);
        VPP_CHECK_LAUNCH(ctx);
    }
    {
        const int blocks = (args.nmb + 255) / 256, cap = ctx->sm_count * 4;
        k_full_wave_outputs<<<blocks < cap ? blocks : cap, 256, 0, ctx->stream>>>(args);
        VPP_CHECK_LAUNCH(ctx);
        k_full_average<<<1, 1, 0, ctx->stream>>>(args);
        VPP_CHECK_LAUNCH(ctx);
    }
    return VPPGPU_OK;
}

}  // namespace

int full_resolve_launch(vppgpu_ctx* ctx, const FullArgs& args, int resolve_grid, int est)
{
    (void)resolve_grid;
    switch (est) {
    case 0: return resolve_launch<0>(ctx, args);
    case 1: return resolve_launch<1>(ctx, args);
    case 2: return resolve_launch<2>(ctx, args);
    case cross::EST_CROSS: return resolve_launch<cross::EST_CROSS>(ctx, args);
    case mrc::EST_V2_LAMBDA: return resolve_launch<mrc::EST_V2_LAMBDA>(ctx, args);
    default: return VPPGPU_ERR_INVALID_ARG;
    }
}

int sad_resolve_launch(vppgpu_ctx* ctx, const FullArgs& args)
{
    k_sad_resolve<<<1, 1024, sad_resolve_smem(args.nmb), ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

int full_residual_launch(vppgpu_ctx* ctx, const FullArgs& args, const int* d_mv, short* d_res)
{
    k_full_residual<<<(args.nmb + 7) / 8, 256, 0, ctx->stream>>>(args, d_mv, d_res);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

}  // namespace vppgpu
