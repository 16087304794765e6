// me_full_resolve.cu -- prediction-dependent tail of MotionEstimatorH264ImplFull.
//
// After k_full_search every macroblock has its prediction-independent results
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
//   k_full_relax       cooperative: up to kRelaxSweeps sweeps re-evaluating
//                      the MBs whose prediction changed.  A sweep without
//                      change is the unique fixed point of the DAG, i.e. the
//                      sequential result.  Otherwise (long copy chains: the
//                      prediction wins and is copied along rows and columns)
//                      block 0 builds a dictionary of the frame's dominant
//                      vectors.
//   k_full_precompute  records of every MB at every dictionary vector.
//   k_full_wave        one CTA replays the exact sequential order, pipelined
//                      by rows: warp w owns rows w, w+32, ...; a row advances
//                      one MB per step once the row above has finished the
//                      MB above-right, signalled through shared-memory
//                      progress counters.  A step is a median, a key match
//                      against the MB's records (prefetched with cp.async)
//                      and, on a miss only, a full evaluation by the warp.
#include "me_full_common.cuh"

namespace vppgpu {
namespace {
using namespace full;

constexpr int kEmpty = 0x7fffffff;  // no vector packs to this (|y| < 32767 quarter pels)
constexpr int kRelaxSweeps = 8;
constexpr int kCacheRelax = 1;      // entries 1..3 round robin in relaxation
constexpr int kCacheDict = 4;       // entries 4..11 dictionary

__device__ __forceinline__ int4 empty_record() { return make_int4(kEmpty, 0, 0, 0); }

__device__ __forceinline__ void load_cur(unsigned char* cur, const FullArgs& a, int n, int m, int lane)
{
    if (lane < 16)
        *reinterpret_cast<uint4*>(cur + 16 * lane) =
            *reinterpret_cast<const uint4*>(a.src8 + (size_t)(m + lane) * a.W + n);
    __syncwarp();
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

// Distortion at the prediction, one warp: QuarterRead's sixteen cases
// (OverlayMem2Dv2::QuarterRead) as one sample of the full-pel, b, h or j
// plane, or the rounded mean of two.  Lane l covers row l/2, columns
// 8*(l&1) .. +7; squared differences with dp4a on per-byte |differences|.
__device__ __forceinline__ int plane_pred_distortion(const FullArgs& a, int n, int m, const PredGeom& g, int lane)
{
    const int r = lane >> 1, c0 = (lane & 1) * 8, st = a.rstride;
    const size_t o = (size_t)(g.oy + r + PAD) * st + (size_t)(g.ox + c0 + PAD);
    const unsigned char* G = a.refp;
    const unsigned char* Bp = a.hpel;
    const unsigned char* Hp = a.hpel + a.plane_size;
    const unsigned char* Jp = a.hpel + 2 * a.plane_size;
    const unsigned char *p1 = G + o, *p2 = G + o;
    bool two = true;
    switch (g.fx | (g.fy << 2)) {
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
    const uint2 cur = __ldg(reinterpret_cast<const uint2*>(a.src8 + (size_t)(m + r) * a.W + n + c0));
    const unsigned d0 = __vabsdiffu4(cur.x, v.x), d1 = __vabsdiffu4(cur.y, v.y);
    return warp_sum((int)__dp4a(d0, d0, __dp4a(d1, d1, 0u)));
}

// Exact-tie macroblocks: the integer scan depends on the rounded prediction.
// Walk the tie tree the search kernel kept (one load per lane), or, for the
// rare macroblock with more ties than the tree holds, replay the scan from
// the kept table and redo the sub-pel stage if the full-pel winner moved.
// Kept out of line.
__device__ __noinline__ void tie_path(const FullArgs& a, int k, int px, int py, int flags, WarpScratch& ws,
                                      int lane, int* mvx, int* mvy, int* minD)
{
    int prx = round_pred(px), pry = round_pred(py);
    if (prx == 0 && pry == 0) return;  // the search kernel already decided ties with (0,0)
    const int* tab = a.tables + (size_t)k * TAB * TAB;
    if (!(flags & FLAG_DEEP)) {
        constexpr int RW = sizeof(TieRun) / sizeof(int), TW = TIE_RUNS * RW;
        const int* tree = tab + TIE_ROW * TAB;
        const int t0 = __ldcg(tree + lane);
        const int t1 = lane < TW - 32 ? __ldcg(tree + 32 + lane) : 0;
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
        return;
    }
    const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
    int xl, xr, yu, yd, mx, my, md, tie;
    full_range(n, m, a.W, a.H, a.motion_range, xl, xr, yu, yd);
    scan_table(GlobalTab{tab}, xl, xr, yu, yd, prx, pry, lane, &mx, &my, &md, &tie);
    int imv = a.spec_imv[k];
    if (mx != mv_x(imv) || my != mv_y(imv)) {
        load_cur(ws.cur, a, n, m, lane);
        Plane8 rp{a.refp, a.rstride};
        load_patch22(ws.sp.patch, rp, n + mx, m + my, lane);
        int qmx, qmy;
        subpel_refine_warp<true>(ws.sp, ws.cur, lane, &md, &qmx, &qmy);
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

// Full evaluation of MB k for raw prediction (px, py), one warp: the record
// {prediction, distortion at it, final vector, final distortion}.
__device__ __noinline__ int4 evaluate(const FullArgs& a, int k, int px, int py, WarpScratch& ws, int lane)
{
    const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
    const int4 sp = a.spec4[k];
    int mvx = mv_x(sp.x), mvy = mv_y(sp.x), minD = sp.y;
    const int zd = sp.z;
    const bool tie = (sp.w & FLAG_TIE) && (round_pred(px) != 0 || round_pred(py) != 0);
    const PredGeom g = pred_geom(n, m, a.W, a.H, px, py);
    if (tie) tie_path(a, k, px, py, sp.w, ws, lane, &mvx, &mvy, &minD);
    const int pd = plane_pred_distortion(a, n, m, g, lane);
    const int pos = best_of3_fast(mvx, mvy, minD, g.pcx, g.pcy, pd, zd, a.lambda, g.pcx, g.pcy);
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
__global__ void __launch_bounds__(256, 4) k_full_sweep0(FullArgs a)
{
    __shared__ WarpScratch S[8];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int k = blockIdx.x * 8 + wib;
    if (k >= a.nmb) return;
    int px, py;
    median_pred(a.final_mv, a.spec4[k].w, k, a.cols, &px, &py);
    const int4 rec = evaluate(a, k, px, py, S[wib], lane);
    if (lane < KCACHE) __stcg(a.cache + (size_t)k * KCACHE + lane, lane == 0 ? rec : empty_record());
    if (lane == 0) {
        a.pred_used[k] = rec.x;
        a.final_dist[k] = rec.w;
        __stcg(a.final_mv + k, rec.z);
    }
}

// ---------------------------------------------------------------------------
struct RelaxSmem {
    union {
        WarpScratch w[8];
        struct {
            int keys[2048];
            int counts[2048];
        } hist;
    } u;
    long long red_total[8];
    int red_count[8];
    int red_key[8];
    int red_val[8];
};

__device__ void write_outputs_and_average(const FullArgs& a, RelaxSmem& S, int gwarp, int nwarps, int lane, int wib)
{
    long long tot = 0;
    int cnt = 0;
    for (int k = gwarp; k < a.nmb; k += nwarps) {
        if (lane == 0) {
            int fmv = __ldcg(a.final_mv + k);
            a.out_mv[k] = fmv;
            int d = a.final_dist[k];
            if (a.out_dist) a.out_dist[k] = d;
            if (a.incl && a.incl[k]) {
                tot += d;
                cnt++;
            }
        }
    }
    if (lane == 0) {
        S.red_total[wib] = tot;
        S.red_count[wib] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        int c = 0;
        for (int w = 0; w < 8; w++) {
            t += S.red_total[w];
            c += S.red_count[w];
        }
        if (c) {
            atomicAdd(reinterpret_cast<unsigned long long*>(&a.ctrl->total), (unsigned long long)t);
            atomicAdd(&a.ctrl->count, c);
        }
    }
}

__global__ void __launch_bounds__(256, 2) k_full_relax(FullArgs a)
{
    __shared__ RelaxSmem S;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gwarp = blockIdx.x * 8 + wib, nwarps = gridDim.x * 8;
    WarpScratch& ws = S.u.w[wib];
    bool converged = false;
    int sweep = 1;
    for (; sweep <= kRelaxSweeps; sweep++) {
        int changed = 0;
        for (int k = gwarp; k < a.nmb; k += nwarps) {
            const int av = __ldcg(&a.spec4[k].w);
            int px, py;
            median_pred(a.final_mv, av, k, a.cols, &px, &py);
            const int key = pack_mv(px, py);
            if (a.pred_used[k] == key) continue;
            int4* cache = a.cache + (size_t)k * KCACHE;
            int4 rec;
            const bool hit = cache_probe(cache, key, lane, &rec);
            if (!hit) rec = evaluate(a, k, px, py, ws, lane);
            if (lane == 0) {
                atomicAdd(&a.ctrl->relax_evals, 1);
                if (!hit) {
                    atomicAdd(&a.ctrl->relax_miss, 1);
                    __stcg(cache + kCacheRelax + (sweep % 3), rec);
                }
                a.pred_used[k] = key;
                a.final_dist[k] = rec.w;
                if (__ldcg(a.final_mv + k) != rec.z) {
                    __stcg(a.final_mv + k, rec.z);
                    changed = 1;
                }
            }
            __syncwarp();
        }
        if (lane == 0 && changed) atomicAdd(&a.changed[sweep], 1);
        if (!grid_sync(a.ctrl->bar, &a.ctrl->status, gridDim.x, a.spin_limit)) return;
        if (*((volatile int*)&a.changed[sweep]) == 0) {
            converged = true;
            break;
        }
    }
    if (converged) {
        write_outputs_and_average(a, S, gwarp, nwarps, lane, wib);
        if (!grid_sync(a.ctrl->bar, &a.ctrl->status, gridDim.x, a.spin_limit)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            long long t = *((volatile long long*)&a.ctrl->total);
            int c = *((volatile int*)&a.ctrl->count);
            if (a.out_avg) *a.out_avg = c ? t / c : 0;
            a.ctrl->sweeps = sweep;
            a.ctrl->converged = 1;
        }
        return;
    }
    // Not converged: block 0 finds the frame's dominant vectors.
    if (blockIdx.x != 0) return;
    for (int i = threadIdx.x; i < 2048; i += blockDim.x) {
        S.u.hist.keys[i] = kEmpty;
        S.u.hist.counts[i] = 0;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < a.nmb; k += blockDim.x) {
        int v = __ldcg(a.final_mv + k);
        unsigned h = ((unsigned)v * 2654435761u) >> 21;  // 11 bits
        for (int probe = 0; probe < 32; probe++) {
            int slot = (h + probe) & 2047;
            int prev = atomicCAS(&S.u.hist.keys[slot], kEmpty, v);
            if (prev == kEmpty || prev == v) {
                atomicAdd(&S.u.hist.counts[slot], 1);
                break;
            }
        }
    }
    __syncthreads();
    for (int d = 0; d < NDICT; d++) {
        int best_c = 0, best_k = kEmpty;
        for (int i = threadIdx.x; i < 2048; i += blockDim.x)
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
    if (threadIdx.x == 0) a.ctrl->sweeps = kRelaxSweeps;
}

// ---------------------------------------------------------------------------
// One warp per MB: records at every dictionary vector the MB's cache lacks,
// then the MB's wavefront record.
__global__ void __launch_bounds__(256, 2) k_full_precompute(FullArgs a)
{
    if (*((volatile int*)&a.ctrl->converged)) return;
    __shared__ WarpScratch S[8];
    __shared__ int dict[NDICT];
    if (threadIdx.x < NDICT) dict[threadIdx.x] = a.dict[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (int k = blockIdx.x * 8 + wib; k < a.nmb; k += gridDim.x * 8) {
        int4* cache = a.cache + (size_t)k * KCACHE;
        int4 mine = lane < KCACHE ? __ldcg(cache + lane) : empty_record();
        for (int d = 0; d < NDICT; d++) {
            const int v = dict[d];
            if (v == kEmpty || __any_sync(0xffffffffu, mine.x == v)) continue;
            const int4 rec = evaluate(a, k, mv_x(v), mv_y(v), S[wib], lane);
            if (lane == kCacheDict + d) mine = rec;
            if (lane == 0) __stcg(cache + kCacheDict + d, rec);
            __syncwarp();
        }
        WaveRec* wr = a.wave_rec + k;
        if (lane < KCACHE) wr->kv[lane] = make_int2(mine.x, mine.z);
        if (lane == KCACHE) wr->av = __ldcg(&a.spec4[k].w);
    }
}

// ---------------------------------------------------------------------------
// Exact order in one CTA.  Lane l of warp w owns row 32w + l and handles
// column t - 2l at step t: its left neighbour is its own previous output,
// above / above-right / above-left are lane l-1's outputs of steps t-2, t-1
// and t-3 (shuffles), so a warp advances 32 rows in lock step with no
// synchronisation.  Lane 0 takes the row above from warp w-1's lane 31
// through shared memory: each vector is its own flag (the array starts as
// kEmpty, which no vector packs to), so no fence sits in the loop.  Each lane prefetches its own wavefront records kRing columns
// ahead with cp.async; a step is a median, twelve key compares and, only for
// a lane whose prediction is in none of its records, a full evaluation by
// the whole warp.
constexpr int kWaveMaxWarps = WAVE_WARPS;  // 32 rows each: 512 rows

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void fetch_wave_rec(WaveRec* dst, const WaveRec* src)
{
#pragma unroll
    for (int q = 0; q < 7; q++)
        cp_async16(reinterpret_cast<int4*>(dst) + q, reinterpret_cast<const int4*>(src) + q);
}

template <int kRing, int kMaxThreads>
__global__ void __launch_bounds__(kMaxThreads, 1) k_full_wave(FullArgs a)
{
    if (*((volatile int*)&a.ctrl->converged)) return;
    extern __shared__ __align__(16) unsigned char wave_smem[];
    const int cols = a.cols, rows = a.nmb / a.cols, nw = blockDim.x >> 5;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    WaveRec* ring = reinterpret_cast<WaveRec*>(wave_smem);             // [nw][kRing][32]
    volatile int* edge = reinterpret_cast<int*>(ring + nw * kRing * 32);  // [nw][cols]: row 32w+31
    __shared__ int abort_flag;
    for (int i = threadIdx.x; i < nw * cols; i += blockDim.x) edge[i] = kEmpty;
    if (threadIdx.x == 0) abort_flag = 0;
    __syncthreads();

    WarpScratch& ws = reinterpret_cast<WarpScratch*>(a.wave_scratch)[w];
    const int r = 32 * w + lane;
    const bool row_ok = r < rows;
    const int lanes_used = min(32, rows - 32 * w);
    const int nsteps = cols + 2 * (lanes_used - 1);
    WaveRec* mine = ring + (w * kRing) * 32 + lane;      // slot s at mine[32 * s]
    const WaveRec* src = a.wave_rec + (size_t)r * cols;
    const volatile int* above = edge + (w - 1) * cols;   // used by lane 0 of warps > 0

    if (row_ok) {
        for (int c = 0; c < kRing - 1; c++) {
            if (c < cols) fetch_wave_rec(mine + 32 * c, src + c);
            cp_async_commit();
        }
    }
    int o1 = 0, o2 = 0, o3 = 0;  // this lane's outputs of steps t-1, t-2, t-3
    int misses = 0;
    for (int t = 0; t < nsteps; t++) {
        const int c = t - 2 * lane;
        const bool active = row_ok && c >= 0 && c < cols;
        int B = __shfl_up_sync(0xffffffffu, o2, 1);
        int C = __shfl_up_sync(0xffffffffu, o1, 1);
        int D = __shfl_up_sync(0xffffffffu, o3, 1);
        bool stop = false;
        if (lane == 0 && w > 0 && active) {
            // the row above, columns c-1 .. c+1, as warp w-1's lane 31 stores them
            long long it = 0;
            while (true) {
                B = above[c];
                C = c + 1 < cols ? above[c + 1] : 0;
                D = c >= 1 ? above[c - 1] : 0;
                if (B != kEmpty && C != kEmpty && D != kEmpty) break;
                if (++it > a.spin_limit || *((volatile int*)&abort_flag)) {
                    stop = true;
                    break;
                }
            }
        }
        if (__any_sync(0xffffffffu, stop)) {
            if (lane == 0) {
                abort_flag = 1;
                atomicOr(&a.ctrl->status, ST_TIMEOUT);
            }
            break;
        }
        int out = 0, px = 0, py = 0, q = -1;
        if (active) {
            if (c + kRing - 1 < cols) fetch_wave_rec(mine + 32 * ((c + kRing - 1) % kRing), src + c + kRing - 1);
            cp_async_commit();
            cp_async_wait<kRing - 1>();
            const WaveRec& rec = mine[32 * (c % kRing)];
            median_from(rec.av, o1, B, C, D, &px, &py);
            const int key = pack_mv(px, py);
#pragma unroll
            for (int e = KCACHE - 1; e >= 0; e--) {
                const int2 kv = rec.kv[e];
                if (kv.x == key) {
                    q = e;
                    out = kv.y;
                }
            }
        }
        unsigned miss = __ballot_sync(0xffffffffu, active && q < 0);
        misses += __popc(miss);
        while (miss) {
            const int f = __ffs(miss) - 1;
            miss &= miss - 1;
            const int fx = __shfl_sync(0xffffffffu, px, f), fy = __shfl_sync(0xffffffffu, py, f);
            const int fk = (32 * w + f) * cols + (t - 2 * f);
            const int4 rec = evaluate(a, fk, fx, fy, ws, lane);
            if (lane == f) {
                out = rec.z;
                a.final_dist[fk] = rec.w;
            }
        }
        if (active) {
            const int k = r * cols + c;
            a.final_mv[k] = out;
            a.wave_choice[k] = q;
            if (lane == 31) edge[w * cols + c] = out;
        }
        o3 = o2;
        o2 = o1;
        o1 = out;
    }
    if (row_ok) cp_async_wait<0>();
    if (lane == 0 && misses) atomicAdd(&a.ctrl->wave_miss, misses);
    __syncthreads();
    if (abort_flag) return;
    // outputs and the included-distortion average (Full.cpp:581-611)
    long long tot = 0;
    int cnt = 0;
    for (int k = threadIdx.x; k < a.nmb; k += blockDim.x) {
        const int fmv = a.final_mv[k];
        a.out_mv[k] = fmv;
        const int q = a.wave_choice[k];
        const int d = q >= 0 ? __ldcg(&a.cache[(size_t)k * KCACHE + q].w) : a.final_dist[k];
        a.final_dist[k] = d;
        if (a.out_dist) a.out_dist[k] = d;
        if (a.incl && a.incl[k]) {
            tot += d;
            cnt++;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        tot += __shfl_xor_sync(0xffffffffu, tot, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    __shared__ long long wt[kWaveMaxWarps];
    __shared__ int wc[kWaveMaxWarps];
    if (lane == 0) {
        wt[w] = tot;
        wc[w] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long T = 0;
        int Cn = 0;
        for (int i = 0; i < nw; i++) {
            T += wt[i];
            Cn += wc[i];
        }
        a.ctrl->total = T;
        a.ctrl->count = Cn;
        if (a.out_avg) *a.out_avg = Cn ? T / Cn : 0;
        a.ctrl->sweeps = kRelaxSweeps + 1000;
    }
}

size_t wave_smem_bytes(int nw, int cols, int ring)
{
    return sizeof(WaveRec) * (size_t)nw * ring * 32 + sizeof(int) * (size_t)nw * cols;
}

constexpr int kWaveMaxCols = 512;  // 8192 / 16

}  // namespace

size_t full_wave_scratch_bytes() { return sizeof(WarpScratch) * WAVE_WARPS; }

int full_resolve_prepare(vppgpu_ctx* ctx, int* resolve_cap)
{
    int per_sm = 0;
    VPP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_full_relax, 256, 0));
    if (per_sm < 1) return VPPGPU_ERR_UNSUPPORTED;
    *resolve_cap = per_sm * ctx->sm_count;
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<8, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(4, kWaveMaxCols, 8)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<3, kWaveMaxWarps * 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(kWaveMaxWarps, kWaveMaxCols, 3)));
    return VPPGPU_OK;
}

int full_resolve_launch(vppgpu_ctx* ctx, const FullArgs& args, int resolve_grid)
{
    const int rows = args.nmb / args.cols, nw = (rows + 31) / 32;
    if (nw > kWaveMaxWarps || args.cols > kWaveMaxCols) return VPPGPU_ERR_UNSUPPORTED;
    k_full_sweep0<<<(args.nmb + 7) / 8, 256, 0, ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    {
        void* params[] = {(void*)&args};
        VPP_CUDA(cudaLaunchCooperativeKernel((const void*)k_full_relax, dim3(resolve_grid), dim3(256), params, 0,
                                             ctx->stream));
        ctx->launches++;
    }
    {
        int blocks = (args.nmb + 7) / 8, cap = ctx->sm_count * 8;
        k_full_precompute<<<blocks < cap ? blocks : cap, 256, 0, ctx->stream>>>(args);
    }
    VPP_CHECK_LAUNCH(ctx);
    if (nw <= 4)
        k_full_wave<8, 128><<<1, nw * 32, wave_smem_bytes(nw, args.cols, 8), ctx->stream>>>(args);
    else
        k_full_wave<3, kWaveMaxWarps * 32><<<1, nw * 32, wave_smem_bytes(nw, args.cols, 3), ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

}  // namespace vppgpu
