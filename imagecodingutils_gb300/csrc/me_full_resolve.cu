// me_full_resolve.cu -- prediction-dependent tail of MotionEstimatorH264ImplFull.
//
// After k_full_search every macroblock has its prediction-independent results
// (sub-pel vector and distortion, zero-vector distortion).  What is left is a
// function of the median prediction (Full.cpp:368-380 rounding, 401-446 tie
// rescan, 532-590 prediction distortion and GetBestVector), and the
// prediction depends on the left / above / above-right (else above-left)
// neighbours' final vectors: a DAG in raster order.
//
//   k_full_sweep0    every MB at once, prediction from the current vectors
//                    (initially the searched ones); caches the distortion at
//                    the prediction it saw.
//   k_full_relax     cooperative: up to kRelaxSweeps sweeps re-evaluating the
//                    MBs whose prediction changed (cache first).  A sweep
//                    without change is the unique fixed point of the DAG,
//                    i.e. the sequential result; most frames stop here.
//                    Otherwise (long copy chains: the prediction wins and is
//                    copied along rows and columns) block 0 builds a
//                    dictionary of the frame's dominant vectors.
//   k_full_precompute  distortion of every MB at every dictionary vector.
//   k_full_wave      one CTA: the exact sequential order as anti-diagonal
//                    steps (t = col + 2*row), vectors in shared memory,
//                    cached distortions prefetched two diagonals ahead with
//                    cp.async; misses are computed by whole warps.
#include "me_full_common.cuh"

namespace vppgpu {
namespace {
using namespace full;

constexpr int kEmpty = 0x7fffffff;  // no vector packs to this (|y| < 32767 quarter pels)
constexpr int kRelaxSweeps = 8;
constexpr int kCacheRelax = 1;      // entries 1..3 round robin in relaxation
constexpr int kCacheDict = 4;       // entries 4..11 dictionary

struct WarpScratch {
    union {
        SubpelScratch sp;
        PdScratch pd;
    } u;
    alignas(16) unsigned char cur[256];
};

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

// Distortion at the prediction, one warp (cur already loaded).
__device__ __forceinline__ int warp_pred_distortion(const FullArgs& a, const PredGeom& g, WarpScratch& ws, int lane)
{
    Plane8 rp{a.refp, a.rstride};
    load_patch22(ws.u.pd.patch, rp, g.ox, g.oy, lane);
    return pd_planar_warp(ws.u.pd, ws.cur, g.fx, g.fy, lane);
}

// Exact-tie macroblocks: the integer scan depends on the rounded prediction;
// replay it from the kept table and redo the sub-pel stage if the full-pel
// winner moved.  Rare, so kept out of line.
__device__ __noinline__ void tie_path(const FullArgs& a, int k, int px, int py, WarpScratch& ws, int lane, int* mvx,
                                      int* mvy, int* minD)
{
    int prx = round_pred(px), pry = round_pred(py);
    if (prx == 0 && pry == 0) return;  // the search kernel already decided ties with (0,0)
    const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
    int xl, xr, yu, yd, mx, my, md, tie;
    full_range(n, m, a.W, a.H, a.motion_range, xl, xr, yu, yd);
    scan_table(GlobalTab{a.tables + (size_t)k * TAB * TAB}, xl, xr, yu, yd, prx, pry, lane, &mx, &my, &md, &tie);
    int imv = a.spec_imv[k];
    if (mx != mv_x(imv) || my != mv_y(imv)) {
        Plane8 rp{a.refp, a.rstride};
        load_patch22(ws.u.sp.patch, rp, n + mx, m + my, lane);
        int qmx, qmy;
        subpel_refine_warp(ws.u.sp, ws.cur, lane, &md, &qmx, &qmy);
        *mvx = 4 * mx + qmx;
        *mvy = 4 * my + qmy;
        *minD = md;
    }
}

// Warp-level cache probe: lanes 0..KCACHE-1 each hold one entry.
__device__ __forceinline__ bool cache_probe(const int2* c, int key, int lane, int* pd)
{
    int2 e = lane < KCACHE ? __ldcg(c + lane) : make_int2(kEmpty, 0);
    unsigned hit = __ballot_sync(0xffffffffu, e.x == key);
    if (!hit) return false;
    *pd = __shfl_sync(0xffffffffu, e.y, __ffs(hit) - 1);
    return true;
}

// Full evaluation of MB k for raw prediction (px, py).  pd_known >= 0 skips
// the distortion computation.  Returns the packed final vector and distance.
__device__ __noinline__ void evaluate(const FullArgs& a, int k, int px, int py, int pd, WarpScratch& ws, int lane, int* out_mv,
                         int* out_d, int* out_pd)
{
    const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
    const int4 sp = a.spec4[k];
    int mvx = mv_x(sp.x), mvy = mv_y(sp.x), minD = sp.y;
    const int zd = sp.z;
    bool tie = (sp.w & FLAG_TIE) && (round_pred(px) != 0 || round_pred(py) != 0);
    PredGeom g = pred_geom(n, m, a.W, a.H, px, py);
    if (pd < 0 || tie) load_cur(ws.cur, a, n, m, lane);
    if (tie) tie_path(a, k, px, py, ws, lane, &mvx, &mvy, &minD);
    if (pd < 0) pd = warp_pred_distortion(a, g, ws, lane);
    int pos = best_of3_fast(mvx, mvy, minD, g.pcx, g.pcy, pd, zd, a.lambda, g.pcx, g.pcy);
    *out_pd = pd;
    if (pos == 0) {
        *out_mv = pack_mv(mvx, mvy);
        *out_d = minD;
    } else if (pos == 1) {
        *out_mv = pack_mv(g.pcx, g.pcy);
        *out_d = pd;
    } else {
        *out_mv = pack_mv(0, 0);
        *out_d = zd;
    }
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_full_sweep0(FullArgs a)
{
    __shared__ WarpScratch S[8];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int k = blockIdx.x * 8 + wib;
    if (k >= a.nmb) return;
    int px, py;
    median_pred(a.final_mv, a.spec4[k].w, k, a.cols, &px, &py);
    int fmv, fd, pd;
    evaluate(a, k, px, py, -1, S[wib], lane, &fmv, &fd, &pd);
    int key = pack_mv(px, py);
    if (lane < KCACHE) __stcg(a.cache + (size_t)k * KCACHE + lane, lane == 0 ? make_int2(key, pd) : make_int2(kEmpty, 0));
    if (lane == 0) {
        a.pred_used[k] = key;
        a.final_dist[k] = fd;
        __stcg(a.final_mv + k, fmv);
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
    bool converged = false, ok = true;
    int sweep = 1;
    for (; sweep <= kRelaxSweeps; sweep++) {
        int changed = 0;
        for (int k = gwarp; k < a.nmb; k += nwarps) {
            const int av = __ldcg(&a.spec4[k].w);
            int px, py;
            median_pred(a.final_mv, av, k, a.cols, &px, &py);
            int key = pack_mv(px, py);
            if (a.pred_used[k] == key) continue;
            int2* cache = a.cache + (size_t)k * KCACHE;
            int pd = -1;
            bool hit = cache_probe(cache, key, lane, &pd);
            int fmv, fd, npd;
            evaluate(a, k, px, py, hit ? pd : -1, ws, lane, &fmv, &fd, &npd);
            if (lane == 0) {
                atomicAdd(&a.ctrl->relax_evals, 1);
                if (!hit) atomicAdd(&a.ctrl->relax_miss, 1);
                if (!hit) __stcg(cache + kCacheRelax + (sweep % 3), make_int2(key, npd));
                a.pred_used[k] = key;
                a.final_dist[k] = fd;
                if (__ldcg(a.final_mv + k) != fmv) {
                    __stcg(a.final_mv + k, fmv);
                    changed = 1;
                }
            }
            __syncwarp();
        }
        if (lane == 0 && changed) atomicAdd(&a.changed[sweep], 1);
        ok = grid_sync(a.ctrl->bar, &a.ctrl->status, gridDim.x, a.spin_limit);
        if (!ok) return;
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
// One warp per (MB, dictionary vector): distortion at that vector, unless the
// MB's cache already holds it.
__global__ void __launch_bounds__(256) k_full_precompute(FullArgs a)
{
    if (*((volatile int*)&a.ctrl->converged)) return;
    __shared__ WarpScratch S[8];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (int task = blockIdx.x * 8 + wib; task < a.nmb * NDICT; task += gridDim.x * 8) {
        const int k = task / NDICT, d = task - k * NDICT;
        const int v = a.dict[d];
        if (v == kEmpty) continue;
        int2* cache = a.cache + (size_t)k * KCACHE;
        int pd;
        if (cache_probe(cache, v, lane, &pd)) continue;
        const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
        load_cur(S[wib].cur, a, n, m, lane);
        PredGeom g = pred_geom(n, m, a.W, a.H, mv_x(v), mv_y(v));
        pd = warp_pred_distortion(a, g, S[wib], lane);
        if (lane == 0) __stcg(cache + kCacheDict + d, make_int2(v, pd));
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Exact wavefront in one CTA.  Diagonal t holds the MBs with col + 2*row == t;
// every MB's neighbours lie on earlier diagonals.
constexpr int kWaveThreads = 512;
constexpr int kWaveMaxDiag = 256;   // MBs on one diagonal: min(rows, ceil(cols/2))
constexpr int kWaveMissWarps = 8;   // warps that evaluate cache misses
constexpr int kWaveRing = 3;

struct WaveEntry {
    int2 cache[KCACHE];  // 96 B
    int4 spec;           // 16 B
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void diag_range(int t, int cols, int rows, int* r_lo, int* cnt)
{
    int lo = t - (cols - 1);
    lo = lo > 0 ? (lo + 1) / 2 : 0;
    int hi = t / 2 < rows - 1 ? t / 2 : rows - 1;
    *r_lo = lo;
    *cnt = hi >= lo ? hi - lo + 1 : 0;
}

__device__ __forceinline__ void prefetch_diag(const FullArgs& a, WaveEntry* slot, int t)
{
    int r_lo, cnt;
    diag_range(t, a.cols, a.nmb / a.cols, &r_lo, &cnt);
    for (int i = threadIdx.x; i < cnt * 7; i += blockDim.x) {
        int e = i / 7, part = i - e * 7;
        int r = r_lo + e, c = t - 2 * r, k = r * a.cols + c;
        if (part < 6)
            cp_async16(&slot[e].cache[2 * part], a.cache + (size_t)k * KCACHE + 2 * part);
        else
            cp_async16(&slot[e].spec, a.spec4 + k);
    }
}

template <bool kSmemVectors>
__global__ void __launch_bounds__(kWaveThreads, 1) k_full_wave(FullArgs a)
{
    if (*((volatile int*)&a.ctrl->converged)) return;
    extern __shared__ __align__(16) unsigned char wave_smem[];
    WaveEntry* ring = reinterpret_cast<WaveEntry*>(wave_smem);                   // kWaveRing x kWaveMaxDiag
    WarpScratch* ws = reinterpret_cast<WarpScratch*>(ring + kWaveRing * kWaveMaxDiag);  // miss warps
    int* miss = reinterpret_cast<int*>(ws + kWaveMissWarps);                                  // kWaveMaxDiag + 1
    int* fin = kSmemVectors ? miss + kWaveMaxDiag + 1 : a.final_mv;              // vectors in raster order
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int cols = a.cols, rows = a.nmb / a.cols;
    const int tmax = (cols - 1) + 2 * (rows - 1);

    prefetch_diag(a, ring + 0 * kWaveMaxDiag, 0);
    cp_async_commit();
    prefetch_diag(a, ring + 1 * kWaveMaxDiag, 1);
    cp_async_commit();
    if (threadIdx.x == 0) miss[kWaveMaxDiag] = 0;

    for (int t = 0; t <= tmax; t++) {
        prefetch_diag(a, ring + ((t + 2) % kWaveRing) * kWaveMaxDiag, t + 2);
        cp_async_commit();
        cp_async_wait<2>();
        __syncthreads();  // diagonal t's entries and diagonal t-1's vectors visible
        WaveEntry* slot = ring + (t % kWaveRing) * kWaveMaxDiag;
        int r_lo, cnt;
        diag_range(t, cols, rows, &r_lo, &cnt);
        for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
            int r = r_lo + e, c = t - 2 * r, k = r * cols + c;
            const WaveEntry& we = slot[e];
            const int av = we.spec.w;
            int A = (av & AV_A) ? fin[k - 1] : 0;
            int B = (av & AV_B) ? fin[k - cols] : 0;
            int C = (av & AV_C) ? fin[k - cols + 1] : 0;
            int D = (!(av & AV_C) && (av & AV_D)) ? fin[k - cols - 1] : 0;
            int px, py;
            median_from(av, A, B, C, D, &px, &py);
            int key = pack_mv(px, py);
            bool tie = (av & FLAG_TIE) && (round_pred(px) != 0 || round_pred(py) != 0);
            int pd = -1;
#pragma unroll
            for (int q = 0; q < KCACHE; q++)
                if (pd < 0 && we.cache[q].x == key) pd = we.cache[q].y;
            if (pd < 0 || tie) {
                int idx = atomicAdd(&miss[kWaveMaxDiag], 1);
                miss[idx] = (k << 1);  // resolved below by a warp
                continue;
            }
            const int n = c * 16, m = r * 16;
            PredGeom g = pred_geom(n, m, a.W, a.H, px, py);
            int mvx = mv_x(we.spec.x), mvy = mv_y(we.spec.x);
            int pos = best_of3_fast(mvx, mvy, we.spec.y, g.pcx, g.pcy, pd, we.spec.z, a.lambda, g.pcx, g.pcy);
            int fmv = pos == 0 ? we.spec.x : (pos == 1 ? pack_mv(g.pcx, g.pcy) : 0);
            int fd = pos == 0 ? we.spec.y : (pos == 1 ? pd : we.spec.z);
            fin[k] = fmv;
            a.final_dist[k] = fd;
        }
        __syncthreads();
        const int nmiss = miss[kWaveMaxDiag];
        if (nmiss) {
            if (threadIdx.x == 0) atomicAdd(&a.ctrl->wave_miss, nmiss);
            for (int i = wid; wid < kWaveMissWarps && i < nmiss; i += kWaveMissWarps) {
                int k = miss[i] >> 1;
                int r = k / cols, c = k - r * cols;
                int av = a.spec4[k].w;
                int A = (av & AV_A) ? fin[k - 1] : 0;
                int B = (av & AV_B) ? fin[k - cols] : 0;
                int C = (av & AV_C) ? fin[k - cols + 1] : 0;
                int D = (!(av & AV_C) && (av & AV_D)) ? fin[k - cols - 1] : 0;
                int px, py;
                median_from(av, A, B, C, D, &px, &py);
                int fmv, fd, pd;
                evaluate(a, k, px, py, -1, ws[wid], lane, &fmv, &fd, &pd);
                (void)r;
                (void)c;
                if (lane == 0) {
                    fin[k] = fmv;
                    a.final_dist[k] = fd;
                }
                __syncwarp();
            }
            __syncthreads();
            if (threadIdx.x == 0) miss[kWaveMaxDiag] = 0;
        }
    }
    __syncthreads();
    // outputs and the included-distortion average (Full.cpp:581-611)
    long long tot = 0;
    int cnt = 0;
    for (int k = threadIdx.x; k < a.nmb; k += blockDim.x) {
        int fmv = fin[k];
        a.out_mv[k] = fmv;
        if (!kSmemVectors) continue;
        __stcg(a.final_mv + k, fmv);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < a.nmb; k += blockDim.x) {
        int d = a.final_dist[k];
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
    __shared__ long long wt[32];
    __shared__ int wc[32];
    if (lane == 0) {
        wt[wid] = tot;
        wc[wid] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long T = 0;
        int Cn = 0;
        for (int w = 0; w < kWaveThreads / 32; w++) {
            T += wt[w];
            Cn += wc[w];
        }
        a.ctrl->total = T;
        a.ctrl->count = Cn;
        if (a.out_avg) *a.out_avg = Cn ? T / Cn : 0;
        a.ctrl->sweeps = kRelaxSweeps + 1000;
    }
}

size_t wave_smem_bytes(int nmb, bool smem_vectors)
{
    size_t b = sizeof(WaveEntry) * kWaveRing * kWaveMaxDiag + sizeof(WarpScratch) * kWaveMissWarps +
               sizeof(int) * (kWaveMaxDiag + 1);
    if (smem_vectors) b += sizeof(int) * (size_t)nmb;
    return b;
}

constexpr int kWaveSmemVectorsMax = 24000;  // MBs whose vectors fit in shared memory next to the ring

}  // namespace

int full_resolve_prepare(vppgpu_ctx* ctx, int* resolve_cap)
{
    int per_sm = 0;
    VPP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_full_relax, 256, 0));
    if (per_sm < 1) return VPPGPU_ERR_UNSUPPORTED;
    *resolve_cap = per_sm * ctx->sm_count;
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(kWaveSmemVectorsMax, true)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_wave<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)wave_smem_bytes(0, false)));
    return VPPGPU_OK;
}

int full_resolve_launch(vppgpu_ctx* ctx, const FullArgs& args, int resolve_grid)
{
    const int rows = args.nmb / args.cols;
    const int diag = rows < (args.cols + 1) / 2 ? rows : (args.cols + 1) / 2;
    if (diag > kWaveMaxDiag) return VPPGPU_ERR_UNSUPPORTED;
    k_full_sweep0<<<(args.nmb + 7) / 8, 256, 0, ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    {
        void* params[] = {(void*)&args};
        VPP_CUDA(cudaLaunchCooperativeKernel((const void*)k_full_relax, dim3(resolve_grid), dim3(256), params, 0,
                                             ctx->stream));
        ctx->launches++;
    }
    {
        int tasks_blocks = (args.nmb * NDICT + 7) / 8, cap = ctx->sm_count * 8;
        k_full_precompute<<<tasks_blocks < cap ? tasks_blocks : cap, 256, 0, ctx->stream>>>(args);
    }
    VPP_CHECK_LAUNCH(ctx);
    if (args.nmb <= kWaveSmemVectorsMax)
        k_full_wave<true><<<1, kWaveThreads, wave_smem_bytes(args.nmb, true), ctx->stream>>>(args);
    else
        k_full_wave<false><<<1, kWaveThreads, wave_smem_bytes(0, false), ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

}  // namespace vppgpu
