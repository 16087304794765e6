// me_full.cu -- MotionEstimatorH264ImplFull on sm_103a.
//
// Reference: MotionEstimatorH264ImplFull::Estimate
// (src/CodecUtils/MotionEstimatorH264ImplFull.cpp:330-613).  Per 16x16
// macroblock: squared-error full search of +-R pels (running-best skip and
// prediction tie-break, :394-446), half-pel then quarter-pel refinement
// (:452-517), distortion at the median-predicted vector (:532-570) and a
// Lagrangian pick between best, predicted and zero vectors (:573-601).
//
// GB300 design
//   k_full_pack     int16 -> u8 (with a 0..255 check) and an edge-replicated
//                   padded reference, one pass over the planes.
//   k_full_search   one CTA per macroblock.  The whole (2R+1)^2 SSD table is
//                   computed as A2 + B2 - 2*sum(a*b): sum(a*b) with dp4a on
//                   four byte-shifted, zero-padded copies of each template
//                   row against word-aligned window rows held in registers
//                   (5 dp4a per 16-pixel row, no byte alignment work), B2 by
//                   separable sliding sums.  A warp then replays the
//                   reference's sequential raster scan over the table with
//                   ballots (only lanes that beat the running minimum are
//                   looked at), and runs the sub-pel stages.  None of this
//                   depends on the predictor except exact ties in the scan,
//                   which are flagged and the table kept for a rescan.
//   k_full_resolve  cooperative kernel.  A macroblock's final vector depends
//                   on its left/above/above-right neighbours' final vectors
//                   through the median predictor (a DAG in raster order).
//                   Each sweep recomputes every macroblock whose prediction
//                   changed, in place; a sweep with no change is the unique
//                   fixed point, i.e. the sequential result.  On a DAG this
//                   needs at most (longest dependency chain + 2) sweeps and
//                   in practice a handful, instead of a ~250-step wavefront.
#include <string.h>

#include "me_common.cuh"
#include "me_internal.h"

namespace vppgpu {
namespace {

constexpr int RMAX = 31;       // table geometry: i in [-31,31] -> ii = i+31, j -> jj = j+32
constexpr int WROWS = 84;      // window rows m-34 .. m+49
constexpr int WSTRIDE = 112;   // window cols n-48 .. n+63
constexpr int H2STRIDE = 81;   // odd stride: conflict-free column walks
constexpr int TAB = 64;        // SSD table is TAB x TAB ints
constexpr int FLAG_TIE = 1;

struct SearchSmem {
    alignas(16) unsigned char win[WROWS][WSTRIDE];
    alignas(16) unsigned ash[16][4][8];  // [y][shift][word]: template row y shifted right by `shift` bytes
    alignas(16) unsigned char cur[256];
    alignas(16) int tab[TAB][TAB];
    union {
        int h2t[TAB][H2STRIDE];  // h2t[jj][r] = sum_x win(r, jj+x)^2
        SubpelScratch sp;
    } u;
    int a2;
    int state[4];  // mx, my, minD, flags broadcast
};

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_full_pack(const short* __restrict__ src16, const short* __restrict__ ref16,
                                                  int W, int H, unsigned char* __restrict__ src8,
                                                  unsigned char* __restrict__ refp, int rstride, int* status)
{
    // padded reference: 4 bytes per thread; source: 4 samples per thread
    const int PW = W + 2 * PAD, PH = H + 2 * PAD;
    const long long nref = (long long)(PW / 4) * PH;  // PW is a multiple of 16
    const long long nsrc = (long long)W * H / 4;
    bool bad = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nref + nsrc;
         i += (long long)gridDim.x * blockDim.x) {
        if (i < nref) {
            int row = (int)(i / (PW / 4)), cq = (int)(i - (long long)row * (PW / 4));
            int y = min(max(row - PAD, 0), H - 1);
            unsigned out = 0;
#pragma unroll
            for (int b = 0; b < 4; b++) {
                int x = min(max(4 * cq + b - PAD, 0), W - 1);
                int v = ref16[(size_t)y * W + x];
                bad |= (v < 0) | (v > 255);
                out |= (unsigned)(v & 0xff) << (8 * b);
            }
            *reinterpret_cast<unsigned*>(refp + (size_t)row * rstride + 4 * cq) = out;
        } else {
            long long j = i - nref;
            const short2* s = reinterpret_cast<const short2*>(src16) + 2 * j;
            short2 a = s[0], b = s[1];
            int v0 = a.x, v1 = a.y, v2 = b.x, v3 = b.y;
            bad |= (v0 < 0) | (v0 > 255) | (v1 < 0) | (v1 > 255) | (v2 < 0) | (v2 > 255) | (v3 < 0) | (v3 > 255);
            unsigned out = (unsigned)(v0 & 0xff) | ((unsigned)(v1 & 0xff) << 8) | ((unsigned)(v2 & 0xff) << 16) |
                           ((unsigned)(v3 & 0xff) << 24);
            reinterpret_cast<unsigned*>(src8)[j] = out;
        }
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(status, ST_PIXEL_RANGE);
}

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
template <typename TabT>
__device__ __forceinline__ void scan_table(const TabT& tab, int xl, int xr, int yu, int yd, int prx, int pry,
                                           int lane, int* omx, int* omy, int* omin, int* tie)
{
    int minD = tab(RMAX, RMAX + 1), mx = 0, my = 0, t = 0;
    for (int i = yu; i <= yd; i++) {
        for (int base = xl; base <= xr; base += 32) {
            int j = base + lane;
            bool valid = (j <= xr) && !(i == 0 && j == 0);
            int d = valid ? tab(i + RMAX, j + RMAX + 1) : 0x7fffffff;
            unsigned pending = 0xffffffffu;
            while (true) {
                bool ok = valid && d <= minD && (i + my >= yu) && (i + my <= yd) && (j + mx >= xl) && (j + mx <= xr);
                unsigned m = __ballot_sync(0xffffffffu, ok) & pending;
                if (!m) break;
                int f = __ffs(m) - 1;
                int df = __shfl_sync(0xffffffffu, d, f);
                int jf = base + f;
                bool accept = true;
                if (df == minD) {
                    t = 1;
                    int cx = mx - prx, cy = my - pry, nx = jf - prx, ny = i - pry;
                    accept = (cy * cy + cx * cx) - (ny * ny + nx * nx) >= 0;
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
    *omx = mx;
    *omy = my;
    *omin = minD;
    *tie = t;
}

struct SmemTab {
    const int (*t)[TAB];
    __device__ int operator()(int r, int c) const { return t[r][c]; }
};
struct GlobalTab {
    const int* t;
    __device__ int operator()(int r, int c) const { return __ldcg(t + r * TAB + c); }
};

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128, 4) k_full_search(FullArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SearchSmem& S = *reinterpret_cast<SearchSmem*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int k = blockIdx.x;
    const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;

    // 1. window (rows m-34.., cols n-48..) and input block
    {
        const unsigned char* wbase = a.refp + (size_t)(m - 34 + PAD) * a.rstride + (n - 48 + PAD);
        for (int i = tid; i < WROWS * (WSTRIDE / 16); i += 128) {
            int r = i / (WSTRIDE / 16), c = i - r * (WSTRIDE / 16);
            *reinterpret_cast<uint4*>(&S.win[r][16 * c]) =
                *reinterpret_cast<const uint4*>(wbase + (size_t)r * a.rstride + 16 * c);
        }
        if (tid < 16)
            *reinterpret_cast<uint4*>(&S.cur[16 * tid]) =
                *reinterpret_cast<const uint4*>(a.src8 + (size_t)(m + tid) * a.W + n);
    }
    __syncthreads();

    // 2. shifted template rows, template energy, horizontal window energies
    if (tid < 64) {
        int y = tid >> 2, s = tid & 3;
        unsigned wds[8];
#pragma unroll
        for (int w = 0; w < 8; w++) {
            unsigned v = 0;
#pragma unroll
            for (int b = 0; b < 4; b++) {
                int x = 4 * w + b - s;
                unsigned px = (x >= 0 && x < 16) ? S.cur[16 * y + x] : 0u;
                v |= px << (8 * b);
            }
            wds[w] = v;
        }
        *reinterpret_cast<uint4*>(&S.ash[y][s][0]) = make_uint4(wds[0], wds[1], wds[2], wds[3]);
        *reinterpret_cast<uint4*>(&S.ash[y][s][4]) = make_uint4(wds[4], wds[5], wds[6], wds[7]);
    } else if (tid < 96) {
        int l = tid - 64, acc = 0;
#pragma unroll
        for (int t = 0; t < 8; t++) {
            int v = S.cur[l + 32 * t];
            acc += v * v;
        }
        acc = warp_sum(acc);
        if (l == 0) S.a2 = acc;
    }
    if (tid < 78) {
        // row r of the dp4a geometry is window row r+3; columns jj+x -> smem col 16+jj+x
        const unsigned char* row = &S.win[tid + 3][16];
        int sum = 0;
#pragma unroll
        for (int x = 0; x < 16; x++) sum += (int)row[x] * row[x];
        S.u.h2t[0][tid] = sum;
        for (int jj = 1; jj < TAB; jj++) {
            int o = row[jj - 1], nw = row[jj + 15];
            sum += nw * nw - o * o;
            S.u.h2t[jj][tid] = sum;
        }
    }
    __syncthreads();

    // 3. vertical window energies -> tab
    if (tid < TAB) {
        const int* col = S.u.h2t[tid];
        int sum = 0;
#pragma unroll
        for (int y = 0; y < 16; y++) sum += col[y];
        S.tab[0][tid] = sum;
        for (int ii = 1; ii < 2 * RMAX + 1; ii++) {
            sum += col[ii + 15] - col[ii - 1];
            S.tab[ii][tid] = sum;
        }
    }
    __syncthreads();

    // 4. cross terms with dp4a; each thread: 8 candidate rows x 4 word offsets, one byte shift
    {
        const int s = lane & 3, qg = (lane >> 2) & 3, ig = 2 * warp + (lane >> 4);
        const int ii0 = 8 * ig;
        unsigned bw[8][8];
        auto load_row = [&](unsigned* dst, int r) {
            const uint4* p = reinterpret_cast<const uint4*>(&S.win[r + 3][16 + 16 * qg]);
            uint4 x0 = p[0], x1 = p[1];
            dst[0] = x0.x; dst[1] = x0.y; dst[2] = x0.z; dst[3] = x0.w;
            dst[4] = x1.x; dst[5] = x1.y; dst[6] = x1.z; dst[7] = x1.w;
        };
#pragma unroll
        for (int r = 0; r < 8; r++) load_row(bw[r], ii0 + r);
        unsigned acc[8][4];
#pragma unroll
        for (int r = 0; r < 8; r++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[r][q] = 0u;
#pragma unroll
        for (int y = 0; y < 16; y++) {
            uint4 a0 = *reinterpret_cast<const uint4*>(&S.ash[y][s][0]);
            unsigned a4 = S.ash[y][s][4];
            const unsigned A[5] = {a0.x, a0.y, a0.z, a0.w, a4};
#pragma unroll
            for (int r = 0; r < 8; r++) {
                const unsigned* B = bw[(r + y) & 7];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    unsigned c = acc[r][q];
#pragma unroll
                    for (int w = 0; w < 5; w++) c = __dp4a(A[w], B[q + w], c);
                    acc[r][q] = c;
                }
            }
            if (y < 15) load_row(bw[y & 7], ii0 + y + 8);
        }
        const int a2 = S.a2;
#pragma unroll
        for (int r = 0; r < 8; r++) {
            int ii = ii0 + r;
            if (ii < 2 * RMAX + 1) {
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    int jj = 4 * (4 * qg + q) + s;
                    S.tab[ii][jj] = a2 + S.tab[ii][jj] - 2 * (int)acc[r][q];
                }
            }
        }
    }
    __syncthreads();

    // 5. sequential scan replay (warp 0)
    int xl, xr, yu, yd;
    full_range(n, m, a.W, a.H, a.motion_range, xl, xr, yu, yd);
    if (warp == 0) {
        int mx, my, minD, tie;
        scan_table(SmemTab{S.tab}, xl, xr, yu, yd, 0, 0, lane, &mx, &my, &minD, &tie);
        if (lane == 0) {
            S.state[0] = mx;
            S.state[1] = my;
            S.state[2] = minD;
            S.state[3] = tie ? FLAG_TIE : 0;
        }
    }
    __syncthreads();
    const int mx = S.state[0], my = S.state[1], flags = S.state[3];
    int minD = S.state[2];
    if (flags & FLAG_TIE) {
        int* dst = a.tables + (size_t)k * TAB * TAB;
        for (int i = tid; i < TAB * TAB / 4; i += 128)
            __stcg(reinterpret_cast<int4*>(dst) + i, reinterpret_cast<const int4*>(&S.tab[0][0])[i]);
    }
    const int zero_d = S.tab[RMAX][RMAX + 1];
    __syncthreads();  // tab / h2t no longer needed: sub-pel scratch may overwrite the union

    // 6. sub-pel refinement (warp 0)
    if (warp == 0) {
        SubpelScratch& sp = S.u.sp;
        for (int i = lane; i < 22 * 22; i += 32) {
            int r = i / 22, c = i - r * 22;
            sp.patch[r][c] = S.win[my + 34 - 3 + r][mx + 48 - 3 + c];
        }
        __syncwarp();
        int qmx, qmy;
        subpel_refine_warp(sp, S.cur, lane, &minD, &qmx, &qmy);
        if (lane == 0) {
            int mvx = 4 * mx + qmx, mvy = 4 * my + qmy;
            a.spec_mv[k] = pack_mv(mvx, mvy);
            a.spec_imv[k] = pack_mv(mx, my);
            a.spec_min[k] = minD;
            a.spec_zero[k] = zero_d;
            a.spec_flags[k] = flags;
            __stcg(a.final_mv + k, pack_mv(mvx, mvy));
        }
    }
}

// ---------------------------------------------------------------------------
struct ResolveSmem {
    SubpelScratch sp[8];
    alignas(16) unsigned char cur[8][256];
    long long red_total[8];
    int red_count[8];
};

__device__ __forceinline__ void warp_load_cur(unsigned char* cur, const FullArgs& a, int n, int m, int lane)
{
    if (lane < 16)
        *reinterpret_cast<uint4*>(cur + 16 * lane) =
            *reinterpret_cast<const uint4*>(a.src8 + (size_t)(m + lane) * a.W + n);
    __syncwarp();
}

// One macroblock's dependent tail for a given prediction (Full.cpp:368-380,
// 401-446 rescan on ties, 452-517 sub-pel when the full-pel winner moved,
// 532-590 prediction distortion and Lagrangian pick).
__device__ void evaluate_mb(const FullArgs& a, int k, int px, int py, SubpelScratch& sp, unsigned char* cur, int lane,
                           int* out_mv, int* out_d)
{
    const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
    warp_load_cur(cur, a, n, m, lane);
    int mv = a.spec_mv[k];
    int mvx = mv_x(mv), mvy = mv_y(mv);
    int minD = a.spec_min[k];
    const int zd = a.spec_zero[k];
    if (a.spec_flags[k] & FLAG_TIE) {
        int prx = round_pred(px), pry = round_pred(py);
        if (prx != 0 || pry != 0) {
            int xl, xr, yu, yd, mx, my, md, tie;
            full_range(n, m, a.W, a.H, a.motion_range, xl, xr, yu, yd);
            scan_table(GlobalTab{a.tables + (size_t)k * TAB * TAB}, xl, xr, yu, yd, prx, pry, lane, &mx, &my, &md,
                       &tie);
            int imv = a.spec_imv[k];
            if (mx != mv_x(imv) || my != mv_y(imv)) {
                Plane8 rp{a.refp, a.rstride};
                load_patch22(sp.patch, rp, n + mx, m + my, lane);
                int qmx, qmy;
                subpel_refine_warp(sp, cur, lane, &md, &qmx, &qmy);
                mvx = 4 * mx + qmx;
                mvy = 4 * my + qmy;
                minD = md;
            }
        }
    }
    // prediction clamped to one macroblock outside the picture (Full.cpp:532-541)
    int pxq = px % 4, pyq = py % 4, px0 = px / 4, py0 = py / 4;
    if (px0 + n > a.W) px0 = 16;
    if (px0 + n < -16) px0 = -16;
    if (py0 + m > a.H) py0 = 16;
    if (py0 + m < -16) py0 = -16;
    int pcx = 4 * px0 + pxq, pcy = 4 * py0 + pyq;
    int fx = pxq < 0 ? pxq + 4 : pxq, fy = pyq < 0 ? pyq + 4 : pyq;
    int ox = n + px0 + (pxq < 0 ? -1 : 0), oy = m + py0 + (pyq < 0 ? -1 : 0);
    Plane8 rp{a.refp, a.rstride};
    load_patch22(sp.patch, rp, ox, oy, lane);
    int pd = qread_ssd_warp(sp.patch, cur, fx, fy, lane);
    int pos = best_of3(mvx, mvy, minD, pcx, pcy, pd, zd, a.lambda, 256.0, pcx, pcy);
    if (pos == 0) {
        *out_mv = pack_mv(mvx, mvy);
        *out_d = minD;
    } else if (pos == 1) {
        *out_mv = pack_mv(pcx, pcy);
        *out_d = pd;
    } else {
        *out_mv = pack_mv(0, 0);
        *out_d = zd;
    }
}

__global__ void __launch_bounds__(256) k_full_resolve(FullArgs a)
{
    __shared__ ResolveSmem S;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gwarp = blockIdx.x * 8 + wib, nwarps = gridDim.x * 8;
    SubpelScratch& sp = S.sp[wib];
    unsigned char* cur = S.cur[wib];
    int sweep = 0;
    bool ok = true;
    for (;; sweep++) {
        int changed = 0;
        for (int k = gwarp; k < a.nmb; k += nwarps) {
            int px, py;
            median_pred(a.final_mv, a.slice, k, a.cols, &px, &py);
            int pp = pack_mv(px, py);
            if (sweep > 0 && a.pred_used[k] == pp) continue;
            int fmv, fd;
            evaluate_mb(a, k, px, py, sp, cur, lane, &fmv, &fd);
            if (lane == 0) {
                a.pred_used[k] = pp;
                a.final_dist[k] = fd;
                if (__ldcg(a.final_mv + k) != fmv) {
                    __stcg(a.final_mv + k, fmv);
                    changed = 1;
                }
            }
            __syncwarp();
        }
        // one counter per sweep (zeroed before launch): no reset races
        if (lane == 0 && changed) atomicAdd(&a.changed[sweep], 1);
        ok = grid_sync(a.ctrl->bar, &a.ctrl->status, gridDim.x, a.spin_limit);
        if (!ok) break;
        if (*((volatile int*)&a.changed[sweep]) == 0) break;
        if (sweep + 1 >= a.sweep_limit) {
            if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&a.ctrl->status, ST_TIMEOUT);
            ok = false;
            break;
        }
    }
    // outputs and the included-distortion average (Full.cpp:581-611)
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
    if (!ok) return;
    if (!grid_sync(a.ctrl->bar, &a.ctrl->status, gridDim.x, a.spin_limit)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        long long t = *((volatile long long*)&a.ctrl->total);
        int c = *((volatile int*)&a.ctrl->count);
        if (a.out_avg) *a.out_avg = c ? t / c : 0;
        a.ctrl->sweeps = sweep + 1;
    }
}

}  // namespace

size_t full_search_smem() { return sizeof(SearchSmem); }

int full_launch(vppgpu_ctx* ctx, const FullArgs& args, int nmb, const short* d_src16, const short* d_ref16,
                int resolve_grid, cudaEvent_t* ev)
{
    if (ev) VPP_CUDA(cudaEventRecord(ev[0], ctx->stream));
    {
        long long work = (long long)((args.W + 2 * PAD) / 4) * (args.H + 2 * PAD) + (long long)args.W * args.H / 4;
        int grid = (int)((work + 255) / 256);
        if (grid > ctx->sm_count * 16) grid = ctx->sm_count * 16;
        k_full_pack<<<grid, 256, 0, ctx->stream>>>(d_src16, d_ref16, args.W, args.H, (unsigned char*)args.src8,
                                                   (unsigned char*)args.refp, args.rstride, &args.ctrl->status);
        VPP_CHECK_LAUNCH(ctx);
    }
    if (ev) VPP_CUDA(cudaEventRecord(ev[1], ctx->stream));
    k_full_search<<<nmb, 128, sizeof(SearchSmem), ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    if (ev) VPP_CUDA(cudaEventRecord(ev[2], ctx->stream));
    {
        void* params[] = {(void*)&args};
        VPP_CUDA(cudaLaunchCooperativeKernel((const void*)k_full_resolve, dim3(resolve_grid), dim3(256), params, 0,
                                             ctx->stream));
        ctx->launches++;
    }
    if (ev) VPP_CUDA(cudaEventRecord(ev[3], ctx->stream));
    return VPPGPU_OK;
}

int full_prepare(vppgpu_ctx* ctx, int nmb, int* resolve_grid)
{
    VPP_CUDA(cudaFuncSetAttribute(k_full_search, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(SearchSmem)));
    int per_sm = 0;
    VPP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_full_resolve, 256, 0));
    if (per_sm < 1) return VPPGPU_ERR_UNSUPPORTED;
    int want = (nmb + 7) / 8;
    int cap = per_sm * ctx->sm_count;
    *resolve_grid = want < cap ? want : cap;
    return VPPGPU_OK;
}

}  // namespace vppgpu
