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
//   k_full_halfpel  b / h / j half-pel planes of the padded reference, used
//                   by every distortion at a predicted vector.
//   resolve         (me_full_resolve.cu) the prediction-dependent tail:
//                   median prediction, tie rescans, prediction distortion
//                   and the Lagrangian pick, in the reference's raster order.
#include <string.h>

#include "me_full_common.cuh"

namespace vppgpu {
namespace {
using namespace full;

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
    int tie_nev[TIE_RUNS];
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

// ---------------------------------------------------------------------------
// Half-pel planes of the padded reference (the H.264 6-tap b, h and j
// samples QuarterRead combines, OverlayMem2Dv2.cpp): b(x,y) between x and
// x+1, h(x,y) between y and y+1, j from the unrounded vertical taps.  Four
// samples per thread; tap coordinates are clamped to the padded buffer, which
// only changes samples within three of its border, never read (a prediction
// stays within 17 samples of the picture, the padding is 48).
__device__ __forceinline__ unsigned char clip_tap(int v, int round, int shift)
{
    return (unsigned char)clip255((v + round) >> shift);
}

__global__ void __launch_bounds__(256) k_full_halfpel(const unsigned char* __restrict__ refp, int rstride, int PW,
                                                      int PH, unsigned char* __restrict__ hpel, size_t plane_size)
{
    const int qw = PW / 4;
    const long long total = (long long)qw * PH;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int Y = (int)(i / qw), X = 4 * (int)(i - (long long)Y * qw);
        // columns X-4 .. X+7 of rows Y-2 .. Y+3 as three words per row
        int g[6][12];
#pragma unroll
        for (int dy = 0; dy < 6; dy++) {
            const int yy = min(max(Y - 2 + dy, 0), PH - 1);
            const unsigned* row = reinterpret_cast<const unsigned*>(refp + (size_t)yy * rstride);
#pragma unroll
            for (int q = 0; q < 3; q++) {
                const int wq = min(max(X / 4 - 1 + q, 0), qw - 1);
                const unsigned w = __ldg(row + wq);
#pragma unroll
                for (int b = 0; b < 4; b++) g[dy][4 * q + b] = (w >> (8 * b)) & 0xff;
            }
        }
        // unrounded vertical taps at columns X-2 .. X+6 (g index 2 .. 10)
        int v[9];
#pragma unroll
        for (int c = 0; c < 9; c++) v[c] = tap6(g[0][c + 2], g[1][c + 2], g[2][c + 2], g[3][c + 2], g[4][c + 2], g[5][c + 2]);
        unsigned ob = 0, oh = 0, oj = 0;
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int x = t + 4;  // g index of column X + t
            const int bv = tap6(g[2][x - 2], g[2][x - 1], g[2][x], g[2][x + 1], g[2][x + 2], g[2][x + 3]);
            ob |= (unsigned)clip_tap(bv, 16, 5) << (8 * t);
            oh |= (unsigned)clip_tap(v[t + 2], 16, 5) << (8 * t);
            const int jv = tap6(v[t], v[t + 1], v[t + 2], v[t + 3], v[t + 4], v[t + 5]);
            oj |= (unsigned)clip_tap(jv, 512, 10) << (8 * t);
        }
        const size_t o = (size_t)Y * rstride + X;
        *reinterpret_cast<unsigned*>(hpel + o) = ob;
        *reinterpret_cast<unsigned*>(hpel + plane_size + o) = oh;
        *reinterpret_cast<unsigned*>(hpel + 2 * plane_size + o) = oj;
    }
}

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

    // 5. row minima, then the sequential scan replay (warp 0)
    int xl, xr, yu, yd;
    full_range(n, m, a.W, a.H, a.motion_range, xl, xr, yu, yd);
    table_row_minima(S.tab, xl, xr, yu, yd, warp, 4, lane);
    __syncthreads();
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
        for (int i = tid; i < TIE_ROW * TAB / 4; i += 128)
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
        const int qmv = pack_mv(4 * mx + qmx, 4 * my + qmy);
        int deep = 0;
        if (flags & FLAG_TIE) {
            // 7. tie tree: the runs reachable by some prediction
            int* tree = a.tables + (size_t)k * TAB * TAB + TIE_ROW * TAB;
            for (int p = 0; p < TIE_RUNS; p++) {
                if (p > 0) {
                    const int hb = 31 - __clz(p);
                    if (S.tie_nev[p & ~(1 << hb)] <= hb) {  // tie hb never met on that path
                        if (lane == 0) S.tie_nev[p] = 0;
                        __syncwarp();
                        continue;
                    }
                }
                int rmx, rmy, rmin, rt, nev, ev[TIE_DEPTH] = {0, 0, 0};
                scan_table_t<true>(SmemTab{S.tab}, xl, xr, yu, yd, 0, 0, p, lane, &rmx, &rmy, &rmin, &rt, &nev, ev);
                int rq = qmv, rqmin = minD;
                if (rmx != mx || rmy != my) {
                    __syncwarp();
                    for (int i = lane; i < 22 * 22; i += 32) {
                        int r = i / 22, c = i - r * 22;
                        sp.patch[r][c] = S.win[rmy + 34 - 3 + r][rmx + 48 - 3 + c];
                    }
                    __syncwarp();
                    int sx, sy;
                    subpel_refine_warp(sp, S.cur, lane, &rmin, &sx, &sy);
                    rq = pack_mv(4 * rmx + sx, 4 * rmy + sy);
                    rqmin = rmin;
                }
                if (lane == 0) {
                    int* run = tree + p * (int)(sizeof(TieRun) / sizeof(int));
                    run[0] = ev[0];
                    run[1] = ev[1];
                    run[2] = ev[2];
                    run[3] = nev;
                    run[4] = rq;
                    run[5] = rqmin;
                    S.tie_nev[p] = nev < 0 ? TIE_DEPTH + 1 : nev;
                }
                deep |= nev < 0;
                __syncwarp();
            }
        }
        if (lane == 0) {
            int av = neighbour_mask(a.slice, k, a.cols, a.nmb / a.cols);
            a.spec4[k] = make_int4(qmv, minD, zero_d, flags | av | (deep ? FLAG_DEEP : 0));
            a.spec_imv[k] = pack_mv(mx, my);
            __stcg(a.final_mv + k, qmv);
        }
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
    {
        const int PW = args.W + 2 * PAD, PH = args.H + 2 * PAD;
        long long work = (long long)(PW / 4) * PH;
        int grid = (int)((work + 255) / 256);
        if (grid > ctx->sm_count * 16) grid = ctx->sm_count * 16;
        k_full_halfpel<<<grid, 256, 0, ctx->stream>>>(args.refp, args.rstride, PW, PH, (unsigned char*)args.hpel,
                                                      args.plane_size);
        VPP_CHECK_LAUNCH(ctx);
    }
    if (ev) VPP_CUDA(cudaEventRecord(ev[1], ctx->stream));
    k_full_search<<<nmb, 128, sizeof(SearchSmem), ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    if (ev) VPP_CUDA(cudaEventRecord(ev[2], ctx->stream));
    int rc = full_resolve_launch(ctx, args, resolve_grid);
    if (rc) return rc;
    if (ev) VPP_CUDA(cudaEventRecord(ev[3], ctx->stream));
    return VPPGPU_OK;
}

int full_prepare(vppgpu_ctx* ctx, int nmb, int* resolve_grid)
{
    VPP_CUDA(cudaFuncSetAttribute(k_full_search, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(SearchSmem)));
    int cap = 0;
    int rc = full_resolve_prepare(ctx, &cap);
    if (rc) return rc;
    int want = (nmb + 7) / 8;
    *resolve_grid = want < cap ? want : cap;
    return VPPGPU_OK;
}

}  // namespace vppgpu
