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
//   k_full_table    one CTA per macroblock, every warp busy.  The whole
//                   (2R+1)^2 SSD table is computed as A2 + B2 - 2*sum(a*b):
//                   sum(a*b) with dp4a, window rows byte-aligned once per
//                   thread (funnel shifts) and held in a register ring, 4
//                   dp4a per 16-pixel row product; B2 by separable sliding
//                   sums in 16-wide runs; row minima; the table goes to
//                   global memory.
//   k_full_refine   one warp per macroblock, many per SM: the reference's
//                   sequential raster scan over the table (ballots; rows whose
//                   minimum cannot win are skipped) and the sub-pel stages.
//                   None of this depends on the predictor except exact ties
//                   in the scan, which are listed.
//   k_full_tietree  for the listed MBs, the scan outcome of every tie
//                   decision pattern (the tie tree), read by the
//                   prediction-dependent stage.
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

struct TableSmem {
    alignas(16) unsigned char win[WROWS][WSTRIDE];
    alignas(16) unsigned char cur[256];
    alignas(16) int tab[TAB][TAB];
    int h2t[TAB][H2STRIDE];  // h2t[jj][r] = sum_x win(r, jj+x)^2
    int a2;
};

struct TieSmem {
    alignas(16) int tab[TAB][TAB];
    int run[TIE_RUNS][sizeof(TieRun) / sizeof(int)];
};

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_full_pack(const JobDesc* __restrict__ job, int W, int H,
                                                  unsigned char* __restrict__ src8, unsigned char* __restrict__ refp,
                                                  int rstride, int* status)
{
    const short* __restrict__ src16 = job->src16;
    const short* __restrict__ ref16 = job->ref16;
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
// c + sum over the four bytes of |a - b| (unsigned bytes): the PTX SIMD
// video instruction with its accumulate form.
__device__ __forceinline__ unsigned sad4_add(unsigned a, unsigned b, unsigned c)
{
    unsigned d;
    asm("vabsdiff4.u32.u32.u32.add %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

// Table stage, one CTA per macroblock, every warp busy: the SSD (kSad: the
// SAD, OverlayMem2Dv2::Tad16x16, OverlayMem2Dv2.cpp:2655-2730) of all
// (2R+1)^2 full-pel candidates, its row minima, to the MB's global table.
// The SAD has no energy decomposition: each word pair is one vabsdiff4 with
// accumulate.
template <bool kSad>
__global__ void __launch_bounds__(128, 5) k_full_table(FullArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TableSmem& S = *reinterpret_cast<TableSmem*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int k = blockIdx.x;
    const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;

    // 1. window (rows m-31.., cols n-32..) and input block
    {
        const unsigned char* wbase = a.refp + (size_t)(m - 31 + PAD) * a.rstride + (n - 32 + PAD);
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

    // 2. template energy
    if (!kSad && tid < 32) {
        int acc = 0;
#pragma unroll
        for (int t = 0; t < 8; t++) {
            const int v = S.cur[tid + 32 * t];
            acc += v * v;
        }
        acc = warp_sum(acc);
        if (tid == 0) S.a2 = acc;
    }

    // 3. cross terms with dp4a; each thread: 8 candidate rows x 4 word offsets, one byte shift s.
    //    Each window row is byte-aligned once for the thread's shift (funnel shifts: word i
    //    holds bytes 4i+s .. 4i+s+3 of the thread's 32-byte slice) and kept in a ring of 8
    //    rows; then every 16-pixel row product is 4 dp4a against the template row.  The
    //    horizontal 16-sample energies of the thread's 4 columns come from the same aligned
    //    words (a self-dp4a per word and a sliding sum), for the window rows the thread owns
    //    (its first 8; rows 64..77 after the loop); they fill the issue slots the dp4a pipe
    //    leaves.
    unsigned acc[8][4];
    const int s = lane & 3, qg = (lane >> 2) & 3, ig = 2 * warp + (lane >> 4);
    const int ii0 = 8 * ig;
    {
        unsigned al[8][7];
        auto load_row = [&](unsigned* dst, int r) {
            const uint4* p = reinterpret_cast<const uint4*>(&S.win[r][16 * qg]);
            const uint4 x0 = p[0], x1 = p[1];
            const unsigned w[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
#pragma unroll
            for (int i = 0; i < 7; i++) dst[i] = __funnelshift_r(w[i], w[i + 1], 8 * s);
        };
        auto row_energy = [&](const unsigned* w, int r) {
            unsigned sq[7];
#pragma unroll
            for (int i = 0; i < 7; i++) sq[i] = __dp4a(w[i], w[i], 0u);
            unsigned e = sq[0] + sq[1] + sq[2] + sq[3];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (q) e += sq[q + 3] - sq[q - 1];
                S.h2t[16 * qg + 4 * q + s][r] = (int)e;
            }
        };
#pragma unroll
        for (int r = 0; r < 8; r++) {
            load_row(al[r], ii0 + r);
            if (!kSad) row_energy(al[r], ii0 + r);
        }
#pragma unroll
        for (int r = 0; r < 8; r++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[r][q] = 0u;
#pragma unroll
        for (int y = 0; y < 16; y++) {
            const uint4 t = *reinterpret_cast<const uint4*>(&S.cur[16 * y]);
            const unsigned A[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
            for (int r = 0; r < 8; r++) {
                const unsigned* B = al[(r + y) & 7];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    unsigned c = acc[r][q];
#pragma unroll
                    for (int w = 0; w < 4; w++)
                        c = kSad ? sad4_add(A[w], B[q + w], c) : __dp4a(A[w], B[q + w], c);
                    acc[r][q] = c;
                }
            }
            if (y < 15) load_row(al[y & 7], ii0 + y + 8);
        }
    }
    // energies of window rows 64..77 (below every row group's own rows): 14 rows x 16 slices
    for (int task = kSad ? (WROWS - 64) * 16 : tid; task < (WROWS - 64) * 16; task += 128) {
        const int r = 64 + (task >> 4), c = task & 15, ts = c & 3, tq = c >> 2;
        const uint4* p = reinterpret_cast<const uint4*>(&S.win[r][16 * tq]);
        const uint4 x0 = p[0], x1 = p[1];
        const unsigned w[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
        unsigned sq[7];
#pragma unroll
        for (int i = 0; i < 7; i++) {
            const unsigned v = __funnelshift_r(w[i], w[i + 1], 8 * ts);
            sq[i] = __dp4a(v, v, 0u);
        }
        unsigned e = sq[0] + sq[1] + sq[2] + sq[3];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (q) e += sq[q + 3] - sq[q - 1];
            S.h2t[16 * tq + 4 * q + ts][r] = (int)e;
        }
    }
    __syncthreads();

    // 4. vertical 16-row sums of the horizontal energies (task: column jj, run ib), then
    //    SSD = A^2 + B^2 - 2 sum(ab) for every candidate
    for (int task = kSad ? TAB * 4 : tid; task < TAB * 4; task += 128) {
        const int jj = task & (TAB - 1), ib = task >> 6;
        const int* col = S.h2t[jj];
        const int r0 = 16 * ib, r1 = min(r0 + 16, 2 * RMAX + 1);
        int sum = 0;
#pragma unroll
        for (int y = 0; y < 16; y++) sum += col[r0 + y];
        S.tab[r0][jj] = sum;
        for (int ii = r0 + 1; ii < r1; ii++) {
            sum += col[ii + 15] - col[ii - 1];
            S.tab[ii][jj] = sum;
        }
    }
    __syncthreads();
    {
        const int a2 = kSad ? 0 : S.a2;
#pragma unroll
        for (int r = 0; r < 8; r++) {
            int ii = ii0 + r;
            if (ii < 2 * RMAX + 1) {
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    int jj = 4 * (4 * qg + q) + s;
                    S.tab[ii][jj] = kSad ? (int)acc[r][q] : a2 + S.tab[ii][jj] - 2 * (int)acc[r][q];
                }
            }
        }
    }
    __syncthreads();

    // 5. row minima, then the table (rows 0 .. 2R) to global memory
    int xl, xr, yu, yd;
    full_range(n, m, a.W, a.H, a.motion_range, xl, xr, yu, yd);
    table_row_minima(S.tab, xl, xr, yu, yd, warp, 4, lane);
    __syncthreads();
    int4* dst = reinterpret_cast<int4*>(a.tables + (size_t)k * TAB * TAB);
    for (int i = tid; i < (2 * RMAX + 1) * TAB / 4; i += 128) __stcg(dst + i, reinterpret_cast<const int4*>(&S.tab[0][0])[i]);
}

// ---------------------------------------------------------------------------
// Refine stage, one warp per macroblock: the reference's sequential scan
// over the table (prediction (0,0) for ties), then the half/quarter-pel
// stages around the winner.  MBs whose scan met an exact tie go to the tie
// list for their tie tree.
__global__ void __launch_bounds__(256, 4) k_full_refine(FullArgs a)
{
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int k = blockIdx.x * 8 + wib;
    if (k >= a.nmb) return;
    const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
    const int* gt = a.tables + (size_t)k * TAB * TAB;
    const uint2 cur = load_cur8(a, n, m, lane);
    int xl, xr, yu, yd, mx, my, minD, tie;
    full_range(n, m, a.W, a.H, a.motion_range, xl, xr, yu, yd);
    scan_table(GlobalTab{gt}, xl, xr, yu, yd, 0, 0, lane, &mx, &my, &minD, &tie);
    const int zero_d = __ldcg(gt + RMAX * TAB + RMAX + 1);
    int qmx = 0, qmy = 0;
    if (!a.intpel) subpel_refine_planes(a, n + mx, m + my, cur, lane, &minD, &qmx, &qmy);
    if (lane == 0) {
        const int qmv = pack_mv(4 * mx + qmx, 4 * my + qmy);
        const int av = neighbour_mask(a.job->slice, k, a.cols, a.nmb / a.cols);
        a.spec4[k] = make_int4(qmv, minD, zero_d, (tie ? FLAG_TIE : 0) | av);
        a.spec_imv[k] = pack_mv(mx, my);
        __stcg(a.final_mv + k, qmv);
        if (tie) a.tie_list[atomicAdd(&a.ctrl->ntie, 1)] = k;
    }
}

// ---------------------------------------------------------------------------
// Tie trees of the listed macroblocks (see TieRun), one CTA per MB: the table
// in shared memory, warp p computes run p (forced scan, then the sub-pel
// stage of its winner when that is not the searched one).  FLAG_DEEP when a
// run reachable by some prediction met more ties than the tree holds (the
// prediction-dependent stage then rescans).
__global__ void __launch_bounds__(TIE_RUNS * 32) k_full_tietree(FullArgs a)
{
    extern __shared__ __align__(16) unsigned char tie_smem[];
    TieSmem& S = *reinterpret_cast<TieSmem*>(tie_smem);
    const int tid = threadIdx.x, lane = tid & 31, p = tid >> 5;
    const int ntie = *((volatile int*)&a.ctrl->ntie);
    for (int t = blockIdx.x; t < ntie; t += gridDim.x) {
        const int k = a.tie_list[t];
        const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
        int* gt = a.tables + (size_t)k * TAB * TAB;
        for (int i = tid; i < (2 * RMAX + 1) * TAB / 4; i += blockDim.x)
            reinterpret_cast<int4*>(&S.tab[0][0])[i] = __ldcg(reinterpret_cast<const int4*>(gt) + i);
        __syncthreads();
        int xl, xr, yu, yd;
        full_range(n, m, a.W, a.H, a.motion_range, xl, xr, yu, yd);
        const int4 sp = a.spec4[k];
        const int imv = a.spec_imv[k];
        int rmx, rmy, rmin, rt, nev, ev[TIE_DEPTH] = {0, 0, 0};
        scan_table_t<true>(SmemTab{S.tab}, xl, xr, yu, yd, 0, 0, p, lane, &rmx, &rmy, &rmin, &rt, &nev, ev);
        int rq = sp.x, rqmin = sp.y;
        if (rmx != mv_x(imv) || rmy != mv_y(imv)) {
            int sx = 0, sy = 0;
            if (!a.intpel) subpel_refine_planes(a, n + rmx, m + rmy, load_cur8(a, n, m, lane), lane, &rmin, &sx, &sy);
            rq = pack_mv(4 * rmx + sx, 4 * rmy + sy);
            rqmin = rmin;
        }
        if (lane == 0) {
            S.run[p][0] = ev[0];
            S.run[p][1] = ev[1];
            S.run[p][2] = ev[2];
            S.run[p][3] = nev;
            S.run[p][4] = rq;
            S.run[p][5] = rqmin;
        }
        __syncthreads();
        constexpr int RW = sizeof(TieRun) / sizeof(int);
        if (tid < TIE_RUNS * RW) gt[TIE_ROW * TAB + tid] = S.run[tid / RW][tid % RW];
        if (tid == 0) {
            // runs a prediction can reach: run p needs tie hb(p) met on the path of p without that bit
            bool reach[TIE_RUNS];
            bool deep = S.run[0][3] < 0;
            reach[0] = true;
            for (int q = 1; q < TIE_RUNS; q++) {
                const int hb = 31 - __clz(q), par = q & ~(1 << hb);
                const int pn = S.run[par][3] < 0 ? TIE_DEPTH + 1 : S.run[par][3];
                reach[q] = reach[par] && pn > hb;
                deep |= reach[q] && S.run[q][3] < 0;
            }
            if (deep) a.spec4[k].w = sp.w | FLAG_DEEP;
        }
        __syncthreads();
    }
}

__global__ void k_set_job(JobDesc* dst, JobDesc v) { *dst = v; }

}  // namespace

int set_job(vppgpu_ctx* ctx, JobDesc* d_job, const JobDesc& v)
{
    k_set_job<<<1, 1, 0, ctx->stream>>>(d_job, v);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

size_t full_search_smem() { return sizeof(TableSmem); }

int full_planes_launch(vppgpu_ctx* ctx, const FullArgs& args)
{
    {
        long long work = (long long)((args.W + 2 * PAD) / 4) * (args.H + 2 * PAD) + (long long)args.W * args.H / 4;
        int grid = (int)((work + 255) / 256);
        if (grid > ctx->sm_count * 16) grid = ctx->sm_count * 16;
        k_full_pack<<<grid, 256, 0, ctx->stream>>>(args.job, args.W, args.H, (unsigned char*)args.src8,
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
    return VPPGPU_OK;
}

int full_launch(vppgpu_ctx* ctx, const FullArgs& args, int nmb, int resolve_grid, cudaEvent_t* ev)
{
    if (ev) VPP_CUDA(cudaEventRecord(ev[0], ctx->stream));
    int rc = full_planes_launch(ctx, args);
    if (rc) return rc;
    if (ev) VPP_CUDA(cudaEventRecord(ev[1], ctx->stream));
    k_full_table<false><<<nmb, 128, sizeof(TableSmem), ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    if (ev) VPP_CUDA(cudaEventRecord(ev[2], ctx->stream));
    k_full_refine<<<(nmb + 7) / 8, 256, 0, ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    k_full_tietree<<<ctx->sm_count, TIE_RUNS * 32, sizeof(TieSmem), ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    if (ev) VPP_CUDA(cudaEventRecord(ev[3], ctx->stream));
    rc = full_resolve_launch(ctx, args, resolve_grid, 0);
    if (rc) return rc;
    if (ev) VPP_CUDA(cudaEventRecord(ev[4], ctx->stream));
    return VPPGPU_OK;
}

// The integer-pel SAD stage (FullArgs::intpel): planes, the SAD table, the
// scan at prediction (0, 0) without sub-pel, tie trees, then the tie wavefront.
int sad_launch(vppgpu_ctx* ctx, const FullArgs& args, int nmb)
{
    int rc = full_planes_launch(ctx, args);
    if (rc) return rc;
    k_full_table<true><<<nmb, 128, sizeof(TableSmem), ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    k_full_refine<<<(nmb + 7) / 8, 256, 0, ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    k_full_tietree<<<ctx->sm_count, TIE_RUNS * 32, sizeof(TieSmem), ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    return sad_resolve_launch(ctx, args);
}

int full_prepare(vppgpu_ctx* ctx, int nmb, int* resolve_grid)
{
    VPP_CUDA(cudaFuncSetAttribute(k_full_table<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(TableSmem)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_table<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(TableSmem)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_tietree, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(TieSmem)));
    int cap = 0;
    int rc = full_resolve_prepare(ctx, &cap);
    if (rc) return rc;
    int want = (nmb + 7) / 8;
    *resolve_grid = want < cap ? want : cap;
    return VPPGPU_OK;
}

}  // namespace vppgpu
