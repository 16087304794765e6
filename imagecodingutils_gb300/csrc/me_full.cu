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
//   k_full_planes   one pass over tiles of the padded reference: int16 ->
//                   u8 (with a 0..255 check) and edge replication, the b / h /
//                   j half-pel planes (sub-pel stages, every distortion at a
//                   predicted vector) and the 16x16 block energies (the B^2 of
//                   every candidate's SSD = A^2 + B^2 - 2 sum(ab)); the input's
//                   byte packing rides along.
//   k_full_search   persistent, warp-specialised: compute warps build each
//                   macroblock's (2R+1)^2 SSD table in shared memory (cross
//                   terms with dp4a, tiles staged by TMA tensor copies), a scan
//                   warp replays the reference's sequential raster scan over
//                   it (rows whose minimum or range cannot win are skipped).
//                   Only the tables of macroblocks whose scan met an exact tie
//                   leave the SM (for their tie tree).
//   k_full_subpel   half-pel then quarter-pel refinement, a warp per MB.
//   k_full_tietree  for the tie MBs, the scan outcome of every tie decision
//                   pattern (the tie tree), read by the prediction-dependent
//                   stage.
//   resolve         (me_full_resolve.cu) the prediction-dependent tail:
//                   median prediction, tie rescans, prediction distortion
//                   and the Lagrangian pick, in the reference's raster order.
#include <string.h>

#include <cudaTypedefs.h>
#include <mutex>

#include "me_full_common.cuh"

namespace vppgpu {
namespace {
using namespace full;

struct TieSmem {
    alignas(16) int tab[TAB][TAB];
    int run[TIE_RUNS][sizeof(TieRun) / sizeof(int)];
};

// ---------------------------------------------------------------------------
// The frame's planes in one pass, a CTA per PL_TX x PL_TY tile of the padded
// reference (PAD samples of edge replication each side, OverlayExtMem2Dv2's
// extended boundary as a coordinate clamp):
//   refp    the padded reference as bytes (0..255 checked)
//   hpel    its H.264 half-pel planes, b (x half: 6-tap (1,-5,20,20,-5,1) on
//           the row, (+16) >> 5), h (y half, on the column) and j (centre:
//           the 6-tap over the unrounded vertical taps, (+512) >> 10), each
//           clipped to 0..255 -- the samples QuarterRead combines
//           (OverlayMem2Dv2.cpp:704-1052)
//   energy  (SSD search only) E(Y, X) = sum of squares of the 16x16 block at
//           (Y, X), for Y <= PH-16, X <= PW-16: the B^2 term of every
//           candidate's SSD = A^2 + B^2 - 2 sum(ab)
// plus a share of the input's byte packing (src8, 0..255 checked).  The tile
// and its halo (2 before, 15 after in each direction) are staged once as
// bytes; taps read clamped coordinates, which differs from a clamped padded
// plane only within 3 samples of its border, never read (a prediction stays
// within 17 samples of the picture).
constexpr int PL_TX = 64, PL_TY = 32;
constexpr int PL_SX = PL_TX + 20, PL_SY = PL_TY + 17;  // staged columns X0-2 .. X0+81, rows Y0-2 .. Y0+46

__device__ __forceinline__ unsigned char clip_tap(int v, int round, int shift)
{
    return (unsigned char)clip255((v + round) >> shift);
}

__global__ void __launch_bounds__(256) k_full_planes(const JobDesc* __restrict__ job, int W, int H, int rstride,
                                                     unsigned char* __restrict__ src8, unsigned char* __restrict__ refp,
                                                     unsigned char* __restrict__ hpel, size_t plane_size,
                                                     int* __restrict__ energy, int* status)
{
    __shared__ __align__(16) unsigned char px[PL_SY][PL_SX];
    __shared__ short vt[PL_TY][PL_TX + 5];            // unrounded vertical taps, columns X0-2 .. X0+66
    __shared__ int hs[PL_TY + 15][PL_TX];             // horizontal 16-sums of squares (energy)
    const short* __restrict__ ref16 = job->ref16;
    const int PW = rstride, PH = H + 2 * PAD;
    const int X0 = blockIdx.x * PL_TX, Y0 = blockIdx.y * PL_TY, tid = threadIdx.x;
    bool bad = false;
    // 1. stage: padded (Y, X) -> frame (clamp(Y - PAD), clamp(X - PAD)), 2 samples per thread step
    for (int i = tid; i < PL_SY * (PL_SX / 2); i += 256) {
        const int r = i / (PL_SX / 2), c = 2 * (i - r * (PL_SX / 2));
        const int y = min(max(Y0 - 2 + r - PAD, 0), H - 1);
        const short* row = ref16 + (size_t)y * W;
        const int v0 = row[min(max(X0 - 2 + c - PAD, 0), W - 1)];
        const int v1 = row[min(max(X0 - 1 + c - PAD, 0), W - 1)];
        bad |= (v0 < 0) | (v0 > 255) | (v1 < 0) | (v1 > 255);
        px[r][c] = (unsigned char)v0;
        px[r][c + 1] = (unsigned char)v1;
    }
    // the input's byte packing, a share per CTA (4 samples per thread step)
    {
        const long long nq = (long long)W * H / 4, nb = (long long)gridDim.x * gridDim.y;
        const long long b = (long long)blockIdx.y * gridDim.x + blockIdx.x;
        const short2* s2 = reinterpret_cast<const short2*>(job->src16);
        for (long long j = b * 256 + tid; j < nq; j += nb * 256) {
            const short2 p = s2[2 * j], q = s2[2 * j + 1];
            const int v0 = p.x, v1 = p.y, v2 = q.x, v3 = q.y;
            bad |= (v0 < 0) | (v0 > 255) | (v1 < 0) | (v1 > 255) | (v2 < 0) | (v2 > 255) | (v3 < 0) | (v3 > 255);
            reinterpret_cast<unsigned*>(src8)[j] = (unsigned)(v0 & 0xff) | ((unsigned)(v1 & 0xff) << 8) |
                                                   ((unsigned)(v2 & 0xff) << 16) | ((unsigned)(v3 & 0xff) << 24);
        }
    }
    if (__any_sync(0xffffffffu, bad) && (tid & 31) == 0) atomicOr(status, ST_PIXEL_RANGE);
    __syncthreads();
    // 2. vertical taps at rows Y0 .. Y0+31, columns X0-2 .. X0+66 (staged rows r .. r+5, column c)
    for (int i = tid; i < PL_TY * (PL_TX + 5); i += 256) {
        const int r = i / (PL_TX + 5), c = i - r * (PL_TX + 5);
        vt[r][c] = (short)tap6(px[r][c], px[r + 1][c], px[r + 2][c], px[r + 3][c], px[r + 4][c], px[r + 5][c]);
    }
    if (energy) {  // horizontal 16-sums of squares, rows Y0 .. Y0+46 (staged row r + 2), columns X0 ..
        for (int t = tid; t < (PL_TY + 15) * (PL_TX / 16); t += 256) {
            const int r = t >> 2, c0 = 16 * (t & 3);
            const unsigned char* p = &px[r + 2][c0 + 2];
            int acc = 0;
#pragma unroll
            for (int d = 0; d < 16; d++) acc += p[d] * p[d];
            hs[r][c0] = acc;
#pragma unroll
            for (int c = 1; c < 16; c++) {
                acc += p[c + 15] * p[c + 15] - p[c - 1] * p[c - 1];
                hs[r][c0 + c] = acc;
            }
        }
    }
    __syncthreads();
    // 3. bytes and half-pel samples, 4 columns per thread task
    for (int t = tid; t < PL_TY * (PL_TX / 4); t += 256) {
        const int r = t >> 4, cq = 4 * (t & 15);
        const int Y = Y0 + r, X = X0 + cq;
        if (Y >= PH || X >= PW) continue;  // PW is a multiple of 16: a task is inside or outside whole
        const unsigned char* row = &px[r + 2][cq + 2];  // sample (Y, X)
        unsigned og = 0, ob = 0, oh = 0, oj = 0;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            og |= (unsigned)row[u] << (8 * u);
            const int bv = tap6(row[u - 2], row[u - 1], row[u], row[u + 1], row[u + 2], row[u + 3]);
            ob |= (unsigned)clip_tap(bv, 16, 5) << (8 * u);
            const short* v = &vt[r][cq + u];  // columns X+u-2 .. X+u+3
            oh |= (unsigned)clip_tap(v[2], 16, 5) << (8 * u);
            const int jv = tap6(v[0], v[1], v[2], v[3], v[4], v[5]);
            oj |= (unsigned)clip_tap(jv, 512, 10) << (8 * u);
        }
        const size_t o = (size_t)Y * rstride + X;
        *reinterpret_cast<unsigned*>(refp + o) = og;
        *reinterpret_cast<unsigned*>(hpel + o) = ob;
        *reinterpret_cast<unsigned*>(hpel + plane_size + o) = oh;
        *reinterpret_cast<unsigned*>(hpel + 2 * plane_size + o) = oj;
    }
    if (energy) {  // vertical 16-sums: column c, 16 rows per task
        for (int t = tid; t < PL_TX * (PL_TY / 16); t += 256) {
            const int c = t & (PL_TX - 1), r0 = 16 * (t >> 6), X = X0 + c;
            int acc = 0;
#pragma unroll
            for (int d = 0; d < 16; d++) acc += hs[r0 + d][c];
#pragma unroll
            for (int r = r0; r < r0 + 16; r++) {
                if (r > r0) acc += hs[r + 15][c] - hs[r - 1][c];
                const int Y = Y0 + r;
                if (X <= PW - 16 && Y <= PH - 16) energy[(size_t)Y * rstride + X] = acc;
            }
        }
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

// ---------------------------------------------------------------------------
// Search stage: one persistent CTA per slot (SEARCH_CTAS_PER_SM per SM),
// macroblocks blockIdx.x, blockIdx.x + gridDim.x, ...; warp-specialised.
//
//   compute warps      the SSD (kSad: the SAD, OverlayMem2Dv2::Tad16x16,
//                      OverlayMem2Dv2.cpp:2655-2730) of all (2R+1)^2 full-pel
//                      candidates of a macroblock into a shared-memory table,
//                      with its row minima; warp 0 also stages the next
//                      macroblock's window and template (TMA tensor copies)
//   scan warp (1)      the reference's sequential raster scan over each
//                      table (prediction (0, 0) for ties, Full.cpp:394-446);
//                      tables of macroblocks whose scan met an exact tie go to
//                      global memory for their tie tree; then, in the buffer
//                      it released, it stages the energies of the candidates
//                      two macroblocks on (a TMA copy; the SSDs overwrite them
//                      in place), so the compute warps never wait for a scan
//                      unless it falls two tables behind.  The sub-pel stages
//                      follow in k_full_subpel, whose global-memory round trips
//                      would otherwise lengthen the scan warp's chain.
//
// Two window buffers and two table buffers; the hand-offs are shared-memory
// barriers (mbarrier) whose waits are bounded: a wait that runs out sets
// ST_TIMEOUT and every role leaves, after the copies it issued landed.
// Launch shape, measured on 1080p frames: 8 candidate rows per thread with the
// template rows in two passes of the ring's period (a loop body small enough
// for the instruction cache; the full 16-step unroll stalled on instruction
// fetch, 0.179 against 0.167 ms), at 3 CTAs per SM, where the loop needs no
// spills (4 CTAs with a 96-register cap: the same time; 4 candidate rows per
// thread, i.e. 8 compute warps, took 0.182 ms at 3 CTAs and 0.190 ms at 2).
constexpr int SEARCH_ROWS = 8;    // candidate rows per thread (the window-row ring's period)
constexpr int SEARCH_UNROLL = 8;  // template rows per unrolled loop body (a multiple of SEARCH_ROWS)
constexpr int SEARCH_WARPS = 64 / (2 * SEARCH_ROWS);  // compute warps: 2 row groups of a warp each
constexpr int SEARCH_THREADS = 32 * (SEARCH_WARPS + 1);
constexpr int SEARCH_CTAS_PER_SM = 3;
constexpr unsigned WIN_BYTES = WROWS * WSTRIDE + 256;     // window rows + template
constexpr unsigned E_BYTES = (2 * RMAX + 1) * TAB * 4;    // candidate rows of energies
// one window, 128-byte aligned, with room for a row 78 that the TMA box does
// not fill (only the unused candidate row 63 reads it)
constexpr int WIN_BUF = (WROWS * WSTRIDE + WSTRIDE + 127) / 128 * 128;
static_assert(SEARCH_UNROLL % SEARCH_ROWS == 0 && 16 % SEARCH_UNROLL == 0, "unroll must cover ring periods");

struct SearchSmem {
    alignas(128) int tab[2][TAB][TAB];  // rows 0 .. 2R: SSDs (column 0: row minima)
    alignas(128) unsigned char win[2][WIN_BUF];  // WROWS rows of WSTRIDE bytes
    alignas(128) unsigned char cur[2][256];
    unsigned long long wfull[2];   // window b staged
    unsigned long long wfree[2];   // window b read by every compute thread
    unsigned long long efull[2];   // SSD: energies staged in table b (the scan released it)
    unsigned long long tfull[2];   // table b written by every compute thread
    unsigned long long tempty[2];  // SAD: table b released by the scan warp
    int abort;
};

// Bounded wait for the phase of parity `par`; false when the search is
// abandoned (this wait ran out, or another role's did).
__device__ __forceinline__ bool search_wait(unsigned long long* bar, unsigned par, const FullArgs& a,
                                            volatile int* abort)
{
    long long it = 0;
    while (!mbar_try_wait(bar, par)) {
        if (*abort) return false;
        if (++it > a.spin_limit) {
            atomicOr(&a.ctrl->status, ST_TIMEOUT);
            *abort = 1;
            return false;
        }
    }
    return true;
}

// Wait (bounded, abort ignored) for the stagings [from, to) on a pair of
// barriers: copies must land before the CTA leaves.
__device__ __forceinline__ void search_drain(unsigned long long* bars, int from, int to, long long limit)
{
    for (int i = from; i < to; i++) {
        long long w = 0;
        while (!mbar_try_wait(&bars[i & 1], (unsigned)(i >> 1) & 1u) && ++w <= limit) {}
    }
}

template <bool kSad>
__global__ void __launch_bounds__(SEARCH_THREADS, SEARCH_CTAS_PER_SM)
    k_full_search(FullArgs a, const __grid_constant__ SearchMaps maps)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SearchSmem& S = *reinterpret_cast<SearchSmem*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nit = (a.nmb - 1 - (int)blockIdx.x) / (int)gridDim.x + 1;  // grid <= nmb: at least one
    volatile int* abort = &S.abort;
    if (tid == 0) {
        for (int b = 0; b < 2; b++) {
            mbar_init(&S.wfull[b], 1);
            mbar_init(&S.wfree[b], 32 * SEARCH_WARPS);
            mbar_init(&S.efull[b], 1);
            mbar_init(&S.tfull[b], 32 * SEARCH_WARPS);
            mbar_init(&S.tempty[b], 32);
        }
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    auto mb_of = [&](int it) { return (int)blockIdx.x + it * (int)gridDim.x; };

    if (warp < SEARCH_WARPS) {
        // ---------------- compute warps ----------------
        // warp 0 stages the window + template of iteration `it` into buffer it & 1
        auto stage_window = [&](int it) {
            if (lane == 0) {
                const int b = it & 1, k = mb_of(it);
                const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
                mbar_expect_tx(&S.wfull[b], WIN_BYTES);
                tma_load_2d(S.win[b], &maps.win, n - 32 + PAD, m - 31 + PAD, &S.wfull[b]);
                tma_load_2d(S.cur[b], &maps.cur, n, m, &S.wfull[b]);
            }
        };
        int wissued = 0;  // warp 0: windows staged for iterations 0 .. wissued-1
        if (warp == 0) {
            stage_window(0);
            wissued = 1;
        }
        const int s = lane & 3, qg = (lane >> 2) & 3, ig = 2 * warp + (lane >> 4);
        const int ii0 = SEARCH_ROWS * ig;
        int it = 0;
        for (; it < nit; it++) {
            const int b = it & 1;
            const unsigned use = (unsigned)(it >> 1) & 1u;  // parity of this buffer's use
            if (warp == 0 && it + 1 < nit) {
                // window buffer b^1 was read in iteration it-1 (its first use: free from the start)
                if (!search_wait(&S.wfree[b ^ 1], ((unsigned)((it + 1) >> 1) & 1u) ^ 1u, a, abort)) break;
                stage_window(it + 1);
                wissued = it + 2;
            }
            if (!search_wait(&S.wfull[b], use, a, abort)) break;

            // cross terms with dp4a (kSad: vabsdiff4 with accumulate); each thread:
            // SEARCH_ROWS candidate rows x 4 word offsets, one byte shift s.  Each window
            // row is byte-aligned once for the thread's shift (funnel shifts: word i holds
            // bytes 4i+s .. 4i+s+3 of the thread's 32-byte slice) and kept in a ring of
            // SEARCH_ROWS rows; every 16-pixel row product is then 4 dp4a against the
            // template row.
            unsigned acc[SEARCH_ROWS][4];
            {
                unsigned al[SEARCH_ROWS][7];
                auto load_row = [&](unsigned* dst, int r) {
                    const uint4* p = reinterpret_cast<const uint4*>(&S.win[b][r * WSTRIDE + 16 * qg]);
                    const uint4 x0 = p[0], x1 = p[1];
                    const unsigned w[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
#pragma unroll
                    for (int i = 0; i < 7; i++) dst[i] = __funnelshift_r(w[i], w[i + 1], 8 * s);
                };
#pragma unroll
                for (int r = 0; r < SEARCH_ROWS; r++) load_row(al[r], ii0 + r);
#pragma unroll
                for (int r = 0; r < SEARCH_ROWS; r++)
#pragma unroll
                    for (int q = 0; q < 4; q++) acc[r][q] = 0u;
#pragma unroll 1
                for (int yq = 0; yq < 16; yq += SEARCH_UNROLL) {
#pragma unroll
                    for (int yu = 0; yu < SEARCH_UNROLL; yu++) {
                        const int y = yq + yu;
                        const uint4 t = *reinterpret_cast<const uint4*>(&S.cur[b][16 * y]);
                        const unsigned A[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
                        for (int r = 0; r < SEARCH_ROWS; r++) {
                            const unsigned* B = al[(r + yu) % SEARCH_ROWS];
#pragma unroll
                            for (int q = 0; q < 4; q++) {
                                unsigned c = acc[r][q];
#pragma unroll
                                for (int w = 0; w < 4; w++)
                                    c = kSad ? sad4_add(A[w], B[q + w], c) : __dp4a(A[w], B[q + w], c);
                                acc[r][q] = c;
                            }
                        }
                        if (y < 15) load_row(al[yu % SEARCH_ROWS], ii0 + y + SEARCH_ROWS);
                    }
                }
            }
            // template energy
            int a2 = 0;
            if (!kSad) {
#pragma unroll
                for (int t = 0; t < 8; t++) {
                    const int v = S.cur[b][lane + 32 * t];
                    a2 += v * v;
                }
                a2 = warp_sum(a2);
            }
            mbar_arrive(&S.wfree[b]);  // this thread is done with window b and its template

            // the table buffer: its energies staged (the scan warp stages them once it released
            // the buffer), or, for the SAD, released
            if (!search_wait(kSad ? &S.tempty[b] : &S.efull[b], kSad ? use ^ 1u : use, a, abort)) break;
            const int k = mb_of(it);
            const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
            int xl, xr, yu, yd;
            full_range(n, m, a.W, a.H, a.motion_range, xl, xr, yu, yd);
#pragma unroll
            for (int r = 0; r < SEARCH_ROWS; r++) {
                const int ii = ii0 + r;
                int v[4], mn = 0x7fffffff;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int jj = 16 * qg + 4 * q + s;
                    v[q] = kSad ? (int)acc[r][q] : a2 + (ii < 2 * RMAX + 1 ? S.tab[b][ii][jj] : 0) - 2 * (int)acc[r][q];
                    const int j = jj - RMAX - 1;
                    if (j >= xl && j <= xr) mn = min(mn, v[q]);
                }
#pragma unroll
                for (int o = 1; o < 16; o <<= 1) mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
                if (ii < 2 * RMAX + 1) {
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const int jj = 16 * qg + 4 * q + s;
                        S.tab[b][ii][jj] = jj == 0 ? mn : v[q];  // column 0 (outside every range): the row minimum
                    }
                }
            }
            mbar_arrive(&S.tfull[b]);
        }
        if (warp == 0) search_drain(S.wfull, it, wissued, a.spin_limit);
    } else {
        // ---------------- scan warp ----------------
        // energies of iteration `it`'s candidates into table buffer it & 1 (SSD)
        auto stage_energy = [&](int it) {
            if (lane == 0) {
                const int b = it & 1, k = mb_of(it);
                const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
                mbar_expect_tx(&S.efull[b], E_BYTES);
                tma_load_2d(&S.tab[b][0][0], &maps.energy, n - 32 + PAD, m - 31 + PAD, &S.efull[b]);
            }
        };
        int eissued = 0;  // energies staged for iterations 0 .. eissued-1
        if (!kSad) {      // both table buffers start free
            eissued = min(nit, 2);
            for (int i = 0; i < eissued; i++) stage_energy(i);
        }
        int it = 0;
        for (; it < nit; it++) {
            const int b = it & 1;
            const int k = mb_of(it);
            const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
            if (!search_wait(&S.tfull[b], (unsigned)(it >> 1) & 1u, a, abort)) break;
            int xl, xr, yu, yd, mx, my, minD, tie;
            full_range(n, m, a.W, a.H, a.motion_range, xl, xr, yu, yd);
            scan_table(SmemTab{S.tab[b]}, xl, xr, yu, yd, 0, 0, lane, &mx, &my, &minD, &tie);
            const int zero_d = S.tab[b][RMAX][RMAX + 1];
            if (tie) {  // its tie tree (and deep rescans) read the table from global memory
                int4* dst = reinterpret_cast<int4*>(a.tables + (size_t)k * TAB * TAB);
                const int4* src = reinterpret_cast<const int4*>(&S.tab[b][0][0]);
                for (int i = lane; i < (2 * RMAX + 1) * TAB / 4; i += 32) __stcg(dst + i, src[i]);
            }
            __syncwarp();
            if (kSad) {
                mbar_arrive(&S.tempty[b]);
            } else if (it + 2 < nit) {
                stage_energy(it + 2);  // the buffer is released: the table two iterations on
                eissued = it + 3;
            }
            if (lane == 0) {  // the full-pel result; k_full_subpel refines it (SSD search)
                const int qmv = pack_mv(4 * mx, 4 * my);
                const int av = neighbour_mask(a.job->slice, k, a.cols, a.nmb / a.cols);
                a.spec4[k] = make_int4(qmv, minD, zero_d, (tie ? FLAG_TIE : 0) | av);
                a.spec_imv[k] = pack_mv(mx, my);
                __stcg(a.final_mv + k, qmv);
                if (tie) a.tie_list[atomicAdd(&a.ctrl->ntie, 1)] = k;
            }
        }
        if (!kSad) search_drain(S.efull, it, eissued, a.spin_limit);
    }
}

// Half-pel then quarter-pel refinement around each macroblock's full-pel
// winner (Full.cpp:452-517), one warp per macroblock, many per SM: the
// prediction-independent result the resolve starts from.
__global__ void __launch_bounds__(256) k_full_subpel(FullArgs a)
{
    const int lane = threadIdx.x & 31, k = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (k >= a.nmb) return;
    const int n = (k % a.cols) * 16, m = (k / a.cols) * 16;
    const int imv = __ldcg(a.spec_imv + k);
    const int mx = mv_x(imv), my = mv_y(imv);
    int minD = __ldcg(&a.spec4[k].y), qmx = 0, qmy = 0;
    subpel_refine_planes(a, n + mx, m + my, load_cur8(a, n, m, lane), lane, &minD, &qmx, &qmy);
    if (lane == 0) {
        const int qmv = pack_mv(4 * mx + qmx, 4 * my + qmy);
        a.spec4[k].x = qmv;
        a.spec4[k].y = minD;
        __stcg(a.final_mv + k, qmv);
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

int full_planes_launch(vppgpu_ctx* ctx, const FullArgs& args)
{
    const int PW = args.W + 2 * PAD, PH = args.H + 2 * PAD;
    dim3 grid((PW + PL_TX - 1) / PL_TX, (PH + PL_TY - 1) / PL_TY);
    k_full_planes<<<grid, 256, 0, ctx->stream>>>(args.job, args.W, args.H, args.rstride, (unsigned char*)args.src8,
                                                 (unsigned char*)args.refp, (unsigned char*)args.hpel, args.plane_size,
                                                 const_cast<int*>(args.energy), &args.ctrl->status);
    VPP_CHECK_LAUNCH(ctx);
    return VPPGPU_OK;
}

namespace {

// The search's grid: SEARCH_CTAS_PER_SM persistent CTAs per SM, at most one per macroblock.
int search_grid(const vppgpu_ctx* ctx, int nmb)
{
    const int g = ctx->sm_count * SEARCH_CTAS_PER_SM;
    return nmb < g ? nmb : g;
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode_tiled = nullptr;
std::once_flag g_encode_once;

// A 2-D tiled map over a row-major plane: width x height elements of
// `elem` bytes, `pitch` bytes per row, boxes of box_w x box_h elements, no
// swizzle (the box lands as box_h packed rows).
int encode_2d(CUtensorMap* map, const void* base, CUtensorMapDataType type, int elem, int width, int height,
              size_t pitch, int box_w, int box_h)
{
    std::call_once(g_encode_once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode_tiled = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    if (!g_encode_tiled) return VPPGPU_ERR_NO_DEVICE;
    if (((uintptr_t)base & 15) || (pitch & 15) || ((size_t)box_w * elem) % 16) return VPPGPU_ERR_INVALID_ARG;
    const cuuint64_t dims[2] = {(cuuint64_t)width, (cuuint64_t)height};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch};
    const cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode_tiled(map, type, 2, const_cast<void*>(base), dims, strides, box, estr,
                                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? VPPGPU_OK : VPPGPU_ERR_CUDA;
}

}  // namespace

int search_maps_encode(const FullArgs& a, SearchMaps* maps)
{
    memset(maps, 0, sizeof(*maps));
    const int PW = a.W + 2 * PAD, PH = a.H + 2 * PAD;
    int rc = encode_2d(&maps->win, a.refp, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, PW, PH, (size_t)a.rstride, WSTRIDE, WROWS);
    if (!rc) rc = encode_2d(&maps->cur, a.src8, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, a.W, a.H, (size_t)a.W, 16, 16);
    if (!rc && a.energy)
        rc = encode_2d(&maps->energy, a.energy, CU_TENSOR_MAP_DATA_TYPE_INT32, 4, PW, PH, (size_t)a.rstride * 4, TAB,
                       2 * RMAX + 1);
    return rc;
}

int full_launch(vppgpu_ctx* ctx, const FullArgs& args, const SearchMaps& maps, int nmb, int resolve_grid,
                cudaEvent_t* ev)
{
    if (ev) VPP_CUDA(cudaEventRecord(ev[0], ctx->stream));
    int rc = full_planes_launch(ctx, args);  // with the block energies (args.energy)
    if (rc) return rc;
    if (ev) VPP_CUDA(cudaEventRecord(ev[1], ctx->stream));
    k_full_search<false><<<search_grid(ctx, nmb), SEARCH_THREADS, sizeof(SearchSmem), ctx->stream>>>(args, maps);
    VPP_CHECK_LAUNCH(ctx);
    if (ev) VPP_CUDA(cudaEventRecord(ev[2], ctx->stream));
    k_full_subpel<<<(nmb + 7) / 8, 256, 0, ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    k_full_tietree<<<ctx->sm_count, TIE_RUNS * 32, sizeof(TieSmem), ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    if (ev) VPP_CUDA(cudaEventRecord(ev[3], ctx->stream));
    rc = full_resolve_launch(ctx, args, resolve_grid, 0);
    if (rc) return rc;
    if (ev) VPP_CUDA(cudaEventRecord(ev[4], ctx->stream));
    return VPPGPU_OK;
}

// The integer-pel SAD stage (FullArgs::intpel): planes, the SAD search (table,
// scan at prediction (0, 0), no sub-pel), tie trees, then the tie wavefront.
int sad_launch(vppgpu_ctx* ctx, const FullArgs& args, const SearchMaps& maps, int nmb)
{
    int rc = full_planes_launch(ctx, args);
    if (rc) return rc;
    k_full_search<true><<<search_grid(ctx, nmb), SEARCH_THREADS, sizeof(SearchSmem), ctx->stream>>>(args, maps);
    VPP_CHECK_LAUNCH(ctx);
    k_full_tietree<<<ctx->sm_count, TIE_RUNS * 32, sizeof(TieSmem), ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    return sad_resolve_launch(ctx, args);
}

int full_prepare(vppgpu_ctx* ctx, int nmb, int* resolve_grid)
{
    VPP_CUDA(cudaFuncSetAttribute(k_full_search<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(SearchSmem)));
    VPP_CUDA(cudaFuncSetAttribute(k_full_search<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(SearchSmem)));
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
