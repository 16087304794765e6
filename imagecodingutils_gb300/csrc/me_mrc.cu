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

}  // namespace vppgpu
