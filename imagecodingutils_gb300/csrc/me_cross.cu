// me_cross.cu -- MotionEstimatorH264ImplCross for sm_103a.
//
// Reference: MotionEstimatorH264ImplCross::Estimate
// (src/CodecUtils/MotionEstimatorH264ImplCross.cpp:354-649).  The prediction
// enters its search only at exact ties (the point not farther from the
// rounded prediction wins), so every macroblock is searched once at
// prediction (0, 0) (k_cross_search); the result holds for any prediction
// unless that search met a tie, and the remaining dependence -- the
// distortion at the prediction and GetBestVector over (best, prediction,
// zero) -- is the full-search estimator's raster-order predictor DAG,
// resolved by its kernels with this estimator's evaluation (estimator 3 of
// me_full_resolve.cu: path distortion, norm 64, lambda 0.9).  A tie
// macroblock's result for any prediction comes from its tie tree (eight
// searches with the first three ties forced, k_cross_tietree), else from a
// search at its rounded prediction kept in a small cache.
#include "me_cross_search.cuh"
#include "me_internal.h"

namespace vppgpu {
namespace {

__global__ void __launch_bounds__(256) k_cross_search(FullArgs f)
{
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int k = blockIdx.x * 8 + wib;
    if (k >= f.nmb) return;
    const cross::CrossResult r = cross::cross_search(f, (k % f.cols) * 16, (k / f.cols) * 16, 0, 0, lane);
    if (lane == 0) {
        if (r.tie) f.tie_list[atomicAdd(&f.ctrl->ntie, 1)] = k;
        const int flags = (r.tie ? full::FLAG_TIE : 0) | neighbour_mask(f.job->slice, k, f.cols, f.nmb / f.cols);
        const int v = pack_mv(r.mvx, r.mvy);
        f.spec4[k] = make_int4(v, r.min_d, r.zero_d, flags);
        f.final_mv[k] = v;
    }
    // searches of a tie MB at other rounded predictions: this one (rounded (0, 0)) and empty slots
    if (r.tie && lane < V2_SEARCH_CACHE)
        f.search_cache[(size_t)k * V2_SEARCH_CACHE + lane] =
            lane == 0 ? make_int4(pack_mv(0, 0), pack_mv(r.mvx, r.mvy), r.min_d, 1) : make_int4(0, 0, 0, -1);
}

// The tie tree of every macroblock whose search met a tie: warp r of a block
// makes run r (its first three ties decided by the bits of r).
__global__ void __launch_bounds__(mrc::V2_TIE_RUNS * 32) k_cross_tietree(FullArgs f)
{
    const int lane = threadIdx.x & 31, run = threadIdx.x >> 5;
    const int ntie = __ldcg(&f.ctrl->ntie);
    mrc::V2TieRun* runs = static_cast<mrc::V2TieRun*>(f.tie_runs);
    for (int i = blockIdx.x; i < ntie; i += gridDim.x) {
        const int k = __ldcg(f.tie_list + i);
        cross::cross_search_run(f, (k % f.cols) * 16, (k / f.cols) * 16, run, runs + (size_t)k * mrc::V2_TIE_RUNS + run,
                                lane);
    }
}

}  // namespace

int cross_launch(vppgpu_ctx* ctx, const FullArgs& args)
{
    int rc = full_planes_launch(ctx, args);
    if (rc) return rc;
    k_cross_search<<<(args.nmb + 7) / 8, 256, 0, ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    k_cross_tietree<<<ctx->sm_count * 2, mrc::V2_TIE_RUNS * 32, 0, ctx->stream>>>(args);
    VPP_CHECK_LAUNCH(ctx);
    return full_resolve_launch(ctx, args, 0, cross::EST_CROSS);
}

}  // namespace vppgpu
