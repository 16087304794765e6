// me_api.cu -- the motion-estimation handle of the vppgpu C ABI: the
// constructor + Create() of an IMotionEstimator implementation (device
// allocations sized once per frame geometry) and its Estimate() calls.
#include <vector>
#include <stdlib.h>
#include <string.h>

#include <new>

#include "me_common.cuh"
#include "me_internal.h"

struct vppgpu_me {
    vppgpu_ctx* ctx;
    int kind, W, H, cols, rows, nmb, motion_range, mode;
    int rstride;
    short* d_src16;
    short* d_ref16;
    unsigned char* d_src8;
    unsigned char* d_refp;
    unsigned char* d_hpel;  // b, h, j planes of the padded reference
    size_t plane_size;
    vppgpu::WaveRec* d_wave_rec;
    int* d_wave_choice;
    unsigned char* d_mrc;  // MultiresCross level planes (mrc_scratch_bytes)
    vppgpu::JobDesc* d_job;  // this estimate's pointers, read by the kernels
    // the Full estimator's kernel sequence, captured once per handle
    cudaGraphExec_t graph;
    unsigned long long graph_kernels;
    int graph_state;  // 0 not tried, 1 captured, -1 unavailable (direct launches)
    int* spec;  // 5 * nmb: {vector, distortion, zero distortion, flags} per MB, then full-pel winners
    int* tables;
    int* energy;  // block energies of the padded reference (full search by SSD)
    vppgpu::SearchMaps* maps;  // the search kernel's tensor maps over this handle's buffers
    int* tie_list;
    int4* cache;
    int* dict;
    int* state; // 3 * nmb: final_mv, final_dist, pred_used
    int* d_out_mv;
    int* d_out_dist;
    long long* d_out_avg;
    unsigned char* d_incl;
    int* d_slice;
    vppgpu::MeCtrl* ctrl;
    int* changed;
    int sweep_limit;
    int resolve_grid;
    int relax_sweeps;  // relaxation sweeps before the wavefront (0..RELAX_SWEEPS)
    int grid_sweeps;   // ... of which over every MB
    int relax_blocks_per_sm;  // grid of a sweep over every MB
    int mrc_warps;     // MultiresCross: macroblocks (warps) per search CTA
    void* d_mrc_args;  // MultiresCrossVer2: device mrc::MrcArgs
    void* d_lattice;   // MultiresCrossVer2: one sub-pel lattice per MB
    int4* d_search_cache;  // MultiresCrossVer2: searches of tie MBs at other predictions
    void* d_tie_runs;      // MultiresCrossVer2: tie trees
    unsigned long long* d_ustate;  // UMHS: sweep states, then the dataflow pass's states (2 * nmb)
    int4* d_urec;                  // UMHS: records (UMHS_RECORDS per MB)
    int* d_uprev;                  // UMHS: previous frame's full-pel starting points
    int* d_uorder;                 // UMHS: dataflow ticket -> macroblock
    int wave_grid;                 // UMHS: CTAs of the dataflow pass
    int bw, bh;                    // block size (16 x 16 but for MotionEstimatorImpl1)
    vppgpu::MeCtrl* h_ctrl;  // pinned
    int last_status;
    // per-kernel timing (vppgpu_me_set_timing)
    int timing;
    int ring_used;
    cudaEvent_t (*ring)[5];
    int timed_n;
    double timed_ms[4];  // pack + half-pel planes, table, refine + tie trees, resolve
};

namespace {
constexpr int kRing = 256;

// The estimators whose search starts at the prediction (UMHS, FHS): one
// pipeline (me_umhs.cu), its own relaxation policy.
bool searches_from_prediction(int kind) { return kind == VPPGPU_ME_UMHS || kind == VPPGPU_ME_FHS; }

void ring_fold(vppgpu_me* me)
{
    for (int i = 0; i < me->ring_used; i++) {
        cudaEventSynchronize(me->ring[i][4]);
        for (int k = 0; k < 4; k++) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, me->ring[i][k], me->ring[i][k + 1]) == cudaSuccess) me->timed_ms[k] += ms;
        }
        me->timed_n++;
    }
    me->ring_used = 0;
}

void ring_free(vppgpu_me* me)
{
    if (!me->ring) return;
    for (int i = 0; i < kRing; i++)
        for (int k = 0; k < 5; k++) cudaEventDestroy(me->ring[i][k]);
    free(me->ring);
    me->ring = nullptr;
}

cudaEvent_t* ring_slot(vppgpu_me* me)
{
    if (!me->timing || !me->ring) return nullptr;
    if (me->ring_used == kRing) ring_fold(me);
    return me->ring[me->ring_used++];
}
}  // namespace

namespace {

void me_free(vppgpu_me* me)
{
    if (!me) return;
    cudaSetDevice(me->ctx->device);
    cudaStreamSynchronize(me->ctx->stream);
    cudaFree(me->d_src16);
    cudaFree(me->d_ref16);
    cudaFree(me->d_src8);
    cudaFree(me->d_refp);
    cudaFree(me->d_hpel);
    cudaFree(me->d_wave_rec);
    cudaFree(me->d_wave_choice);
    cudaFree(me->d_mrc);
    cudaFree(me->d_mrc_args);
    cudaFree(me->d_lattice);
    cudaFree(me->d_search_cache);
    cudaFree(me->d_tie_runs);
    cudaFree(me->d_ustate);
    cudaFree(me->d_urec);
    cudaFree(me->d_uprev);
    cudaFree(me->d_uorder);
    cudaFree(me->d_job);
    if (me->graph) cudaGraphExecDestroy(me->graph);
    cudaFree(me->spec);
    cudaFree(me->tables);
    cudaFree(me->energy);
    delete me->maps;
    cudaFree(me->tie_list);
    cudaFree(me->cache);
    cudaFree(me->dict);
    cudaFree(me->state);
    cudaFree(me->d_out_mv);
    cudaFree(me->d_out_dist);
    cudaFree(me->d_out_avg);
    cudaFree(me->d_incl);
    cudaFree(me->d_slice);
    cudaFree(me->ctrl);
    cudaFree(me->changed);
    cudaFreeHost(me->h_ctrl);
    ring_free(me);
    free(me);
}

template <typename T>
int dalloc(T** p, size_t count)
{
    if (cudaMalloc((void**)p, sizeof(T) * (count ? count : 1)) != cudaSuccess) return VPPGPU_ERR_OUT_OF_MEMORY;
    return VPPGPU_OK;
}

vppgpu::FullArgs full_args(vppgpu_me* me, double lambda)
{
    vppgpu::FullArgs a{};
    a.W = me->W;
    a.H = me->H;
    a.cols = me->cols;
    a.nmb = me->nmb;
    a.motion_range = me->motion_range;
    a.rstride = me->rstride;
    a.src8 = me->d_src8;
    a.refp = me->d_refp;
    a.hpel = me->d_hpel;
    a.plane_size = me->plane_size;
    a.wave_rec = me->d_wave_rec;
    a.wave_choice = me->d_wave_choice;
    a.spec4 = reinterpret_cast<int4*>(me->spec);
    a.spec_imv = me->spec + 4 * (size_t)me->nmb;
    a.cache = me->cache;
    a.dict = me->dict;
    a.tables = me->tables;
    a.energy = me->energy;
    a.tie_list = me->tie_list;
    a.final_mv = me->state;
    a.final_dist = me->state + me->nmb;
    a.pred_used = me->state + 2 * me->nmb;
    a.job = me->d_job;
    a.ctrl = me->ctrl;
    a.changed = me->changed;
    a.dirty = reinterpret_cast<unsigned*>(me->changed + vppgpu::RELAX_SWEEPS + 2);
    a.lambda = lambda;
    a.sweep_limit = me->sweep_limit;
    a.relax_sweeps = me->relax_sweeps;
    a.grid_sweeps = me->grid_sweeps;
    a.relax_blocks_per_sm = me->relax_blocks_per_sm;
    a.mrc = me->d_mrc_args;
    a.lattice = me->d_lattice;
    a.search_cache = me->d_search_cache;
    a.tie_runs = me->d_tie_runs;
    a.mode = me->mode;
    a.spin_limit = 20000000LL;  // ~2 s of polling before a barrier gives up
    return a;
}

vppgpu::UmhsArgs umhs_args(vppgpu_me* me)
{
    vppgpu::UmhsArgs u{};
    u.f = full_args(me, 1.05);
    u.state = me->d_ustate;
    u.wave = me->d_ustate + me->nmb;
    u.rec = me->d_urec;
    u.prev = me->d_uprev;
    u.order = me->d_uorder;
    u.sweeps = me->relax_sweeps < 1 ? 1 : me->relax_sweeps;
    u.diag_limit = 1024;
    u.fhs = me->kind == VPPGPU_ME_FHS;
    return u;
}

// lambda: the full-search estimator's GetBestVector lambda (1.05), or with
// v2_lambda the lambda of Ver2's Lagrangian overload.
int run(vppgpu_me* me, const short* d_src16, const short* d_ref16, const unsigned char* d_incl, const int* d_slice,
        int* d_mv, int* d_dist, long long* d_avg, double lambda, bool v2_lambda = false)
{
    vppgpu_ctx* ctx = me->ctx;
    VPP_CUDA(cudaMemsetAsync(me->ctrl, 0, sizeof(vppgpu::MeCtrl), ctx->stream));
    if (me->kind == VPPGPU_ME_H263_MULTIRES_CROSS_V2) {
        const vppgpu::H263V2Job j{me->W,      me->H,      me->motion_range, me->mode,      me->relax_sweeps,
                                  d_src16,    d_ref16,    me->d_mrc,        d_incl,        d_mv,
                                  d_dist,     d_avg,      me->ctrl,         (int4*)me->spec, me->state,
                                  me->state + me->nmb,    me->d_urec,       me->changed,   me->d_wave_choice,
                                  me->tie_list, me->d_tie_runs, 2 * ctx->sm_count};
        return vppgpu::h263v2_launch(ctx, j);
    }
    if (me->kind == VPPGPU_ME_MULTIRES_CROSS || me->kind == VPPGPU_ME_H263_MULTIRES_CROSS)
        return vppgpu::mrc_launch(ctx, me->W, me->H, me->motion_range, me->mode, d_src16, d_ref16, me->d_mrc, d_incl,
                                  d_mv, d_dist, d_avg, me->ctrl, me->mrc_warps,
                                  me->kind == VPPGPU_ME_H263_MULTIRES_CROSS);
    int rc = vppgpu::set_job(ctx, me->d_job, vppgpu::JobDesc{d_src16, d_ref16, d_incl, d_slice, d_mv, d_dist, d_avg});
    if (rc) return rc;
    if (me->kind == VPPGPU_ME_CROSS) {
        // GetBestVector's lambda 0.9 (MotionEstimatorH264ImplCross.cpp:621)
        VPP_CUDA(cudaMemsetAsync(me->changed, 0, sizeof(int) * (size_t)me->sweep_limit, ctx->stream));
        return vppgpu::cross_launch(ctx, full_args(me, 0.9));
    }
    if (me->kind == VPPGPU_ME_MULTIRES_CROSS_V2 || me->kind == VPPGPU_ME_MULTIRES) {
        // GetBestVector's lambda: 0.9 (MultiresCrossVer2.cpp:1050), 1.1 (Multires.cpp:958)
        const bool v2 = me->kind == VPPGPU_ME_MULTIRES_CROSS_V2;
        VPP_CUDA(cudaMemsetAsync(me->changed, 0, sizeof(int) * (size_t)me->sweep_limit, ctx->stream));
        if (v2 && v2_lambda)  // Estimate(long*, void* lambda) (MultiresCrossVer2.cpp:1162-1742)
            return vppgpu::mrc2_launch(ctx, 4, me->mode, me->d_mrc, full_args(me, lambda), d_src16, d_ref16);
        return vppgpu::mrc2_launch(ctx, v2 ? 1 : 2, me->mode, me->d_mrc, full_args(me, v2 ? 0.9 : 1.1), d_src16,
                                   d_ref16);
    }
    if (searches_from_prediction(me->kind)) {
        VPP_CUDA(cudaMemsetAsync(me->changed, 0, sizeof(int) * (size_t)me->sweep_limit, ctx->stream));
        return vppgpu::umhs_launch(ctx, umhs_args(me), me->wave_grid);
    }
    if (me->kind == VPPGPU_ME_IMPL1) return vppgpu::impl1_launch(ctx, full_args(me, 0.0), me->bw, me->bh, me->motion_range);
    if (me->kind == VPPGPU_ME_IMPL2)
        return vppgpu::impl2_launch(ctx, full_args(me, 0.0), me->d_mrc, me->motion_range, me->mode);
    if (me->kind == VPPGPU_ME_FULL_SAD) {
        // the integer-pel stage only: no sub-pel, no prediction check, no GetBestVector
        vppgpu::FullArgs a = full_args(me, 0.0);
        a.intpel = 1;
        return vppgpu::sad_launch(ctx, a, *me->maps, me->nmb);
    }
    const vppgpu::FullArgs a = full_args(me, lambda);
    cudaEvent_t* ev = ring_slot(me);
    if (!ev && me->graph_state == 0) {
        // capture the per-estimate sequence once; every later estimate is one graph launch
        me->graph_state = -1;
        cudaGraph_t g = nullptr;
        const unsigned long long before = ctx->launches;
        if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            int crc = VPPGPU_OK;
            if (cudaMemsetAsync(me->changed, 0, sizeof(int) * (size_t)me->sweep_limit, ctx->stream) != cudaSuccess)
                crc = VPPGPU_ERR_CUDA;
            if (!crc) crc = vppgpu::full_launch(ctx, a, *me->maps, me->nmb, me->resolve_grid, nullptr);
            const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
            if (!crc && e == cudaSuccess && g && cudaGraphInstantiate(&me->graph, g, 0) == cudaSuccess) {
                me->graph_state = 1;
                me->graph_kernels = ctx->launches - before;
            }
            if (g) cudaGraphDestroy(g);
        }
        ctx->launches = before;
        cudaGetLastError();  // a failed capture leaves no sticky error: fall back to direct launches
    }
    if (!ev && me->graph_state == 1) {
        VPP_CUDA(cudaGraphLaunch(me->graph, ctx->stream));
        ctx->launches += me->graph_kernels;
        return VPPGPU_OK;
    }
    VPP_CUDA(cudaMemsetAsync(me->changed, 0, sizeof(int) * (size_t)me->sweep_limit, ctx->stream));
    return vppgpu::full_launch(ctx, a, *me->maps, me->nmb, me->resolve_grid, ev);
}

int status_from_ctrl(const vppgpu::MeCtrl& c) { return vppgpu::status_from_bits(c.status); }

// The dataflow passes' ticket order: anti-diagonals c + 2r, rows ascending, so that every neighbour a
// prediction reads has a lower ticket; and their grid, one CTA of 4 warps per SM (a wavefront holds at
// most min(rows, cols / 2) macroblocks at a time, and warps holding later tickets only wait).
int upload_diagonal_order(vppgpu_me* me)
{
    std::vector<int> order;
    order.reserve(me->nmb);
    for (int d = 0; d <= (me->cols - 1) + 2 * (me->rows - 1); d++)
        for (int r = 0; r < me->rows; r++) {
            const int c = d - 2 * r;
            if (c >= 0 && c < me->cols) order.push_back(r * me->cols + c);
        }
    if (cudaMemcpy(me->d_uorder, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return VPPGPU_ERR_CUDA;
    const int g = (me->nmb + 3) / 4;
    me->wave_grid = g < me->ctx->sm_count ? g : me->ctx->sm_count;
    return VPPGPU_OK;
}

bool aligned(const void* p, size_t a) { return ((uintptr_t)p & (a - 1)) == 0; }

}  // namespace

namespace vppgpu {

int status_from_bits(int bits)
{
    if (bits & ST_PIXEL_RANGE) return VPPGPU_ERR_PIXEL_RANGE;
    if (bits & ST_TIMEOUT) return VPPGPU_ERR_TIMEOUT;
    if (bits & ST_OUT_OF_BOUNDS) return VPPGPU_ERR_UNSUPPORTED;
    return VPPGPU_OK;
}

const int* me_status_word(vppgpu_me* me) { return &me->ctrl->status; }

}  // namespace vppgpu

extern "C" {

int vppgpu_me_create_blocks(vppgpu_ctx* ctx, int kind, int width, int height, int block_w, int block_h,
                            int motion_range, vppgpu_me** out)
{
    if (!ctx || !out) return VPPGPU_ERR_INVALID_ARG;
    *out = nullptr;
    if (kind == VPPGPU_ME_IMPL1 || kind == VPPGPU_ME_IMPL2) {
        // MotionEstimatorImpl1 / Impl2 (pSrc, pRef, w, h, macroBlkWidth, macroBlkHeight, motionRange): range in
        // full pels; blocks tiling the picture (the reference reads past its input otherwise): 16x16 or 8x8
        // for Impl1, 16x16 for Impl2 (its distortions are hard-wired to 16x16 / 8x8 / 4x4 levels)
        if (width < 16 || height < block_h || (width % 16) != 0 || motion_range < 1) return VPPGPU_ERR_INVALID_ARG;
        const bool blocks_ok = kind == VPPGPU_ME_IMPL1
                                   ? ((block_w == 16 && block_h == 16) || (block_w == 8 && block_h == 8))
                                   : (block_w == 16 && block_h == 16);
        if (!blocks_ok || (height % block_h) != 0) return VPPGPU_ERR_UNSUPPORTED;
        if (width > 8192 || height > 8192 || motion_range > 32) return VPPGPU_ERR_UNSUPPORTED;
        if (kind == VPPGPU_ME_IMPL2 && motion_range < 4) return VPPGPU_ERR_UNSUPPORTED;
        int rc = vppgpu::bind(ctx);
        if (rc) return rc;
        vppgpu_me* me = (vppgpu_me*)calloc(1, sizeof(vppgpu_me));
        if (!me) return VPPGPU_ERR_OUT_OF_MEMORY;
        me->ctx = ctx;
        me->kind = kind;
        me->W = width;
        me->H = height;
        me->bw = block_w;
        me->bh = block_h;
        me->cols = width / block_w;
        me->rows = height / block_h;
        me->nmb = me->cols * me->rows;
        me->motion_range = motion_range;
        me->mode = 1;  // Impl2's default, MotionEstimatorImpl2.cpp:120
        me->rstride = width + 2 * vppgpu::PAD;
        me->sweep_limit = 1;
        const size_t npix = (size_t)width * height;
        me->plane_size = (size_t)me->rstride * (height + 2 * vppgpu::PAD);
        if ((rc = dalloc(&me->d_src16, npix)) || (rc = dalloc(&me->d_ref16, npix)) ||
            (rc = dalloc(&me->d_src8, npix)) || (rc = dalloc(&me->d_refp, me->plane_size)) ||
            (rc = dalloc(&me->d_hpel, 3 * me->plane_size)) || (rc = dalloc(&me->d_job, 1)) ||
            (rc = dalloc(&me->changed, 1)) || (rc = dalloc(&me->d_out_mv, me->nmb)) ||
            (rc = dalloc(&me->d_out_dist, me->nmb)) || (rc = dalloc(&me->d_out_avg, 1)) ||
            (rc = dalloc(&me->d_incl, me->nmb)) || (rc = dalloc(&me->d_slice, me->nmb)) ||
            (rc = dalloc(&me->ctrl, 1)) ||
            (kind == VPPGPU_ME_IMPL2 && (rc = dalloc(&me->d_mrc, vppgpu::impl2_scratch_bytes(width, height))))) {
            me_free(me);
            return rc;
        }
        if (cudaMallocHost((void**)&me->h_ctrl, sizeof(vppgpu::MeCtrl)) != cudaSuccess) {
            me_free(me);
            return VPPGPU_ERR_OUT_OF_MEMORY;
        }
        *out = me;
        return VPPGPU_OK;
    }
    if (block_w != 16 || block_h != 16) return VPPGPU_ERR_UNSUPPORTED;
    return vppgpu_me_create(ctx, kind, width, height, motion_range, out);
}

int vppgpu_me_create(vppgpu_ctx* ctx, int kind, int width, int height, int motion_range, vppgpu_me** out)
{
    if (!ctx || !out) return VPPGPU_ERR_INVALID_ARG;
    *out = nullptr;
    if (kind == VPPGPU_ME_IMPL1 || kind == VPPGPU_ME_IMPL2)
        return vppgpu_me_create_blocks(ctx, kind, width, height, 16, 16, motion_range, out);
    // ranges below 4 (less than one full pel) are refused: the reference runs a
    // sub-pel-only search there, which nothing pins
    if (width < 16 || height < 16 || (width % 16) != 0 || motion_range < 4) return VPPGPU_ERR_INVALID_ARG;
    if (width > 8192 || height > 8192) return VPPGPU_ERR_UNSUPPORTED;
    if (motion_range > 128) return VPPGPU_ERR_UNSUPPORTED;
    if ((kind < VPPGPU_ME_FULL || kind > VPPGPU_ME_FHS) && kind != VPPGPU_ME_H263_MULTIRES_CROSS_V2)
        return VPPGPU_ERR_UNSUPPORTED;
    // the H.263 MultiresCross estimators' range is in half pels: at most 64 (+-31 pels), as 128 quarter pels
    if ((kind == VPPGPU_ME_H263_MULTIRES_CROSS || kind == VPPGPU_ME_H263_MULTIRES_CROSS_V2) && motion_range > 64)
        return VPPGPU_ERR_UNSUPPORTED;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    vppgpu_me* me = (vppgpu_me*)calloc(1, sizeof(vppgpu_me));
    if (!me) return VPPGPU_ERR_OUT_OF_MEMORY;
    me->ctx = ctx;
    me->kind = kind;
    me->W = width;
    me->H = height;
    me->cols = width / 16;
    me->rows = height / 16;
    me->nmb = me->cols * me->rows;
    me->bw = me->bh = 16;
    me->motion_range = motion_range;
    // Cross and UMHS default to quarter pel (…ImplCross.cpp:184, …ImplUMHS.cpp:259)
    me->mode = (kind == VPPGPU_ME_CROSS || searches_from_prediction(kind)) ? 0 : 1;
    me->rstride = width + 2 * vppgpu::PAD;
    me->sweep_limit = vppgpu::RELAX_SWEEPS + 2 + (me->nmb + 31) / 32;  // sweep counters, then the dirty bitmap
    if (searches_from_prediction(kind) && me->sweep_limit < 2 * vppgpu::UMHS_EVALS)  // change and search counts
        me->sweep_limit = 2 * vppgpu::UMHS_EVALS;
    // Sweep policy by how the estimator's predictions settle on moving content
    // (measured over 1080p pans): the full-search estimator mostly settles
    // within 8 sweeps over every MB, a few more over the dirty sets; Multires
    // keeps settling with more sweeps, cheaply over the dirty sets; Ver2
    // rarely settles, so its wavefront starts early.
    me->relax_sweeps = kind == VPPGPU_ME_MULTIRES_CROSS_V2 ? 4 : (searches_from_prediction(kind) ? 20 : vppgpu::RELAX_SWEEPS);
    me->grid_sweeps = kind == VPPGPU_ME_MULTIRES ? 4 : (kind == VPPGPU_ME_MULTIRES_CROSS_V2 ? 4 : 8);
    me->relax_blocks_per_sm = 4;
    me->mrc_warps = 8;
    size_t npix = (size_t)width * height;
    size_t npad = (size_t)me->rstride * (height + 2 * vppgpu::PAD);
    me->plane_size = npad;
    if (kind == VPPGPU_ME_MULTIRES_CROSS || kind == VPPGPU_ME_H263_MULTIRES_CROSS) {
        // MotionEstimatorH264ImplMultiresCross / H263ImplMultiresCross (…) + Create(): the level planes and outputs
        if ((rc = dalloc(&me->d_src16, npix)) || (rc = dalloc(&me->d_ref16, npix)) ||
            (rc = dalloc(&me->d_mrc, vppgpu::mrc_scratch_bytes(width, height))) ||
            (rc = dalloc(&me->d_out_mv, me->nmb)) || (rc = dalloc(&me->d_out_dist, me->nmb)) ||
            (rc = dalloc(&me->d_out_avg, 1)) || (rc = dalloc(&me->d_incl, me->nmb)) ||
            (rc = dalloc(&me->d_slice, me->nmb)) || (rc = dalloc(&me->ctrl, 1))) {
            me_free(me);
            return rc;
        }
        if (cudaMallocHost((void**)&me->h_ctrl, sizeof(vppgpu::MeCtrl)) != cudaSuccess) {
            me_free(me);
            return VPPGPU_ERR_OUT_OF_MEMORY;
        }
        *out = me;
        return VPPGPU_OK;
    }
    if (kind == VPPGPU_ME_CROSS) {
        // MotionEstimatorH264ImplCross(…, pMVPred, …) + Create(): the padded reference with its half-pel
        // planes, per-MB prediction state, tie trees and the cache of searches at other rounded predictions
        if ((rc = dalloc(&me->d_src16, npix)) || (rc = dalloc(&me->d_ref16, npix)) ||
            (rc = dalloc(&me->d_src8, npix)) || (rc = dalloc(&me->d_refp, npad)) ||
            (rc = dalloc(&me->d_hpel, 3 * npad)) ||
            (rc = dalloc(&me->d_search_cache, (size_t)me->nmb * vppgpu::V2_SEARCH_CACHE)) ||
            (rc = dalloc((unsigned char**)&me->d_tie_runs, vppgpu::mrc_tie_runs_bytes() * (size_t)me->nmb)) ||
            (rc = dalloc(&me->tie_list, me->nmb)) ||
            (rc = dalloc(&me->d_job, 1)) || (rc = dalloc(&me->spec, 5 * (size_t)me->nmb)) ||
            (rc = dalloc(&me->state, 3 * (size_t)me->nmb)) ||
            (rc = dalloc(&me->cache, (size_t)me->nmb * vppgpu::KCACHE)) || (rc = dalloc(&me->dict, vppgpu::NDICT)) ||
            (rc = dalloc(&me->d_wave_rec, vppgpu::wave_rec_count(me->cols, me->rows))) ||
            (rc = dalloc(&me->d_wave_choice, me->nmb)) || (rc = dalloc(&me->changed, (size_t)me->sweep_limit)) ||
            (rc = dalloc(&me->d_out_mv, me->nmb)) || (rc = dalloc(&me->d_out_dist, me->nmb)) ||
            (rc = dalloc(&me->d_out_avg, 1)) || (rc = dalloc(&me->d_incl, me->nmb)) ||
            (rc = dalloc(&me->d_slice, me->nmb)) || (rc = dalloc(&me->ctrl, 1))) {
            me_free(me);
            return rc;
        }
        if (cudaMallocHost((void**)&me->h_ctrl, sizeof(vppgpu::MeCtrl)) != cudaSuccess) {
            me_free(me);
            return VPPGPU_ERR_OUT_OF_MEMORY;
        }
        if ((rc = vppgpu::full_prepare(ctx, me->nmb, &me->resolve_grid))) {
            me_free(me);
            return rc;
        }
        *out = me;
        return VPPGPU_OK;
    }
    if (kind == VPPGPU_ME_H263_MULTIRES_CROSS_V2) {
        // MotionEstimatorH263ImplMultiresCrossVer2(…, pMVPred, pDistortionIncluded) + Create(): the level
        // planes, the searches at prediction (0, 0) and tie trees, relaxation and exact-pass vectors,
        // records, the sweeps' work lists
        const size_t nall = (size_t)me->cols * ((height + 15) / 16);  // a partial bottom row searched too
        me->relax_sweeps = vppgpu::UMHS_SWEEPS;  // 24: past it the sweeps cost more than the misses they save
        if (me->sweep_limit < 64 + vppgpu::H263V2_SWEEPS) me->sweep_limit = 64 + vppgpu::H263V2_SWEEPS;
        if ((rc = dalloc(&me->d_src16, npix)) || (rc = dalloc(&me->d_ref16, npix)) ||
            (rc = dalloc(&me->d_mrc, vppgpu::mrc_scratch_bytes(width, height))) ||
            (rc = dalloc(&me->spec, 4 * nall)) || (rc = dalloc(&me->state, 2 * (size_t)me->nmb)) ||
            (rc = dalloc(&me->d_urec, (size_t)me->nmb * vppgpu::H263V2_RECORDS)) ||
            (rc = dalloc(&me->changed, (size_t)me->sweep_limit)) || (rc = dalloc(&me->tie_list, nall)) || (rc = dalloc(&me->d_wave_choice, 3 * (size_t)me->nmb)) ||
            (rc = dalloc((unsigned char**)&me->d_tie_runs, vppgpu::mrc_tie_runs_bytes() * nall)) ||
            (rc = dalloc(&me->d_out_mv, me->nmb)) || (rc = dalloc(&me->d_out_dist, me->nmb)) ||
            (rc = dalloc(&me->d_out_avg, 1)) || (rc = dalloc(&me->d_incl, me->nmb)) ||
            (rc = dalloc(&me->d_slice, me->nmb)) || (rc = dalloc(&me->ctrl, 1))) {
            me_free(me);
            return rc;
        }
        if (cudaMallocHost((void**)&me->h_ctrl, sizeof(vppgpu::MeCtrl)) != cudaSuccess) {
            me_free(me);
            return VPPGPU_ERR_OUT_OF_MEMORY;
        }
        if ((rc = vppgpu::h263v2_prepare())) {
            me_free(me);
            return rc;
        }
        *out = me;
        return VPPGPU_OK;
    }
    if (searches_from_prediction(kind)) {
        // MotionEstimatorH264ImplUMHS(…, pMVPred, pDistortionIncluded, pPrevFrmMBlk) + Create(): the padded
        // reference with its half-pel planes, sweep and dataflow states, records, the previous frame's
        // starting points (zero until vppgpu_me_set_prev_frame) and the dataflow order
        if ((rc = dalloc(&me->d_src16, npix)) || (rc = dalloc(&me->d_ref16, npix)) ||
            (rc = dalloc(&me->d_src8, npix)) || (rc = dalloc(&me->d_refp, npad)) ||
            (rc = dalloc(&me->d_hpel, 3 * npad)) || (rc = dalloc(&me->d_job, 1)) ||
            (rc = dalloc(&me->d_ustate, 2 * (size_t)me->nmb)) ||
            (rc = dalloc(&me->d_urec, (size_t)me->nmb * vppgpu::UMHS_RECORDS)) ||
            (rc = dalloc(&me->d_uprev, me->nmb)) || (rc = dalloc(&me->d_uorder, me->nmb)) ||
            (rc = dalloc(&me->changed, (size_t)me->sweep_limit)) ||
            (rc = dalloc(&me->d_out_mv, me->nmb)) || (rc = dalloc(&me->d_out_dist, me->nmb)) ||
            (rc = dalloc(&me->d_out_avg, 1)) || (rc = dalloc(&me->d_incl, me->nmb)) ||
            (rc = dalloc(&me->d_slice, me->nmb)) || (rc = dalloc(&me->ctrl, 1))) {
            me_free(me);
            return rc;
        }
        if (cudaMallocHost((void**)&me->h_ctrl, sizeof(vppgpu::MeCtrl)) != cudaSuccess) {
            me_free(me);
            return VPPGPU_ERR_OUT_OF_MEMORY;
        }
        if ((rc = upload_diagonal_order(me)) ||
            (cudaMemset(me->d_uprev, 0, sizeof(int) * (size_t)me->nmb) != cudaSuccess && (rc = VPPGPU_ERR_CUDA)) ||
            (cudaMemset(me->d_ustate, 0, sizeof(unsigned long long) * (size_t)me->nmb) != cudaSuccess &&
             (rc = VPPGPU_ERR_CUDA))) {
            me_free(me);
            return rc;
        }
        if ((rc = vppgpu::umhs_prepare())) {
            me_free(me);
            return rc;
        }
        *out = me;
        return VPPGPU_OK;
    }
    if (kind == VPPGPU_ME_MULTIRES_CROSS_V2 || kind == VPPGPU_ME_MULTIRES) {
        // MotionEstimatorH264ImplMultiresCrossVer2 / Multires (…, pMVPred, …) + Create(): level planes, the
        // padded reference with its half-pel planes, per-MB prediction state
        if ((rc = dalloc(&me->d_src16, npix)) || (rc = dalloc(&me->d_ref16, npix)) ||
            (rc = dalloc(&me->d_src8, npix)) || (rc = dalloc(&me->d_refp, npad)) ||
            (rc = dalloc(&me->d_hpel, 3 * npad)) ||
            (rc = dalloc(&me->d_mrc, vppgpu::mrc_scratch_bytes(width, height))) ||
            (rc = dalloc((unsigned char**)&me->d_mrc_args, vppgpu::mrc_args_bytes())) ||
            (rc = dalloc((unsigned char**)&me->d_lattice, vppgpu::mrc_lattice_bytes() * (size_t)me->nmb)) ||
            (rc = dalloc(&me->d_search_cache, (size_t)me->nmb * vppgpu::V2_SEARCH_CACHE)) ||
            (rc = dalloc((unsigned char**)&me->d_tie_runs, vppgpu::mrc_tie_runs_bytes() * (size_t)me->nmb)) ||
            (rc = dalloc(&me->tie_list, me->nmb)) ||
            (rc = dalloc(&me->d_job, 1)) || (rc = dalloc(&me->spec, 5 * (size_t)me->nmb)) ||
            (rc = dalloc(&me->state, 3 * (size_t)me->nmb)) ||
            (rc = dalloc(&me->cache, (size_t)me->nmb * vppgpu::KCACHE)) || (rc = dalloc(&me->dict, vppgpu::NDICT)) ||
            (rc = dalloc(&me->d_wave_rec, vppgpu::wave_rec_count(me->cols, me->rows))) ||
            (rc = dalloc(&me->d_wave_choice, me->nmb)) || (rc = dalloc(&me->changed, (size_t)me->sweep_limit)) ||
            (rc = dalloc(&me->d_out_mv, me->nmb)) || (rc = dalloc(&me->d_out_dist, me->nmb)) ||
            (rc = dalloc(&me->d_out_avg, 1)) || (rc = dalloc(&me->d_incl, me->nmb)) ||
            (rc = dalloc(&me->d_slice, me->nmb)) || (rc = dalloc(&me->ctrl, 1))) {
            me_free(me);
            return rc;
        }
        if (cudaMallocHost((void**)&me->h_ctrl, sizeof(vppgpu::MeCtrl)) != cudaSuccess) {
            me_free(me);
            return VPPGPU_ERR_OUT_OF_MEMORY;
        }
        if ((rc = vppgpu::full_prepare(ctx, me->nmb, &me->resolve_grid))) {
            me_free(me);
            return rc;
        }
        *out = me;
        return VPPGPU_OK;
    }
    if ((rc = dalloc(&me->d_src16, npix)) || (rc = dalloc(&me->d_ref16, npix)) || (rc = dalloc(&me->d_src8, npix)) ||
        (rc = dalloc(&me->d_refp, npad)) || (rc = dalloc(&me->d_hpel, 3 * npad)) ||
        (rc = dalloc(&me->d_wave_rec, vppgpu::wave_rec_count(me->cols, me->rows))) || (rc = dalloc(&me->d_wave_choice, me->nmb)) || (rc = dalloc(&me->spec, 5 * (size_t)me->nmb)) ||
        (rc = dalloc(&me->tables, (size_t)me->nmb * 64 * 64)) ||
        (kind == VPPGPU_ME_FULL && (rc = dalloc(&me->energy, npad))) || (rc = dalloc(&me->d_job, 1)) || (rc = dalloc(&me->tie_list, me->nmb)) || (rc = dalloc(&me->state, 3 * (size_t)me->nmb)) ||
        (rc = dalloc(&me->cache, (size_t)me->nmb * vppgpu::KCACHE)) || (rc = dalloc(&me->dict, vppgpu::NDICT)) ||
        (rc = dalloc(&me->d_out_mv, me->nmb)) || (rc = dalloc(&me->d_out_dist, me->nmb)) ||
        (rc = dalloc(&me->d_out_avg, 1)) || (rc = dalloc(&me->d_incl, me->nmb)) ||
        (rc = dalloc(&me->d_slice, me->nmb)) || (rc = dalloc(&me->ctrl, 1)) ||
        (rc = dalloc(&me->changed, (size_t)me->sweep_limit))) {
        me_free(me);
        return rc;
    }
    if (cudaMallocHost((void**)&me->h_ctrl, sizeof(vppgpu::MeCtrl)) != cudaSuccess) {
        me_free(me);
        return VPPGPU_ERR_OUT_OF_MEMORY;
    }
    if ((rc = vppgpu::full_prepare(ctx, me->nmb, &me->resolve_grid))) {
        me_free(me);
        return rc;
    }
    if (kind == VPPGPU_ME_FULL || kind == VPPGPU_ME_FULL_SAD) {
        me->maps = new (std::nothrow) vppgpu::SearchMaps();
        if (!me->maps) {
            me_free(me);
            return VPPGPU_ERR_OUT_OF_MEMORY;
        }
        if ((rc = vppgpu::search_maps_encode(full_args(me, 0.0), me->maps))) {
            me_free(me);
            return rc;
        }
    }
    *out = me;
    return VPPGPU_OK;
}

int vppgpu_me_destroy(vppgpu_me* me)
{
    if (!me) return VPPGPU_ERR_INVALID_ARG;
    me_free(me);
    return VPPGPU_OK;
}

int vppgpu_me_set_mode(vppgpu_me* me, int mode)
{
    if (!me) return VPPGPU_ERR_INVALID_ARG;
    // SetMode(0) picks by picture area for the multi-resolution estimators (MultiresCross.cpp:501-513);
    // Cross and UMHS keep the mode as given (MotionEstimatorH264ImplCross.h:99, …ImplUMHS.h:107)
    if (mode == 0 && me->kind != VPPGPU_ME_FULL && me->kind != VPPGPU_ME_CROSS && !searches_from_prediction(me->kind) &&
        me->kind != VPPGPU_ME_IMPL1)
        mode = (me->W * me->H > 40000) ? 2 : 1;
    me->mode = mode;
    return VPPGPU_OK;
}

int vppgpu_me_get_mode(vppgpu_me* me, int* mode)
{
    if (!me || !mode) return VPPGPU_ERR_INVALID_ARG;
    *mode = me->mode;
    return VPPGPU_OK;
}

int vppgpu_me_num_mbs(vppgpu_me* me, int* n)
{
    if (!me || !n) return VPPGPU_ERR_INVALID_ARG;
    *n = me->nmb;
    return VPPGPU_OK;
}

int vppgpu_me_estimate_device(vppgpu_me* me, const short* d_src, const short* d_ref, const unsigned char* d_incl,
                              const int* d_slice, short* d_mv_out, int* d_mb_dist_out, long long* d_avg_out)
{
    if (!me || !d_src || !d_ref || !d_mv_out) return VPPGPU_ERR_INVALID_ARG;
    if (!aligned(d_src, 4) || !aligned(d_ref, 4) || !aligned(d_mv_out, 4)) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    me->last_status = VPPGPU_OK;
    return run(me, d_src, d_ref, d_incl, d_slice, (int*)d_mv_out, d_mb_dist_out, d_avg_out, 1.05);
}

static int estimate_host(vppgpu_me* me, const short* src, const short* ref, const unsigned char* incl,
                         const int* slice, short* mv_out, int* mb_dist_out, long* avg, double lambda,
                         bool v2_lambda = false)
{
    if (!me || !src || !ref || !mv_out) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    cudaStream_t st = me->ctx->stream;
    size_t plane = sizeof(short) * (size_t)me->W * me->H;
    VPP_CUDA(cudaMemcpyAsync(me->d_src16, src, plane, cudaMemcpyHostToDevice, st));
    VPP_CUDA(cudaMemcpyAsync(me->d_ref16, ref, plane, cudaMemcpyHostToDevice, st));
    if (incl) VPP_CUDA(cudaMemcpyAsync(me->d_incl, incl, (size_t)me->nmb, cudaMemcpyHostToDevice, st));
    if (slice) VPP_CUDA(cudaMemcpyAsync(me->d_slice, slice, sizeof(int) * me->nmb, cudaMemcpyHostToDevice, st));
    rc = run(me, me->d_src16, me->d_ref16, incl ? me->d_incl : nullptr, slice ? me->d_slice : nullptr,
             me->d_out_mv, mb_dist_out ? me->d_out_dist : nullptr, nullptr, lambda, v2_lambda);
    if (rc) return rc;
    VPP_CUDA(cudaMemcpyAsync(mv_out, me->d_out_mv, sizeof(int) * me->nmb, cudaMemcpyDeviceToHost, st));
    if (mb_dist_out)
        VPP_CUDA(cudaMemcpyAsync(mb_dist_out, me->d_out_dist, sizeof(int) * me->nmb, cudaMemcpyDeviceToHost, st));
    VPP_CUDA(cudaMemcpyAsync(me->h_ctrl, me->ctrl, sizeof(vppgpu::MeCtrl), cudaMemcpyDeviceToHost, st));
    VPP_CUDA(cudaStreamSynchronize(st));
    me->last_status = status_from_ctrl(*me->h_ctrl);
    if (me->last_status) return me->last_status;
    if (avg) *avg = me->h_ctrl->count ? (long)(me->h_ctrl->total / me->h_ctrl->count) : 0;
    return VPPGPU_OK;
}

int vppgpu_me_estimate(vppgpu_me* me, const short* src, const short* ref, const unsigned char* incl,
                       const int* slice, short* mv_out, int* mb_dist_out, long* avg)
{
    return estimate_host(me, src, ref, incl, slice, mv_out, mb_dist_out, avg, 1.05);
}

int vppgpu_me_set_prev_frame(vppgpu_me* me, const short* prev_mv, const unsigned char* prev_intra)
{
    if (!me) return VPPGPU_ERR_INVALID_ARG;
    if (me->kind != VPPGPU_ME_UMHS) return VPPGPU_ERR_UNSUPPORTED;
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    // the starting point of MotionEstimatorH264ImplUMHS.cpp:551-571: the
    // vector in full pels (C division), none for intra macroblocks; a block
    // origin outside [-16, W] x [-16, H] would make the reference read
    // outside its buffers should it win
    std::vector<int> start((size_t)me->nmb, 0);
    for (int k = 0; prev_mv && k < me->nmb; k++) {
        if (prev_intra && prev_intra[k]) continue;
        const int x = prev_mv[2 * k] / 4, y = prev_mv[2 * k + 1] / 4;
        const int ox = (k % me->cols) * 16 + x, oy = (k / me->cols) * 16 + y;
        if (ox < -16 || ox > me->W || oy < -16 || oy > me->H) return VPPGPU_ERR_INVALID_ARG;
        start[k] = (int)((unsigned)(x & 0xffff) | ((unsigned)y << 16));
    }
    VPP_CUDA(cudaMemcpyAsync(me->d_uprev, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice,
                             me->ctx->stream));
    VPP_CUDA(cudaStreamSynchronize(me->ctx->stream));
    return VPPGPU_OK;
}

int vppgpu_me_estimate_lambda(vppgpu_me* me, const short* src, const short* ref, const unsigned char* incl,
                              const int* slice, double lambda, short* mv_out, int* mb_dist_out, long* avg)
{
    // Ver2's overload: GetBestVector at every search level and at the end
    // with this lambda (MultiresCrossVer2.cpp:1162-1742).  The other
    // estimators have none: IMotionEstimator's default Estimate(long*, void*)
    // ignores the parameter (IMotionEstimator.h:94).
    if (me && me->kind == VPPGPU_ME_MULTIRES_CROSS_V2)
        return estimate_host(me, src, ref, incl, slice, mv_out, mb_dist_out, avg, lambda, true);
    return estimate_host(me, src, ref, incl, slice, mv_out, mb_dist_out, avg, 1.05);
}

int vppgpu_me_last_status(vppgpu_me* me)
{
    if (!me) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    VPP_CUDA(cudaMemcpyAsync(me->h_ctrl, me->ctrl, sizeof(vppgpu::MeCtrl), cudaMemcpyDeviceToHost, me->ctx->stream));
    VPP_CUDA(cudaStreamSynchronize(me->ctx->stream));
    return status_from_ctrl(*me->h_ctrl);
}

int vppgpu_me_set_timing(vppgpu_me* me, int enable)
{
    if (!me) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    if (enable && !me->ring) {
        me->ring = (cudaEvent_t(*)[5])calloc(kRing, sizeof(*me->ring));
        if (!me->ring) return VPPGPU_ERR_OUT_OF_MEMORY;
        for (int i = 0; i < kRing; i++)
            for (int k = 0; k < 5; k++) VPP_CUDA(cudaEventCreate(&me->ring[i][k]));
    }
    me->timing = enable != 0;
    me->ring_used = 0;
    me->timed_n = 0;
    for (int k = 0; k < 4; k++) me->timed_ms[k] = 0.0;
    return VPPGPU_OK;
}

int vppgpu_me_timing(vppgpu_me* me, int* n, double* pack_ms, double* search_ms, double* resolve_ms)
{
    if (!me || !n || !pack_ms || !search_ms || !resolve_ms) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    if (me->ring) ring_fold(me);
    *n = me->timed_n;
    *pack_ms = me->timed_ms[0];
    *search_ms = me->timed_ms[1] + me->timed_ms[2];
    *resolve_ms = me->timed_ms[3];
    return VPPGPU_OK;
}

int vppgpu_me_timing_stages(vppgpu_me* me, int* n, double* stage_ms4)
{
    if (!me || !n || !stage_ms4) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    if (me->ring) ring_fold(me);
    *n = me->timed_n;
    for (int k = 0; k < 4; k++) stage_ms4[k] = me->timed_ms[k];
    return VPPGPU_OK;
}

int vppgpu_me_last_sweeps(vppgpu_me* me, int* sweeps)
{
    if (!me || !sweeps) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    VPP_CUDA(cudaMemcpyAsync(me->h_ctrl, me->ctrl, sizeof(vppgpu::MeCtrl), cudaMemcpyDeviceToHost, me->ctx->stream));
    VPP_CUDA(cudaStreamSynchronize(me->ctx->stream));
    *sweeps = me->h_ctrl->sweeps;
    return VPPGPU_OK;
}

}  // extern "C"

extern "C" int vppgpu_me_set_relax_sweeps(vppgpu_me* me, int sweeps)
{
    if (!me || sweeps < 0 ||
        sweeps > (me->kind == VPPGPU_ME_H263_MULTIRES_CROSS_V2
                      ? vppgpu::H263V2_SWEEPS
                      : (searches_from_prediction(me->kind) ? vppgpu::UMHS_SWEEPS : vppgpu::RELAX_SWEEPS)))
        return VPPGPU_ERR_INVALID_ARG;
    if (me->kind == VPPGPU_ME_MULTIRES_CROSS || me->kind == VPPGPU_ME_H263_MULTIRES_CROSS ||
        me->kind == VPPGPU_ME_FULL_SAD || me->kind == VPPGPU_ME_IMPL1 || me->kind == VPPGPU_ME_IMPL2)
        return VPPGPU_ERR_UNSUPPORTED;
    if (sweeps == me->relax_sweeps) return VPPGPU_OK;
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    me->relax_sweeps = sweeps;
    if (me->graph) {  // the captured sequence has the old number of sweep launches
        VPP_CUDA(cudaStreamSynchronize(me->ctx->stream));
        cudaGraphExecDestroy(me->graph);
        me->graph = nullptr;
    }
    me->graph_state = 0;
    return VPPGPU_OK;
}

// ---------------------------------------------------------------------------
// Autotuning: the launch shapes and the relaxation policy that suit the
// caller's content on this GPU, chosen by timing each candidate on one frame
// pair.  Every candidate gives the same vectors (checked); only the time
// differs.
namespace {

struct TuneCfg {
    int relax, grid, bps, warps;
};

void apply_cfg(vppgpu_me* me, const TuneCfg& c)
{
    me->relax_sweeps = c.relax;
    me->grid_sweeps = c.grid;
    me->relax_blocks_per_sm = c.bps;
    me->mrc_warps = c.warps;
}

}  // namespace

extern "C" int vppgpu_me_autotune_pairs(vppgpu_me* me, const short* const* d_src, const short* const* d_ref,
                                        int npairs, int reps, int* chosen);

extern "C" int vppgpu_me_autotune(vppgpu_me* me, const short* d_src, const short* d_ref, int reps, int* chosen)
{
    return vppgpu_me_autotune_pairs(me, &d_src, &d_ref, 1, reps, chosen);
}

extern "C" int vppgpu_me_autotune_pairs(vppgpu_me* me, const short* const* d_src, const short* const* d_ref,
                                        int npairs, int reps, int* chosen)
{
    if (!me || !d_src || !d_ref || npairs < 1 || reps < 1) return VPPGPU_ERR_INVALID_ARG;
    for (int p = 0; p < npairs; p++)
        if (!d_src[p] || !d_ref[p]) return VPPGPU_ERR_INVALID_ARG;
    if (me->kind == VPPGPU_ME_FULL_SAD || me->kind == VPPGPU_ME_IMPL1 ||
        me->kind == VPPGPU_ME_IMPL2) {  // one configuration: nothing to tune
        if (chosen) *chosen = 0;
        return VPPGPU_OK;
    }
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    cudaStream_t st = me->ctx->stream;
    std::vector<TuneCfg> cands;
    const TuneCfg cur{me->relax_sweeps, me->grid_sweeps, me->relax_blocks_per_sm, me->mrc_warps};
    cands.push_back(cur);
    if (me->kind == VPPGPU_ME_MULTIRES_CROSS || me->kind == VPPGPU_ME_H263_MULTIRES_CROSS) {
        for (int w : {2, 4, 8})
            if (w != cur.warps) cands.push_back({cur.relax, cur.grid, cur.bps, w});
    } else if (me->kind == VPPGPU_ME_H263_MULTIRES_CROSS_V2) {  // the sweeps before the exact pass
        for (int r : {4, 8, 14, 20, 24})
            if (r != cur.relax) cands.push_back({r, cur.grid, cur.bps, cur.warps});
    } else if (searches_from_prediction(me->kind)) {  // only the sweeps before the dataflow pass matter
        for (int r : {4, 8, 12, 16, 20, 24})
            if (r != cur.relax) cands.push_back({r, cur.grid, cur.bps, cur.warps});
    } else {
        const int policies[][2] = {{4, 4}, {8, 8}, {14, 8}, {14, 4}, {14, 2}};
        for (const auto& p : policies)
            for (int bps : {2, 4, 8})
                if (p[0] != cur.relax || p[1] != cur.grid || bps != cur.bps)
                    cands.push_back({p[0], p[1], bps, cur.warps});
    }
    // time direct launches for every candidate (the captured graph is rebuilt afterwards)
    if (me->graph) {
        VPP_CUDA(cudaStreamSynchronize(st));
        cudaGraphExecDestroy(me->graph);
        me->graph = nullptr;
    }
    me->graph_state = -1;
    std::vector<int> ref_mv((size_t)me->nmb * npairs), mv((size_t)me->nmb * npairs);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        me->graph_state = 0;
        return VPPGPU_ERR_CUDA;
    }
    float best_ms = 0.f;
    int best = 0;
    for (size_t i = 0; i < cands.size() && !rc; i++) {
        apply_cfg(me, cands[i]);
        if ((rc = run(me, d_src[0], d_ref[0], nullptr, nullptr, me->d_out_mv, nullptr, nullptr, 1.05))) break;  // warm-up
        if (cudaEventRecord(e0, st) != cudaSuccess) rc = VPPGPU_ERR_CUDA;
        for (int r = 0; r < reps && !rc; r++)
            for (int p = 0; p < npairs && !rc; p++) {
                rc = run(me, d_src[p], d_ref[p], nullptr, nullptr, me->d_out_mv, nullptr, nullptr, 1.05);
                if (!rc && r == reps - 1 &&  // the vectors of the last repetition, pair by pair
                    cudaMemcpyAsync((i ? mv.data() : ref_mv.data()) + (size_t)p * me->nmb, me->d_out_mv,
                                    sizeof(int) * (size_t)me->nmb, cudaMemcpyDeviceToHost, st) != cudaSuccess)
                    rc = VPPGPU_ERR_CUDA;
            }
        if (rc || cudaEventRecord(e1, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
            if (!rc) rc = VPPGPU_ERR_CUDA;
            break;
        }
        VPP_CUDA(cudaMemcpyAsync(me->h_ctrl, me->ctrl, sizeof(vppgpu::MeCtrl), cudaMemcpyDeviceToHost, st));
        VPP_CUDA(cudaStreamSynchronize(st));
        if ((rc = status_from_ctrl(*me->h_ctrl))) break;
        if (i && mv != ref_mv) {  // a launch shape changed a result: never expected
            rc = VPPGPU_ERR_CUDA;
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (i == 0 || ms < best_ms) {
            best_ms = ms;
            best = (int)i;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    apply_cfg(me, rc ? cur : cands[best]);
    me->graph_state = 0;
    if (chosen) *chosen = rc ? 0 : best;
    return rc;
}

extern "C" int vppgpu_me_autotune_host(vppgpu_me* me, const short* src, const short* ref, int reps, int* chosen)
{
    if (!me || !src || !ref) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    const size_t plane = sizeof(short) * (size_t)me->W * me->H;
    VPP_CUDA(cudaMemcpyAsync(me->d_src16, src, plane, cudaMemcpyHostToDevice, me->ctx->stream));
    VPP_CUDA(cudaMemcpyAsync(me->d_ref16, ref, plane, cudaMemcpyHostToDevice, me->ctx->stream));
    return vppgpu_me_autotune(me, me->d_src16, me->d_ref16, reps, chosen);
}

extern "C" int vppgpu_me_get_tuning(vppgpu_me* me, int* tuning4)
{
    if (!me || !tuning4) return VPPGPU_ERR_INVALID_ARG;
    tuning4[0] = me->relax_sweeps;
    tuning4[1] = me->grid_sweeps;
    tuning4[2] = me->relax_blocks_per_sm;
    tuning4[3] = me->mrc_warps;
    return VPPGPU_OK;
}

extern "C" int vppgpu_me_residual_device(vppgpu_me* me, const short* d_mv, short* d_residual)
{
    if (!me || !d_mv || !d_residual) return VPPGPU_ERR_INVALID_ARG;
    if (me->kind != VPPGPU_ME_FULL) return VPPGPU_ERR_UNSUPPORTED;
    if (!aligned(d_mv, 4) || !aligned(d_residual, 16)) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    return vppgpu::full_residual_launch(me->ctx, full_args(me, 1.05), (const int*)d_mv, d_residual);
}

extern "C" int vppgpu_me_last_stats(vppgpu_me* me, int* stats8)
{
    if (!me || !stats8) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    VPP_CUDA(cudaMemcpyAsync(me->h_ctrl, me->ctrl, sizeof(vppgpu::MeCtrl), cudaMemcpyDeviceToHost, me->ctx->stream));
    VPP_CUDA(cudaStreamSynchronize(me->ctx->stream));
    const vppgpu::MeCtrl& c = *me->h_ctrl;
    int v[8] = {c.sweeps, c.converged, c.relax_evals, c.relax_miss, c.wave_miss, c.status, c.count, c.ntie};
    for (int i = 0; i < 8; i++) stats8[i] = v[i];
    return VPPGPU_OK;
}

extern "C" int vppgpu_me_last_relax_changes(vppgpu_me* me, int* changes, int n)
{
    if (!me || !changes || n < 0 || n > vppgpu::RELAX_SWEEPS) return VPPGPU_ERR_INVALID_ARG;
    if (!me->changed) return VPPGPU_ERR_UNSUPPORTED;  // estimators without a relaxation
    int rc = vppgpu::bind(me->ctx);
    if (rc) return rc;
    VPP_CUDA(cudaStreamSynchronize(me->ctx->stream));
    if (n) VPP_CUDA(cudaMemcpy(changes, me->changed + 1, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost));
    return VPPGPU_OK;
}

// ---------------------------------------------------------------------------
// Batched estimation: many independent frame pairs, any mix of sizes, spread
// over several streams so that one frame's latency-bound stages run beside
// another frame's search.  Jobs go to streams longest first (by macroblock
// count), each to the stream with the least work so far; each stream keeps
// one estimator per frame geometry, created on first use and reused by later
// batches.  The batch is ordered after the work already on the context's
// stream and before work enqueued there later.
// ---------------------------------------------------------------------------
namespace {
constexpr int kBatchMaxStreams = 16;

struct BatchSlot {
    vppgpu_ctx* ctx = nullptr;  // own stream
    struct Entry {
        int W, H, range;
        vppgpu_me* me;
    };
    Entry pool[8];
    int npool = 0;
    long long load = 0;
};
}  // namespace

struct vppgpu_me_batch {
    vppgpu_ctx* parent;
    int kind;
    int nslots;
    BatchSlot slot[kBatchMaxStreams];
    vppgpu::MeCtrl* h_ctrl;  // pinned, one per job of the current batch
    int cap;
    int* order;
    int* where;
    cudaEvent_t start, done[kBatchMaxStreams];
};

namespace {

void batch_free(vppgpu_me_batch* b)
{
    if (!b) return;
    cudaSetDevice(b->parent->device);
    for (int s = 0; s < b->nslots; s++) {
        BatchSlot& sl = b->slot[s];
        for (int i = 0; i < sl.npool; i++) vppgpu_me_destroy(sl.pool[i].me);
        if (sl.ctx) vppgpu_ctx_destroy(sl.ctx);
        if (b->done[s]) cudaEventDestroy(b->done[s]);
    }
    if (b->start) cudaEventDestroy(b->start);
    if (b->h_ctrl) cudaFreeHost(b->h_ctrl);
    free(b->order);
    free(b->where);
    free(b);
}

int slot_estimator(vppgpu_me_batch* b, BatchSlot& sl, int W, int H, int range, vppgpu_me** out)
{
    for (int i = 0; i < sl.npool; i++)
        if (sl.pool[i].W == W && sl.pool[i].H == H && sl.pool[i].range == range) {
            *out = sl.pool[i].me;
            return VPPGPU_OK;
        }
    if (sl.npool == 8) {  // evict the oldest geometry
        vppgpu_me_destroy(sl.pool[0].me);
        for (int i = 1; i < 8; i++) sl.pool[i - 1] = sl.pool[i];
        sl.npool--;
    }
    vppgpu_me* me = nullptr;
    int rc = vppgpu_me_create(sl.ctx, b->kind, W, H, range, &me);
    if (rc) return rc;
    sl.pool[sl.npool++] = {W, H, range, me};
    *out = me;
    return VPPGPU_OK;
}

}  // namespace

extern "C" {

int vppgpu_me_batch_create(vppgpu_ctx* ctx, int kind, int streams, vppgpu_me_batch** out)
{
    if (!ctx || !out || streams < 1) return VPPGPU_ERR_INVALID_ARG;
    *out = nullptr;
    if (kind < VPPGPU_ME_FULL || kind > VPPGPU_ME_FULL_SAD) return VPPGPU_ERR_UNSUPPORTED;
    int rc = vppgpu::bind(ctx);
    if (rc) return rc;
    vppgpu_me_batch* b = (vppgpu_me_batch*)calloc(1, sizeof(vppgpu_me_batch));
    if (!b) return VPPGPU_ERR_OUT_OF_MEMORY;
    b->parent = ctx;
    b->kind = kind;
    b->nslots = streams < kBatchMaxStreams ? streams : kBatchMaxStreams;
    for (int s = 0; s < b->nslots; s++) {
        new (&b->slot[s]) BatchSlot();
        if ((rc = vppgpu_ctx_create(ctx->device, &b->slot[s].ctx)) ||
            cudaEventCreateWithFlags(&b->done[s], cudaEventDisableTiming) != cudaSuccess) {
            batch_free(b);
            return rc ? rc : VPPGPU_ERR_CUDA;
        }
    }
    if (cudaEventCreateWithFlags(&b->start, cudaEventDisableTiming) != cudaSuccess) {
        batch_free(b);
        return VPPGPU_ERR_CUDA;
    }
    *out = b;
    return VPPGPU_OK;
}

int vppgpu_me_batch_destroy(vppgpu_me_batch* b)
{
    if (!b) return VPPGPU_ERR_INVALID_ARG;
    batch_free(b);
    return VPPGPU_OK;
}

int vppgpu_me_batch_run(vppgpu_me_batch* b, const vppgpu_me_job* jobs, int n, int* status_out, long* avg_out)
{
    if (!b || (n > 0 && !jobs) || n < 0) return VPPGPU_ERR_INVALID_ARG;
    int rc = vppgpu::bind(b->parent);
    if (rc) return rc;
    for (int j = 0; j < n; j++) {
        const vppgpu_me_job& J = jobs[j];
        if (!J.src || !J.ref || !J.mv_out || J.width < 16 || J.height < 16 || J.width % 16) return VPPGPU_ERR_INVALID_ARG;
        if (J.levels_out && (!J.residual_out || !J.recon_out || J.qp < 0 || J.qp > 51 || b->kind != VPPGPU_ME_FULL))
            return VPPGPU_ERR_INVALID_ARG;
    }
    if (n > b->cap) {
        if (b->h_ctrl) cudaFreeHost(b->h_ctrl);
        free(b->order);
        free(b->where);
        b->h_ctrl = nullptr;
        b->order = (int*)malloc(sizeof(int) * (size_t)n);
        b->where = (int*)malloc(sizeof(int) * (size_t)n);
        b->cap = 0;
        if (!b->order || !b->where || cudaMallocHost((void**)&b->h_ctrl, sizeof(vppgpu::MeCtrl) * (size_t)n) != cudaSuccess)
            return VPPGPU_ERR_OUT_OF_MEMORY;
        b->cap = n;
    }
    // longest job first, each to the least-loaded stream
    for (int j = 0; j < n; j++) b->order[j] = j;
    auto mbs = [&](int j) { return (long long)(jobs[j].width / 16) * (jobs[j].height / 16); };
    for (int i = 1; i < n; i++) {  // insertion sort, descending
        int v = b->order[i], k = i - 1;
        while (k >= 0 && mbs(b->order[k]) < mbs(v)) {
            b->order[k + 1] = b->order[k];
            k--;
        }
        b->order[k + 1] = v;
    }
    for (int s = 0; s < b->nslots; s++) b->slot[s].load = 0;
    for (int i = 0; i < n; i++) {
        int best = 0;
        for (int s = 1; s < b->nslots; s++)
            if (b->slot[s].load < b->slot[best].load) best = s;
        b->where[b->order[i]] = best;
        b->slot[best].load += mbs(b->order[i]);
    }
    VPP_CUDA(cudaEventRecord(b->start, b->parent->stream));
    for (int s = 0; s < b->nslots; s++) VPP_CUDA(cudaStreamWaitEvent(b->slot[s].ctx->stream, b->start, 0));
    for (int i = 0; i < n; i++) {
        const int j = b->order[i];
        const vppgpu_me_job& J = jobs[j];
        BatchSlot& sl = b->slot[b->where[j]];
        vppgpu_me* me = nullptr;
        if ((rc = slot_estimator(b, sl, J.width, J.height, J.motion_range, &me))) return rc;
        if ((rc = vppgpu_me_estimate_device(me, J.src, J.ref, J.dist_included, nullptr, J.mv_out, J.mb_dist_out,
                                            nullptr)))
            return rc;
        VPP_CUDA(cudaMemcpyAsync(b->h_ctrl + j, me->ctrl, sizeof(vppgpu::MeCtrl), cudaMemcpyDeviceToHost,
                                 sl.ctx->stream));
        if (J.levels_out) {
            // the coding stage on the same stream: residual at the vectors, then T+Q and its inverse over the
            // full macroblock rows (rows below them carry no residual)
            if ((rc = vppgpu_me_residual_device(me, J.mv_out, J.residual_out))) return rc;
            if ((rc = vppgpu_tq_roundtrip_plane_device(sl.ctx, J.residual_out, J.levels_out, J.recon_out, J.width,
                                                       16 * (J.height / 16), J.width, J.qp, 0,
                                                       VPPGPU_INV_ROWS_FIRST, nullptr)))
                return rc;
        }
    }
    for (int s = 0; s < b->nslots; s++) {
        VPP_CUDA(cudaEventRecord(b->done[s], b->slot[s].ctx->stream));
        VPP_CUDA(cudaStreamWaitEvent(b->parent->stream, b->done[s], 0));
    }
    VPP_CUDA(cudaStreamSynchronize(b->parent->stream));
    int first = VPPGPU_OK;
    for (int j = 0; j < n; j++) {
        const int st = status_from_ctrl(b->h_ctrl[j]);
        if (status_out) status_out[j] = st;
        if (avg_out) avg_out[j] = b->h_ctrl[j].count ? (long)(b->h_ctrl[j].total / b->h_ctrl[j].count) : 0;
        if (st && !first) first = st;
    }
    return first;
}

int vppgpu_me_batch_launch_count(vppgpu_me_batch* b, unsigned long long* count)
{
    if (!b || !count) return VPPGPU_ERR_INVALID_ARG;
    unsigned long long c = 0;
    for (int s = 0; s < b->nslots; s++) c += b->slot[s].ctx->launches;
    *count = c;
    return VPPGPU_OK;
}

}  // extern "C"
