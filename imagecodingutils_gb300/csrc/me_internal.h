// me_internal.h -- host/device argument blocks of the motion estimators.
#pragma once

#include "vppgpu_internal.cuh"

namespace vppgpu {

// Per-estimate device control block, zeroed before every estimate.
struct MeCtrl {
    int status;      // ST_* bits
    unsigned bar[2]; // grid barrier: arrivals, generation
    int sweeps;      // resolve sweeps used
    long long total; // sum of included distortions
    int count;       // number of included macroblocks
    int pad;
};

struct FullArgs {
    int W, H, cols, nmb, motion_range, rstride;
    const unsigned char* src8;  // W x H input, unpadded
    const unsigned char* refp;  // padded reference (PAD samples each side)
    // speculative (prediction-independent) results of k_full_search
    int* spec_mv;    // packed quarter-pel vector after sub-pel refinement
    int* spec_imv;   // packed full-pel winner
    int* spec_min;   // distortion of spec_mv
    int* spec_zero;  // distortion of the zero vector
    int* spec_flags; // FLAG_TIE: the scan met an exact tie
    int* tables;     // 64x64 SSD table per macroblock (kept for tie macroblocks)
    // fixed-point state of k_full_resolve
    int* final_mv;
    int* final_dist;
    int* pred_used;
    const int* slice;          // nullable
    const unsigned char* incl; // nullable
    int* out_mv;               // packed short2 per macroblock
    int* out_dist;             // nullable
    long long* out_avg;        // nullable
    MeCtrl* ctrl;
    int* changed;              // one counter per sweep
    double lambda;
    int sweep_limit;
    long long spin_limit;
};

size_t full_search_smem();
int full_prepare(vppgpu_ctx* ctx, int nmb, int* resolve_grid);
// ev: nullptr, or 4 events recorded before the pack kernel, before the
// search kernel, before the resolve kernel and after it.
int full_launch(vppgpu_ctx* ctx, const FullArgs& args, int nmb, const short* d_src16, const short* d_ref16,
                int resolve_grid, cudaEvent_t* ev);

}  // namespace vppgpu
