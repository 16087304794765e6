// me_internal.h -- host/device argument blocks of the motion estimators.
#pragma once

#include "vppgpu_internal.cuh"

namespace vppgpu {

// Per-estimate device control block, zeroed before every estimate.
struct MeCtrl {
    int status;      // ST_* bits
    unsigned bar[2]; // grid barrier: arrivals, generation
    int sweeps;      // relaxation sweeps used (+1000 when the wavefront finished the frame)
    long long total; // sum of included distortions
    int count;       // number of included macroblocks
    int converged;   // relaxation reached the fixed point
    int relax_evals; // MB evaluations in the relaxation sweeps
    int relax_miss;  // ... of which computed the prediction distortion
    int wave_miss;   // MBs the wavefront had to evaluate in full
    int pad;
};

// What the wavefront needs of one macroblock, 112 bytes (seven 16-byte
// copies): its records as {prediction, final vector} pairs and its
// neighbour-availability word.
struct WaveRec {
    int2 kv[12];
    int av;
    int pad[3];
};

struct FullArgs {
    int W, H, cols, nmb, motion_range, rstride;
    const unsigned char* src8;  // W x H input, unpadded
    const unsigned char* refp;  // padded reference (PAD samples each side)
    // half-pel planes of the padded reference, same geometry as refp, one
    // after the other: b (horizontal), h (vertical), j (centre)
    const unsigned char* hpel;
    size_t plane_size;          // bytes of one padded plane
    // speculative (prediction-independent) results of k_full_search, per MB:
    // {packed quarter-pel vector after sub-pel refinement, its distortion,
    //  zero-vector distortion, flags (FLAG_TIE | neighbour availability)}
    int4* spec4;
    int* spec_imv;   // packed full-pel winner
    int* tables;     // 64x64 SSD table per macroblock (kept for tie macroblocks)
    // resolve state
    int* final_mv;
    int* final_dist;
    int* pred_used;
    int4* cache;     // KCACHE records per MB: {prediction, distortion at it, final vector, final distortion}
    int* dict;       // dominant vectors of the frame (NDICT)
    const int* slice;          // nullable
    const unsigned char* incl; // nullable
    int* out_mv;               // packed short2 per macroblock
    int* out_dist;             // nullable
    long long* out_avg;        // nullable
    MeCtrl* ctrl;
    int* changed;              // one counter per sweep
    void* wave_scratch;        // WAVE_WARPS per-warp scratch areas of the wavefront
    WaveRec* wave_rec;         // per MB
    int* wave_choice;          // per MB: record the wavefront took, or -1 (evaluated, final_dist holds it)
    double lambda;
    int sweep_limit;
    long long spin_limit;
};

constexpr int KCACHE = 12;  // cache entries per macroblock
constexpr int NDICT = 8;    // dictionary vectors
constexpr int WAVE_WARPS = 16;  // most warps of the single-CTA wavefront (32 rows each)

size_t full_search_smem();
// Launch the prediction-dependent tail (sweep 0, relaxation, dictionary
// precompute, exact wavefront) of an estimate whose search has run.
int full_resolve_launch(vppgpu_ctx* ctx, const FullArgs& args, int resolve_grid);
int full_resolve_prepare(vppgpu_ctx* ctx, int* resolve_cap);
size_t full_wave_scratch_bytes();  // bytes behind FullArgs::wave_scratch
int full_prepare(vppgpu_ctx* ctx, int nmb, int* resolve_grid);
// ev: nullptr, or 4 events recorded before the pack kernel, before the
// search kernel, before the resolve kernel and after it.
int full_launch(vppgpu_ctx* ctx, const FullArgs& args, int nmb, const short* d_src16, const short* d_ref16,
                int resolve_grid, cudaEvent_t* ev);

}  // namespace vppgpu
