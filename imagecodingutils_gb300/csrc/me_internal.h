// me_internal.h -- host/device argument blocks of the motion estimators.
#pragma once

#include <cuda.h>  // CUtensorMap (types only; the encoder is reached through the runtime's driver entry point)

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
    int ntie;        // entries of FullArgs::tie_list
    int ticket;      // MultiresCrossVer2 dataflow pass: next macroblock
    int tie_mbs;     // H263 MultiresCrossVer2: entries of its tie list
};

constexpr int KCACHE = 32;  // records per macroblock

// What the wavefront needs of one macroblock, 272 bytes: its records as a
// hash table of 64 four-byte entries (16 buckets of 4; an entry is the
// prediction as two signed 11-bit halves, bits 0..21, and how the final
// vector follows from it, bits 22..23: 0 the searched vector, 1 the
// prediction itself, 2 zero; 0xffffffff is empty), the searched vector and
// the neighbour-availability word.  Stored along the wavefront's diagonals:
// band b (rows 32b..32b+31), step t, lane l (row 32b+l, column t-2l) at
// (b*(cols+62) + t)*32 + l, so the 32 records one warp needs at one step are
// contiguous.
struct WaveRec {
    unsigned slot[64];
    int spec;
    int av;
    int pad[2];
};
__host__ __device__ inline size_t wave_rec_count(int cols, int rows)
{
    return (size_t)((rows + 31) / 32) * (cols + 62) * 32;
}
__host__ __device__ inline size_t wave_rec_index(int cols, int r, int c)
{
    return ((size_t)(r >> 5) * (cols + 62) + c + 2 * (r & 31)) * 32 + (r & 31);
}

// The per-estimate pointers, read by the kernels from device memory so that a
// captured kernel sequence (CUDA graph) serves every estimate of a handle.
struct JobDesc {
    const short* src16;        // input luma, W x H int16
    const short* ref16;        // reference luma
    const unsigned char* incl; // nullable: pDistortionIncluded
    const int* slice;          // nullable: macroblock slice map
    int* out_mv;               // packed short2 per macroblock
    int* out_dist;             // nullable
    long long* out_avg;        // nullable
};

struct FullArgs {
    int W, H, cols, nmb, motion_range, rstride;
    const unsigned char* src8;  // W x H input, unpadded
    const unsigned char* refp;  // padded reference (PAD samples each side)
    // half-pel planes of the padded reference, same geometry as refp, one
    // after the other: b (horizontal), h (vertical), j (centre)
    const unsigned char* hpel;
    size_t plane_size;          // bytes of one padded plane
    // speculative (prediction-independent) results of the search, per MB:
    // {packed quarter-pel vector after sub-pel refinement, its distortion,
    //  zero-vector distortion, flags (FLAG_TIE | neighbour availability)}
    int4* spec4;
    int* spec_imv;   // packed full-pel winner
    int* tables;     // 64x64 SSD table per macroblock, kept for the tie macroblocks only (row
                     // minima in column 0, tie tree in row 63)
    const int* energy;  // 16x16 block energies of the padded reference (int, rstride per row)
    int* tie_list;   // macroblocks whose scan met an exact tie (MeCtrl::ntie of them)
    // resolve state
    int* final_mv;
    int* final_dist;
    int* pred_used;
    int4* cache;     // KCACHE records per MB: {prediction, distortion at it, final vector, final distortion}
    int* dict;       // dominant vectors of the frame (NDICT)
    const JobDesc* job;        // device
    MeCtrl* ctrl;
    int* changed;              // MBs changed per sweep
    unsigned* dirty;           // one bit per MB: dependents of the MBs the last grid sweep changed
    WaveRec* wave_rec;         // wave_rec_count(cols, rows) records
    int* wave_choice;          // per MB: the prediction the wavefront found a record for, or 0x7fffffff
                               // (evaluated there; final_mv / final_dist hold the result)
    double lambda;
    int sweep_limit;
    int relax_sweeps;          // relaxation sweeps before the wavefront (0..RELAX_SWEEPS)
    int grid_sweeps;           // ... of which over every MB (the rest visit the dirty sets)
    int relax_blocks_per_sm;   // grid of a sweep over every MB
    long long spin_limit;
    // MultiresCrossVer2 only: the search's level planes (device mrc::MrcArgs)
    // and one sub-pel lattice per macroblock for searches at a prediction
    const void* mrc;
    void* lattice;
    int4* search_cache;  // V2_SEARCH_CACHE per MB: {rounded prediction, vector, distortion, tie levels or -1}
    void* tie_runs;      // 8 tie-tree runs (mrc::V2TieRun, 32 bytes) per MB
    int mode;            // Cross: 0 quarter, 1 half, 2 full pel
    int intpel;          // 1: the integer-pel SAD stage (no sub-pel, no prediction check)
};
constexpr int V2_SEARCH_CACHE = 4;

constexpr int NDICT = 8;    // dictionary vectors
constexpr int WAVE_WARPS = 5;   // most warps (bands of 32 rows) of one wavefront launch

// MultiresCross (me_mrc.cu): level planes in one scratch buffer.
constexpr int ST_OUT_OF_BOUNDS = 4;  // a read the reference would make outside its buffer
size_t mrc_scratch_bytes(int W, int H);
// warps: macroblocks (warps) per CTA of the search kernel, 2, 4 or 8.
int mrc_launch(vppgpu_ctx* ctx, int W, int H, int motion_range, int mode, const short* d_src16, const short* d_ref16,
               unsigned char* scratch, const unsigned char* incl, int* out_mv, int* out_dist, long long* out_avg,
               MeCtrl* ctrl, int warps = 8, bool h263 = false);

// MotionEstimatorH263ImplMultiresCrossVer2 (me_mrc.cu): the level planes in `scratch`
// (mrc_scratch_bytes), per-MB search results (s0; tie_list and tie_runs too: every macroblock of
// (H + 15) / 16 rows), relaxation and exact-pass vectors, records (H263V2_RECORDS per MB), per-sweep
// change counts and work lists; motion_range in half pels.
constexpr int H263V2_RECORDS = 4;
constexpr int H263V2_SWEEPS = 48;  // most relaxation sweeps
struct H263V2Job {
    int W, H, motion_range, mode, sweeps;
    const short* src16;
    const short* ref16;
    unsigned char* scratch;
    const unsigned char* incl;
    int* out_mv;
    int* out_dist;
    long long* out_avg;
    MeCtrl* ctrl;
    int4* s0;
    int* state;
    int* wave;
    int4* rec;
    int* changed;    // at least 64 + H263V2_SWEEPS entries
    int* lists;      // 3 * N_MB: the sweeps' work lists and queue marks
    int* tie_list;   // macroblocks whose search at (0, 0) met a tie
    void* tie_runs;  // their tie trees (mrc_tie_runs_bytes() per MB)
    int tree_grid;   // CTAs of the tie-tree kernel
};
int h263v2_launch(vppgpu_ctx* ctx, const H263V2Job& j);
int h263v2_prepare();  // once per process before the first launch (shared-memory limit)

// Device address of the status word (ST_* bits) of a handle's current
// estimate, and the C ABI status those bits stand for.
const int* me_status_word(vppgpu_me* me);
int status_from_bits(int bits);

// MultiresCrossVer2 (me_mrc.cu): level planes in `scratch`, the search at
// prediction (0, 0) into args.spec4 / final_mv, then the full-search
// estimator's prediction-dependent resolve with the Ver2 evaluation.
// args.mrc points to mrc_args_bytes() of device memory; args.lattice to
// nmb * mrc_lattice_bytes().
constexpr int RELAX_SWEEPS = 14;
size_t mrc_args_bytes();
size_t mrc_lattice_bytes();
size_t mrc_tie_runs_bytes();  // per macroblock
// MotionEstimatorH264ImplCross (me_cross.cu): the planes, the search at
// prediction (0, 0) into args.spec4 / final_mv (args.search_cache seeded for
// the tie macroblocks), then the resolve with the Cross evaluation
// (estimator 3).
int cross_launch(vppgpu_ctx* ctx, const FullArgs& args);
// est: 1 MultiresCrossVer2, 2 Multires (the same pipeline, their own search),
// 4 Ver2's Lagrangian overload (args.lambda is its lambda).
int mrc2_launch(vppgpu_ctx* ctx, int est, int mode, unsigned char* scratch, const FullArgs& args,
                const short* d_src16, const short* d_ref16);

// MotionEstimatorH264ImplUMHS (me_umhs.cu).  Its search starts at the
// prediction, so every macroblock's result is a function of its prediction
// (vector and distortion): relaxation sweeps evaluate every macroblock at the
// prediction of the current neighbour states and keep the evaluations as
// records; unless a sweep changes nothing (the fixed point, which is the
// sequential result), a dataflow pass over the wavefront order settles the
// exact raster result, looking predictions up in the records first.
constexpr int UMHS_RECORDS = 8;  // records per macroblock
constexpr int UMHS_SWEEPS = 24;  // most relaxation sweeps
constexpr int UMHS_EVALS = UMHS_SWEEPS + 2;  // FullArgs::changed index of the per-sweep search counts
struct UmhsArgs {
    FullArgs f;                 // planes, geometry, job, control, change counters
    unsigned long long* state;  // per MB: sweep state, packed vector | distortion << 32
    unsigned long long* wave;   // per MB: the dataflow pass's state, all ones until written
    int4* rec;                  // UMHS_RECORDS per MB: {prediction, outcome word, vector, distortion}
    const int* prev;            // per MB: the previous frame's full-pel starting point (packed; 0: none)
    const int* order;           // dataflow ticket -> macroblock (anti-diagonals c + 2r, rows ascending)
    int sweeps;                 // relaxation sweeps before the dataflow pass (>= 1)
    int diag_limit;             // last-sweep searches up to which the one-CTA diagonal pass starts
    int fhs;                    // 1: MotionEstimatorH264ImplFHS's search, 0: UMHS's
};
// The planes, `sweeps` relaxation sweeps, the dataflow pass (wave_grid CTAs of
// 4 warps) and the outputs.
int umhs_launch(vppgpu_ctx* ctx, const UmhsArgs& args, int wave_grid);
// MotionEstimatorImpl1 (me_impl1.cu): the planes, then a warp per bw x bh block
// (16x16 or 8x8) searching [-range, range-1]^2 full pels (range <= 32).
int impl1_launch(vppgpu_ctx* ctx, const FullArgs& args, int bw, int bh, int range);
// MotionEstimatorImpl2 (me_impl.cu): the planes, the level-1 / level-2 planes in
// `scratch` (impl2_scratch_bytes), then a warp per 16x16 block; mode 1 two
// levels, 2 three; range in full pels (4..32).
size_t impl2_scratch_bytes(int W, int H);
int impl2_launch(vppgpu_ctx* ctx, const FullArgs& args, unsigned char* scratch, int range, int mode);
// Once per device: the diagonal pass's shared-memory limit.
int umhs_prepare();

// Write this estimate's pointers to the device descriptor (a one-thread
// kernel with the descriptor as its parameter: stream-ordered, no host copy).
int set_job(vppgpu_ctx* ctx, JobDesc* d_job, const JobDesc& v);

// Motion-compensated luma residual of the last estimate's planes at vectors d_mv.
int full_residual_launch(vppgpu_ctx* ctx, const FullArgs& args, const int* d_mv, short* d_res);

// 2-D tensor maps the search kernel stages its tiles with (one TMA copy each
// per macroblock): the padded reference (80 x 78 window box), the packed
// input (16 x 16 template box) and the block energies (64 x 63 box).  They
// describe buffers, not a frame: encode once per buffer set.
struct SearchMaps {
    CUtensorMap win, cur, energy;
};
int search_maps_encode(const FullArgs& args, SearchMaps* maps);
// Byte-packed input (args.src8), padded reference and its half-pel planes
// from the int16 planes of args.job, and the block energies when args.energy
// is set (the SSD full search), in one kernel.
int full_planes_launch(vppgpu_ctx* ctx, const FullArgs& args);
// Launch the prediction-dependent tail (sweep 0, relaxation, dictionary
// precompute, exact wavefront) of an estimate whose search has run.
// est: 0 MotionEstimatorH264ImplFull, 1 MotionEstimatorH264ImplMultiresCrossVer2,
// 2 MotionEstimatorH264ImplMultires, 3 MotionEstimatorH264ImplCross, 4 Ver2's
// Lagrangian overload.
int full_resolve_launch(vppgpu_ctx* ctx, const FullArgs& args, int resolve_grid, int est);
int full_resolve_prepare(vppgpu_ctx* ctx, int* resolve_cap);
int full_prepare(vppgpu_ctx* ctx, int nmb, int* resolve_grid);
// ev: nullptr, or 5 events recorded before the pack kernel, before the
// search kernel, after it (before the sub-pel stage and the tie trees),
// before the resolve and after it.
int full_launch(vppgpu_ctx* ctx, const FullArgs& args, const SearchMaps& maps, int nmb, int resolve_grid,
                cudaEvent_t* ev);
// Integer-pel SAD full search: the MotionEstimatorH264ImplFull integer stage
// (MotionEstimatorH264ImplFull.cpp:341-446) with the MEH264IF_ABS_DIFF distortion.
int sad_launch(vppgpu_ctx* ctx, const FullArgs& args, const SearchMaps& maps, int nmb);
// Its prediction-dependent tail: the tie macroblocks in wavefront order, then the outputs.
int sad_resolve_launch(vppgpu_ctx* ctx, const FullArgs& args);

}  // namespace vppgpu
