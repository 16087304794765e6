/*
 * vppgpu.h -- C ABI of the GB300 (sm_103a) encoder hot path for vpp
 * (CSIR-RTVC/ImageCodingUtils).
 *
 * Every entry point is extern "C", takes plain pointers and sizes and returns
 * an int status (VPPGPU_OK = 0, negative on error); nothing throws across the
 * boundary.  Host-pointer entry points are synchronous: they copy inputs to
 * the device, run the kernels on the context's stream and copy results back.
 * `_device` entry points take device pointers, only enqueue work on the
 * context's stream and return at once.
 *
 * The interfaces each call replaces are cited per declaration (paths inside
 * the vpp source tree).  Pixel planes are `short` (vpp's yuvType and
 * OverlayMem2Dv2 element type) holding 0..255 luma; motion vectors are
 * quarter-pel {short x, short y} pairs per 16x16 macroblock in raster order,
 * the VectorStructList SIMPLE2D layout (include/CodecUtils/VectorStructList.h:56-60).
 *
 * Thread safety: one handle per host thread, as for the vpp classes
 * (single-threaded, non-reentrant per object).
 */
#ifndef VPPGPU_H
#define VPPGPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define VPPGPU_OK                 0
#define VPPGPU_ERR_INVALID_ARG   -1  /* null pointer, bad size or mode            */
#define VPPGPU_ERR_CUDA          -2  /* a CUDA runtime call failed                */
#define VPPGPU_ERR_OUT_OF_MEMORY -3  /* device or pinned allocation failed        */
#define VPPGPU_ERR_PIXEL_RANGE   -4  /* a luma sample outside 0..255              */
#define VPPGPU_ERR_TIMEOUT       -5  /* a bounded device-side wait gave up        */
#define VPPGPU_ERR_UNSUPPORTED   -6  /* configuration outside the supported set   */
#define VPPGPU_ERR_NOT_READY     -7  /* handle not created / creation failed      */
#define VPPGPU_ERR_NO_DEVICE     -8  /* no CUDA device, or not an sm_103 part     */

/* Human-readable name of a status code (static storage). */
const char* vppgpu_status_string(int status);

/* ---- context ------------------------------------------------------------ */
/* A context binds one CUDA device and one stream.  No vpp counterpart: the
 * vpp classes run on the calling thread; the context is where their GPU
 * replacements enqueue work. */
typedef struct vppgpu_ctx vppgpu_ctx;

int vppgpu_ctx_create(int device, vppgpu_ctx** out);
int vppgpu_ctx_destroy(vppgpu_ctx* ctx);
/* Use a caller-owned cudaStream_t (passed as void*) instead of the context's
 * own stream; NULL restores the context's stream. */
int vppgpu_ctx_set_stream(vppgpu_ctx* ctx, void* cuda_stream);
int vppgpu_ctx_get_stream(vppgpu_ctx* ctx, void** cuda_stream);
int vppgpu_ctx_synchronize(vppgpu_ctx* ctx);
/* Number of kernels this context has launched so far. */
int vppgpu_ctx_launch_count(vppgpu_ctx* ctx, unsigned long long* count);

/* ---- motion estimation -------------------------------------------------- */
/* Estimator kinds: the IMotionEstimator implementations replaced. */
#define VPPGPU_ME_FULL              0  /* MotionEstimatorH264ImplFull              */
#define VPPGPU_ME_MULTIRES          1  /* MotionEstimatorH264ImplMultires          */
#define VPPGPU_ME_MULTIRES_CROSS    2  /* MotionEstimatorH264ImplMultiresCross     */
#define VPPGPU_ME_MULTIRES_CROSS_V2 3  /* MotionEstimatorH264ImplMultiresCrossVer2 */
#define VPPGPU_ME_CROSS             4  /* MotionEstimatorH264ImplCross             */
#define VPPGPU_ME_H263_MULTIRES_CROSS 5 /* MotionEstimatorH263ImplMultiresCross:
                                            motion range (<= 64) and vectors in half pels */
/* The integer-pel stage of MotionEstimatorH264ImplFull::Estimate
 * (src/CodecUtils/MotionEstimatorH264ImplFull.cpp:341-446) with its
 * MEH264IF_ABS_DIFF distortion: OverlayMem2Dv2::Tad16x16 for the zero vector and
 * Tad16x16LessThan for the scan (src/ImageUtils/OverlayMem2Dv2.cpp:2655-2960).
 * Vectors are the full-pel winners in quarter pels, distortions their SAD; no
 * sub-pel stage, prediction check or GetBestVector.  The median prediction
 * still decides exact ties, so the estimator keeps the predictor contract. */
#define VPPGPU_ME_FULL_SAD          6
/* MotionEstimatorH264ImplUMHS (src/CodecUtils/MotionEstimatorH264ImplUMHS.cpp:446-945):
 * the unsymmetrical-cross multi-hexagon-grid search from the median prediction,
 * built as by its eight-argument constructor (…ImplUMHS.cpp:231-254; the others
 * leave the previous-frame macroblocks unset while Estimate reads them).  Its
 * predictor also predicts a distortion (MacroBlockH264.cpp:818-915), so the
 * caller's predictor side effect is Set16x16MotionVector(k, x, y, mb_dist_out[k])
 * (H264MotionVectorPredictorImpl1.h:112-121).  Modes 0 quarter (default), 1 half,
 * 2 full pel, kept as given. */
#define VPPGPU_ME_UMHS              7
/* MotionEstimatorH264ImplFHS (src/CodecUtils/MotionEstimatorH264ImplFHS.cpp:497-900):
 * the four-scale hexagon search from the median prediction on 80-point
 * extrapolated path distortions (Td16x16OptimalPathLessThan, :1685-1790) with
 * integer costs, its own half / quarter-pel stages (:1109-1480) and the
 * prediction check.  The same predictor contract as VPPGPU_ME_UMHS (a predicted
 * distortion; Set16x16MotionVector with mb_dist_out); no previous-frame input
 * (the reference's use of it is disabled, :627-673).  Modes 0 quarter (default),
 * 1 half, 2 full pel.  Where the reference's quarter-pel pass would read sub-pel
 * samples its cache holds from earlier macroblocks (the half-pel stage left
 * early without an improvement), this macroblock's samples are used; such
 * macroblocks are counted in vppgpu_me_last_stats()[7]. */
#define VPPGPU_ME_FHS               8
/* MotionEstimatorImpl1 (src/CodecUtils/MotionEstimatorImpl1.cpp:275-395): the
 * H.263-style full search of [-motion_range, motion_range-1]^2 FULL pels by SSD,
 * the OverlayMem2Dv2::HalfRead half-pel refinement and the weighted choice
 * between the winner and the zero vector; no predictor.  Vectors in HALF pels
 * (the reference stores them as chars in a SimpleMotionVectorList), one per
 * block of the size given to vppgpu_me_create_blocks (16x16 through
 * vppgpu_me_create); avg_distortion over every block.  1 <= motion_range <= 32;
 * heights must be a multiple of the block height (the reference reads past
 * its input for a partial row). */
#define VPPGPU_ME_IMPL1             9
/* MotionEstimatorImpl2 (src/CodecUtils/MotionEstimatorImpl2.cpp:505-826): a SAD
 * pyramid for 16x16 blocks, motion_range in FULL pels (4..32): SetMode(2) (or 0
 * above 40000 pixels) a full search at level 2 then +-2 at level 1, SetMode(1)
 * (the default) a full search at level 1; +-2 at level 0, ties towards the
 * origin; HalfRead half pel; the weighted zero-vector choice.  Vectors in HALF
 * pels, as for VPPGPU_ME_IMPL1. */
#define VPPGPU_ME_IMPL2             10
/* MotionEstimatorH263ImplMultiresCrossVer2
 * (src/CodecUtils/MotionEstimatorH263ImplMultiresCrossVer2.cpp:537-1151) with
 * H263MotionVectorPredictorImpl1 (src/CodecUtils/H263MotionVectorPredictorImpl1.cpp:72-128):
 * the H.263 MultiresCross search with ties decided towards the prediction of
 * each level, then the better of the prediction (clamped, HalfRead for its
 * half-pel part) and the zero vector against the searched vector.  Motion
 * range (<= 64) and vectors in half pels; avg_distortion over every macroblock
 * when incl is NULL (the partial bottom row's too).  The prediction is the
 * H.263 median of the vectors this estimate writes (left; above; above-right,
 * zero beyond the right edge; the left one in the top row): there is no
 * predictor object to pass and slice maps are ignored. */
#define VPPGPU_ME_H263_MULTIRES_CROSS_V2 11

typedef struct vppgpu_me vppgpu_me;

/* Constructor + Create() of the estimator (src/CodecUtils/MotionEstimatorH264ImplFull.cpp:132-153,
 * 216-320; same shape for the other kinds): allocates all device state for a
 * width x height luma frame and a quarter-pel motion range.  width must be a
 * multiple of 16; a partial bottom macroblock row (height % 16 != 0) is not
 * reported, as in the reference (Full.cpp:293, 594).  Supported ranges:
 * 4 <= motion_range <= 128 (search of at most +-31 pels); ranges 0..3, for
 * which the reference runs a sub-pel-only search, are refused with
 * VPPGPU_ERR_INVALID_ARG. */
int vppgpu_me_create(vppgpu_ctx* ctx, int kind, int width, int height, int motion_range,
                     vppgpu_me** out);
/* The same for estimators whose constructor takes a block size: MotionEstimatorImpl1's
 * (pSrc, pRef, w, h, macroBlkWidth, macroBlkHeight, motionRange) (MotionEstimatorImpl1.cpp:111-135),
 * blocks 16x16 or 8x8, and MotionEstimatorImpl2's (MotionEstimatorImpl2.cpp:111-181), 16x16.  Every
 * other kind accepts 16x16 only. */
int vppgpu_me_create_blocks(vppgpu_ctx* ctx, int kind, int width, int height, int block_w, int block_h,
                            int motion_range, vppgpu_me** out);
int vppgpu_me_destroy(vppgpu_me* me);
/* IMotionEstimator::SetMode / GetMode (include/CodecUtils/IMotionEstimator.h:80-81). */
int vppgpu_me_set_mode(vppgpu_me* me, int mode);
int vppgpu_me_get_mode(vppgpu_me* me, int* mode);
/* Number of vectors an estimate produces: (width/16)*(height/16). */
int vppgpu_me_num_mbs(vppgpu_me* me, int* n);

/* IMotionEstimator::Estimate(long* avgDistortion) (IMotionEstimator.h:90-93;
 * MotionEstimatorH264ImplFull::Estimate, Full.cpp:330-613), host buffers.
 *   src, ref       width*height shorts, luma 0..255 (else VPPGPU_ERR_PIXEL_RANGE)
 *   dist_included  NULL or one flag per macroblock: the reference's
 *                  pDistortionIncluded constructor argument
 *   mb_slice       NULL (one slice) or one slice id per macroblock: the
 *                  neighbourhood MacroBlockH264::Initialise wires for the
 *                  median predictor (src/CodecUtils/MacroBlockH264.cpp:319-)
 *   mv_out         2 shorts per macroblock (the VectorStructList contents)
 *   mb_dist_out    NULL or one int per macroblock: distortion of the chosen vector
 *   avg_distortion NULL or the avgDistortion out-parameter
 * The caller then applies mv_out to its IMotionVectorPredictor with
 * Set16x16MotionVector(k, x, y) for every k, the side effect the reference has
 * (include/CodecUtils/H264MotionVectorPredictorImpl1.h:103-111). */
int vppgpu_me_estimate(vppgpu_me* me, const short* src, const short* ref,
                       const unsigned char* dist_included, const int* mb_slice,
                       short* mv_out, int* mb_dist_out, long* avg_distortion);

/* Same with device pointers; enqueued on the context stream.  avg_out is a
 * device long long. */
int vppgpu_me_estimate_device(vppgpu_me* me, const short* d_src, const short* d_ref,
                              const unsigned char* d_dist_included, const int* d_mb_slice,
                              short* d_mv_out, int* d_mb_dist_out, long long* d_avg_out);

/* IMotionEstimator::Estimate(long*, void* param) with a Lagrange multiplier:
 * for VPPGPU_ME_MULTIRES_CROSS_V2 the Lagrangian overload
 * (MotionEstimatorH264ImplMultiresCrossVer2.cpp:1162-1742: GetBestVector at
 * every search level and at the end with this lambda); every other kind
 * ignores the parameter (IMotionEstimator.h:94) and runs Estimate(long*). */
int vppgpu_me_estimate_lambda(vppgpu_me* me, const short* src, const short* ref,
                              const unsigned char* dist_included, const int* mb_slice,
                              double lambda, short* mv_out, int* mb_dist_out,
                              long* avg_distortion);

/* The previous frame's macroblocks of MotionEstimatorH264ImplUMHS's
 * pPrevFrmMBlk argument (…ImplUMHS.cpp:231-254, read at :551-571): per macroblock
 * its 16x16 vector (MacroBlockH264::_mvX[0], _mvY[0], quarter pels; 2 shorts) and
 * intra flag (MacroBlockH264::_intraFlag; NULL: all inter).  prev_mv NULL: all
 * zero.  Kept for every later estimate of the handle until set again.  A vector
 * whose block origin (full pels, C division) leaves [-16, width] x [-16, height],
 * which an earlier estimate never produces and for which the reference would
 * read outside its buffers, is refused with VPPGPU_ERR_INVALID_ARG.  Other kinds:
 * VPPGPU_ERR_UNSUPPORTED.  Synchronous. */
int vppgpu_me_set_prev_frame(vppgpu_me* me, const short* prev_mv, const unsigned char* prev_intra);

/* Status of the last device-side estimate (pixel-range or timeout flags);
 * synchronises the context stream. */
int vppgpu_me_last_status(vppgpu_me* me);

/* Number of resolve sweeps the last estimate needed (predictor fixed point). */
int vppgpu_me_last_sweeps(vppgpu_me* me, int* sweeps);

/* Estimators with a predictor, no vpp counterpart: at most this many
 * relaxation sweeps (0..14, UMHS 0..24; defaults 14 Full and Multires, 4 Ver2, 20 UMHS; fewer when
 * the changes stop falling fast) run before the exact wavefront decides the
 * macroblocks whose predictions have not settled.  Results do not depend on it. */
int vppgpu_me_set_relax_sweeps(vppgpu_me* me, int sweeps);

/* Autotuning, no vpp counterpart: times the estimator's tunable launch shapes
 * and relaxation policy on one device frame pair (reps estimates each; every
 * candidate must and is checked to give the same vectors) and keeps the
 * fastest; *chosen (nullable) is its index, 0 = the configuration before the
 * call.  Tunables: MultiresCross -- macroblocks per search CTA (2, 4, 8);
 * the others -- relaxation sweeps / of which over every MB, and the CTAs per
 * SM of such a sweep.  vppgpu_me_get_tuning returns {relaxation sweeps, grid
 * sweeps, sweep CTAs per SM, search macroblocks per CTA}. */
int vppgpu_me_autotune(vppgpu_me* me, const short* d_src, const short* d_ref, int reps, int* chosen);
/* Same over several device frame pairs (each candidate timed over all). */
int vppgpu_me_autotune_pairs(vppgpu_me* me, const short* const* d_src, const short* const* d_ref, int npairs,
                             int reps, int* chosen);
/* Same with host planes (copied once). */
int vppgpu_me_autotune_host(vppgpu_me* me, const short* src, const short* ref, int reps, int* chosen);
int vppgpu_me_get_tuning(vppgpu_me* me, int* tuning4);

/* Counters of the last estimate's prediction-dependent stage: {sweeps,
 * converged-by-relaxation, relaxation evaluations, of which distortion
 * computations (UMHS / FHS: searches in the relaxation), MBs the wavefront
 * evaluated in full, status bits, included MBs, a kind-specific count (Full:
 * macroblocks whose scan met a tie; FHS: quarter-pel passes over samples the
 * reference would take from earlier macroblocks)}.  Synchronises the context
 * stream.  No vpp counterpart. */
int vppgpu_me_last_stats(vppgpu_me* me, int* stats8);
/* Macroblocks whose final vector changed in each relaxation sweep 1 .. n of
 * the last estimate (n <= 14; 0 for sweeps that did not run).  Synchronises
 * the context stream.  No vpp counterpart: a diagnostic of the relaxation
 * policy (vppgpu_me_set_relax_sweeps). */
int vppgpu_me_last_relax_changes(vppgpu_me* me, int* changes, int n);

/* Observability, no vpp counterpart.  While enabled, every estimate records
 * CUDA events around its three kernels on the context stream (no host
 * synchronisation); vppgpu_me_timing synchronises and returns how many
 * estimates were timed and the summed milliseconds of the pack, search and
 * resolve kernels.  Enabling resets the sums. */
int vppgpu_me_set_timing(vppgpu_me* me, int enable);
int vppgpu_me_timing(vppgpu_me* me, int* n, double* pack_ms, double* search_ms, double* resolve_ms);
/* The same sums split by stage: {pack + half-pel planes, SSD table, scan +
 * sub-pel + tie trees, prediction-dependent resolve}. */
int vppgpu_me_timing_stages(vppgpu_me* me, int* n, double* stage_ms4);

/* Motion-compensated luma residual of the last estimate of a Full estimator:
 * for every macroblock, input minus the reference read at its vector
 * (MotionCompensatorH264ImplStd::Compensate luma, MotionCompensatorH264ImplStd.cpp:413-431:
 * QuarterRead at the quarter-pel vector, a copy for a full-pel one; then
 * OverlayMem2Dv2::Sub16x16), as int16 W x H (16-byte aligned).  d_mv: 2 shorts
 * per macroblock, e.g. the estimate's own output.  Enqueued on the context
 * stream after the estimate.  A vector whose prediction lies more than 32
 * samples outside the picture (never one the estimator returns) gets a zero
 * residual and makes vppgpu_me_last_status return VPPGPU_ERR_UNSUPPORTED. */
int vppgpu_me_residual_device(vppgpu_me* me, const short* d_mv, short* d_residual);

/* Batched estimation, no vpp counterpart (the codecs estimate one frame at a
 * time).  A batch runs many independent frame pairs of any mix of sizes on
 * `streams` streams of its own, so that the latency-bound stages of one
 * frame overlap the search of others; outputs are identical to estimating
 * each job alone.  Device pointers; a job's planes are W x H luma 0..255.
 * vppgpu_me_batch_run enqueues after the work on the context's stream,
 * waits for the batch, and returns per job its status and avgDistortion
 * (either array may be NULL); the return value is the first non-zero job
 * status.  Estimators are created per stream and frame geometry on first
 * use and kept for later batches. */
typedef struct vppgpu_me_batch vppgpu_me_batch;
typedef struct {
    const short* src;                    /* device, W x H */
    const short* ref;                    /* device, W x H */
    int width, height, motion_range;
    const unsigned char* dist_included;  /* device, one flag per MB, or NULL */
    short* mv_out;                       /* device, 2 shorts per MB */
    int* mb_dist_out;                    /* device, one int per MB, or NULL */
    /* Optional coding stage of the job (levels_out NULL: none): the
     * motion-compensated luma residual at the estimated vectors
     * (vppgpu_me_residual_device) into residual_out, then its 4x4 forward
     * transform + quantisation at `qp` (inter rounding) and the dequantised
     * inverse (vppgpu_tq_roundtrip_plane_device, rows first) over the full
     * macroblock rows into levels_out / recon_out.  Device, W x H shorts each;
     * Full estimator batches only. */
    short* residual_out;
    short* levels_out;
    short* recon_out;
    int qp;
} vppgpu_me_job;
int vppgpu_me_batch_create(vppgpu_ctx* ctx, int kind, int streams, vppgpu_me_batch** out);
int vppgpu_me_batch_destroy(vppgpu_me_batch* b);
int vppgpu_me_batch_run(vppgpu_me_batch* b, const vppgpu_me_job* jobs, int n, int* status_out, long* avg_out);
int vppgpu_me_batch_launch_count(vppgpu_me_batch* b, unsigned long long* count);

/* ---- motion compensation ------------------------------------------------ */
/* MotionCompensatorH264ImplStd(range) + Create(ref, width, height, 16, 16)
 * (src/CodecUtils/MotionCompensatorH264ImplStd.cpp:76-258).  The frame is
 * contiguous 4:2:0 int16: Y width*height, then U and V (width/2)*(height/2). */
typedef struct vppgpu_mc vppgpu_mc;
int vppgpu_mc_create(vppgpu_ctx* ctx, int width, int height, int range, vppgpu_mc** out);
int vppgpu_mc_destroy(vppgpu_mc* mc);
/* Compensate(pMotionList) (…ImplStd.cpp:323-473): every macroblock of the
 * frame replaced by the block its quarter-pel vector points at (luma
 * QuarterRead, chroma EighthRead at the same vector in eighth-pel units; a
 * zero vector keeps the block), read from the frame as it was before the
 * call.  Host version in place like the reference; the device version writes
 * d_out_yuv, which may be d_ref_yuv.  Vectors: 2 shorts per macroblock of the
 * full macroblock rows, within the range (the reference's extended border). */
int vppgpu_mc_compensate(vppgpu_mc* mc, short* yuv, const short* mv);
int vppgpu_mc_compensate_device(vppgpu_mc* mc, const short* d_ref_yuv, const short* d_mv, short* d_out_yuv);
/* OverlayMem2Dv2::Add16x16WithClip255 / Add8x8WithClip255 and Sub16x16 /
 * Sub8x8 (OverlayMem2Dv2.cpp:1195-1426) over n samples of whole planes:
 * a = clip255(a + b) (prediction + residual -> reconstruction), a -= b
 * (input - prediction -> residual).  16-byte aligned device pointers. */
int vppgpu_add_clip255_device(vppgpu_ctx* ctx, short* d_a, const short* d_b, long long n);
int vppgpu_sub_device(vppgpu_ctx* ctx, short* d_a, const short* d_b, long long n);

/* Serving, no vpp counterpart: a continuous-batching request loop for
 * sequence jobs.  A request is nframes host luma planes (W x H, back to back;
 * kept valid until the request completes); for every frame pair the server
 * estimates the Full-search vectors (motion_range), forms the
 * motion-compensated luma residual and runs the 4x4 transform + quantisation
 * round trip on it (inter rounding, qp), returning the vectors
 * ((nframes-1) x N_MB x 2 shorts, nullable) and per pair a digest
 * sum(levels + 3*reconstruction) (nullable).  Frames are uploaded once and
 * stay on the device as the next pair's reference.  `slots` worker threads
 * with their own streams take the oldest queued request whose device buffers
 * fit under `hbm_budget` bytes (0: half of the free memory), so requests
 * arriving while others run are admitted as slots and memory free up and
 * overlap on the device.  Results are identical to running each request
 * alone.  poll() returns completed tickets with status and submit-to-done
 * latency. */
typedef struct vppgpu_server vppgpu_server;
typedef struct {
    int width, height, nframes, motion_range, qp;
    const short* frames;               /* host */
    short* mv_out;                     /* host, nullable */
    unsigned long long* digest_out;    /* host, nframes-1 values, nullable */
} vppgpu_seq_request;
int vppgpu_server_create(vppgpu_ctx* ctx, int slots, unsigned long long hbm_budget, vppgpu_server** out);
/* Create every slot's estimator for one frame geometry now (otherwise the
 * first request of that geometry on a slot creates it). */
int vppgpu_server_prepare(vppgpu_server* s, int width, int height, int motion_range);
int vppgpu_server_submit(vppgpu_server* s, const vppgpu_seq_request* r, unsigned long long* ticket);
int vppgpu_server_poll(vppgpu_server* s, int max, unsigned long long* tickets, int* status, double* latency_ms,
                       int* n);
int vppgpu_server_wait_idle(vppgpu_server* s);
int vppgpu_server_stats(vppgpu_server* s, unsigned long long* reserved_peak, int* running_peak);
int vppgpu_server_destroy(vppgpu_server* s);

/* Measured dp4a issue rate of the whole device (instructions per second),
 * the integer-ALU roofline of the motion search.  No vpp counterpart. */
int vppgpu_calibrate_dp4a(vppgpu_ctx* ctx, double* dp4a_per_second);

/* Full search without any device allocation.  No counterpart in the
 * reference: it exists for callers that must not allocate device memory once
 * running (real-time encoders with a fixed budget, plugins inside a host
 * that owns all allocations, code paths that forbid allocator calls after
 * start-up).  Same kernels and results as vppgpu_me_estimate_device, but all
 * intermediate buffers live in one 12 MiB static device array held by every
 * GPU that loads the library until the process exits.  Limits: at most
 * VPPGPU_NOALLOC_MAX_MBS stored macroblocks and width, height at most
 * VPPGPU_NOALLOC_MAX_DIM, else VPPGPU_ERR_UNSUPPORTED.  Inputs and outputs are
 * the caller's device buffers; cuda_stream is a cudaStream_t (NULL: default
 * stream); the call returns when the results are written.  All calls share
 * the array, so calls that overlap on the GPU race and must be serialised.
 * The first call on a device (with that device current) looks up the array's
 * address; with lazy module loading it is also when the driver reserves the
 * array, so make it at start-up, before any stream capture.  motion_range
 * as for vppgpu_me_create (4..128). */
#define VPPGPU_NOALLOC_MAX_MBS 396
#define VPPGPU_NOALLOC_MAX_DIM 1024
int vppgpu_me_full_estimate_noalloc(const short* d_src, const short* d_ref, int width, int height,
                                    int motion_range, const unsigned char* d_dist_included,
                                    const int* d_mb_slice, short* d_mv_out, int* d_mb_dist_out,
                                    long* avg_distortion, void* cuda_stream);

/* ---- 4x4 integer transform + H.264 quantisation ------------------------- */
/* Modes (include/CodecUtils/IForwardTransform.h:119-125). */
#define VPPGPU_TQ_TRANSFORM_AND_QUANT 0
#define VPPGPU_TQ_TRANSFORM_ONLY      1
#define VPPGPU_TQ_QUANT_ONLY          2
/* Data layouts. */
#define VPPGPU_LAYOUT_BLOCKS 0  /* contiguous 16-short 4x4 blocks: FastForward4x4ITImpl1/2,
                                   FastInverse4x4ITImpl1 (one Transform(void*) per block) */
#define VPPGPU_LAYOUT_MB16   1  /* 256-short 16x16 raster macroblocks:
                                   FastForward4x4On16x16ITImpl1 / FastInverse4x4On16x16ITImpl1 */
/* Inverse pass order: rows first (FastInverse4x4ITImpl1) or columns first
 * (FastInverse4x4On16x16ITImpl1); the int16 stores between the passes make
 * the two differ. */
#define VPPGPU_INV_ROWS_FIRST 0
#define VPPGPU_INV_COLS_FIRST 1

/* IForwardTransform::Transform(void*) over nunits units in place
 * (src/CodecUtils/FastForward4x4ITImpl1.cpp:100-201; On16x16: FastForward4x4On16x16ITImpl1.cpp:457-757),
 * with SetMode(mode), SetParameter(QUANT_ID, qp), SetParameter(INTRA_FLAG_ID, intra). */
int vppgpu_fwd4x4(vppgpu_ctx* ctx, short* data, long long nunits, int layout, int mode, int qp,
                  int intra);
int vppgpu_fwd4x4_device(vppgpu_ctx* ctx, short* d_data, long long nunits, int layout, int mode,
                         int qp, int intra);

/* IInverseTransform::InverseTransform(void*) over nunits units in place
 * (src/CodecUtils/FastInverse4x4ITImpl1.cpp:119-244; On16x16: FastInverse4x4On16x16ITImpl1.cpp:120-361).
 * weight16: NULL (flat 16) or the SetScale() array of 16 ints (FastInverse4x4ITImpl1.cpp:251-268).
 * The blocks layout runs rows first, the mb16 layout columns first. */
int vppgpu_inv4x4(vppgpu_ctx* ctx, short* data, long long nunits, int layout, int mode, int qp,
                  const int* weight16);
int vppgpu_inv4x4_device(vppgpu_ctx* ctx, short* d_data, long long nunits, int layout, int mode,
                         int qp, const int* weight16);

/* Fused residual round trip over a raster plane (width, height multiples of
 * 4, row stride in shorts): every 4x4 block goes through forward transform +
 * quantisation (mode 0), the levels are written to `levels`, then through
 * dequantisation + inverse transform (mode 0, `inv_order`), written to
 * `recon`.  This is BlockH264::ForwardTransform/Quantise followed by
 * InverseQuantise/InverseTransform (src/CodecUtils/BlockH264.cpp:136-196)
 * for a whole plane in one pass. */
int vppgpu_tq_roundtrip_plane(vppgpu_ctx* ctx, const short* residual, short* levels, short* recon,
                              int width, int height, int stride, int qp, int intra,
                              int inv_order, const int* weight16);
int vppgpu_tq_roundtrip_plane_device(vppgpu_ctx* ctx, const short* d_residual, short* d_levels,
                                     short* d_recon, int width, int height, int stride, int qp,
                                     int intra, int inv_order, const int* weight16);

/* One plane of a batched round trip. */
typedef struct vppgpu_tq_job {
    const short* residual; /* device */
    short* levels;         /* device */
    short* recon;          /* device */
    int width, height, stride;
    int qp, intra;
} vppgpu_tq_job;

/* Many planes (e.g. the Y, U, V planes of many frames, each at its own QP and
 * intra/inter rounding) in one launch; `d_jobs` is a device array of njobs
 * descriptors. */
int vppgpu_tq_roundtrip_planes_device(vppgpu_ctx* ctx, const vppgpu_tq_job* d_jobs, int njobs, int inv_order,
                                      const int* weight16);

/* DC Hadamard transforms over nunits contiguous blocks in place, with
 * SetMode(mode) and SetParameter(QUANT_ID, qp): size 4 = the Intra16x16 luma
 * DC block, FastForwardDC4x4ITImpl1::Transform(void*)
 * (src/CodecUtils/FastForwardDC4x4ITImpl1.cpp:101-196) and
 * FastInverseDC4x4ITImpl1::InverseTransform(void*) (FastInverseDC4x4ITImpl1.cpp:111-202);
 * size 2 = the chroma DC block, FastForwardDC2x2ITImpl1.cpp:100-164 and
 * FastInverseDC2x2ITImpl1.cpp:110-157.  weight: NULL (flat 16) or the
 * SetScale() array of size*size ints (FastInverseDC4x4ITImpl1.cpp:224-240). */
int vppgpu_fwd_dc(vppgpu_ctx* ctx, short* data, long long nunits, int size, int mode, int qp);
int vppgpu_fwd_dc_device(vppgpu_ctx* ctx, short* d_data, long long nunits, int size, int mode, int qp);
int vppgpu_inv_dc(vppgpu_ctx* ctx, short* data, long long nunits, int size, int mode, int qp, const int* weight);
int vppgpu_inv_dc_device(vppgpu_ctx* ctx, short* d_data, long long nunits, int size, int mode, int qp,
                         const int* weight);

/* FastForwardDC4x4ITImpl1::QuantiseValue (src/CodecUtils/FastForwardDC4x4ITImpl1.cpp:268-283),
 * host-side scalar helper (FastForwardDC2x2ITImpl1::QuantiseValue returns 0). */
int vppgpu_dc_quantise_value(short val, int qp);

/* FastForward4x4ITImpl2::QuantiseValue (src/CodecUtils/FastForward4x4ITImpl2.cpp:640-683),
 * host-side scalar helper kept for API completeness. */
int vppgpu_quantise_value(short val, int pos, int qp, int intra);

/* ---- RGB24 -> YUV420 ----------------------------------------------------- */
#define VPPGPU_RGB_FIXED_POINT 0  /* FastFixedPointRGB24toYUV420Converter  */
#define VPPGPU_RGB_REAL        1  /* RealRGB24toYUV420Converter            */
#define VPPGPU_RGB_REAL_IMPL2  2  /* RealRGB24toYUV420ConverterImpl2       */

/* RGBtoYUV420Converter::Convert(pRgb, pY, pU, pV) (include/ImageUtils/RGBtoYUV420Converter.h:57-86;
 * src/ImageUtils/FastFixedPointRGB24toYUV420Converter.cpp:94-169,
 * src/ImageUtils/RealRGB24toYUV420Converter.cpp:83-242): packed B,G,R bytes in,
 * planar shorts out (Y width*height, U and V (width/2)*(height/2)).  flip
 * reads the source bottom-up (Real converters; the fixed-point one ignores
 * it, as in the reference). */
int vppgpu_rgb24_to_yuv420(vppgpu_ctx* ctx, int kind, const unsigned char* bgr, int width,
                           int height, int chr_off, int flip, short* y, short* u, short* v);
int vppgpu_rgb24_to_yuv420_device(vppgpu_ctx* ctx, int kind, const unsigned char* d_bgr, int width,
                                  int height, int chr_off, int flip, short* d_y, short* d_u,
                                  short* d_v);

/* nframes frames stored back to back (BGR, Y, U, V each contiguous per frame)
 * converted in one launch. */
int vppgpu_rgb24_to_yuv420_frames_device(vppgpu_ctx* ctx, int kind, const unsigned char* d_bgr, int nframes,
                                         int width, int height, int chr_off, int flip, short* d_y, short* d_u,
                                         short* d_v);

/* ---- YUV420 -> RGB24 ----------------------------------------------------- */
#define VPPGPU_YUV_REAL       0  /* RealYUV420toRGB24Converter                               */
#define VPPGPU_YUV_REAL_IMPL2 1  /* RealYUV420toRGB24ConverterImpl2, ...Impl2Ver16           */
#define VPPGPU_YUV_CCIR601    2  /* RealYUV420toRGB24CCIR601Converter, ...CCIR601ConverterVer16 */
#define VPPGPU_YUV_FAST_6BIT  3  /* Fast6BitYUV420toRGB24Converter (6-bit samples; rotate only) */
#define VPPGPU_YUV_REAL_6BIT  4  /* Real6BitYUV420toRGB24Converter (6-bit samples; rotate only) */

/* YUV420toRGBConverter::Convert(pY, pU, pV, pRgb) (include/ImageUtils/YUV420toRGBConverter.h:66;
 * src/ImageUtils/RealYUV420toRGB24Converter.cpp:66-352, RealYUV420toRGB24ConverterImpl2.cpp:94-368,
 * RealYUV420toRGB24CCIR601Converter.cpp:59-241), with SetChrominanceOffset(chr_off), SetRotate(rotate)
 * and SetFlip(flip): planar shorts in (Y width*height, U and V (width/2)*(height/2)), packed B,G,R
 * bytes out, width*height*3.  flip writes the rows bottom-up and takes precedence over rotate (the
 * CCIR601 converters ignore it); rotate writes the transpose (pixel (x, y) at byte 3*(x*height + y)).
 * chr_off is used by RealYUV420toRGB24Converter's unrotated paths only, as in the reference.
 * VPPGPU_YUV_FAST_6BIT / VPPGPU_YUV_REAL_6BIT (src/ImageUtils/Fast6BitYUV420toRGB24Converter.cpp:47-245,
 * Real6BitYUV420toRGB24Converter.cpp:53-246) take 6-bit samples (0..63, scaled by 4 inside) and
 * ignore chr_off and flip, as their Convert() does. */
int vppgpu_yuv420_to_rgb24(vppgpu_ctx* ctx, int kind, const short* y, const short* u, const short* v, int width,
                           int height, int chr_off, int rotate, int flip, unsigned char* rgb);
int vppgpu_yuv420_to_rgb24_device(vppgpu_ctx* ctx, int kind, const short* d_y, const short* d_u, const short* d_v,
                                  int width, int height, int chr_off, int rotate, int flip, unsigned char* d_rgb);

/* nframes frames stored back to back (Y, U, V and RGB each contiguous per frame) in one launch. */
int vppgpu_yuv420_to_rgb24_frames_device(vppgpu_ctx* ctx, int kind, const short* d_y, const short* d_u,
                                         const short* d_v, int nframes, int width, int height, int chr_off,
                                         int rotate, int flip, unsigned char* d_rgb);

/* Fast6BitYUV420toRGB24ZoomConverter (include/ImageUtils/Fast6BitYUV420toRGB24ZoomConverter.h:33-60,
 * src/ImageUtils/Fast6BitYUV420toRGB24ZoomConverter.cpp:48-230) with SetOutputDimensions(out_width,
 * out_height): 6-bit planar shorts of width x height in, out_width x out_height packed B,G,R out,
 * each output sample a 16-weight smoothing at its nearest source position.  Output sizes must be
 * even, and every source position (int)(scale * i + 0.5) inside the planes: the reference reads
 * outside its buffers otherwise (e.g. at a 2x zoom), refused with VPPGPU_ERR_UNSUPPORTED. */
int vppgpu_yuv420_to_rgb24_zoom(vppgpu_ctx* ctx, const short* y, const short* u, const short* v, int width,
                                int height, int out_width, int out_height, unsigned char* rgb);
int vppgpu_yuv420_to_rgb24_zoom_device(vppgpu_ctx* ctx, const short* d_y, const short* d_u, const short* d_v,
                                       int width, int height, int out_width, int out_height, unsigned char* d_rgb);

#ifdef __cplusplus
}
#endif
#endif /* VPPGPU_H */
