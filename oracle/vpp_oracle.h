/*
 * vpp_oracle.h -- CPU oracle for the vpp encoder hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (CSIR-RTVC/ImageCodingUtils, "vpp") used as the checker for the
 * CUDA implementation.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline legs of bench.py may load it.  The product path never calls it.
 *
 * Parity of this restatement is pinned against the reference's own C++ code,
 * compiled from its sources by oracle/Makefile into oracle/_ref/ and driven
 * through oracle/ref_harness.cpp; the golden fixtures under tests/golden/ were
 * produced by that compiled reference (tests/golden/make_golden.py).
 *
 * Conventions shared with the reference:
 *   - pixel planes are `short` (int16), luma values 0..255;
 *   - motion vectors are quarter-pel {short x, short y} per 16x16 macroblock,
 *     raster order (VectorStructList SIMPLE2D, include/CodecUtils/VectorStructList.h:56-60);
 *   - motion_range is in quarter-pel units (MotionEstimatorH264ImplFull.cpp:125).
 */
#ifndef VPP_ORACLE_H
#define VPP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Motion estimation                                                         */
/* ------------------------------------------------------------------------ */

/* Number of macroblocks whose vectors the reference stores for a w x h frame:
 * (w/16) * (h/16) (MotionEstimatorH264ImplFull.cpp:293).  A partial bottom MB
 * row (h % 16 != 0) is searched by the reference but its results are dropped
 * (Full.cpp:594); the oracle skips it. */
int vo_num_mbs(int w, int h);

/* MotionEstimatorH264ImplFull::Estimate (src/CodecUtils/MotionEstimatorH264ImplFull.cpp:330-613)
 * with the H264MotionVectorPredictorImpl1 median predictor over a single-slice
 * (or per-MB `slice`) macroblock array.
 *   dist_incl : NULL, or one flag per stored MB (reference `pDistortionIncluded`).
 *   slice     : NULL (one slice), or one slice id per stored MB.
 *   mv_out    : 2*N_MB shorts (x,y pairs).
 *   mb_dist   : NULL or N_MB ints: distortion of the selected vector (Fifo item
 *               chosen by GetBestVector, Full.cpp:579-590).
 *   avg_dist  : the reference's avgDistortion out-param.
 * Returns 0 on success, negative on invalid arguments. */
/* MotionEstimatorH264ImplCross::Estimate (oracle_me_full.c): cross search with
 * the 64-point path distortion and its extrapolating LessThan, the full-search
 * estimator's sub-pel window, GetBestVector lambda 0.9 / norm 64.  mode 0
 * quarter, 1 half, 2 full pel.  tie_out (optional): 1 where the full-pel search
 * met an exact tie. */
int vo_me_cross(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                const unsigned char* dist_incl, const int* slice, short* mv_out, int* mb_dist, long* avg_dist,
                int* tie_out);

/* MotionEstimatorH264ImplUMHS::Estimate (src/CodecUtils/MotionEstimatorH264ImplUMHS.cpp:446-945):
 * unsymmetrical-cross multi-hexagon-grid search started at the median
 * prediction, whose distortion (the five-argument predictor,
 * MacroBlockH264.cpp:818-915) enters an early exit; the previous frame's
 * co-located vector is a starting point.  mode 0 quarter, 1 half, 2 full pel.
 *   prev_mv    : NULL (all zero) or 2*N_MB shorts, the previous frame's
 *                macroblock vectors (MacroBlockH264::_mvX[0], _mvY[0]);
 *   prev_intra : NULL (all inter) or N_MB flags (MacroBlockH264::_intraFlag).
 * mb_dist receives the distortion the predictor stores with each vector.
 * Returns -3 for a previous-frame vector whose block origin leaves
 * [-16, w] x [-16, h]: the reference would read outside its buffers. */
int vo_me_umhs(const short* src, const short* ref, int w, int h, int motion_range, int mode,
               const unsigned char* dist_incl, const int* slice, const short* prev_mv,
               const unsigned char* prev_intra, short* mv_out, int* mb_dist, long* avg_dist);

/* MotionEstimatorH264ImplFHS::Estimate (src/CodecUtils/MotionEstimatorH264ImplFHS.cpp:497-900):
 * hexagon search started at the median prediction on 80-point extrapolated path
 * distortions with integer costs, its own half / quarter stages and the
 * prediction check.  mode 0 quarter, 1 half, 2 full pel.  stale_out (optional):
 * how many macroblocks met the reference's stale sub-pel cache reads, which the
 * oracle replaces by this macroblock's samples (see oracle_me_full.c).
 * mb_dist receives the distortion the predictor stores with each vector. */
int vo_me_fhs(const short* src, const short* ref, int w, int h, int motion_range, int mode,
              const unsigned char* dist_incl, const int* slice, short* mv_out, int* mb_dist, long* avg_dist,
              int* stale_out);

/* MotionEstimatorImpl1::Estimate (src/CodecUtils/MotionEstimatorImpl1.cpp:275-395): full
 * search of [-range, range-1]^2 full pels (range in pels, 1..63) for bw x bh blocks
 * (even bw <= 16, bh <= 16, dividing w and h), HalfRead half-pel refinement,
 * the weighted zero-vector choice; vectors in half pels (chars in the
 * reference's SimpleMotionVectorList), per-block chosen distortion, the average
 * over every block. */
int vo_me_impl1(const short* src, const short* ref, int w, int h, int bw, int bh, int range, short* mv_out,
                int* mb_dist, long* avg_dist);

/* MotionEstimatorImpl2::Estimate (src/CodecUtils/MotionEstimatorImpl2.cpp:505-826): 16x16
 * blocks, range in full pels (4..63); mode 2 (SetMode(0) above 40000 pixels) a full
 * SAD search at level 2 then +-2 at level 1, else a full search at level 1;
 * +-2 at level 0, ties towards the origin; HalfRead half pel; the weighted
 * zero-vector choice; half-pel char vectors, per-block distortion, the average. */
int vo_me_impl2(const short* src, const short* ref, int w, int h, int range, int mode, short* mv_out, int* mb_dist,
                long* avg_dist);

int vo_me_full(const short* src, const short* ref, int w, int h, int motion_range,
               const unsigned char* dist_incl, const int* slice,
               short* mv_out, int* mb_dist, long* avg_dist);

/* Instrumented variant: additionally returns, per MB, the integer-pel winner
 * (ix, iy), the sub-pel stage winner (mvx, mvy, min_d), the zero-vector and
 * predicted-vector distortions and the clamped prediction used by
 * GetBestVector.  Any output pointer may be NULL. */
int vo_me_full_detail(const short* src, const short* ref, int w, int h, int motion_range,
                      const unsigned char* dist_incl, const int* slice,
                      short* mv_out, int* mb_dist, long* avg_dist,
                      int* int_mv, int* sub_mv, int* min_d, int* zero_d,
                      int* pred_mv, int* pred_d);

/* Integer-pel full search only (the hot loop of Full.cpp:350-446) with the
 * sum-of-absolute-differences metric (OverlayMem2Dv2::Tad16x16 /
 * Tad16x16LessThan) or the squared metric, the same running-best skip and
 * predictor tie-break, the predictor being fed the integer winner in
 * quarter-pel units.  metric: 0 = SSD, 1 = SAD. */
int vo_me_full_intpel(const short* src, const short* ref, int w, int h, int motion_range,
                      int metric, short* mv_out, int* mb_dist);

/* MotionEstimatorH264ImplMultiresCross::Estimate
 * (src/CodecUtils/MotionEstimatorH264ImplMultiresCross.cpp:525-1019): 3-level
 * pyramid, cross search at the coarsest level, partial-distortion refinement,
 * sub-pel window, accept-or-zero heuristic; no predictor.  mode 0 (auto),
 * 1 or 2 as SetMode.  The partial bottom macroblock row is searched and,
 * with dist_incl NULL, counted in the average, as in the reference.
 * Returns -3 if the reference itself would read outside its buffers. */
int vo_me_multires_cross(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                         const unsigned char* dist_incl, short* mv_out, int* mb_dist, long* avg_dist);

/* MotionEstimatorH263ImplMultiresCross::Estimate
 * (src/CodecUtils/MotionEstimatorH263ImplMultiresCross.cpp:531-1010): motion
 * range and vectors in half pels, HalfRead half-pel stage. */
int vo_me_h263_multires_cross(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                              const unsigned char* dist_incl, short* mv_out, int* mb_dist, long* avg_dist);
/* MotionEstimatorH263ImplMultiresCrossVer2 with H263MotionVectorPredictorImpl1: half-pel vectors,
 * the chosen distortion per macroblock, avgDistortion (all macroblocks when dist_incl is NULL). */
int vo_me_h263_multires_cross_ver2(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                                   const unsigned char* dist_incl, short* mv_out, int* mb_dist, long* avg_dist);

/* MotionEstimatorH264ImplMultiresCrossVer2::Estimate(long*)
 * (src/CodecUtils/MotionEstimatorH264ImplMultiresCrossVer2.cpp:537-1151): the
 * MultiresCross search with ties towards the rounded median prediction of
 * each level, the pred-vector check and GetBestVector (lambda 0.9).  Full
 * macroblock rows only.  slice: NULL or one slice id per MB.  tie_out: NULL
 * or per MB the integer stages that met an equal distortion (bits: 1 level 2,
 * 2 level 1, 4 level 0). */
int vo_me_multires_cross_v2(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                            const unsigned char* dist_incl, const int* slice, short* mv_out, int* mb_dist,
                            long* avg_dist, int* tie_out);

/* MotionEstimatorH264ImplMultiresCrossVer2::Estimate(long*, void* lambda)
 * (src/CodecUtils/MotionEstimatorH264ImplMultiresCrossVer2.cpp:1162-1742):
 * GetBestVector (MultiresCrossVer2.h:168-197) over the last five improvements
 * of every search level, then the pred-vector check and the final choice with
 * the given lambda.  Other arguments as above. */
int vo_me_multires_cross_v2_lambda(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                                   double lambda, const unsigned char* dist_incl, const int* slice, short* mv_out,
                                   int* mb_dist, long* avg_dist);

/* MotionEstimatorH264ImplMultires::Estimate
 * (src/CodecUtils/MotionEstimatorH264ImplMultires.cpp:557-1024): full searches
 * at levels 2 and 1, +-2 at level 0, sub-pel in the MultiresCross-style
 * window, ties towards the prediction rounded to each level, the pred-vector
 * check and GetBestVector (lambda 1.1).  Arguments as for Ver2. */
int vo_me_multires(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                   const unsigned char* dist_incl, const int* slice, short* mv_out, int* mb_dist, long* avg_dist,
                   int* tie_out);

/* MotionCompensatorH264ImplStd::Compensate(pMotionList)
 * (src/CodecUtils/MotionCompensatorH264ImplStd.cpp:323-473): yuv is the
 * contiguous 4:2:0 reference (Y w*h, U, V (w/2)*(h/2)), compensated in place
 * by the quarter-pel vectors (2 shorts per macroblock, full macroblock rows). */
int vo_mc_compensate(short* yuv, int w, int h, int range, const short* mv);
/* Add16x16WithClip255 / Add8x8WithClip255 and Sub16x16 / Sub8x8 over n samples. */
void vo_add_clip255(short* a, const short* b, long long n);
void vo_sub(short* a, const short* b, long long n);

/* OverlayMem2Dv2::QuarterRead (src/ImageUtils/OverlayMem2Dv2.cpp:704-1052) of
 * a 16x16 block whose full-pel origin is (x, y) in a frame extended by edge
 * replication, at quarter offsets (qx, qy) in -3..3. */
void vo_quarter_read16(const short* plane, int w, int h, int x, int y, int qx, int qy,
                       short* dst256);

/* OverlayMem2Dv2::Half 2:1 decimation (OverlayMem2Dv2.cpp:3018-3033). */
void vo_half(const short* src, int w, int h, short* dst);

/* ------------------------------------------------------------------------ */
/* 4x4 integer transform + H.264 quantisation                                */
/* ------------------------------------------------------------------------ */
/* Modes (IForwardTransform.h:119-125): 0 = transform+quant, 1 = transform only,
 * 2 = quant only.  `layout`: 0 = contiguous 16-short blocks (FastForward4x4ITImpl1,
 * FastInverse4x4ITImpl1), 1 = 16x16 raster macroblocks of 256 shorts
 * (FastForward4x4On16x16ITImpl1, FastInverse4x4On16x16ITImpl1). */
void vo_fwd4x4(short* data, int nunits, int layout, int mode, int qp, int intra);
void vo_inv4x4(short* data, int nunits, int layout, int mode, int qp, const int* weight_scale16);
/* FastForward4x4ITImpl2::QuantiseValue (FastForward4x4ITImpl2.cpp:640-683). */
int vo_quantise_value(short val, int pos, int qp, int intra);

/* DC Hadamard transforms (oracle_dc.c): size 4 = FastForward/InverseDC4x4ITImpl1,
 * size 2 = FastForward/InverseDC2x2ITImpl1; nunits contiguous size*size blocks. */
void vo_fwd_dc(short* data, int nunits, int size, int mode, int qp);
void vo_inv_dc(short* data, int nunits, int size, int mode, int qp, const int* weight);
int vo_dc_quantise_value(short val, int qp);

/* YUV420 -> RGB24 (oracle_yuv2rgb.c): kind 0 RealYUV420toRGB24Converter,
 * 1 RealYUV420toRGB24ConverterImpl2 (and Ver16), 2 RealYUV420toRGB24CCIR601Converter
 * (and Ver16); rgb holds width*height*3 bytes. */
void vo_yuv420_to_rgb24(int kind, const short* py, const short* pu, const short* pv, int w, int h, int chr_off,
                        int rotate, int flip, unsigned char* rgb);
/* kind 3 Fast6BitYUV420toRGB24Converter, 4 Real6BitYUV420toRGB24Converter */
void vo_yuv420_to_rgb24_6bit(int kind, const short* py, const short* pu, const short* pv, int w, int h, int rotate,
                             unsigned char* rgb);
/* Fast6BitYUV420toRGB24ZoomConverter to an ow x oh output; -1 for sizes it cannot hold */
int vo_yuv420_to_rgb24_zoom(const short* py, const short* pu, const short* pv, int w, int h, int ow, int oh,
                            unsigned char* rgb);

/* ------------------------------------------------------------------------ */
/* RGB24 -> YUV420                                                           */
/* ------------------------------------------------------------------------ */
/* kind: 0 = FastFixedPointRGB24toYUV420Converter (integer),
 *       1 = RealRGB24toYUV420Converter (IEEE double),
 *       2 = RealRGB24toYUV420ConverterImpl2 (IEEE double, other rounding).
 * flip: bottom-up source rows (Real converters only; FastFixedPoint ignores it). */
int vo_rgb24_to_yuv420(int kind, const unsigned char* bgr, int w, int h, int chr_off, int flip,
                       short* y, short* u, short* v);

/* ------------------------------------------------------------------------ */
/* Multi-threaded CPU baseline drivers (one estimator state per thread over   */
/* independent frame pairs; the reference has no internal threading).        */
/* ------------------------------------------------------------------------ */
int vo_bench_me_full(const short* const* srcs, const short* const* refs, int nframes,
                     int w, int h, int motion_range, int nthreads, short* mv_out);

#ifdef __cplusplus
}
#endif
#endif
