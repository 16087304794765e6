/*
 * oracle_internal.h -- TEST INFRASTRUCTURE ONLY: helpers shared by the CPU
 * oracle's translation units.
 */
#ifndef VPP_ORACLE_INTERNAL_H
#define VPP_ORACLE_INTERNAL_H
#include <stddef.h>
#include "vpp_oracle.h"

short* vo_ext_alloc(const short* plane, int w, int h, int border);
void vo_ext_fill(short* e, const short* plane, int w, int h, int border);
int vo_clamp_origin(int v, int src_len, int blk_len);
int vo_tsd16(const short* a, int as, const short* b, int bs);
int vo_tsd16_lt(const short* a, int as, const short* b, int bs, int min);
int vo_tad16(const short* a, int as, const short* b, int bs);
int vo_tad16_lt(const short* a, int as, const short* b, int bs, int min);
int vo_tsd_n(const short* a, int as, const short* b, int bs, int n);
int vo_tsd_partial_lt(const short* a, int as, const short* b, int bs, int n, int min);
int vo_tsd4_lt(const short* a, int as, const short* b, int bs, int min);
extern const int vo_phase_col[17];
extern const int vo_phase_row[17];
int vo_hp_b(const short* e, int es, int x, int y);
int vo_hp_h(const short* e, int es, int x, int y);
int vo_hp_j(const short* e, int es, int x, int y);
int vo_qpel_sample(const short* e, int es, int x, int y, int fx, int fy);
void vo_qread16_ext(const short* e, int es, int ox, int oy, int qx, int qy, short* dst);

/* Median 16x16 motion-vector prediction state (H264MotionVectorPredictorImpl1,
 * include/CodecUtils/H264MotionVectorPredictorImpl1.h:77-121, over the
 * neighbourhood MacroBlockH264::Initialise wires, MacroBlockH264.cpp:319-). */
typedef struct {
    int cols, rows;
    const int* slice; /* NULL = one slice */
    int* mvx;
    int* mvy;
} vo_pred_state;

int vo_pred_init(vo_pred_state* st, int cols, int rows, const int* slice);
void vo_pred_free(vo_pred_state* st);
void vo_pred_get(const vo_pred_state* st, int k, int* px, int* py);
void vo_pred_set(vo_pred_state* st, int k, int mvx, int mvy);
int vo_median3(int x, int y, int z);

/* Fifo-fed Lagrangian pick of MotionEstimatorH264ImplFull::GetBestVector
 * (include/CodecUtils/MotionEstimatorH264ImplFull.h:140-168) over the five
 * slots (best, pred, zero, zero, zero). Returns the chosen slot. */
int vo_best_vector5(const int* xs, const int* ys, const int* ds, double lambda, double norm,
                    int xref, int yref);

#endif
