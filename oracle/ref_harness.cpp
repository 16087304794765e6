/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * A thin extern "C" driver around the reference's own C++ classes, compiled
 * together with the reference sources (read where they lie) by
 * oracle/Makefile into oracle/_ref/libvppref.so.  It exists to pin the C
 * restatement in oracle/*.c and to generate the golden fixtures; it contains
 * no algorithm of its own, only object set-up in the way a vpp codec does it.
 */
#include <malloc.h>
#include <math.h>
#include <string.h>
#include <stdlib.h>

#include "MacroBlockH264.h"
#include "H264MotionVectorPredictorImpl1.h"
#include "MotionEstimatorH264ImplFull.h"
#include "MotionEstimatorH264ImplMultires.h"
#include "MotionEstimatorH264ImplMultiresCross.h"
#include "MotionEstimatorH264ImplMultiresCrossVer2.h"
#include "MotionEstimatorH264ImplCross.h"
#include "MotionEstimatorH264ImplUMHS.h"
#include "MotionEstimatorH264ImplFHS.h"
#include "MotionEstimatorImpl1.h"
#include "MotionEstimatorImpl2.h"
#include "SimpleMotionVectorList.h"
#include "MotionEstimatorH263ImplMultiresCross.h"
#include "MotionEstimatorH263ImplMultiresCrossVer2.h"
#include "H263MotionVectorPredictorImpl1.h"
#include "VectorStructList.h"
#include "MotionCompensatorH264ImplStd.h"
#include "FastForward4x4ITImpl1.h"
#include "FastForward4x4ITImpl2.h"
#include "FastInverse4x4ITImpl1.h"
#include "FastForward4x4On16x16ITImpl1.h"
#include "FastInverse4x4On16x16ITImpl1.h"
#include "RealYUV420toRGB24Converter.h"
#include "RealYUV420toRGB24ConverterImpl2.h"
#include "RealYUV420toRGB24ConverterImpl2Ver16.h"
#include "RealYUV420toRGB24CCIR601Converter.h"
#include "RealYUV420toRGB24CCIR601ConverterVer16.h"
#include "Fast6BitYUV420toRGB24Converter.h"
#include "Real6BitYUV420toRGB24Converter.h"
#include "Fast6BitYUV420toRGB24ZoomConverter.h"
#include "FastForwardDC4x4ITImpl1.h"
#include "FastInverseDC4x4ITImpl1.h"
#include "FastForwardDC2x2ITImpl1.h"
#include "FastInverseDC2x2ITImpl1.h"
#include "FastFixedPointRGB24toYUV420Converter.h"
#include "RealRGB24toYUV420Converter.h"
#include "RealRGB24toYUV420ConverterImpl2.h"

namespace {

/* A macroblock array laid out as a codec lays it out: rows x cols with the
 * neighbourhood wired by MacroBlockH264::Initialise.  Rows are rounded up so
 * the reference's partial bottom row (h % 16 != 0) reads valid memory.
 *
 * Every macroblock of a partial bottom row asks the predictor for index N_MB
 * (vecPos stops at maxLength, MotionEstimatorH264ImplFull.cpp:594-601) and its
 * results are dropped.  When that prediction points below the picture,
 * Full.cpp:536-537 replaces it with +16 rows, which for this row places the
 * pred-vector QuarterRead (Full.cpp:551) up to 3 rows past the extended
 * reference (OverlayMem2Dv2.cpp:989-1010; AddressSanitizer reports a heap
 * overflow there).  Putting the partial row in a slice of its own makes that
 * prediction (0,0), keeping the reference in bounds without changing any
 * stored result. */
struct MbGrid {
    int rows, cols;
    MacroBlockH264* flat;
    MacroBlockH264** rowp;
    MbGrid(int w, int h) {
        cols = w / 16;
        rows = (h + 15) / 16;
        int full_rows = h / 16;
        flat = new MacroBlockH264[rows * cols];
        rowp = new MacroBlockH264*[rows];
        for (int r = 0; r < rows; r++) rowp[r] = &flat[r * cols];
        MacroBlockH264::Initialise(rows, cols, 0, full_rows * cols - 1, 0, rowp);
        if (rows > full_rows)
            MacroBlockH264::Initialise(rows, cols, full_rows * cols, rows * cols - 1, 1, rowp);
    }
    ~MbGrid() { delete[] rowp; delete[] flat; }
};

/* Flags with one extra trailing `false`: the reference reads the flag at index
 * N_MB for the macroblocks of a partial bottom row (they are dropped). */
bool* make_flags(const unsigned char* incl, int nmb) {
    if (!incl) return NULL;
    bool* f = new bool[nmb + 1];
    for (int i = 0; i < nmb; i++) f[i] = incl[i] != 0;
    f[nmb] = false;
    return f;
}

void copy_vectors(VectorStructList* l, int nmb, short* out) {
    for (int i = 0; i < nmb; i++) {
        out[2 * i] = (short)l->GetSimpleElement(i, 0);
        out[2 * i + 1] = (short)l->GetSimpleElement(i, 1);
    }
}

/* The integer-pel stage of MotionEstimatorH264ImplFull::Estimate
 * (MotionEstimatorH264ImplFull.cpp:341-446) with its MEH264IF_ABS_DIFF
 * distortion.  The switch is #undef'd inside the .cpp, so the loop is stated
 * here, on the reference's own members: the extended reference overlay filled
 * as Estimate fills it, OverlayMem2Dv2::Tad16x16 / Tad16x16LessThan,
 * GetMotionRange and the predictor.  The chosen full-pel vector (in quarter
 * pels) goes to the predictor as Estimate's final vector does (:593-600). */
class FullSadStage : public MotionEstimatorH264ImplFull {
public:
    using MotionEstimatorH264ImplFull::MotionEstimatorH264ImplFull;
    void run(int nmb, const bool* incl, short* mv_out, int* dist_out, long* avg_out) {
        _pExtRefOver->SetOrigin(0, 0);
        _pExtRefOver->SetOverlayDim(_imgWidth, _imgHeight);
        _pExtRefOver->Write(*_pRefOver);
        _pExtRefOver->FillBoundaryProxy();
        _pExtRefOver->SetOverlayDim(_macroBlkWidth, _macroBlkHeight);
        int vecPos = 0, included = 0;
        long total = 0;
        for (int m = 0; m < _imgHeight; m += _macroBlkHeight)
            for (int n = 0; n < _imgWidth; n += _macroBlkWidth) {
                int predX, predY;
                _pMVPred->Get16x16Prediction(NULL, vecPos, &predX, &predY);
                const int prx = predX < 0 ? (predX - 2) / 4 : (predX + 2) / 4;
                const int pry = predY < 0 ? (predY - 2) / 4 : (predY + 2) / 4;
                _pInOver->SetOrigin(n, m);
                _pExtRefOver->SetOrigin(n, m);
                int minDiff = _pInOver->Tad16x16(*_pExtRefOver);
                int mx = 0, my = 0, xl, xr, yu, yd;
                GetMotionRange(n, m, 0, 0, &xl, &xr, &yu, &yd, _motionRange / 4);
                for (int i = yu; i <= yd; i++)
                    for (int j = xl; j <= xr; j++) {
                        if (!(i || j)) continue;
                        if (i + my < yu || i + my > yd || j + mx < xl || j + mx > xr) continue;
                        _pExtRefOver->SetOrigin(n + j, m + i);
                        const int d = _pInOver->Tad16x16LessThan(*_pExtRefOver, minDiff);
                        if (d > minDiff) continue;
                        if (d == minDiff) {
                            const int cx = mx - prx, cy = my - pry, nx = j - prx, ny = i - pry;
                            if ((cy * cy + cx * cx) - (ny * ny + nx * nx) < 0) continue;
                        }
                        minDiff = d;
                        mx = j;
                        my = i;
                    }
                if (vecPos < nmb) {
                    mv_out[2 * vecPos] = (short)(4 * mx);
                    mv_out[2 * vecPos + 1] = (short)(4 * my);
                    if (dist_out) dist_out[vecPos] = minDiff;
                    if (incl && incl[vecPos]) {
                        included++;
                        total += minDiff;
                    }
                    _pMVPred->Set16x16MotionVector(vecPos, 4 * mx, 4 * my);
                    vecPos++;
                }
            }
        if (avg_out) *avg_out = included ? total / included : 0;
    }
};

}  // namespace

extern "C" {

/* FullSadStage over one frame pair: vectors (quarter pels), per-MB SAD and the
 * included-distortion average (0 without flags, as Full.cpp:582-609). */
int ref_me_full_sad(const short* src, const short* ref, int w, int h, int motion_range, const unsigned char* incl,
                    short* mv_out, int* dist_out, long* avg_out)
{
    int nmb = (w / 16) * (h / 16);
    MbGrid grid(w, h);
    H264MotionVectorPredictorImpl1 pred(grid.flat);
    bool* flags = make_flags(incl, nmb);
    FullSadStage* me = new FullSadStage(src, ref, w, h, motion_range, &pred, flags);
    if (!me->Create()) { delete me; delete[] flags; return -2; }
    me->run(nmb, flags, mv_out, dist_out, avg_out);
    delete me;
    delete[] flags;
    return 0;
}

/* kind: 0 Full, 1 Multires, 2 MultiresCross, 3 MultiresCrossVer2, 4 Cross, 5 H263MultiresCross,
 * 6 H263MultiresCrossVer2 (with an H263MotionVectorPredictorImpl1).
 * lambda: NULL, or a pointer passed to Estimate(long*, void*) (Ver2 only).
 * Returns 0 on success. */
int ref_me_estimate(int kind, const short* src, const short* ref, int w, int h, int motion_range,
                    int mode, const unsigned char* incl, const double* lambda, int nframes_same_object,
                    short* mv_out, long* avg_out)
{
    int nmb = (w / 16) * (h / 16);
    MbGrid grid(w, h);
    H264MotionVectorPredictorImpl1 pred(grid.flat);
    H263MotionVectorPredictorImpl1 pred263(w, h);
    bool* flags = make_flags(incl, nmb);
    IMotionEstimator* me = NULL;
    /* The multi-resolution estimators read window samples they never write
     * (see oracle_me_multires.c).  Allocations made while constructing and
     * creating the estimator are zero-filled (glibc M_PERTURB with 0xff fills
     * new allocations with 0x00), which pins those samples to 0. */
    mallopt(M_PERTURB, 0xff);
    switch (kind) {
    case 0: me = new MotionEstimatorH264ImplFull(src, ref, w, h, motion_range, &pred, flags); break;
    case 1: me = new MotionEstimatorH264ImplMultires(src, ref, w, h, motion_range, &pred, flags); break;
    case 2: me = new MotionEstimatorH264ImplMultiresCross(src, ref, w, h, motion_range, flags); break;
    case 3: me = new MotionEstimatorH264ImplMultiresCrossVer2(src, ref, w, h, motion_range, &pred, flags); break;
    case 4: me = new MotionEstimatorH264ImplCross(src, ref, w, h, motion_range, &pred, flags); break;
    case 5: me = new MotionEstimatorH263ImplMultiresCross(src, ref, w, h, motion_range, flags); break;
    case 6: me = new MotionEstimatorH263ImplMultiresCrossVer2(src, ref, w, h, motion_range, &pred263, flags); break;
    default: mallopt(M_PERTURB, 0); delete[] flags; return -1;
    }
    int created = me->Create();
    mallopt(M_PERTURB, 0);
    if (!created) { delete me; delete[] flags; return -2; }
    me->SetMode(mode);
    long avg = 0;
    void* res = NULL;
    for (int f = 0; f < (nframes_same_object > 0 ? nframes_same_object : 1); f++)
        res = lambda ? me->Estimate(&avg, (void*)lambda) : me->Estimate(&avg);
    copy_vectors((VectorStructList*)res, nmb, mv_out);
    if (avg_out) *avg_out = avg;
    delete me;
    delete[] flags;
    return 0;
}

/* MotionEstimatorH264ImplUMHS through its eight-argument constructor (the
 * others leave the previous-frame macroblocks unset, which Estimate reads).
 * prev_mv / prev_intra (nullable: zero vectors, inter) fill the previous
 * frame's macroblock array; entries past N_MB, read by a partial bottom row
 * whose results are dropped, are intra.  dist_out: the distortion the
 * estimator hands the predictor with each vector (MacroBlockH264::_distortion[0]). */
int ref_me_umhs(const short* src, const short* ref, int w, int h, int motion_range, int mode,
                const unsigned char* incl, const short* prev_mv, const unsigned char* prev_intra, short* mv_out,
                int* dist_out, long* avg_out)
{
    int nmb = (w / 16) * (h / 16);
    MbGrid grid(w, h);
    H264MotionVectorPredictorImpl1 pred(grid.flat);
    MacroBlockH264* prev = new MacroBlockH264[nmb + w / 16];
    for (int i = 0; i < nmb + w / 16; i++) {
        prev[i]._intraFlag = i < nmb ? (prev_intra ? (prev_intra[i] != 0) : 0) : 1;
        prev[i]._mvX[MacroBlockH264::_16x16] = (i < nmb && prev_mv) ? prev_mv[2 * i] : 0;
        prev[i]._mvY[MacroBlockH264::_16x16] = (i < nmb && prev_mv) ? prev_mv[2 * i + 1] : 0;
    }
    bool* flags = make_flags(incl, nmb);
    MotionEstimatorH264ImplUMHS* me = new MotionEstimatorH264ImplUMHS(src, ref, w, h, motion_range, &pred, flags, prev);
    if (!me->Create()) { delete me; delete[] flags; delete[] prev; return -2; }
    me->SetMode(mode);
    long avg = 0;
    void* res = me->Estimate(&avg);
    copy_vectors((VectorStructList*)res, nmb, mv_out);
    if (dist_out)
        for (int i = 0; i < nmb; i++) dist_out[i] = grid.flat[i]._distortion[0];
    if (avg_out) *avg_out = avg;
    delete me;
    delete[] flags;
    delete[] prev;
    return 0;
}

/* MotionEstimatorH264ImplFHS through its seven-argument constructor: vectors,
 * the distortion handed to the predictor with each, the average.  Its
 * quarter-pel cache is allocated zero-filled (glibc M_PERTURB), so reads it
 * makes before any macroblock filled a sample are reproducible. */
int ref_me_fhs(const short* src, const short* ref, int w, int h, int motion_range, int mode,
               const unsigned char* incl, short* mv_out, int* dist_out, long* avg_out)
{
    int nmb = (w / 16) * (h / 16);
    MbGrid grid(w, h);
    H264MotionVectorPredictorImpl1 pred(grid.flat);
    bool* flags = make_flags(incl, nmb);
    mallopt(M_PERTURB, 0xff);
    MotionEstimatorH264ImplFHS* me = new MotionEstimatorH264ImplFHS(src, ref, w, h, motion_range, &pred, flags);
    int created = me->Create();
    mallopt(M_PERTURB, 0);
    if (!created) { delete me; delete[] flags; return -2; }
    me->SetMode(mode);
    long avg = 0;
    void* res = me->Estimate(&avg);
    copy_vectors((VectorStructList*)res, nmb, mv_out);
    if (dist_out)
        for (int i = 0; i < nmb; i++) dist_out[i] = grid.flat[i]._distortion[0];
    if (avg_out) *avg_out = avg;
    delete me;
    delete[] flags;
    return 0;
}

/* MotionEstimatorImpl1 (pSrc, pRef, w, h, macroBlkWidth, macroBlkHeight,
 * motionRange): its SimpleMotionVectorList of (char x, char y) half-pel
 * vectors, read as signed chars, and avgDistortion. */
int ref_me_impl1(const short* src, const short* ref, int w, int h, int bw, int bh, int range, short* mv_out,
                 long* avg_out)
{
    MotionEstimatorImpl1 me(src, ref, w, h, bw, bh, range);
    if (!me.Create()) return -2;
    long avg = 0;
    SimpleMotionVectorList* l = (SimpleMotionVectorList*)me.Estimate(&avg);
    const signed char* p = (const signed char*)l->GetDataPtr();
    const int step = l->GetPatternSize(), n = l->GetLength();
    for (int i = 0; i < n; i++) {
        mv_out[2 * i] = p[(size_t)i * step];
        mv_out[2 * i + 1] = p[(size_t)i * step + 1];
    }
    if (avg_out) *avg_out = avg;
    return 0;
}

/* MotionEstimatorImpl2 (pSrc, pRef, w, h, 16, 16, motionRange) after SetMode(mode). */
int ref_me_impl2(const short* src, const short* ref, int w, int h, int range, int mode, short* mv_out, long* avg_out)
{
    MotionEstimatorImpl2 me(src, ref, w, h, 16, 16, range);
    if (!me.Create()) return -2;
    me.SetMode(mode);
    long avg = 0;
    SimpleMotionVectorList* l = (SimpleMotionVectorList*)me.Estimate(&avg);
    const signed char* p = (const signed char*)l->GetDataPtr();
    const int step = l->GetPatternSize(), n = l->GetLength();
    for (int i = 0; i < n; i++) {
        mv_out[2 * i] = p[(size_t)i * step];
        mv_out[2 * i + 1] = p[(size_t)i * step + 1];
    }
    if (avg_out) *avg_out = avg;
    return 0;
}

/* MotionCompensatorH264ImplStd(range) + Create(yuv, w, h, 16, 16) +
 * Compensate(list of the N_MB vectors): yuv (contiguous 4:2:0) is compensated
 * in place.  Heights are multiples of 16 (the reference reads vectors past its
 * list for a partial bottom row). */
int ref_mc_compensate(int w, int h, int range, short* yuv, const short* mv)
{
    if (h % 16) return -1;
    MotionCompensatorH264ImplStd mc(range);
    if (!mc.Create(yuv, w, h, 16, 16)) return -2;
    const int nmb = (w / 16) * (h / 16);
    VectorStructList list(VectorStructList::SIMPLE2D);
    list.SetLength(nmb);
    for (int i = 0; i < nmb; i++) {
        list.SetSimpleElement(i, 0, mv[2 * i]);
        list.SetSimpleElement(i, 1, mv[2 * i + 1]);
    }
    mc.Compensate(&list);
    return 0;
}

/* impl: 0 FastForward4x4ITImpl1, 1 FastForward4x4ITImpl2 (16-short blocks),
 *       2 FastForward4x4On16x16ITImpl1 (256-short macroblocks). */
int ref_fwd_transform(int impl, short* data, int nunits, int mode, int qp, int intra)
{
    IForwardTransform* t = NULL;
    int unit = 16;
    if (impl == 0) t = new FastForward4x4ITImpl1();
    else if (impl == 1) t = new FastForward4x4ITImpl2();
    else if (impl == 2) { t = new FastForward4x4On16x16ITImpl1(); unit = 256; }
    else return -1;
    t->SetMode(mode);
    t->SetParameter(IForwardTransform::INTRA_FLAG_ID, intra);
    t->SetParameter(IForwardTransform::QUANT_ID, qp);
    for (int u = 0; u < nunits; u++) t->Transform(data + (size_t)u * unit);
    delete t;
    return 0;
}

/* impl: 0 FastInverse4x4ITImpl1 (16-short blocks), 1 FastInverse4x4On16x16ITImpl1. */
int ref_inv_transform(int impl, short* data, int nunits, int mode, int qp, const int* weight16)
{
    IInverseTransform* t = NULL;
    int unit = 16;
    if (impl == 0) t = new FastInverse4x4ITImpl1();
    else if (impl == 1) { t = new FastInverse4x4On16x16ITImpl1(); unit = 256; }
    else return -1;
    if (weight16) t->SetScale((void*)weight16);
    t->SetMode(mode);
    t->SetParameter(IInverseTransform::QUANT_ID, qp);
    for (int u = 0; u < nunits; u++) t->InverseTransform(data + (size_t)u * unit);
    delete t;
    return 0;
}

/* size 4: FastForwardDC4x4ITImpl1, size 2: FastForwardDC2x2ITImpl1. */
int ref_fwd_dc(short* data, int nunits, int size, int mode, int qp)
{
    IForwardTransform* t = NULL;
    if (size == 4) t = new FastForwardDC4x4ITImpl1();
    else if (size == 2) t = new FastForwardDC2x2ITImpl1();
    else return -1;
    t->SetMode(mode);
    t->SetParameter(IForwardTransform::QUANT_ID, qp);
    for (int u = 0; u < nunits; u++) t->Transform(data + (size_t)u * size * size);
    delete t;
    return 0;
}

/* size 4: FastInverseDC4x4ITImpl1, size 2: FastInverseDC2x2ITImpl1; weight: NULL or size*size ints. */
int ref_inv_dc(short* data, int nunits, int size, int mode, int qp, const int* weight)
{
    IInverseTransform* t = NULL;
    if (size == 4) t = new FastInverseDC4x4ITImpl1();
    else if (size == 2) t = new FastInverseDC2x2ITImpl1();
    else return -1;
    if (weight) t->SetScale((void*)weight);
    t->SetMode(mode);
    t->SetParameter(IInverseTransform::QUANT_ID, qp);
    for (int u = 0; u < nunits; u++) t->InverseTransform(data + (size_t)u * size * size);
    delete t;
    return 0;
}

/* kind: 0 RealYUV420toRGB24Converter, 1 ...Impl2, 2 ...CCIR601, 3 ...Impl2Ver16, 4 ...CCIR601Ver16. */
int ref_yuv_to_rgb(int kind, short* y, short* u, short* v, int w, int h, int chr_off, int rotate, int flip,
                   unsigned char* rgb)
{
    YUV420toRGBConverter* c = NULL;
    if (kind == 0) c = new RealYUV420toRGB24Converter(w, h);
    else if (kind == 1) c = new RealYUV420toRGB24ConverterImpl2(w, h);
    else if (kind == 2) c = new RealYUV420toRGB24CCIR601Converter(w, h);
    else if (kind == 3) c = new RealYUV420toRGB24ConverterImpl2Ver16(w, h);
    else if (kind == 4) c = new RealYUV420toRGB24CCIR601ConverterVer16(w, h);
    else if (kind == 5) c = new Fast6BitYUV420toRGB24Converter(w, h);
    else if (kind == 6) c = new Real6BitYUV420toRGB24Converter(w, h);
    else return -1;
    /* the two-argument constructors leave the chrominance offset unset */
    c->SetChrominanceOffset(chr_off);
    c->SetRotate(rotate);
    c->SetFlip(flip != 0);
    c->Convert(y, u, v, rgb);
    delete c;
    return 0;
}

/* Fast6BitYUV420toRGB24ZoomConverter to an ow x oh output (no rotation). */
int ref_yuv_to_rgb_zoom(short* y, short* u, short* v, int w, int h, int ow, int oh, unsigned char* rgb)
{
    Fast6BitYUV420toRGB24ZoomConverter c(w, h);
    c.SetOutputDimensions(ow, oh);
    c.Convert(y, u, v, rgb);
    return 0;
}

int ref_dc_quantise_value(short val, int qp)
{
    FastForwardDC4x4ITImpl1 t;
    return t.QuantiseValue(val, 0, qp);
}

int ref_quantise_value(short val, int pos, int qp, int intra)
{
    FastForward4x4ITImpl2 t;
    t.SetParameter(IForwardTransform::INTRA_FLAG_ID, intra);
    return t.QuantiseValue(val, pos, qp);
}

/* kind: 0 FastFixedPoint, 1 Real, 2 RealImpl2. */
int ref_rgb_to_yuv(int kind, const unsigned char* bgr, int w, int h, int chr_off, int flip,
                   short* y, short* u, short* v)
{
    RGBtoYUV420Converter* c = NULL;
    if (kind == 0) c = new FastFixedPointRGB24toYUV420Converter(w, h, chr_off);
    else if (kind == 1) c = new RealRGB24toYUV420Converter(w, h, chr_off);
    else if (kind == 2) c = new RealRGB24toYUV420ConverterImpl2(w, h, chr_off);
    else return -1;
    c->SetFlip(flip != 0);
    c->Convert((void*)bgr, y, u, v);
    delete c;
    return 0;
}

}  // extern "C"
