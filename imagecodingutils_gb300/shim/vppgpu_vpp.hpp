// vppgpu_vpp.hpp -- drop-in C++ classes for vpp codecs, header only.
//
// Each class implements one of vpp's plugin interfaces by calling the C ABI
// of include/vppgpu.h, so a codec swaps
//     new MotionEstimatorH264ImplFull(pSrc, pRef, w, h, range, pMVPred, pDistIncl)
// for
//     new GpuMotionEstimatorH264ImplFull(pSrc, pRef, w, h, range, pMVPred, pDistIncl)
// and keeps everything else.
//
// Build inside the vpp tree with -DVPPGPU_WITH_VPP: the classes then derive
// from vpp's own IMotionEstimator, IForwardTransform, IInverseTransform,
// RGBtoYUV420Converter and YUV420toRGBConverter and return vpp's
// VectorStructList.  Without that
// macro, minimal local declarations with the same method signatures are
// used (for this repository's tests and for codecs that only need the
// methods).
#pragma once

#include <stddef.h>
#include <string.h>

#include "../../include/vppgpu.h"

#ifdef VPPGPU_WITH_VPP
#include "IForwardTransform.h"
#include "IInverseTransform.h"
#include "IMotionEstimator.h"
#include "IMotionVectorPredictor.h"
#include "MacroBlockH264.h"
#include "RGBtoYUV420Converter.h"
#include "SimpleMotionVectorList.h"
#include "VectorStructList.h"
#include "YUV420toRGBConverter.h"
#else
// ---- local declarations mirroring the vpp interfaces (same signatures) ----
class IMotionEstimator {
public:
    virtual ~IMotionEstimator() {}
    virtual int Create(void) = 0;
    virtual void Reset(void) = 0;
    virtual int Ready(void) = 0;
    virtual void SetMode(int mode) = 0;
    virtual int GetMode(void) = 0;
    virtual void* Estimate(const void* pSrc, const void* pRef, long* avgDistortion) = 0;
    virtual void* Estimate(long* avgDistortion) = 0;
    virtual void* Estimate(long* avgDistortion, void* param) { (void)param; return Estimate(avgDistortion); }
};

class IMotionVectorPredictor {
public:
    virtual ~IMotionVectorPredictor() {}
    virtual int Create(void) = 0;
    virtual int Get16x16Prediction(void* pList, int blk, int* predX, int* predY) = 0;
    virtual int Get16x16Prediction(void* pList, int blk, int* predX, int* predY, int* distortion)
    {
        (void)pList; (void)blk; (void)predX; (void)predY; (void)distortion;
        return 0;
    }
    virtual void Set16x16MotionVector(int blk, int mvX, int mvY) = 0;
    virtual void Set16x16MotionVector(int blk, int mvX, int mvY, int distortion)
    {
        (void)blk; (void)mvX; (void)mvY; (void)distortion;
    }
};

// vpp's SimpleMotionVectorList (VectorList(SIMPLE, 2, sizeof(char))): one
// {char x, char y} pattern per block.
class SimpleMotionVectorList {
public:
    SimpleMotionVectorList() : _length(0), _pData(NULL) {}
    virtual ~SimpleMotionVectorList() { delete[] _pData; }
    virtual int SetLength(int length) {
        delete[] _pData;
        _pData = new char[2 * (size_t)(length > 0 ? length : 1)];
        _length = length;
        return 1;
    }
    int GetPatternSize(void) { return 2; }
    int GetLength(void) { return _length; }
    void* GetDataPtr(void) { return _pData; }

private:
    int _length;
    char* _pData;
};

// The SIMPLE2D layout of vpp's VectorStructList: one {short x, short y} per block.
class VectorStructList {
public:
    static const int SIMPLE2D = 0;
    explicit VectorStructList(int type) : _type(type), _length(0), _pData(NULL) {}
    virtual ~VectorStructList() { delete[] _pData; }
    virtual int SetLength(int length) {
        delete[] _pData;
        _pData = new short[2 * (size_t)(length > 0 ? length : 1)];
        _length = length;
        return 1;
    }
    int GetType(void) { return _type; }
    int GetLength(void) { return _length; }
    void* GetListPtr(void) { return _pData; }
    virtual void SetSimpleElement(int pos, int element, int val) { _pData[2 * pos + (element ? 1 : 0)] = (short)val; }
    virtual int GetSimpleElement(int pos, int element) { return _pData[2 * pos + (element ? 1 : 0)]; }

protected:
    int _type, _length;
    short* _pData;
};

class IForwardTransform {
public:
    virtual ~IForwardTransform() {}
    virtual void Transform(void* ptr) = 0;
    virtual void Transform(void* pIn, void* pCoeff) = 0;
    virtual void SetScale(void* pScale) = 0;
    virtual void* GetScale(void) = 0;
    virtual void SetMode(int mode) = 0;
    virtual int GetMode(void) = 0;
    virtual void SetParameter(int paramID, int paramVal) = 0;
    virtual int GetParameter(int paramID) = 0;
    virtual int QuantiseValue(short val, int pos, int qp) = 0;
    static const int QUANT_ID = 0;
    static const int INTRA_FLAG_ID = 1;
    static const int TransformAndQuant = 0;
    static const int TransformOnly = 1;
    static const int QuantOnly = 2;
};

class IInverseTransform {
public:
    virtual ~IInverseTransform() {}
    virtual void InverseTransform(void* ptr) = 0;
    virtual void InverseTransform(void* pCoeff, void* pOut) = 0;
    virtual void SetScale(void* pScale) = 0;
    virtual void* GetScale(void) = 0;
    virtual void SetMode(int mode) = 0;
    virtual int GetMode(void) = 0;
    virtual void SetParameter(int paramID, int paramVal) = 0;
    virtual int GetParameter(int paramID) = 0;
    static const int QUANT_ID = 0;
    static const int TransformAndQuant = 0;
    static const int TransformOnly = 1;
    static const int QuantOnly = 2;
};

typedef short yuvType;
class RGBtoYUV420Converter {
public:
    RGBtoYUV420Converter(void) { _width = 0; _height = 0; _chrOff = 0; _flip = false; }
    RGBtoYUV420Converter(int width, int height) { _width = width; _height = height; _chrOff = 0; _flip = false; }
    RGBtoYUV420Converter(int width, int height, int chrOff) { _width = width; _height = height; _chrOff = chrOff; _flip = false; }
    virtual ~RGBtoYUV420Converter(void) {}
    virtual void Convert(void* pRgb, void* pY, void* pU, void* pV) = 0;
    int GetWidth(void) { return _width; }
    int GetHeight(void) { return _height; }
    int GetChrominanceOffset() const { return _chrOff; }
    bool GetFlip() const { return _flip; }
    void SetDimensions(int width, int height) { _width = width; _height = height; }
    void SetFlip(bool flip) { _flip = flip; }
    void SetChrominanceOffset(int val) { _chrOff = val; }

protected:
    int _width, _height, _chrOff;
    bool _flip;
};

class YUV420toRGBConverter {
public:
    YUV420toRGBConverter(void) { _width = 0; _height = 0; _rotate = 0; _chrOff = 0; _flip = false; }
    YUV420toRGBConverter(int width, int height) { _width = width; _height = height; _rotate = 0; _chrOff = 0; _flip = false; }
    YUV420toRGBConverter(int width, int height, int chrOff)
    {
        _width = width; _height = height; _rotate = 0; _chrOff = chrOff; _flip = false;
    }
    virtual ~YUV420toRGBConverter(void) {}
    virtual void Convert(void* pY, void* pU, void* pV, void* pRgb) = 0;
    int GetWidth(void) { return _width; }
    int GetHeight(void) { return _height; }
    int GetRotate(void) { return _rotate; }
    int GetChrominanceOffset(void) { return _chrOff; }
    bool GetFlip(void) { return _flip; }
    void SetDimensions(int width, int height) { _width = width; _height = height; }
    void SetRotate(int rotate) { _rotate = rotate; }
    void SetChrominanceOffset(int val) { _chrOff = val; }
    void SetFlip(bool flip) { _flip = flip; }

protected:
    int _width, _height, _rotate, _chrOff;
    bool _flip;
};
#endif  // VPPGPU_WITH_VPP

namespace vppgpu_vpp {

// One CUDA context per process unless the codec installs its own.
inline vppgpu_ctx*& default_context()
{
    static vppgpu_ctx* ctx = NULL;
    return ctx;
}

inline vppgpu_ctx* context()
{
    vppgpu_ctx*& c = default_context();
    if (!c && vppgpu_ctx_create(0, &c) != VPPGPU_OK) c = NULL;
    return c;
}

}  // namespace vppgpu_vpp

// ---------------------------------------------------------------------------
// IMotionEstimator replacements.  Constructor arguments, Create()/Ready()
// two-stage set-up, SetMode/GetMode and the returned VectorStructList follow
// MotionEstimatorH264ImplFull (src/CodecUtils/MotionEstimatorH264ImplFull.cpp:111-320).
// Every Estimate() re-reads the planes given at construction and, as the
// reference does, hands each final vector to the predictor
// (Set16x16MotionVector) so later frames and stages see them.
// ---------------------------------------------------------------------------
class GpuMotionEstimatorH264Base : public IMotionEstimator {
public:
    GpuMotionEstimatorH264Base(int kind, const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                               int motionRange, IMotionVectorPredictor* pMVPred, void* pDistortionIncluded)
        : _kind(kind), _pSrc(pSrc), _pRef(pRef), _w(imgWidth), _h(imgHeight), _range(motionRange),
          _pMVPred(pMVPred), _pIncl((bool*)pDistortionIncluded), _mode(1), _me(NULL), _list(NULL),
          _incl(NULL), _dist(NULL), _predDist(false), _last(VPPGPU_OK)
    {
    }
    virtual ~GpuMotionEstimatorH264Base() { Destroy(); }

    virtual int Create(void)
    {
        Destroy();
        vppgpu_ctx* ctx = vppgpu_vpp::context();
        if (!ctx || vppgpu_me_create(ctx, _kind, _w, _h, _range, &_me) != VPPGPU_OK) {
            _me = NULL;
            return 0;
        }
        vppgpu_me_set_mode(_me, _mode);
        int n = 0;
        vppgpu_me_num_mbs(_me, &n);
        _list = new VectorStructList(VectorStructList::SIMPLE2D);
        _list->SetLength(n);
        _incl = new unsigned char[n > 0 ? n : 1];
        _dist = new int[n > 0 ? n : 1];
        return 1;
    }
    virtual void Reset(void) {}
    virtual int Ready(void) { return _me ? 1 : 0; }
    virtual void SetMode(int mode)
    {
        _mode = mode;
        if (_me) vppgpu_me_set_mode(_me, mode);
    }
    virtual int GetMode(void) { return _mode; }
    virtual void* Estimate(const void* pSrc, const void* pRef, long* avgDistortion)
    {
        (void)pSrc;
        (void)pRef;
        return Estimate(avgDistortion);
    }
    virtual void* Estimate(long* avgDistortion) { return Run(avgDistortion, false, 0.0); }
    virtual void* Estimate(long* avgDistortion, void* param)
    {
        return param ? Run(avgDistortion, true, *(double*)param) : Estimate(avgDistortion);
    }

    // Status of the last Estimate() (vppgpu status code); the vpp interface
    // itself has no error channel.
    int LastStatus(void) const { return _last; }

protected:
    void* Run(long* avg, bool with_lambda, double lambda)
    {
        if (!_me) return NULL;
        int n = _list->GetLength();
        const unsigned char* incl = NULL;
        if (_pIncl) {
            for (int i = 0; i < n; i++) _incl[i] = _pIncl[i] ? 1 : 0;
            incl = _incl;
        }
        short* mv = (short*)_list->GetListPtr();
        long a = 0;
        int* dist = _predDist ? _dist : NULL;
        _last = with_lambda ? vppgpu_me_estimate_lambda(_me, (const short*)_pSrc, (const short*)_pRef, incl, NULL,
                                                        lambda, mv, dist, &a)
                            : vppgpu_me_estimate(_me, (const short*)_pSrc, (const short*)_pRef, incl, NULL, mv,
                                                 dist, &a);
        if (avg) *avg = _last == VPPGPU_OK ? a : 0;
        if (_last != VPPGPU_OK) return NULL;
        if (_pMVPred) {
            if (_predDist)  // estimators whose predictor also predicts a distortion
                for (int k = 0; k < n; k++) _pMVPred->Set16x16MotionVector(k, mv[2 * k], mv[2 * k + 1], dist[k]);
            else
                for (int k = 0; k < n; k++) _pMVPred->Set16x16MotionVector(k, mv[2 * k], mv[2 * k + 1]);
        }
        return (void*)_list;
    }
    void Destroy(void)
    {
        if (_me) vppgpu_me_destroy(_me);
        _me = NULL;
        delete _list;
        _list = NULL;
        delete[] _incl;
        _incl = NULL;
        delete[] _dist;
        _dist = NULL;
    }

    int _kind;
    const void* _pSrc;
    const void* _pRef;
    int _w, _h, _range;
    IMotionVectorPredictor* _pMVPred;
    bool* _pIncl;
    int _mode;
    vppgpu_me* _me;
    VectorStructList* _list;
    unsigned char* _incl;
    int* _dist;      // per-macroblock distortions handed to the predictor
    bool _predDist;  // Set16x16MotionVector(k, x, y, distortion) instead of (k, x, y)
    int _last;
};

class GpuMotionEstimatorH264ImplFull : public GpuMotionEstimatorH264Base {
public:
    GpuMotionEstimatorH264ImplFull(const void* pSrc, const void* pRef, int imgWidth, int imgHeight, int motionRange,
                                   IMotionVectorPredictor* pMVPred)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_FULL, pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred, NULL)
    {
    }
    GpuMotionEstimatorH264ImplFull(const void* pSrc, const void* pRef, int imgWidth, int imgHeight, int motionRange,
                                   IMotionVectorPredictor* pMVPred, void* pDistortionIncluded)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_FULL, pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred,
                                     pDistortionIncluded)
    {
    }
};

// The multi-resolution estimators, with the constructors of the reference
// classes (…MultiresCross.h:77-88, …MultiresCrossVer2.cpp:111-153,
// …Multires.cpp:107-171).  MultiresCross has no predictor; the reference's
// Multires estimates only through its constructor with pMVPred.
class GpuMotionEstimatorH264ImplMultiresCross : public GpuMotionEstimatorH264Base {
public:
    GpuMotionEstimatorH264ImplMultiresCross(const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                                            int motionRange)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_MULTIRES_CROSS, pSrc, pRef, imgWidth, imgHeight, motionRange, NULL,
                                     NULL)
    {
    }
    GpuMotionEstimatorH264ImplMultiresCross(const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                                            int motionRange, void* pDistortionIncluded)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_MULTIRES_CROSS, pSrc, pRef, imgWidth, imgHeight, motionRange, NULL,
                                     pDistortionIncluded)
    {
    }
};

class GpuMotionEstimatorH264ImplMultiresCrossVer2 : public GpuMotionEstimatorH264Base {
public:
    GpuMotionEstimatorH264ImplMultiresCrossVer2(const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                                                int motionRange, IMotionVectorPredictor* pMVPred)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_MULTIRES_CROSS_V2, pSrc, pRef, imgWidth, imgHeight, motionRange,
                                     pMVPred, NULL)
    {
    }
    GpuMotionEstimatorH264ImplMultiresCrossVer2(const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                                                int motionRange, IMotionVectorPredictor* pMVPred,
                                                void* pDistortionIncluded)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_MULTIRES_CROSS_V2, pSrc, pRef, imgWidth, imgHeight, motionRange,
                                     pMVPred, pDistortionIncluded)
    {
    }
};

// MotionEstimatorH263ImplMultiresCross: motionRange (at most 64) and the vectors in half pels.
class GpuMotionEstimatorH263ImplMultiresCross : public GpuMotionEstimatorH264Base {
public:
    GpuMotionEstimatorH263ImplMultiresCross(const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                                            int motionRange)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_H263_MULTIRES_CROSS, pSrc, pRef, imgWidth, imgHeight, motionRange,
                                     NULL, NULL)
    {
    }
    GpuMotionEstimatorH263ImplMultiresCross(const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                                            int motionRange, void* pDistortionIncluded)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_H263_MULTIRES_CROSS, pSrc, pRef, imgWidth, imgHeight, motionRange,
                                     NULL, pDistortionIncluded)
    {
    }
};

// MotionEstimatorH263ImplMultiresCrossVer2 (src/CodecUtils/MotionEstimatorH263ImplMultiresCrossVer2.cpp):
// motionRange (at most 64) and the vectors in half pels.  The reference asks its predictor
// (an H263MotionVectorPredictorImpl1) for the H.263 median of the vectors it has written; the device
// computes that median itself, so pMVPred is taken for the signature and not called (the reference
// never sets vectors on it either).
class GpuMotionEstimatorH263ImplMultiresCrossVer2 : public GpuMotionEstimatorH264Base {
public:
    GpuMotionEstimatorH263ImplMultiresCrossVer2(const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                                                int motionRange, IMotionVectorPredictor* pMVPred)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_H263_MULTIRES_CROSS_V2, pSrc, pRef, imgWidth, imgHeight, motionRange,
                                     NULL, NULL)
    {
        (void)pMVPred;
    }
    GpuMotionEstimatorH263ImplMultiresCrossVer2(const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                                                int motionRange, IMotionVectorPredictor* pMVPred,
                                                void* pDistortionIncluded)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_H263_MULTIRES_CROSS_V2, pSrc, pRef, imgWidth, imgHeight, motionRange,
                                     NULL, pDistortionIncluded)
    {
        (void)pMVPred;
    }
};

// The integer-pel stage of MotionEstimatorH264ImplFull with its MEH264IF_ABS_DIFF
// distortion (MotionEstimatorH264ImplFull.cpp:341-446, OverlayMem2Dv2::Tad16x16 /
// Tad16x16LessThan): full-pel winners in quarter pels, their SAD as distortion.
class GpuMotionEstimatorH264ImplFullSad : public GpuMotionEstimatorH264Base {
public:
    GpuMotionEstimatorH264ImplFullSad(const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                                      int motionRange, IMotionVectorPredictor* pMVPred)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_FULL_SAD, pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred, NULL)
    {
    }
    GpuMotionEstimatorH264ImplFullSad(const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                                      int motionRange, IMotionVectorPredictor* pMVPred, void* pDistortionIncluded)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_FULL_SAD, pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred,
                                     pDistortionIncluded)
    {
    }
};

// MotionEstimatorH264ImplCross: quarter pel by default (SetMode 0; 1 half, 2 full pel).
class GpuMotionEstimatorH264ImplCross : public GpuMotionEstimatorH264Base {
public:
    GpuMotionEstimatorH264ImplCross(const void* pSrc, const void* pRef, int imgWidth, int imgHeight, int motionRange,
                                    IMotionVectorPredictor* pMVPred)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_CROSS, pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred, NULL)
    {
        _mode = 0;
    }
    GpuMotionEstimatorH264ImplCross(const void* pSrc, const void* pRef, int imgWidth, int imgHeight, int motionRange,
                                    IMotionVectorPredictor* pMVPred, void* pDistortionIncluded)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_CROSS, pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred,
                                     pDistortionIncluded)
    {
        _mode = 0;
    }
};

class GpuMotionEstimatorH264ImplMultires : public GpuMotionEstimatorH264Base {
public:
    GpuMotionEstimatorH264ImplMultires(const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                                       int motionRange, IMotionVectorPredictor* pMVPred, void* pDistortionIncluded)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_MULTIRES, pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred,
                                     pDistortionIncluded)
    {
    }
};

// The estimators that search from the prediction and predict a distortion
// too: MotionEstimatorH264ImplUMHS (…ImplUMHS.cpp:187-254) and
// MotionEstimatorH264ImplFHS (…ImplFHS.cpp:230-297), quarter pel by default,
// SetMode kept as given.  Each vector goes to the predictor with its
// distortion (H264MotionVectorPredictorImpl1.h:112-121).  UMHS reads the
// previous frame's macroblocks (vectors and intra flags) on every Estimate():
// from the MacroBlockH264 array of its eight-argument constructor when built
// against vpp, or from the arrays given to SetPrevFrame().
class GpuMotionEstimatorH264ImplUMHS : public GpuMotionEstimatorH264Base {
public:
    GpuMotionEstimatorH264ImplUMHS(const void* pSrc, const void* pRef, int imgWidth, int imgHeight, int motionRange,
                                   IMotionVectorPredictor* pMVPred, void* pDistortionIncluded = NULL)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_UMHS, pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred,
                                     pDistortionIncluded),
          _prevMv(NULL), _prevIntra(NULL)
#ifdef VPPGPU_WITH_VPP
          , _pPrevFrmMBlk(NULL)
#endif
    {
        _mode = 0;
        _predDist = true;
    }
#ifdef VPPGPU_WITH_VPP
    GpuMotionEstimatorH264ImplUMHS(const void* pSrc, const void* pRef, int imgWidth, int imgHeight, int motionRange,
                                   IMotionVectorPredictor* pMVPred, void* pDistortionIncluded,
                                   MacroBlockH264* pPrevFrmMBlk)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_UMHS, pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred,
                                     pDistortionIncluded),
          _prevMv(NULL), _prevIntra(NULL), _pPrevFrmMBlk(pPrevFrmMBlk)
    {
        _mode = 0;
        _predDist = true;
    }
#endif
    virtual ~GpuMotionEstimatorH264ImplUMHS() { FreePrev(); }
    // The previous frame's 16x16 vectors (2 shorts per macroblock, quarter pels)
    // and intra flags (NULL: all inter); read on every Estimate(), not copied.
    void SetPrevFrame(const short* prevMv, const unsigned char* prevIntra)
    {
        _prevMv = prevMv;
        _prevIntra = prevIntra;
    }
    virtual void* Estimate(long* avgDistortion)
    {
        if (!_me) return NULL;
        const short* mv = _prevMv;
        const unsigned char* intra = _prevIntra;
#ifdef VPPGPU_WITH_VPP
        int n = _list->GetLength();
        if (_pPrevFrmMBlk) {  // MacroBlockH264::_mvX[_16x16], _mvY[_16x16], _intraFlag
            if (!_mvBuf) _mvBuf = new short[2 * (size_t)n];
            if (!_intraBuf) _intraBuf = new unsigned char[n];
            for (int k = 0; k < n; k++) {
                _mvBuf[2 * k] = (short)_pPrevFrmMBlk[k]._mvX[MacroBlockH264::_16x16];
                _mvBuf[2 * k + 1] = (short)_pPrevFrmMBlk[k]._mvY[MacroBlockH264::_16x16];
                _intraBuf[k] = _pPrevFrmMBlk[k]._intraFlag ? 1 : 0;
            }
            mv = _mvBuf;
            intra = _intraBuf;
        }
#endif
        _last = vppgpu_me_set_prev_frame(_me, mv, intra);
        if (_last != VPPGPU_OK) {
            if (avgDistortion) *avgDistortion = 0;
            return NULL;
        }
        return GpuMotionEstimatorH264Base::Estimate(avgDistortion);
    }
    virtual void* Estimate(const void* pSrc, const void* pRef, long* avgDistortion)
    {
        (void)pSrc;
        (void)pRef;
        return Estimate(avgDistortion);
    }

private:
    void FreePrev(void)
    {
#ifdef VPPGPU_WITH_VPP
        delete[] _mvBuf;
        delete[] _intraBuf;
        _mvBuf = NULL;
        _intraBuf = NULL;
#endif
    }
    const short* _prevMv;
    const unsigned char* _prevIntra;
#ifdef VPPGPU_WITH_VPP
    MacroBlockH264* _pPrevFrmMBlk;
    short* _mvBuf = NULL;
    unsigned char* _intraBuf = NULL;
#endif
};

class GpuMotionEstimatorH264ImplFHS : public GpuMotionEstimatorH264Base {
public:
    GpuMotionEstimatorH264ImplFHS(const void* pSrc, const void* pRef, int imgWidth, int imgHeight, int motionRange,
                                  IMotionVectorPredictor* pMVPred, void* pDistortionIncluded = NULL)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_FHS, pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred,
                                     pDistortionIncluded)
    {
        _mode = 0;
        _predDist = true;
    }
#ifdef VPPGPU_WITH_VPP
    // the previous-frame macroblocks are accepted and not read, as in the reference (…ImplFHS.cpp:627-673)
    GpuMotionEstimatorH264ImplFHS(const void* pSrc, const void* pRef, int imgWidth, int imgHeight, int motionRange,
                                  IMotionVectorPredictor* pMVPred, void* pDistortionIncluded, MacroBlockH264*)
        : GpuMotionEstimatorH264Base(VPPGPU_ME_FHS, pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred,
                                     pDistortionIncluded)
    {
        _mode = 0;
        _predDist = true;
    }
#endif
};

// MotionEstimatorImpl1 (pSrc, pRef, w, h, macroBlkWidth, macroBlkHeight, motionRange)
// (src/CodecUtils/MotionEstimatorImpl1.cpp:111-395): blocks 16x16 or 8x8, the range
// in full pels; Estimate() returns a SimpleMotionVectorList of half-pel
// (char x, char y) vectors, as the reference does.  No predictor.
class GpuMotionEstimatorImpl1 : public IMotionEstimator {
public:
    GpuMotionEstimatorImpl1(const void* pSrc, const void* pRef, int imgWidth, int imgHeight, int macroBlkWidth,
                            int macroBlkHeight, int motionRange)
        : _kind(VPPGPU_ME_IMPL1), _pSrc(pSrc), _pRef(pRef), _w(imgWidth), _h(imgHeight), _bw(macroBlkWidth),
          _bh(macroBlkHeight), _range(motionRange), _mode(0), _me(NULL), _list(NULL), _mv(NULL), _last(VPPGPU_OK)
    {
    }
    virtual ~GpuMotionEstimatorImpl1() { Destroy(); }
    virtual int Create(void)
    {
        Destroy();
        vppgpu_ctx* ctx = vppgpu_vpp::context();
        if (!ctx || vppgpu_me_create_blocks(ctx, _kind, _w, _h, _bw, _bh, _range, &_me) != VPPGPU_OK) {
            _me = NULL;
            return 0;
        }
        vppgpu_me_set_mode(_me, _mode);
        vppgpu_me_get_mode(_me, &_mode);
        int n = 0;
        vppgpu_me_num_mbs(_me, &n);
        _list = new SimpleMotionVectorList();
        _list->SetLength(n);
        _mv = new short[2 * (size_t)(n > 0 ? n : 1)];
        return 1;
    }
    virtual void Reset(void) {}
    virtual int Ready(void) { return _me ? 1 : 0; }
    virtual void SetMode(int mode)
    {
        _mode = mode;
        if (_me) {  // Impl2 picks its levels by area for mode 0, as the reference does
            vppgpu_me_set_mode(_me, mode);
            vppgpu_me_get_mode(_me, &_mode);
        }
    }
    virtual int GetMode(void) { return _mode; }
    virtual void* Estimate(const void* pSrc, const void* pRef, long* avgDistortion)
    {
        (void)pSrc;
        (void)pRef;
        return Estimate(avgDistortion);
    }
    virtual void* Estimate(long* avgDistortion)
    {
        if (!_me) return NULL;
        long a = 0;
        _last = vppgpu_me_estimate(_me, (const short*)_pSrc, (const short*)_pRef, NULL, NULL, _mv, NULL, &a);
        if (avgDistortion) *avgDistortion = _last == VPPGPU_OK ? a : 0;
        if (_last != VPPGPU_OK) return NULL;
        char* p = (char*)_list->GetDataPtr();
        const int step = _list->GetPatternSize();
        for (int k = 0; k < _list->GetLength(); k++) {  // the half-pel vectors fit in chars (|v| <= 65)
            p[(size_t)k * step] = (char)_mv[2 * k];
            p[(size_t)k * step + 1] = (char)_mv[2 * k + 1];
        }
        return (void*)_list;
    }
    int LastStatus(void) const { return _last; }

protected:
    GpuMotionEstimatorImpl1(int kind, int mode, const void* pSrc, const void* pRef, int imgWidth, int imgHeight,
                            int macroBlkWidth, int macroBlkHeight, int motionRange)
        : _kind(kind), _pSrc(pSrc), _pRef(pRef), _w(imgWidth), _h(imgHeight), _bw(macroBlkWidth),
          _bh(macroBlkHeight), _range(motionRange), _mode(mode), _me(NULL), _list(NULL), _mv(NULL), _last(VPPGPU_OK)
    {
    }

private:
    void Destroy(void)
    {
        if (_me) vppgpu_me_destroy(_me);
        _me = NULL;
        delete _list;
        _list = NULL;
        delete[] _mv;
        _mv = NULL;
    }
    int _kind;
    const void* _pSrc;
    const void* _pRef;
    int _w, _h, _bw, _bh, _range, _mode;
    vppgpu_me* _me;
    SimpleMotionVectorList* _list;
    short* _mv;
    int _last;
};

// MotionEstimatorImpl2 (src/CodecUtils/MotionEstimatorImpl2.cpp:111-826): the SAD
// pyramid, 16x16 blocks, the range in full pels; SetMode(1) (the default) two
// levels, 2 three, 0 by area; the same SimpleMotionVectorList output.
class GpuMotionEstimatorImpl2 : public GpuMotionEstimatorImpl1 {
public:
    GpuMotionEstimatorImpl2(const void* pSrc, const void* pRef, int imgWidth, int imgHeight, int macroBlkWidth,
                            int macroBlkHeight, int motionRange)
        : GpuMotionEstimatorImpl1(VPPGPU_ME_IMPL2, 1, pSrc, pRef, imgWidth, imgHeight, macroBlkWidth, macroBlkHeight,
                                  motionRange)
    {
    }
};

// ---------------------------------------------------------------------------
// IForwardTransform / IInverseTransform replacements (FastForward4x4ITImpl1,
// FastInverse4x4ITImpl1 and their On16x16 variants).  Transform(void*) takes
// one unit like the reference; TransformBlocks() takes many at once, which is
// where the GPU pays off.
// ---------------------------------------------------------------------------
class GpuForward4x4IT : public IForwardTransform {
public:
    explicit GpuForward4x4IT(int layout = VPPGPU_LAYOUT_BLOCKS)
        : _layout(layout), _mode(TransformAndQuant), _q(1), _intra(1) {}
    virtual void Transform(void* ptr) { TransformBlocks(ptr, 1); }
    virtual void Transform(void* pIn, void* pCoeff)
    {
        memcpy(pCoeff, pIn, sizeof(short) * Unit());
        Transform(pCoeff);
    }
    void TransformBlocks(void* ptr, long long nunits)
    {
        vppgpu_fwd4x4(vppgpu_vpp::context(), (short*)ptr, nunits, _layout, _mode, _q, _intra);
    }
    virtual void SetScale(void* pScale) { (void)pScale; }
    virtual void* GetScale(void) { return NULL; }
    virtual void SetMode(int mode) { _mode = mode; }
    virtual int GetMode(void) { return _mode; }
    virtual void SetParameter(int paramID, int paramVal)
    {
        if (paramID == QUANT_ID) _q = paramVal;
        else if (paramID == INTRA_FLAG_ID) _intra = paramVal;
    }
    virtual int GetParameter(int paramID) { return paramID == QUANT_ID ? _q : _intra; }
    virtual int QuantiseValue(short val, int pos, int qp)
    {
        _q = qp;
        return vppgpu_quantise_value(val, pos, qp, _intra);
    }

protected:
    size_t Unit() const { return _layout == VPPGPU_LAYOUT_BLOCKS ? 16 : 256; }
    int _layout, _mode, _q, _intra;
};

class GpuInverse4x4IT : public IInverseTransform {
public:
    explicit GpuInverse4x4IT(int layout = VPPGPU_LAYOUT_BLOCKS) : _layout(layout), _mode(TransformAndQuant), _q(1)
    {
        for (int i = 0; i < 16; i++) _weight[i] = 16;
    }
    virtual void InverseTransform(void* ptr) { InverseTransformBlocks(ptr, 1); }
    virtual void InverseTransform(void* pCoeff, void* pOut)
    {
        memcpy(pOut, pCoeff, sizeof(short) * (_layout == VPPGPU_LAYOUT_BLOCKS ? 16 : 256));
        InverseTransform(pOut);
    }
    void InverseTransformBlocks(void* ptr, long long nunits)
    {
        vppgpu_inv4x4(vppgpu_vpp::context(), (short*)ptr, nunits, _layout, _mode, _q, _weight);
    }
    virtual void SetScale(void* pScale) { memcpy(_weight, pScale, sizeof(_weight)); }
    virtual void* GetScale(void) { return (void*)_weight; }
    virtual void SetMode(int mode) { _mode = mode; }
    virtual int GetMode(void) { return _mode; }
    virtual void SetParameter(int paramID, int paramVal)
    {
        if (paramID == QUANT_ID) _q = paramVal;
    }
    virtual int GetParameter(int paramID) { (void)paramID; return _q; }

protected:
    int _layout, _mode, _q;
    int _weight[16];
};

// ---------------------------------------------------------------------------
// DC Hadamard transforms: size 4 replaces FastForwardDC4x4ITImpl1 /
// FastInverseDC4x4ITImpl1 (Intra16x16 luma DC), size 2 FastForwardDC2x2ITImpl1
// / FastInverseDC2x2ITImpl1 (chroma DC).  TransformBlocks() takes many
// blocks at once.
// ---------------------------------------------------------------------------
class GpuForwardDCIT : public IForwardTransform {
public:
    explicit GpuForwardDCIT(int size = 4) : _size(size), _mode(TransformAndQuant), _q(1) {}
    virtual void Transform(void* ptr) { TransformBlocks(ptr, 1); }
    virtual void Transform(void* pIn, void* pCoeff)
    {
        memcpy(pCoeff, pIn, sizeof(short) * _size * _size);
        Transform(pCoeff);
    }
    void TransformBlocks(void* ptr, long long nunits)
    {
        vppgpu_fwd_dc(vppgpu_vpp::context(), (short*)ptr, nunits, _size, _mode, _q);
    }
    virtual void SetScale(void* pScale) { (void)pScale; }
    virtual void* GetScale(void) { return NULL; }
    virtual void SetMode(int mode) { _mode = mode; }
    virtual int GetMode(void) { return _mode; }
    virtual void SetParameter(int paramID, int paramVal)
    {
        if (paramID == QUANT_ID) _q = paramVal;
    }
    virtual int GetParameter(int paramID) { (void)paramID; return _q; }
    virtual int QuantiseValue(short val, int pos, int qp)
    {
        (void)pos;
        if (_size != 4) return 0;  // FastForwardDC2x2ITImpl1 has no quantiser of single values
        _q = qp;
        return vppgpu_dc_quantise_value(val, qp);
    }

protected:
    int _size, _mode, _q;
};

class GpuInverseDCIT : public IInverseTransform {
public:
    explicit GpuInverseDCIT(int size = 4) : _size(size), _mode(TransformAndQuant), _q(1)
    {
        for (int i = 0; i < 16; i++) _weight[i] = 16;
    }
    virtual void InverseTransform(void* ptr) { InverseTransformBlocks(ptr, 1); }
    virtual void InverseTransform(void* pCoeff, void* pOut)
    {
        memcpy(pOut, pCoeff, sizeof(short) * _size * _size);
        InverseTransform(pOut);
    }
    void InverseTransformBlocks(void* ptr, long long nunits)
    {
        vppgpu_inv_dc(vppgpu_vpp::context(), (short*)ptr, nunits, _size, _mode, _q, _weight);
    }
    virtual void SetScale(void* pScale) { memcpy(_weight, pScale, sizeof(int) * _size * _size); }
    virtual void* GetScale(void) { return (void*)_weight; }
    virtual void SetMode(int mode) { _mode = mode; }
    virtual int GetMode(void) { return _mode; }
    virtual void SetParameter(int paramID, int paramVal)
    {
        if (paramID == QUANT_ID) _q = paramVal;
    }
    virtual int GetParameter(int paramID) { (void)paramID; return _q; }

protected:
    int _size, _mode, _q;
    int _weight[16];
};

// ---------------------------------------------------------------------------
// The GPU slot vpp reserves for colour conversion (an empty class in the
// reference, include/ImageUtils/FastGpuRGB24toYUV420Converter.h).
// ---------------------------------------------------------------------------
class FastGpuRGB24toYUV420Converter : public RGBtoYUV420Converter {
public:
    FastGpuRGB24toYUV420Converter(void) : _kind(VPPGPU_RGB_FIXED_POINT) {}
    FastGpuRGB24toYUV420Converter(int width, int height) : RGBtoYUV420Converter(width, height), _kind(VPPGPU_RGB_FIXED_POINT) {}
    FastGpuRGB24toYUV420Converter(int width, int height, int chrOff)
        : RGBtoYUV420Converter(width, height, chrOff), _kind(VPPGPU_RGB_FIXED_POINT)
    {
        _flip = false;
    }
    void SetArithmetic(int kind) { _kind = kind; }
    virtual void Convert(void* pRgb, void* pY, void* pU, void* pV)
    {
        vppgpu_rgb24_to_yuv420(vppgpu_vpp::context(), _kind, (const unsigned char*)pRgb, _width, _height, _chrOff,
                               _flip ? 1 : 0, (short*)pY, (short*)pU, (short*)pV);
    }

protected:
    int _kind;
};

// ---------------------------------------------------------------------------
// YUV420toRGBConverter on the GPU with the arithmetic of one of vpp's Real
// converters: VPPGPU_YUV_REAL (RealYUV420toRGB24Converter), VPPGPU_YUV_REAL_IMPL2
// (RealYUV420toRGB24ConverterImpl2 / ...Impl2Ver16) or VPPGPU_YUV_CCIR601
// (RealYUV420toRGB24CCIR601Converter / ...Ver16).  The constructor sets the
// chrominance offset as the reference's two-argument constructors do not;
// call SetChrominanceOffset() as with the reference.
// ---------------------------------------------------------------------------
class GpuYUV420toRGB24Converter : public YUV420toRGBConverter {
public:
    GpuYUV420toRGB24Converter(int width, int height, int kind = VPPGPU_YUV_REAL_IMPL2)
        : YUV420toRGBConverter(width, height, 0), _kind(kind) {}
    virtual void Convert(void* pY, void* pU, void* pV, void* pRgb)
    {
        vppgpu_yuv420_to_rgb24(vppgpu_vpp::context(), _kind, (const short*)pY, (const short*)pU, (const short*)pV,
                               _width, _height, _chrOff, _rotate, _flip ? 1 : 0, (unsigned char*)pRgb);
    }

protected:
    int _kind;
};
