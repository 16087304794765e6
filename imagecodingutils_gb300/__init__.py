"""GB300 (sm_103a) encoder hot path of vpp (CSIR-RTVC/ImageCodingUtils).

Python mirror of the reference's C++ plugin interfaces over the C ABI in
``include/vppgpu.h``.  Class, method and parameter names follow the
reference so code and tests read like the vpp originals:

* ``MotionEstimatorH264ImplFull`` -- ``IMotionEstimator``
  (include/CodecUtils/IMotionEstimator.h:51-96): ``Create``, ``Reset``,
  ``Ready``, ``SetMode``/``GetMode``, ``Estimate``.
* ``FastForward4x4ITImpl1`` / ``FastForward4x4ITImpl2`` /
  ``FastForward4x4On16x16ITImpl1`` -- ``IForwardTransform``
  (include/CodecUtils/IForwardTransform.h:56-127).
* ``FastInverse4x4ITImpl1`` / ``FastInverse4x4On16x16ITImpl1`` -- ``IInverseTransform``.
* ``FastGpuRGB24toYUV420Converter`` -- ``RGBtoYUV420Converter``
  (include/ImageUtils/RGBtoYUV420Converter.h:57-86), the reference's own
  reserved (empty) GPU slot.

Every call runs the CUDA kernels; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import VppGpuError, check, load

__all__ = [
    "Context", "get_context", "MotionEstimatorH264ImplFull", "MotionEstimatorH264ImplMultires",
    "MotionEstimatorH264ImplMultiresCross", "MotionEstimatorH264ImplMultiresCrossVer2", "MotionEstimatorH264ImplCross", "MotionEstimatorH264ImplFullSad", "MotionEstimatorH264ImplUMHS", "MotionEstimatorH264ImplFHS", "MotionEstimatorImpl1", "MotionEstimatorImpl2",
    "MotionEstimatorH263ImplMultiresCross",
    "MotionEstimatorH263ImplMultiresCrossVer2", "MotionEstimatorBatch",
    "Server", "FastForward4x4ITImpl1", "FastForward4x4ITImpl2",
    "FastForward4x4On16x16ITImpl1", "FastInverse4x4ITImpl1", "FastInverse4x4On16x16ITImpl1", "FastForwardDC4x4ITImpl1",
    "FastForwardDC2x2ITImpl1", "FastInverseDC4x4ITImpl1", "FastInverseDC2x2ITImpl1",
    "FastGpuRGB24toYUV420Converter", "RealYUV420toRGB24Converter", "RealYUV420toRGB24ConverterImpl2",
    "RealYUV420toRGB24ConverterImpl2Ver16", "RealYUV420toRGB24CCIR601Converter",
    "RealYUV420toRGB24CCIR601ConverterVer16", "Fast6BitYUV420toRGB24Converter", "Real6BitYUV420toRGB24Converter",
    "Fast6BitYUV420toRGB24ZoomConverter", "MotionCompensatorH264ImplStd", "VppGpuError", "load",
]


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Context:
    """One CUDA device and stream (vppgpu_ctx)."""

    def __init__(self, device: int = 0):
        lib = load()
        h = C.c_void_p()
        check(lib.vppgpu_ctx_create(device, C.byref(h)), "vppgpu_ctx_create")
        self.handle = h
        self.device = device

    def synchronize(self):
        check(load().vppgpu_ctx_synchronize(self.handle), "vppgpu_ctx_synchronize")

    def set_stream(self, stream_ptr: int | None):
        check(load().vppgpu_ctx_set_stream(self.handle, C.c_void_p(stream_ptr) if stream_ptr else None),
              "vppgpu_ctx_set_stream")

    def launch_count(self) -> int:
        n = C.c_ulonglong()
        check(load().vppgpu_ctx_launch_count(self.handle, C.byref(n)), "vppgpu_ctx_launch_count")
        return n.value

    def close(self):
        if getattr(self, "handle", None):
            load().vppgpu_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Context | None = None


def get_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


# ---------------------------------------------------------------------------
# Motion estimation
# ---------------------------------------------------------------------------
class _MotionEstimatorBase:
    KIND = _lib.ME_FULL
    DEFAULT_MODE = 1

    def __init__(self, pSrc, pRef, imgWidth: int, imgHeight: int, motionRange: int = 64, pMVPred=None,
                 pDistortionIncluded=None, mb_slice=None, ctx: Context | None = None):
        # The planes are captured by reference and re-read on every Estimate(),
        # as the reference does with its pSrc/pRef constructor arguments.
        self._src = pSrc
        self._ref = pRef
        self._w = int(imgWidth)
        self._h = int(imgHeight)
        self._range = int(motionRange)
        self._pred = pMVPred
        self._incl = None if pDistortionIncluded is None else np.ascontiguousarray(pDistortionIncluded, np.uint8)
        self._slice = None if mb_slice is None else np.ascontiguousarray(mb_slice, np.int32)
        self._ctx = ctx or get_context()
        self._h_me = None
        self._mode = self.DEFAULT_MODE
        self.last_mb_distortion = None

    # IMotionEstimator
    def Create(self) -> int:
        self._destroy()
        h = C.c_void_p()
        rc = load().vppgpu_me_create(self._ctx.handle, self.KIND, self._w, self._h, self._range, C.byref(h))
        if rc != _lib.OK:
            return 0
        self._h_me = h
        load().vppgpu_me_set_mode(self._h_me, self._mode)
        return 1

    def Reset(self) -> None:
        pass

    def Ready(self) -> int:
        return 1 if self._h_me else 0

    def SetMode(self, mode: int) -> None:
        self._mode = int(mode)
        if self._h_me:
            load().vppgpu_me_set_mode(self._h_me, self._mode)

    def GetMode(self) -> int:
        return self._mode

    def num_mbs(self) -> int:
        return (self._w // 16) * (self._h // 16)

    def Estimate(self, *args, param: float | None = None, want_mb_distortion: bool = True):
        """Estimate() -> (vectors[N_MB, 2] int16 quarter-pel, avgDistortion).

        Estimate(pSrc, pRef) ignores its arguments and uses the constructor
        planes, exactly like the reference (MotionEstimatorH264ImplFull.h:109-110).
        Estimate(param) or Estimate(param=lambda) is Estimate(long*, void* param)
        (IMotionEstimator.h:94): MultiresCrossVer2's Lagrangian overload, the
        plain estimate for the other estimators, which ignore the parameter."""
        if len(args) == 1:
            param = args[0]
        if not self._h_me:
            raise VppGpuError(_lib.ERR_NOT_READY, "Estimate before Create")
        src = np.ascontiguousarray(self._src, np.int16)
        ref = np.ascontiguousarray(self._ref, np.int16)
        if src.size != self._w * self._h or ref.size != self._w * self._h:
            raise ValueError("source/reference plane size does not match the estimator")
        n = self.num_mbs()
        mv = np.empty((n, 2), np.int16)
        dist = np.empty(n, np.int32) if want_mb_distortion else None
        avg = C.c_long(0)
        if param is None:
            check(load().vppgpu_me_estimate(self._h_me, _ptr(src), _ptr(ref), _ptr(self._incl), _ptr(self._slice),
                                            _ptr(mv), _ptr(dist), C.byref(avg)), "vppgpu_me_estimate")
        else:
            check(load().vppgpu_me_estimate_lambda(self._h_me, _ptr(src), _ptr(ref), _ptr(self._incl),
                                                   _ptr(self._slice), float(param), _ptr(mv), _ptr(dist),
                                                   C.byref(avg)), "vppgpu_me_estimate_lambda")
        self.last_mb_distortion = dist
        setter = getattr(self._pred, "Set16x16MotionVector", None)
        if setter is not None:  # side effect of the reference on its predictor
            for k in range(n):
                setter(k, int(mv[k, 0]), int(mv[k, 1]))
        return mv, avg.value

    def Autotune(self, reps: int = 2) -> dict:
        """Time the estimator's launch shapes and relaxation policy on the
        constructor planes and keep the fastest (vppgpu_me_autotune; results
        are the same for every choice).  Returns the chosen tuning."""
        if not self._h_me:
            raise VppGpuError(_lib.ERR_NOT_READY, "Autotune before Create")
        src = np.ascontiguousarray(self._src, np.int16)
        ref = np.ascontiguousarray(self._ref, np.int16)
        idx = C.c_int()
        check(load().vppgpu_me_autotune_host(self._h_me, _ptr(src), _ptr(ref), int(reps), C.byref(idx)),
              "vppgpu_me_autotune_host")
        return dict(self.tuning(), choice=idx.value)

    def tuning(self) -> dict:
        t = (C.c_int * 4)()
        check(load().vppgpu_me_get_tuning(self._h_me, t), "vppgpu_me_get_tuning")
        return {"relax_sweeps": t[0], "grid_sweeps": t[1], "sweep_ctas_per_sm": t[2], "search_mbs_per_cta": t[3]}

    def last_sweeps(self) -> int:
        s = C.c_int()
        check(load().vppgpu_me_last_sweeps(self._h_me, C.byref(s)), "vppgpu_me_last_sweeps")
        return s.value

    def _destroy(self):
        # a handle outlived by its context (finalizers at interpreter exit run
        # in any order) is left to the process exit: destroying it would
        # touch the freed context
        if self._h_me and self._ctx.handle:
            load().vppgpu_me_destroy(self._h_me)
        self._h_me = None

    def __del__(self):
        try:
            self._destroy()
        except Exception:
            pass


class MotionEstimatorH264ImplFull(_MotionEstimatorBase):
    """GPU MotionEstimatorH264ImplFull (src/CodecUtils/MotionEstimatorH264ImplFull.cpp)."""

    KIND = _lib.ME_FULL


class MotionEstimatorH264ImplCross(_MotionEstimatorBase):
    """GPU MotionEstimatorH264ImplCross (src/CodecUtils/MotionEstimatorH264ImplCross.cpp):
    cross search of halving steps with the 64-point path distortion and its
    extrapolating early exit, the full-search sub-pel window, ties towards the
    rounded prediction, the pred-vector check and GetBestVector (lambda 0.9,
    norm 64).  SetMode(0) quarter pel (the default), 1 half, 2 full pel."""

    KIND = _lib.ME_CROSS
    DEFAULT_MODE = 0


class MotionEstimatorH264ImplFullSad(_MotionEstimatorBase):
    """GPU integer-pel stage of MotionEstimatorH264ImplFull with the
    MEH264IF_ABS_DIFF distortion (src/CodecUtils/MotionEstimatorH264ImplFull.cpp:341-446,
    OverlayMem2Dv2::Tad16x16 / Tad16x16LessThan): full search of the range by SAD,
    ties towards the rounded median prediction, vectors the full-pel winners in
    quarter pels, distortions their SAD, no sub-pel stage or GetBestVector."""

    KIND = _lib.ME_FULL_SAD


class MotionEstimatorH264ImplUMHS(_MotionEstimatorBase):
    """GPU MotionEstimatorH264ImplUMHS (src/CodecUtils/MotionEstimatorH264ImplUMHS.cpp):
    the unsymmetrical-cross multi-hexagon-grid search from the median prediction,
    as built by the reference's eight-argument constructor
    (pSrc, pRef, w, h, motionRange, pMVPred, pDistortionIncluded, pPrevFrmMBlk).
    pPrevFrmMBlk is given as (prev_mv[N_MB, 2] quarter-pel, prev_intra[N_MB] or
    None), the _mvX[0] / _mvY[0] / _intraFlag fields of the previous frame's
    macroblocks; it is re-read on every Estimate(), as the reference reads the
    caller's array.  The predictor side effect carries the distortion:
    Set16x16MotionVector(k, x, y, d).  SetMode(0) quarter pel (the default),
    1 half, 2 full pel."""

    KIND = _lib.ME_UMHS
    DEFAULT_MODE = 0

    def __init__(self, pSrc, pRef, imgWidth: int, imgHeight: int, motionRange: int = 64, pMVPred=None,
                 pDistortionIncluded=None, pPrevFrmMBlk=None, mb_slice=None, ctx: Context | None = None):
        super().__init__(pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred, pDistortionIncluded, mb_slice, ctx)
        self._prev = pPrevFrmMBlk

    def Estimate(self, *args, param: float | None = None, want_mb_distortion: bool = True):
        if not self._h_me:
            raise VppGpuError(_lib.ERR_NOT_READY, "Estimate before Create")
        pmv, pin = (None, None) if self._prev is None else self._prev
        pmv = None if pmv is None else np.ascontiguousarray(pmv, np.int16)
        pin = None if pin is None else np.ascontiguousarray(pin, np.uint8)
        check(load().vppgpu_me_set_prev_frame(self._h_me, _ptr(pmv), _ptr(pin)), "vppgpu_me_set_prev_frame")
        pred, self._pred = self._pred, None
        try:
            mv, avg = super().Estimate(*args, param=param, want_mb_distortion=True)
        finally:
            self._pred = pred
        if self._pred is not None:  # the reference hands the predictor each vector with its distortion
            d = self.last_mb_distortion
            for k in range(self.num_mbs()):
                self._pred.Set16x16MotionVector(k, int(mv[k, 0]), int(mv[k, 1]), int(d[k]))
        return mv, avg


class MotionEstimatorH264ImplFHS(_MotionEstimatorBase):
    """GPU MotionEstimatorH264ImplFHS (src/CodecUtils/MotionEstimatorH264ImplFHS.cpp):
    the four-scale hexagon search from the median prediction on 80-point
    extrapolated path distortions with integer costs, its half / quarter-pel
    stages and the prediction check.  Constructor as the reference's
    (pSrc, pRef, w, h, motionRange, pMVPred[, pDistortionIncluded[, pPrevFrmMBlk]]);
    the previous-frame macroblocks are accepted and not read, as in the
    reference.  The predictor side effect carries the distortion:
    Set16x16MotionVector(k, x, y, d).  SetMode(0) quarter pel (the default),
    1 half, 2 full pel."""

    KIND = _lib.ME_FHS
    DEFAULT_MODE = 0

    def __init__(self, pSrc, pRef, imgWidth: int, imgHeight: int, motionRange: int = 64, pMVPred=None,
                 pDistortionIncluded=None, pPrevFrmMBlk=None, mb_slice=None, ctx: Context | None = None):
        super().__init__(pSrc, pRef, imgWidth, imgHeight, motionRange, pMVPred, pDistortionIncluded, mb_slice, ctx)

    def Estimate(self, *args, param: float | None = None, want_mb_distortion: bool = True):
        pred, self._pred = self._pred, None
        try:
            mv, avg = super().Estimate(*args, param=param, want_mb_distortion=True)
        finally:
            self._pred = pred
        if self._pred is not None:  # the reference hands the predictor each vector with its distortion
            d = self.last_mb_distortion
            for k in range(self.num_mbs()):
                self._pred.Set16x16MotionVector(k, int(mv[k, 0]), int(mv[k, 1]), int(d[k]))
        return mv, avg


class MotionEstimatorImpl1(_MotionEstimatorBase):
    """GPU MotionEstimatorImpl1 (src/CodecUtils/MotionEstimatorImpl1.cpp): constructor
    (pSrc, pRef, imgWidth, imgHeight, macroBlkWidth, macroBlkHeight, motionRange) as the
    reference's, blocks 16x16 or 8x8, motionRange in full pels (1..32).  Estimate()
    returns the half-pel vectors (the reference's SimpleMotionVectorList of chars)
    and avgDistortion over every block; no predictor."""

    KIND = _lib.ME_IMPL1
    DEFAULT_MODE = 0

    def __init__(self, pSrc, pRef, imgWidth: int, imgHeight: int, macroBlkWidth: int = 16,
                 macroBlkHeight: int = 16, motionRange: int = 16, ctx: Context | None = None):
        super().__init__(pSrc, pRef, imgWidth, imgHeight, motionRange, None, None, None, ctx)
        self._bw = int(macroBlkWidth)
        self._bh = int(macroBlkHeight)

    def Create(self) -> int:
        self._destroy()
        h = C.c_void_p()
        rc = load().vppgpu_me_create_blocks(self._ctx.handle, self.KIND, self._w, self._h, self._bw, self._bh,
                                            self._range, C.byref(h))
        if rc != _lib.OK:
            return 0
        self._h_me = h
        load().vppgpu_me_set_mode(self._h_me, self._mode)
        return 1

    def num_mbs(self) -> int:
        return (self._w // self._bw) * (self._h // self._bh)


class MotionEstimatorImpl2(MotionEstimatorImpl1):
    """GPU MotionEstimatorImpl2 (src/CodecUtils/MotionEstimatorImpl2.cpp): the SAD
    pyramid, 16x16 blocks, motionRange in full pels (4..32); SetMode(1) (the
    default) two levels, 2 three, 0 picks by area.  Half-pel vectors and
    avgDistortion over every block; no predictor."""

    KIND = _lib.ME_IMPL2
    DEFAULT_MODE = 1

    def GetMode(self) -> int:
        m = C.c_int(self._mode)
        if self._h_me:
            load().vppgpu_me_get_mode(self._h_me, C.byref(m))
        return m.value


class MotionEstimatorH264ImplMultiresCross(_MotionEstimatorBase):
    """GPU MotionEstimatorH264ImplMultiresCross (src/CodecUtils/MotionEstimatorH264ImplMultiresCross.cpp).
    No predictor; avgDistortion counts every macroblock (the partial bottom row
    too) when pDistortionIncluded is None, as the reference does."""

    KIND = _lib.ME_MULTIRES_CROSS

    def GetMode(self) -> int:
        if self._h_me:  # SetMode(0) resolves by picture area
            m = C.c_int()
            check(load().vppgpu_me_get_mode(self._h_me, C.byref(m)), "vppgpu_me_get_mode")
            return m.value
        return self._mode


class MotionEstimatorH263ImplMultiresCross(MotionEstimatorH264ImplMultiresCross):
    """GPU MotionEstimatorH263ImplMultiresCross
    (src/CodecUtils/MotionEstimatorH263ImplMultiresCross.cpp): the MultiresCross
    levels with the H.263 half-pel stage (OverlayMem2Dv2::HalfRead corners, then
    the points beside the winner); motionRange (at most 64) and the vectors in
    half pels."""

    KIND = _lib.ME_H263_MULTIRES_CROSS


class MotionEstimatorH263ImplMultiresCrossVer2(MotionEstimatorH264ImplMultiresCross):
    """GPU MotionEstimatorH263ImplMultiresCrossVer2
    (src/CodecUtils/MotionEstimatorH263ImplMultiresCrossVer2.cpp) with the
    H.263 median prediction of H263MotionVectorPredictorImpl1: the H.263
    MultiresCross search with ties towards the prediction, then the better of
    the clamped prediction and the zero vector against the searched vector;
    motionRange (at most 64) and vectors in half pels.  The prediction comes
    from the vectors the estimate writes, so pMVPred (an
    H263MotionVectorPredictorImpl1 in the reference, which only reads the
    vector list) is neither consulted nor written."""

    KIND = _lib.ME_H263_MULTIRES_CROSS_V2

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self._pred = None  # the reference sets no vectors on its predictor


class MotionEstimatorH264ImplMultires(MotionEstimatorH264ImplMultiresCross):
    """GPU MotionEstimatorH264ImplMultires (src/CodecUtils/MotionEstimatorH264ImplMultires.cpp):
    full searches at levels 2 and 1, +-2 at level 0, sub-pel, ties towards the
    prediction rounded to each level, the pred-vector check and GetBestVector
    (lambda 1.1).  The reference needs its pMVPred constructor argument."""

    KIND = _lib.ME_MULTIRES


class MotionEstimatorH264ImplMultiresCrossVer2(MotionEstimatorH264ImplMultiresCross):
    """GPU MotionEstimatorH264ImplMultiresCrossVer2
    (src/CodecUtils/MotionEstimatorH264ImplMultiresCrossVer2.cpp): the
    MultiresCross search with ties towards the median prediction, the
    pred-vector check and GetBestVector (lambda 0.9).  Estimate(param=lambda)
    is the Lagrangian overload (…MultiresCrossVer2.cpp:1162-1742):
    GetBestVector over the last five improvements of every search level,
    then the final choice with that lambda."""

    KIND = _lib.ME_MULTIRES_CROSS_V2


class MotionCompensatorH264ImplStd:
    """GPU MotionCompensatorH264ImplStd (src/CodecUtils/MotionCompensatorH264ImplStd.cpp):
    Create(ref, w, h) takes the contiguous 4:2:0 int16 frame (Y, U, V) and
    Compensate(vectors) replaces its macroblocks in place by the blocks the
    quarter-pel vectors point at, as the reference does."""

    def __init__(self, range_: int = 32, ctx: Context | None = None):
        self._range = int(range_)
        self._ctx = ctx or get_context()
        self._h = None
        self._ref = None

    def Create(self, ref, imgWidth: int, imgHeight: int, macroBlkWidth: int = 16, macroBlkHeight: int = 16) -> int:
        self._destroy()
        if macroBlkWidth != 16 or macroBlkHeight != 16:
            return 0
        h = C.c_void_p()
        if load().vppgpu_mc_create(self._ctx.handle, int(imgWidth), int(imgHeight), self._range, C.byref(h)) != _lib.OK:
            return 0
        self._h = h
        self._ref = ref
        self._w, self._hgt = int(imgWidth), int(imgHeight)
        return 1

    def Compensate(self, vectors) -> None:
        if not self._h:
            raise VppGpuError(_lib.ERR_NOT_READY, "Compensate before Create")
        if not (isinstance(self._ref, np.ndarray) and self._ref.dtype == np.int16 and self._ref.flags.c_contiguous):
            raise ValueError("the reference frame must be a contiguous int16 array (Y, U, V)")
        mv = np.ascontiguousarray(vectors, np.int16)
        check(load().vppgpu_mc_compensate(self._h, _ptr(self._ref), _ptr(mv)), "vppgpu_mc_compensate")

    def _destroy(self):
        if self._h and self._ctx.handle:  # as for the estimators
            load().vppgpu_mc_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self._destroy()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# 4x4 transforms
# ---------------------------------------------------------------------------
QUANT_ID = 0
INTRA_FLAG_ID = 1
TransformAndQuant, TransformOnly, QuantOnly = 0, 1, 2


class MotionEstimatorBatch:
    """Many independent frame pairs of mixed sizes in one call
    (vppgpu_me_batch_*; no vpp counterpart).  Jobs are tuples of device
    pointers: (src, ref, width, height, motion_range, mv_out[, mb_dist_out[,
    dist_included[, residual_out, levels_out, recon_out, qp]]]); the last four
    add the coding stage (residual at the vectors, T+Q at qp and its inverse).
    run() returns (statuses, avgDistortions)."""

    def __init__(self, streams: int = 4, kind: int = _lib.ME_FULL, ctx: Context | None = None):
        self._ctx = ctx or get_context()
        h = C.c_void_p()
        check(load().vppgpu_me_batch_create(self._ctx.handle, kind, int(streams), C.byref(h)), "vppgpu_me_batch_create")
        self.handle = h

    def run(self, jobs):
        n = len(jobs)
        arr = (_lib.MeJob * max(n, 1))()
        for i, j in enumerate(jobs):
            src, ref, w, hgt, mr, mv = j[:6]
            dist = j[6] if len(j) > 6 else None
            incl = j[7] if len(j) > 7 else None
            res, lev, rec, qp = j[8:12] if len(j) > 8 else (None, None, None, 0)
            arr[i] = _lib.MeJob(src, ref, w, hgt, mr, incl, mv, dist, res, lev, rec, qp)
        st = (C.c_int * max(n, 1))()
        avg = (C.c_long * max(n, 1))()
        rc = load().vppgpu_me_batch_run(self.handle, arr, n, st, avg)
        if rc != _lib.OK and not any(list(st)[:n]):  # refused as a whole (arguments, CUDA), not a job's status
            raise VppGpuError(rc, "vppgpu_me_batch_run")
        return list(st)[:n], list(avg)[:n]

    def launch_count(self) -> int:
        c = C.c_ulonglong()
        check(load().vppgpu_me_batch_launch_count(self.handle, C.byref(c)), "vppgpu_me_batch_launch_count")
        return c.value

    def close(self):
        if getattr(self, "handle", None) and self._ctx.handle:  # as for the estimators
            load().vppgpu_me_batch_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching request loop (vppgpu_server_*; no vpp counterpart).
    submit(frames[nframes, H, W] int16, motion_range, qp) -> ticket; the
    result arrays (vectors, digests) are filled when poll()/wait_idle() report
    the ticket done."""

    def __init__(self, slots: int = 4, hbm_budget: int = 0, ctx: Context | None = None):
        self._ctx = ctx or get_context()
        h = C.c_void_p()
        check(load().vppgpu_server_create(self._ctx.handle, int(slots), int(hbm_budget), C.byref(h)),
              "vppgpu_server_create")
        self.handle = h
        self._live = {}

    def prepare(self, width: int, height: int, motion_range: int = 128):
        check(load().vppgpu_server_prepare(self.handle, int(width), int(height), int(motion_range)),
              "vppgpu_server_prepare")

    def submit(self, frames, motion_range: int = 128, qp: int = 28, want_vectors: bool = True):
        f = np.ascontiguousarray(frames, np.int16)
        nfr, h, w = f.shape
        nmb = (w // 16) * (h // 16)
        mv = np.zeros((max(nfr - 1, 0), nmb, 2), np.int16) if want_vectors else None
        dig = np.zeros(max(nfr - 1, 0), np.uint64)
        req = _lib.SeqRequest(w, h, nfr, int(motion_range), int(qp), f.ctypes.data,
                              mv.ctypes.data if mv is not None else None, dig.ctypes.data)
        t = C.c_ulonglong()
        check(load().vppgpu_server_submit(self.handle, C.byref(req), C.byref(t)), "vppgpu_server_submit")
        self._live[t.value] = (f, mv, dig)  # keep the buffers alive until done
        return t.value, mv, dig

    def poll(self, max_n: int = 1024):
        tk = (C.c_ulonglong * max_n)()
        st = (C.c_int * max_n)()
        lat = (C.c_double * max_n)()
        n = C.c_int()
        check(load().vppgpu_server_poll(self.handle, max_n, tk, st, lat, C.byref(n)), "vppgpu_server_poll")
        out = []
        for i in range(n.value):
            self._live.pop(tk[i], None)
            out.append((tk[i], st[i], lat[i]))
        return out

    def wait_idle(self):
        check(load().vppgpu_server_wait_idle(self.handle), "vppgpu_server_wait_idle")

    def stats(self):
        b = C.c_ulonglong()
        r = C.c_int()
        check(load().vppgpu_server_stats(self.handle, C.byref(b), C.byref(r)), "vppgpu_server_stats")
        return {"reserved_peak_bytes": b.value, "running_peak": r.value}

    def close(self):
        if getattr(self, "handle", None) and self._ctx.handle:  # as for the estimators
            load().vppgpu_server_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _ForwardBase:
    LAYOUT = _lib.LAYOUT_BLOCKS
    UNIT = 16

    def __init__(self, ctx: Context | None = None):
        self._ctx = ctx or get_context()
        self._mode = TransformAndQuant
        self._intra = 1
        self._q = 1

    def SetMode(self, mode):
        self._mode = int(mode)

    def GetMode(self):
        return self._mode

    def SetParameter(self, paramID, paramVal):
        if paramID == QUANT_ID:
            self._q = int(paramVal)
        elif paramID == INTRA_FLAG_ID:
            self._intra = int(paramVal)

    def GetParameter(self, paramID):
        return self._q if paramID == QUANT_ID else self._intra

    def SetScale(self, pScale):
        pass

    def GetScale(self):
        return None

    def Transform(self, ptr, pCoeff=None):
        """In place on an int16 array holding a whole number of units, or
        Transform(pIn, pCoeff): copy then transform pCoeff."""
        if pCoeff is not None:
            np.copyto(pCoeff, ptr)
            ptr = pCoeff
        a = _as_units(ptr, self.UNIT)
        check(load().vppgpu_fwd4x4(self._ctx.handle, _ptr(a), a.size // self.UNIT, self.LAYOUT, self._mode, self._q,
                                   self._intra), "vppgpu_fwd4x4")
        if a is not ptr:
            np.copyto(ptr, a.reshape(ptr.shape))
        return ptr

    def QuantiseValue(self, val, pos, qp):
        self._q = int(qp)
        return load().vppgpu_quantise_value(int(val), int(pos), int(qp), self._intra)


class FastForward4x4ITImpl1(_ForwardBase):
    LAYOUT, UNIT = _lib.LAYOUT_BLOCKS, 16


class FastForward4x4ITImpl2(_ForwardBase):
    LAYOUT, UNIT = _lib.LAYOUT_BLOCKS, 16


class FastForward4x4On16x16ITImpl1(_ForwardBase):
    LAYOUT, UNIT = _lib.LAYOUT_MB16, 256


class _InverseBase:
    LAYOUT = _lib.LAYOUT_BLOCKS
    UNIT = 16

    def __init__(self, ctx: Context | None = None):
        self._ctx = ctx or get_context()
        self._mode = TransformAndQuant
        self._q = 1
        self._weight = np.full(16, 16, np.int32)

    def SetMode(self, mode):
        self._mode = int(mode)

    def GetMode(self):
        return self._mode

    def SetParameter(self, paramID, paramVal):
        if paramID == QUANT_ID:
            self._q = int(paramVal)

    def GetParameter(self, paramID):
        return self._q

    def SetScale(self, pScale):
        self._weight = np.ascontiguousarray(pScale, np.int32).reshape(16).copy()

    def GetScale(self):
        return self._weight

    def InverseTransform(self, ptr, pOut=None):
        if pOut is not None:
            np.copyto(pOut, ptr)
            ptr = pOut
        a = _as_units(ptr, self.UNIT)
        check(load().vppgpu_inv4x4(self._ctx.handle, _ptr(a), a.size // self.UNIT, self.LAYOUT, self._mode, self._q,
                                   _ptr(self._weight)), "vppgpu_inv4x4")
        if a is not ptr:
            np.copyto(ptr, a.reshape(ptr.shape))
        return ptr


class FastInverse4x4ITImpl1(_InverseBase):
    LAYOUT, UNIT = _lib.LAYOUT_BLOCKS, 16


class FastInverse4x4On16x16ITImpl1(_InverseBase):
    LAYOUT, UNIT = _lib.LAYOUT_MB16, 256


class _DcForwardBase:
    """The DC Hadamard forward transforms: Transform(ptr) on an int16 array of
    whole size*size blocks, in place, or Transform(pIn, pCoeff)."""
    SIZE = 4

    def __init__(self, ctx: Context | None = None):
        self._ctx = ctx or get_context()
        self._mode = TransformAndQuant
        self._q = 1

    def SetMode(self, mode):
        self._mode = int(mode)

    def GetMode(self):
        return self._mode

    def SetParameter(self, paramID, paramVal):
        if paramID == QUANT_ID:
            self._q = int(paramVal)

    def GetParameter(self, paramID):
        return self._q

    def SetScale(self, pScale):
        pass

    def GetScale(self):
        return None

    def Transform(self, ptr, pCoeff=None):
        if pCoeff is not None:
            np.copyto(pCoeff, ptr)
            ptr = pCoeff
        a = _as_units(ptr, self.SIZE * self.SIZE)
        check(load().vppgpu_fwd_dc(self._ctx.handle, _ptr(a), a.size // (self.SIZE * self.SIZE), self.SIZE,
                                   self._mode, self._q), "vppgpu_fwd_dc")
        if a is not ptr:
            np.copyto(ptr, a.reshape(ptr.shape))
        return ptr


class FastForwardDC4x4ITImpl1(_DcForwardBase):
    """Intra16x16 luma DC (src/CodecUtils/FastForwardDC4x4ITImpl1.cpp)."""
    SIZE = 4

    def QuantiseValue(self, val, pos, qp):
        self._q = int(qp)
        return load().vppgpu_dc_quantise_value(int(val), int(qp))


class FastForwardDC2x2ITImpl1(_DcForwardBase):
    """Chroma DC (src/CodecUtils/FastForwardDC2x2ITImpl1.cpp)."""
    SIZE = 2

    def QuantiseValue(self, val, pos, qp):
        return 0


class _DcInverseBase:
    SIZE = 4

    def __init__(self, ctx: Context | None = None):
        self._ctx = ctx or get_context()
        self._mode = TransformAndQuant
        self._q = 1
        self._weight = np.full(self.SIZE * self.SIZE, 16, np.int32)

    def SetMode(self, mode):
        self._mode = int(mode)

    def GetMode(self):
        return self._mode

    def SetParameter(self, paramID, paramVal):
        if paramID == QUANT_ID:
            self._q = int(paramVal)

    def GetParameter(self, paramID):
        return self._q

    def SetScale(self, pScale):
        self._weight = np.ascontiguousarray(pScale, np.int32).reshape(self.SIZE * self.SIZE).copy()

    def GetScale(self):
        return self._weight

    def InverseTransform(self, ptr, pOut=None):
        if pOut is not None:
            np.copyto(pOut, ptr)
            ptr = pOut
        a = _as_units(ptr, self.SIZE * self.SIZE)
        check(load().vppgpu_inv_dc(self._ctx.handle, _ptr(a), a.size // (self.SIZE * self.SIZE), self.SIZE,
                                   self._mode, self._q, _ptr(self._weight)), "vppgpu_inv_dc")
        if a is not ptr:
            np.copyto(ptr, a.reshape(ptr.shape))
        return ptr


class FastInverseDC4x4ITImpl1(_DcInverseBase):
    """Intra16x16 luma DC (src/CodecUtils/FastInverseDC4x4ITImpl1.cpp)."""
    SIZE = 4


class FastInverseDC2x2ITImpl1(_DcInverseBase):
    """Chroma DC (src/CodecUtils/FastInverseDC2x2ITImpl1.cpp)."""
    SIZE = 2


def _as_units(a, unit):
    if not isinstance(a, np.ndarray) or a.dtype != np.int16:
        raise TypeError("transform data must be an int16 numpy array")
    if a.size % unit:
        raise ValueError(f"transform data must hold a whole number of {unit}-sample units")
    return a if a.flags.c_contiguous else np.ascontiguousarray(a)


def tq_roundtrip_plane(residual, qp, intra, inv_order=_lib.INV_ROWS_FIRST, weight16=None, ctx=None):
    """Levels and reconstruction of a residual plane (BlockH264 forward + quant,
    dequant + inverse for every 4x4 block)."""
    ctx = ctx or get_context()
    res = np.ascontiguousarray(residual, np.int16)
    h, w = res.shape
    lev = np.empty_like(res)
    rec = np.empty_like(res)
    wt = None if weight16 is None else np.ascontiguousarray(weight16, np.int32)
    check(load().vppgpu_tq_roundtrip_plane(ctx.handle, _ptr(res), _ptr(lev), _ptr(rec), w, h, w, int(qp), int(intra),
                                           int(inv_order), _ptr(wt)), "vppgpu_tq_roundtrip_plane")
    return lev, rec


# ---------------------------------------------------------------------------
# Colour conversion
# ---------------------------------------------------------------------------
class FastGpuRGB24toYUV420Converter:
    """RGBtoYUV420Converter filled in on the GPU.  kind selects the arithmetic
    of FastFixedPointRGB24toYUV420Converter (default), RealRGB24toYUV420Converter
    or RealRGB24toYUV420ConverterImpl2."""

    def __init__(self, width=0, height=0, chrOff=0, kind=_lib.RGB_FIXED_POINT, ctx: Context | None = None):
        self._width, self._height, self._chrOff, self._flip = int(width), int(height), int(chrOff), False
        self._kind = int(kind)
        self._ctx = ctx or get_context()

    def GetWidth(self):
        return self._width

    def GetHeight(self):
        return self._height

    def GetChrominanceOffset(self):
        return self._chrOff

    def GetFlip(self):
        return self._flip

    def SetDimensions(self, width, height):
        self._width, self._height = int(width), int(height)

    def SetFlip(self, flip):
        self._flip = bool(flip)

    def SetChrominanceOffset(self, val):
        self._chrOff = int(val)

    def Convert(self, pRgb, pY, pU, pV):
        rgb = np.ascontiguousarray(pRgb, np.uint8)
        for p in (pY, pU, pV):
            if p.dtype != np.int16 or not p.flags.c_contiguous:
                raise TypeError("output planes must be contiguous int16 arrays")
        check(load().vppgpu_rgb24_to_yuv420(self._ctx.handle, self._kind, _ptr(rgb), self._width, self._height,
                                            self._chrOff, int(self._flip), _ptr(pY), _ptr(pU), _ptr(pV)),
              "vppgpu_rgb24_to_yuv420")


# ---------------------------------------------------------------------------
# YUV420 -> RGB24 (display side)
# ---------------------------------------------------------------------------
class _YUV420toRGB24Base:
    """YUV420toRGBConverter (include/ImageUtils/YUV420toRGBConverter.h) on the
    GPU: Convert(pY, pU, pV, pRgb) fills pRgb (uint8, width*height*3 packed
    B,G,R) from int16 planes.  KIND selects the reference class's arithmetic."""
    KIND = _lib.YUV_REAL_IMPL2

    def __init__(self, width=0, height=0, chrOff=0, ctx: Context | None = None):
        self._width, self._height, self._chrOff = int(width), int(height), int(chrOff)
        self._rotate, self._flip = 0, False
        self._ctx = ctx or get_context()

    def GetWidth(self):
        return self._width

    def GetHeight(self):
        return self._height

    def GetRotate(self):
        return self._rotate

    def GetChrominanceOffset(self):
        return self._chrOff

    def GetFlip(self):
        return self._flip

    def SetDimensions(self, width, height):
        self._width, self._height = int(width), int(height)

    def SetRotate(self, rotate):
        self._rotate = int(rotate)

    def SetChrominanceOffset(self, val):
        self._chrOff = int(val)

    def SetFlip(self, flip):
        self._flip = bool(flip)

    def Convert(self, pY, pU, pV, pRgb):
        for p in (pY, pU, pV):
            if not isinstance(p, np.ndarray) or p.dtype != np.int16 or not p.flags.c_contiguous:
                raise TypeError("input planes must be contiguous int16 arrays")
        if pRgb.dtype != np.uint8 or not pRgb.flags.c_contiguous or pRgb.size != self._width * self._height * 3:
            raise TypeError("pRgb must be a contiguous uint8 array of width*height*3 bytes")
        check(load().vppgpu_yuv420_to_rgb24(self._ctx.handle, self.KIND, _ptr(pY), _ptr(pU), _ptr(pV), self._width,
                                            self._height, self._chrOff, self._rotate, int(self._flip), _ptr(pRgb)),
              "vppgpu_yuv420_to_rgb24")


class RealYUV420toRGB24Converter(_YUV420toRGB24Base):
    """src/ImageUtils/RealYUV420toRGB24Converter.cpp (chrOff on the unrotated paths)."""
    KIND = _lib.YUV_REAL


class RealYUV420toRGB24ConverterImpl2(_YUV420toRGB24Base):
    """src/ImageUtils/RealYUV420toRGB24ConverterImpl2.cpp."""
    KIND = _lib.YUV_REAL_IMPL2


class RealYUV420toRGB24ConverterImpl2Ver16(_YUV420toRGB24Base):
    """src/ImageUtils/RealYUV420toRGB24ConverterImpl2Ver16.cpp (the Impl2 arithmetic)."""
    KIND = _lib.YUV_REAL_IMPL2


class RealYUV420toRGB24CCIR601Converter(_YUV420toRGB24Base):
    """src/ImageUtils/RealYUV420toRGB24CCIR601Converter.cpp (no flip)."""
    KIND = _lib.YUV_CCIR601


class RealYUV420toRGB24CCIR601ConverterVer16(_YUV420toRGB24Base):
    """src/ImageUtils/RealYUV420toRGB24CCIR601ConverterVer16.cpp (the CCIR601 arithmetic)."""
    KIND = _lib.YUV_CCIR601


class Fast6BitYUV420toRGB24Converter(_YUV420toRGB24Base):
    """src/ImageUtils/Fast6BitYUV420toRGB24Converter.cpp: 6-bit samples, integer
    terms; rotate only (the flip and the chrominance offset are not used)."""
    KIND = _lib.YUV_FAST_6BIT


class Real6BitYUV420toRGB24Converter(_YUV420toRGB24Base):
    """src/ImageUtils/Real6BitYUV420toRGB24Converter.cpp: 6-bit samples scaled by
    4, the Real double terms; rotate only."""
    KIND = _lib.YUV_REAL_6BIT


class Fast6BitYUV420toRGB24ZoomConverter(_YUV420toRGB24Base):
    """src/ImageUtils/Fast6BitYUV420toRGB24ZoomConverter.cpp: 6-bit planes of the
    constructor's size to an output of SetOutputDimensions' size (even sizes whose
    source positions stay inside the planes; rotation is not supported, as in the
    reference)."""

    def __init__(self, width=0, height=0, ctx: Context | None = None):
        super().__init__(width, height, 0, ctx)
        self._out_w, self._out_h = 1, 1

    def GetOutputWidth(self):
        return self._out_w

    def GetOutputHeight(self):
        return self._out_h

    def SetOutputDimensions(self, width, height):
        self._out_w, self._out_h = int(width), int(height)

    def Convert(self, pY, pU, pV, pRgb):
        if self._rotate:
            return  # the reference's Convert does nothing when rotated
        for p in (pY, pU, pV):
            if not isinstance(p, np.ndarray) or p.dtype != np.int16 or not p.flags.c_contiguous:
                raise TypeError("input planes must be contiguous int16 arrays")
        if pRgb.dtype != np.uint8 or not pRgb.flags.c_contiguous or pRgb.size != self._out_w * self._out_h * 3:
            raise TypeError("pRgb must be a contiguous uint8 array of out_width*out_height*3 bytes")
        check(load().vppgpu_yuv420_to_rgb24_zoom(self._ctx.handle, _ptr(pY), _ptr(pU), _ptr(pV), self._width,
                                                 self._height, self._out_w, self._out_h, _ptr(pRgb)),
              "vppgpu_yuv420_to_rgb24_zoom")
