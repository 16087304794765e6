"""ctypes access to the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/liboracle.so`` (the plain-C restatement of the reference hot
path) and, where it was built, ``oracle/_ref/libvppref.so`` (the reference's
own C++ sources compiled unmodified, driven through ``ref_harness.cpp``).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this module; the product path never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libvppref.so")
# Where the reference's sources lie: VPP_REFERENCE_TREE, else the build
# container's checkout (absent on other hosts: the reference build and the
# tests that need it are then skipped).
REF_TREE = os.environ.get("VPP_REFERENCE_TREE", "/root/reference")

_P = C.c_void_p
_I = C.c_int
_L = C.c_long


def build(with_reference: bool | None = None, jobs: int = 8) -> None:
    """Compile the oracle (and the reference library when its tree exists)."""
    subprocess.run(["make", "-s", "-C", HERE, f"-j{jobs}", "liboracle.so"], check=True)
    if with_reference is None:
        with_reference = os.path.isdir(os.path.join(REF_TREE, "src"))
    if with_reference:
        subprocess.run(["make", "-s", "-C", HERE, f"-j{jobs}", "ref", f"REF={REF_TREE}"], check=True)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


class Oracle:
    """The C restatement."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build(with_reference=False)
        self.lib = C.CDLL(path)
        L = self.lib
        L.vo_num_mbs.argtypes = [_I, _I]
        L.vo_me_full.argtypes = [_P, _P, _I, _I, _I, _P, _P, _P, _P, C.POINTER(_L)]
        L.vo_me_full_detail.argtypes = [_P, _P, _I, _I, _I, _P, _P, _P, _P, C.POINTER(_L)] + [_P] * 6
        L.vo_me_full_intpel.argtypes = [_P, _P, _I, _I, _I, _I, _P, _P]
        L.vo_me_multires_cross.argtypes = [_P, _P, _I, _I, _I, _I, _P, _P, _P, C.POINTER(_L)]
        L.vo_me_h263_multires_cross.argtypes = [_P, _P, _I, _I, _I, _I, _P, _P, _P, C.POINTER(_L)]
        L.vo_me_h263_multires_cross_ver2.argtypes = [_P, _P, _I, _I, _I, _I, _P, _P, _P, C.POINTER(_L)]
        L.vo_me_multires_cross_v2.argtypes = [_P, _P, _I, _I, _I, _I, _P, _P, _P, _P, C.POINTER(_L), _P]
        L.vo_me_cross.argtypes = [_P, _P, _I, _I, _I, _I, _P, _P, _P, _P, C.POINTER(_L), _P]
        L.vo_me_multires.argtypes = [_P, _P, _I, _I, _I, _I, _P, _P, _P, _P, C.POINTER(_L), _P]
        L.vo_me_multires_cross_v2_lambda.argtypes = [_P, _P, _I, _I, _I, _I, C.c_double, _P, _P, _P, _P,
                                                     C.POINTER(_L)]
        L.vo_me_umhs.argtypes = [_P, _P, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, C.POINTER(_L)]
        L.vo_me_impl2.argtypes = [_P, _P, _I, _I, _I, _I, _P, _P, C.POINTER(_L)]
        L.vo_me_impl1.argtypes = [_P, _P, _I, _I, _I, _I, _I, _P, _P, C.POINTER(_L)]
        L.vo_me_fhs.argtypes = [_P, _P, _I, _I, _I, _I, _P, _P, _P, _P, C.POINTER(_L), C.POINTER(_I)]
        L.vo_mc_compensate.argtypes = [_P, _I, _I, _I, _P]
        L.vo_add_clip255.argtypes = [_P, _P, C.c_longlong]
        L.vo_sub.argtypes = [_P, _P, C.c_longlong]
        L.vo_quarter_read16.argtypes = [_P, _I, _I, _I, _I, _I, _I, _P]
        L.vo_half.argtypes = [_P, _I, _I, _P]
        L.vo_fwd4x4.argtypes = [_P, _I, _I, _I, _I, _I]
        L.vo_inv4x4.argtypes = [_P, _I, _I, _I, _I, _P]
        L.vo_quantise_value.argtypes = [C.c_short, _I, _I, _I]
        L.vo_fwd_dc.argtypes = [_P, _I, _I, _I, _I]
        L.vo_inv_dc.argtypes = [_P, _I, _I, _I, _I, _P]
        L.vo_dc_quantise_value.argtypes = [C.c_short, _I]
        L.vo_yuv420_to_rgb24.argtypes = [_I, _P, _P, _P, _I, _I, _I, _I, _I, _P]
        L.vo_yuv420_to_rgb24_6bit.argtypes = [_I, _P, _P, _P, _I, _I, _I, _P]
        L.vo_yuv420_to_rgb24_zoom.argtypes = [_P, _P, _P, _I, _I, _I, _I, _P]
        L.vo_rgb24_to_yuv420.argtypes = [_I, _P, _I, _I, _I, _I, _P, _P, _P]
        L.vo_bench_me_full.argtypes = [_P, _P, _I, _I, _I, _I, _I, _P]

    def me_full(self, src, ref, motion_range, dist_incl=None, slice_map=None, detail=False):
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        nmb = self.lib.vo_num_mbs(w, h)
        mv = np.zeros((nmb, 2), np.int16)
        dist = np.zeros(nmb, np.int32)
        avg = _L(0)
        incl = None if dist_incl is None else np.ascontiguousarray(dist_incl, dtype=np.uint8)
        sl = None if slice_map is None else np.ascontiguousarray(slice_map, dtype=np.int32)
        if not detail:
            rc = self.lib.vo_me_full(_ptr(src), _ptr(ref), w, h, motion_range, _ptr(incl), _ptr(sl),
                                     _ptr(mv), _ptr(dist), C.byref(avg))
            if rc:
                raise ValueError(f"vo_me_full rc={rc}")
            return mv, dist, avg.value
        extra = {k: np.zeros((nmb, 2) if k.endswith("mv") else nmb, np.int32)
                 for k in ("int_mv", "sub_mv", "min_d", "zero_d", "pred_mv", "pred_d")}
        rc = self.lib.vo_me_full_detail(_ptr(src), _ptr(ref), w, h, motion_range, _ptr(incl), _ptr(sl),
                                        _ptr(mv), _ptr(dist), C.byref(avg),
                                        *[_ptr(extra[k]) for k in ("int_mv", "sub_mv", "min_d", "zero_d",
                                                                   "pred_mv", "pred_d")])
        if rc:
            raise ValueError(f"vo_me_full_detail rc={rc}")
        return mv, dist, avg.value, extra

    def me_h263_multires_cross(self, src, ref, motion_range, mode=1, dist_incl=None):
        """MotionEstimatorH263ImplMultiresCross: motion range and vectors in half pels."""
        return self.me_multires_cross(src, ref, motion_range, mode, dist_incl, _fn=self.lib.vo_me_h263_multires_cross)

    def me_h263_multires_cross_ver2(self, src, ref, motion_range, mode=1, dist_incl=None):
        """MotionEstimatorH263ImplMultiresCrossVer2 with the H.263 median predictor: half pels."""
        return self.me_multires_cross(src, ref, motion_range, mode, dist_incl,
                                      _fn=self.lib.vo_me_h263_multires_cross_ver2)

    def me_multires_cross(self, src, ref, motion_range, mode=1, dist_incl=None, _fn=None):
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        nmb = self.lib.vo_num_mbs(w, h)
        mv = np.zeros((nmb, 2), np.int16)
        dist = np.zeros(nmb, np.int32)
        avg = _L(0)
        incl = None if dist_incl is None else np.ascontiguousarray(dist_incl, dtype=np.uint8)
        rc = (_fn or self.lib.vo_me_multires_cross)(_ptr(src), _ptr(ref), w, h, motion_range, mode, _ptr(incl),
                                                    _ptr(mv), _ptr(dist), C.byref(avg))
        if rc:
            raise ValueError(f"vo_me_multires_cross rc={rc}")
        return mv, dist, avg.value

    def me_multires(self, src, ref, motion_range, mode=1, dist_incl=None, slice_map=None, with_ties=False):
        return self._me_pred(self.lib.vo_me_multires, src, ref, motion_range, mode, dist_incl, slice_map, with_ties)

    def me_multires_cross_v2(self, src, ref, motion_range, mode=1, dist_incl=None, slice_map=None,
                             with_ties=False):
        return self._me_pred(self.lib.vo_me_multires_cross_v2, src, ref, motion_range, mode, dist_incl, slice_map,
                             with_ties)

    def me_multires_cross_v2_lambda(self, src, ref, motion_range, lam, mode=1, dist_incl=None, slice_map=None):
        """Ver2's Estimate(long*, void* lambda): GetBestVector at every level."""
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        nmb = self.lib.vo_num_mbs(w, h)
        mv = np.zeros((nmb, 2), np.int16)
        dist = np.zeros(nmb, np.int32)
        avg = _L(0)
        incl = None if dist_incl is None else np.ascontiguousarray(dist_incl, dtype=np.uint8)
        sl = None if slice_map is None else np.ascontiguousarray(slice_map, dtype=np.int32)
        rc = self.lib.vo_me_multires_cross_v2_lambda(_ptr(src), _ptr(ref), w, h, motion_range, mode, float(lam),
                                                     _ptr(incl), _ptr(sl), _ptr(mv), _ptr(dist), C.byref(avg))
        if rc:
            raise ValueError(f"vo_me_multires_cross_v2_lambda rc={rc}")
        return mv, dist, avg.value

    def me_cross(self, src, ref, motion_range, mode=0, dist_incl=None, slice_map=None, with_ties=False):
        """MotionEstimatorH264ImplCross (mode 0 quarter, 1 half, 2 full pel)."""
        return self._me_pred(self.lib.vo_me_cross, src, ref, motion_range, mode, dist_incl, slice_map, with_ties)

    def me_umhs(self, src, ref, motion_range, mode=0, dist_incl=None, slice_map=None, prev_mv=None,
                prev_intra=None):
        """MotionEstimatorH264ImplUMHS: vectors, the distortion stored with each, the average."""
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        nmb = self.lib.vo_num_mbs(w, h)
        mv = np.zeros((nmb, 2), np.int16)
        dist = np.zeros(nmb, np.int32)
        avg = _L(0)
        incl = None if dist_incl is None else np.ascontiguousarray(dist_incl, dtype=np.uint8)
        sl = None if slice_map is None else np.ascontiguousarray(slice_map, dtype=np.int32)
        pmv = None if prev_mv is None else np.ascontiguousarray(prev_mv, dtype=np.int16)
        pin = None if prev_intra is None else np.ascontiguousarray(prev_intra, dtype=np.uint8)
        rc = self.lib.vo_me_umhs(_ptr(src), _ptr(ref), w, h, motion_range, mode, _ptr(incl), _ptr(sl), _ptr(pmv),
                                 _ptr(pin), _ptr(mv), _ptr(dist), C.byref(avg))
        if rc:
            raise ValueError(f"vo_me_umhs rc={rc}")
        return mv, dist, avg.value

    def me_fhs(self, src, ref, motion_range, mode=0, dist_incl=None, slice_map=None, with_stale=False):
        """MotionEstimatorH264ImplFHS: vectors, the distortion stored with each, the
        average (and the number of stale sub-pel cache reads replaced)."""
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        nmb = self.lib.vo_num_mbs(w, h)
        mv = np.zeros((nmb, 2), np.int16)
        dist = np.zeros(nmb, np.int32)
        avg = _L(0)
        stale = _I(0)
        incl = None if dist_incl is None else np.ascontiguousarray(dist_incl, dtype=np.uint8)
        sl = None if slice_map is None else np.ascontiguousarray(slice_map, dtype=np.int32)
        rc = self.lib.vo_me_fhs(_ptr(src), _ptr(ref), w, h, motion_range, mode, _ptr(incl), _ptr(sl), _ptr(mv),
                                _ptr(dist), C.byref(avg), C.byref(stale))
        if rc:
            raise ValueError(f"vo_me_fhs rc={rc}")
        return (mv, dist, avg.value, stale.value) if with_stale else (mv, dist, avg.value)

    def me_impl2(self, src, ref, range_, mode=1):
        """MotionEstimatorImpl2: half-pel vectors, per-block distortion, the average."""
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        n = (w // 16) * (h // 16)
        mv = np.zeros((n, 2), np.int16)
        dist = np.zeros(n, np.int32)
        avg = _L(0)
        rc = self.lib.vo_me_impl2(_ptr(src), _ptr(ref), w, h, range_, mode, _ptr(mv), _ptr(dist), C.byref(avg))
        if rc:
            raise ValueError(f"vo_me_impl2 rc={rc}")
        return mv, dist, avg.value

    def me_impl1(self, src, ref, range_, bw=16, bh=16):
        """MotionEstimatorImpl1: half-pel vectors, per-block distortion, the average."""
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        n = (w // bw) * (h // bh)
        mv = np.zeros((n, 2), np.int16)
        dist = np.zeros(n, np.int32)
        avg = _L(0)
        rc = self.lib.vo_me_impl1(_ptr(src), _ptr(ref), w, h, bw, bh, range_, _ptr(mv), _ptr(dist), C.byref(avg))
        if rc:
            raise ValueError(f"vo_me_impl1 rc={rc}")
        return mv, dist, avg.value

    def _me_pred(self, fn, src, ref, motion_range, mode, dist_incl, slice_map, with_ties):
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        nmb = self.lib.vo_num_mbs(w, h)
        mv = np.zeros((nmb, 2), np.int16)
        dist = np.zeros(nmb, np.int32)
        ties = np.zeros(nmb, np.int32)
        avg = _L(0)
        incl = None if dist_incl is None else np.ascontiguousarray(dist_incl, dtype=np.uint8)
        sl = None if slice_map is None else np.ascontiguousarray(slice_map, dtype=np.int32)
        rc = fn(_ptr(src), _ptr(ref), w, h, motion_range, mode, _ptr(incl), _ptr(sl), _ptr(mv), _ptr(dist),
                C.byref(avg), _ptr(ties))
        if rc:
            raise ValueError(f"{fn.__name__} rc={rc}")
        return (mv, dist, avg.value, ties) if with_ties else (mv, dist, avg.value)

    def mc_compensate(self, y, u, v, mv, range_):
        """MotionCompensatorH264ImplStd::Compensate: the compensated (y, u, v) planes."""
        h, w = y.shape
        yuv = np.concatenate([np.ravel(y), np.ravel(u), np.ravel(v)]).astype(np.int16)
        mvs = np.ascontiguousarray(mv, dtype=np.int16)
        rc = self.lib.vo_mc_compensate(_ptr(yuv), w, h, range_, _ptr(mvs))
        if rc:
            raise ValueError(f"vo_mc_compensate rc={rc}")
        n, c = w * h, (w // 2) * (h // 2)
        return yuv[:n].reshape(h, w), yuv[n:n + c].reshape(h // 2, w // 2), yuv[n + c:].reshape(h // 2, w // 2)

    def add_clip255(self, a, b):
        out = np.array(a, dtype=np.int16, copy=True, order="C")
        bb = np.ascontiguousarray(b, dtype=np.int16)
        self.lib.vo_add_clip255(_ptr(out), _ptr(bb), out.size)
        return out

    def sub(self, a, b):
        out = np.array(a, dtype=np.int16, copy=True, order="C")
        bb = np.ascontiguousarray(b, dtype=np.int16)
        self.lib.vo_sub(_ptr(out), _ptr(bb), out.size)
        return out

    def me_full_intpel(self, src, ref, motion_range, metric=1):
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        nmb = self.lib.vo_num_mbs(w, h)
        mv = np.zeros((nmb, 2), np.int16)
        dist = np.zeros(nmb, np.int32)
        rc = self.lib.vo_me_full_intpel(_ptr(src), _ptr(ref), w, h, motion_range, metric, _ptr(mv), _ptr(dist))
        if rc:
            raise ValueError(f"vo_me_full_intpel rc={rc}")
        return mv, dist

    def quarter_read16(self, plane, x, y, qx, qy):
        h, w = plane.shape
        plane = np.ascontiguousarray(plane, dtype=np.int16)
        out = np.zeros((16, 16), np.int16)
        self.lib.vo_quarter_read16(_ptr(plane), w, h, x, y, qx, qy, _ptr(out))
        return out

    def half(self, plane):
        h, w = plane.shape
        plane = np.ascontiguousarray(plane, dtype=np.int16)
        out = np.zeros((h // 2, w // 2), np.int16)
        self.lib.vo_half(_ptr(plane), w, h, _ptr(out))
        return out

    def fwd4x4(self, data, layout, mode, qp, intra):
        d = np.array(data, dtype=np.int16, copy=True, order="C")
        unit = 16 if layout == 0 else 256
        self.lib.vo_fwd4x4(_ptr(d), d.size // unit, layout, mode, qp, intra)
        return d

    def inv4x4(self, data, layout, mode, qp, weight=None):
        d = np.array(data, dtype=np.int16, copy=True, order="C")
        unit = 16 if layout == 0 else 256
        wt = None if weight is None else np.ascontiguousarray(weight, dtype=np.int32)
        self.lib.vo_inv4x4(_ptr(d), d.size // unit, layout, mode, qp, _ptr(wt))
        return d

    def quantise_value(self, val, pos, qp, intra):
        return self.lib.vo_quantise_value(int(val), pos, qp, intra)

    def fwd_dc(self, data, size, mode, qp):
        """size 4: FastForwardDC4x4ITImpl1, size 2: FastForwardDC2x2ITImpl1, on
        contiguous size*size blocks."""
        d = np.array(data, dtype=np.int16, copy=True, order="C")
        self.lib.vo_fwd_dc(_ptr(d), d.size // (size * size), size, mode, qp)
        return d

    def inv_dc(self, data, size, mode, qp, weight=None):
        d = np.array(data, dtype=np.int16, copy=True, order="C")
        wt = None if weight is None else np.ascontiguousarray(weight, dtype=np.int32)
        self.lib.vo_inv_dc(_ptr(d), d.size // (size * size), size, mode, qp, _ptr(wt))
        return d

    def dc_quantise_value(self, val, qp):
        return self.lib.vo_dc_quantise_value(int(val), qp)

    def yuv_to_rgb(self, kind, y, u, v, chr_off=-128, rotate=0, flip=0):
        """kind 0 RealYUV420toRGB24Converter, 1 ...Impl2, 2 ...CCIR601; packed
        B,G,R bytes (height, width, 3), or (width, height, 3) when rotated."""
        h, w = y.shape
        y, u, v = (np.ascontiguousarray(a, dtype=np.int16) for a in (y, u, v))
        out = np.zeros((w, h, 3) if rotate and not (kind != 2 and flip) else (h, w, 3), np.uint8)
        self.lib.vo_yuv420_to_rgb24(kind, _ptr(y), _ptr(u), _ptr(v), w, h, chr_off, rotate, flip, _ptr(out))
        return out

    def yuv_to_rgb_6bit(self, kind, y, u, v, rotate=0):
        """kind 3 Fast6BitYUV420toRGB24Converter, 4 Real6BitYUV420toRGB24Converter
        (no flip or chrominance offset): (height, width, 3), or transposed."""
        h, w = y.shape
        y, u, v = (np.ascontiguousarray(a, dtype=np.int16) for a in (y, u, v))
        out = np.zeros((w, h, 3) if rotate else (h, w, 3), np.uint8)
        self.lib.vo_yuv420_to_rgb24_6bit(kind, _ptr(y), _ptr(u), _ptr(v), w, h, rotate, _ptr(out))
        return out

    def yuv_to_rgb_zoom(self, y, u, v, out_w, out_h):
        """Fast6BitYUV420toRGB24ZoomConverter to out_h x out_w x 3."""
        h, w = y.shape
        y, u, v = (np.ascontiguousarray(a, dtype=np.int16) for a in (y, u, v))
        out = np.zeros((out_h, out_w, 3), np.uint8)
        if self.lib.vo_yuv420_to_rgb24_zoom(_ptr(y), _ptr(u), _ptr(v), w, h, out_w, out_h, _ptr(out)):
            raise ValueError("output size outside the zoom converter's range")
        return out

    def rgb_to_yuv(self, kind, bgr, chr_off=0, flip=0):
        h, w, _ = bgr.shape
        bgr = np.ascontiguousarray(bgr, dtype=np.uint8)
        y = np.zeros((h, w), np.int16)
        u = np.zeros((h // 2, w // 2), np.int16)
        v = np.zeros((h // 2, w // 2), np.int16)
        rc = self.lib.vo_rgb24_to_yuv420(kind, _ptr(bgr), w, h, chr_off, flip, _ptr(y), _ptr(u), _ptr(v))
        if rc:
            raise ValueError(f"vo_rgb24_to_yuv420 rc={rc}")
        return y, u, v

    def bench_me_full(self, srcs, refs, motion_range, nthreads):
        h, w = srcs[0].shape
        n = len(srcs)
        keep = [np.ascontiguousarray(a, dtype=np.int16) for a in list(srcs) + list(refs)]
        sp = (_P * n)(*[k.ctypes.data for k in keep[:n]])
        rp = (_P * n)(*[k.ctypes.data for k in keep[n:]])
        mv = np.zeros((n, self.lib.vo_num_mbs(w, h), 2), np.int16)
        rc = self.lib.vo_bench_me_full(sp, rp, n, w, h, motion_range, nthreads, _ptr(mv))
        if rc:
            raise ValueError(f"vo_bench_me_full rc={rc}")
        return mv


class Reference:
    """The reference's own C++ classes (only where oracle/_ref was built)."""

    KIND = {"full": 0, "multires": 1, "multires_cross": 2, "multires_cross_v2": 3, "cross": 4,
            "h263_multires_cross": 5, "h263_multires_cross_v2": 6}

    def __init__(self, path: str = REF_SO):
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_me_estimate.argtypes = [_I, _P, _P, _I, _I, _I, _I, _P, _P, _I, _P, C.POINTER(_L)]
        L.ref_me_full_sad.argtypes = [_P, _P, _I, _I, _I, _P, _P, _P, C.POINTER(_L)]
        L.ref_me_umhs.argtypes = [_P, _P, _I, _I, _I, _I, _P, _P, _P, _P, _P, C.POINTER(_L)]
        L.ref_me_impl2.argtypes = [_P, _P, _I, _I, _I, _I, _P, C.POINTER(_L)]
        L.ref_me_impl1.argtypes = [_P, _P, _I, _I, _I, _I, _I, _P, C.POINTER(_L)]
        L.ref_me_fhs.argtypes = [_P, _P, _I, _I, _I, _I, _P, _P, _P, C.POINTER(_L)]
        L.ref_fwd_transform.argtypes = [_I, _P, _I, _I, _I, _I]
        L.ref_inv_transform.argtypes = [_I, _P, _I, _I, _I, _P]
        L.ref_quantise_value.argtypes = [C.c_short, _I, _I, _I]
        L.ref_fwd_dc.argtypes = [_P, _I, _I, _I, _I]
        L.ref_inv_dc.argtypes = [_P, _I, _I, _I, _I, _P]
        L.ref_dc_quantise_value.argtypes = [C.c_short, _I]
        L.ref_yuv_to_rgb.argtypes = [_I, _P, _P, _P, _I, _I, _I, _I, _I, _P]
        L.ref_yuv_to_rgb_zoom.argtypes = [_P, _P, _P, _I, _I, _I, _I, _P]
        L.ref_rgb_to_yuv.argtypes = [_I, _P, _I, _I, _I, _I, _P, _P, _P]
        L.ref_mc_compensate.argtypes = [_I, _I, _I, _P, _P]

    @staticmethod
    def available(path: str = REF_SO) -> bool:
        return os.path.exists(path)

    def me(self, kind, src, ref, motion_range, mode=1, dist_incl=None, lam=None, repeat=1):
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        nmb = (w // 16) * (h // 16)
        mv = np.zeros((nmb, 2), np.int16)
        avg = _L(0)
        incl = None if dist_incl is None else np.ascontiguousarray(dist_incl, dtype=np.uint8)
        lamv = None if lam is None else np.array([lam], np.float64)
        rc = self.lib.ref_me_estimate(self.KIND[kind], _ptr(src), _ptr(ref), w, h, motion_range, mode,
                                      _ptr(incl), _ptr(lamv), repeat, _ptr(mv), C.byref(avg))
        if rc:
            raise ValueError(f"ref_me_estimate rc={rc}")
        return mv, avg.value

    def me_full_sad(self, src, ref, motion_range, dist_incl=None):
        """The integer-pel SAD stage of MotionEstimatorH264ImplFull on the
        reference's own overlays (ref_harness.cpp FullSadStage): vectors, SADs
        and the included-distortion average."""
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        nmb = (w // 16) * (h // 16)
        mv = np.zeros((nmb, 2), np.int16)
        dist = np.zeros(nmb, np.int32)
        avg = _L(0)
        incl = None if dist_incl is None else np.ascontiguousarray(dist_incl, dtype=np.uint8)
        rc = self.lib.ref_me_full_sad(_ptr(src), _ptr(ref), w, h, motion_range, _ptr(incl), _ptr(mv), _ptr(dist),
                                      C.byref(avg))
        if rc:
            raise ValueError(f"ref_me_full_sad rc={rc}")
        return mv, dist, avg.value

    def me_umhs(self, src, ref, motion_range, mode=0, dist_incl=None, prev_mv=None, prev_intra=None):
        """MotionEstimatorH264ImplUMHS (eight-argument constructor): vectors, the
        distortion stored with each for the predictor, the average."""
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        nmb = (w // 16) * (h // 16)
        mv = np.zeros((nmb, 2), np.int16)
        dist = np.zeros(nmb, np.int32)
        avg = _L(0)
        incl = None if dist_incl is None else np.ascontiguousarray(dist_incl, dtype=np.uint8)
        pmv = None if prev_mv is None else np.ascontiguousarray(prev_mv, dtype=np.int16)
        pin = None if prev_intra is None else np.ascontiguousarray(prev_intra, dtype=np.uint8)
        rc = self.lib.ref_me_umhs(_ptr(src), _ptr(ref), w, h, motion_range, mode, _ptr(incl), _ptr(pmv), _ptr(pin),
                                  _ptr(mv), _ptr(dist), C.byref(avg))
        if rc:
            raise ValueError(f"ref_me_umhs rc={rc}")
        return mv, dist, avg.value

    def me_impl2(self, src, ref, range_, mode=1):
        """MotionEstimatorImpl2 after SetMode(mode): half-pel vectors and avgDistortion."""
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        n = (w // 16) * (h // 16)
        mv = np.zeros((n, 2), np.int16)
        avg = _L(0)
        rc = self.lib.ref_me_impl2(_ptr(src), _ptr(ref), w, h, range_, mode, _ptr(mv), C.byref(avg))
        if rc:
            raise ValueError(f"ref_me_impl2 rc={rc}")
        return mv, avg.value

    def me_impl1(self, src, ref, range_, bw=16, bh=16):
        """MotionEstimatorImpl1: half-pel vectors and avgDistortion."""
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        n = (w // bw) * (h // bh)
        mv = np.zeros((n, 2), np.int16)
        avg = _L(0)
        rc = self.lib.ref_me_impl1(_ptr(src), _ptr(ref), w, h, bw, bh, range_, _ptr(mv), C.byref(avg))
        if rc:
            raise ValueError(f"ref_me_impl1 rc={rc}")
        return mv, avg.value

    def me_fhs(self, src, ref, motion_range, mode=0, dist_incl=None):
        """MotionEstimatorH264ImplFHS: vectors, the distortion stored with each, the average."""
        h, w = src.shape
        src = np.ascontiguousarray(src, dtype=np.int16)
        ref = np.ascontiguousarray(ref, dtype=np.int16)
        nmb = (w // 16) * (h // 16)
        mv = np.zeros((nmb, 2), np.int16)
        dist = np.zeros(nmb, np.int32)
        avg = _L(0)
        incl = None if dist_incl is None else np.ascontiguousarray(dist_incl, dtype=np.uint8)
        rc = self.lib.ref_me_fhs(_ptr(src), _ptr(ref), w, h, motion_range, mode, _ptr(incl), _ptr(mv), _ptr(dist),
                                 C.byref(avg))
        if rc:
            raise ValueError(f"ref_me_fhs rc={rc}")
        return mv, dist, avg.value

    def mc_compensate(self, y, u, v, mv, range_):
        h, w = y.shape
        yuv = np.concatenate([np.ravel(y), np.ravel(u), np.ravel(v)]).astype(np.int16)
        mvs = np.ascontiguousarray(mv, dtype=np.int16)
        rc = self.lib.ref_mc_compensate(w, h, range_, _ptr(yuv), _ptr(mvs))
        if rc:
            raise ValueError(f"ref_mc_compensate rc={rc}")
        n, c = w * h, (w // 2) * (h // 2)
        return yuv[:n].reshape(h, w), yuv[n:n + c].reshape(h // 2, w // 2), yuv[n + c:].reshape(h // 2, w // 2)

    def fwd(self, impl, data, mode, qp, intra):
        d = np.array(data, dtype=np.int16, copy=True, order="C")
        unit = 256 if impl == 2 else 16
        self.lib.ref_fwd_transform(impl, _ptr(d), d.size // unit, mode, qp, intra)
        return d

    def inv(self, impl, data, mode, qp, weight=None):
        d = np.array(data, dtype=np.int16, copy=True, order="C")
        unit = 256 if impl == 1 else 16
        wt = None if weight is None else np.ascontiguousarray(weight, dtype=np.int32)
        self.lib.ref_inv_transform(impl, _ptr(d), d.size // unit, mode, qp, _ptr(wt))
        return d

    def quantise_value(self, val, pos, qp, intra):
        return self.lib.ref_quantise_value(int(val), pos, qp, intra)

    def fwd_dc(self, data, size, mode, qp):
        d = np.array(data, dtype=np.int16, copy=True, order="C")
        self.lib.ref_fwd_dc(_ptr(d), d.size // (size * size), size, mode, qp)
        return d

    def inv_dc(self, data, size, mode, qp, weight=None):
        d = np.array(data, dtype=np.int16, copy=True, order="C")
        wt = None if weight is None else np.ascontiguousarray(weight, dtype=np.int32)
        self.lib.ref_inv_dc(_ptr(d), d.size // (size * size), size, mode, qp, _ptr(wt))
        return d

    def dc_quantise_value(self, val, qp):
        return self.lib.ref_dc_quantise_value(int(val), qp)

    def yuv_to_rgb(self, kind, y, u, v, chr_off=-128, rotate=0, flip=0):
        """kind 0..2 as Oracle.yuv_to_rgb; 3 Impl2Ver16, 4 CCIR601Ver16."""
        h, w = y.shape
        y, u, v = (np.ascontiguousarray(a, dtype=np.int16) for a in (y, u, v))
        out = np.zeros((w, h, 3) if rotate and not (kind not in (2, 4) and flip) else (h, w, 3), np.uint8)
        rc = self.lib.ref_yuv_to_rgb(kind, _ptr(y), _ptr(u), _ptr(v), w, h, chr_off, rotate, flip, _ptr(out))
        if rc:
            raise ValueError(f"ref_yuv_to_rgb rc={rc}")
        return out

    def yuv_to_rgb_6bit(self, kind, y, u, v, rotate=0):
        """kind 3 Fast6BitYUV420toRGB24Converter, 4 Real6BitYUV420toRGB24Converter."""
        h, w = y.shape
        y, u, v = (np.ascontiguousarray(a, dtype=np.int16) for a in (y, u, v))
        out = np.zeros((w, h, 3) if rotate else (h, w, 3), np.uint8)
        rc = self.lib.ref_yuv_to_rgb(kind + 2, _ptr(y), _ptr(u), _ptr(v), w, h, 0, rotate, 0, _ptr(out))
        if rc:
            raise ValueError(f"ref_yuv_to_rgb rc={rc}")
        return out

    def yuv_to_rgb_zoom(self, y, u, v, out_w, out_h):
        """Fast6BitYUV420toRGB24ZoomConverter to out_h x out_w x 3."""
        h, w = y.shape
        y, u, v = (np.ascontiguousarray(a, dtype=np.int16) for a in (y, u, v))
        out = np.zeros((out_h, out_w, 3), np.uint8)
        self.lib.ref_yuv_to_rgb_zoom(_ptr(y), _ptr(u), _ptr(v), w, h, out_w, out_h, _ptr(out))
        return out

    def rgb_to_yuv(self, kind, bgr, chr_off=0, flip=0):
        h, w, _ = bgr.shape
        bgr = np.ascontiguousarray(bgr, dtype=np.uint8)
        y = np.zeros((h, w), np.int16)
        u = np.zeros((h // 2, w // 2), np.int16)
        v = np.zeros((h // 2, w // 2), np.int16)
        self.lib.ref_rgb_to_yuv(kind, _ptr(bgr), w, h, chr_off, flip, _ptr(y), _ptr(u), _ptr(v))
        return y, u, v
