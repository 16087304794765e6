"""ctypes binding of the C ABI in ``include/vppgpu.h`` (``lib/libvppgpu.so``).

There is no CPU fallback: if the library is missing or no GB300 is present the
calls raise.  ``build()`` (or ``__graft_entry__.build()``) compiles it.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libvppgpu.so")

_P = C.c_void_p
_I = C.c_int
_LL = C.c_longlong

# status codes (include/vppgpu.h)
OK = 0
ERR_INVALID_ARG = -1
ERR_CUDA = -2
ERR_OUT_OF_MEMORY = -3
ERR_PIXEL_RANGE = -4
ERR_TIMEOUT = -5
ERR_UNSUPPORTED = -6
ERR_NOT_READY = -7
ERR_NO_DEVICE = -8

ME_FULL, ME_MULTIRES, ME_MULTIRES_CROSS, ME_MULTIRES_CROSS_V2, ME_CROSS, ME_H263_MULTIRES_CROSS = 0, 1, 2, 3, 4, 5
ME_FULL_SAD = 6
ME_UMHS = 7
ME_FHS = 8
ME_IMPL1 = 9
ME_IMPL2 = 10
ME_H263_MULTIRES_CROSS_V2 = 11
LAYOUT_BLOCKS, LAYOUT_MB16 = 0, 1
INV_ROWS_FIRST, INV_COLS_FIRST = 0, 1
RGB_FIXED_POINT, RGB_REAL, RGB_REAL_IMPL2 = 0, 1, 2
YUV_REAL, YUV_REAL_IMPL2, YUV_CCIR601, YUV_FAST_6BIT, YUV_REAL_6BIT = 0, 1, 2, 3, 4

# name -> (restype, argtypes); the symbol list is also the export check of the tests
SIGNATURES = {
    "vppgpu_status_string": (C.c_char_p, [_I]),
    "vppgpu_ctx_create": (_I, [_I, C.POINTER(_P)]),
    "vppgpu_ctx_destroy": (_I, [_P]),
    "vppgpu_ctx_set_stream": (_I, [_P, _P]),
    "vppgpu_ctx_get_stream": (_I, [_P, C.POINTER(_P)]),
    "vppgpu_ctx_synchronize": (_I, [_P]),
    "vppgpu_ctx_launch_count": (_I, [_P, C.POINTER(C.c_ulonglong)]),
    "vppgpu_me_create": (_I, [_P, _I, _I, _I, _I, C.POINTER(_P)]),
    "vppgpu_me_create_blocks": (_I, [_P, _I, _I, _I, _I, _I, _I, C.POINTER(_P)]),
    "vppgpu_me_destroy": (_I, [_P]),
    "vppgpu_me_set_mode": (_I, [_P, _I]),
    "vppgpu_me_get_mode": (_I, [_P, C.POINTER(_I)]),
    "vppgpu_me_num_mbs": (_I, [_P, C.POINTER(_I)]),
    "vppgpu_me_estimate": (_I, [_P, _P, _P, _P, _P, _P, _P, C.POINTER(C.c_long)]),
    "vppgpu_me_estimate_device": (_I, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "vppgpu_me_estimate_lambda": (_I, [_P, _P, _P, _P, _P, C.c_double, _P, _P, C.POINTER(C.c_long)]),
    "vppgpu_me_set_prev_frame": (_I, [_P, _P, _P]),
    "vppgpu_me_last_status": (_I, [_P]),
    "vppgpu_me_set_relax_sweeps": (_I, [_P, _I]),
    "vppgpu_me_autotune": (_I, [_P, _P, _P, _I, C.POINTER(_I)]),
    "vppgpu_me_get_tuning": (_I, [_P, _P]),
    "vppgpu_me_autotune_host": (_I, [_P, _P, _P, _I, C.POINTER(_I)]),
    "vppgpu_me_autotune_pairs": (_I, [_P, _P, _P, _I, _I, C.POINTER(_I)]),
    "vppgpu_me_last_sweeps": (_I, [_P, C.POINTER(_I)]),
    "vppgpu_me_last_stats": (_I, [_P, _P]),
    "vppgpu_me_last_relax_changes": (_I, [_P, _P, _I]),
    "vppgpu_me_set_timing": (_I, [_P, _I]),
    "vppgpu_me_timing": (_I, [_P, C.POINTER(_I), C.POINTER(C.c_double), C.POINTER(C.c_double),
                              C.POINTER(C.c_double)]),
    "vppgpu_me_timing_stages": (_I, [_P, C.POINTER(_I), _P]),
    "vppgpu_me_residual_device": (_I, [_P, _P, _P]),
    "vppgpu_mc_create": (_I, [_P, _I, _I, _I, C.POINTER(_P)]),
    "vppgpu_mc_destroy": (_I, [_P]),
    "vppgpu_mc_compensate": (_I, [_P, _P, _P]),
    "vppgpu_mc_compensate_device": (_I, [_P, _P, _P, _P]),
    "vppgpu_add_clip255_device": (_I, [_P, _P, _P, C.c_longlong]),
    "vppgpu_sub_device": (_I, [_P, _P, _P, C.c_longlong]),
    "vppgpu_server_create": (_I, [_P, _I, C.c_ulonglong, C.POINTER(_P)]),
    "vppgpu_server_prepare": (_I, [_P, _I, _I, _I]),
    "vppgpu_server_submit": (_I, [_P, _P, C.POINTER(C.c_ulonglong)]),
    "vppgpu_server_poll": (_I, [_P, _I, _P, _P, _P, C.POINTER(_I)]),
    "vppgpu_server_wait_idle": (_I, [_P]),
    "vppgpu_server_stats": (_I, [_P, C.POINTER(C.c_ulonglong), C.POINTER(_I)]),
    "vppgpu_server_destroy": (_I, [_P]),
    "vppgpu_me_batch_create": (_I, [_P, _I, _I, C.POINTER(_P)]),
    "vppgpu_me_batch_destroy": (_I, [_P]),
    "vppgpu_me_batch_run": (_I, [_P, _P, _I, _P, _P]),
    "vppgpu_me_batch_launch_count": (_I, [_P, C.POINTER(C.c_ulonglong)]),
    "vppgpu_calibrate_dp4a": (_I, [_P, C.POINTER(C.c_double)]),
    "vppgpu_me_full_estimate_noalloc": (_I, [_P, _P, _I, _I, _I, _P, _P, _P, _P, C.POINTER(C.c_long), _P]),
    "vppgpu_fwd4x4": (_I, [_P, _P, _LL, _I, _I, _I, _I]),
    "vppgpu_fwd4x4_device": (_I, [_P, _P, _LL, _I, _I, _I, _I]),
    "vppgpu_inv4x4": (_I, [_P, _P, _LL, _I, _I, _I, _P]),
    "vppgpu_inv4x4_device": (_I, [_P, _P, _LL, _I, _I, _I, _P]),
    "vppgpu_tq_roundtrip_plane": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P]),
    "vppgpu_tq_roundtrip_plane_device": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P]),
    "vppgpu_tq_roundtrip_planes_device": (_I, [_P, _P, _I, _I, _P]),
    "vppgpu_quantise_value": (_I, [C.c_short, _I, _I, _I]),
    "vppgpu_fwd_dc": (_I, [_P, _P, _LL, _I, _I, _I]),
    "vppgpu_fwd_dc_device": (_I, [_P, _P, _LL, _I, _I, _I]),
    "vppgpu_inv_dc": (_I, [_P, _P, _LL, _I, _I, _I, _P]),
    "vppgpu_inv_dc_device": (_I, [_P, _P, _LL, _I, _I, _I, _P]),
    "vppgpu_dc_quantise_value": (_I, [C.c_short, _I]),
    "vppgpu_rgb24_to_yuv420": (_I, [_P, _I, _P, _I, _I, _I, _I, _P, _P, _P]),
    "vppgpu_rgb24_to_yuv420_device": (_I, [_P, _I, _P, _I, _I, _I, _I, _P, _P, _P]),
    "vppgpu_rgb24_to_yuv420_frames_device": (_I, [_P, _I, _P, _I, _I, _I, _I, _I, _P, _P, _P]),
    "vppgpu_yuv420_to_rgb24": (_I, [_P, _I, _P, _P, _P, _I, _I, _I, _I, _I, _P]),
    "vppgpu_yuv420_to_rgb24_device": (_I, [_P, _I, _P, _P, _P, _I, _I, _I, _I, _I, _P]),
    "vppgpu_yuv420_to_rgb24_frames_device": (_I, [_P, _I, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P]),
    "vppgpu_yuv420_to_rgb24_zoom": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _P]),
    "vppgpu_yuv420_to_rgb24_zoom_device": (_I, [_P, _P, _P, _P, _I, _I, _I, _I, _P]),
}

_lib = None


class VppGpuError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {status_string(status)} ({status})")


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} not built; run imagecodingutils_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(s: int) -> str:
    try:
        return load().vppgpu_status_string(s).decode()
    except Exception:  # the library may be absent when formatting a load error
        return "unknown"


def check(status: int, what: str) -> None:
    if status != OK:
        raise VppGpuError(status, what)


class MeJob(C.Structure):
    """vppgpu_me_job (include/vppgpu.h)."""
    _fields_ = [("src", C.c_void_p), ("ref", C.c_void_p), ("width", C.c_int), ("height", C.c_int),
                ("motion_range", C.c_int), ("dist_included", C.c_void_p), ("mv_out", C.c_void_p),
                ("mb_dist_out", C.c_void_p), ("residual_out", C.c_void_p), ("levels_out", C.c_void_p),
                ("recon_out", C.c_void_p), ("qp", C.c_int)]


class SeqRequest(C.Structure):
    """vppgpu_seq_request (include/vppgpu.h)."""
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("nframes", C.c_int), ("motion_range", C.c_int),
                ("qp", C.c_int), ("frames", C.c_void_p), ("mv_out", C.c_void_p), ("digest_out", C.c_void_p)]
