"""GPU parity at the headline size, pinned to the reference itself: every
estimator on three frame pairs of the 1920x1080 benchmark sequence at
motionRange 128 against tests/golden/me_1080p.npz, which the compiled
reference produced (vectors and avgDistortion with every macroblock included;
the integer-pel SAD stage also per-macroblock SADs).  The frames are
regenerated by the seeded generator and checked against the fixture's SHA-256.
The device estimators also run through vppgpu_me_estimate_device on resident
frames (the benchmark's own call), which must give the host call's vectors."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CLASSES = {"full": "MotionEstimatorH264ImplFull", "multires_cross": "MotionEstimatorH264ImplMultiresCross",
           "multires_cross_v2": "MotionEstimatorH264ImplMultiresCrossVer2",
           "multires": "MotionEstimatorH264ImplMultires", "cross": "MotionEstimatorH264ImplCross",
           "full_sad": "MotionEstimatorH264ImplFullSad"}
ESTIMATORS = [("full", 1), ("multires_cross", 0), ("multires_cross", 1), ("multires_cross", 2),
              ("multires_cross_v2", 0), ("multires_cross_v2", 1), ("multires_cross_v2", 2),
              ("multires", 0), ("multires", 1), ("multires", 2), ("cross", 0), ("full_sad", None)]


def fixture_key(pair, kind, mode):
    return f"p{pair}_{kind}" + ("" if mode is None else f"_m{mode}")


@pytest.mark.parametrize("kind,mode", ESTIMATORS)
def test_against_reference_1080p(vpp, ctx, hd_golden, kind, mode):
    g, fr, w, h, mr = (hd_golden[k] for k in ("g", "frames", "w", "h", "motion_range"))
    incl = np.ones((w // 16) * (h // 16), np.uint8)
    for t in hd_golden["pairs"]:
        key = fixture_key(t, kind, mode)
        me = getattr(vpp, CLASSES[kind])(fr[t + 1], fr[t], w, h, mr, pDistortionIncluded=incl, ctx=ctx)
        assert me.Create() == 1
        if mode is not None:
            me.SetMode(mode)
        mv, avg = me.Estimate()
        np.testing.assert_array_equal(mv, g[f"{key}_mv"], err_msg=key)
        assert avg == int(g[f"{key}_avg"][0]), key
        if kind == "full_sad":
            np.testing.assert_array_equal(me.last_mb_distortion, g[f"{key}_dist"], err_msg=key)


def test_device_call_matches_reference_1080p(vpp, ctx, hd_golden):
    """vppgpu_me_estimate_device on resident frames, the form the benchmark
    times, for the full-search estimator over the three pairs in sequence on one
    handle (its captured graph replayed)."""
    torch = pytest.importorskip("torch")
    from imagecodingutils_gb300 import _lib
    L = vpp.load()
    g, fr, w, h, mr = (hd_golden[k] for k in ("g", "frames", "w", "h", "motion_range"))
    dev = torch.from_numpy(np.stack(fr)).cuda()
    nmb = (w // 16) * (h // 16)
    d_mv = torch.empty((nmb, 2), dtype=torch.int16, device="cuda")
    handle = C.c_void_p()
    _lib.check(L.vppgpu_me_create(ctx.handle, _lib.ME_FULL, w, h, mr, C.byref(handle)), "vppgpu_me_create")
    try:
        for t in list(hd_golden["pairs"]) * 2:
            torch.cuda.synchronize()
            _lib.check(L.vppgpu_me_estimate_device(handle, C.c_void_p(dev[t + 1].data_ptr()),
                                                   C.c_void_p(dev[t].data_ptr()), None, None,
                                                   C.c_void_p(d_mv.data_ptr()), None, None),
                       "vppgpu_me_estimate_device")
            ctx.synchronize()
            np.testing.assert_array_equal(d_mv.cpu().numpy(), g[f"p{t}_full_m1_mv"])
    finally:
        L.vppgpu_me_destroy(handle)
