"""The allocation-free full-search entry point against the allocating one.

vppgpu_me_full_estimate_noalloc serves callers that cannot allocate device
memory while running (an encoder with a device budget fixed at start-up, a
plugin whose host owns every allocation); it keeps all of its intermediate
buffers in a fixed static device array.  This test calls it through the C ABI
twice in a row on different frames (the second call reuses the array the first
one left behind) and checks vectors, per-macroblock distortions and the
average against the ordinary entry point and the CPU oracle, bit for bit; a
further call repeating the second one must leave the device's free memory
unchanged.  Frames at the size limits are accepted and checked, frames past
them refused.  Collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu


def _p(t):
    return C.c_void_p(t.data_ptr())


def _noalloc(L, torch, fr, w, h, mr, incl):
    nmb = (w // 16) * (h // 16)
    d_src = torch.from_numpy(fr[1]).cuda()
    d_ref = torch.from_numpy(fr[0]).cuda()
    d_incl = torch.from_numpy(incl).cuda()
    d_mv = torch.full((nmb, 2), -7, dtype=torch.int16, device="cuda")
    d_dist = torch.full((nmb,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    avg = C.c_long(-1)
    free0 = torch.cuda.mem_get_info()[0]
    rc = L.vppgpu_me_full_estimate_noalloc(_p(d_src), _p(d_ref), w, h, mr, _p(d_incl), None, _p(d_mv), _p(d_dist),
                                           C.byref(avg), None)
    free1 = torch.cuda.mem_get_info()[0]
    return rc, d_mv.cpu().numpy(), d_dist.cpu().numpy(), avg.value, free0 - free1


def test_noalloc_matches_allocating_entry_point(vpp, orc):
    torch = pytest.importorskip("torch")
    L = vpp.load()
    w, h, mr = 352, 288, 128
    nmb = (w // 16) * (h // 16)
    for seed in (5, 6, 6):  # two calls in a row on different frames, then the second repeated
        fr = synth.pan_sequence(900 + seed, w, h, 2)
        incl = (synth.splitmix64(seed, nmb) % np.uint64(4) != 0).astype(np.uint8)
        rc, mv, dist, avg, used = _noalloc(L, torch, fr, w, h, mr, incl)
        assert rc == 0, vpp._lib.status_string(rc)

        me = vpp.MotionEstimatorH264ImplFull(fr[1], fr[0], w, h, mr, pDistortionIncluded=incl)
        assert me.Create() == 1
        mv_ref, avg_ref = me.Estimate()
        np.testing.assert_array_equal(mv, mv_ref)
        np.testing.assert_array_equal(dist, me.last_mb_distortion)
        assert avg == avg_ref
        mv_o, dist_o, avg_o = orc.me_full(fr[1], fr[0], mr, dist_incl=incl)
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(dist, dist_o)
        assert avg == avg_o
        del me
    # the repeated call ran the kernels the call before it had loaded: it took no device memory
    assert used == 0, f"the allocation-free call took {used} bytes of device memory"


@pytest.mark.parametrize("w,h", [(1024, 96), (16, 1024), (1024, 16)])
def test_noalloc_at_its_size_limits(vpp, orc, w, h):
    """Frames as wide or as tall as VPPGPU_NOALLOC_MAX_DIM (the wavefront
    record bound of the array's layout) against the oracle."""
    torch = pytest.importorskip("torch")
    L = vpp.load()
    fr = synth.pan_sequence(77 + w + h, w, h, 2)
    incl = np.ones((w // 16) * (h // 16), np.uint8)
    rc, mv, dist, avg, _ = _noalloc(L, torch, fr, w, h, 128, incl)
    assert rc == 0, vpp._lib.status_string(rc)
    mv_o, dist_o, avg_o = orc.me_full(fr[1], fr[0], 128, dist_incl=incl)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)
    assert avg == avg_o


@pytest.mark.parametrize("w,h,mr,want", [(640, 480, 128, "ERR_UNSUPPORTED"),   # 1200 macroblocks > 396
                                         (1040, 16, 128, "ERR_UNSUPPORTED"),   # 65 macroblocks, wider than 1024
                                         (16, 1040, 128, "ERR_UNSUPPORTED"),   # taller than 1024
                                         (176, 144, 3, "ERR_INVALID_ARG"),     # below one full pel
                                         (176, 144, 132, "ERR_UNSUPPORTED")])  # beyond +-31 pels
def test_noalloc_rejects_what_it_cannot_hold(vpp, w, h, mr, want):
    torch = pytest.importorskip("torch")
    L = vpp.load()
    buf = torch.zeros((h, w), dtype=torch.int16, device="cuda")
    nmb = max(1, (w // 16) * (h // 16))
    mv = torch.zeros((nmb, 2), dtype=torch.int16, device="cuda")
    rc = L.vppgpu_me_full_estimate_noalloc(_p(buf), _p(buf), w, h, mr, None, None, _p(mv), None, None, None)
    assert rc == getattr(vpp._lib, want)
