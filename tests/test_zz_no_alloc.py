"""The allocation-free full-search entry point against the allocating one.

vppgpu_me_full_estimate_noalloc serves callers that cannot allocate device
memory while running; it keeps all of its intermediate buffers in a fixed
static device array.  This test calls it through the C ABI twice in a row on
different frames (the second call reuses the array the first one left
behind) and checks vectors, per-macroblock distortions and the average
against the ordinary entry point, bit for bit.  Collected last so that a run
stopping at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu


def _p(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_matches_allocating_entry_point(vpp):
    torch = pytest.importorskip("torch")
    L = vpp.load()
    w, h, mr = 352, 288, 128
    nmb = (w // 16) * (h // 16)
    for seed in (5, 6):  # two calls in a row
        fr = synth.pan_sequence(900 + seed, w, h, 2)
        incl = (synth.splitmix64(seed, nmb) % np.uint64(4) != 0).astype(np.uint8)
        d_src = torch.from_numpy(fr[1]).cuda()
        d_ref = torch.from_numpy(fr[0]).cuda()
        d_incl = torch.from_numpy(incl).cuda()
        d_mv = torch.full((nmb, 2), -7, dtype=torch.int16, device="cuda")
        d_dist = torch.full((nmb,), -7, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        avg = C.c_long(-1)
        rc = L.vppgpu_me_full_estimate_noalloc(_p(d_src), _p(d_ref), w, h, mr, _p(d_incl), None, _p(d_mv),
                                               _p(d_dist), C.byref(avg), None)
        assert rc == 0, vpp._lib.status_string(rc)

        me = vpp.MotionEstimatorH264ImplFull(fr[1], fr[0], w, h, mr, pDistortionIncluded=incl)
        assert me.Create() == 1
        mv_ref, avg_ref = me.Estimate()
        np.testing.assert_array_equal(d_mv.cpu().numpy(), mv_ref)
        np.testing.assert_array_equal(d_dist.cpu().numpy(), me.last_mb_distortion)
        assert avg.value == avg_ref


def test_noalloc_rejects_frames_beyond_its_limit(vpp):
    torch = pytest.importorskip("torch")
    L = vpp.load()
    w, h = 640, 480  # 1200 macroblocks > VPPGPU_NOALLOC_MAX_MBS
    buf = torch.zeros((h, w), dtype=torch.int16, device="cuda")
    mv = torch.zeros((1200, 2), dtype=torch.int16, device="cuda")
    rc = L.vppgpu_me_full_estimate_noalloc(_p(buf), _p(buf), w, h, 128, None, None, _p(mv), None, None, None)
    assert rc == vpp._lib.ERR_UNSUPPORTED
