"""Motion-compensated luma residual (vppgpu_me_residual_device) against the
CPU oracle: for every macroblock, input minus the reference's QuarterRead at
the estimated vector (the reference's MotionCompensatorH264ImplStd luma path
followed by Sub16x16)."""
import ctypes as C

import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed,w,h", [(81, 176, 144), (82, 352, 288), (83, 208, 120)])
def test_residual_matches_oracle(vpp, ctx, orc, seed, w, h):
    torch = pytest.importorskip("torch")
    from imagecodingutils_gb300 import _lib
    L = vpp.load()
    dev = torch.device("cuda", 0)
    fr = synth.pan_sequence(seed, w, h, 2)
    cols, rows = w // 16, h // 16
    nmb = cols * rows
    src = torch.from_numpy(fr[1]).to(dev)
    ref = torch.from_numpy(fr[0]).to(dev)
    mv = torch.zeros((nmb, 2), dtype=torch.int16, device=dev)
    res = torch.zeros((h, w), dtype=torch.int16, device=dev)
    me = C.c_void_p()
    _lib.check(L.vppgpu_me_create(ctx.handle, _lib.ME_FULL, w, h, 128, C.byref(me)), "create")
    _lib.check(L.vppgpu_me_estimate_device(me, C.c_void_p(src.data_ptr()), C.c_void_p(ref.data_ptr()), None, None,
                                           C.c_void_p(mv.data_ptr()), None, None), "estimate")
    _lib.check(L.vppgpu_me_residual_device(me, C.c_void_p(mv.data_ptr()), C.c_void_p(res.data_ptr())), "residual")
    ctx.synchronize()
    mvh, resh = mv.cpu().numpy(), res.cpu().numpy()
    mv_o, _, _ = orc.me_full(fr[1], fr[0], 128)
    np.testing.assert_array_equal(mvh, mv_o)
    for k in range(nmb):
        n, m = (k % cols) * 16, (k // cols) * 16
        vx, vy = int(mvh[k, 0]), int(mvh[k, 1])
        qx, qy = int(np.fmod(vx, 4)), int(np.fmod(vy, 4))    # C remainders
        px, py = int((vx - qx) // 4), int((vy - qy) // 4)     # C quotients
        pred = orc.quarter_read16(fr[0], n + px, m + py, qx, qy)
        want = fr[1][m:m + 16, n:n + 16].astype(np.int32) - pred.astype(np.int32)
        np.testing.assert_array_equal(resh[m:m + 16, n:n + 16], want, err_msg=f"MB {k} vector {vx},{vy}")
    L.vppgpu_me_destroy(me)


def test_residual_given_vectors_and_out_of_range(vpp, ctx, orc):
    """Vectors chosen by the caller: in range they give the oracle's residual;
    a prediction more than 32 samples outside the picture gives a zero block
    and VPPGPU_ERR_UNSUPPORTED from vppgpu_me_last_status."""
    torch = pytest.importorskip("torch")
    from imagecodingutils_gb300 import _lib
    L = vpp.load()
    dev = torch.device("cuda", 0)
    w, h = 176, 144
    fr = synth.pan_sequence(84, w, h, 2)
    cols, rows = w // 16, h // 16
    nmb = cols * rows
    rng = np.random.default_rng(84)
    mvh = rng.integers(-64, 65, size=(nmb, 2)).astype(np.int16)  # within 16 samples
    far = [3, 40, 77]
    mvh[far[0]] = (-4 * 200, 0)
    mvh[far[1]] = (0, 4 * 300)
    mvh[far[2]] = (4 * 33 + 4 * w, 0)
    src = torch.from_numpy(fr[1]).to(dev)
    ref = torch.from_numpy(fr[0]).to(dev)
    scratch = torch.zeros((nmb, 2), dtype=torch.int16, device=dev)
    mv = torch.from_numpy(mvh).to(dev)
    res = torch.full((h, w), 7, dtype=torch.int16, device=dev)
    me = C.c_void_p()
    _lib.check(L.vppgpu_me_create(ctx.handle, _lib.ME_FULL, w, h, 128, C.byref(me)), "create")
    _lib.check(L.vppgpu_me_estimate_device(me, C.c_void_p(src.data_ptr()), C.c_void_p(ref.data_ptr()), None, None,
                                           C.c_void_p(scratch.data_ptr()), None, None), "estimate")
    assert L.vppgpu_me_last_status(me) == 0
    _lib.check(L.vppgpu_me_residual_device(me, C.c_void_p(mv.data_ptr()), C.c_void_p(res.data_ptr())), "residual")
    ctx.synchronize()
    assert L.vppgpu_me_last_status(me) == -6
    resh = res.cpu().numpy()
    for k in range(nmb):
        n, m = (k % cols) * 16, (k // cols) * 16
        if k in far:
            assert not resh[m:m + 16, n:n + 16].any()
            continue
        vx, vy = int(mvh[k, 0]), int(mvh[k, 1])
        qx, qy = int(np.fmod(vx, 4)), int(np.fmod(vy, 4))
        px, py = int((vx - qx) // 4), int((vy - qy) // 4)
        pred = orc.quarter_read16(fr[0], n + px, m + py, qx, qy)
        want = fr[1][m:m + 16, n:n + 16].astype(np.int32) - pred.astype(np.int32)
        np.testing.assert_array_equal(resh[m:m + 16, n:n + 16], want, err_msg=f"MB {k} vector {vx},{vy}")
    L.vppgpu_me_destroy(me)
