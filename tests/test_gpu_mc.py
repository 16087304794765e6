"""GPU MotionCompensatorH264ImplStd (vppgpu_mc_*): the compensated 4:2:0 frame
bit-exact with the reference's golden fixtures and with the oracle on further
sizes; in-place host semantics and the device entry point with a separate
output; the add-with-clip and subtract plane helpers against the oracle; and
the encoder loop prediction + residual = input for a zero-quantisation step."""
import ctypes as C

import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = ["qcif_r16", "cif_r32", "small_r8"]


def compensate(vpp, ctx, y, u, v, mv, rg):
    h, w = y.shape
    yuv = np.concatenate([np.ravel(y), np.ravel(u), np.ravel(v)]).astype(np.int16)
    mc = vpp.MotionCompensatorH264ImplStd(rg, ctx=ctx)
    assert mc.Create(yuv, w, h) == 1
    mc.Compensate(mv)
    n, c = w * h, (w // 2) * (h // 2)
    return yuv[:n].reshape(h, w), yuv[n:n + c].reshape(h // 2, w // 2), yuv[n + c:].reshape(h // 2, w // 2)


@pytest.mark.parametrize("case", CASES)
def test_against_golden(vpp, ctx, golden, case):
    g = golden("mc.npz")
    w, h, rg = (int(v) for v in g[f"{case}_meta"])
    y, u, v = (g[f"{case}_{k}"].astype(np.int16) for k in ("y", "u", "v"))
    cy, cu, cv = compensate(vpp, ctx, y, u, v, g[f"{case}_mv"], rg)
    np.testing.assert_array_equal(cy, g[f"{case}_cy"])
    np.testing.assert_array_equal(cu, g[f"{case}_cu"])
    np.testing.assert_array_equal(cv, g[f"{case}_cv"])


@pytest.mark.parametrize("seed,w,h,rg", [(71, 1920, 1088, 32), (72, 208, 120, 24), (73, 640, 368, 16)])
def test_against_oracle(vpp, ctx, orc, seed, w, h, rg):
    y = synth.pan_sequence(seed, w, h, 1)[0]
    u = synth.pan_sequence(seed + 1, w // 2, h // 2, 1)[0]
    v = synth.pan_sequence(seed + 2, w // 2, h // 2, 1)[0]
    nmb = (w // 16) * (h // 16)
    mv = ((synth.splitmix64(seed, 2 * nmb) % np.uint64(8 * rg + 1)).astype(np.int64) - 4 * rg).astype(np.int16)
    mv = mv.reshape(nmb, 2)
    got = compensate(vpp, ctx, y, u, v, mv, rg)
    for a, b in zip(got, orc.mc_compensate(y, u, v, mv, rg)):
        np.testing.assert_array_equal(a, b)


def test_device_entry_and_plane_helpers(vpp, ctx, orc):
    """Device compensation into a separate frame, then residual = input - prediction
    and reconstruction = clip(prediction + residual) == input."""
    torch = pytest.importorskip("torch")
    from imagecodingutils_gb300 import _lib
    L = vpp.load()
    dev = torch.device("cuda", 0)
    w, h, rg = 352, 288, 32
    fr = synth.pan_sequence(74, w, h, 2)
    u = synth.pan_sequence(75, w // 2, h // 2, 1)[0]
    v = synth.pan_sequence(76, w // 2, h // 2, 1)[0]
    mv_o, _, _ = orc.me_full(fr[1], fr[0], 128)
    ref = torch.from_numpy(np.concatenate([fr[0].ravel(), u.ravel(), v.ravel()]).astype(np.int16)).to(dev)
    pred = torch.empty_like(ref)
    mv = torch.from_numpy(mv_o).to(dev)
    mc = C.c_void_p()
    _lib.check(L.vppgpu_mc_create(ctx.handle, w, h, rg, C.byref(mc)), "create")
    _lib.check(L.vppgpu_mc_compensate_device(mc, C.c_void_p(ref.data_ptr()), C.c_void_p(mv.data_ptr()),
                                             C.c_void_p(pred.data_ptr())), "compensate")
    ctx.synchronize()
    oy, ou, ov = orc.mc_compensate(fr[0], u, v, mv_o, rg)
    n = w * h
    np.testing.assert_array_equal(pred[:n].cpu().numpy().reshape(h, w), oy)
    np.testing.assert_array_equal(pred[n:].cpu().numpy(), np.concatenate([ou.ravel(), ov.ravel()]))
    np.testing.assert_array_equal(ref.cpu().numpy()[:n].reshape(h, w), fr[0])  # input untouched
    # residual of the luma and back
    inp = torch.from_numpy(fr[1].astype(np.int16).ravel()).to(dev)
    res = inp.clone()
    _lib.check(L.vppgpu_sub_device(ctx.handle, C.c_void_p(res.data_ptr()), C.c_void_p(pred.data_ptr()), n), "sub")
    rec = pred[:n].clone()
    _lib.check(L.vppgpu_add_clip255_device(ctx.handle, C.c_void_p(rec.data_ptr()), C.c_void_p(res.data_ptr()), n),
               "add")
    ctx.synchronize()
    np.testing.assert_array_equal(res.cpu().numpy(), orc.sub(fr[1].ravel(), oy.ravel()))
    np.testing.assert_array_equal(rec.cpu().numpy(), fr[1].ravel())
    # odd length: the tail path of the plane helpers
    a = torch.from_numpy(np.arange(-500, 499, dtype=np.int16)).to(dev)
    b = torch.from_numpy(np.full(999, 37, np.int16)).to(dev)
    ah = a.cpu().numpy()
    _lib.check(L.vppgpu_add_clip255_device(ctx.handle, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), 999), "add")
    ctx.synchronize()
    np.testing.assert_array_equal(a.cpu().numpy(), orc.add_clip255(ah, np.full(999, 37, np.int16)))
    L.vppgpu_mc_destroy(mc)
