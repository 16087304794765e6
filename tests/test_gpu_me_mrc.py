"""GPU MotionEstimatorH264ImplMultiresCross parity: vectors and avgDistortion
bit-exact with the reference's golden fixtures (modes 0/1/2, with and without
pDistortionIncluded, a partial bottom row), and vectors, per-macroblock
distortions and averages bit-exact with the CPU oracle on further seeded
sizes and ranges."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = ["qcif_r64", "cif_r128", "partial_r128", "small_r32"]


def estimate(vpp, ctx, src, ref, mr, mode, incl=None):
    h, w = src.shape
    me = vpp.MotionEstimatorH264ImplMultiresCross(src, ref, w, h, mr, pDistortionIncluded=incl, ctx=ctx)
    assert me.Create() == 1
    me.SetMode(mode)
    mv, avg = me.Estimate()
    return mv, me.last_mb_distortion, avg, me


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_against_golden(vpp, ctx, golden, case, mode):
    g = golden("me_mrc.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    mv, _, avg, me = estimate(vpp, ctx, src, ref, mr, mode)
    np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"])
    assert avg == int(g[f"{case}_m{mode}_avg"][0])
    if mode == 0:
        assert me.GetMode() == (2 if w * h > 40000 else 1)
    nmb = (w // 16) * (h // 16)
    mvi, _, avgi, _ = estimate(vpp, ctx, src, ref, mr, mode, np.ones(nmb, np.uint8))
    np.testing.assert_array_equal(mvi, mv)
    assert avgi == int(g[f"{case}_m{mode}_avg"][1])


@pytest.mark.parametrize("seed,w,h,mr,mode", [(61, 352, 288, 128, 2), (62, 352, 288, 128, 1), (63, 176, 144, 64, 1),
                                              (64, 208, 120, 96, 2), (65, 64, 64, 128, 2), (66, 320, 176, 32, 1),
                                              (67, 640, 360, 128, 2), (68, 48, 32, 16, 1)])
def test_against_oracle(vpp, ctx, orc, seed, w, h, mr, mode):
    fr = synth.pan_sequence(seed, w, h, 2)
    nmb = (w // 16) * (h // 16)
    incl = (synth.splitmix64(seed, nmb) % np.uint64(3) != 0).astype(np.uint8)
    for dist_incl in (None, incl):
        mv, dist, avg, _ = estimate(vpp, ctx, fr[1], fr[0], mr, mode, dist_incl)
        mv_o, dist_o, avg_o = orc.me_multires_cross(fr[1], fr[0], mr, mode=mode, dist_incl=dist_incl)
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(dist, dist_o)
        assert avg == avg_o


def test_pixel_range_rejected(vpp, ctx):
    fr = synth.pan_sequence(69, 176, 144, 2)
    bad = fr[1].copy()
    bad[10, 10] = -3
    me = vpp.MotionEstimatorH264ImplMultiresCross(bad, fr[0], 176, 144, 128, ctx=ctx)
    assert me.Create() == 1
    with pytest.raises(vpp.VppGpuError):
        me.Estimate()
