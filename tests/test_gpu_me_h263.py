"""GPU MotionEstimatorH263ImplMultiresCross parity: vectors and avgDistortion
bit-exact with the reference's golden fixtures (modes 0/1/2, with and without
pDistortionIncluded, a partial bottom row), and vectors, per-macroblock
distortions and averages bit-exact with the CPU oracle on further seeded sizes
and half-pel ranges."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = ["qcif_r32", "cif_r64", "partial_r64", "small_r16"]


def estimate(vpp, ctx, src, ref, mr, mode, incl=None):
    h, w = src.shape
    me = vpp.MotionEstimatorH263ImplMultiresCross(src, ref, w, h, mr, pDistortionIncluded=incl, ctx=ctx)
    assert me.Create() == 1
    me.SetMode(mode)
    mv, avg = me.Estimate()
    return mv, me.last_mb_distortion, avg, me


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_against_golden(vpp, ctx, golden, case, mode):
    g = golden("me_h263mrc.npz")
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


@pytest.mark.parametrize("seed,w,h,mr,mode", [(91, 352, 288, 64, 2), (92, 352, 288, 64, 1), (93, 176, 144, 30, 1),
                                              (94, 208, 120, 48, 2), (95, 64, 64, 64, 2), (96, 320, 176, 16, 1),
                                              (97, 640, 360, 64, 2), (98, 48, 32, 8, 1), (99, 1920, 1088, 64, 2)])
def test_against_oracle(vpp, ctx, orc, seed, w, h, mr, mode):
    fr = synth.pan_sequence(seed, w, h, 2)
    nmb = (w // 16) * (h // 16)
    incl = (synth.splitmix64(seed, nmb) % np.uint64(3) != 0).astype(np.uint8)
    for dist_incl in (None, incl):
        mv, dist, avg, _ = estimate(vpp, ctx, fr[1], fr[0], mr, mode, dist_incl)
        mv_o, dist_o, avg_o = orc.me_h263_multires_cross(fr[1], fr[0], mr, mode=mode, dist_incl=dist_incl)
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(dist, dist_o)
        assert avg == avg_o


def test_range_limit(vpp, ctx):
    fr = synth.pan_sequence(100, 64, 48, 2)
    me = vpp.MotionEstimatorH263ImplMultiresCross(fr[1], fr[0], 64, 48, 66, ctx=ctx)
    assert me.Create() == 0  # half-pel range above 64 (+-31 pels) is not supported
