"""GPU parity of MultiresCrossVer2's Lagrangian overload, Estimate(long*,
void* lambda) (src/CodecUtils/MotionEstimatorH264ImplMultiresCrossVer2.cpp:1162-1742):
vectors and avgDistortion bit-exact with the compiled reference's golden
fixtures at lambdas 0, 0.9, 2.5 and 20 (modes 0/1/2, a partial bottom row,
integer-shift content) and at 1080p, and vectors, per-macroblock distortions
and averages bit-exact with the CPU oracle on further sizes, lambdas (a
negative one too), slice maps, tie-rich content, and with the exact wavefront
deciding every macroblock."""
import ctypes as C

import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = ["qcif_r64", "cif_r128", "partial_r128", "small_r32", "shift_r128"]


def estimate(vpp, ctx, src, ref, mr, mode, lam, incl=None, slice_map=None, sweeps=None):
    h, w = src.shape
    me = vpp.MotionEstimatorH264ImplMultiresCrossVer2(src, ref, w, h, mr, pDistortionIncluded=incl,
                                                      mb_slice=slice_map, ctx=ctx)
    assert me.Create() == 1
    me.SetMode(mode)
    if sweeps is not None:
        assert vpp.load().vppgpu_me_set_relax_sweeps(me._h_me, sweeps) == 0
    mv, avg = me.Estimate(param=lam)
    return mv, me.last_mb_distortion, avg, me


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_against_golden(vpp, ctx, golden, case, mode):
    g, gl = golden("me_mrc2.npz"), golden("me_mrc2_lambda.npz")
    mr = int(g[f"{case}_meta"][2])
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    for li, lam in enumerate(gl["lambdas"]):
        mv, _, avg, _ = estimate(vpp, ctx, src, ref, mr, mode, float(lam), g[f"{case}_incl"])
        np.testing.assert_array_equal(mv, gl[f"{case}_m{mode}_l{li}_mv"], err_msg=f"lambda {lam}")
        assert avg == int(gl[f"{case}_m{mode}_l{li}_avg"][0])


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("sweeps", [None, 0])
def test_against_golden_1080p(vpp, ctx, golden, hd_golden, mode, sweeps):
    """Pair 0 of the 1080p benchmark sequence at motionRange 128, with the
    default relaxation and with none (the wavefront decides every MB)."""
    gl = golden("me_mrc2_lambda.npz")
    fr, mr = hd_golden["frames"], hd_golden["motion_range"]
    incl = np.ones((hd_golden["w"] // 16) * (hd_golden["h"] // 16), np.uint8)
    for lam in (0.9, 4.0):
        mv, _, avg, me = estimate(vpp, ctx, fr[1], fr[0], mr, mode, lam, incl, sweeps=sweeps)
        np.testing.assert_array_equal(mv, gl[f"hd_m{mode}_lam{lam:g}_mv"], err_msg=f"lambda {lam}")
        assert avg == int(gl[f"hd_m{mode}_lam{lam:g}_avg"][0])
        if sweeps == 0:
            assert me.last_sweeps() >= 1000


@pytest.mark.parametrize("seed,w,h,mr,mode,lam", [(91, 352, 288, 128, 2, 1.5), (92, 176, 144, 64, 1, 0.25),
                                                  (93, 208, 120, 96, 2, 7.0), (94, 64, 64, 128, 2, -0.5),
                                                  (95, 640, 360, 128, 1, 3.0), (96, 48, 32, 16, 1, 1e6)])
def test_against_oracle(vpp, ctx, orc, seed, w, h, mr, mode, lam):
    fr = synth.pan_sequence(seed, w, h, 2)
    nmb = (w // 16) * (h // 16)
    incl = (synth.splitmix64(seed, nmb) % np.uint64(3) != 0).astype(np.uint8)
    for dist_incl in (None, incl):
        mv, dist, avg, _ = estimate(vpp, ctx, fr[1], fr[0], mr, mode, lam, dist_incl)
        mv_o, dist_o, avg_o = orc.me_multires_cross_v2_lambda(fr[1], fr[0], mr, lam, mode=mode, dist_incl=dist_incl)
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(dist, dist_o)
        assert avg == avg_o


def test_slices_and_ties(vpp, ctx, orc):
    """A slice map (slices of 5 MB rows), and flat / periodic content whose
    searches meet exact ties at every level."""
    w, h = 352, 288
    fr = synth.pan_sequence(97, w, h, 2)
    sl = np.repeat(np.arange(h // 16) // 5, w // 16).astype(np.int32)
    mv, dist, _, _ = estimate(vpp, ctx, fr[1], fr[0], 128, 2, 1.25, slice_map=sl)
    mv_o, dist_o, _ = orc.me_multires_cross_v2_lambda(fr[1], fr[0], 128, 1.25, mode=2, slice_map=sl)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)
    w, h = 128, 96
    yy, xx = np.mgrid[0:h, 0:w]
    a = ((xx // 8 + yy // 8) % 2 * 40 + 100).astype(np.int16)
    b = np.roll(a, (3, 5), axis=(0, 1))
    b[20:40, 30:60] = 128
    for mode in (1, 2):
        mv, dist, _, _ = estimate(vpp, ctx, b, a, 128, mode, 0.9)
        mv_o, dist_o, _ = orc.me_multires_cross_v2_lambda(b, a, 128, 0.9, mode=mode)
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(dist, dist_o)


def test_overload_and_plain_estimates_alternate(vpp, ctx, orc):
    """One handle: plain, Lagrangian, plain again; each matches its own
    oracle (no state of one estimate leaks into the next).  The other
    estimators ignore the parameter, as IMotionEstimator's default does."""
    w, h = 352, 288
    fr = synth.pan_sequence(98, w, h, 2)
    me = vpp.MotionEstimatorH264ImplMultiresCrossVer2(fr[1], fr[0], w, h, 128, ctx=ctx)
    assert me.Create() == 1
    me.SetMode(2)
    plain = orc.me_multires_cross_v2(fr[1], fr[0], 128, mode=2)[0]
    lagr = orc.me_multires_cross_v2_lambda(fr[1], fr[0], 128, 3.0, mode=2)[0]
    assert (plain != lagr).any()
    np.testing.assert_array_equal(me.Estimate()[0], plain)
    np.testing.assert_array_equal(me.Estimate(3.0)[0], lagr)
    np.testing.assert_array_equal(me.Estimate()[0], plain)
    full = vpp.MotionEstimatorH264ImplFull(fr[1], fr[0], w, h, 64, ctx=ctx)
    assert full.Create() == 1
    np.testing.assert_array_equal(full.Estimate(param=7.0)[0], full.Estimate()[0])
