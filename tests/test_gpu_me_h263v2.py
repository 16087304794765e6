"""GPU MotionEstimatorH263ImplMultiresCrossVer2 parity: vectors and
avgDistortion bit-exact with the reference's golden fixtures (modes 0/1/2,
with and without pDistortionIncluded, a partial bottom row, the 1080p
benchmark pair), and vectors, per-macroblock distortions and averages
bit-exact with the CPU oracle on further sizes, ranges and content; the
result does not depend on how many relaxation sweeps run before the exact
pass."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth
from tests.golden.make_golden import umhs_frames

pytestmark = pytest.mark.gpu

CASES = ["qcif_r32", "cif_r64", "partial_r64", "small_r16", "wide_r48"]


def estimate(vpp, ctx, src, ref, mr, mode, incl=None, sweeps=None):
    h, w = src.shape
    me = vpp.MotionEstimatorH263ImplMultiresCrossVer2(src, ref, w, h, mr, pDistortionIncluded=incl, ctx=ctx)
    assert me.Create() == 1
    me.SetMode(mode)
    if sweeps is not None:
        assert vpp.load().vppgpu_me_set_relax_sweeps(me._h_me, sweeps) == 0
    mv, avg = me.Estimate()
    return mv, me.last_mb_distortion, avg, me


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_against_golden(vpp, ctx, golden, case, mode):
    g = golden("me_h263mrc2.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    mv, _, avg, me = estimate(vpp, ctx, src, ref, mr, mode)
    np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"])
    assert avg == int(g[f"{case}_m{mode}_avg"][0])
    if mode == 0:
        assert me.GetMode() == (2 if w * h > 40000 else 1)
    mvi, _, avgi, _ = estimate(vpp, ctx, src, ref, mr, mode, g[f"{case}_incl"])
    np.testing.assert_array_equal(mvi, mv)
    assert avgi == int(g[f"{case}_m{mode}_avg"][1])


@pytest.mark.parametrize("mode", [0, 1])
def test_1080p_against_golden(vpp, ctx, golden, hd_golden, mode):
    g = golden("me_h263mrc2.npz")
    assert g["hd_frames_sha256"].tobytes() == hd_golden["g"]["frames_sha256"].tobytes()
    fr = hd_golden["frames"]
    mv, _, avg, _ = estimate(vpp, ctx, fr[1], fr[0], int(g["hd_meta"][3]), mode)
    np.testing.assert_array_equal(mv, g[f"hd_m{mode}_mv"])
    assert avg == int(g[f"hd_m{mode}_avg"][0])


@pytest.mark.parametrize("seed,w,h,mr,mode,gen", [(81, 352, 288, 64, 2, "noisy"), (82, 352, 288, 64, 1, "pan"),
                                                 (83, 176, 144, 30, 1, "shift"), (84, 208, 120, 48, 2, "noisy"),
                                                 (85, 64, 64, 64, 2, "pan"), (86, 320, 176, 16, 1, "noisy"),
                                                 (87, 640, 360, 64, 2, "shift"), (88, 48, 32, 8, 1, "pan"),
                                                 (89, 1920, 1088, 64, 2, "noisy"), (90, 1280, 720, 40, 1, "pan")])
def test_against_oracle(vpp, ctx, orc, seed, w, h, mr, mode, gen):
    fr = umhs_frames(seed, w, h, gen)
    nmb = (w // 16) * (h // 16)
    incl = (synth.splitmix64(seed, nmb) % np.uint64(3) != 0).astype(np.uint8)
    for dist_incl in (None, incl):
        mv, dist, avg, _ = estimate(vpp, ctx, fr[1], fr[0], mr, mode, dist_incl)
        mv_o, dist_o, avg_o = orc.me_h263_multires_cross_ver2(fr[1], fr[0], mr, mode=mode, dist_incl=dist_incl)
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(dist, dist_o)
        assert avg == avg_o


@pytest.mark.parametrize("sweeps", [0, 1, 3, 8, 24, 48])
def test_result_independent_of_sweeps(vpp, ctx, orc, sweeps):
    """Relaxation either reaches the fixed point (the sequential result) or
    hands over to the one-CTA exact pass: every setting gives the same vectors."""
    w, h, mr = 640, 368, 64
    fr = umhs_frames(91, w, h, "pan")
    mv_o, dist_o, avg_o = orc.me_h263_multires_cross_ver2(fr[1], fr[0], mr, mode=2)
    mv, dist, avg, me = estimate(vpp, ctx, fr[1], fr[0], mr, 2, sweeps=sweeps)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)
    assert avg == avg_o
    used = me.last_sweeps()
    assert used >= 1000 or 1 <= used <= sweeps


def test_sequence_through_one_handle(vpp, ctx, orc):
    w, h, mr = 1920, 1080, 64
    fr = synth.pan_sequence(2468, w, h, 4)
    cur, ref = fr[1].copy(), fr[0].copy()
    me = vpp.MotionEstimatorH263ImplMultiresCrossVer2(cur, ref, w, h, mr, ctx=ctx)
    assert me.Create() == 1
    me.SetMode(0)
    pairs = [(fr[t + 1], fr[t]) for t in range(3)] + [tuple(umhs_frames(8, w, h, "noisy")[::-1])]
    for t, (a, b) in enumerate(pairs):
        cur[...] = a
        ref[...] = b
        mv, avg = me.Estimate()
        mv_o, dist_o, avg_o = orc.me_h263_multires_cross_ver2(a, b, mr, mode=2)
        np.testing.assert_array_equal(mv, mv_o, err_msg=f"pair {t}")
        np.testing.assert_array_equal(me.last_mb_distortion, dist_o, err_msg=f"pair {t}")
        assert avg == avg_o


@pytest.mark.parametrize("seed,w,h,mr,gen", [(121, 48, 2048, 32, "pan"), (122, 3840, 2160, 64, "noisy"),
                                              (123, 16, 512, 16, "shift")])
def test_tall_and_4k_frames(vpp, ctx, orc, seed, w, h, mr, gen):
    """The exact pass keeps a thread and a ring per macroblock row: 128 and
    135 rows, and a single column."""
    fr = umhs_frames(seed, w, h, gen)
    mv_o, dist_o, avg_o = orc.me_h263_multires_cross_ver2(fr[1], fr[0], mr, mode=0)
    mv, dist, avg, _ = estimate(vpp, ctx, fr[1], fr[0], mr, 0, sweeps=2)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)
    assert avg == avg_o


def test_range_limit(vpp, ctx):
    fr = synth.pan_sequence(100, 64, 48, 2)
    me = vpp.MotionEstimatorH263ImplMultiresCrossVer2(fr[1], fr[0], 64, 48, 66, ctx=ctx)
    assert me.Create() == 0  # half-pel range above 64 (+-31 pels) is not supported
