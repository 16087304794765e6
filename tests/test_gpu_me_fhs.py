"""GPU parity of MotionEstimatorH264ImplFHS: vectors, the distortion stored
with each vector and avgDistortion bit-exact with the reference's golden
fixtures (modes 0/1/2 on pan, shift and part-noise content, the 1080p
benchmark pair), and with the CPU oracle on further sizes, motion ranges, slice
maps, relaxation settings and a chained 1080p sequence."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth
from tests.golden.make_golden import umhs_frames

pytestmark = pytest.mark.gpu

CASES = ["qcif_r64", "cif_r128", "shift_r128", "noisy_r128", "small_r32"]


def estimate(vpp, ctx, src, ref, mr, mode=0, incl=None, slice_map=None, sweeps=None):
    h, w = src.shape
    me = vpp.MotionEstimatorH264ImplFHS(src, ref, w, h, mr, pDistortionIncluded=incl, mb_slice=slice_map, ctx=ctx)
    assert me.Create() == 1
    me.SetMode(mode)
    if sweeps is not None:
        assert vpp.load().vppgpu_me_set_relax_sweeps(me._h_me, sweeps) == 0
    mv, avg = me.Estimate()
    return mv, me.last_mb_distortion, avg, me


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_against_golden(vpp, ctx, golden, case, mode):
    g, gu = golden("me_fhs.npz"), golden("me_umhs.npz")
    w, h, mr = (int(v) for v in gu[f"{case}_meta"])
    src, ref = gu[f"{case}_src"].astype(np.int16), gu[f"{case}_ref"].astype(np.int16)
    mv, dist, avg, me = estimate(vpp, ctx, src, ref, mr, mode, gu[f"{case}_incl"])
    assert me.GetMode() == mode
    np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"])
    np.testing.assert_array_equal(dist, g[f"{case}_m{mode}_dist"])
    assert avg == int(g[f"{case}_m{mode}_avg"][0])


def test_1080p_against_golden(vpp, ctx, golden, hd_golden):
    g = golden("me_fhs.npz")
    assert g["hd_frames_sha256"].tobytes() == hd_golden["g"]["frames_sha256"].tobytes()
    fr, mr = hd_golden["frames"], hd_golden["motion_range"]
    incl = np.ones((hd_golden["w"] // 16) * (hd_golden["h"] // 16), np.uint8)
    mv, dist, avg, _ = estimate(vpp, ctx, fr[1], fr[0], mr, 0, incl)
    np.testing.assert_array_equal(mv, g["hd_mv"])
    np.testing.assert_array_equal(dist, g["hd_dist"])
    assert avg == int(g["hd_avg"][0])


@pytest.mark.parametrize("seed,w,h,mr,mode,gen", [(101, 176, 144, 128, 0, "noisy"), (102, 208, 120, 96, 1, "pan"),
                                                 (103, 96, 64, 16, 0, "shift"), (104, 640, 368, 128, 0, "noisy"),
                                                 (105, 352, 288, 64, 2, "shift"), (106, 1280, 720, 128, 0, "pan")])
def test_against_oracle(vpp, ctx, orc, seed, w, h, mr, mode, gen):
    fr = umhs_frames(seed, w, h, gen)
    incl = (synth.splitmix64(seed, (w // 16) * (h // 16)) & np.uint64(1)).astype(np.uint8)
    mv_o, dist_o, avg_o = orc.me_fhs(fr[1], fr[0], mr, mode=mode, dist_incl=incl)
    mv, dist, avg, _ = estimate(vpp, ctx, fr[1], fr[0], mr, mode, incl)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)
    assert avg == avg_o


def test_slices(vpp, ctx, orc):
    w, h, mr = 352, 288, 128
    fr = umhs_frames(107, w, h, "noisy")
    cols, rows = w // 16, h // 16
    sl = (np.arange(cols * rows) // (cols * 4 + 3)).astype(np.int32)
    mv_o, dist_o, _ = orc.me_fhs(fr[1], fr[0], mr, slice_map=sl)
    mv, dist, _, _ = estimate(vpp, ctx, fr[1], fr[0], mr, slice_map=sl)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)


@pytest.mark.parametrize("sweeps", [0, 1, 3, 20, 24])
def test_result_independent_of_sweeps(vpp, ctx, orc, sweeps):
    w, h, mr = 640, 368, 128
    fr = umhs_frames(108, w, h, "noisy")
    mv_o, dist_o, _ = orc.me_fhs(fr[1], fr[0], mr)
    mv, dist, _, _ = estimate(vpp, ctx, fr[1], fr[0], mr, sweeps=sweeps)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)


def test_1080p_sequence(vpp, ctx, orc):
    """Consecutive 1080p pairs through one handle (the relaxation starts from
    the previous estimate's states), then unrelated content."""
    w, h, mr = 1920, 1080, 128
    fr = synth.pan_sequence(5432, w, h, 4)
    cur, ref = fr[1].copy(), fr[0].copy()
    me = vpp.MotionEstimatorH264ImplFHS(cur, ref, w, h, mr, ctx=ctx)
    assert me.Create() == 1
    pairs = [(fr[t + 1], fr[t]) for t in range(3)] + [tuple(umhs_frames(6, w, h, "noisy")[::-1])]
    for t, (a, b) in enumerate(pairs):
        cur[...] = a
        ref[...] = b
        mv, _ = me.Estimate()
        mv_o, dist_o, _ = orc.me_fhs(a, b, mr)
        np.testing.assert_array_equal(mv, mv_o, err_msg=f"pair {t}")
        np.testing.assert_array_equal(me.last_mb_distortion, dist_o, err_msg=f"pair {t}")


def test_predictor_side_effect_carries_distortion(vpp, ctx):
    class Pred:
        def __init__(self):
            self.calls = []

        def Set16x16MotionVector(self, k, x, y, d=None):
            self.calls.append((k, x, y, d))

    fr = umhs_frames(109, 96, 64, "noisy")
    p = Pred()
    me = vpp.MotionEstimatorH264ImplFHS(fr[1], fr[0], 96, 64, 64, pMVPred=p, ctx=ctx)
    assert me.Create() == 1
    mv, _ = me.Estimate()
    assert [c[0] for c in p.calls] == list(range(24))
    assert all(c[1:3] == (int(mv[c[0], 0]), int(mv[c[0], 1])) and c[3] == int(me.last_mb_distortion[c[0]])
               for c in p.calls)
