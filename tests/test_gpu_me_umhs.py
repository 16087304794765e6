"""GPU parity of MotionEstimatorH264ImplUMHS: vectors, the distortion stored
with each vector and avgDistortion bit-exact with the reference's golden
fixtures (modes 0/1/2, previous-frame vectors and intra flags, pan, shift and
part-noise content, the 1080p benchmark pair), and with the CPU oracle on
further sizes, motion ranges, slice maps and relaxation settings; the results
do not depend on how many relaxation sweeps run before the dataflow pass."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth
from tests.golden.make_golden import prev_frame_vectors, umhs_frames

pytestmark = pytest.mark.gpu

CASES = ["qcif_r64", "cif_r128", "shift_r128", "noisy_r128", "small_r32"]


def estimate(vpp, ctx, src, ref, mr, mode=0, incl=None, prev=None, slice_map=None, sweeps=None):
    h, w = src.shape
    me = vpp.MotionEstimatorH264ImplUMHS(src, ref, w, h, mr, pDistortionIncluded=incl, pPrevFrmMBlk=prev,
                                         mb_slice=slice_map, ctx=ctx)
    assert me.Create() == 1
    me.SetMode(mode)
    if sweeps is not None:
        vpp.load().vppgpu_me_set_relax_sweeps(me._h_me, sweeps)
    mv, avg = me.Estimate()
    return mv, me.last_mb_distortion, avg, me


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_against_golden(vpp, ctx, golden, case, mode):
    g = golden("me_umhs.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    src, ref = g[f"{case}_src"].astype(np.int16), g[f"{case}_ref"].astype(np.int16)
    prev = (g[f"{case}_prev_mv"], g[f"{case}_prev_intra"])
    mv, dist, avg, me = estimate(vpp, ctx, src, ref, mr, mode, g[f"{case}_incl"], prev)
    assert me.GetMode() == mode  # SetMode keeps the mode as given
    np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"])
    np.testing.assert_array_equal(dist, g[f"{case}_m{mode}_dist"])
    assert avg == int(g[f"{case}_m{mode}_avg"][0])
    if mode == 0:
        mv0, dist0, avg0, _ = estimate(vpp, ctx, src, ref, mr)
        np.testing.assert_array_equal(mv0, g[f"{case}_noprev_mv"])
        np.testing.assert_array_equal(dist0, g[f"{case}_noprev_dist"])
        assert avg0 == 0


def test_1080p_against_golden(vpp, ctx, golden, hd_golden):
    g = golden("me_umhs.npz")
    assert g["hd_frames_sha256"].tobytes() == hd_golden["g"]["frames_sha256"].tobytes()
    fr, mr = hd_golden["frames"], hd_golden["motion_range"]
    incl = np.ones((hd_golden["w"] // 16) * (hd_golden["h"] // 16), np.uint8)
    mv, dist, avg, _ = estimate(vpp, ctx, fr[1], fr[0], mr, 0, incl)
    np.testing.assert_array_equal(mv, g["hd_mv"])
    np.testing.assert_array_equal(dist, g["hd_dist"])
    assert avg == int(g["hd_avg"][0])


@pytest.mark.parametrize("seed,w,h,mr,mode,gen", [(91, 176, 144, 128, 0, "noisy"), (92, 208, 120, 96, 1, "pan"),
                                                 (93, 96, 64, 16, 0, "shift"), (94, 640, 368, 128, 0, "noisy"),
                                                 (95, 352, 288, 64, 2, "noisy"), (96, 1280, 720, 128, 0, "pan")])
def test_against_oracle(vpp, ctx, orc, seed, w, h, mr, mode, gen):
    fr = umhs_frames(seed, w, h, gen)
    pmv, pin = prev_frame_vectors(seed, w, h, mr)
    incl = (synth.splitmix64(seed, (w // 16) * (h // 16)) & np.uint64(1)).astype(np.uint8)
    mv_o, dist_o, avg_o = orc.me_umhs(fr[1], fr[0], mr, mode=mode, dist_incl=incl, prev_mv=pmv, prev_intra=pin)
    mv, dist, avg, _ = estimate(vpp, ctx, fr[1], fr[0], mr, mode, incl, (pmv, pin))
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)
    assert avg == avg_o


def test_slices(vpp, ctx, orc):
    w, h, mr = 352, 288, 128
    fr = umhs_frames(97, w, h, "noisy")
    cols, rows = w // 16, h // 16
    sl = (np.arange(cols * rows) // (cols * 5 + 7)).astype(np.int32)  # slices cut inside macroblock rows
    mv_o, dist_o, _ = orc.me_umhs(fr[1], fr[0], mr, slice_map=sl)
    mv, dist, _, _ = estimate(vpp, ctx, fr[1], fr[0], mr, slice_map=sl)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)


@pytest.mark.parametrize("sweeps", [0, 1, 2, 6, 14])
def test_result_independent_of_sweeps(vpp, ctx, orc, sweeps):
    """Relaxation only seeds records and may reach the fixed point early; the
    dataflow pass decides the rest, so every setting gives the sequential result."""
    w, h, mr = 640, 368, 128
    fr = umhs_frames(98, w, h, "noisy")
    pmv, pin = prev_frame_vectors(98, w, h, mr)
    mv_o, dist_o, _ = orc.me_umhs(fr[1], fr[0], mr, prev_mv=pmv, prev_intra=pin)
    mv, dist, _, _ = estimate(vpp, ctx, fr[1], fr[0], mr, prev=(pmv, pin), sweeps=sweeps)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)


def test_1080p_sequence(vpp, ctx, orc):
    """Several pairs of a 1080p pan through one handle, each pair's vectors the
    previous frame's starting points, as a codec chains them."""
    w, h, mr = 1920, 1080, 128
    fr = synth.pan_sequence(4321, w, h, 4)
    cur = fr[1].copy()
    ref = fr[0].copy()
    me = vpp.MotionEstimatorH264ImplUMHS(cur, ref, w, h, mr, ctx=ctx)
    assert me.Create() == 1
    prev = None
    for t in range(3):
        cur[...] = fr[t + 1]
        ref[...] = fr[t]
        me._prev = prev
        mv, _ = me.Estimate()
        mv_o, dist_o, _ = orc.me_umhs(fr[t + 1], fr[t], mr, prev_mv=None if prev is None else prev[0])
        np.testing.assert_array_equal(mv, mv_o, err_msg=f"pair {t}")
        np.testing.assert_array_equal(me.last_mb_distortion, dist_o, err_msg=f"pair {t}")
        prev = (mv.copy(), None)
    # the relaxation starts from the previous estimate's states: unrelated
    # content before must not change a result
    noisy = umhs_frames(5, w, h, "noisy")
    cur[...] = noisy[1]
    ref[...] = noisy[0]
    me._prev = None
    mv, _ = me.Estimate()
    mv_o, dist_o, _ = orc.me_umhs(noisy[1], noisy[0], mr)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(me.last_mb_distortion, dist_o)


def test_predictor_side_effect_carries_distortion(vpp, ctx):
    class Pred:
        def __init__(self):
            self.calls = []

        def Set16x16MotionVector(self, k, x, y, d=None):
            self.calls.append((k, x, y, d))

    fr = umhs_frames(99, 96, 64, "noisy")
    p = Pred()
    me = vpp.MotionEstimatorH264ImplUMHS(fr[1], fr[0], 96, 64, 64, pMVPred=p, ctx=ctx)
    assert me.Create() == 1
    mv, _ = me.Estimate()
    assert [c[0] for c in p.calls] == list(range(24))
    assert all(c[1:3] == (int(mv[c[0], 0]), int(mv[c[0], 1])) and c[3] == int(me.last_mb_distortion[c[0]])
               for c in p.calls)


def test_prev_vectors_outside_the_frame_are_refused(vpp, ctx):
    fr = synth.pan_sequence(3, 64, 48, 2)
    pmv = np.zeros((12, 2), np.int16)
    pmv[0] = (-4 * 17, 0)
    me = vpp.MotionEstimatorH264ImplUMHS(fr[1], fr[0], 64, 48, 128, pPrevFrmMBlk=(pmv, None), ctx=ctx)
    assert me.Create() == 1
    with pytest.raises(vpp.VppGpuError):
        me.Estimate()
    pin = np.zeros(12, np.uint8)
    pin[0] = 1  # an intra macroblock's vector is not read
    me._prev = (pmv, pin)
    me.Estimate()
