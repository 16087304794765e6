"""GPU parity of the estimators with a predictor besides the full search,
MotionEstimatorH264ImplMultiresCrossVer2, MotionEstimatorH264ImplMultires and
MotionEstimatorH264ImplCross:
vectors and avgDistortion bit-exact with the reference's golden fixtures (modes 0/1/2,
with and without pDistortionIncluded, a partial bottom row, integer-shift
content), and vectors, per-macroblock distortions and averages bit-exact with
the CPU oracle on further seeded sizes, slice maps, tie-rich content and a
1080p sequence whose predictions do not settle in the relaxation sweeps (the
exact wavefront then decides)."""
import ctypes as C

import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = ["qcif_r64", "cif_r128", "partial_r128", "small_r32", "shift_r128"]
# estimator class, oracle method, golden fixture file
KINDS = {"ver2": ("MotionEstimatorH264ImplMultiresCrossVer2", "me_multires_cross_v2", "me_mrc2.npz"),
         "multires": ("MotionEstimatorH264ImplMultires", "me_multires", "me_mr.npz"),
         "cross": ("MotionEstimatorH264ImplCross", "me_cross", "me_cross.npz")}


@pytest.fixture(params=list(KINDS))
def kind(request):
    return request.param


def oracle_fn(orc, kind):
    return getattr(orc, KINDS[kind][1])


def estimate(vpp, ctx, src, ref, mr, mode, incl=None, slice_map=None, kind="ver2"):
    h, w = src.shape
    me = getattr(vpp, KINDS[kind][0])(src, ref, w, h, mr, pDistortionIncluded=incl, mb_slice=slice_map, ctx=ctx)
    assert me.Create() == 1
    me.SetMode(mode)
    mv, avg = me.Estimate()
    return mv, me.last_mb_distortion, avg, me


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_against_golden(vpp, ctx, golden, case, mode, kind):
    g = golden(KINDS[kind][2])
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    mv, _, avg, me = estimate(vpp, ctx, src, ref, mr, mode, kind=kind)
    np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"])
    assert avg == 0
    if mode == 0:  # the multi-resolution estimators pick by area, Cross keeps quarter pel
        assert me.GetMode() == (0 if kind == "cross" else (2 if w * h > 40000 else 1))
    mvi, _, avgi, _ = estimate(vpp, ctx, src, ref, mr, mode, g[f"{case}_incl"], kind=kind)
    np.testing.assert_array_equal(mvi, mv)
    assert avgi == int(g[f"{case}_m{mode}_avg"][0])


@pytest.mark.parametrize("seed,w,h,mr,mode", [(71, 352, 288, 128, 2), (72, 352, 288, 128, 1), (73, 176, 144, 64, 1),
                                              (74, 208, 120, 96, 2), (75, 64, 64, 128, 2), (76, 320, 176, 32, 1),
                                              (77, 640, 360, 128, 2), (78, 48, 32, 16, 1)])
def test_against_oracle(vpp, ctx, orc, seed, w, h, mr, mode, kind):
    fr = synth.pan_sequence(seed, w, h, 2)
    nmb = (w // 16) * (h // 16)
    incl = (synth.splitmix64(seed, nmb) % np.uint64(3) != 0).astype(np.uint8)
    for dist_incl in (None, incl):
        mv, dist, avg, _ = estimate(vpp, ctx, fr[1], fr[0], mr, mode, dist_incl, kind=kind)
        mv_o, dist_o, avg_o = oracle_fn(orc, kind)(fr[1], fr[0], mr, mode=mode, dist_incl=dist_incl)
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(dist, dist_o)
        assert avg == avg_o


def test_slices(vpp, ctx, orc, kind):
    w, h = 352, 288
    fr = synth.pan_sequence(79, w, h, 2)
    cols, rows = w // 16, h // 16
    sl = np.repeat(np.arange(rows) // 5, cols).astype(np.int32)  # slices of 5 macroblock rows
    mv, dist, _, _ = estimate(vpp, ctx, fr[1], fr[0], 128, 2, slice_map=sl, kind=kind)
    mv_o, dist_o, _ = oracle_fn(orc, kind)(fr[1], fr[0], 128, mode=2, slice_map=sl)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)


def test_tie_rich_content(vpp, ctx, orc, kind):
    """Flat and periodic content: many searches meet exact ties, so the
    prediction decides them and those macroblocks are searched again."""
    w, h = 128, 96
    yy, xx = np.mgrid[0:h, 0:w]
    a = ((xx // 8 + yy // 8) % 2 * 40 + 100).astype(np.int16)
    b = np.roll(a, (3, 5), axis=(0, 1))
    b[20:40, 30:60] = 128
    for mode in (1, 2):
        mv, dist, _, _ = estimate(vpp, ctx, b, a, 128, mode, kind=kind)
        mv_o, dist_o, _, ties = oracle_fn(orc, kind)(b, a, 128, mode=mode, with_ties=True)
        assert ties.sum() > 0
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(dist, dist_o)


@pytest.mark.parametrize("sweeps", [8, 0, 3])
def test_1080p_sequence_and_wavefront(vpp, ctx, orc, sweeps, kind):
    """Frame pairs of the 1080p benchmark sequence with the default 8 sweeps,
    none, or 3 relaxation sweeps, after which the exact wavefront decides the
    macroblocks that have not settled; every result matches."""
    L = vpp.load()
    fr = synth.pan_sequence(1234, 1920, 1080, 4)
    used = []
    for t in range(1, 4):
        mv_o, dist_o, _ = oracle_fn(orc, kind)(fr[t], fr[t - 1], 128, mode=0)
        h, w = fr[t].shape
        me = getattr(vpp, KINDS[kind][0])(fr[t], fr[t - 1], w, h, 128, ctx=ctx)
        assert me.Create() == 1
        assert L.vppgpu_me_set_relax_sweeps(me._h_me, sweeps) == 0
        me.SetMode(0)
        mv, _ = me.Estimate()
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(me.last_mb_distortion, dist_o)
        s = C.c_int()
        L.vppgpu_me_last_sweeps(me._h_me, C.byref(s))
        used.append(s.value)
    if sweeps == 0:
        assert all(u >= 1000 for u in used), used  # no relaxation: the wavefront decided every frame


def test_pixel_range_rejected(vpp, ctx, kind):
    fr = synth.pan_sequence(80, 176, 144, 2)
    bad = fr[1].copy()
    bad[10, 10] = 300
    me = getattr(vpp, KINDS[kind][0])(bad, fr[0], 176, 144, 128, ctx=ctx)
    assert me.Create() == 1
    with pytest.raises(vpp.VppGpuError):
        me.Estimate()
