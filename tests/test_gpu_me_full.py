"""GPU MotionEstimatorH264ImplFull parity: vectors, per-macroblock
distortions and avgDistortion bit-exact with the reference's golden fixtures
and with the CPU oracle, including edge cases (ties on flat content, slices,
partial bottom rows, small ranges) and full-size 1080p frames."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu

ME_CASES = ["qcif_r64", "qcif_r128", "cif_r128", "partial_r128", "shift_r64"]


def estimate(vpp, ctx, src, ref, mr, incl=None, slice_map=None):
    h, w = src.shape
    me = vpp.MotionEstimatorH264ImplFull(src, ref, w, h, mr, pDistortionIncluded=incl, mb_slice=slice_map, ctx=ctx)
    assert me.Create() == 1
    mv, avg = me.Estimate()
    return mv, me.last_mb_distortion, avg, me


@pytest.mark.parametrize("case", ME_CASES)
def test_against_golden(vpp, ctx, golden, case):
    g = golden("me_full.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    incl = np.ones((w // 16) * (h // 16), np.uint8)
    mv, dist, avg, _ = estimate(vpp, ctx, src, ref, mr, incl)
    np.testing.assert_array_equal(mv, g[f"{case}_mv"])
    assert avg == int(g[f"{case}_avg"][0])
    if f"{case}_mbdist" in g:
        np.testing.assert_array_equal(dist, g[f"{case}_mbdist"])
    _, _, avg0, _ = estimate(vpp, ctx, src, ref, mr)
    assert avg0 == 0


@pytest.mark.parametrize("seed,w,h,mr", [(41, 352, 288, 128), (42, 176, 144, 64), (43, 208, 120, 96),
                                         (44, 64, 64, 128), (45, 16, 16, 128), (46, 320, 176, 8),
                                         (47, 48, 32, 4), (48, 352, 280, 128)])
def test_against_oracle(vpp, ctx, orc, seed, w, h, mr):
    fr = synth.pan_sequence(seed, w, h, 2)
    nmb = (w // 16) * (h // 16)
    incl = (synth.splitmix64(seed, nmb) % np.uint64(3) != 0).astype(np.uint8)
    mv, dist, avg, _ = estimate(vpp, ctx, fr[1], fr[0], mr, incl)
    mv_o, dist_o, avg_o = orc.me_full(fr[1], fr[0], mr, dist_incl=incl)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)
    assert avg == avg_o


def test_ties_on_flat_and_periodic_content(vpp, ctx, orc):
    """Checkerboard + flat patch: many exact SSD ties, decided by the
    prediction-relative tie-break and resolved through the predictor chain."""
    w, h = 192, 128
    yy, xx = np.mgrid[0:h, 0:w]
    a = ((xx // 8 + yy // 8) % 2 * 40 + 100).astype(np.int16)
    b = np.roll(a, (3, 5), axis=(0, 1))
    b[20:60, 30:120] = 128
    a[70:100, 10:50] = 90
    b[70:100, 14:54] = 90
    for mr in (64, 128):
        mv, dist, avg, _ = estimate(vpp, ctx, b, a, mr, np.ones(96, np.uint8))
        mv_o, dist_o, avg_o = orc.me_full(b, a, mr, dist_incl=np.ones(96, np.uint8))
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(dist, dist_o)
        assert avg == avg_o


def test_constant_frames(vpp, ctx, orc):
    a = np.full((64, 96), 77, np.int16)
    mv, dist, _, _ = estimate(vpp, ctx, a, a, 128)
    mv_o, dist_o, _ = orc.me_full(a, a, 128)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)


def test_slices(vpp, ctx, orc):
    w, h = 176, 144
    fr = synth.pan_sequence(51, w, h, 2)
    sl = np.repeat(np.arange(3), 33).astype(np.int32)  # three slices of 33 macroblocks
    mv, dist, _, _ = estimate(vpp, ctx, fr[1], fr[0], 128, slice_map=sl)
    mv_o, dist_o, _ = orc.me_full(fr[1], fr[0], 128, slice_map=sl)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)


def test_repeated_estimates_reuse_handle(vpp, ctx, orc):
    """The planes are re-read on every Estimate() (the caller overwrites them)."""
    w, h = 176, 144
    fr = synth.pan_sequence(52, w, h, 4)
    src, ref = fr[1].copy(), fr[0].copy()
    me = vpp.MotionEstimatorH264ImplFull(src, ref, w, h, 128, ctx=ctx)
    assert me.Create() == 1
    for t in range(3):
        src[...] = fr[t + 1]
        ref[...] = fr[t]
        mv, _ = me.Estimate()
        mv_o, _, _ = orc.me_full(fr[t + 1], fr[t], 128)
        np.testing.assert_array_equal(mv, mv_o)


def test_predictor_side_effect(vpp, ctx):
    class Pred:
        def __init__(self):
            self.v = {}

        def Set16x16MotionVector(self, k, x, y):
            self.v[k] = (x, y)

    fr = synth.pan_sequence(53, 64, 48, 2)
    p = Pred()
    me = vpp.MotionEstimatorH264ImplFull(fr[1], fr[0], 64, 48, 128, pMVPred=p, ctx=ctx)
    me.Create()
    mv, _ = me.Estimate()
    assert [p.v[k] for k in range(12)] == [tuple(int(c) for c in row) for row in mv]


def test_pixel_range_is_rejected(vpp, ctx):
    a = np.full((32, 32), 10, np.int16)
    b = a.copy()
    b[5, 5] = 256
    me = vpp.MotionEstimatorH264ImplFull(b, a, 32, 32, 64, ctx=ctx)
    me.Create()
    with pytest.raises(vpp.VppGpuError) as e:
        me.Estimate()
    assert e.value.status == -4
    b[5, 5] = -1
    with pytest.raises(vpp.VppGpuError):
        me.Estimate()
    b[5, 5] = 255  # the handle stays usable
    me.Estimate()


def test_invalid_geometry(vpp, ctx):
    me = vpp.MotionEstimatorH264ImplFull(np.zeros((32, 40), np.int16), np.zeros((32, 40), np.int16), 40, 32, 64, ctx=ctx)
    assert me.Create() == 0  # width not a multiple of 16
    me = vpp.MotionEstimatorH264ImplFull(np.zeros((32, 32), np.int16), np.zeros((32, 32), np.int16), 32, 32, 256, ctx=ctx)
    assert me.Create() == 0  # beyond the supported +-31 pel search


@pytest.mark.parametrize("h", [1088, 1080])
def test_1080p_against_oracle(vpp, ctx, orc, h):
    """Full-size frame (8160 / 8040 macroblocks) at motionRange 128."""
    w = 1920
    fr = synth.pan_sequence(60 + h, w, h, 2)
    nmb = (w // 16) * (h // 16)
    incl = np.ones(nmb, np.uint8)
    mv, dist, avg, me = estimate(vpp, ctx, fr[1], fr[0], 128, incl)
    mv_o, dist_o, avg_o = orc.me_full(fr[1], fr[0], 128, dist_incl=incl)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)
    assert avg == avg_o
    assert me.last_sweeps() >= 1


@pytest.mark.parametrize("sweeps", [0, 2])
def test_wavefront_after_few_relaxation_sweeps(vpp, ctx, orc, sweeps):
    """With no or two relaxation sweeps the exact wavefront decides most of
    the frame; the result is the sequential one either way (the captured
    kernel sequence is rebuilt after the change)."""
    w, h = 640, 368
    fr = synth.pan_sequence(90 + sweeps, w, h, 3)
    me = vpp.MotionEstimatorH264ImplFull(fr[1], fr[0], w, h, 128, ctx=ctx)
    assert me.Create() == 1
    me.Estimate()  # captured with the default 8 sweeps
    L = vpp.load()
    assert L.vppgpu_me_set_relax_sweeps(me._h_me, sweeps) == 0
    for t in (1, 2):
        me._src, me._ref = fr[t], fr[t - 1]
        mv, _ = me.Estimate()
        mv_o, dist_o, _ = orc.me_full(fr[t], fr[t - 1], 128)
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(me.last_mb_distortion, dist_o)
        if sweeps == 0:
            assert me.last_sweeps() == 1000


@pytest.mark.parametrize("mr", [0, 1, 2, 3])
def test_sub_pel_only_ranges_are_refused(vpp, ctx, mr):
    """motionRange 0..3 makes the reference search sub-pel positions only;
    nothing pins that, so every estimator kind refuses it at creation."""
    import ctypes as C

    from imagecodingutils_gb300 import _lib
    L = vpp.load()
    for kind in range(_lib.ME_FULL, _lib.ME_FULL_SAD + 1):
        h = C.c_void_p()
        assert L.vppgpu_me_create(ctx.handle, kind, 176, 144, mr, C.byref(h)) == _lib.ERR_INVALID_ARG
        assert not h.value
    me = vpp.MotionEstimatorH264ImplFull(np.zeros((144, 176), np.int16), np.zeros((144, 176), np.int16), 176, 144,
                                         mr, ctx=ctx)
    assert me.Create() == 0
