"""Autotuning (vppgpu_me_autotune): for every estimator kind the tuner picks a
launch shape / relaxation policy, and estimates afterwards still give the
oracle's vectors and distortions."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu

KINDS = [("MotionEstimatorH264ImplFull", "me_full", {}),
         ("MotionEstimatorH264ImplMultires", "me_multires", {"mode": 0}),
         ("MotionEstimatorH264ImplMultiresCross", "me_multires_cross", {"mode": 0}),
         ("MotionEstimatorH264ImplMultiresCrossVer2", "me_multires_cross_v2", {"mode": 0})]


@pytest.mark.parametrize("cls,ofn,kw", KINDS)
def test_autotune_keeps_results(vpp, ctx, orc, cls, ofn, kw):
    w, h = 640, 368
    fr = synth.pan_sequence(95, w, h, 3)
    me = getattr(vpp, cls)(fr[1], fr[0], w, h, 128, ctx=ctx)
    assert me.Create() == 1
    me.SetMode(0)
    before = me.tuning()
    t = me.Autotune(reps=1)
    assert t["choice"] >= 0
    assert set(t) >= set(before)
    for k in (1, 2):
        me._src, me._ref = fr[k], fr[k - 1]
        mv, _ = me.Estimate()
        mv_o, dist_o, _ = getattr(orc, ofn)(fr[k], fr[k - 1], 128, **kw)
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(me.last_mb_distortion, dist_o)
