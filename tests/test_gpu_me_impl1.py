"""GPU parity of MotionEstimatorImpl1 (the H.263-style full search with
half-pel refinement and the weighted zero-vector choice): half-pel vectors,
per-block distortions and avgDistortion bit-exact with the reference's golden
fixtures (16x16 and 8x8 blocks, ranges 7..32 pels) and with the CPU oracle on
further sizes and a 1080p frame."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth
from tests.golden.make_golden import umhs_frames

pytestmark = pytest.mark.gpu

CASES = ["qcif16_r16", "qcif8_r16", "cif16_r15", "small16_r7", "small8_r31", "qcif16_r32"]


def estimate(vpp, ctx, src, ref, bw, bh, rng):
    h, w = src.shape
    me = vpp.MotionEstimatorImpl1(src, ref, w, h, bw, bh, rng, ctx=ctx)
    assert me.Create() == 1
    mv, avg = me.Estimate()
    return mv, me.last_mb_distortion, avg


@pytest.mark.parametrize("case", CASES)
def test_against_golden(vpp, ctx, golden, case):
    g = golden("me_impl1.npz")
    w, h, bw, bh, rng = (int(v) for v in g[f"{case}_meta"])
    mv, dist, avg = estimate(vpp, ctx, g[f"{case}_src"].astype(np.int16), g[f"{case}_ref"].astype(np.int16), bw, bh,
                             rng)
    np.testing.assert_array_equal(mv, g[f"{case}_mv"])
    assert avg == int(g[f"{case}_avg"][0])


@pytest.mark.parametrize("seed,w,h,bw,bh,rng,gen", [(131, 176, 144, 16, 16, 12, "noisy"), (132, 208, 120, 8, 8, 20, "pan"),
                                                   (133, 128, 96, 16, 16, 1, "shift"), (134, 640, 368, 8, 8, 32, "noisy"),
                                                   (135, 1920, 1088, 16, 16, 16, "pan")])
def test_against_oracle(vpp, ctx, orc, seed, w, h, bw, bh, rng, gen):
    fr = umhs_frames(seed, w, h, gen)
    mv_o, dist_o, avg_o = orc.me_impl1(fr[1], fr[0], rng, bw, bh)
    mv, dist, avg = estimate(vpp, ctx, fr[1], fr[0], bw, bh, rng)
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(dist, dist_o)
    assert avg == avg_o


def test_limits(vpp, ctx):
    fr = synth.pan_sequence(3, 64, 48, 2)
    L = vpp.load()
    import ctypes as C
    h = C.c_void_p()
    assert L.vppgpu_me_create_blocks(ctx.handle, 9, 64, 48, 16, 16, 33, C.byref(h)) == -6  # range above 32
    assert L.vppgpu_me_create_blocks(ctx.handle, 9, 64, 40, 16, 16, 8, C.byref(h)) == -6   # partial block row
    assert L.vppgpu_me_create_blocks(ctx.handle, 9, 64, 48, 8, 16, 8, C.byref(h)) == -6    # 8x16 blocks
    assert L.vppgpu_me_create_blocks(ctx.handle, 0, 64, 48, 8, 8, 64, C.byref(h)) == -6    # other kinds: 16x16
    mv, _, _ = estimate(vpp, ctx, fr[1], fr[0], 16, 16, 8)
    assert mv.shape == (12, 2)


IMPL2_CASES = ["qcif_r16_m1", "qcif_r16_m2", "cif_r15_m2", "small_r8_m1", "cif_r32_m2", "wide_r20_m1"]


@pytest.mark.parametrize("case", IMPL2_CASES)
def test_impl2_against_golden(vpp, ctx, golden, case):
    """MotionEstimatorImpl2 (the SAD pyramid) against the reference's fixtures."""
    g = golden("me_impl2.npz")
    w, h, rng, mode = (int(v) for v in g[f"{case}_meta"])
    me = vpp.MotionEstimatorImpl2(g[f"{case}_src"].astype(np.int16), g[f"{case}_ref"].astype(np.int16), w, h, 16, 16,
                                  rng, ctx=ctx)
    assert me.Create() == 1
    me.SetMode(mode)
    mv, avg = me.Estimate()
    np.testing.assert_array_equal(mv, g[f"{case}_mv"])
    assert avg == int(g[f"{case}_avg"][0])


@pytest.mark.parametrize("seed,w,h,rng,mode,gen", [(161, 176, 144, 12, 1, "noisy"), (162, 352, 288, 24, 0, "pan"),
                                                  (163, 128, 96, 6, 2, "shift"), (164, 1920, 1088, 16, 0, "pan"),
                                                  (165, 640, 368, 32, 1, "noisy")])
def test_impl2_against_oracle(vpp, ctx, orc, seed, w, h, rng, mode, gen):
    fr = umhs_frames(seed, w, h, gen)
    mv_o, dist_o, avg_o = orc.me_impl2(fr[1], fr[0], rng, mode)
    me = vpp.MotionEstimatorImpl2(fr[1], fr[0], w, h, 16, 16, rng, ctx=ctx)
    assert me.Create() == 1
    me.SetMode(mode)
    mv, avg = me.Estimate()
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(me.last_mb_distortion, dist_o)
    assert avg == avg_o
