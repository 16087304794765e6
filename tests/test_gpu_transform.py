"""GPU 4x4 transform / quantisation parity with the reference's golden
fixtures and the CPU oracle (bit-exact)."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu


def test_forward_all_qps_against_golden(vpp, ctx, golden):
    g = golden("transform.npz")
    x = g["x"]
    for cls in (vpp.FastForward4x4ITImpl1, vpp.FastForward4x4ITImpl2):
        t = cls(ctx)
        for qp in range(52):
            for intra in (0, 1):
                t.SetParameter(1, intra)
                t.SetParameter(0, qp)
                np.testing.assert_array_equal(t.Transform(x.copy()), g[f"fwd_q{qp}_i{intra}"], err_msg=f"qp{qp} i{intra}")
    t16 = vpp.FastForward4x4On16x16ITImpl1(ctx)
    for qp in range(52):
        for intra in (0, 1):
            t16.SetParameter(1, intra)
            t16.SetParameter(0, qp)
            np.testing.assert_array_equal(t16.Transform(x.copy()), g[f"fwd16_q{qp}_i{intra}"])


def test_inverse_all_qps_against_golden(vpp, ctx, golden):
    g = golden("transform.npz")
    inv, inv16 = vpp.FastInverse4x4ITImpl1(ctx), vpp.FastInverse4x4On16x16ITImpl1(ctx)
    for qp in range(52):
        lev = g[f"fwd_q{qp}_i1"]
        inv.SetParameter(0, qp)
        inv16.SetParameter(0, qp)
        np.testing.assert_array_equal(inv.InverseTransform(lev.copy()), g[f"inv_q{qp}"], err_msg=f"qp{qp}")
        np.testing.assert_array_equal(inv16.InverseTransform(lev.copy()), g[f"inv16_q{qp}"], err_msg=f"qp{qp}")


def test_modes_and_scale_against_golden(vpp, ctx, golden):
    g = golden("transform.npz")
    x = g["x"]
    fwd, inv, inv16 = vpp.FastForward4x4ITImpl1(ctx), vpp.FastInverse4x4ITImpl1(ctx), vpp.FastInverse4x4On16x16ITImpl1(ctx)
    for qp in (0, 11, 23, 24, 28, 51):
        for mode in (1, 2):
            fwd.SetMode(mode); fwd.SetParameter(0, qp); fwd.SetParameter(1, 1)
            np.testing.assert_array_equal(fwd.Transform(x.copy()), g[f"fwd_m{mode}_q{qp}"])
            inv.SetMode(mode); inv.SetParameter(0, qp)
            np.testing.assert_array_equal(inv.InverseTransform(x.copy()), g[f"inv_m{mode}_q{qp}"])
            inv16.SetMode(mode); inv16.SetParameter(0, qp)
            np.testing.assert_array_equal(inv16.InverseTransform(x.copy()), g[f"inv16_m{mode}_q{qp}"])
        w = vpp.FastInverse4x4ITImpl1(ctx)
        w.SetScale(g["weight"])
        w.SetParameter(0, qp)
        np.testing.assert_array_equal(w.InverseTransform(g[f"fwd_q{qp}_i0"].copy()), g[f"invw_q{qp}"])


@pytest.mark.parametrize("qp,intra,order", [(0, 1, 0), (17, 0, 0), (28, 0, 1), (51, 1, 1), (23, 1, 0), (24, 0, 1)])
def test_plane_roundtrip_1080p_against_oracle(vpp, ctx, orc, qp, intra, order):
    """Full-size 1920x1080 residual plane: levels and reconstruction of every
    4x4 block equal the oracle's block-by-block result."""
    w, h = 1920, 1080
    res = synth.residual_blocks(100 + qp, w * h).reshape(h, w)
    lev, rec = vpp.tq_roundtrip_plane(res, qp, intra, inv_order=order, ctx=ctx)
    blocks = res.reshape(h // 4, 4, w // 4, 4).transpose(0, 2, 1, 3).reshape(-1, 16)
    lev_o = orc.fwd4x4(blocks, 0, 0, qp, intra)
    if order == 0:
        rec_o = orc.inv4x4(lev_o, 0, 0, qp)
    else:
        # column-first order is the On16x16 class's: evaluate it per block by
        # placing each block in the top-left corner of a 16x16 macroblock
        mbs = np.zeros((lev_o.shape[0], 16, 16), np.int16)
        mbs[:, :4, :4] = lev_o.reshape(-1, 4, 4)
        rec_o = orc.inv4x4(mbs.reshape(-1, 256), 1, 0, qp).reshape(-1, 16, 16)[:, :4, :4].reshape(-1, 16)
    back = lambda b: b.reshape(h // 4, w // 4, 4, 4).transpose(0, 2, 1, 3).reshape(h, w)
    np.testing.assert_array_equal(lev, back(lev_o))
    np.testing.assert_array_equal(rec, back(rec_o))


def test_int16_wraparound_inputs(vpp, ctx, orc):
    """Full-range int16 inputs overflow the 16-bit intermediates; the wrap
    points must match."""
    x = ((synth.splitmix64(77, 16 * 4096) % np.uint64(65536)).astype(np.int64) - 32768).astype(np.int16)
    for qp in (0, 30, 51):
        t = vpp.FastForward4x4ITImpl1(ctx)
        t.SetParameter(0, qp)
        np.testing.assert_array_equal(t.Transform(x.copy()), orc.fwd4x4(x, 0, 0, qp, 1))
        i = vpp.FastInverse4x4ITImpl1(ctx)
        i.SetParameter(0, qp)
        np.testing.assert_array_equal(i.InverseTransform(x.copy()), orc.inv4x4(x, 0, 0, qp))


def test_empty_input(vpp, ctx):
    t = vpp.FastForward4x4ITImpl1(ctx)
    assert t.Transform(np.zeros(0, np.int16)).size == 0
