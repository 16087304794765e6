"""GPU DC Hadamard transforms (FastForward/InverseDC4x4ITImpl1, DC2x2ITImpl1)
against the reference's golden fixtures and the CPU oracle, bit-exact."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [(4, "FastForwardDC4x4ITImpl1", "FastInverseDC4x4ITImpl1"),
         (2, "FastForwardDC2x2ITImpl1", "FastInverseDC2x2ITImpl1")]


@pytest.mark.parametrize("size,fwd_name,inv_name", SIZES)
def test_dc_all_qps_against_golden(vpp, ctx, golden, size, fwd_name, inv_name):
    g = golden("dc.npz")
    x = g[f"s{size}_x"]
    fwd, inv = getattr(vpp, fwd_name)(ctx), getattr(vpp, inv_name)(ctx)
    for qp in range(52):
        fwd.SetParameter(vpp.QUANT_ID, qp)
        inv.SetParameter(vpp.QUANT_ID, qp)
        lev = fwd.Transform(x.copy())
        np.testing.assert_array_equal(lev, g[f"s{size}_fwd_q{qp}"], err_msg=f"fwd qp{qp}")
        np.testing.assert_array_equal(inv.InverseTransform(lev), g[f"s{size}_inv_q{qp}"], err_msg=f"inv qp{qp}")


@pytest.mark.parametrize("size,fwd_name,inv_name", SIZES)
def test_dc_modes_and_scale_against_golden(vpp, ctx, golden, size, fwd_name, inv_name):
    g = golden("dc.npz")
    x, xi, wt = g[f"s{size}_x"], g[f"s{size}_xi"], g[f"s{size}_weight"]
    fwd, inv = getattr(vpp, fwd_name)(ctx), getattr(vpp, inv_name)(ctx)
    for qp in (0, 11, 23, 28, 35, 36, 51):
        fwd.SetParameter(vpp.QUANT_ID, qp)
        inv.SetParameter(vpp.QUANT_ID, qp)
        for mode in (1, 2):
            fwd.SetMode(mode)
            inv.SetMode(mode)
            np.testing.assert_array_equal(fwd.Transform(x.copy()), g[f"s{size}_fwd_m{mode}_q{qp}"])
            np.testing.assert_array_equal(inv.InverseTransform(xi.copy()), g[f"s{size}_inv_m{mode}_q{qp}"])
        inv.SetMode(0)
        inv.SetScale(wt)
        np.testing.assert_array_equal(inv.InverseTransform(xi.copy()), g[f"s{size}_invw_q{qp}"])
        inv.SetScale(np.full(size * size, 16, np.int32))


def test_dc_quantise_value(vpp, ctx, golden):
    g = golden("dc.npz")
    t = vpp.FastForwardDC4x4ITImpl1(ctx)
    for val, qp, want in g["quantise_value"]:
        assert t.QuantiseValue(int(val), 0, int(qp)) == want
    assert vpp.FastForwardDC2x2ITImpl1(ctx).QuantiseValue(100, 0, 28) == 0


@pytest.mark.parametrize("size", [4, 2])
def test_dc_device_large_and_unaligned_against_oracle(vpp, ctx, orc, size):
    """Many blocks through the device entry point (vector accesses), and the
    same blocks at an offset that forbids them (scalar accesses)."""
    import torch
    n = size * size
    rng = np.random.default_rng(100 + size)
    x = rng.integers(-32768, 32768, n * 50000).astype(np.int16)
    L = vpp.load()
    for qp in (0, 17, 28, 40, 51):
        for mode in (0, 1, 2):
            want = orc.fwd_dc(x, size, mode, qp)
            d = torch.from_numpy(x).cuda()
            assert L.vppgpu_fwd_dc_device(ctx.handle, C.c_void_p(d.data_ptr()), x.size // n, size, mode, qp) == 0
            torch.cuda.synchronize()
            np.testing.assert_array_equal(d.cpu().numpy(), want)
            # one short in: 2-byte aligned only
            d2 = torch.zeros(x.size + 1, dtype=torch.int16, device="cuda")
            d2[1:] = torch.from_numpy(x).cuda()
            assert L.vppgpu_fwd_dc_device(ctx.handle, C.c_void_p(d2.data_ptr() + 2), x.size // n, size, mode,
                                          qp) == 0
            torch.cuda.synchronize()
            np.testing.assert_array_equal(d2[1:].cpu().numpy(), want)
            xi = (x // 64).astype(np.int16)
            wt = rng.integers(1, 40, n).astype(np.int32)
            want_i = orc.inv_dc(xi, size, mode, qp, wt)
            di = torch.from_numpy(xi).cuda()
            assert L.vppgpu_inv_dc_device(ctx.handle, C.c_void_p(di.data_ptr()), xi.size // n, size, mode, qp,
                                          C.c_void_p(wt.ctypes.data)) == 0
            torch.cuda.synchronize()
            np.testing.assert_array_equal(di.cpu().numpy(), want_i)


def test_dc_argument_checks(vpp, ctx):
    L = vpp.load()
    x = np.zeros(16, np.int16)
    p = C.c_void_p(x.ctypes.data)
    assert L.vppgpu_fwd_dc(ctx.handle, p, 1, 3, 0, 28) != 0      # size
    assert L.vppgpu_fwd_dc(ctx.handle, p, 1, 4, 3, 28) != 0      # mode
    assert L.vppgpu_fwd_dc(ctx.handle, p, 1, 4, 0, 52) != 0      # qp
    assert L.vppgpu_inv_dc(ctx.handle, None, 1, 4, 0, 28, None) != 0
    assert L.vppgpu_fwd_dc(ctx.handle, p, 0, 4, 0, 28) == 0      # nothing to do
