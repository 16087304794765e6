"""GPU YUV420 -> RGB24 (the Real converters) against the reference's golden
fixtures and the CPU oracle, bit-exact, including every (u, v) chroma pair
(the cases the kernel evaluates in double)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CLASSES = [("RealYUV420toRGB24Converter", 0, 0), ("RealYUV420toRGB24ConverterImpl2", 1, 1),
           ("RealYUV420toRGB24CCIR601Converter", 2, 2), ("RealYUV420toRGB24ConverterImpl2Ver16", 1, 3),
           ("RealYUV420toRGB24CCIR601ConverterVer16", 2, 4)]


@pytest.mark.parametrize("cls,okind,gkind", CLASSES)
def test_yuv_to_rgb_against_golden(vpp, ctx, golden, cls, okind, gkind):
    g = golden("yuv2rgb.npz")
    for name in ("n", "wide"):
        if gkind == 0 and name == "wide":
            continue
        y, u, v = g[f"{name}_y"], g[f"{name}_u"], g[f"{name}_v"]
        h, w = y.shape
        c = getattr(vpp, cls)(w, h, ctx=ctx)
        c.SetChrominanceOffset(-128)
        for rot in (0, 1):
            for flip in (0, 1):
                c.SetRotate(rot)
                c.SetFlip(flip)
                want = g[f"{name}_k{gkind}_r{rot}_f{flip}"]
                out = np.zeros(w * h * 3, np.uint8)
                c.Convert(y, u, v, out)
                np.testing.assert_array_equal(out.reshape(want.shape), want, err_msg=f"{name} r{rot} f{flip}")


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("okind", [0, 1, 2])
def test_yuv_to_rgb_every_chroma_pair_against_oracle(vpp, ctx, orc, okind):
    """A 512x512 frame whose 256x256 chroma planes hold every (u, v) pair,
    through the vector kernel (rows), the flip and the rotate layouts."""
    import torch
    rng = np.random.default_rng(20 + okind)
    u = np.repeat(np.arange(256, dtype=np.int16)[:, None], 256, axis=1)
    v = np.repeat(np.arange(256, dtype=np.int16)[None, :], 256, axis=0)
    y = rng.integers(0, 256, (512, 512)).astype(np.int16)
    L = vpp.load()
    dy, du, dv = _dev(torch, y), _dev(torch, u), _dev(torch, v)
    for rot, flip in ((0, 0), (0, 1), (1, 0)):
        want = orc.yuv_to_rgb(okind, y, u, v, -128, rot, flip)
        out = torch.zeros(512 * 512 * 3, dtype=torch.uint8, device="cuda")
        assert L.vppgpu_yuv420_to_rgb24_device(ctx.handle, okind, C.c_void_p(dy.data_ptr()), C.c_void_p(du.data_ptr()),
                                               C.c_void_p(dv.data_ptr()), 512, 512, -128, rot, flip,
                                               C.c_void_p(out.data_ptr())) == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy().reshape(want.shape), want, err_msg=f"r{rot} f{flip}")


@pytest.mark.parametrize("okind", [1, 2])
def test_yuv_to_rgb_frames_wide_range_against_oracle(vpp, ctx, orc, okind):
    """Several 1920x1080 frames in one launch with samples outside 0..255."""
    import torch
    rng = np.random.default_rng(30 + okind)
    n, w, h = 3, 1920, 1080
    ys = rng.integers(-400, 700, (n, h, w)).astype(np.int16)
    us = rng.integers(-400, 700, (n, h // 2, w // 2)).astype(np.int16)
    vs = rng.integers(-400, 700, (n, h // 2, w // 2)).astype(np.int16)
    L = vpp.load()
    dy, du, dv = _dev(torch, ys), _dev(torch, us), _dev(torch, vs)
    out = torch.zeros(n * w * h * 3, dtype=torch.uint8, device="cuda")
    assert L.vppgpu_yuv420_to_rgb24_frames_device(ctx.handle, okind, C.c_void_p(dy.data_ptr()),
                                                  C.c_void_p(du.data_ptr()), C.c_void_p(dv.data_ptr()), n, w, h, 0,
                                                  0, 0, C.c_void_p(out.data_ptr())) == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(n, h, w, 3)
    for f in range(n):
        np.testing.assert_array_equal(got[f], orc.yuv_to_rgb(okind, ys[f], us[f], vs[f], 0, 0, 0), err_msg=f"frame {f}")


def test_yuv_to_rgb_odd_geometry_and_unaligned(vpp, ctx, orc):
    """Width not a multiple of 8 and an output offset by one byte take the
    one-block-per-thread kernel."""
    import torch
    rng = np.random.default_rng(40)
    L = vpp.load()
    for (w, h) in ((22, 14), (2, 2), (130, 66)):
        y = rng.integers(0, 256, (h, w)).astype(np.int16)
        u = rng.integers(0, 256, (h // 2, w // 2)).astype(np.int16)
        v = rng.integers(0, 256, (h // 2, w // 2)).astype(np.int16)
        for kind in (0, 1, 2):
            want = orc.yuv_to_rgb(kind, y, u, v, -128, 0, 0)
            dy, du, dv = _dev(torch, y), _dev(torch, u), _dev(torch, v)
            out = torch.zeros(w * h * 3 + 1, dtype=torch.uint8, device="cuda")
            assert L.vppgpu_yuv420_to_rgb24_device(ctx.handle, kind, C.c_void_p(dy.data_ptr()),
                                                   C.c_void_p(du.data_ptr()), C.c_void_p(dv.data_ptr()), w, h, -128,
                                                   0, 0, C.c_void_p(out.data_ptr() + 1)) == 0
            torch.cuda.synchronize()
            np.testing.assert_array_equal(out[1:].cpu().numpy().reshape(h, w, 3), want, err_msg=f"{w}x{h} k{kind}")


def test_yuv_to_rgb_argument_checks(vpp, ctx):
    L = vpp.load()
    a = np.zeros(64, np.int16)
    o = np.zeros(64 * 3, np.uint8)
    p = C.c_void_p(a.ctypes.data)
    assert L.vppgpu_yuv420_to_rgb24(ctx.handle, 5, p, p, p, 8, 8, 0, 0, 0, C.c_void_p(o.ctypes.data)) != 0  # no kind 5
    assert L.vppgpu_yuv420_to_rgb24(ctx.handle, 1, p, p, p, 7, 8, 0, 0, 0, C.c_void_p(o.ctypes.data)) != 0
    assert L.vppgpu_yuv420_to_rgb24(ctx.handle, 1, None, p, p, 8, 8, 0, 0, 0, C.c_void_p(o.ctypes.data)) != 0


SIX = [("Fast6BitYUV420toRGB24Converter", 3), ("Real6BitYUV420toRGB24Converter", 4)]


@pytest.mark.parametrize("cls,kind", SIX)
def test_six_bit_against_golden(vpp, ctx, golden, cls, kind):
    """The 6-bit converters: 6-bit samples, wider ones, and samples past
    +-16000 (Real6Bit's double path), rows and transpose; flip is ignored."""
    g = golden("yuv2rgb.npz")
    for name in ("six", "sixwide", "sixhuge"):
        y, u, v = g[f"{name}_y"], g[f"{name}_u"], g[f"{name}_v"]
        h, w = y.shape
        c = getattr(vpp, cls)(w, h, ctx=ctx)
        for rot in (0, 1):
            c.SetRotate(rot)
            c.SetFlip(1)
            want = g[f"{name}_k{kind}_r{rot}"]
            out = np.zeros(w * h * 3, np.uint8)
            c.Convert(y, u, v, out)
            np.testing.assert_array_equal(out.reshape(want.shape), want, err_msg=f"{name} r{rot}")


@pytest.mark.parametrize("cls,kind", SIX)
def test_six_bit_1080p_against_oracle(vpp, ctx, orc, cls, kind):
    from imagecodingutils_gb300 import synth
    w, h = 1920, 1080
    r = lambda seed, shape: ((synth.splitmix64(seed, int(np.prod(shape))) % np.uint64(64)).astype(np.int16)
                             .reshape(shape))
    y, u, v = r(90 + kind, (h, w)), r(91 + kind, (h // 2, w // 2)), r(92 + kind, (h // 2, w // 2))
    c = getattr(vpp, cls)(w, h, ctx=ctx)
    for rot in (0, 1):
        c.SetRotate(rot)
        out = np.zeros(w * h * 3, np.uint8)
        c.Convert(y, u, v, out)
        want = orc.yuv_to_rgb_6bit(kind, y, u, v, rot)
        np.testing.assert_array_equal(out.reshape(want.shape), want)


def test_zoom_against_golden_and_oracle(vpp, ctx, golden, orc):
    from imagecodingutils_gb300 import _lib, synth
    g = golden("yuv2rgb.npz")
    ZOOM_SIZES = [tuple(int(x) for x in p) for p in g["zoom_sizes"]]
    y, u, v = g["six_y"], g["six_u"], g["six_v"]
    h, w = y.shape
    c = vpp.Fast6BitYUV420toRGB24ZoomConverter(w, h, ctx=ctx)
    for ow, oh in ZOOM_SIZES:
        c.SetOutputDimensions(ow, oh)
        out = np.zeros(ow * oh * 3, np.uint8)
        c.Convert(y, u, v, out)
        np.testing.assert_array_equal(out.reshape(oh, ow, 3), g[f"zoom_{ow}x{oh}"], err_msg=f"{ow}x{oh}")
    c.SetOutputDimensions(2 * w, 2 * h)  # past the planes in the reference: refused
    with pytest.raises(vpp.VppGpuError) as e:
        c.Convert(y, u, v, np.zeros(4 * w * h * 3, np.uint8))
    assert e.value.status == _lib.ERR_UNSUPPORTED
    # a larger frame against the oracle: 1920x1080 to 1440x810 (3/4)
    W, H = 1920, 1080
    r = lambda seed, shape: ((synth.splitmix64(seed, int(np.prod(shape))) % np.uint64(64)).astype(np.int16)
                             .reshape(shape))
    y, u, v = r(95, (H, W)), r(96, (H // 2, W // 2)), r(97, (H // 2, W // 2))
    c = vpp.Fast6BitYUV420toRGB24ZoomConverter(W, H, ctx=ctx)
    c.SetOutputDimensions(1440, 810)
    out = np.zeros(1440 * 810 * 3, np.uint8)
    c.Convert(y, u, v, out)
    np.testing.assert_array_equal(out.reshape(810, 1440, 3), orc.yuv_to_rgb_zoom(y, u, v, 1440, 810))
