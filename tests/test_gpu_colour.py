"""GPU RGB24 -> YUV420 parity with the reference's golden fixtures and the
CPU oracle (bit-exact for the integer and both IEEE-double converters)."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu


def convert(vpp, ctx, kind, bgr, co, flip):
    h, w, _ = bgr.shape
    y = np.empty((h, w), np.int16)
    u = np.empty((h // 2, w // 2), np.int16)
    v = np.empty((h // 2, w // 2), np.int16)
    c = vpp.FastGpuRGB24toYUV420Converter(w, h, co, kind=kind, ctx=ctx)
    c.SetFlip(flip)
    c.Convert(bgr, y, u, v)
    return y, u, v


def test_against_golden(vpp, ctx, golden):
    g = golden("colour.npz")
    for kind in (0, 1, 2):
        for flip in (0, 1):
            for co in (0, 128):
                y, u, v = convert(vpp, ctx, kind, g["bgr"], co, flip)
                np.testing.assert_array_equal(y, g[f"k{kind}_f{flip}_c{co}_y"])
                np.testing.assert_array_equal(u, g[f"k{kind}_f{flip}_c{co}_u"])
                np.testing.assert_array_equal(v, g[f"k{kind}_f{flip}_c{co}_v"])


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("w,h", [(1920, 1080), (1922, 6), (2, 2), (1000, 750)])
def test_against_oracle(vpp, ctx, orc, kind, w, h):
    bgr = synth.rgb_frame(w + h + kind, w, h)
    for co in (0, 128):
        got = convert(vpp, ctx, kind, bgr, co, 0)
        want = orc.rgb_to_yuv(kind, bgr, co, 0)
        for a, b in zip(got, want):
            np.testing.assert_array_equal(a, b)


def test_extreme_colours(vpp, ctx, orc):
    """Saturated primaries exercise every clamp of the luma and chroma ranges."""
    vals = np.array([0, 1, 127, 128, 254, 255], np.uint8)
    b, g, r = np.meshgrid(vals, vals, vals, indexing="ij")
    px = np.stack([b.ravel(), g.ravel(), r.ravel()], -1)  # 216 colours
    bgr = np.repeat(np.repeat(px.reshape(6, 36, 3), 2, 0), 2, 1)  # each colour fills a 2x2 block
    for kind in (0, 1, 2):
        got = convert(vpp, ctx, kind, bgr, 128, 0)
        want = orc.rgb_to_yuv(kind, bgr, 128, 0)
        for a, bb in zip(got, want):
            np.testing.assert_array_equal(a, bb)
