"""The CPU oracle against the golden fixtures produced by the reference itself
(tests/golden/make_golden.py), and -- where oracle/_ref was built -- against
the compiled reference on further seeded cases."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth
from oracle import oracle as oracle_mod

ME_CASES = ["qcif_r64", "qcif_r128", "cif_r128", "partial_r128", "shift_r64"]


@pytest.mark.parametrize("case", ME_CASES)
def test_me_full_matches_reference_vectors(orc, golden, case):
    g = golden("me_full.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    incl = np.ones((w // 16) * (h // 16), np.uint8)
    mv, dist, avg = orc.me_full(src, ref, mr, dist_incl=incl)
    np.testing.assert_array_equal(mv, g[f"{case}_mv"])
    assert avg == int(g[f"{case}_avg"][0])
    # without pDistortionIncluded the reference reports 0
    mv2, _, avg2 = orc.me_full(src, ref, mr)
    np.testing.assert_array_equal(mv2, mv)
    assert avg2 == 0


@pytest.mark.parametrize("case", ["config1", "cif_r128", "partial_r64", "tiles_r64", "tiles_r128"])
def test_me_full_sad_matches_reference(orc, golden, case):
    """The integer-pel SAD stage (vo_me_full_intpel, metric 1) against the
    reference's own stage on its overlays (Tad16x16 / Tad16x16LessThan)."""
    g = golden("me_full_sad.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    frames = g[f"{case}_frames"].astype(np.int16)
    for t in range(len(frames) - 1):
        mv, dist = orc.me_full_intpel(frames[t + 1], frames[t], mr, metric=1)
        np.testing.assert_array_equal(mv, g[f"{case}_mv"][t])
        np.testing.assert_array_equal(dist, g[f"{case}_dist"][t])
        assert int(dist.sum()) // dist.size == int(g[f"{case}_avg"][t])


def test_me_full_sad_matches_compiled_reference():
    """Further seeded pairs against the compiled reference (where oracle/_ref exists)."""
    if not oracle_mod.Reference.available():
        pytest.skip("oracle/_ref not built here")
    orc, ref = oracle_mod.Oracle(), oracle_mod.Reference()
    for seed, w, h, mr, gen in [(41, 208, 120, 48, synth.pan_sequence), (42, 96, 64, 128, synth.tile_sequence),
                                (43, 176, 144, 64, synth.shift_sequence)]:
        fr = gen(seed, w, h, 2)
        mv, dist = orc.me_full_intpel(fr[1], fr[0], mr, metric=1)
        mv_r, dist_r, _ = ref.me_full_sad(fr[1], fr[0], mr)
        np.testing.assert_array_equal(mv, mv_r)
        np.testing.assert_array_equal(dist, dist_r)


def test_me_full_matches_reference_per_mb_distortion(orc, golden):
    g = golden("me_full.npz")
    src = g["qcif_r64_src"].astype(np.int16)
    ref = g["qcif_r64_ref"].astype(np.int16)
    _, dist, _ = orc.me_full(src, ref, 64, dist_incl=np.ones(99, np.uint8))
    np.testing.assert_array_equal(dist, g["qcif_r64_mbdist"])


def test_transform_matches_reference(orc, golden):
    g = golden("transform.npz")
    x = g["x"]
    for qp in range(52):
        for intra in (0, 1):
            np.testing.assert_array_equal(orc.fwd4x4(x, 0, 0, qp, intra), g[f"fwd_q{qp}_i{intra}"])
            np.testing.assert_array_equal(orc.fwd4x4(x, 1, 0, qp, intra), g[f"fwd16_q{qp}_i{intra}"])
        lev = g[f"fwd_q{qp}_i1"]
        np.testing.assert_array_equal(orc.inv4x4(lev, 0, 0, qp), g[f"inv_q{qp}"])
        np.testing.assert_array_equal(orc.inv4x4(lev, 1, 0, qp), g[f"inv16_q{qp}"])
    for qp in (0, 11, 23, 24, 28, 51):
        for mode in (1, 2):
            np.testing.assert_array_equal(orc.fwd4x4(x, 0, mode, qp, 1), g[f"fwd_m{mode}_q{qp}"])
            np.testing.assert_array_equal(orc.inv4x4(x, 0, mode, qp), g[f"inv_m{mode}_q{qp}"])
            np.testing.assert_array_equal(orc.inv4x4(x, 1, mode, qp), g[f"inv16_m{mode}_q{qp}"])
        np.testing.assert_array_equal(orc.inv4x4(g[f"fwd_q{qp}_i0"], 0, 0, qp, g["weight"]), g[f"invw_q{qp}"])
    for val, pos, qp, intra, want in g["quantise_value"]:
        assert orc.quantise_value(int(val), int(pos), int(qp), int(intra)) == want


@pytest.mark.parametrize("size", [4, 2])
def test_dc_transforms_match_reference(orc, golden, size):
    """FastForward/InverseDC4x4ITImpl1 (size 4) and DC2x2ITImpl1 (size 2)."""
    g = golden("dc.npz")
    x, xi, wt = g[f"s{size}_x"], g[f"s{size}_xi"], g[f"s{size}_weight"]
    for qp in range(52):
        np.testing.assert_array_equal(orc.fwd_dc(x, size, 0, qp), g[f"s{size}_fwd_q{qp}"], err_msg=f"qp{qp}")
        np.testing.assert_array_equal(orc.inv_dc(g[f"s{size}_fwd_q{qp}"], size, 0, qp), g[f"s{size}_inv_q{qp}"])
    for qp in (0, 11, 23, 28, 35, 36, 51):
        for mode in (1, 2):
            np.testing.assert_array_equal(orc.fwd_dc(x, size, mode, qp), g[f"s{size}_fwd_m{mode}_q{qp}"])
            np.testing.assert_array_equal(orc.inv_dc(xi, size, mode, qp), g[f"s{size}_inv_m{mode}_q{qp}"])
        np.testing.assert_array_equal(orc.inv_dc(xi, size, 0, qp, wt), g[f"s{size}_invw_q{qp}"])
    if size == 4:
        for val, qp, want in g["quantise_value"]:
            assert orc.dc_quantise_value(int(val), int(qp)) == want


def test_dc_transforms_against_compiled_reference(orc):
    if not oracle_mod.Reference.available():
        pytest.skip("oracle/_ref not built (the reference sources are absent here)")
    ref = oracle_mod.Reference()
    rng = np.random.default_rng(7)
    for size in (4, 2):
        n = size * size
        x = rng.integers(-32768, 32768, n * 200).astype(np.int16)
        xi = rng.integers(-512, 513, n * 200).astype(np.int16)
        for qp in range(0, 52, 3):
            for mode in (0, 1, 2):
                np.testing.assert_array_equal(orc.fwd_dc(x, size, mode, qp), ref.fwd_dc(x, size, mode, qp))
                np.testing.assert_array_equal(orc.inv_dc(xi, size, mode, qp), ref.inv_dc(xi, size, mode, qp))


def test_yuv_to_rgb_matches_reference(orc, golden):
    """Oracle kinds 0-2 against the five Real converters (Ver16 classes share
    the Impl2 / CCIR601 arithmetic)."""
    g = golden("yuv2rgb.npz")
    for name in ("n", "wide"):
        y, u, v = g[f"{name}_y"], g[f"{name}_u"], g[f"{name}_v"]
        for kind, okind in ((0, 0), (1, 1), (2, 2), (3, 1), (4, 2)):
            if kind == 0 and name == "wide":
                continue
            for rot in (0, 1):
                for flip in (0, 1):
                    np.testing.assert_array_equal(orc.yuv_to_rgb(okind, y, u, v, -128, rot, flip),
                                                  g[f"{name}_k{kind}_r{rot}_f{flip}"], err_msg=f"{name} k{kind}")


def test_six_bit_yuv_to_rgb_matches_reference(orc, golden):
    """Fast6BitYUV420toRGB24Converter (kind 3) and Real6BitYUV420toRGB24Converter
    (kind 4) on 6-bit samples, samples past that range and samples past +-16000,
    both layouts; Fast6BitYUV420toRGB24ZoomConverter at several output sizes."""
    g = golden("yuv2rgb.npz")
    ZOOM_SIZES = [tuple(int(x) for x in p) for p in g["zoom_sizes"]]
    for name in ("six", "sixwide", "sixhuge"):
        y, u, v = g[f"{name}_y"], g[f"{name}_u"], g[f"{name}_v"]
        for kind in (3, 4):
            for rot in (0, 1):
                np.testing.assert_array_equal(orc.yuv_to_rgb_6bit(kind, y, u, v, rot), g[f"{name}_k{kind}_r{rot}"],
                                              err_msg=f"{name} k{kind} r{rot}")
    y, u, v = g["six_y"], g["six_u"], g["six_v"]
    for ow, oh in ZOOM_SIZES:
        np.testing.assert_array_equal(orc.yuv_to_rgb_zoom(y, u, v, ow, oh), g[f"zoom_{ow}x{oh}"], err_msg=f"{ow}x{oh}")
    with pytest.raises(ValueError):  # a 2x zoom: the reference reads past its planes
        orc.yuv_to_rgb_zoom(y, u, v, 2 * y.shape[1], 2 * y.shape[0])


def test_colour_matches_reference(orc, golden):
    g = golden("colour.npz")
    for kind in (0, 1, 2):
        for flip in (0, 1):
            for co in (0, 128):
                y, u, v = orc.rgb_to_yuv(kind, g["bgr"], co, flip)
                np.testing.assert_array_equal(y, g[f"k{kind}_f{flip}_c{co}_y"])
                np.testing.assert_array_equal(u, g[f"k{kind}_f{flip}_c{co}_u"])
                np.testing.assert_array_equal(v, g[f"k{kind}_f{flip}_c{co}_v"])


def test_inverse_pass_orders_differ(orc):
    """The two inverse classes round differently (int16 stores between passes
    in a different order), so both must be reproduced."""
    x = synth.residual_blocks(99, 16 * 256)
    lev = orc.fwd4x4(x, 0, 0, 4, 1)
    assert not np.array_equal(orc.inv4x4(lev, 0, 0, 4), orc.inv4x4(lev, 1, 0, 4))


ref_available = pytest.mark.skipif(not oracle_mod.Reference.available(), reason="reference not built here")


@ref_available
@pytest.mark.parametrize("seed,w,h,mr", [(31, 64, 48, 128), (32, 80, 64, 64), (33, 48, 40, 40), (34, 32, 32, 128)])
def test_me_full_against_compiled_reference(orc, seed, w, h, mr):
    ref_lib = oracle_mod.Reference()
    fr = synth.pan_sequence(seed, w, h, 2)
    incl = (synth.splitmix64(seed, (w // 16) * (h // 16)) & np.uint64(1)).astype(np.uint8)
    mv_r, avg_r = ref_lib.me("full", fr[1], fr[0], mr, dist_incl=incl)
    mv_o, _, avg_o = orc.me_full(fr[1], fr[0], mr, dist_incl=incl)
    np.testing.assert_array_equal(mv_o, mv_r)
    assert avg_o == avg_r


@ref_available
def test_me_full_flat_content_ties(orc):
    """Flat and periodic content makes many exact ties: the prediction-based
    tie-break decides the vectors."""
    ref_lib = oracle_mod.Reference()
    w, h = 96, 64
    yy, xx = np.mgrid[0:h, 0:w]
    a = ((xx // 8 + yy // 8) % 2 * 40 + 100).astype(np.int16)
    b = np.roll(a, (3, 5), axis=(0, 1))
    b[20:40, 30:60] = 128
    mv_r, _ = ref_lib.me("full", b, a, 128)
    mv_o, _, _ = orc.me_full(b, a, 128)
    np.testing.assert_array_equal(mv_o, mv_r)


MRC_CASES = ["qcif_r64", "cif_r128", "partial_r128", "small_r32"]


@pytest.mark.parametrize("case", MRC_CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_me_multires_cross_matches_reference(orc, golden, case, mode):
    g = golden("me_mrc.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    mv, _, avg = orc.me_multires_cross(src, ref, mr, mode=mode)
    np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"])
    assert avg == int(g[f"{case}_m{mode}_avg"][0])
    mvi, _, avgi = orc.me_multires_cross(src, ref, mr, mode=mode, dist_incl=np.ones((w // 16) * (h // 16), np.uint8))
    np.testing.assert_array_equal(mvi, mv)
    assert avgi == int(g[f"{case}_m{mode}_avg"][1])


H263_CASES = ["qcif_r32", "cif_r64", "partial_r64", "small_r16"]


@pytest.mark.parametrize("case", H263_CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_me_h263_multires_cross_matches_reference(orc, golden, case, mode):
    """MotionEstimatorH263ImplMultiresCross (half-pel ranges and vectors)."""
    g = golden("me_h263mrc.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    mv, _, avg = orc.me_h263_multires_cross(src, ref, mr, mode=mode)
    np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"])
    assert avg == int(g[f"{case}_m{mode}_avg"][0])
    mvi, _, avgi = orc.me_h263_multires_cross(src, ref, mr, mode=mode,
                                               dist_incl=np.ones((w // 16) * (h // 16), np.uint8))
    np.testing.assert_array_equal(mvi, mv)
    assert avgi == int(g[f"{case}_m{mode}_avg"][1])


H263V2_CASES = ["qcif_r32", "cif_r64", "partial_r64", "small_r16", "wide_r48"]


@pytest.mark.parametrize("case", H263V2_CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_me_h263_multires_cross_ver2_matches_reference(orc, golden, case, mode):
    """MotionEstimatorH263ImplMultiresCrossVer2 (H.263 median predictor over the
    vectors written so far, the y-sum quirk of its tie rule, the clamped
    half-pel prediction against the zero vector)."""
    g = golden("me_h263mrc2.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    mv, _, avg = orc.me_h263_multires_cross_ver2(src, ref, mr, mode=mode)
    np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"])
    assert avg == int(g[f"{case}_m{mode}_avg"][0])
    mvi, _, avgi = orc.me_h263_multires_cross_ver2(src, ref, mr, mode=mode, dist_incl=g[f"{case}_incl"])
    np.testing.assert_array_equal(mvi, mv)
    assert avgi == int(g[f"{case}_m{mode}_avg"][1])


def test_me_h263_multires_cross_ver2_1080p_matches_reference(orc, golden, hd_golden):
    g = golden("me_h263mrc2.npz")
    assert g["hd_frames_sha256"].tobytes() == hd_golden["g"]["frames_sha256"].tobytes()
    fr = hd_golden["frames"]
    for mode in (0, 1):
        mv, _, avg = orc.me_h263_multires_cross_ver2(fr[1], fr[0], int(g["hd_meta"][3]), mode=mode)
        np.testing.assert_array_equal(mv, g[f"hd_m{mode}_mv"])
        assert avg == int(g[f"hd_m{mode}_avg"][0])


@ref_available
@pytest.mark.parametrize("seed,w,h,mr,mode,gen", [(71, 176, 144, 64, 2, "noisy"), (72, 640, 360, 64, 0, "pan"),
                                                 (73, 96, 64, 16, 1, "noisy"), (74, 320, 176, 40, 2, "shift")])
def test_me_h263_multires_cross_ver2_against_compiled_reference(orc, seed, w, h, mr, mode, gen):
    from tests.golden.make_golden import umhs_frames
    fr = umhs_frames(seed, w, h, gen)
    r = oracle_mod.Reference()
    incl = (synth.splitmix64(seed, (w // 16) * (h // 16)) & np.uint64(1)).astype(np.uint8)
    for dist_incl in (None, incl):
        mv, _, avg = orc.me_h263_multires_cross_ver2(fr[1], fr[0], mr, mode=mode, dist_incl=dist_incl)
        mv_r, avg_r = r.me("h263_multires_cross_v2", fr[1], fr[0], mr, mode=mode, dist_incl=dist_incl)
        np.testing.assert_array_equal(mv, mv_r)
        assert avg == avg_r


MRC2_CASES = ["qcif_r64", "cif_r128", "partial_r128", "small_r32", "shift_r128"]


@pytest.mark.parametrize("case", MRC2_CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_me_multires_cross_v2_matches_reference(orc, golden, case, mode):
    g = golden("me_mrc2.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    mv, _, avg = orc.me_multires_cross_v2(src, ref, mr, mode=mode)
    np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"])
    assert avg == 0  # no pDistortionIncluded: nothing is counted
    mvi, _, avgi = orc.me_multires_cross_v2(src, ref, mr, mode=mode, dist_incl=g[f"{case}_incl"])
    np.testing.assert_array_equal(mvi, mv)
    assert avgi == int(g[f"{case}_m{mode}_avg"][0])


@pytest.mark.parametrize("case", MRC2_CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_me_multires_cross_v2_lambda_matches_reference(orc, golden, case, mode):
    """Ver2's Estimate(long*, void* lambda) at lambdas 0, 0.9, 2.5 and 20:
    GetBestVector at every level, then the final choice with that lambda."""
    g, gl = golden("me_mrc2.npz"), golden("me_mrc2_lambda.npz")
    mr = int(g[f"{case}_meta"][2])
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    plain = orc.me_multires_cross_v2(src, ref, mr, mode=mode)[0]
    differs = 0
    for li, lam in enumerate(gl["lambdas"]):
        mv, _, avg = orc.me_multires_cross_v2_lambda(src, ref, mr, float(lam), mode=mode, dist_incl=g[f"{case}_incl"])
        np.testing.assert_array_equal(mv, gl[f"{case}_m{mode}_l{li}_mv"], err_msg=f"lambda {lam}")
        assert avg == int(gl[f"{case}_m{mode}_l{li}_avg"][0])
        differs += int((mv != plain).any(axis=1).sum())
    if case != "small_r32":
        assert differs > 0  # the overload is not Estimate(long*) under another name


def test_me_multires_cross_v2_lambda_1080p_matches_reference(orc, hd_golden, golden):
    """The lambda overload on pair 0 of the 1080p benchmark sequence."""
    gl = golden("me_mrc2_lambda.npz")
    fr, mr = hd_golden["frames"], hd_golden["motion_range"]
    assert gl["hd_frames_sha256"].tobytes() == hd_golden["g"]["frames_sha256"].tobytes()
    incl = np.ones((hd_golden["w"] // 16) * (hd_golden["h"] // 16), np.uint8)
    for mode in (1, 2):
        for lam in (0.9, 4.0):
            mv, _, avg = orc.me_multires_cross_v2_lambda(fr[1], fr[0], mr, lam, mode=mode, dist_incl=incl)
            np.testing.assert_array_equal(mv, gl[f"hd_m{mode}_lam{lam:g}_mv"], err_msg=f"mode {mode} lambda {lam}")
            assert avg == int(gl[f"hd_m{mode}_lam{lam:g}_avg"][0])


@ref_available
@pytest.mark.parametrize("seed,w,h,mr,mode,lam", [(56, 176, 144, 128, 0, 1.5), (57, 352, 288, 64, 1, 0.25),
                                                  (58, 208, 120, 96, 2, 7.0), (59, 96, 64, 64, 2, -0.5),
                                                  (60, 640, 360, 128, 1, 3.0)])
def test_me_multires_cross_v2_lambda_against_compiled_reference(orc, seed, w, h, mr, mode, lam):
    """Other sizes, ranges and lambdas (a negative one too), with a random
    inclusion map."""
    ref_lib = oracle_mod.Reference()
    fr = synth.pan_sequence(seed, w, h, 2)
    incl = (synth.splitmix64(seed, (w // 16) * (h // 16)) & np.uint64(1)).astype(np.uint8)
    mv_r, avg_r = ref_lib.me("multires_cross_v2", fr[1], fr[0], mr, mode=mode, dist_incl=incl, lam=lam)
    mv_o, _, avg_o = orc.me_multires_cross_v2_lambda(fr[1], fr[0], mr, lam, mode=mode, dist_incl=incl)
    np.testing.assert_array_equal(mv_o, mv_r)
    assert avg_o == avg_r


@pytest.mark.parametrize("case", MRC2_CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_me_cross_matches_reference(orc, golden, case, mode):
    """MotionEstimatorH264ImplCross (mode 0 quarter, 1 half, 2 full pel)."""
    g = golden("me_cross.npz")
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    mr = int(g[f"{case}_meta"][2])
    mv, _, avg = orc.me_cross(src, ref, mr, mode=mode)
    np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"])
    assert avg == 0
    mvi, _, avgi = orc.me_cross(src, ref, mr, mode=mode, dist_incl=g[f"{case}_incl"])
    np.testing.assert_array_equal(mvi, mv)
    assert avgi == int(g[f"{case}_m{mode}_avg"][0])


@ref_available
def test_me_cross_flat_content_ties(orc):
    """Periodic content: the cross search meets exact ties that the rounded
    prediction decides."""
    ref_lib = oracle_mod.Reference()
    w, h = 128, 96
    yy, xx = np.mgrid[0:h, 0:w]
    a = ((xx // 8 + yy // 8) % 2 * 40 + 100).astype(np.int16)
    b = np.roll(a, (3, 5), axis=(0, 1))
    b[20:40, 30:60] = 128
    for mode in (0, 1, 2):
        mv_r, _ = ref_lib.me("cross", b, a, 128, mode=mode)
        mv_o, _, _, ties = orc.me_cross(b, a, 128, mode=mode, with_ties=True)
        assert ties.sum() > 0
        np.testing.assert_array_equal(mv_o, mv_r)


@ref_available
@pytest.mark.parametrize("seed,w,h,mr,mode", [(51, 176, 144, 128, 0), (52, 352, 288, 128, 1), (53, 208, 120, 96, 2),
                                              (54, 96, 64, 64, 2), (55, 640, 360, 128, 0)])
def test_me_multires_cross_v2_against_compiled_reference(orc, seed, w, h, mr, mode):
    ref_lib = oracle_mod.Reference()
    fr = synth.pan_sequence(seed, w, h, 2)
    incl = (synth.splitmix64(seed, (w // 16) * (h // 16)) & np.uint64(1)).astype(np.uint8)
    mv_r, avg_r = ref_lib.me("multires_cross_v2", fr[1], fr[0], mr, mode=mode, dist_incl=incl)
    mv_o, _, avg_o = orc.me_multires_cross_v2(fr[1], fr[0], mr, mode=mode, dist_incl=incl)
    np.testing.assert_array_equal(mv_o, mv_r)
    assert avg_o == avg_r


@ref_available
def test_me_multires_cross_v2_flat_content_ties(orc):
    """Periodic content with flat patches: many exact ties, decided by the
    distance to each level's rounded prediction."""
    ref_lib = oracle_mod.Reference()
    w, h = 128, 96
    yy, xx = np.mgrid[0:h, 0:w]
    a = ((xx // 8 + yy // 8) % 2 * 40 + 100).astype(np.int16)
    b = np.roll(a, (3, 5), axis=(0, 1))
    b[20:40, 30:60] = 128
    for mode in (1, 2):
        mv_r, _ = ref_lib.me("multires_cross_v2", b, a, 128, mode=mode)
        mv_o, _, _, ties = orc.me_multires_cross_v2(b, a, 128, mode=mode, with_ties=True)
        np.testing.assert_array_equal(mv_o, mv_r)
        assert ties.sum() > 0


@pytest.mark.parametrize("case", MRC2_CASES)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_me_multires_matches_reference(orc, golden, case, mode):
    g = golden("me_mr.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    src = g[f"{case}_src"].astype(np.int16)
    ref = g[f"{case}_ref"].astype(np.int16)
    mv, _, avg = orc.me_multires(src, ref, mr, mode=mode)
    np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"])
    assert avg == 0
    mvi, _, avgi = orc.me_multires(src, ref, mr, mode=mode, dist_incl=g[f"{case}_incl"])
    np.testing.assert_array_equal(mvi, mv)
    assert avgi == int(g[f"{case}_m{mode}_avg"][0])


@ref_available
@pytest.mark.parametrize("seed,w,h,mr,mode", [(56, 176, 144, 128, 0), (57, 352, 288, 128, 1), (58, 208, 120, 96, 2),
                                              (59, 640, 360, 128, 0)])
def test_me_multires_against_compiled_reference(orc, seed, w, h, mr, mode):
    ref_lib = oracle_mod.Reference()
    fr = synth.pan_sequence(seed, w, h, 2)
    incl = (synth.splitmix64(seed, (w // 16) * (h // 16)) & np.uint64(1)).astype(np.uint8)
    mv_r, avg_r = ref_lib.me("multires", fr[1], fr[0], mr, mode=mode, dist_incl=incl)
    mv_o, _, avg_o = orc.me_multires(fr[1], fr[0], mr, mode=mode, dist_incl=incl)
    np.testing.assert_array_equal(mv_o, mv_r)
    assert avg_o == avg_r


MC_CASES = ["qcif_r16", "cif_r32", "small_r8"]


@pytest.mark.parametrize("case", MC_CASES)
def test_mc_compensate_matches_reference(orc, golden, case):
    g = golden("mc.npz")
    w, h, rg = (int(v) for v in g[f"{case}_meta"])
    y, u, v = (g[f"{case}_{k}"].astype(np.int16) for k in ("y", "u", "v"))
    cy, cu, cv = orc.mc_compensate(y, u, v, g[f"{case}_mv"], rg)
    np.testing.assert_array_equal(cy, g[f"{case}_cy"])
    np.testing.assert_array_equal(cu, g[f"{case}_cu"])
    np.testing.assert_array_equal(cv, g[f"{case}_cv"])


@ref_available
def test_mc_compensate_against_compiled_reference(orc):
    ref_lib = oracle_mod.Reference()
    w, h, rg = 640, 352, 32
    y = synth.pan_sequence(64, w, h, 1)[0]
    u = synth.pan_sequence(65, w // 2, h // 2, 1)[0]
    v = synth.pan_sequence(66, w // 2, h // 2, 1)[0]
    nmb = (w // 16) * (h // 16)
    mv = ((synth.splitmix64(67, 2 * nmb) % np.uint64(8 * rg + 1)).astype(np.int64) - 4 * rg).astype(np.int16)
    mv = mv.reshape(nmb, 2)
    for a, b in zip(orc.mc_compensate(y, u, v, mv, rg), ref_lib.mc_compensate(y, u, v, mv, rg)):
        np.testing.assert_array_equal(a, b)


def test_add_clip_and_sub(orc):
    rng = np.random.default_rng(7)
    a = rng.integers(0, 256, 1000).astype(np.int16)
    r = rng.integers(-300, 300, 1000).astype(np.int16)
    np.testing.assert_array_equal(orc.add_clip255(a, r), np.clip(a.astype(np.int32) + r, 0, 255))
    np.testing.assert_array_equal(orc.sub(a, r), (a.astype(np.int32) - r).astype(np.int16))


HD_PORT = {"full": "me_full", "multires_cross": "me_multires_cross", "multires_cross_v2": "me_multires_cross_v2",
           "multires": "me_multires", "cross": "me_cross"}


def test_port_matches_reference_at_1080p(orc, hd_golden):
    """The headline size: the oracle port against the compiled reference's
    1080p fixtures (the benchmark's own frame pairs, motionRange 128) for every
    estimator and mode, and for the integer-pel SAD stage."""
    from concurrent.futures import ThreadPoolExecutor

    g, fr, mr = hd_golden["g"], hd_golden["frames"], hd_golden["motion_range"]
    nmb = (hd_golden["w"] // 16) * (hd_golden["h"] // 16)
    incl = np.ones(nmb, np.uint8)
    keys = sorted({k.rsplit("_", 1)[0] for k in g if k.startswith("p") and k.endswith("_mv")})

    def run(key):  # key: p<pair>_<estimator>_m<mode>, or p<pair>_full_sad
        pair, est = key[1:].split("_", 1)
        src, ref = fr[int(pair) + 1], fr[int(pair)]
        if est == "full_sad":
            mv, dist = orc.me_full_intpel(src, ref, mr, metric=1)
            return key, mv, int(dist.sum()) // nmb, dist
        kind, mode = est.rsplit("_m", 1)
        kw = {} if kind == "full" else {"mode": int(mode)}
        mv, _, avg = getattr(orc, HD_PORT[kind])(src, ref, mr, dist_incl=incl, **kw)
        return key, mv, avg, None

    with ThreadPoolExecutor(8) as ex:  # ctypes releases the GIL: one estimate per thread
        results = list(ex.map(run, keys))
    assert len(results) == 3 * 12
    for key, mv, avg, dist in results:
        np.testing.assert_array_equal(mv, g[f"{key}_mv"], err_msg=key)
        assert avg == int(g[f"{key}_avg"][0]), key
        if dist is not None:
            np.testing.assert_array_equal(dist, g[f"{key}_dist"], err_msg=key)


UMHS_CASES = ["qcif_r64", "cif_r128", "shift_r128", "noisy_r128", "small_r32"]


@pytest.mark.parametrize("case", UMHS_CASES)
def test_me_umhs_matches_reference(orc, golden, case):
    """MotionEstimatorH264ImplUMHS: vectors, the distortion stored with each
    vector for the predictor, and the average, modes 0/1/2 with previous-frame
    vectors and intra flags, and once without either."""
    g = golden("me_umhs.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    src, ref = g[f"{case}_src"].astype(np.int16), g[f"{case}_ref"].astype(np.int16)
    for mode in (0, 1, 2):
        mv, dist, avg = orc.me_umhs(src, ref, mr, mode=mode, dist_incl=g[f"{case}_incl"],
                                    prev_mv=g[f"{case}_prev_mv"], prev_intra=g[f"{case}_prev_intra"])
        np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"], err_msg=f"mode {mode}")
        np.testing.assert_array_equal(dist, g[f"{case}_m{mode}_dist"], err_msg=f"mode {mode}")
        assert avg == int(g[f"{case}_m{mode}_avg"][0])
    mv, dist, avg = orc.me_umhs(src, ref, mr)
    np.testing.assert_array_equal(mv, g[f"{case}_noprev_mv"])
    np.testing.assert_array_equal(dist, g[f"{case}_noprev_dist"])
    assert avg == 0


def test_me_umhs_1080p_matches_reference(orc, golden, hd_golden):
    g = golden("me_umhs.npz")
    assert g["hd_frames_sha256"].tobytes() == hd_golden["g"]["frames_sha256"].tobytes()
    fr, mr = hd_golden["frames"], hd_golden["motion_range"]
    incl = np.ones((hd_golden["w"] // 16) * (hd_golden["h"] // 16), np.uint8)
    mv, dist, avg = orc.me_umhs(fr[1], fr[0], mr, mode=0, dist_incl=incl)
    np.testing.assert_array_equal(mv, g["hd_mv"])
    np.testing.assert_array_equal(dist, g["hd_dist"])
    assert avg == int(g["hd_avg"][0])


def test_me_umhs_refuses_prev_vectors_outside_the_frame(orc):
    """A previous-frame vector whose block leaves [-16, w] x [-16, h] would make
    the reference read outside its buffers should it win: refused."""
    fr = synth.pan_sequence(3, 64, 48, 2)
    pmv = np.zeros((12, 2), np.int16)
    pmv[0] = (-4 * 17, 0)
    with pytest.raises(ValueError, match="rc=-3"):
        orc.me_umhs(fr[1], fr[0], 128, prev_mv=pmv)
    pin = np.zeros(12, np.uint8)
    pin[0] = 1  # an intra macroblock's vector is not read
    orc.me_umhs(fr[1], fr[0], 128, prev_mv=pmv, prev_intra=pin)


@ref_available
@pytest.mark.parametrize("seed,w,h,mr,mode,gen", [(81, 176, 144, 128, 0, "noisy"), (82, 208, 120, 96, 1, "pan"),
                                                 (83, 96, 64, 256, 0, "shift"), (84, 640, 368, 128, 0, "noisy"),
                                                 (85, 352, 288, 16, 2, "noisy")])
def test_me_umhs_against_compiled_reference(orc, seed, w, h, mr, mode, gen):
    from tests.golden.make_golden import prev_frame_vectors, umhs_frames
    ref_lib = oracle_mod.Reference()
    fr = umhs_frames(seed, w, h, gen)
    pmv, pin = prev_frame_vectors(seed, w, h, mr)
    incl = (synth.splitmix64(seed, (w // 16) * (h // 16)) & np.uint64(1)).astype(np.uint8)
    r = ref_lib.me_umhs(fr[1], fr[0], mr, mode=mode, dist_incl=incl, prev_mv=pmv, prev_intra=pin)
    o = orc.me_umhs(fr[1], fr[0], mr, mode=mode, dist_incl=incl, prev_mv=pmv, prev_intra=pin)
    np.testing.assert_array_equal(o[0], r[0])
    np.testing.assert_array_equal(o[1], r[1])
    assert o[2] == r[2]


@pytest.mark.parametrize("case", UMHS_CASES)
def test_me_fhs_matches_reference(orc, golden, case):
    """MotionEstimatorH264ImplFHS on the me_umhs frames: vectors, stored
    distortions and the average, modes 0/1/2."""
    g, gu = golden("me_fhs.npz"), golden("me_umhs.npz")
    w, h, mr = (int(v) for v in gu[f"{case}_meta"])
    src, ref = gu[f"{case}_src"].astype(np.int16), gu[f"{case}_ref"].astype(np.int16)
    for mode in (0, 1, 2):
        mv, dist, avg = orc.me_fhs(src, ref, mr, mode=mode, dist_incl=gu[f"{case}_incl"])
        np.testing.assert_array_equal(mv, g[f"{case}_m{mode}_mv"], err_msg=f"mode {mode}")
        np.testing.assert_array_equal(dist, g[f"{case}_m{mode}_dist"], err_msg=f"mode {mode}")
        assert avg == int(g[f"{case}_m{mode}_avg"][0])


def test_me_fhs_1080p_matches_reference(orc, golden, hd_golden):
    g = golden("me_fhs.npz")
    assert g["hd_frames_sha256"].tobytes() == hd_golden["g"]["frames_sha256"].tobytes()
    fr, mr = hd_golden["frames"], hd_golden["motion_range"]
    incl = np.ones((hd_golden["w"] // 16) * (hd_golden["h"] // 16), np.uint8)
    mv, dist, avg, stale = orc.me_fhs(fr[1], fr[0], mr, mode=0, dist_incl=incl, with_stale=True)
    assert stale == 0
    np.testing.assert_array_equal(mv, g["hd_mv"])
    np.testing.assert_array_equal(dist, g["hd_dist"])
    assert avg == int(g["hd_avg"][0])


@ref_available
@pytest.mark.parametrize("seed,w,h,mr,mode,gen", [(86, 176, 144, 128, 0, "noisy"), (87, 208, 120, 96, 1, "pan"),
                                                 (88, 96, 64, 256, 0, "shift"), (89, 640, 368, 128, 0, "noisy"),
                                                 (90, 352, 288, 16, 2, "shift")])
def test_me_fhs_against_compiled_reference(orc, seed, w, h, mr, mode, gen):
    from tests.golden.make_golden import umhs_frames
    ref_lib = oracle_mod.Reference()
    fr = umhs_frames(seed, w, h, gen)
    incl = (synth.splitmix64(seed, (w // 16) * (h // 16)) & np.uint64(1)).astype(np.uint8)
    r = ref_lib.me_fhs(fr[1], fr[0], mr, mode=mode, dist_incl=incl)
    o = orc.me_fhs(fr[1], fr[0], mr, mode=mode, dist_incl=incl)
    np.testing.assert_array_equal(o[0], r[0])
    np.testing.assert_array_equal(o[1], r[1])
    assert o[2] == r[2]


IMPL1_CASES = ["qcif16_r16", "qcif8_r16", "cif16_r15", "small16_r7", "small8_r31", "qcif16_r32"]


@pytest.mark.parametrize("case", IMPL1_CASES)
def test_me_impl1_matches_reference(orc, golden, case):
    """MotionEstimatorImpl1: half-pel vectors and avgDistortion."""
    g = golden("me_impl1.npz")
    w, h, bw, bh, rng = (int(v) for v in g[f"{case}_meta"])
    mv, dist, avg = orc.me_impl1(g[f"{case}_src"].astype(np.int16), g[f"{case}_ref"].astype(np.int16), rng, bw, bh)
    np.testing.assert_array_equal(mv, g[f"{case}_mv"])
    assert avg == int(g[f"{case}_avg"][0])
    assert int(dist.sum()) // dist.size == avg


@ref_available
@pytest.mark.parametrize("seed,w,h,bw,bh,rng,gen", [(121, 176, 144, 16, 16, 12, "noisy"), (122, 208, 120, 8, 8, 20, "pan"),
                                                   (123, 128, 96, 16, 16, 24, "shift")])
def test_me_impl1_against_compiled_reference(orc, seed, w, h, bw, bh, rng, gen):
    from tests.golden.make_golden import umhs_frames
    fr = umhs_frames(seed, w, h, gen)
    mv_r, avg_r = oracle_mod.Reference().me_impl1(fr[1], fr[0], rng, bw, bh)
    mv, _, avg = orc.me_impl1(fr[1], fr[0], rng, bw, bh)
    np.testing.assert_array_equal(mv, mv_r)
    assert avg == avg_r


IMPL2_CASES = ["qcif_r16_m1", "qcif_r16_m2", "cif_r15_m2", "small_r8_m1", "cif_r32_m2", "wide_r20_m1"]


@pytest.mark.parametrize("case", IMPL2_CASES)
def test_me_impl2_matches_reference(orc, golden, case):
    """MotionEstimatorImpl2: half-pel vectors and avgDistortion."""
    g = golden("me_impl2.npz")
    w, h, rng, mode = (int(v) for v in g[f"{case}_meta"])
    mv, dist, avg = orc.me_impl2(g[f"{case}_src"].astype(np.int16), g[f"{case}_ref"].astype(np.int16), rng, mode)
    np.testing.assert_array_equal(mv, g[f"{case}_mv"])
    assert avg == int(g[f"{case}_avg"][0])


@ref_available
@pytest.mark.parametrize("seed,w,h,rng,mode,gen", [(151, 176, 144, 12, 1, "noisy"), (152, 352, 288, 24, 0, "pan"),
                                                  (153, 128, 96, 6, 2, "shift")])
def test_me_impl2_against_compiled_reference(orc, seed, w, h, rng, mode, gen):
    from tests.golden.make_golden import umhs_frames
    fr = umhs_frames(seed, w, h, gen)
    mv_r, avg_r = oracle_mod.Reference().me_impl2(fr[1], fr[0], rng, mode)
    mv, _, avg = orc.me_impl2(fr[1], fr[0], rng, mode)
    np.testing.assert_array_equal(mv, mv_r)
    assert avg == avg_r
