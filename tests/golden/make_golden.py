"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own C++ classes (compiled unmodified from its sources by
``make -C oracle ref`` into oracle/_ref/libvppref.so) on seeded synthetic
inputs and stores inputs and outputs:

* me_full.npz     MotionEstimatorH264ImplFull vectors and avgDistortion for
                  QCIF / CIF / partial-row pairs at motion ranges 64 and 128,
                  plus per-macroblock distortions for one QCIF pair (one
                  estimate per macroblock with a single pDistortionIncluded flag)
* me_mrc.npz      MotionEstimatorH264ImplMultiresCross vectors and
                  avgDistortion, modes 0/1/2, with and without
                  pDistortionIncluded (the partial bottom row counts in the
                  average when it is NULL)
* me_mrc2.npz     MotionEstimatorH264ImplMultiresCrossVer2 vectors and
                  avgDistortion, modes 0/1/2, with and without
                  pDistortionIncluded (pan and integer-shift content)
* me_mrc2_lambda.npz  Ver2's Estimate(long*, void* lambda): the me_mrc2 cases
                  at lambdas 0, 0.9, 2.5 and 20 (modes 0/1/2), and the 1080p
                  benchmark pair 0 at lambdas 0.9 and 4 (modes 1/2)
* me_mr.npz       MotionEstimatorH264ImplMultires, the same cases as me_mrc2
* me_full_sad.npz the integer-pel stage of MotionEstimatorH264ImplFull with
                  its MEH264IF_ABS_DIFF distortion (SAD): the QCIF +-16 shifted
                  sequence, pan and tiled (tie-heavy) pairs, vectors, SADs and
                  averages
* mc.npz          MotionCompensatorH264ImplStd::Compensate of 4:2:0 frames by
                  seeded vectors over the whole range (zero, full-pel, negative
                  fractions), QCIF / CIF / 64x48
* transform.npz   FastForward4x4ITImpl1 / Impl2 / On16x16 levels and
                  FastInverse4x4ITImpl1 / On16x16 reconstructions over QP 0..51,
                  intra and inter, modes 0/1/2, a custom SetScale, and
                  FastForward4x4ITImpl2::QuantiseValue
* colour.npz      the three RGB24->YUV420 converters, flip and chroma offsets
* yuv2rgb.npz     the five Real YUV420->RGB24 converters, every rotate / flip,
                  the two 6-bit converters (6-bit, wider and +-32767 samples,
                  both layouts) and the 6-bit zoom converter at several sizes
* me_umhs.npz     MotionEstimatorH264ImplUMHS (eight-argument constructor):
                  pan, integer-shift and part-noise pairs at QCIF / CIF and
                  motion ranges 64 / 128, modes 0/1/2, seeded previous-frame
                  vectors and intra flags, vectors, the distortion stored with
                  each and avgDistortion; and pair 0 of the 1080p benchmark
                  sequence (mode 0, zero previous vectors)
* me_fhs.npz      MotionEstimatorH264ImplFHS: the me_umhs cases (frames stored
                  in me_umhs.npz) at modes 0/1/2 with pDistortionIncluded,
                  vectors, the distortion stored with each and avgDistortion,
                  and pair 0 of the 1080p benchmark sequence (mode 0)
* me_impl1.npz    MotionEstimatorImpl1 (the H.263-style full search with half-pel
                  refinement and the weighted zero-vector choice): pan, shift and
                  part-noise pairs, 16x16 and 8x8 blocks, ranges 7..32 pels;
                  half-pel vectors and avgDistortion
* me_impl2.npz    MotionEstimatorImpl2 (the SAD pyramid): pan, shift and part-noise
                  pairs, ranges 8..32 pels, modes 1 and 2; half-pel vectors and
                  avgDistortion
* me_1080p.npz    the headline size: Full, MultiresCross / Ver2 / Multires
                  (modes 0, 1, 2), Cross and the integer-pel SAD stage on three
                  frame pairs of the 1920x1080 benchmark sequence at
                  motionRange 128 (frames regenerated by synth, pinned by their
                  SHA-256)

Usage: python tests/golden/make_golden.py [name ...]   (needs the reference tree;
names: me_1080p me_full me_full_sad me_mrc me_mrc2 me_mrc2_lambda me_mr me_cross me_h263mrc me_h263mrc2 me_umhs me_fhs me_impl1 me_impl2 mc
transform dc yuv2rgb colour, default all)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from imagecodingutils_gb300 import synth  # noqa: E402
from oracle import oracle  # noqa: E402

ME_CASES = [  # (name, w, h, motion_range, seed)
    ("qcif_r64", 176, 144, 64, 1),
    ("qcif_r128", 176, 144, 128, 3),
    ("cif_r128", 352, 288, 128, 2),
    ("partial_r128", 176, 152, 128, 4),
    ("shift_r64", 176, 144, 64, 5),
]


def me_fixtures(ref: oracle.Reference) -> dict:
    out = {}
    for name, w, h, mr, seed in ME_CASES:
        if name.startswith("shift"):
            fr = synth.shift_sequence(seed, w, h, 2)
        else:
            fr = synth.pan_sequence(seed, w, h, 2)
        src, rf = fr[1], fr[0]
        nmb = (w // 16) * (h // 16)
        incl = np.ones(nmb, np.uint8)
        mv, avg = ref.me("full", src, rf, mr, dist_incl=incl)
        mv0, avg0 = ref.me("full", src, rf, mr)
        assert np.array_equal(mv, mv0) and avg0 == 0
        out[f"{name}_src"] = src.astype(np.uint8)
        out[f"{name}_ref"] = rf.astype(np.uint8)
        out[f"{name}_meta"] = np.array([w, h, mr], np.int32)
        out[f"{name}_mv"] = mv
        out[f"{name}_avg"] = np.array([avg], np.int64)
        if name == "qcif_r64":
            d = np.zeros(nmb, np.int64)
            for k in range(nmb):
                one = np.zeros(nmb, np.uint8)
                one[k] = 1
                _, d[k] = ref.me("full", src, rf, mr, dist_incl=one)
            out[f"{name}_mbdist"] = d
    return out


SAD_CASES = [  # (name, w, h, motion_range, seed, generator)
    ("config1", 176, 144, 64, 11, "shift"),   # QCIF +-16, the reference's own CPU case
    ("cif_r128", 352, 288, 128, 12, "pan"),
    ("partial_r64", 176, 152, 64, 13, "pan"),
    ("tiles_r64", 176, 144, 64, 14, "tiles"),
    ("tiles_r128", 352, 288, 128, 15, "tiles"),
]


def sad_fixtures(ref: oracle.Reference) -> dict:
    """The integer-pel SAD stage of MotionEstimatorH264ImplFull (the harness's
    FullSadStage on the reference's overlays): per case the first frame pairs of
    the sequence (four frames of config1, two otherwise), vectors, SADs and the
    all-included average; the average without flags is 0."""
    out = {}
    gens = {"shift": synth.shift_sequence, "pan": synth.pan_sequence, "tiles": synth.tile_sequence}
    for name, w, h, mr, seed, gen in SAD_CASES:
        nf = 4 if name == "config1" else 2
        fr = gens[gen](seed, w, h, nf)
        nmb = (w // 16) * (h // 16)
        out[f"{name}_frames"] = np.stack(fr).astype(np.uint8)
        out[f"{name}_meta"] = np.array([w, h, mr], np.int32)
        mvs, ds, avgs = [], [], []
        for t in range(nf - 1):
            mv, d, avg = ref.me_full_sad(fr[t + 1], fr[t], mr, dist_incl=np.ones(nmb, np.uint8))
            mv0, d0, avg0 = ref.me_full_sad(fr[t + 1], fr[t], mr)
            assert np.array_equal(mv, mv0) and np.array_equal(d, d0) and avg0 == 0
            mvs.append(mv)
            ds.append(d)
            avgs.append(avg)
        out[f"{name}_mv"] = np.stack(mvs)
        out[f"{name}_dist"] = np.stack(ds)
        out[f"{name}_avg"] = np.array(avgs, np.int64)
    return out


MRC_CASES = [  # (name, w, h, motion_range, seed)
    ("qcif_r64", 176, 144, 64, 21),
    ("cif_r128", 352, 288, 128, 22),
    ("partial_r128", 352, 280, 128, 23),
    ("small_r32", 64, 48, 32, 24),
]


# MotionEstimatorH263ImplMultiresCross: motion ranges in half pels
H263_CASES = [("qcif_r32", 176, 144, 32, 25), ("cif_r64", 352, 288, 64, 26), ("partial_r64", 352, 280, 64, 27),
              ("small_r16", 64, 48, 16, 28)]


def mrc_fixtures(ref: oracle.Reference, kind: str = "multires_cross", cases=None) -> dict:
    out = {}
    for name, w, h, mr, seed in (MRC_CASES if cases is None else cases):
        fr = synth.pan_sequence(seed, w, h, 2)
        src, rf = fr[1], fr[0]
        nmb = (w // 16) * (h // 16)
        out[f"{name}_src"] = src.astype(np.uint8)
        out[f"{name}_ref"] = rf.astype(np.uint8)
        out[f"{name}_meta"] = np.array([w, h, mr], np.int32)
        for mode in (0, 1, 2):
            mv, avg = ref.me(kind, src, rf, mr, mode=mode)
            mvi, avgi = ref.me(kind, src, rf, mr, mode=mode, dist_incl=np.ones(nmb, np.uint8))
            assert np.array_equal(mv, mvi)
            out[f"{name}_m{mode}_mv"] = mv
            out[f"{name}_m{mode}_avg"] = np.array([avg, avgi], np.int64)
    return out


MRC2_CASES = [  # (name, w, h, motion_range, seed, generator)
    ("qcif_r64", 176, 144, 64, 41, "pan"),
    ("cif_r128", 352, 288, 128, 42, "pan"),
    ("partial_r128", 352, 280, 128, 43, "pan"),
    ("small_r32", 64, 48, 32, 44, "pan"),
    ("shift_r128", 352, 288, 128, 45, "shift"),
]


def mrc2_fixtures(ref: oracle.Reference, kind: str = "multires_cross_v2") -> dict:
    out = {}
    for name, w, h, mr, seed, gen in MRC2_CASES:
        fr = (synth.shift_sequence if gen == "shift" else synth.pan_sequence)(seed, w, h, 2)
        src, rf = fr[1], fr[0]
        nmb = (w // 16) * (h // 16)
        incl = (np.arange(nmb) % 3 != 0).astype(np.uint8)
        out[f"{name}_src"] = src.astype(np.uint8)
        out[f"{name}_ref"] = rf.astype(np.uint8)
        out[f"{name}_meta"] = np.array([w, h, mr], np.int32)
        out[f"{name}_incl"] = incl
        for mode in (0, 1, 2):
            mv, avg = ref.me(kind, src, rf, mr, mode=mode)
            mvi, avgi = ref.me(kind, src, rf, mr, mode=mode, dist_incl=incl)
            assert np.array_equal(mv, mvi) and avg == 0
            out[f"{name}_m{mode}_mv"] = mv
            out[f"{name}_m{mode}_avg"] = np.array([avgi], np.int64)
    return out


LAMBDAS = (0.0, 0.9, 2.5, 20.0)


def mrc2_lambda_fixtures(ref: oracle.Reference) -> dict:
    """Ver2's Estimate(long*, void* lambda) on the me_mrc2 cases at LAMBDAS
    (modes 0/1/2, with the me_mrc2 inclusion map; the frames are stored in
    me_mrc2.npz only), and on pair 0 of the 1080p
    benchmark sequence at motionRange 128, modes 1 and 2, lambdas 0.9 and 4."""
    out = {"lambdas": np.array(LAMBDAS, np.float64)}
    for name, w, h, mr, seed, gen in MRC2_CASES:
        fr = (synth.shift_sequence if gen == "shift" else synth.pan_sequence)(seed, w, h, 2)
        src, rf = fr[1], fr[0]
        nmb = (w // 16) * (h // 16)
        incl = (np.arange(nmb) % 3 != 0).astype(np.uint8)
        # the frames, meta and inclusion map are those of me_mrc2.npz
        for mode in (0, 1, 2):
            for li, lam in enumerate(LAMBDAS):
                mv, avg = ref.me("multires_cross_v2", src, rf, mr, mode=mode, dist_incl=incl, lam=lam)
                out[f"{name}_m{mode}_l{li}_mv"] = mv
                out[f"{name}_m{mode}_l{li}_avg"] = np.array([avg], np.int64)
    fr, digest = hd_frames()
    out["hd_meta"] = np.array([HD_SEED, HD_W, HD_H, HD_RANGE, 0], np.int32)
    out["hd_frames_sha256"] = digest
    incl = np.ones((HD_W // 16) * (HD_H // 16), np.uint8)
    for mode in (1, 2):
        for lam in (0.9, 4.0):
            mv, avg = ref.me("multires_cross_v2", fr[1], fr[0], HD_RANGE, mode=mode, dist_incl=incl, lam=lam)
            out[f"hd_m{mode}_lam{lam:g}_mv"] = mv
            out[f"hd_m{mode}_lam{lam:g}_avg"] = np.array([avg], np.int64)
    return out


UMHS_CASES = [  # (name, w, h, motion_range, seed, generator)
    ("qcif_r64", 176, 144, 64, 71, "pan"),
    ("cif_r128", 352, 288, 128, 72, "pan"),
    ("shift_r128", 176, 144, 128, 73, "shift"),
    ("noisy_r128", 352, 288, 128, 74, "noisy"),
    ("small_r32", 64, 48, 32, 75, "noisy"),
]


def prev_frame_vectors(seed: int, w: int, h: int, motion_range: int):
    """Seeded previous-frame macroblock vectors (quarter pels) whose blocks stay
    within [-16, w] x [-16, h] (as an earlier estimate's do), and intra flags."""
    rng = np.random.default_rng(seed)
    cols, rows = w // 16, h // 16
    nmb = cols * rows
    mv = rng.integers(-motion_range, motion_range, size=(nmb, 2)).astype(np.int64)
    full = np.where(mv < 0, -((-mv) // 4), mv // 4)
    x = (np.arange(nmb) % cols) * 16 + full[:, 0]
    y = (np.arange(nmb) // cols) * 16 + full[:, 1]
    mv[:, 0] = np.where((x < -16) | (x > w), 0, mv[:, 0])
    mv[:, 1] = np.where((y < -16) | (y > h), 0, mv[:, 1])
    intra = (rng.random(nmb) < 0.2).astype(np.uint8)
    return mv.astype(np.int16), intra


def umhs_frames(seed: int, w: int, h: int, gen: str):
    """A frame pair: the pan or shift sequence, or ("noisy") a pan pair whose
    second frame has 40 % of its macroblocks replaced by uniform noise (large
    distortions take every stage of the search)."""
    if gen == "shift":
        return synth.shift_sequence(seed, w, h, 2)
    fr = synth.pan_sequence(seed, w, h, 2)
    if gen == "noisy":
        rng = np.random.default_rng(seed)
        mask = np.kron(rng.random((h // 16, w // 16)) < 0.4, np.ones((16, 16), bool))
        noise = rng.integers(0, 256, size=mask.shape).astype(np.int16)
        cur = fr[1].copy()
        cur[:mask.shape[0], :mask.shape[1]][mask] = noise[mask]
        fr = [fr[0], cur]
    return fr


def umhs_fixtures(ref: oracle.Reference) -> dict:
    out = {}
    for name, w, h, mr, seed, gen in UMHS_CASES:
        fr = umhs_frames(seed, w, h, gen)
        src, rf = fr[1], fr[0]
        nmb = (w // 16) * (h // 16)
        incl = (np.arange(nmb) % 4 != 1).astype(np.uint8)
        pmv, pin = prev_frame_vectors(seed + 1000, w, h, mr)
        out[f"{name}_src"] = src.astype(np.uint8)
        out[f"{name}_ref"] = rf.astype(np.uint8)
        out[f"{name}_meta"] = np.array([w, h, mr], np.int32)
        out[f"{name}_incl"] = incl
        out[f"{name}_prev_mv"] = pmv
        out[f"{name}_prev_intra"] = pin
        for mode in (0, 1, 2):
            mv, d, avg = ref.me_umhs(src, rf, mr, mode=mode, dist_incl=incl, prev_mv=pmv, prev_intra=pin)
            out[f"{name}_m{mode}_mv"] = mv
            out[f"{name}_m{mode}_dist"] = d
            out[f"{name}_m{mode}_avg"] = np.array([avg], np.int64)
        # without previous vectors or inclusion flags
        mv, d, avg = ref.me_umhs(src, rf, mr, mode=0)
        out[f"{name}_noprev_mv"] = mv
        out[f"{name}_noprev_dist"] = d
    fr, digest = hd_frames()
    incl = np.ones((HD_W // 16) * (HD_H // 16), np.uint8)
    out["hd_meta"] = np.array([HD_SEED, HD_W, HD_H, HD_RANGE, 0], np.int32)
    out["hd_frames_sha256"] = digest
    mv, d, avg = ref.me_umhs(fr[1], fr[0], HD_RANGE, mode=0, dist_incl=incl)
    out["hd_mv"] = mv
    out["hd_dist"] = d
    out["hd_avg"] = np.array([avg], np.int64)
    return out


H263V2_CASES = [  # (name, w, h, half-pel motion range, seed, generator)
    ("qcif_r32", 176, 144, 32, 61, "pan"),
    ("cif_r64", 352, 288, 64, 62, "noisy"),
    ("partial_r64", 352, 280, 64, 63, "shift"),
    ("small_r16", 64, 48, 16, 64, "noisy"),
    ("wide_r48", 208, 120, 48, 65, "pan"),
]


def h263v2_fixtures(ref: oracle.Reference) -> dict:
    """MotionEstimatorH263ImplMultiresCrossVer2 with H263MotionVectorPredictorImpl1:
    vectors and avgDistortion at modes 0/1/2, without and with a seeded
    pDistortionIncluded, and the 1080p benchmark pair at the largest range."""
    out = {}
    for name, w, h, mr, seed, gen in H263V2_CASES:
        fr = umhs_frames(seed, w, h, gen)
        src, rf = fr[1], fr[0]
        nmb = (w // 16) * (h // 16)
        incl = (synth.splitmix64(seed, nmb) % np.uint64(3) != 0).astype(np.uint8)
        out[f"{name}_src"] = src.astype(np.uint8)
        out[f"{name}_ref"] = rf.astype(np.uint8)
        out[f"{name}_meta"] = np.array([w, h, mr], np.int32)
        out[f"{name}_incl"] = incl
        for mode in (0, 1, 2):
            mv, avg = ref.me("h263_multires_cross_v2", src, rf, mr, mode=mode)
            mvi, avgi = ref.me("h263_multires_cross_v2", src, rf, mr, mode=mode, dist_incl=incl)
            assert np.array_equal(mv, mvi)
            out[f"{name}_m{mode}_mv"] = mv
            out[f"{name}_m{mode}_avg"] = np.array([avg, avgi], np.int64)
    fr, digest = hd_frames()
    out["hd_meta"] = np.array([HD_SEED, HD_W, HD_H, 64], np.int32)
    out["hd_frames_sha256"] = digest
    for mode in (0, 1):
        mv, avg = ref.me("h263_multires_cross_v2", fr[1], fr[0], 64, mode=mode)
        out[f"hd_m{mode}_mv"] = mv
        out[f"hd_m{mode}_avg"] = np.array([avg], np.int64)
    return out


def fhs_fixtures(ref: oracle.Reference) -> dict:
    out = {}
    for name, w, h, mr, seed, gen in UMHS_CASES:
        fr = umhs_frames(seed, w, h, gen)
        src, rf = fr[1], fr[0]
        nmb = (w // 16) * (h // 16)
        incl = (np.arange(nmb) % 4 != 1).astype(np.uint8)
        for mode in (0, 1, 2):
            mv, d, avg = ref.me_fhs(src, rf, mr, mode=mode, dist_incl=incl)
            out[f"{name}_m{mode}_mv"] = mv
            out[f"{name}_m{mode}_dist"] = d
            out[f"{name}_m{mode}_avg"] = np.array([avg], np.int64)
    fr, digest = hd_frames()
    incl = np.ones((HD_W // 16) * (HD_H // 16), np.uint8)
    out["hd_frames_sha256"] = digest
    mv, d, avg = ref.me_fhs(fr[1], fr[0], HD_RANGE, mode=0, dist_incl=incl)
    out["hd_mv"] = mv
    out["hd_dist"] = d
    out["hd_avg"] = np.array([avg], np.int64)
    return out


IMPL1_CASES = [  # (name, w, h, block w, block h, range in pels, seed, generator)
    ("qcif16_r16", 176, 144, 16, 16, 16, 111, "pan"),
    ("qcif8_r16", 176, 144, 8, 8, 16, 112, "noisy"),
    ("cif16_r15", 352, 288, 16, 16, 15, 113, "shift"),
    ("small16_r7", 64, 48, 16, 16, 7, 114, "noisy"),
    ("small8_r31", 96, 64, 8, 8, 31, 115, "pan"),
    ("qcif16_r32", 176, 144, 16, 16, 32, 116, "shift"),
]


def impl1_fixtures(ref: oracle.Reference) -> dict:
    out = {}
    for name, w, h, bw, bh, rng, seed, gen in IMPL1_CASES:
        fr = umhs_frames(seed, w, h, gen)
        mv, avg = ref.me_impl1(fr[1], fr[0], rng, bw, bh)
        out[f"{name}_src"] = fr[1].astype(np.uint8)
        out[f"{name}_ref"] = fr[0].astype(np.uint8)
        out[f"{name}_meta"] = np.array([w, h, bw, bh, rng], np.int32)
        out[f"{name}_mv"] = mv
        out[f"{name}_avg"] = np.array([avg], np.int64)
    return out


IMPL2_CASES = [  # (name, w, h, range in pels, mode, seed, generator)
    ("qcif_r16_m1", 176, 144, 16, 1, 141, "pan"),
    ("qcif_r16_m2", 176, 144, 16, 2, 142, "noisy"),
    ("cif_r15_m2", 352, 288, 15, 2, 143, "shift"),
    ("small_r8_m1", 64, 48, 8, 1, 144, "noisy"),
    ("cif_r32_m2", 352, 288, 32, 2, 145, "pan"),
    ("wide_r20_m1", 208, 112, 20, 1, 146, "shift"),
]


def impl2_fixtures(ref: oracle.Reference) -> dict:
    out = {}
    for name, w, h, rng, mode, seed, gen in IMPL2_CASES:
        fr = umhs_frames(seed, w, h, gen)
        mv, avg = ref.me_impl2(fr[1], fr[0], rng, mode)
        out[f"{name}_src"] = fr[1].astype(np.uint8)
        out[f"{name}_ref"] = fr[0].astype(np.uint8)
        out[f"{name}_meta"] = np.array([w, h, rng, mode], np.int32)
        out[f"{name}_mv"] = mv
        out[f"{name}_avg"] = np.array([avg], np.int64)
    return out


MC_CASES = [("qcif_r16", 176, 144, 16, 61), ("cif_r32", 352, 288, 32, 62), ("small_r8", 64, 48, 8, 63)]


def mc_fixtures(ref: oracle.Reference) -> dict:
    out = {}
    for name, w, h, rg, seed in MC_CASES:
        y = synth.pan_sequence(seed, w, h, 1)[0]
        u = synth.pan_sequence(seed + 100, w // 2, h // 2, 1)[0]
        v = synth.pan_sequence(seed + 200, w // 2, h // 2, 1)[0]
        nmb = (w // 16) * (h // 16)
        mv = ((synth.splitmix64(seed, 2 * nmb) % np.uint64(8 * rg + 1)).astype(np.int64) - 4 * rg).astype(np.int16)
        mv = mv.reshape(nmb, 2)
        mv[::7] = 0
        mv[1::11] = (4, -8)
        cy, cu, cv = ref.mc_compensate(y, u, v, mv, rg)
        out[f"{name}_meta"] = np.array([w, h, rg], np.int32)
        out[f"{name}_mv"] = mv
        for k, a in (("y", y), ("u", u), ("v", v), ("cy", cy), ("cu", cu), ("cv", cv)):
            out[f"{name}_{k}"] = a.astype(np.uint8)
    return out


def transform_fixtures(ref: oracle.Reference) -> dict:
    lap = synth.residual_blocks(11, 16 * 64)
    full = ((synth.splitmix64(12, 16 * 16) % np.uint64(65536)).astype(np.int64) - 32768).astype(np.int16)
    x = np.concatenate([lap, full])
    out = {"x": x}
    weight = (np.arange(16, dtype=np.int32) * 3 + 7)
    out["weight"] = weight
    for qp in range(52):
        for intra in (0, 1):
            lev = ref.fwd(0, x, 0, qp, intra)
            assert np.array_equal(lev, ref.fwd(1, x, 0, qp, intra))
            out[f"fwd_q{qp}_i{intra}"] = lev
            out[f"fwd16_q{qp}_i{intra}"] = ref.fwd(2, x, 0, qp, intra)
        lev = out[f"fwd_q{qp}_i1"]
        out[f"inv_q{qp}"] = ref.inv(0, lev, 0, qp)
        out[f"inv16_q{qp}"] = ref.inv(1, lev, 0, qp)
    for qp in (0, 11, 23, 24, 28, 51):
        for mode in (1, 2):
            out[f"fwd_m{mode}_q{qp}"] = ref.fwd(0, x, mode, qp, 1)
            out[f"inv_m{mode}_q{qp}"] = ref.inv(0, x, mode, qp)
            out[f"inv16_m{mode}_q{qp}"] = ref.inv(1, x, mode, qp)
        out[f"invw_q{qp}"] = ref.inv(0, out[f"fwd_q{qp}_i0"], 0, qp, weight)
    qv = []
    for qp in (0, 7, 28, 51):
        for pos in range(16):
            for val in (-32768, -300, -1, 0, 1, 255, 1000, 32767):
                for intra in (0, 1):
                    qv.append((val, pos, qp, intra, ref.quantise_value(val, pos, qp, intra)))
    out["quantise_value"] = np.array(qv, np.int32)
    return out


def dc_fixtures(ref: oracle.Reference) -> dict:
    """DC Hadamard transforms: forward inputs span small DC values, typical
    Intra16x16 DC magnitudes and the full int16 range (wrap-around of the
    short stores); inverse inputs are the forward levels and values up to
    +-2048 (no int overflow in the reference's products)."""
    out = {}
    for size in (4, 2):
        n = size * size
        r = lambda seed, m, lim: ((synth.splitmix64(seed, m) % np.uint64(2 * lim + 1)).astype(np.int64) - lim)
        x = np.concatenate([r(31 + size, n * 24, 300), r(41 + size, n * 24, 4080),
                            r(51 + size, n * 16, 32768).clip(-32768, 32767)]).astype(np.int16)
        xi = r(61 + size, n * 48, 2048).astype(np.int16)
        weight = (np.arange(n, dtype=np.int32) * 5 + 9)
        out[f"s{size}_x"], out[f"s{size}_xi"], out[f"s{size}_weight"] = x, xi, weight
        for qp in range(52):
            lev = ref.fwd_dc(x, size, 0, qp)
            out[f"s{size}_fwd_q{qp}"] = lev
            out[f"s{size}_inv_q{qp}"] = ref.inv_dc(lev, size, 0, qp)
        for qp in (0, 11, 23, 28, 35, 36, 51):
            for mode in (1, 2):
                out[f"s{size}_fwd_m{mode}_q{qp}"] = ref.fwd_dc(x, size, mode, qp)
                out[f"s{size}_inv_m{mode}_q{qp}"] = ref.inv_dc(xi, size, mode, qp)
            out[f"s{size}_invw_q{qp}"] = ref.inv_dc(xi, size, 0, qp, weight)
    qv = []
    for qp in (0, 7, 28, 40, 51):
        for val in (-32768, -4080, -300, -1, 0, 1, 255, 1000, 32767):
            qv.append((val, qp, ref.dc_quantise_value(val, qp)))
    out["quantise_value"] = np.array(qv, np.int32)
    return out


def yuv2rgb_fixtures(ref: oracle.Reference) -> dict:
    """YUV420 -> RGB24: the five Real converters (kinds 0-4 of ref_yuv_to_rgb)
    on a 64x48 frame of 0..255 samples, every rotate / flip combination
    (RealYUV420toRGB24Converter with chrOff -128: its byte casts stay in
    range), and Impl2 / CCIR601 on samples outside 0..255."""
    out = {}
    w, h = 64, 48
    r = lambda seed, shape, lo, hi: ((synth.splitmix64(seed, int(np.prod(shape))) % np.uint64(hi - lo + 1))
                                     .astype(np.int64) + lo).astype(np.int16).reshape(shape)
    planes = {"n": (r(71, (h, w), 0, 255), r(72, (h // 2, w // 2), 0, 255), r(73, (h // 2, w // 2), 0, 255)),
              "wide": (r(74, (h, w), -300, 600), r(75, (h // 2, w // 2), -200, 500),
                       r(76, (h // 2, w // 2), -200, 500))}
    for name, (y, u, v) in planes.items():
        out[f"{name}_y"], out[f"{name}_u"], out[f"{name}_v"] = y, u, v
        for kind in (0, 1, 2, 3, 4):
            if kind == 0 and name == "wide":
                continue
            for rot in (0, 1):
                for flip in (0, 1):
                    out[f"{name}_k{kind}_r{rot}_f{flip}"] = ref.yuv_to_rgb(kind, y, u, v, -128, rot, flip)
    # the 6-bit converters: 6-bit samples (their domain), samples past it, and
    # samples past +-16000 (Real6Bit's per-pixel double path)
    six = {"six": (r(77, (h, w), 0, 63), r(78, (h // 2, w // 2), 0, 63), r(79, (h // 2, w // 2), 0, 63)),
           "sixwide": (r(80, (h, w), -300, 600), r(81, (h // 2, w // 2), -200, 500), r(82, (h // 2, w // 2), -200, 500)),
           "sixhuge": (r(83, (h, w), -32768, 32767), r(84, (h // 2, w // 2), -32768, 32767),
                       r(85, (h // 2, w // 2), -32768, 32767))}
    for name, (y, u, v) in six.items():
        out[f"{name}_y"], out[f"{name}_u"], out[f"{name}_v"] = y, u, v
        for kind in (3, 4):
            for rot in (0, 1):
                out[f"{name}_k{kind}_r{rot}"] = ref.yuv_to_rgb_6bit(kind, y, u, v, rot)
    # Fast6BitYUV420toRGB24ZoomConverter at output sizes whose source positions stay inside the planes
    y, u, v = six["six"]
    out["zoom_sizes"] = np.array(ZOOM_SIZES, np.int32)
    for ow, oh in ZOOM_SIZES:
        out[f"zoom_{ow}x{oh}"] = ref.yuv_to_rgb_zoom(y, u, v, ow, oh)
    return out


ZOOM_SIZES = [(64, 48), (96, 72), (32, 24), (100, 50), (48, 36), (66, 94)]


def colour_fixtures(ref: oracle.Reference) -> dict:
    bgr = synth.rgb_frame(21, 64, 48)
    out = {"bgr": bgr}
    for kind in (0, 1, 2):
        for flip in (0, 1):
            for co in (0, 128):
                y, u, v = ref.rgb_to_yuv(kind, bgr, co, flip)
                out[f"k{kind}_f{flip}_c{co}_y"] = y
                out[f"k{kind}_f{flip}_c{co}_u"] = u
                out[f"k{kind}_f{flip}_c{co}_v"] = v
    return out


HD_SEED, HD_W, HD_H, HD_RANGE = 1234, 1920, 1080, 128   # the benchmark's own 1080p sequence
HD_PAIRS = (0, 5, 17)                                     # frame pairs (t+1 on t) of that sequence
HD_ESTIMATORS = [("full", 1), ("multires_cross", 0), ("multires_cross", 1), ("multires_cross", 2),
                 ("multires_cross_v2", 0), ("multires_cross_v2", 1), ("multires_cross_v2", 2),
                 ("multires", 0), ("multires", 1), ("multires", 2), ("cross", 0)]


def hd_frames():
    """Frames 0..max(HD_PAIRS)+1 of the 1080p benchmark sequence and the
    SHA-256 of their int16 bytes (the fixtures store the digest, not the
    4 MB frames: synth regenerates them bit for bit)."""
    import hashlib
    fr = synth.pan_sequence(HD_SEED, HD_W, HD_H, max(HD_PAIRS) + 2)
    digest = hashlib.sha256(b"".join(np.ascontiguousarray(f, np.int16).tobytes() for f in fr)).digest()
    return fr, np.frombuffer(digest, np.uint8)


def hd_fixtures(ref: oracle.Reference) -> dict:
    """The headline size: every estimator on pairs HD_PAIRS of the 1080p
    benchmark sequence at motionRange 128 -- vectors and avgDistortion with
    all macroblocks included (SetMode as listed; MultiresCross counts every
    macroblock anyway), and the integer-pel SAD stage's vectors, SADs and
    average."""
    fr, digest = hd_frames()
    nmb = (HD_W // 16) * (HD_H // 16)
    incl = np.ones(nmb, np.uint8)
    out = {"meta": np.array([HD_SEED, HD_W, HD_H, HD_RANGE, *HD_PAIRS], np.int32), "frames_sha256": digest}
    for t in HD_PAIRS:
        src, rf = fr[t + 1], fr[t]
        for kind, mode in HD_ESTIMATORS:
            mv, avg = ref.me(kind, src, rf, HD_RANGE, mode=mode, dist_incl=incl)
            out[f"p{t}_{kind}_m{mode}_mv"] = mv
            out[f"p{t}_{kind}_m{mode}_avg"] = np.array([avg], np.int64)
        mv, d, avg = ref.me_full_sad(src, rf, HD_RANGE, dist_incl=incl)
        out[f"p{t}_full_sad_mv"] = mv
        out[f"p{t}_full_sad_dist"] = d
        out[f"p{t}_full_sad_avg"] = np.array([avg], np.int64)
    return out


def main() -> None:
    oracle.build(with_reference=True)
    ref = oracle.Reference()
    makers = {"me_1080p": hd_fixtures,
              "me_full": me_fixtures, "me_full_sad": sad_fixtures, "me_mrc": mrc_fixtures, "me_mrc2": mrc2_fixtures,
              "me_mrc2_lambda": mrc2_lambda_fixtures,
              "me_mr": lambda r: mrc2_fixtures(r, "multires"), "me_cross": lambda r: mrc2_fixtures(r, "cross"),
              "me_h263mrc": lambda r: mrc_fixtures(r, "h263_multires_cross", H263_CASES),
              "me_h263mrc2": h263v2_fixtures,
              "me_umhs": umhs_fixtures, "me_fhs": fhs_fixtures, "me_impl1": impl1_fixtures, "me_impl2": impl2_fixtures,
              "mc": mc_fixtures,
              "transform": transform_fixtures, "dc": dc_fixtures, "yuv2rgb": yuv2rgb_fixtures,
              "colour": colour_fixtures}
    names = sys.argv[1:] or list(makers)
    for name in names:
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **makers[name](ref))
    print("golden fixtures", ", ".join(names), "written to", HERE)


if __name__ == "__main__":
    main()
