"""GPU integer-pel SAD full search (the MotionEstimatorH264ImplFull integer
stage with its MEH264IF_ABS_DIFF distortion): vectors, per-macroblock SADs and
averages bit-exact with the reference's golden fixtures (the QCIF +-16 shifted
sequence, pan pairs, a partial bottom row, tiled content whose scans meet exact
ties that the prediction decides), and with the CPU oracle on more sizes,
ranges and a 1080p frame."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = ["config1", "cif_r128", "partial_r64", "tiles_r64", "tiles_r128"]


def make(vpp, ctx, src, ref, mr, incl=None):
    h, w = src.shape
    me = vpp.MotionEstimatorH264ImplFullSad(src, ref, w, h, mr, pDistortionIncluded=incl, ctx=ctx)
    assert me.Create() == 1
    return me


@pytest.mark.parametrize("case", CASES)
def test_against_golden(vpp, ctx, golden, case):
    g = golden("me_full_sad.npz")
    w, h, mr = (int(v) for v in g[f"{case}_meta"])
    frames = g[f"{case}_frames"].astype(np.int16)
    nmb = (w // 16) * (h // 16)
    # one object over the sequence: the caller overwrites the planes between estimates
    src, ref = frames[1].copy(), frames[0].copy()
    me = make(vpp, ctx, src, ref, mr, np.ones(nmb, np.uint8))
    plain = make(vpp, ctx, src, ref, mr)
    for t in range(len(frames) - 1):
        src[...] = frames[t + 1]
        ref[...] = frames[t]
        mv, avg = me.Estimate()
        np.testing.assert_array_equal(mv, g[f"{case}_mv"][t])
        np.testing.assert_array_equal(me.last_mb_distortion, g[f"{case}_dist"][t])
        assert avg == int(g[f"{case}_avg"][t])
        mv0, avg0 = plain.Estimate()
        np.testing.assert_array_equal(mv0, mv)
        assert avg0 == 0


def test_config1_sequence(vpp, ctx, orc):
    """The reference's own CPU case: QCIF 176x144, 10 frames, +-16 pels."""
    fr = synth.shift_sequence(11, 176, 144, 10)
    src, ref = fr[1].copy(), fr[0].copy()
    me = make(vpp, ctx, src, ref, 64)
    for t in range(9):
        src[...] = fr[t + 1]
        ref[...] = fr[t]
        mv, _ = me.Estimate()
        mv_o, d_o = orc.me_full_intpel(fr[t + 1], fr[t], 64, metric=1)
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(me.last_mb_distortion, d_o)


@pytest.mark.parametrize("seed,w,h,mr,gen", [(31, 352, 288, 64, "pan"), (32, 176, 144, 128, "shift"),
                                             (33, 208, 120, 48, "pan"), (34, 48, 32, 8, "pan"),
                                             (35, 640, 360, 128, "tiles"), (36, 320, 176, 4, "pan"),
                                             (37, 1920, 1080, 128, "pan"), (38, 1280, 720, 64, "tiles")])
def test_against_oracle(vpp, ctx, orc, seed, w, h, mr, gen):
    gens = {"shift": synth.shift_sequence, "pan": synth.pan_sequence, "tiles": synth.tile_sequence}
    fr = gens[gen](seed, w, h, 2)
    nmb = (w // 16) * (h // 16)
    incl = (synth.splitmix64(seed, nmb) % np.uint64(3) != 0).astype(np.uint8)
    mv_o, d_o = orc.me_full_intpel(fr[1], fr[0], mr, metric=1)
    sel = incl.astype(bool)
    avg_o = int(d_o[sel].sum()) // int(sel.sum()) if sel.any() else 0
    me = make(vpp, ctx, fr[1], fr[0], mr, incl)
    mv, avg = me.Estimate()
    np.testing.assert_array_equal(mv, mv_o)
    np.testing.assert_array_equal(me.last_mb_distortion, d_o)
    assert avg == avg_o


def test_batched_form(vpp, ctx, orc):
    """The batched form (vppgpu_me_batch_*, several streams) of the SAD search
    gives every job the vectors, SADs and average of estimating it alone."""
    torch = pytest.importorskip("torch")
    from imagecodingutils_gb300 import _lib
    dev = torch.device("cuda", 0)
    sizes = [(176, 144, 64), (352, 288, 128), (640, 368, 128), (208, 120, 48), (176, 144, 64)]
    jobs, keep = [], []
    for i, (w, h, mr) in enumerate(sizes):
        fr = (synth.tile_sequence if i % 2 else synth.pan_sequence)(400 + i, w, h, 2)
        nmb = (w // 16) * (h // 16)
        src, ref = torch.from_numpy(fr[1]).to(dev), torch.from_numpy(fr[0]).to(dev)
        incl = torch.from_numpy((synth.splitmix64(400 + i, nmb) % np.uint64(3) != 0).astype(np.uint8)).to(dev)
        mv = torch.zeros((nmb, 2), dtype=torch.int16, device=dev)
        dist = torch.zeros(nmb, dtype=torch.int32, device=dev)
        keep.append((fr, incl, mv, dist, w, h, mr, src, ref))  # the device inputs stay alive
        jobs.append((src.data_ptr(), ref.data_ptr(), w, h, mr, mv.data_ptr(), dist.data_ptr(), incl.data_ptr()))
    batch = vpp.MotionEstimatorBatch(streams=3, kind=_lib.ME_FULL_SAD, ctx=ctx)
    for _ in range(2):
        st, avg = batch.run(jobs)
        torch.cuda.synchronize()
        assert st == [0] * len(jobs)
        for (fr, incl, mv, dist, w, h, mr, _, _), a in zip(keep, avg):
            mv_o, d_o = orc.me_full_intpel(fr[1], fr[0], mr, metric=1)
            sel = incl.cpu().numpy().astype(bool)
            np.testing.assert_array_equal(mv.cpu().numpy(), mv_o)
            np.testing.assert_array_equal(dist.cpu().numpy(), d_o)
            assert a == (int(d_o[sel].sum()) // int(sel.sum()) if sel.any() else 0)
    batch.close()
