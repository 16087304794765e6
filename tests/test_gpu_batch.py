"""Batched estimation (vppgpu_me_batch_*): a mix of frame sizes and ranges on
several streams gives, for every job, the vectors, distortions and
avgDistortion of estimating that job alone, and those of the CPU oracle on
the small sizes."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu

SIZES = [(176, 144, 128), (352, 288, 128), (176, 144, 64), (640, 368, 128), (352, 288, 96), (1280, 720, 128),
         (208, 120, 128), (176, 144, 128)]


def test_batch_matches_single_and_oracle(vpp, ctx, orc):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    jobs, keep = [], []
    for i, (w, h, mr) in enumerate(SIZES):
        fr = synth.pan_sequence(300 + i, w, h, 2)
        nmb = (w // 16) * (h // 16)
        src = torch.from_numpy(fr[1]).to(dev)
        ref = torch.from_numpy(fr[0]).to(dev)
        incl = torch.from_numpy((synth.splitmix64(300 + i, nmb) % np.uint64(3) != 0).astype(np.uint8)).to(dev)
        mv = torch.zeros((nmb, 2), dtype=torch.int16, device=dev)
        dist = torch.zeros(nmb, dtype=torch.int32, device=dev)
        keep.append((fr, src, ref, incl, mv, dist, w, h, mr))
        jobs.append((src.data_ptr(), ref.data_ptr(), w, h, mr, mv.data_ptr(), dist.data_ptr(), incl.data_ptr()))
    batch = vpp.MotionEstimatorBatch(streams=3, ctx=ctx)
    for rep in range(2):  # the second run reuses the per-stream estimators
        st, avg = batch.run(jobs)
        torch.cuda.synchronize()
        assert st == [0] * len(jobs)
        for (fr, src, ref, incl, mv, dist, w, h, mr), a in zip(keep, avg):
            me = vpp.MotionEstimatorH264ImplFull(fr[1], fr[0], w, h, mr, pDistortionIncluded=incl.cpu().numpy(), ctx=ctx)
            assert me.Create() == 1
            mv1, avg1 = me.Estimate()
            np.testing.assert_array_equal(mv.cpu().numpy(), mv1)
            np.testing.assert_array_equal(dist.cpu().numpy(), me.last_mb_distortion)
            assert a == avg1
            if w * h <= 352 * 288:
                mv_o, dist_o, avg_o = orc.me_full(fr[1], fr[0], mr, dist_incl=incl.cpu().numpy())
                np.testing.assert_array_equal(mv1, mv_o)
                assert avg1 == avg_o
    assert batch.launch_count() > 0
    batch.close()


def test_batch_reports_per_job_status(vpp, ctx):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    w, h = 176, 144
    fr = synth.pan_sequence(7, w, h, 2)
    good = torch.from_numpy(fr[1]).to(dev)
    ref = torch.from_numpy(fr[0]).to(dev)
    bad = good.clone()
    bad[3, 5] = 300  # outside 0..255
    mv = [torch.zeros((99, 2), dtype=torch.int16, device=dev) for _ in range(2)]
    batch = vpp.MotionEstimatorBatch(streams=2, ctx=ctx)
    st, _ = batch.run([(good.data_ptr(), ref.data_ptr(), w, h, 128, mv[0].data_ptr()),
                       (bad.data_ptr(), ref.data_ptr(), w, h, 128, mv[1].data_ptr())])
    assert st[0] == 0
    assert st[1] == -4  # VPPGPU_ERR_PIXEL_RANGE
    batch.close()
