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


def test_batch_coding_stage_matches_oracle(vpp, ctx, orc):
    """Jobs with the coding stage (residual at the vectors, T+Q at QP 28 inter
    and its inverse): vectors, residual, levels and reconstruction of every job
    equal the oracle's chain (Full estimate, QuarterRead residual, 4x4 round
    trip), on several streams, with a partial bottom row and a job without the
    stage in the same batch."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    sizes = [(176, 144, 128, 28), (352, 288, 128, 28), (208, 120, 96, 17), (176, 152, 128, 40)]
    jobs, keep = [], []
    for i, (w, h, mr, qp) in enumerate(sizes):
        fr = synth.pan_sequence(320 + i, w, h, 2)
        src, ref = torch.from_numpy(fr[1]).to(dev), torch.from_numpy(fr[0]).to(dev)
        nmb = (w // 16) * (h // 16)
        mv = torch.zeros((nmb, 2), dtype=torch.int16, device=dev)
        bufs = [torch.full((h, w), 9, dtype=torch.int16, device=dev) for _ in range(3)]
        keep.append((fr, src, ref, mv, bufs, w, h, mr, qp))
        jobs.append((src.data_ptr(), ref.data_ptr(), w, h, mr, mv.data_ptr(), None, None,
                     *[b.data_ptr() for b in bufs], qp))
    fr = synth.pan_sequence(330, 176, 144, 2)
    plain_src, plain_ref = torch.from_numpy(fr[1]).to(dev), torch.from_numpy(fr[0]).to(dev)
    plain_mv = torch.zeros((99, 2), dtype=torch.int16, device=dev)
    jobs.append((plain_src.data_ptr(), plain_ref.data_ptr(), 176, 144, 128, plain_mv.data_ptr()))
    batch = vpp.MotionEstimatorBatch(streams=3, ctx=ctx)
    st, _ = batch.run(jobs)
    torch.cuda.synchronize()
    assert st == [0] * len(jobs)
    np.testing.assert_array_equal(plain_mv.cpu().numpy(), orc.me_full(fr[1], fr[0], 128)[0])
    for fr, src, ref, mv, (res, lev, rec), w, h, mr, qp in keep:
        mv_o, _, _ = orc.me_full(fr[1], fr[0], mr)
        np.testing.assert_array_equal(mv.cpu().numpy(), mv_o)
        cols, rows = w // 16, h // 16
        hh = 16 * rows
        res_o = np.zeros((hh, w), np.int32)
        for k in range(cols * rows):
            n, m = (k % cols) * 16, (k // cols) * 16
            vx, vy = int(mv_o[k, 0]), int(mv_o[k, 1])
            qx, qy = int(np.fmod(vx, 4)), int(np.fmod(vy, 4))
            pred = orc.quarter_read16(fr[0], n + (vx - qx) // 4, m + (vy - qy) // 4, qx, qy)
            res_o[m:m + 16, n:n + 16] = fr[1][m:m + 16, n:n + 16].astype(np.int32) - pred
        np.testing.assert_array_equal(res.cpu().numpy()[:hh], res_o)
        blocks = res_o.astype(np.int16).reshape(hh // 4, 4, w // 4, 4).transpose(0, 2, 1, 3).reshape(-1, 16)
        lev_o = orc.fwd4x4(blocks, 0, 0, qp, 0)
        rec_o = orc.inv4x4(lev_o, 0, 0, qp)
        back = lambda b: b.reshape(hh // 4, w // 4, 4, 4).transpose(0, 2, 1, 3).reshape(hh, w)
        np.testing.assert_array_equal(lev.cpu().numpy()[:hh], back(lev_o))
        np.testing.assert_array_equal(rec.cpu().numpy()[:hh], back(rec_o))
    bad = list(jobs[0])
    bad[11] = 52  # QP out of range
    with pytest.raises(vpp.VppGpuError):
        batch.run([tuple(bad)])
    batch.close()
