"""Serving loop (vppgpu_server_*): sequence requests of mixed sizes submitted
together run concurrently on several slots and give, per request, the same
vectors and transform digests as the same request alone, and as the CPU
oracle (Full estimate, QuarterRead residual, 4x4 round trip) per frame pair."""
import numpy as np
import pytest

from imagecodingutils_gb300 import synth

pytestmark = pytest.mark.gpu

REQS = [(176, 144, 4, 128, 28), (352, 288, 3, 128, 22), (208, 120, 5, 96, 30), (176, 144, 3, 64, 28),
        (352, 288, 4, 128, 36), (176, 144, 5, 128, 12)]


def oracle_request(orc, frames, mr, qp):
    nfr, h, w = frames.shape
    cols, rows = w // 16, h // 16
    mvs, digs = [], []
    for t in range(1, nfr):
        mv, _, _ = orc.me_full(frames[t], frames[t - 1], mr)
        res = np.zeros((16 * rows, w), np.int32)
        for k in range(cols * rows):
            n, m = (k % cols) * 16, (k // cols) * 16
            vx, vy = int(mv[k, 0]), int(mv[k, 1])
            qx, qy = int(np.fmod(vx, 4)), int(np.fmod(vy, 4))
            pred = orc.quarter_read16(frames[t - 1], n + (vx - qx) // 4, m + (vy - qy) // 4, qx, qy)
            res[m:m + 16, n:n + 16] = frames[t][m:m + 16, n:n + 16].astype(np.int32) - pred
        hh = 16 * rows
        blocks = res.astype(np.int16).reshape(hh // 4, 4, w // 4, 4).transpose(0, 2, 1, 3).reshape(-1, 16)
        lev = orc.fwd4x4(blocks, 0, 0, qp, 0)
        rec = orc.inv4x4(lev, 0, 0, qp)
        digs.append(int(lev.astype(np.int64).sum() + 3 * rec.astype(np.int64).sum()) & (2 ** 64 - 1))
        mvs.append(mv)
    return np.stack(mvs), np.array(digs, np.uint64)


def test_server_mix_matches_alone_and_oracle(vpp, ctx, orc):
    seqs = [np.stack(synth.pan_sequence(700 + i, w, h, nf)) for i, (w, h, nf, _, _) in enumerate(REQS)]
    srv = vpp.Server(slots=3, ctx=ctx)
    outs = [srv.submit(s, mr, qp) for s, (_, _, _, mr, qp) in zip(seqs, REQS)]
    srv.wait_idle()
    done = srv.poll()
    assert sorted(t for t, _, _ in done) == sorted(t for t, _, _ in outs)
    assert all(st == 0 for _, st, _ in done)
    assert all(lat > 0 for _, _, lat in done)
    assert srv.stats()["running_peak"] >= 2  # requests overlapped
    srv.close()
    alone = vpp.Server(slots=1, ctx=ctx)
    for s, (_, _, _, mr, qp), (_, mv, dig) in zip(seqs, REQS, outs):
        _, mv1, dig1 = alone.submit(s, mr, qp)
        alone.wait_idle()
        np.testing.assert_array_equal(mv1, mv)
        np.testing.assert_array_equal(dig1, dig)
    alone.close()
    for s, (_, _, _, mr, qp), (_, mv, dig) in list(zip(seqs, REQS, outs))[:3]:
        mv_o, dig_o = oracle_request(orc, s, mr, qp)
        np.testing.assert_array_equal(mv, mv_o)
        np.testing.assert_array_equal(dig, dig_o)


def test_server_budget_and_bad_request(vpp, ctx):
    srv = vpp.Server(slots=2, hbm_budget=400_000, ctx=ctx)  # one QCIF job's buffers (~260 KB) at a time
    seq = np.stack(synth.pan_sequence(777, 176, 144, 3))
    outs = [srv.submit(seq, 128, 28) for _ in range(3)]
    srv.wait_idle()
    assert all(st == 0 for _, st, _ in srv.poll())
    assert srv.stats()["running_peak"] == 1
    for o in outs[1:]:
        np.testing.assert_array_equal(o[1], outs[0][1])
        np.testing.assert_array_equal(o[2], outs[0][2])
    big = np.zeros((3, 1088, 1920), np.int16)
    with pytest.raises(vpp.VppGpuError):
        srv.submit(big, 128, 28)  # cannot fit the budget
    bad = seq.copy()
    bad[1, 5, 5] = 999
    srv.submit(bad, 128, 28)
    srv.wait_idle()
    assert [st for _, st, _ in srv.poll()] == [-4]
    srv.close()
