"""The multi-GPU bench path on CPU: two gloo ranks (127.0.0.1) run the
host logic of `bench.py --gpus 2` -- independent shards, max-over-ranks
timing, whole-job throughput, the reference arm's rank > 0 exit -- with no
GPU.  The path shards by sequence with no data-path collective."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    # per-rank timings: the slowest rank's numbers set the whole job's
    dev_ms, e2e_ms = bench.max_over_ranks(torch, dist, [10.0 + 5 * rank, 20.0 - 3 * rank], "cpu")
    dist.barrier()
    seeds = [None] * world
    dist.all_gather_object(seeds, bench.shard_seed(rank))
    ref_rc = bench.run_reference(None, rank, world) if rank > 0 else 0
    out.put((rank, dev_ms, e2e_ms, seeds, ref_rc))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, dev_ms, e2e_ms, seeds, ref_rc in res:
        assert dev_ms == 15.0 and e2e_ms == 20.0  # max over ranks on every rank
        assert len(set(seeds)) == 2                # independent shards
        assert ref_rc == 0                         # the reference arm: only rank 0 works and prints


def test_whole_job_rate():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.whole_job_rate(8040 * 100, 2, 1000.0) == pytest.approx(8040 * 100 * 2)
    assert bench.shard_seed(0) != bench.shard_seed(1)
