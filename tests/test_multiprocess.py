"""CPU: the bench's multi-rank path (replicas, one text per rank, no
collective on the data path) with world_size 2 on gloo: the job time is the
slowest rank's, the job throughput counts every rank's symbols, ranks build
different texts, and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [3.0, 5.0][rank]  # rank 1 is the slow one
        job_ms = bench.max_over_ranks(ms, dist, "cpu")
        value = bench.job_throughput(world, 1 << 30, job_ms / 1e3)
        dist.barrier()

        class Args:
            steps, warmup, gpus = 1, 1, world

        ref = bench.run_reference(Args, rank) if rank == 1 else None
        q.put((rank, job_ms, value, bench.replica_seed(rank), ref))
    finally:
        dist.destroy_process_group()


def test_replicas_two_ranks_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    (r0, ms0, v0, seed0, _), (r1, ms1, v1, seed1, ref1) = got
    assert ms0 == ms1 == 5.0                     # the job takes as long as its slowest rank
    assert v0 == v1 == pytest.approx(2 * (1 << 30) / 5e-3 / 1e9)
    assert seed0 != seed1                        # each rank builds its own text
    assert ref1 == 0                             # the reference arm does no work off rank 0
