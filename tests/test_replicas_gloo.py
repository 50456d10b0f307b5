"""The N > 1 path of bench.py on CPU: two gloo ranks run replicas, the timed
region's times are reduced with MAX over ranks, and the whole-job value is
all ranks' useful bytes over the slowest rank's time (the GPU run uses the
same functions over NCCL)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = [10.0 + 5.0 * rank, 20.0 - rank]  # per-rank total_ms, e2e_ms
        slow = bench.max_over_ranks(local, dist, "cpu")
        dist.barrier()
        q.put((rank, slow, bench.whole_job_gbs(bench.N, slow[0], 4, world)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_reduce_to_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    import sys
    sys.path.insert(0, ROOT)
    import bench
    for rank, slow, value in res:
        assert slow == [15.0, 20.0]
        assert value == pytest.approx(bench.useful_gbs(bench.N, 15.0 / 1e3, 4 * world))
