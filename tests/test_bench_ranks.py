"""bench.py's replica path on CPU: two gloo ranks agree on the slowest
rank's time, and the whole-job rate counts every rank's work (the GPU bench
runs one filter per GPU, no data exchange, and reduces its timings this way
over NCCL)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        slowest = bench.max_over_ranks(1.0 + rank, dist, "cpu")
        out.put((rank, slowest, bench.job_rate(1e6, world, slowest)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_slowest():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.0, 2.0]
    assert res[0][2] == pytest.approx(1.0)  # 2 ranks x 1e6 keys in 2 s = 1 Mkeys/s


def test_single_rank_passes_through():
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.job_rate(2e6, 1, 2.0) == pytest.approx(1.0)
