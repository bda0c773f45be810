"""The bench's replica harness on two CPU ranks (gloo).

Frames are independent, so N GPUs run N replicas with no exchange on the
data path; the only collective is the timing reduction (the slowest rank's
time).  These checks run that reduction and the reference arm's rank
handling in two processes with the gloo backend.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        # each replica reports its own time; every rank must see the largest
        got = bench.max_over_ranks(10.0 + 5.0 * rank)
        # the reference arm runs on rank 0 only: other ranks return at once
        ran = None
        if rank != 0:
            ran = bench.run_reference(type("A", (), {"steps": 1, "warmup": 0})())
        out.put((rank, got, bench.dist_env(), ran))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_reference_arm_on_two_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in results] == [15.0, 15.0]
    assert [r[2] for r in results] == [(2, 0, 0), (2, 1, 1)]
    assert results[1][3] is None


def test_max_over_ranks_single_process_is_identity():
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
