"""The multi-GPU path of bench.py on CPU: world size 2 over gloo (127.0.0.1).

The path shards nothing -- every rank runs a replica of the city batch -- so
the host logic to cover is the job's time (the maximum over ranks, which
bench.max_over_ranks computes for the device and end-to-end figures) and the
reference arm, which only rank 0 runs."""
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

torch = pytest.importorskip("torch")
dist = pytest.importorskip("torch.distributed")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        mine = [3.25, 7.5][rank]
        got = bench.max_over_ranks(mine, "cpu")
        ran = bench.reference_arm(None) if rank != 0 else "skipped"  # ranks other than 0 return at once
        out.put((rank, got, ran))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_job_time_is_the_maximum_over_two_gloo_ranks():
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
    assert res == [(0, 7.5, "skipped"), (1, 7.5, None)]


def test_one_rank_keeps_its_own_time():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(4.0, "cpu") == 4.0
