"""Multi-rank host logic of bench.py on CPU: two gloo ranks on 127.0.0.1."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    step = 0.10 + 0.05 * rank                   # rank 1 is the slower one
    slowest = bench.rank_reduce_max(step, dist, "cpu")
    rate = bench.whole_job_rate(world, 42, slowest)
    # the reference arm runs on rank 0 only; the others return 0 without work
    skipped = None
    if rank != 0:
        class A:  # the arguments reference_arm reads before it checks the rank
            workload, steps, warmup, gpus = "nmax10_lanczos100", 1, 0, world
        skipped = bench.reference_arm(A())
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, slowest, rate, skipped))


def test_two_gloo_ranks_agree_on_slowest_step_and_rate():
    world, port = 2, _free_port()
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, rate, skipped in res:
        assert slowest == pytest.approx(0.15)
        assert rate == pytest.approx(2 * 42 / 0.15)
    assert res[1][3] == 0


def test_single_process_needs_no_group():
    import bench
    assert bench.rank_reduce_max(0.3, None, "cpu") == 0.3
    assert bench.whole_job_rate(1, 42, 0.2) == pytest.approx(210.0)
