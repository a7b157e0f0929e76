"""Multi-rank host logic of bench.py on CPU: gloo, world_size 2.

Replicas only (every rank renders its own frames); the job's step time is the
slowest rank's, and the reference arm runs on rank 0 alone.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        w, r, local = bench.dist_env()
        ms = 2.0 + 3.0 * rank  # rank 1 is the slow one
        slow = bench.max_over_ranks(ms, w, "cpu")
        value = bench.job_mpix_per_s(1920 * 1080, w, slow)
        dist.barrier()
        q.put((r, w, slow, value))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    assert [g[0] for g in got] == [0, 1] and all(g[1] == 2 for g in got)
    assert all(g[2] == 5.0 for g in got)  # every rank sees the slowest rank's time
    want = 2 * 1920 * 1080 / 5e-3 / 1e6
    assert all(abs(g[3] - want) < 1e-9 for g in got)


def test_reference_arm_runs_on_rank0_only(capsys):
    import bench

    class A:
        warmup, steps, gpus = 0, 1, 2
    bench.run_reference(A, 2, 1)  # rank 1: no work, no output
    assert capsys.readouterr().out == ""
