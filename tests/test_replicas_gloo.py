"""The multi-GPU path of bench.py: independent replicas, one per rank, whose
timings are combined by a max over ranks (no data-path collective).

Runs two `gloo` ranks on the CPU. Registration itself is per-GPU and is
covered by the GPU tests; here the rank logic is checked: the max-over-ranks
reduction, the whole-job rate, and that only rank 0 runs the CPU reference arm.
"""
import multiprocessing as mp
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    try:
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                          WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
        sys.path.insert(0, ROOT)
        import torch.distributed as dist

        import bench

        assert bench.dist_env() == (rank, world, rank)
        dist.init_process_group(backend="gloo", rank=rank, world_size=world)
        # rank r pretends its timed region took (10 + r) ms of device time and
        # (1 + 2r) s end to end
        total_ms, e2e_s = bench.max_over_ranks([10.0 + rank, 1.0 + 2.0 * rank], world, "cpu")
        rate = bench.whole_job_rate(4, world, total_ms * 1e-3)

        # the reference arm: ranks other than 0 return at once, without work
        class Args:
            workload = "c1_emicp_1007"
            seed = 0
            steps = 1
            warmup = 0
            cpu_sample_s = 0.0

        ran_reference = None
        if rank != 0:
            bench.run_reference(Args(), rank, world)
            ran_reference = False
        dist.barrier()
        dist.destroy_process_group()
        q.put((rank, total_ms, e2e_s, rate, ran_reference))
    except Exception as e:  # surfaced by the parent
        q.put((rank, "error", repr(e), None, None))


def test_replicas_max_over_ranks_gloo():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(world):
        r = q.get(timeout=180)
        out[r[0]] = r
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(world):
        assert out[r][1] != "error", out[r]
        _, total_ms, e2e_s, rate, _ = out[r]
        # every rank sees the slowest rank's times
        assert total_ms == pytest.approx(11.0)
        assert e2e_s == pytest.approx(3.0)
        # 4 registrations on each of 2 ranks in 11 ms
        assert rate == pytest.approx(8 / 0.011)
    assert out[1][4] is False


def test_whole_job_rate_single_rank():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.whole_job_rate(10, 1, 2.0) == pytest.approx(5.0)
    assert bench.max_over_ranks([1.5, 2.5], 1, "cpu") == [1.5, 2.5]
