"""The N > 1 path of bench.py (replicas only: one independent GPU step loop
per rank, no collective in the step) with two gloo ranks on the CPU: the
timed duration is the maximum over ranks and the whole-job throughput
counts every rank's cells; the reference arm prints from rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, ROOT)
        import bench
        ms, value = bench.replicas_result(10.0 + 5.0 * rank, 1000, 4, world,
                                          torch.device("cpu"))
        out[rank] = (ms, value)
    finally:
        dist.destroy_process_group()


def test_replicas_timing_is_the_max_over_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert set(res) == {0, 1}
    for ms, value in res.values():
        assert ms == 15.0
        assert value == pytest.approx(1000 * 2 * 4 / 15e-3 / 1e6)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    ms, value = bench.replicas_result(8.0, 500, 2, 1, torch.device("cpu"))
    assert ms == 8.0 and value == pytest.approx(500 * 2 / 8e-3 / 1e6)


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
