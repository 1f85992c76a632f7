"""The multi-GPU path on CPU: `bench.py --gpus N` runs N independent replicas (a single cloth does
not shard; batches partition with no collective on the data path), so the only cross-rank steps
are the barrier and the MAX of the timings. Two gloo ranks on 127.0.0.1 check the aggregate the
bench reports, and that the reference arm runs on rank 0 alone.
"""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, seconds, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        rate, t_max = bench.replica_rate(600, seconds[rank], world)
        out[rank] = (rate, t_max)
    finally:
        dist.destroy_process_group()


def test_replica_rate_takes_the_slowest_rank():
    world, port = 2, _free_port()
    seconds = [0.25, 0.40]
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, seconds, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        results = dict(out)
    for r in range(world):
        rate, t_max = results[r]
        assert t_max == 0.40 and rate == pytest.approx(world * 600 / 0.40)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    rate, t_max = bench.replica_rate(100, 0.5, 1)
    assert rate == 200.0 and t_max == 0.5


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference"])
    assert bench.main() == 0
    assert capsys.readouterr().out == ""
