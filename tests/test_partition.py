"""A batch of independent cloths split across ranks (pd_gb300.partition), on the CPU.

Two gloo ranks on 127.0.0.1 each step their part of a batch (here with the oracle, the CPU
restatement of the substep) and gather the final states on rank 0, which must equal the states of
one process stepping the whole batch, bit for bit. The split itself: every cloth on exactly one
rank, the same split on every rank, loads balanced to within the largest cloth.
"""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _costs(meshes, cfgs):
    from pd_gb300 import partition as PT
    return PT.scene_costs(meshes, cfgs)


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_partition_covers_every_cloth_once_and_balances(world):
    from oracle import workloads as OW
    from pd_gb300 import partition as PT
    meshes, cfgs, _ = OW.batch(count=512)
    costs = _costs(meshes, cfgs)
    parts = PT.partition(costs, world)
    assert len(parts) == world
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(512))
    assert all(p == sorted(p) for p in parts)
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs) + 1e-9 * sum(costs)
    assert PT.partition(costs, world) == parts  # deterministic


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from oracle import oracle as O, workloads as OW
    from pd_gb300 import partition as PT
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        meshes, cfgs, _ = OW.batch(count=10, max_side=22, threads=1)
        parts = PT.partition(_costs(meshes, cfgs), world)
        local = []
        for i in parts[rank]:
            sim = O.OracleSim(meshes[i], cfgs[i])
            sim.step(6)
            local.append(sim.state())
        got = PT.gather_states(parts, local, rank, world)
        if rank == 0:
            out["states"] = [(x.copy(), v.copy()) for x, v in got]
            out["parts"] = parts
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_the_one_rank_result():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(300)
            assert p.exitcode == 0
        res = dict(out)
    assert all(len(p) > 0 for p in res["parts"])
    sys.path.insert(0, ROOT)
    from oracle import oracle as O, workloads as OW
    meshes, cfgs, _ = OW.batch(count=10, max_side=22, threads=1)
    for i, (m, c) in enumerate(zip(meshes, cfgs)):
        sim = O.OracleSim(m, c)
        sim.step(6)
        x, v = sim.state()
        gx, gv = res["states"][i]
        assert np.array_equal(gx.view(np.uint64), x.view(np.uint64)), i
        assert np.array_equal(gv.view(np.uint64), v.view(np.uint64)), i


def test_gather_on_one_rank_is_the_identity():
    from pd_gb300 import partition as PT
    parts = PT.partition([3.0, 1.0, 2.0], 1)
    states = [(np.full((2, 3), i), np.zeros((2, 3))) for i in range(3)]
    assert PT.gather_states(parts, states, 0, 1) == states
    with pytest.raises(ValueError):
        PT.gather_states(parts, states[:2], 0, 1)
