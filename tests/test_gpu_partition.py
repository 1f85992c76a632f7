"""A batch split across ranks on the GPU: two processes (gloo for the final gather), each stepping its
part of a batch with the product's simulator, gather on rank 0 exactly the states one process gets
stepping the whole batch. The two processes share the one GPU here; their kernels are independent
(no rank waits on another's kernel), as on separate GPUs. One CTA per cloth (cluster_ctas = 1) keeps
each cloth's launch plan independent of the batch it is in, so the bits are comparable.
"""
import copy
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SUBSTEPS = 12


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _batch(precision):
    from pd_gb300 import workloads as W
    scenes, cfgs, _ = W.batch(count=14, max_side=48)
    cfgs = [copy.copy(c) for c in cfgs]
    for c in cfgs:
        c.precision = precision
        c.cluster_ctas = 1
    return scenes, cfgs


def _rank(rank, world, port, precision, out):
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import pd_gb300 as P
    from pd_gb300 import partition as PT
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        scenes, cfgs = _batch(precision)
        parts = PT.partition(PT.scene_costs(scenes, cfgs), world)
        mine = parts[rank]
        sim = P.Simulator([scenes[i] for i in mine], [cfgs[i] for i in mine])
        sim.step(SUBSTEPS)
        local = [sim.state(k) for k in range(len(mine))]
        got = PT.gather_states(parts, local, rank, world)
        if rank == 0:
            out["states"] = [(x.copy(), v.copy()) for x, v in got]
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("precision", [4, 1])
def test_two_ranks_gather_the_one_process_batch(pdg, precision):
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, precision, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(600)
            assert p.exitcode == 0
        states = dict(out)["states"]
    scenes, cfgs = _batch(precision)
    sim = pdg.Simulator(scenes, cfgs)
    sim.step(SUBSTEPS)
    for i in range(len(scenes)):
        x, v = sim.state(i)
        gx, gv = states[i]
        assert np.array_equal(gx.view(np.uint64), x.view(np.uint64)), i
        assert np.array_equal(gv.view(np.uint64), v.view(np.uint64)), i
