"""The benchmark workloads at their full sizes against the FP64 CPU oracle, run as the bench runs them.

* cloth256: one 256 × 256 cloth (65,536 vertices, 195,585 distance + shear edges, 130,048 bend
  stencils), 20 iterations, 300 substeps: MIXED (correction form on a grid team of CTAs) and FP32
  projection within 1e-5 of the oracle after all 300 substeps, FP64 within 1e-10.
* batch: the 512 cloths of 16²–128² in one launch, MIXED, 300 substeps: the 16 largest cloths and 16
  more drawn with a fixed seed, each within 1e-5 of its own oracle run.
* differentiable: the 64 × 64 cloth over 120 substeps (10 iterations each): loss and gradients of the
  GPU adjoint against the oracle's FP64 adjoint.

The oracle runs of the batch go to spawned worker processes (one thread each), started after the
GPU is in use, which spawning allows.
"""
import copy
import multiprocessing as mp
import os

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import max_rel, oracle_twin

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-5
TOL_FP64 = 1e-10


@pytest.fixture(scope="module")
def cloth256_oracle(pdg):
    scenes, cfg, S = W.cloth256()
    probe = pdg.Simulator(scenes[0], cfg)  # the elimination order every mode uses
    perm = probe.factor()["perm"]
    probe.close()
    orc = oracle_twin(scenes[0], cfg, perm=perm, threads=os.cpu_count() or 1)
    its_a, _ = orc.step(100)
    x100 = orc.state()[0]
    its_b, _ = orc.step(S - 100)
    return {"scene": scenes[0], "cfg": cfg, "S": S, "x100": x100, "x": orc.state()[0],
            "its": np.concatenate([its_a, its_b])}


def _run(pdg, ref, precision, substeps):
    c = copy.copy(ref["cfg"])
    c.precision = precision
    sim = pdg.Simulator(ref["scene"], c)
    sim.step(substeps)
    return sim


@pytest.mark.parametrize("precision", [4, 2])
def test_cloth256_reduced_precision_300_substeps(pdg, cloth256_oracle, precision):
    ref = cloth256_oracle
    sim = _run(pdg, ref, precision, ref["S"])
    info = sim.info()
    assert info["cluster_ctas"] > 16  # one cloth on a grid team, as benchmarked
    x = sim.state()[0]
    err = max_rel(x, ref["x"])
    assert err <= TOL_MIXED, err
    pins = np.flatnonzero(ref["scene"].pinned)
    assert np.array_equal(x[pins], ref["scene"].positions[pins])


def test_cloth256_fp64(pdg, cloth256_oracle):
    ref = cloth256_oracle
    c = copy.copy(ref["cfg"])
    c.precision = 1
    sim = pdg.Simulator(ref["scene"], c)
    sim.step(100)
    its_a = sim.iteration_log()[0].copy()
    assert max_rel(sim.state()[0], ref["x100"]) <= TOL_FP64
    sim.step(ref["S"] - 100)
    its_b = sim.iteration_log()[0]
    assert np.array_equal(np.concatenate([its_a, its_b]), ref["its"])
    assert max_rel(sim.state()[0], ref["x"]) <= TOL_FP64


# ---------------------------------------------------------------------------- 512-cloth batch
_BATCH = None


def _batch_init():
    global _BATCH
    from oracle import workloads as OW
    _BATCH = OW.batch(count=512, threads=1)


def _batch_oracle(i):
    """Final positions of batch cloth i after the workload's substeps on the oracle (1 thread)."""
    from oracle import oracle as O
    meshes, cfgs, S = _BATCH
    sim = O.OracleSim(meshes[i], cfgs[i])
    sim.step(S)
    return i, sim.state()[0]


def test_batch512_mixed_300_substeps(pdg):
    scenes, cfgs, S = W.batch(count=512)
    cfgs = [copy.copy(c) for c in cfgs]
    for c in cfgs:
        c.precision = 4
    sizes = np.array([s.n for s in scenes])
    largest = list(np.argsort(-sizes, kind="stable")[:16])
    rest = [i for i in range(512) if i not in largest]
    sample = list(np.random.default_rng(512).choice(rest, 16, replace=False))
    picks = sorted(int(i) for i in largest + sample)
    ctx = mp.get_context("spawn")
    workers = max(1, min(len(picks), os.cpu_count() or 1))
    with ctx.Pool(workers, initializer=_batch_init) as pool:
        pending = pool.map_async(_batch_oracle, picks, chunksize=1)
        sim = pdg.Simulator(scenes, cfgs)  # the run as benchmarked: every cloth in one handle
        sim.step(S)
        got = {i: sim.state(i)[0] for i in picks}
        want = dict(pending.get(timeout=1800))
    errs = {i: max_rel(got[i], want[i]) for i in picks}
    worst = max(errs, key=errs.get)
    assert errs[worst] <= TOL_MIXED, (worst, errs[worst], int(sizes[worst]))
    for i in picks:
        pins = np.flatnonzero(scenes[i].pinned)
        assert np.array_equal(got[i][pins], scenes[i].positions[pins]), i


# ---------------------------------------------------------------------------- 64 × 64 gradients
def test_differentiable_64x64_gradient_matches_cpu_adjoint(pdg):
    scene, cfg, S, kstar = W.differentiable()
    c = copy.copy(cfg)
    c.precision = 1
    twin = oracle_twin(scene, c, threads=os.cpu_count() or 1)
    twin.set_edge_stiffness(kstar)
    twin.step(S)
    targets = twin.state()[0]
    rng = np.random.default_rng(64)
    force = rng.normal(0.0, 0.05, (scene.n, 3))
    sim = pdg.Simulator(scene, c)
    g = sim.gradient(S, targets, force)
    orc = oracle_twin(scene, c, perm=sim.factor()["perm"])
    r = orc.gradient(S, targets, force)
    assert abs(g["loss"] - r["loss"]) <= 1e-10 * r["loss"]
    for key in ("dkappa", "dv0", "dforce"):
        rel = np.linalg.norm(g[key] - r[key]) / np.linalg.norm(r[key])
        assert rel < 1e-8, (key, rel)
