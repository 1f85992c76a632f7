"""The oracle's own workload builder (used by the CPU arms of the bench) builds exactly the cloths
the product's workload builder does: same arrays, same bits, same configuration knobs."""
import numpy as np
import pytest

from tests.helpers import bits

FIELDS = [("positions", "positions"), ("masses", "masses"), ("pinned", "pinned"), ("edges", "edges"),
          ("edge_rest", "edge_rest"), ("edge_stiffness", "edge_k"), ("bends", "bends"), ("bend_stiffness", "bend_k")]


def _same(scene, mesh):
    for a, b in FIELDS:
        x = np.asarray(getattr(scene, a))
        y = np.asarray(getattr(mesh, b))
        assert x.shape == y.shape or x.size == y.size == 0, a
        if x.dtype == np.float64:
            assert np.array_equal(bits(x), bits(y)), a
        else:
            assert np.array_equal(x.reshape(y.shape), y), a


def _same_cfg(cfg, ocfg):
    for f in ("dt", "velocity_damping", "max_iterations", "rel_tolerance", "abs_tolerance", "residual_tolerance"):
        assert getattr(cfg, f) == getattr(ocfg, f), f
    assert tuple(cfg.gravity) == tuple(ocfg.gravity)


@pytest.mark.parametrize("name", ["cloth40_plain", "cloth40_full", "cloth256"])
def test_single_cloth_workloads_match(pdg, name):
    from oracle import workloads as OW
    from pd_gb300 import workloads as W
    scenes, cfg, sub = W.WORKLOADS[name]()
    meshes, ocfgs, osub = OW.build(name)
    assert sub == osub and len(scenes) == len(meshes) == 1
    _same(scenes[0], meshes[0])
    _same_cfg(cfg, ocfgs[0])


def test_batch_workload_matches(pdg):
    from oracle import workloads as OW
    from pd_gb300 import workloads as W
    scenes, cfgs, sub = W.batch(count=40)
    meshes, ocfgs, osub = OW.batch(count=40)
    assert sub == osub
    for s, c, m, oc in zip(scenes, cfgs, meshes, ocfgs):
        _same(s, m)
        _same_cfg(c, oc)


def test_differentiable_workload_matches(pdg):
    from oracle import workloads as OW
    from pd_gb300 import workloads as W
    scene, cfg, sub, kstar = W.differentiable(side=20, seed=7)
    mesh, ocfg, osub, okstar = OW.differentiable(side=20, seed=7)
    assert sub == osub
    _same(scene, mesh)
    _same_cfg(cfg, ocfg)
    assert np.array_equal(bits(kstar), bits(okstar))
