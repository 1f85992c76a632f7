"""Triangle meshes from OBJ text (Mesh::loadObj, core/mesh/Mesh.cpp:56-153) stepped on the GPU
against the oracle: bit-identical in the reference-order FP64 mode, within 1e-10 in FP64 and 1e-5
in MIXED. The sheet's vertices are listed in a shuffled order, so vertex numbering carries no
locality."""
import copy

import numpy as np
import pytest

from tests.helpers import bits, max_rel, obj_sheet, oracle_twin

pytestmark = pytest.mark.gpu


def obj_scene(pdg, nx=13, ny=10, seed=3, **kw):
    cfg = pdg.SceneConfig(stiffness=3000.0, dt=1 / 240, max_iterations=20, **kw)
    scene = pdg.make_obj(obj_sheet(nx, ny, seed=seed), cfg)
    # pin the two file vertices nearest the corners of the sheet's first row
    x = scene.positions
    scene.pinned[int(np.argmin(x[:, 0] + x[:, 2]))] = 1
    scene.pinned[int(np.argmin(-x[:, 0] + x[:, 2]))] = 1
    return scene, cfg


def test_reference_order_bit_identical(pdg):
    scene, cfg = obj_scene(pdg)
    sim = pdg.Simulator(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(30)
    it_o, cv_o = orc.step(30)
    it_g, cv_g = sim.iteration_log()
    assert np.array_equal(it_g, it_o) and np.array_equal(cv_g, cv_o)
    xg, vg = sim.state()
    xo, vo = orc.state()
    assert np.array_equal(bits(xg), bits(xo)) and np.array_equal(bits(vg), bits(vo))


@pytest.mark.parametrize("precision,tol", [(1, 1e-10), (4, 1e-5)])
@pytest.mark.parametrize("ctas", [0, 1])
def test_fast_modes_within_tolerance(pdg, precision, tol, ctas):
    scene, cfg = obj_scene(pdg, nx=17, ny=12, seed=5)
    c = copy.copy(cfg)
    c.precision = precision
    c.cluster_ctas = ctas
    sim = pdg.Simulator(scene, c)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(120)
    it_o, _ = orc.step(120)
    assert max_rel(sim.state()[0], orc.state()[0]) < tol
    assert np.mean(sim.iteration_log()[0] == it_o) > 0.95


def test_batch_of_obj_and_grid_cloths(pdg):
    a, cfg = obj_scene(pdg, nx=9, ny=9, seed=1)
    b, _ = obj_scene(pdg, nx=15, ny=6, seed=2)
    g = pdg.make_grid(pdg.SceneConfig(grid_nx=12, grid_ny=12, stiffness=3000.0))
    c = copy.copy(cfg)
    c.precision = pdg.PD_PRECISION_MIXED
    sim = pdg.Simulator([a, b, g], [c] * 3)
    sim.step(40)
    for i, s in enumerate((a, b, g)):
        orc = oracle_twin(s, cfg, perm=sim.factor(i)["perm"])
        orc.step(40)
        assert max_rel(sim.state(i)[0], orc.state()[0]) < 1e-5, i
