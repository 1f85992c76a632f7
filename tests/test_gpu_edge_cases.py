"""Edge cases the reference's own checks exercise (_verify/check.cpp: free fall, pinned vertices
exact, all pinned), plus the ragged and boundary sizes of this implementation, in every precision
mode: a lone vertex with no constraints, a cloth with every vertex pinned, zero iterations, a batch
mixing a one-vertex scene with a cloth at the explicit-inverse limit, and the first size above it.
"""
import copy

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import bits, max_rel, oracle_twin

pytestmark = pytest.mark.gpu

PRECISIONS = [0, 1, 2, 3, 4]
TOL = {0: 0.0, 1: 1e-10, 2: 1e-5, 3: 1e-5, 4: 1e-5}


def with_precision(cfg, p, ctas=0):
    c = copy.copy(cfg)
    c.precision = p
    c.cluster_ctas = ctas
    return c


def lone_vertex(pdg):
    return pdg.GridScene(np.array([[0.1, 0.5, -0.2]]), np.array([0.05]), np.zeros(1, np.uint8),
                         np.zeros((0, 2), np.int32), np.zeros(0), np.zeros(0))


@pytest.mark.parametrize("p", PRECISIONS)
def test_free_fall_of_a_lone_vertex(pdg, p):
    """check.cpp item 5: one free vertex, no constraints: x = x0 − h²·g·(1 + 2 + …) exactly as the
    oracle computes it."""
    cfg = W._base(max_iterations=4)
    scene = lone_vertex(pdg)
    sim = pdg.Simulator(scene, with_precision(cfg, p))
    orc = oracle_twin(scene, cfg)
    sim.step(10)
    orc.step(10)
    xg, vg = sim.state()
    xo, vo = orc.state()
    if p == 0:
        assert np.array_equal(bits(xg), bits(xo)) and np.array_equal(bits(vg), bits(vo))
    else:
        # FP32 modes: Ã⁻¹ = h²/m rounded to FP32 scales each correction, so the gap is ~6e-8 of
        # the per-substep displacement (measured 1.2e-10 of |x| after 10 substeps)
        assert max_rel(xg, xo) <= TOL[p] and max_rel(vg, vo) <= TOL[p]


@pytest.mark.parametrize("p", PRECISIONS)
def test_all_pinned_cloth_never_moves(pdg, p):
    """check.cpp item 4 with every vertex pinned: positions stay exactly at the pins."""
    cfg = W._base(grid_nx=8, grid_ny=6, grid_spacing=0.05, max_iterations=5, pin_mode=2)
    scene = pdg.make_grid(cfg)
    scene.pinned[:] = 1
    sim = pdg.Simulator(scene, with_precision(cfg, p))
    sim.step(20)
    x, v = sim.state()
    assert np.array_equal(x, scene.positions) and not np.any(v)


@pytest.mark.parametrize("p", PRECISIONS)
def test_zero_iterations(pdg, p):
    """max_iterations = 0: no PD iteration, the state is the velocity update of x = x_n."""
    cfg = W._base(grid_nx=10, grid_ny=10, grid_spacing=0.05, max_iterations=0)
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, with_precision(cfg, p))
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(5)
    orc.step(5)
    if p == 4:
        # MIXED keeps positions as FP32 hi/lo pairs (48-bit significands), so x_n itself is
        # rounded to 2⁻⁴⁸ relative when the pairs are formed
        assert max_rel(sim.state()[0], orc.state()[0]) <= 1e-14
    else:
        assert np.array_equal(sim.state()[0], orc.state()[0])
    assert sim.stats()["iterations_used"] == 0


@pytest.mark.parametrize("p", [1, 3, 4])
def test_ragged_batch_at_the_inverse_limit(pdg, p):
    """A one-vertex scene, a 48×64 cloth (3072 vertices: the explicit-inverse limit) and a small
    cloth in one batch; then 3073 vertices, which leaves the explicit inverse for the correction
    kernel."""
    small = W._base(grid_nx=9, grid_ny=7, grid_spacing=0.05, max_iterations=8, shear_stiffness=800.0)
    big = W._base(grid_nx=48, grid_ny=64, grid_spacing=1 / 63, max_iterations=8)
    scenes = [lone_vertex(pdg), pdg.make_grid(big), pdg.make_grid(small)]
    cfgs = [small, big, small]
    sim = pdg.Simulator(scenes, [with_precision(c, p) for c in cfgs])
    sim.step(6)
    for i, (s, c) in enumerate(zip(scenes, cfgs)):
        orc = oracle_twin(s, c, perm=sim.factor(i)["perm"])
        orc.step(6)
        assert max_rel(sim.state(i)[0], orc.state()[0]) <= max(TOL[p], 1e-15), i
    if p == 4:
        # a one-vertex member leaves no room for a team of CTAs per cloth: the correction kernel
        assert sim.info()["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL32_CORRECTION
        alone = pdg.Simulator(scenes[1], with_precision(big, p))
        assert alone.info()["solve_kind"] == pdg.PD_SOLVE_DENSE32_TEAM
        alone.step(6)
        orc = oracle_twin(scenes[1], big, perm=alone.factor()["perm"])
        orc.step(6)
        assert max_rel(alone.state()[0], orc.state()[0]) < 1e-5
        over = pdg.GridScene(*[getattr(scenes[1], f) for f in ("positions", "masses", "pinned", "edges", "edge_rest",
                                                                 "edge_stiffness")])
        over.positions = np.vstack([over.positions, [[0.5, 0.3, 0.5]]])
        over.masses = np.append(over.masses, over.masses[0])
        over.pinned = np.append(over.pinned, 0).astype(np.uint8)
        one = pdg.Simulator(over, with_precision(big, p))
        assert one.info()["solve_kind"] == pdg.PD_SOLVE_SUPERNODAL32_CORRECTION
        one.step(6)
        orc = oracle_twin(over, big, perm=one.factor()["perm"])
        orc.step(6)
        assert max_rel(one.state()[0], orc.state()[0]) < 1e-5
