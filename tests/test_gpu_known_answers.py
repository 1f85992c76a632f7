"""The reference's known-answer scenes stepped on the GPU: the pinned chain of
_verify/chain_test.cpp (a line graph, so an elimination tree unlike a cloth's) and the translated
springs and cloth of _verify/translation_invariance.cpp (pins away from the origin, where a missing
κ·q term would show), and the pin-mask change of tests/chain/spring_vertical.cpp that must
reanalyze. Each against the oracle on the same scene, plus the scene's own answer.
"""
import numpy as np
import pytest

from tests.helpers import bits, max_rel, oracle_twin

pytestmark = pytest.mark.gpu

TOL = {1: 1e-10, 4: 1e-5}


def chain_scene(pdg, n, k):
    ell = 0.05
    pos = np.zeros((n, 3))
    pos[:, 1] = np.arange(n) * ell
    pinned = np.zeros(n, np.uint8)
    pinned[0] = 1
    edges = np.stack([np.arange(n - 1), np.arange(1, n)], axis=1).astype(np.int32)
    return pdg.GridScene(positions=pos, masses=np.full(n, 0.005), pinned=pinned, edges=edges,
                         edge_rest=np.full(n - 1, ell), edge_stiffness=np.full(n - 1, k),
                         velocities=np.zeros((n, 3)), pin_positions=pos.copy())


def chain_length(x, edges):
    return float(np.sum(np.linalg.norm(x[edges[:, 0]] - x[edges[:, 1]], axis=1)))


@pytest.mark.parametrize("p", [0, 1, 4])
def test_pinned_chain(pdg, p):
    """A 100-vertex chain standing on its pin: reference order bit for bit over 200 substeps; the
    other modes over 8000 damped substeps within their bar, FP64 also at the analytic length change
    m·g·n(n − 1)/(2κ) to 1e-6."""
    n, k = 100, 1.0e4
    scene = chain_scene(pdg, n, k)
    cfg = pdg.SceneConfig(dt=1.0 / 120.0, velocity_damping=0.5, max_iterations=40, rel_tolerance=0.0,
                          abs_tolerance=1e-16, precision=p)
    sim = pdg.Simulator(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    steps = 200 if p == 0 else 8000
    sim.step(steps)
    orc.step(steps)
    x = sim.state()[0]
    if p == 0:
        assert np.array_equal(bits(x), bits(orc.state()[0]))
        return
    assert max_rel(x, orc.state()[0]) <= TOL[p]
    if p == 1:
        change = 0.005 * 9.81 * n * (n - 1) / (2.0 * k)
        assert abs(((n - 1) * 0.05 - chain_length(x, scene.edges)) - change) <= 1e-6 * change


@pytest.mark.parametrize("p", [0, 1])
@pytest.mark.parametrize("pin", [(0, 0, 0), (3, -2, 7)])
def test_spring_at_rest_length_without_gravity_stays_put(pdg, p, pin):
    pos = np.array([pin, np.asarray(pin, np.float64) + [0.0, 0.0, 0.1]], np.float64)
    scene = pdg.GridScene(positions=pos, masses=np.array([0.05, 0.05]), pinned=np.array([1, 0], np.uint8),
                          edges=np.array([[0, 1]], np.int32), edge_rest=np.array([0.1]),
                          edge_stiffness=np.array([1.0e4]), velocities=np.zeros((2, 3)), pin_positions=pos.copy())
    cfg = pdg.SceneConfig(dt=1.0 / 120.0, gravity=(0.0, 0.0, 0.0), velocity_damping=0.0, max_iterations=40,
                          rel_tolerance=0.0, abs_tolerance=1e-18, precision=p)
    sim = pdg.Simulator(scene, cfg)
    sim.step(50)
    assert np.linalg.norm(sim.state()[0][1] - pos[1]) < 1e-12


@pytest.mark.parametrize("p", [0, 1, 4])
def test_translated_cloth(pdg, p):
    """An 8×8 cloth shifted by (5, 7, −3), 300 substeps: against the oracle on the shifted scene
    (bit for bit in reference order), and in the FP64 modes every edge length as unshifted to 1e-6."""
    lengths = []
    for shift in ((0.0, 0.0, 0.0), (5.0, 7.0, -3.0)):
        cfg = pdg.SceneConfig(grid_nx=8, grid_ny=8, grid_spacing=0.05, stiffness=1.0e4, dt=1.0 / 120.0,
                              max_iterations=20, rel_tolerance=1e-8, precision=p)
        scene = pdg.make_grid(cfg)
        scene.positions = np.asarray(scene.positions, np.float64) + np.asarray(shift)
        scene.pin_positions = scene.positions.copy()
        sim = pdg.Simulator(scene, cfg)
        orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
        sim.step(300)
        orc.step(300)
        x = sim.state()[0]
        if p == 0:
            assert np.array_equal(bits(x), bits(orc.state()[0]))
        else:
            assert max_rel(x, orc.state()[0]) <= TOL[p]
        e = np.asarray(scene.edges, np.int32).reshape(-1, 2)
        lengths.append(np.linalg.norm(x[e[:, 0]] - x[e[:, 1]], axis=1))
    if p != 4:
        assert np.max(np.abs(lengths[0] - lengths[1]) / np.maximum(lengths[0], 1e-12)) < 1e-6


@pytest.mark.parametrize("p", [0, 1, 4])
def test_pin_mask_change_reanalyzes(pdg, p):
    """Pinning an interior vertex of a 6×6 cloth mid-run removes its coupling blocks, so Ã's pattern
    changes: one new analysis and factorization, none after (spring_vertical.cpp:528-560). The
    stepping after the change matches an oracle started from the state at the change with the new
    pin mask (the substep depends on x and v alone), bit for bit in reference order."""
    cfg = pdg.SceneConfig(grid_nx=6, grid_ny=6, grid_spacing=0.05, stiffness=1.0e4, max_iterations=4,
                          rel_tolerance=0.0, abs_tolerance=0.0, precision=p)
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(6)
    orc.step(6)
    assert sim.info()["analyze_count"] == 1
    v = 2 * 6 + 2
    pinned = np.asarray(scene.pinned, np.uint8).copy()
    assert pinned[v] == 0
    pinned[v] = 1
    sim.set_pinned(pinned)  # the new pin holds its current position
    info = sim.info()
    assert info["analyze_count"] == 2 and info["factorize_count"] == 2
    x, vel = orc.state()
    q = np.asarray(scene.positions, np.float64).copy()
    q[v] = x[v]
    after = pdg.GridScene(positions=x, masses=scene.masses, pinned=pinned, edges=scene.edges,
                          edge_rest=scene.edge_rest, edge_stiffness=scene.edge_stiffness, velocities=vel,
                          pin_positions=q)
    orc2 = oracle_twin(after, cfg, perm=sim.factor()["perm"])
    sim.step(6)
    orc2.step(6)
    info = sim.info()
    assert info["analyze_count"] == 2 and info["factorize_count"] == 2
    got = sim.state()[0]
    assert np.all(np.isfinite(got))
    if p == 0:
        assert np.array_equal(bits(got), bits(orc2.state()[0]))
    else:
        assert max_rel(got, orc2.state()[0]) <= TOL[p]
