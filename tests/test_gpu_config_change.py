"""SceneConfig edits on a live handle (pd_sim_set_config): a precision, CTA-count or explicit-inverse
limit change re-plans and lays the handle out again, so the handle then steps exactly like one
created with the new configuration from the state at the change (bit for bit: both run the same
deterministic kernels on the same factor), and the pinned vertices stay put."""
import copy

import numpy as np
import pytest

from tests.helpers import bits, max_rel, oracle_twin

pytestmark = pytest.mark.gpu


def _scene(pdg, nx=24, ny=20):
    cfg = pdg.SceneConfig(grid_nx=nx, grid_ny=ny, grid_spacing=1.0 / (nx - 1), stiffness=2300.0,
                          shear_stiffness=1000.0, bend_stiffness=50.0, dt=1.0 / 300.0, velocity_damping=0.0,
                          max_iterations=12, mass_mode=1, pin_mode=1)
    return pdg.make_grid(cfg), cfg


def _fresh_like(pdg, scene, cfg, x, v):
    sim = pdg.Simulator(scene, cfg)
    sim.set_state(0, x, v)
    return sim


# precision sequence, each with (cluster_ctas, dense_max_vertices)
SEQUENCE = [
    (0, 0, 0),    # FP64_EXACT
    (4, 0, 0),    # MIXED: the team kernel
    (1, 0, 0),    # FP64 supernodal, planner's cluster
    (4, 1, 0),    # MIXED on one CTA: correction form
    (1, 4, 0),    # FP64 on a 4-CTA cluster
    (3, 0, 0),    # FP32 solve + refinement
    (2, 0, 0),    # FP32 projection
    (0, 0, 0),    # back to FP64_EXACT
]


def test_precision_and_plan_changes_step_like_a_fresh_handle(pdg):
    scene, cfg = _scene(pdg)
    c0 = copy.copy(cfg)
    c0.precision = SEQUENCE[0][0]
    live = pdg.Simulator(scene, c0)
    live.step(4)
    kinds = []
    for prec, ctas, dense in SEQUENCE[1:]:
        x, v = live.state()
        c = copy.copy(cfg)
        c.precision, c.cluster_ctas, c.dense_max_vertices = prec, ctas, dense
        live.set_config(c)
        ref = _fresh_like(pdg, scene, c, x, v)
        assert live.info()["solve_kind"] == ref.info()["solve_kind"]
        assert live.info()["cluster_ctas"] == ref.info()["cluster_ctas"]
        kinds.append(live.info()["solve_kind"])
        live.step(6)
        ref.step(6)
        xl, vl = live.state()
        xr, vr = ref.state()
        assert np.array_equal(bits(xl), bits(xr)), (prec, ctas, float(np.max(np.abs(xl - xr))))
        assert np.array_equal(bits(vl), bits(vr)), (prec, ctas)
        pins = np.flatnonzero(scene.pinned)
        assert np.array_equal(xl[pins], scene.positions[pins])
    # the sequence really visited different kernel families
    assert len(set(kinds)) >= 4, kinds


def test_switched_handle_tracks_the_oracle(pdg):
    """After EXACT → MIXED → FP64 switches mid-run, the trajectory stays within each mode's bar of
    the FP64 oracle that never switched (MIXED's 1e-5 dominates)."""
    scene, cfg = _scene(pdg)
    c = copy.copy(cfg)
    c.precision = 0
    live = pdg.Simulator(scene, c)
    orc = oracle_twin(scene, c, perm=live.factor()["perm"])
    for prec in (0, 4, 1):
        c = copy.copy(cfg)
        c.precision = prec
        live.set_config(c)
        live.step(20)
        orc.step(20)
    assert max_rel(live.state()[0], orc.state()[0]) < 1e-5
