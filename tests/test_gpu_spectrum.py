"""Spectrum of the linearised PD iteration on the GPU (pd_sim_spectrum; the reference's
_verify/iteration_spectrum.cpp) against the oracle's power iteration from the same state, the
closed form of a spring, and the reference's own consistency criterion: the contraction the real
iteration shows (residuals after 8 and 16 iterations from one state) is at most 1.15 × ρ(T).
"""
import copy

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import bits, oracle_twin

pytestmark = pytest.mark.gpu


def cfg_with(cfg, precision, **kw):
    c = copy.copy(cfg)
    c.precision = precision
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def rel(a, b):
    return abs(a - b) / abs(b)


@pytest.mark.parametrize("p", [0, 1, 4])
def test_spectrum_matches_oracle(pdg, p):
    cfg = cfg_with(W._base(grid_nx=20, grid_ny=18, grid_spacing=1 / 19, max_iterations=20, shear_stiffness=1000.0,
                           bend_stiffness=50.0), p)
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(30)
    orc.step(30)
    before = sim.state()
    g = sim.spectrum(0, 400)
    o = orc.spectrum(400)
    tol = 1e-9 if p == 0 else 1e-5  # MIXED positions differ from the oracle's by ~1e-7
    for k in ("rho_plain", "rho_plain_prev", "lambda_max", "lambda_max_prev"):
        assert rel(g[k], o[k]) <= tol, (k, g[k], o[k])
    assert g["lambda_min"] == 1.0 - g["rho_plain"] and 0.0 < g["rho_cheb"] < g["rho_plain"] < 1.0
    after = sim.state()
    assert np.array_equal(bits(before[0]), bits(after[0])) and np.array_equal(bits(before[1]), bits(after[1]))


def test_spectrum_spring_closed_form(pdg):
    m, h, k = 0.05, 1.0 / 120.0, 1.0e4
    scene = pdg.GridScene(np.array([[0.0, 0.0, 0.0], [0.0, 0.12, 0.0]]), np.array([m, m]), np.array([1, 0], np.uint8),
                          np.array([[0, 1]], np.int32), np.array([0.1]), np.array([k]))
    cfg = cfg_with(W._base(dt=h, max_iterations=10), 1)
    sim = pdg.Simulator(scene, cfg)
    g = sim.spectrum(0, 60)
    mh2 = m / (h * h)
    assert rel(g["rho_plain"], k / (mh2 + k)) <= 1e-13
    assert abs(g["lambda_max"] - 1.0) <= 1e-13


def test_measured_contraction_within_prediction(pdg):
    """iteration_spectrum.cpp:340-362: from one quasi-static state, (r16 / r8)^(1/8) of the real
    iteration against ρ(T) — at most 1.15 × the prediction."""
    cfg = cfg_with(W._base(grid_nx=24, grid_ny=24, grid_spacing=1 / 23, max_iterations=40), 1)
    scene = pdg.make_grid(cfg)
    sim = pdg.Simulator(scene, cfg)
    sim.step(300)
    rho = sim.spectrum(0, 400)["rho_plain"]
    sim.set_config(cfg_with(cfg, 1, max_iterations=16, residual_tolerance=1e-30))
    sim.set_residual_trace(True)
    sim.step(1)
    r = sim.residual_trace(0)[0]
    measured = (r[15] / r[7]) ** (1.0 / 8.0)
    assert 0.0 < measured <= 1.15 * rho, (measured, rho)


def test_spectrum_argument_errors(pdg):
    cfg = cfg_with(W._base(grid_nx=6, grid_ny=5, grid_spacing=0.05, max_iterations=3), 1)
    sim = pdg.Simulator(pdg.make_grid(cfg), cfg)
    for bad in (0, -3):
        with pytest.raises(pdg.PdError):
            sim.spectrum(0, bad)
    with pytest.raises(pdg.PdError):
        sim.spectrum(1, 10)
