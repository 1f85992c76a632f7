"""Over-relaxed iterates — the reference's PD_CHEB modes (core/sim/Integrator.cpp:476-645) — on
the GPU against the oracle: bit-identical in the reference-order FP64 mode (positions, velocities,
iteration counts), within 1e-10 in the FP64 supernodal mode, within 1e-5 in the FP32 modes; and
the reference's printed 60×60 Chebyshev residual reproduced through the GPU.
"""
import copy

import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import bits, max_rel, oracle_twin

pytestmark = pytest.mark.gpu

BLENDS = {
    "rho": dict(cheb_mode=1),  # ρ = 0.98 after 10 plain iterations (the reference's defaults)
    "rho-early": dict(cheb_mode=1, cheb_start=2, cheb_rho=0.9),
    "interval": dict(cheb_mode=2, cheb_m=1.0, cheb_d=0.5),
}
GATES = {  # small cloths: the residual gate fires in some substeps; the displacement gate; none met
    "residual": dict(grid_nx=12, grid_ny=12, grid_spacing=0.05, max_iterations=30, residual_tolerance=0.3),
    "displacement": dict(grid_nx=10, grid_ny=14, grid_spacing=0.05, max_iterations=25, residual_tolerance=0.0,
                         rel_tolerance=5e-2),
    "budget": dict(grid_nx=14, grid_ny=10, grid_spacing=0.05, max_iterations=16, residual_tolerance=1e-3,
                   shear_stiffness=800.0, bend_stiffness=20.0),
}


def scene_cfg(pdg, gate, blend, precision, ctas=0, dense=0):
    cfg = W._base(velocity_damping=0.02, **GATES[gate])
    for k, v in BLENDS[blend].items():
        setattr(cfg, k, v)
    scene = pdg.make_grid(cfg)
    c = copy.copy(cfg)
    c.precision = precision
    c.cluster_ctas = ctas
    c.dense_max_vertices = dense
    return scene, cfg, c


@pytest.mark.parametrize("blend", list(BLENDS))
@pytest.mark.parametrize("gate", list(GATES))
def test_reference_order_bit_identical(pdg, gate, blend):
    scene, cfg, c = scene_cfg(pdg, gate, blend, pdg.PD_PRECISION_FP64_EXACT)
    sim = pdg.Simulator(scene, c)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    for _ in range(2):
        sim.step(20)
        it_o, cv_o = orc.step(20)
        it_g, cv_g = sim.iteration_log()
        assert np.array_equal(it_g, it_o) and np.array_equal(cv_g, cv_o)
    xg, vg = sim.state()
    xo, vo = orc.state()
    assert np.array_equal(bits(xg), bits(xo)) and np.array_equal(bits(vg), bits(vo))
    assert sim.stats()["last_residual"] == orc.stats()["last_residual"]


def test_reference_order_full_cloth_bit_identical(pdg):
    scenes, cfg, _ = W.cloth40_full()
    cfg.cheb_mode = 1
    sim = pdg.Simulator(scenes[0], cfg)
    orc = oracle_twin(scenes[0], cfg, perm=sim.factor()["perm"])
    sim.step(12)
    it_o, _ = orc.step(12)
    assert np.array_equal(sim.iteration_log()[0], it_o)
    assert np.array_equal(bits(sim.state()[0]), bits(orc.state()[0]))


@pytest.mark.parametrize("blend", list(BLENDS))
@pytest.mark.parametrize("ctas", [1, 16])
def test_fp64_within_tolerance(pdg, blend, ctas):
    scenes, cfg, _ = W.cloth40_full()
    for k, v in BLENDS[blend].items():
        setattr(cfg, k, v)
    c = copy.copy(cfg)
    c.precision = pdg.PD_PRECISION_FP64
    c.cluster_ctas = ctas
    sim = pdg.Simulator(scenes[0], c)
    orc = oracle_twin(scenes[0], cfg, perm=sim.factor()["perm"])
    sim.step(120)
    it_o, _ = orc.step(120)
    assert np.array_equal(sim.iteration_log()[0], it_o)
    assert max_rel(sim.state()[0], orc.state()[0]) < 1e-10


def test_reference_printed_chebyshev_residual(pdg):
    """docs/chebyshev.md:280-287: pd_bench --grid 60 60 --steps 300 with PD_CHEB=1 at 20 and 80
    iterations prints last residuals 9.37677 and 3.51819 (plain PD: 12.3328, 6.14024)."""
    for iters, want in ((20, 9.37677), (80, 3.51819)):
        cfg = pdg.SceneConfig(grid_nx=60, grid_ny=60, stiffness=1e4, max_iterations=iters, cheb_mode=1,
                              precision=pdg.PD_PRECISION_FP64)
        sim = pdg.Simulator(pdg.make_grid(cfg), cfg)
        sim.step(300)
        st = sim.stats()
        assert st["early_exit_count"] == 0
        assert float(f"{st['last_residual']:.6g}") == want


# FP32 kernels: (precision, CTAs per cloth, dense limit) → the kernel the planner picks
FP32_KERNELS = {
    "mixed-team": (4, 0, 0),             # substepDeltaKernel
    "mixed-correction": (4, 1, 0),       # substepCorrKernel
    "mixed-correction-cluster": (4, 16, -1),  # substepCorrClusterKernel
    "fp32-solve": (3, 1, 0),             # substepMixedKernel
    "fp32-solve-dense": (3, 16, 0),      # substepDenseClusterKernel
}


@pytest.mark.parametrize("blend", ["rho-early", "interval"])
@pytest.mark.parametrize("gate", list(GATES))
@pytest.mark.parametrize("kernel", list(FP32_KERNELS))
def test_fp32_kernels_within_tolerance(pdg, kernel, gate, blend):
    prec, ctas, dense = FP32_KERNELS[kernel]
    scene, cfg, c = scene_cfg(pdg, gate, blend, prec, ctas, dense)
    sim = pdg.Simulator(scene, c)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(60)
    it_o, cv_o = orc.step(60)
    it_g, cv_g = sim.iteration_log()
    assert max_rel(sim.state()[0], orc.state()[0]) < 1e-5
    assert np.mean(it_g == it_o) > 0.95 and np.mean(cv_g == cv_o) > 0.95


def test_mixed_team_full_cloth_600_substeps(pdg):
    scenes, cfg, substeps = W.cloth40_full()
    cfg.cheb_mode = 1
    c = copy.copy(cfg)
    c.precision = pdg.PD_PRECISION_MIXED
    sim = pdg.Simulator(scenes[0], c)
    assert sim.info()["solve_kind"] == pdg.PD_SOLVE_DENSE32_TEAM
    orc = oracle_twin(scenes[0], cfg, perm=sim.factor()["perm"])
    sim.step(substeps)
    it_o, _ = orc.step(substeps)
    assert max_rel(sim.state()[0], orc.state()[0]) < 1e-5
    assert np.mean(sim.iteration_log()[0] == it_o) > 0.99


def test_gradient_refuses_over_relaxation(pdg):
    scene, cfg, _, _ = W.differentiable(side=8, substeps=2)
    cfg.cheb_mode = 1
    sim = pdg.Simulator(scene, cfg)
    with pytest.raises(pdg.PdError):
        sim.gradient(2, scene.positions)
