"""Synthetic cloth workloads (seeded, deterministic on every platform).

Each builder returns ``(scenes, config, substeps)``: regular grids in the xz-plane built by the
library's ``pd_make_grid`` (the reference ``makeScene``), with the parameters below.

* ``cloth40_plain``  40×40, 1 m², spacing 1/39, uniform mass 1 kg, corners of row 0 pinned,
                     κ = 2300 on the 3120 structural edges, h = 1/300, 10 iterations,
                     residual gate 1e-3·|g|, no damping, 600 substeps.
* ``cloth40_full``   the same cloth plus 1521 shear diagonals (κs = 1000) and 3040 midpoint bend
                     stencils (κb = 50), 40 iterations, residual gate 1e-3·|g|, 600 substeps.
* ``cloth256``       256×256, 2 m × 2 m, corners of row 0 pinned, κ 2300 / 1000 / 50,
                     uniform mass 4 kg (1 kg/m²), initial y jitter U(±1e-4) m from a seed,
                     rest lengths from the unjittered grid, h = 1/300, 20 iterations, 300 substeps.
* ``batch``          N independent cloths: nx, ny uniform integers in [16, 128], spacing
                     1/(max(nx, ny) − 1) m, uniform mass 1 kg, κ log-uniform in [500, 20000],
                     shear on for half (κs = 0.4κ), bend for a quarter (κb = 0.02κ), pins drawn from
                     {two corners of the top row, the whole top row, one top corner}, h = 1/300,
                     10 iterations, 300 substeps.
* ``differentiable`` 64×64, 1 m², corners of row 0 pinned, distance + shear edges, uniform mass
                     1 kg, h = 1/300, 10 iterations with the gate off, no damping, 120 substeps.
                     Returns the scene (every edge at κ = 2300), the config, the substep count and
                     the hidden per-edge stiffness κ*_e = 2300·exp(N(0, 0.3²)) from a seed; the loss
                     targets are the final positions of a run with κ*.
Random draws use splitmix64 on integers, so every machine produces the same scenes.
"""
from __future__ import annotations

import math

import numpy as np

from .api import SceneConfig, make_grid

MASK64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 generator (Steele, Lea & Flood 2014): integer-only, platform independent."""

    def __init__(self, seed: int):
        self.state = seed & MASK64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self) -> float:
        """Uniform in [0, 1) with 53 random bits."""
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))

    def randint(self, lo: int, hi: int) -> int:
        """Uniform integer in [lo, hi]."""
        return lo + (self.next_u64() % (hi - lo + 1))


def _base(**kw) -> SceneConfig:
    c = SceneConfig(dt=1.0 / 300.0, velocity_damping=0.0, stiffness=2300.0, residual_tolerance=1e-3,
                    mass_mode=1, total_mass=1.0, pin_mode=1)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def cloth40_plain():
    cfg = _base(grid_nx=40, grid_ny=40, grid_spacing=1.0 / 39.0, max_iterations=10)
    return [make_grid(cfg)], cfg, 600


def cloth40_full():
    cfg = _base(grid_nx=40, grid_ny=40, grid_spacing=1.0 / 39.0, max_iterations=40,
                shear_stiffness=1000.0, bend_stiffness=50.0)
    return [make_grid(cfg)], cfg, 600


def cloth256(seed: int = 256):
    cfg = _base(grid_nx=256, grid_ny=256, grid_spacing=2.0 / 255.0, max_iterations=20,
                shear_stiffness=1000.0, bend_stiffness=50.0, total_mass=4.0)
    scene = make_grid(cfg)
    rng = SplitMix64(seed)
    jitter = np.array([(2.0 * rng.uniform() - 1.0) * 1e-4 for _ in range(scene.n)])
    scene.positions = scene.positions.copy()
    scene.positions[:, 1] += jitter
    return [scene], cfg, 300


def batch(count: int = 512, seed: int = 512, max_side: int = 128):
    rng = SplitMix64(seed)
    scenes, cfgs = [], []
    for _ in range(count):
        nx = rng.randint(16, max_side)
        ny = rng.randint(16, max_side)
        kappa = math.exp(math.log(500.0) + rng.uniform() * (math.log(20000.0) - math.log(500.0)))
        shear = rng.uniform() < 0.5
        bend = rng.uniform() < 0.25
        pin_mode = (0, 2, 3)[rng.randint(0, 2)]
        cfg = _base(grid_nx=nx, grid_ny=ny, grid_spacing=1.0 / (max(nx, ny) - 1), max_iterations=10,
                    stiffness=kappa, shear_stiffness=0.4 * kappa if shear else 0.0,
                    bend_stiffness=0.02 * kappa if bend else 0.0, pin_mode=pin_mode)
        scenes.append(make_grid(cfg))
        cfgs.append(cfg)
    return scenes, cfgs, 300


WORKLOADS = {"cloth40_plain": cloth40_plain, "cloth40_full": cloth40_full, "cloth256": cloth256,
             "batch": batch}


def _normal(rng: SplitMix64) -> float:
    """Standard normal by Box–Muller from two splitmix64 uniforms."""
    u1 = max(rng.uniform(), 1e-300)
    u2 = rng.uniform()
    return math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)


def differentiable(side: int = 64, substeps: int = 120, seed: int = 5):
    cfg = _base(grid_nx=side, grid_ny=side, grid_spacing=1.0 / (side - 1), max_iterations=10,
                shear_stiffness=2300.0, residual_tolerance=0.0, rel_tolerance=0.0, abs_tolerance=0.0)
    scene = make_grid(cfg)
    rng = SplitMix64(seed)
    kstar = np.array([2300.0 * math.exp(0.3 * _normal(rng)) for _ in range(scene.edges.shape[0])])
    return scene, cfg, substeps, kstar
