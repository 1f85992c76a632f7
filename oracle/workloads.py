"""The benchmark workloads built by the oracle alone (TEST INFRASTRUCTURE ONLY).

The CPU arms of ``bench.py`` (the timed reference arm and ``cpu_baseline``) build their cloths
here, through the oracle's own restatement of the reference's grid construction
(``oracle_make_grid``: core/mesh/Mesh.cpp:12-54,183-285, core/sim/Scene.cpp:39-177), so that no
process that times the reference algorithm loads the product library. The seeded parameter draws
are the product's workload definitions restated: the same splitmix64 stream, the same draws in
the same order. ``tests/test_workloads.py`` checks that every workload built here equals, array
for array and bit for bit, the one the product builds.

Each builder returns ``(meshes, configs, substeps)`` with ``configs`` of type ``oracle.Config``.
"""
from __future__ import annotations

import math

import numpy as np

from . import oracle as O

MASK64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 (Steele, Lea & Flood 2014), integer only: the same stream on every machine."""

    def __init__(self, seed: int):
        self.state = seed & MASK64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))

    def randint(self, lo: int, hi: int) -> int:
        return lo + (self.next_u64() % (hi - lo + 1))


def _config(iterations, residual_tolerance=1e-3, rel_tolerance=1e-3, abs_tolerance=1e-12, threads=0):
    return O.Config(dt=1.0 / 300.0, gravity=(0.0, -9.81, 0.0), velocity_damping=0.0,
                    max_iterations=iterations, rel_tolerance=rel_tolerance, abs_tolerance=abs_tolerance,
                    residual_tolerance=residual_tolerance, threads=threads)


def _grid(nx, ny, spacing, k, ks=0.0, kb=0.0, total_mass=1.0, pin_mode=1):
    return O.make_grid(O.GridSpec(nx=nx, ny=ny, spacing=spacing, stiffness=k, shear_stiffness=ks,
                                  bend_stiffness=kb, mass_mode=1, total_mass=total_mass, pin_mode=pin_mode))


def cloth40_plain(threads=0):
    return [_grid(40, 40, 1.0 / 39.0, 2300.0)], [_config(10, threads=threads)], 600


def cloth40_full(threads=0):
    return [_grid(40, 40, 1.0 / 39.0, 2300.0, 1000.0, 50.0)], [_config(40, threads=threads)], 600


def cloth256(seed: int = 256, threads=0):
    mesh = _grid(256, 256, 2.0 / 255.0, 2300.0, 1000.0, 50.0, total_mass=4.0)
    rng = SplitMix64(seed)
    jitter = np.array([(2.0 * rng.uniform() - 1.0) * 1e-4 for _ in range(mesh.n)])
    mesh.positions = mesh.positions.copy()
    mesh.positions[:, 1] += jitter
    return [mesh], [_config(20, threads=threads)], 300


def batch(count: int = 512, seed: int = 512, max_side: int = 128, threads=0):
    rng = SplitMix64(seed)
    meshes, cfgs = [], []
    for _ in range(count):
        nx = rng.randint(16, max_side)
        ny = rng.randint(16, max_side)
        kappa = math.exp(math.log(500.0) + rng.uniform() * (math.log(20000.0) - math.log(500.0)))
        shear = rng.uniform() < 0.5
        bend = rng.uniform() < 0.25
        pin_mode = (0, 2, 3)[rng.randint(0, 2)]
        meshes.append(_grid(nx, ny, 1.0 / (max(nx, ny) - 1), kappa, 0.4 * kappa if shear else 0.0,
                            0.02 * kappa if bend else 0.0, pin_mode=pin_mode))
        cfgs.append(_config(10, threads=threads))
    return meshes, cfgs, 300


def _normal(rng: SplitMix64) -> float:
    u1 = max(rng.uniform(), 1e-300)
    u2 = rng.uniform()
    return math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)


def differentiable(side: int = 64, substeps: int = 120, seed: int = 5, threads=0):
    """(mesh, config, substeps, hidden per-edge stiffness κ*) of the gradient workload."""
    mesh = _grid(side, side, 1.0 / (side - 1), 2300.0, 2300.0)
    rng = SplitMix64(seed)
    kstar = np.array([2300.0 * math.exp(0.3 * _normal(rng)) for _ in range(mesh.edges.shape[0])])
    cfg = _config(10, residual_tolerance=0.0, rel_tolerance=0.0, abs_tolerance=0.0, threads=threads)
    return mesh, cfg, substeps, kstar


WORKLOADS = {"cloth40_plain": cloth40_plain, "cloth40_full": cloth40_full, "cloth256": cloth256}


def build(name: str, batch_count: int = 512, threads=0):
    """(meshes, configs, substeps) of a named workload."""
    if name == "batch":
        return batch(count=batch_count, threads=threads)
    return WORKLOADS[name](threads=threads)
