"""Host logic of the product against the oracle, and the C ABI's exported surface (no GPU work)."""
import ctypes
import os
import re

import numpy as np
import pytest

from pd_gb300 import workloads as W
from pd_gb300.api import scene_coloring, scene_factor
from tests.helpers import bits, oracle_twin

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "pd_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(pd_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol(pdg):
    lib = ctypes.CDLL(pdg.api.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


GRIDS = [
    dict(grid_nx=40, grid_ny=40, grid_spacing=0.025, stiffness=1e4),
    dict(grid_nx=40, grid_ny=40, grid_spacing=1 / 39, stiffness=2300, shear_stiffness=1000, bend_stiffness=50,
         mass_mode=1, total_mass=1.0, pin_mode=1, dt=1 / 300),
    dict(grid_nx=13, grid_ny=29, grid_spacing=0.04, stiffness=777.0, shear_stiffness=311.0, bend_stiffness=9.0,
         bend_sampling=3, pin_mode=2),
    dict(grid_nx=21, grid_ny=7, grid_spacing=0.05, bend_stiffness=5.0, bend_sampling=1, bend_stride=2, pin_mode=3),
]


def oracle_spec(oracle, c):
    return oracle.GridSpec(nx=c.grid_nx, ny=c.grid_ny, spacing=c.grid_spacing, stiffness=c.stiffness,
                           density=c.density, shear_stiffness=c.shear_stiffness, bend_stiffness=c.bend_stiffness,
                           bend_sampling=c.bend_sampling, bend_stride=c.bend_stride, mass_mode=c.mass_mode,
                           total_mass=c.total_mass, pin_mode=c.pin_mode)


@pytest.mark.parametrize("kw", GRIDS)
def test_grid_colouring_and_factor_match_oracle_bitwise(pdg, oracle, kw):
    cfg = pdg.SceneConfig(**kw)
    scene = pdg.make_grid(cfg)
    om = oracle.make_grid(oracle_spec(oracle, cfg))
    pairs = [("positions", "positions"), ("masses", "masses"), ("pinned", "pinned"), ("edges", "edges"),
             ("edge_rest", "edge_rest"), ("edge_stiffness", "edge_k"), ("bends", "bends"),
             ("bend_stiffness", "bend_k")]
    for a, b in pairs:
        x, y = getattr(scene, a), getattr(om, b)
        assert x.shape == y.shape and np.array_equal(x, y), a
    f, info = scene_factor(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=f["perm"])
    of = orc.factor()
    for k in ("perm", "colptr", "rowidx"):
        assert np.array_equal(of[k], f[k]), k
    assert np.array_equal(bits(of["val"]), bits(f["val"])) and np.array_equal(bits(of["dinv"]), bits(f["dinv"]))
    col, cc = scene_coloring(scene)
    oc = orc.coloring()
    assert cc == oc["count"] == info["color_count"] and np.array_equal(col, oc["color_of"])
    assert info["factorize_count"] == 1 and info["forward_levels"] > 0


def test_ordering_is_a_valid_permutation_for_batch_scenes(pdg):
    scenes, cfgs, _ = W.batch(count=6, seed=3, max_side=40)
    for s, c in zip(scenes, cfgs):
        f, info = scene_factor(s, c)
        assert sorted(f["perm"].tolist()) == list(range(s.n))
        assert info["factor_nnz"] == f["colptr"][-1]


def test_host_rejects_invalid_scenes(pdg):
    cfg = pdg.SceneConfig(grid_nx=6, grid_ny=6)
    base = pdg.make_grid(cfg)
    bad = pdg.make_grid(cfg)
    bad.edges = bad.edges.copy()
    bad.edges[3] = [2, 2]
    with pytest.raises(pdg.PdError) as e:
        scene_factor(bad, cfg)
    assert e.value.code == 1 and "itself" in str(e.value)
    bad = pdg.make_grid(cfg)
    bad.bends = np.array([[0, 1, 99]], np.int32)
    bad.bend_stiffness = np.array([1.0])
    with pytest.raises(pdg.PdError):
        scene_factor(bad, cfg)
    with pytest.raises(pdg.PdError):
        scene_factor(base, pdg.SceneConfig(dt=0.0))
    with pytest.raises(pdg.PdError) as e:
        scene_factor(base, pdg.SceneConfig(precision=7))
    assert e.value.code == 5
    free = pdg.make_grid(pdg.SceneConfig(grid_nx=3, grid_ny=3, pin_mode=4))
    free.masses = np.zeros_like(free.masses)  # no inertia and no pins: L is singular
    free.edge_stiffness = np.zeros_like(free.edge_stiffness)
    with pytest.raises(pdg.PdError) as e:
        scene_factor(free, pdg.SceneConfig())
    assert e.value.code == 3


def test_workloads_are_deterministic(pdg):
    a, _, _ = W.batch(count=4, seed=9, max_side=30)
    b, _, _ = W.batch(count=4, seed=9, max_side=30)
    for x, y in zip(a, b):
        assert np.array_equal(x.positions, y.positions) and np.array_equal(x.edge_stiffness, y.edge_stiffness)
    s, cfg, sub = W.cloth40_full()
    assert s[0].edges.shape[0] == 4641 and s[0].bends.shape[0] == 3040 and sub == 600
    assert abs(s[0].masses.sum() - 1.0) < 1e-12


def test_config_defaults_match_the_c_abi(pdg):
    """pd_scene_config_default and the Python SceneConfig agree field by field (incl. the
    over-relaxation knobs: off, ρ 0.98, 10 plain iterations, interval centre 1 and half-width 1)."""
    lib = ctypes.CDLL(pdg.api.LIB_PATH)
    c = pdg.api._Cfg()
    lib.pd_scene_config_default(ctypes.byref(c))
    d = pdg.SceneConfig()
    for name, _ in pdg.api._Cfg._fields_:
        got = tuple(c.gravity) if name == "gravity" else getattr(c, name)
        assert got == getattr(d, name), name
    base = pdg.make_grid(pdg.SceneConfig(grid_nx=6, grid_ny=6))
    with pytest.raises(pdg.PdError) as e:
        scene_factor(base, pdg.SceneConfig(cheb_mode=3))
    assert e.value.code == 1


@pytest.mark.parametrize("seed,curved", [(0, True), (1, False), (2, True)])
def test_obj_mesh_matches_oracle_bitwise(pdg, oracle, seed, curved):
    """pd_make_obj against the oracle's restated Mesh::loadObj: vertices, unique edges in
    first-seen order, rest lengths and surface masses bit for bit, then colouring and factor."""
    from tests.helpers import obj_sheet
    text = obj_sheet(11, 8, seed=seed, curved=curved)
    cfg = pdg.SceneConfig(stiffness=777.0, density=1.7)
    scene = pdg.make_obj(text, cfg)
    om = oracle.make_obj(text, stiffness=777.0, density=1.7)
    for a, b in [("positions", "positions"), ("masses", "masses"), ("edges", "edges"), ("edge_rest", "edge_rest"),
                 ("edge_stiffness", "edge_k")]:
        x, y = getattr(scene, a), getattr(om, b)
        assert x.shape == y.shape and np.array_equal(bits(x) if x.dtype == np.float64 else x,
                                                     bits(y) if y.dtype == np.float64 else y), a
    assert not np.any(scene.pinned) and scene.bends.shape[0] == 0
    scene.pinned[[0, 5]] = 1
    f, info = scene_factor(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=f["perm"])
    of = orc.factor()
    assert np.array_equal(of["colptr"], f["colptr"]) and np.array_equal(bits(of["val"]), bits(f["val"]))
    with pytest.raises(pdg.PdError):
        pdg.make_obj("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 9\n", cfg)
