"""The allocation-free solve, pd_solve_noalloc, against the allocating solve pd_sim_solve.

pd_solve_noalloc exists for callers that cannot call cudaMalloc when they solve (an engine that
hands out device memory only from its own pool, a loop where allocation is banned, a plugin host
that owns the device heap): they keep the factor, b and x in their own device memory and the
library supplies a fixed built-in workspace. This test plays such a caller: it places the factor
and the right-hand sides in device memory it owns (torch tensors), calls the entry point through
the C ABI twice in a row with different right-hand sides, and checks each result against
pd_sim_solve on the same scene, bit for bit (both follow the reference's solve order). The file
sorts last so that a stop-at-first-failure run has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from pd_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _dev_ptr(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_solve_matches_allocating_solve_twice(pdg):
    import torch

    lib = pdg.load_library()
    fn = lib.pd_solve_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int32] + [C.c_void_p] * 7 + [C.c_void_p]
    torch.cuda.set_device(0)

    scenes, cfg, _ = W.cloth40_full()
    sim = pdg.Simulator(scenes[0], cfg)
    f = sim.factor()
    n = scenes[0].n
    dev = torch.device("cuda", 0)
    perm = torch.from_numpy(f["perm"]).to(dev)
    colptr = torch.from_numpy(f["colptr"]).to(dev)
    rowidx = torch.from_numpy(f["rowidx"]).to(dev)
    val = torch.from_numpy(f["val"]).to(dev)
    dinv = torch.from_numpy(f["dinv"]).to(dev)
    rng = np.random.default_rng(11)
    for call in range(2):
        b = rng.standard_normal((n, 3)) * (10.0 ** call)
        db = torch.from_numpy(b.reshape(-1).copy()).to(dev)
        dx = torch.full((3 * n,), float("nan"), dtype=torch.float64, device=dev)
        rc = fn(n, _dev_ptr(perm), _dev_ptr(colptr), _dev_ptr(rowidx), _dev_ptr(val), _dev_ptr(dinv),
                _dev_ptr(db), _dev_ptr(dx), None)
        assert rc == 0, lib.pd_last_error().decode()
        torch.cuda.synchronize()
        x_noalloc = dx.cpu().numpy().reshape(n, 3)
        x_ref = sim.solve(b)
        assert np.array_equal(x_noalloc.view(np.uint64), x_ref.view(np.uint64)), call


def _noalloc_solve(pdg, f, b):
    """One pd_solve_noalloc call on the factor `f` (host arrays copied into caller-owned device
    memory) for the right-hand side b (n × 3); returns x on the host."""
    import torch

    lib = pdg.load_library()
    fn = lib.pd_solve_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int32] + [C.c_void_p] * 7 + [C.c_void_p]
    dev = torch.device("cuda", 0)
    arrs = [torch.from_numpy(np.ascontiguousarray(f[k])).to(dev) for k in ("perm", "colptr", "rowidx", "val", "dinv")]
    n = b.shape[0]
    db = torch.from_numpy(b.reshape(-1).copy()).to(dev)
    dx = torch.full((3 * n,), float("nan"), dtype=torch.float64, device=dev)
    rc = fn(n, *[_dev_ptr(a) for a in arrs], _dev_ptr(db), _dev_ptr(dx), None)
    assert rc == 0, lib.pd_last_error().decode()
    torch.cuda.synchronize()
    return dx.cpu().numpy().reshape(n, 3)


def test_noalloc_on_a_mixed_handle_factor(pdg):
    """A MIXED handle's pd_sim_solve runs the FP64 supernodal solve (reordered sums): the
    allocation-free solve of its factor agrees with it to 1e-10 relative, on two calls in a row."""
    import copy
    import torch

    torch.cuda.set_device(0)
    scenes, cfg, _ = W.cloth40_full()
    c = copy.copy(cfg)
    c.precision = pdg.PD_PRECISION_MIXED
    sim = pdg.Simulator(scenes[0], c)
    f = sim.factor()
    rng = np.random.default_rng(5)
    for call in range(2):
        b = rng.standard_normal((scenes[0].n, 3)) * (10.0 ** call)
        x = _noalloc_solve(pdg, f, b)
        x_ref = sim.solve(b)
        assert np.max(np.abs(x - x_ref)) / np.max(np.abs(x_ref)) < 1e-10, call


def test_noalloc_at_the_workspace_limit(pdg):
    """n = PD_NOALLOC_MAX_VERTICES exactly (a 256 × 256 cloth, 65,536 vertices): accepted, and
    bit-identical to pd_sim_solve."""
    import torch

    torch.cuda.set_device(0)
    cfg = pdg.SceneConfig(grid_nx=256, grid_ny=256, grid_spacing=2.0 / 255.0, dt=1.0 / 300.0,
                          mass_mode=1, total_mass=4.0, pin_mode=1)
    scene = pdg.make_grid(cfg)
    assert scene.n == 65536
    sim = pdg.Simulator(scene, cfg)
    b = np.random.default_rng(3).standard_normal((scene.n, 3))
    x = _noalloc_solve(pdg, sim.factor(), b)
    assert np.array_equal(x.view(np.uint64), sim.solve(b).view(np.uint64))


def test_noalloc_rejects_oversized_problem(pdg):
    import torch

    lib = pdg.load_library()
    fn = lib.pd_solve_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int32] + [C.c_void_p] * 7 + [C.c_void_p]
    torch.cuda.set_device(0)
    t = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = _dev_ptr(t)
    rc = fn(65536 + 1, p, p, p, p, p, p, p, None)
    assert rc == 1
    assert "exceed" in lib.pd_last_error().decode()
