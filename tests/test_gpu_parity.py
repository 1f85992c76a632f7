"""GPU parity: the CUDA substep against the CPU oracle through the C ABI.

The FP64 reference-order mode must be bit-identical to the oracle (same scene arrays, same
elimination order), including the per-substep iteration counts chosen by the residual gate.
"""
import numpy as np
import pytest

from pd_gb300 import workloads as W
from tests.helpers import bits, oracle_twin

pytestmark = pytest.mark.gpu


def run_pair(pdg, scene, cfg, substeps, chunk=None):
    sim = pdg.Simulator(scene, cfg)
    perm = sim.factor()["perm"]
    orc = oracle_twin(scene, cfg, perm=perm)
    chunk = chunk or substeps
    done = 0
    while done < substeps:
        k = min(chunk, substeps - done)
        sim.step(k)
        it_g, cv_g = sim.iteration_log()
        it_o, cv_o = orc.step(k)
        assert np.array_equal(it_g, it_o), (done, it_g, it_o)
        assert np.array_equal(cv_g, cv_o)
        done += k
    return sim, orc


def assert_same_state(sim, orc, i=0):
    xg, vg = sim.state(i)
    xo, vo = orc.state()
    assert np.array_equal(bits(xg), bits(xo)), np.max(np.abs(xg - xo))
    assert np.array_equal(bits(vg), bits(vo)), np.max(np.abs(vg - vo))


def test_cloth40_plain_bit_identical(pdg):
    scenes, cfg, _ = W.cloth40_plain()
    sim, orc = run_pair(pdg, scenes[0], cfg, 120, chunk=40)
    assert_same_state(sim, orc)
    st = sim.stats()
    assert st["last_residual"] == orc.stats()["last_residual"]
    assert sim.info()["factorize_count"] == 1


def test_cloth40_full_bit_identical(pdg):
    scenes, cfg, _ = W.cloth40_full()
    sim, orc = run_pair(pdg, scenes[0], cfg, 24, chunk=12)
    assert_same_state(sim, orc)


def test_reference_bench_scene_bit_identical(pdg):
    """The reference's own bench scene (edge-lumped masses, top-row corner pins, κ=1e4, h=1/120)."""
    cfg = pdg.SceneConfig(stiffness=1e4, max_iterations=40, residual_tolerance=0.3)
    scene = pdg.make_grid(cfg)
    sim, orc = run_pair(pdg, scene, cfg, 30)
    assert_same_state(sim, orc)


def test_gate_fires_and_matches(pdg):
    """A loose residual gate makes substeps exit early; the GPU must pick the same counts."""
    cfg = W._base(grid_nx=12, grid_ny=12, grid_spacing=0.05, max_iterations=30, residual_tolerance=0.3,
                  velocity_damping=0.02)
    scene = pdg.make_grid(cfg)
    sim, orc = run_pair(pdg, scene, cfg, 200, chunk=50)
    assert_same_state(sim, orc)
    assert sim.stats()["early_exit_count"] == orc.stats()["early_exit_count"] > 0


def test_displacement_gate_matches(pdg):
    cfg = W._base(grid_nx=10, grid_ny=14, grid_spacing=0.05, max_iterations=25, residual_tolerance=0.0,
                  rel_tolerance=5e-2)
    scene = pdg.make_grid(cfg)
    sim, orc = run_pair(pdg, scene, cfg, 100)
    assert_same_state(sim, orc)


def test_batch_matches_individual_runs(pdg):
    scenes, cfgs, _ = W.batch(count=5, seed=7, max_side=32)
    sim = pdg.Simulator(scenes, cfgs)
    sim.step(20)
    for i, (s, c) in enumerate(zip(scenes, cfgs)):
        one = pdg.Simulator(s, c)
        one.step(20)
        xb, vb = sim.state(i)
        x1, v1 = one.state()
        assert np.array_equal(bits(xb), bits(x1))
        assert np.array_equal(bits(vb), bits(v1))
        orc = oracle_twin(s, c, perm=one.factor()["perm"])
        orc.step(20)
        xo, _ = orc.state()
        assert np.array_equal(bits(xb), bits(xo))


def test_pinned_vertices_exact_and_pin_move(pdg):
    scenes, cfg, _ = W.cloth40_plain()
    scene = scenes[0]
    sim = pdg.Simulator(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    pins = np.flatnonzero(scene.pinned)
    sim.step(10)
    orc.step(10)
    x, v = sim.state()
    assert np.array_equal(x[pins], scene.positions[pins]) and not np.any(v[pins])
    q = scene.positions.copy()
    q[pins, 0] += 0.05  # drag the handles: only the RHS changes
    sim.set_pin_positions(q)
    orc.set_pin_positions(q)
    sim.step(10)
    orc.step(10)
    assert_same_state(sim, orc)
    x, _ = sim.state()
    assert np.array_equal(x[pins], q[pins])
    assert sim.info()["factorize_count"] == 1


def test_stiffness_change_refactorizes_once(pdg):
    scenes, cfg, _ = W.cloth40_plain()
    scene = scenes[0]
    sim = pdg.Simulator(scene, cfg)
    orc = oracle_twin(scene, cfg, perm=sim.factor()["perm"])
    sim.step(5)
    orc.step(5)
    k = scene.edge_stiffness * 1.5
    sim.set_edge_stiffness(k)
    orc.set_edge_stiffness(k)
    sim.step(5)
    orc.step(5)
    assert_same_state(sim, orc)
    assert sim.info()["factorize_count"] == 2
    sim.set_edge_stiffness(k)  # unchanged values: no refactorization
    assert sim.info()["factorize_count"] == 2


def test_solve_matches_oracle_and_linear_residual(pdg):
    scenes, cfg, _ = W.cloth40_full()
    sim = pdg.Simulator(scenes[0], cfg)
    orc = oracle_twin(scenes[0], cfg, perm=sim.factor()["perm"])
    rng = np.random.default_rng(3)
    b = rng.standard_normal((scenes[0].n, 3))
    xg = sim.solve(b)
    xo = orc.solve(b)
    assert np.array_equal(bits(xg), bits(xo))
    rp, ci, val = orc.matrix()
    A = np.zeros((scenes[0].n, scenes[0].n))
    for r in range(scenes[0].n):
        A[r, ci[rp[r]:rp[r + 1]]] = val[rp[r]:rp[r + 1]]
    res = np.max(np.abs(A @ xg - b)) / np.max(np.abs(b))
    assert res < 1e-12


def test_global_solver_dropin(pdg):
    """IGlobalSolver surface: analyze / factorize / solve / solveComponent on the 3n × 3n L."""
    scenes, cfg, _ = W.cloth40_plain()
    orc = oracle_twin(scenes[0], cfg)
    rp, ci, val = orc.matrix()
    n = scenes[0].n
    # expand Ã to L = Ã ⊗ I₃ in compressed-column form (symmetric, so CSR of Ã = CSC)
    cols, rows, vals = [], [], []
    for c in range(n):
        for d in range(3):
            for p in range(rp[c], rp[c + 1]):
                rows.append(3 * ci[p] + d)
                vals.append(val[p])
            cols.append(len(rows))
    col_ptr = np.concatenate([[0], np.array(cols)]).astype(np.int32)
    s = pdg.GpuDirectSolver()
    s.analyze(3 * n, col_ptr, np.array(rows, np.int32))
    assert s.analyzed() and s.parallel_components() == 3
    s.factorize(3 * n, col_ptr, np.array(rows, np.int32), np.array(vals))
    b = np.random.default_rng(1).standard_normal(3 * n)
    x = s.solve(b)
    xo = orc.solve(b).reshape(-1)
    assert np.max(np.abs(x - xo)) / np.max(np.abs(xo)) < 1e-12
    xc = np.zeros(3 * n)
    for c in range(3):
        s.solve_component(c, b, xc)
    assert np.array_equal(bits(xc), bits(x))
    st = s.stats()
    assert st["analyze_calls"] == 1 and st["factorize_calls"] == 1 and st["solve_calls"] == 1


def test_solve_component_from_three_threads(pdg):
    """The reference's Integrator solves x, y and z from three OpenMP threads at once
    (core/sim/Integrator.cpp:558-565, IGlobalSolver.h:94-97). Three host threads, each with its own
    right-hand side, solve their component concurrently 40 times into one shared x; every column
    must equal that column of a three-column solve of its own b, bit for bit, and no thread may
    touch another's entries."""
    import threading
    scenes, cfg, _ = W.cloth40_full()
    orc = oracle_twin(scenes[0], cfg)
    rp, ci, val = orc.matrix()
    n = scenes[0].n
    cols, rows, vals = [], [], []
    for c in range(n):
        for d in range(3):
            for p in range(rp[c], rp[c + 1]):
                rows.append(3 * ci[p] + d)
                vals.append(val[p])
            cols.append(len(rows))
    col_ptr = np.concatenate([[0], np.array(cols)]).astype(np.int32)
    s = pdg.GpuDirectSolver()
    s.analyze(3 * n, col_ptr, np.array(rows, np.int32))
    s.factorize(3 * n, col_ptr, np.array(rows, np.int32), np.array(vals))
    rng = np.random.default_rng(7)
    rounds = 40
    bs = [[rng.standard_normal(3 * n) for _ in range(3)] for _ in range(rounds)]
    want = [[s.solve(bs[r][c])[c::3].copy() for c in range(3)] for r in range(rounds)]
    got = [np.full(3 * n, np.nan) for _ in range(rounds)]
    errors = []
    start = threading.Barrier(3)

    def worker(c):
        try:
            start.wait()
            for r in range(rounds):
                s.solve_component(c, bs[r][c], got[r])
        except Exception as e:  # noqa: BLE001 — reported below
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(c,)) for c in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(120)
    assert not errors, errors
    for r in range(rounds):
        for c in range(3):
            assert np.array_equal(bits(got[r][c::3]), bits(want[r][c])), (r, c)


def test_spring_closed_form_and_equilibrium(pdg):
    """pd_check items 2-5: one-step closed form, equilibrium ℓ − mg/κ, pinned exact, free fall."""
    h, m, ell, k, g = 1.0 / 120.0, 0.05, 0.1, 1.0e4, 9.81
    cfg = pdg.SceneConfig(dt=h, stiffness=k, velocity_damping=0.0, max_iterations=40,
                          rel_tolerance=0.0, abs_tolerance=1e-18)
    scene = pdg.GridScene(positions=np.array([[0.0, 0.0, 0.0], [0.0, 0.12, 0.0]]), masses=np.array([m, m]),
                          pinned=np.array([1, 0], np.uint8), edges=np.array([[0, 1]], np.int32),
                          edge_rest=np.array([ell]), edge_stiffness=np.array([k]))
    sim = pdg.Simulator(scene, cfg)
    sim.step(1)
    x, _ = sim.state()
    yhat = 0.12 - h * h * g
    mh2 = m / (h * h)
    assert abs(x[1, 1] - (mh2 * yhat + k * ell) / (mh2 + k)) < 1e-12
    sim.step(20000 - 1)
    x, _ = sim.state()
    assert abs(x[1, 1] - (ell - m * g / k)) < 1e-6 * ell
    assert x[0, 0] == 0.0 and x[0, 1] == 0.0 and x[0, 2] == 0.0
    free = pdg.GridScene(positions=np.zeros((1, 3)), masses=np.ones(1), pinned=np.zeros(1, np.uint8),
                         edges=np.zeros((0, 2), np.int32), edge_rest=np.zeros(0), edge_stiffness=np.zeros(0))
    fc = pdg.SceneConfig(dt=h, velocity_damping=0.0, max_iterations=4)
    fs = pdg.Simulator(free, fc)
    fs.step(1)
    x, _ = fs.state()
    assert abs(x[0, 1] - (-h * h * g)) < 1e-14


def test_invalid_inputs_raise(pdg):
    scenes, cfg, _ = W.cloth40_plain()
    bad = scenes[0]
    bad.edges = bad.edges.copy()
    bad.edges[0, 1] = 10 ** 6
    with pytest.raises(pdg.PdError) as e:
        pdg.Simulator(bad, cfg)
    assert e.value.code == 1
    scenes, cfg, _ = W.cloth40_plain()
    sim = pdg.Simulator(scenes[0], cfg)
    with pytest.raises(pdg.PdError):
        sim.state(5)
    with pytest.raises(pdg.PdError):
        sim.set_state(0, x=np.full((scenes[0].n, 3), np.nan))
