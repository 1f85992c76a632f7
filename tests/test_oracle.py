"""The CPU oracle pinned against the reference's own known answers and published outputs.

Sources: _verify/check.cpp:75-244 (pd_check items), tests/chain/spring_vertical.cpp,
tests/chain/convergence_criterion.cpp, tests/primitives/test_distance_term.cpp, and the golden
physics outputs printed in docs/perf.md:858,888,1422-1424, docs/solver-feasibility.md:143-146 and
docs/chebyshev.md:280-287.
"""
import math

import numpy as np
import pytest

H, M, ELL, K, G = 1.0 / 120.0, 0.05, 0.1, 1.0e4, 9.81


def spring(O, y0, kd=0.0, iters=40, v0=0.0, k=K, h=H, mass=M, rel=0.0, abs_tol=1e-18, res_tol=1e-3):
    mesh = O.Mesh(positions=np.array([[0.0, 0.0, 0.0], [0.0, y0, 0.0]]), masses=np.array([mass, mass]),
                  pinned=np.array([1, 0], np.uint8), edges=np.array([[0, 1]], np.int32),
                  edge_rest=np.array([ELL]), edge_k=np.array([k]),
                  velocities=np.array([[0.0, 0.0, 0.0], [0.0, v0, 0.0]]))
    cfg = O.Config(dt=h, velocity_damping=kd, max_iterations=iters, rel_tolerance=rel,
                   abs_tolerance=abs_tol, residual_tolerance=res_tol)
    return O.OracleSim(mesh, cfg)


def closed_form(yhat, mass, k, h):
    mh2 = mass / (h * h)
    return (mh2 * yhat + k * ELL) / (mh2 + k)


# ---------------------------------------------------------------- pd_check (_verify/check.cpp)
def test_check1_projection_length(oracle):
    d = oracle.project_one([0, 0, 0], [0, 0.31, 0], ELL)
    assert abs(np.linalg.norm(d) - ELL) < 1e-14


def test_check2_one_step_closed_form(oracle):
    s = spring(oracle, 0.12)
    s.step(1)
    x, _ = s.state()
    assert abs(x[1, 1] - closed_form(0.12 - H * H * G, M, K, H)) < 1e-12


def test_check3_equilibrium(oracle):
    s = spring(oracle, 0.12)
    s.step(20000)
    x, _ = s.state()
    assert abs(x[1, 1] - (ELL - M * G / K)) < 1e-6 * ELL


def test_check4_pinned_exact(oracle):
    s = spring(oracle, 0.12)
    worst = 0.0
    for _ in range(200):
        s.step(1)
        x, _ = s.state()
        worst = max(worst, abs(x[0, 1]))
    assert worst == 0.0


def test_check5_free_fall(oracle):
    mesh = oracle.Mesh(positions=np.zeros((1, 3)), masses=np.ones(1), pinned=np.zeros(1, np.uint8),
                       edges=np.zeros((0, 2), np.int32), edge_rest=np.zeros(0), edge_k=np.zeros(0))
    s = oracle.OracleSim(mesh, oracle.Config(dt=H, velocity_damping=0.0, max_iterations=4))
    s.step(1)
    x, _ = s.state()
    assert abs(x[0, 1] - (-H * H * G)) < 1e-14


def test_check6_cloth_bounded(oracle):
    m = oracle.make_grid(oracle.GridSpec(nx=12, ny=12, spacing=0.05, stiffness=K))
    s = oracle.OracleSim(m, oracle.Config(dt=H, max_iterations=10, rel_tolerance=1e-3))
    s.step(400)
    x, _ = s.state()
    assert np.all(np.isfinite(x)) and np.max(np.abs(x[:, 1])) < 1.0


def test_check7_factorize_once(oracle):
    m = oracle.make_grid(oracle.GridSpec(nx=20, ny=20, spacing=0.02, stiffness=K))
    s = oracle.OracleSim(m, oracle.Config(dt=H, max_iterations=10))
    s.step(200)
    assert s.stats()["factorize_count"] == 1


def test_check8_force_sign(oracle):
    for y1 in (0.06, 0.08, 0.0999, 0.1001, 0.12, 0.15):
        for free_is_b in (True, False):
            if free_is_b:
                pa, pb = np.zeros(3), np.array([0, y1, 0.0])
                x_free, x_pin = pb, pa
            else:
                pa, pb = np.array([0, y1, 0.0]), np.zeros(3)
                x_free, x_pin = pa, pb
            d = oracle.project_one(pa, pb, ELL)
            r = np.linalg.norm(x_free - x_pin)
            true_force = (x_free - x_pin) * (-K * (r - ELL) / r)
            code_force = (d * (-K) if free_is_b else d * K) - x_free * K
            assert abs(code_force[1] - true_force[1]) <= 1e-6


# ---------------------------------------------------------- spring (tests/chain/spring_vertical.cpp)
@pytest.mark.parametrize("k,h,y0", [(1.0, 1 / 60, 0.12), (100.0, 1 / 60, 0.12), (1e4, 1 / 60, 0.12),
                                    (1e4, 1 / 120, 0.12), (1e4, 1 / 240, 0.12), (1e4, 1 / 120, 0.09),
                                    (100.0, 1 / 120, 0.08)])
def test_fixed_point_matches_closed_form(oracle, k, h, y0):
    s = spring(oracle, y0, iters=60, k=k, h=h, abs_tol=1e-16)
    s.step(1)
    x, _ = s.state()
    assert abs(x[1, 1] / ELL - closed_form(y0 - h * h * G, M, k, h) / ELL) < 1e-12


def test_matches_independent_recurrence(oracle):
    y, v = 0.12, 0.0
    s = spring(oracle, 0.12, iters=60, abs_tol=1e-16)
    worst_p = worst_v = 0.0
    for _ in range(300):
        yhat = y + H * v - H * H * G
        y_new = closed_form(yhat, M, K, H)
        v = (y_new - y) / H
        y = y_new
        s.step(1)
        x, vel = s.state()
        worst_p = max(worst_p, abs(x[1, 1] - y) / ELL)
        worst_v = max(worst_v, abs(vel[1, 1] - v) * H / ELL)
    assert worst_p <= 1e-11 and worst_v <= 1e-11


def test_linear_residual_and_factor_reuse(oracle):
    m = oracle.make_grid(oracle.GridSpec(nx=20, ny=20, spacing=0.02, stiffness=K, shear_stiffness=K,
                                         bend_stiffness=100.0))
    s = oracle.OracleSim(m, oracle.Config(dt=H))
    rp, ci, val = s.matrix()
    A = np.zeros((m.n, m.n))
    for r in range(m.n):
        A[r, ci[rp[r]:rp[r + 1]]] = val[rp[r]:rp[r + 1]]
    rng = np.random.default_rng(0)
    for _ in range(2):  # the same factor serves a second right-hand side
        b = rng.standard_normal((m.n, 3))
        x = s.solve(b)
        assert np.max(np.abs(A @ x - b)) / np.max(np.abs(b)) < 1e-12
    assert s.stats()["factorize_count"] == 1


# ---------------------------------------------------------- golden outputs (docs/perf.md)
GOLDEN = {  # iters, tol -> residual, strain max, strain mean, elastic, total (or None)
    (10, 1e-3): (24.10, 0.057035, 0.00134129, 0.318593, None),
    (20, 0.3): (13.3816, 0.0581053, 0.00134602, 0.320141, None),
    (40, 0.3): (8.63991, 0.0585735, 0.0013502, 0.322049, -10.5941),
    (80, 1e-3): (6.40876, 0.0586015, 0.00135108, 0.322604, None),
}


def sig(a, b, digits=6):
    return float(f"{a:.{digits}g}") == float(f"{b:.{digits}g}")


@pytest.mark.parametrize("iters,tol", list(GOLDEN))
def test_reference_bench_golden_outputs(oracle, iters, tol):
    """pd_bench 40×40, κ=1e4, h=1/120, 300 substeps: outputs as printed by the reference."""
    m = oracle.make_grid(oracle.GridSpec(nx=40, ny=40, spacing=0.025, stiffness=1e4))
    s = oracle.OracleSim(m, oracle.Config(dt=1 / 120, velocity_damping=0.02, max_iterations=iters,
                                          residual_tolerance=tol))
    worst = 0.0
    conv = 0
    for _ in range(300):
        _, c = s.step(1)
        conv += int(c[0])
        worst = max(worst, s.stats()["max_strain"])
    st = s.stats()
    res, smax, smean, el, tot = GOLDEN[(iters, tol)]
    assert conv == 0
    assert sig(st["last_residual"], res, 4 if iters == 10 else 6)
    assert sig(st["max_strain"], smax) and sig(st["mean_strain"], smean) and sig(st["elastic_energy"], el)
    assert st["matrix_nnz"] * 3 == 23496 and st["color_count"] == 6
    if tot is not None:
        assert sig(st["total_energy"], tot) and sig(worst, 0.0652267)


CHEB_GOLDEN = {  # iterations -> last residual, plain PD and PD_CHEB=1 (ρ 0.98, 10 plain iterations)
    10: (27.3033, 27.3033),
    20: (12.3328, 9.37677),
    40: (8.59041, 7.40925),
    80: (6.14024, 3.51819),
}


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("iters", list(CHEB_GOLDEN))
def test_reference_chebyshev_golden_outputs(oracle, iters, mode):
    """docs/chebyshev.md:280-287: pd_bench --grid 60 60 --steps 300 (κ=1e4, h=1/120, damping
    0.02, residual gate 1e-3 never met) with and without PD_CHEB=1: the last residual."""
    m = oracle.make_grid(oracle.GridSpec(nx=60, ny=60, spacing=0.025, stiffness=1e4))
    s = oracle.OracleSim(m, oracle.Config(dt=1 / 120, velocity_damping=0.02, max_iterations=iters,
                                          residual_tolerance=1e-3, cheb_mode=mode))
    s.step(300)
    st = s.stats()
    assert st["early_exit_count"] == 0
    assert sig(st["last_residual"], CHEB_GOLDEN[iters][mode])


def test_chebyshev_weights_and_warmup(oracle):
    """Blending starts after cheb_start plain iterations (bit-identical to plain PD before), and the
    interval mode's roots blend from the first iteration."""
    m = oracle.make_grid(oracle.GridSpec(nx=12, ny=12, spacing=0.025, stiffness=1e4))
    runs = {}
    for key, cfg in {"plain": dict(cheb_mode=0), "warm": dict(cheb_mode=1, cheb_start=12),
                     "rho": dict(cheb_mode=1, cheb_start=3), "roots": dict(cheb_mode=2, cheb_m=0.5, cheb_d=0.45)}.items():
        s = oracle.OracleSim(m, oracle.Config(dt=1 / 120, max_iterations=12, residual_tolerance=0.0,
                                              rel_tolerance=0.0, abs_tolerance=0.0, **cfg))
        s.step(20)
        runs[key] = s.state()[0]
    assert np.array_equal(runs["plain"], runs["warm"])  # k > cheb_start never holds with 12 iterations
    assert not np.array_equal(runs["plain"], runs["rho"])
    assert not np.array_equal(runs["plain"], runs["roots"])
    assert np.all(np.isfinite(runs["roots"]))


def test_reference_bend_golden_outputs(oracle):
    """docs/perf.md:856-862: PD_BEND=1000 row of the κ_b scan (40 iterations, 300 substeps)."""
    m = oracle.make_grid(oracle.GridSpec(nx=40, ny=40, spacing=0.025, stiffness=1e4, bend_stiffness=1000.0))
    s = oracle.OracleSim(m, oracle.Config(dt=1 / 120, velocity_damping=0.02, max_iterations=40,
                                          residual_tolerance=0.3))
    s.step(300)
    st = s.stats()
    assert sig(st["last_residual"], 5235.6, 5) and sig(st["max_strain"], 0.04993, 4)
    assert sig(st["mean_strain"], 0.00139981) and sig(st["elastic_energy"], 0.42291, 5)


# ---------------------------------------------------- topology (tests/primitives/test_distance_term.cpp)
@pytest.mark.parametrize("nx,ny", [(2, 2), (3, 5), (40, 40), (17, 9)])
def test_grid_counts_and_coloring(oracle, nx, ny):
    m = oracle.make_grid(oracle.GridSpec(nx=nx, ny=ny, shear_stiffness=1.0, bend_stiffness=1.0))
    ne_struct = 2 * nx * ny - nx - ny
    assert m.edges.shape[0] == ne_struct + (nx - 1) * (ny - 1)
    assert m.bends.shape[0] == (nx - 2) * ny + (ny - 2) * nx
    pairs = {tuple(sorted(e)) for e in m.edges.tolist()}
    assert len(pairs) == m.edges.shape[0]
    s = oracle.OracleSim(m, oracle.Config())
    c = s.coloring()
    col = c["color_of"]
    # proper: no two edges of one colour share a vertex; complete: every edge coloured
    for v in range(m.n):
        inc = c["vedges"][c["vstart"][v]:c["vstart"][v + 1]]
        assert len(set(col[inc].tolist())) == len(inc)
    assert col.max() + 1 == c["count"]
    deg = np.bincount(m.edges.reshape(-1), minlength=m.n).max()
    assert c["count"] >= deg


def test_flat_cloth_has_zero_bend_force_and_rhs(oracle):
    m = oracle.make_grid(oracle.GridSpec(nx=8, ny=8, spacing=0.1, bend_stiffness=500.0, pin_mode=4))
    s = oracle.OracleSim(m, oracle.Config())
    assert not np.any(s.bend_rhs())


def test_bend_rhs_analytic_three_points(oracle):
    """Three collinear points, outer two pinned: b_middle gets −k·w_b·(q_a + q_c) = +2k·(q_a + q_c)."""
    k = 100.0
    pos = np.array([[0.0, 0.0, 0.0], [0.5, 0.3, 0.0], [1.0, 0.0, 0.0]])
    mesh = oracle.Mesh(positions=pos, masses=np.ones(3), pinned=np.array([1, 0, 1], np.uint8),
                       edges=np.zeros((0, 2), np.int32), edge_rest=np.zeros(0), edge_k=np.zeros(0),
                       bends=np.array([[0, 1, 2]], np.int32), bend_k=np.array([k]))
    s = oracle.OracleSim(mesh, oracle.Config())
    rhs = s.bend_rhs()
    assert np.allclose(rhs[1], 2 * k * (pos[0] + pos[2])) and not np.any(rhs[[0, 2]])


# ------------------------------------------------- gate (tests/chain/convergence_criterion.cpp)
def test_gate_is_translation_invariant(oracle):
    base = oracle.make_grid(oracle.GridSpec(nx=10, ny=10, spacing=0.05, stiffness=K))
    iters = []
    for shift in (0.0, 1000.0):
        m = oracle.make_grid(oracle.GridSpec(nx=10, ny=10, spacing=0.05, stiffness=K))
        m.positions = base.positions + shift
        s = oracle.OracleSim(m, oracle.Config(dt=H, max_iterations=30, residual_tolerance=0.0,
                                              rel_tolerance=1e-2))
        it, _ = s.step(30)
        iters.append(it)
    assert np.array_equal(iters[0], iters[1])


def test_zero_tolerances_disable_early_exit(oracle):
    m = oracle.make_grid(oracle.GridSpec(nx=8, ny=8, spacing=0.05, stiffness=K))
    s = oracle.OracleSim(m, oracle.Config(dt=H, max_iterations=7, residual_tolerance=0.0, rel_tolerance=0.0,
                                          abs_tolerance=0.0))
    it, cv = s.step(20)
    assert np.all(it == 7) and not np.any(cv)


def test_tangential_convergence_rate(oracle):
    """A spring pulled sideways needs many iterations: completion ≈ 1 − q^N, q = κ/(κ + m/h²)."""
    k, h = 1e4, 1 / 120
    q = k / (k + M / (h * h))
    done = []
    for n_it in (1, 5, 20):
        mesh = oracle.Mesh(positions=np.array([[0.0, 0.0, 0.0], [0.0, -ELL, 0.0]]), masses=np.array([M, M]),
                           pinned=np.array([1, 0], np.uint8), edges=np.array([[0, 1]], np.int32),
                           edge_rest=np.array([ELL]), edge_k=np.array([k]),
                           velocities=np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]]))
        s = oracle.OracleSim(mesh, oracle.Config(dt=h, gravity=(0.0, 0.0, 0.0), velocity_damping=0.0,
                                                 max_iterations=n_it, residual_tolerance=0.0, rel_tolerance=0.0,
                                                 abs_tolerance=0.0))
        s.step(1)
        x, _ = s.state()
        done.append(x[1, 0])
    assert done[0] < done[1] < done[2]
    assert q > 0.9 and math.isfinite(done[2])


def test_thread_count_independence(oracle):
    m = oracle.make_grid(oracle.GridSpec(nx=40, ny=40, spacing=0.025, stiffness=1e4, shear_stiffness=1e4,
                                         bend_stiffness=10.0))
    out = []
    for t in (1, 3, 8):
        s = oracle.OracleSim(m, oracle.Config(dt=1 / 120, max_iterations=8, threads=t))
        s.step(5)
        out.append(s.state()[0])
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])


def _fd_problem(side=10, substeps=12, seed=3):
    from pd_gb300 import workloads as W
    from tests.helpers import oracle_twin
    scene, cfg, S, kstar = W.differentiable(side=side, substeps=substeps)
    twin = oracle_twin(scene, cfg)
    twin.set_edge_stiffness(kstar)
    twin.step(S)
    targets = twin.state()[0]
    rng = np.random.default_rng(seed)
    force = rng.normal(0.0, 0.05, (scene.n, 3))
    return scene, cfg, S, targets, force, rng


def test_oracle_gradient_matches_central_differences():
    """The CPU reference gradient (adjoint, FP64) against central differences of its own loss,
    directions in stiffness, initial velocity and external force."""
    from tests.helpers import oracle_twin
    scene, cfg, S, targets, force, rng = _fd_problem()
    orc = oracle_twin(scene, cfg)
    g = orc.gradient(S, targets, force)
    x0, v0 = orc.state()
    k0 = np.asarray(scene.edge_stiffness, np.float64)

    def loss(k, v, f):
        o = oracle_twin(scene, cfg)
        o.set_edge_stiffness(k)
        o.set_state(x0, v)
        return o.gradient(S, targets, f, grad=False)["loss"]

    eps = 1e-4
    for _ in range(3):
        dk = k0 * rng.normal(0.0, 0.05, k0.shape)
        dv = rng.normal(0.0, 0.1, v0.shape)
        df = rng.normal(0.0, 0.05, force.shape)
        fd = (loss(k0 + eps * dk, v0 + eps * dv, force + eps * df)
              - loss(k0 - eps * dk, v0 - eps * dv, force - eps * df)) / (2 * eps)
        adj = g["dkappa"] @ dk + np.sum(g["dv0"] * dv) + np.sum(g["dforce"] * df)
        assert abs(fd - adj) <= 1e-6 * abs(adj), (fd, adj)
    # the state is left unchanged and the loss-only call agrees
    assert np.array_equal(orc.state()[0], x0)
    assert orc.gradient(S, targets, force, grad=False)["loss"] == g["loss"]


# ---------------------------------------------------------- OBJ meshes (core/mesh/Mesh.cpp:56-153)
def test_obj_known_answers(oracle):
    tri = "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n"
    m = oracle.make_obj(tri, stiffness=500.0, density=3.0)
    assert m.edges.tolist() == [[0, 1], [1, 2], [2, 0]]
    assert np.allclose(m.edge_rest, [1.0, math.sqrt(2.0), 1.0], rtol=0, atol=1e-15)
    assert np.all(m.edge_k == 500.0)
    assert np.allclose(m.masses, 3.0 * 0.5 / 3.0, rtol=0, atol=1e-16)
    # a quad as two triangles in slash styles; a four-index face keeps its first three corners
    quad = "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1/1 2/2 3/3\nf 1//1 3//3 4//4 2//2\n"
    m = oracle.make_obj(quad, density=1.0)
    assert m.edges.tolist() == [[0, 1], [1, 2], [2, 0], [2, 3], [3, 0]]
    assert np.allclose(m.masses, [1 / 3, 1 / 6, 1 / 3, 1 / 6], rtol=0, atol=1e-16)
    # a repeated corner adds no edge; an unused vertex takes the smallest positive mass
    deg = "v 0 0 0\nv 2 0 0\nv 0 2 0\nv 5 5 5\nf 1 2 3\nf 1 1 2\n"
    m = oracle.make_obj(deg)
    assert len(m.edges) == 3 and m.masses[3] == m.masses[0]
    for bad in ("v 0 0 0\n", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 x\n", "v 0 0 0\nv 1 0 0\nf 1 2 3\n",
                "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 1 2\n"):
        with pytest.raises(ValueError):
            oracle.make_obj(bad)


def test_residual_trace_matches_gate(oracle):
    """step_traced records every iteration's gate residual: as many as the iterations used, the
    last one the stats' last residual, NaN after an early exit."""
    m = oracle.make_grid(oracle.GridSpec(nx=12, ny=12, spacing=0.05, stiffness=K))
    cfg = oracle.Config(dt=H, max_iterations=30, residual_tolerance=0.6)
    a, b = oracle.OracleSim(m, cfg), oracle.OracleSim(m, cfg)
    tr = a.step_traced(20)
    it, _ = b.step(20)
    assert np.array_equal((~np.isnan(tr)).sum(axis=1), it) and (it < 30).any()
    last = tr[-1][~np.isnan(tr[-1])][-1]
    assert last == a.stats()["last_residual"] == b.stats()["last_residual"]


# ------------------------------------------- spectrum of the PD map (_verify/iteration_spectrum.cpp)
def test_spectrum_spring_closed_form(oracle):
    """One free vertex on one edge to a pinned vertex: B = (m/h²·I + κ·n nᵀ)/(m/h² + κ), so
    λ_max(B) = 1 (along the edge) and ρ(T) = κ/(m/h² + κ) (across it)."""
    s = spring(oracle, 0.12)
    r = s.spectrum(60)
    mh2 = M / (H * H)
    assert abs(r["rho_plain"] - K / (mh2 + K)) <= 1e-14
    assert abs(r["lambda_max"] - 1.0) <= 1e-14


def _dense_pd_operator(oracle, s, mesh):
    """B = A⁻¹(M/h² + N + Σ_s k·A_sᵀA_s) on the free components, built densely from the oracle's
    assembled A and the current positions."""
    n = mesh.positions.shape[0]
    rp, ci, val = s.matrix()
    A = np.zeros((n, n))
    for r in range(n):
        A[r, ci[rp[r]:rp[r + 1]]] = val[rp[r]:rp[r + 1]]
    A3 = np.kron(A, np.eye(3))
    x, _ = s.state()
    C = np.zeros((3 * n, 3 * n))
    h = s.cfg.dt if hasattr(s, "cfg") else H
    for v in range(n):
        C[3 * v:3 * v + 3, 3 * v:3 * v + 3] += mesh.masses[v] / (h * h) * np.eye(3)
    for (a, b), k in zip(mesh.edges, mesh.edge_k):
        rel = x[a] - x[b]
        nn = rel / np.linalg.norm(rel)
        P = k * np.outer(nn, nn)
        for i, j, sg in ((a, a, 1), (b, b, 1), (a, b, -1), (b, a, -1)):
            C[3 * i:3 * i + 3, 3 * j:3 * j + 3] += sg * P
    w = (1.0, -2.0, 1.0)
    for (a, b, c), k in zip(mesh.bends, mesh.bend_k):
        vs = (a, b, c)
        for p in range(3):
            for q in range(3):
                C[3 * vs[p]:3 * vs[p] + 3, 3 * vs[q]:3 * vs[q] + 3] += k * w[p] * w[q] * np.eye(3)
    free = np.repeat(mesh.pinned == 0, 3)
    Bm = np.linalg.solve(A3, C)
    return Bm[np.ix_(free, free)]


def test_spectrum_matches_dense_eigenvalues(oracle):
    """A 6×5 cloth with shear and bending, moved off its rest pose: the power-iteration estimates
    against the eigenvalues of the dense operator."""
    spec = oracle.GridSpec(nx=6, ny=5, spacing=0.1, stiffness=3000.0, shear_stiffness=900.0, bend_stiffness=40.0)
    mesh = oracle.make_grid(spec)
    cfg = oracle.Config(dt=1.0 / 120.0, max_iterations=20, residual_tolerance=0.0, rel_tolerance=0.0,
                        abs_tolerance=0.0)
    s = oracle.OracleSim(mesh, cfg)
    s.step(15)
    ev = np.linalg.eigvals(_dense_pd_operator(oracle, s, mesh)).real
    r = s.spectrum(4000)
    assert abs(r["lambda_max"] - ev.max()) <= 1e-9
    # T's two largest |eigenvalues| nearly coincide here, so the estimate settles more slowly
    assert abs(r["rho_plain"] - np.max(np.abs(1.0 - ev))) <= 1e-6
    assert 0.0 < ev.min() and ev.max() <= 1.0 + 1e-12  # B's spectrum lies in (0, 1]
