"""More of the reference's known answers for the oracle: the scatter's signs and pin-elimination
term (tests/primitives/test_distance_term.cpp:108-221), the colour-ordered scatter against an
edge-order sum (:465-506), the bend stencil's matrix rows and constant right-hand side (:961-1012),
translation invariance (_verify/translation_invariance.cpp), the pinned chain's analytic
length change (_verify/chain_test.cpp), the projection-direction and bend audits
(_verify/direction_audit.cpp, _verify/bend_audit.cpp), the projection's definition, the refactorization
stamp and grid construction (test_distance_term.cpp:44-99,293-330,769-935,1274-1330) and the spring
fixed points (tests/chain/spring_vertical.cpp:130-152,231-252,442-512). Every reference value is restated here from the test's
description; the expected sums are computed independently in numpy.
"""
import math

import numpy as np
import pytest


def two_vertices(O, pos, pinned, q, k, rest, mass=0.1):
    mesh = O.Mesh(positions=np.asarray(pos, np.float64), masses=np.full(2, mass),
                  pinned=np.asarray(pinned, np.uint8), edges=np.array([[0, 1]], np.int32),
                  edge_rest=np.array([rest]), edge_k=np.array([k]), pin_positions=np.asarray(q, np.float64))
    return O.OracleSim(mesh, O.Config())


def projection(xa, xb, rest):
    raw = np.asarray(xa, np.float64) - np.asarray(xb, np.float64)
    ln = math.sqrt(float(raw @ raw))
    return np.zeros(3) if ln <= 1e-12 else raw * (rest / ln)


# ------------------------------------------------ scatter signs (test_distance_term.cpp:108-139)
def test_scatter_uses_the_standard_pd_sign(oracle):
    """d = ℓ·unit(x_a − x_b); b_a += κd, b_b −= κd; with a at the origin and b at +0.3ŷ the
    y components are −κℓ and +κℓ and every other component is zero."""
    k, rest = 500.0, 0.1
    pos = [[0.0, 0.0, 0.0], [0.0, 0.3, 0.0]]
    s = two_vertices(oracle, pos, [0, 0], pos, k, rest)
    b = s.rhs(np.zeros((2, 3)), overwrite_pins=False).reshape(-1)
    assert abs(b[1] - (-k * rest)) <= 1e-12 and abs(b[4] - k * rest) <= 1e-12
    assert b[0] == 0.0 and b[2] == 0.0 and b[3] == 0.0 and b[5] == 0.0
    assert abs(np.linalg.norm(projection(pos[0], pos[1], rest)) - rest) <= 1e-15


# ------------------------------------- pin elimination (test_distance_term.cpp:141-221)
def test_pin_elimination_adds_kappa_times_the_pin_position(oracle):
    """One end pinned: the free end's row gains κ·q of the pinned end (its coupling moved to the
    right-hand side); the pinned row takes nothing; both ends pinned skips the constraint."""
    k, rest = 300.0, 0.1
    # (a) vertex 1 pinned at q_1, vertex 0 free somewhere unrelated to q_1
    pos = [[0.7, -0.2, 0.3], [2.0, 1.0, -4.0]]
    q = [[0.0, 0.0, 0.0], [2.0, 1.0, -4.0]]
    s = two_vertices(oracle, pos, [0, 1], q, k, rest)
    b = s.rhs(np.zeros((2, 3)), overwrite_pins=False)
    want = k * projection(pos[0], pos[1], rest) + k * np.asarray(q[1])
    assert np.max(np.abs(b[0] - want)) <= 1e-12 and not np.any(b[1])
    # (b) vertex 0 pinned, vertex 1 free: the other branch
    pos = [[-1.5, 0.4, 0.25], [0.0, rest, 0.0]]
    q = [[-1.5, 0.4, 0.25], [0.0, 0.0, 0.0]]
    s = two_vertices(oracle, pos, [1, 0], q, k, rest)
    b = s.rhs(np.zeros((2, 3)), overwrite_pins=False)
    want = -k * projection(pos[0], pos[1], rest) + k * np.asarray(q[0])
    assert np.max(np.abs(b[1] - want)) <= 1e-12 and not np.any(b[0])
    # (c) both pinned: the constraint contributes nothing
    pos = [[0.0, 0.0, 0.0], [0.0, 2 * rest, 0.0]]
    s = two_vertices(oracle, pos, [1, 1], pos, k, rest)
    assert not np.any(s.rhs(np.zeros((2, 3)), overwrite_pins=False))


# ------------------------- colour-ordered scatter vs edge order (test_distance_term.cpp:392-506)
def perturbed_grid(O, n=20, spacing=0.02, k=2.0e3):
    m = O.make_grid(O.GridSpec(nx=n, ny=n, spacing=spacing, stiffness=k, pin_mode=4))
    v = np.arange(n * n)
    i, j = (v % n).astype(np.float64), (v // n).astype(np.float64)
    m.positions = m.positions + spacing * np.stack([0.20 * np.sin(1.7 * i + 0.5 * j),
                                                    0.30 * np.cos(0.9 * i - 1.3 * j),
                                                    0.25 * np.sin(0.4 * i + 2.1 * j)], axis=1)
    m.pinned = np.zeros(n * n, np.uint8)
    m.pinned[[0, n * n - 1]] = 1  # both one-end-pinned branches occur
    m.pin_positions = m.positions.copy()
    return m


def edge_order_scatter(m):
    """b_a += κd, b_b −= κd, one end pinned adds κ·q to the free end: summed in edge order."""
    b = np.zeros((m.n, 3))
    for (a, c), rest, k in zip(m.edges, m.edge_rest, m.edge_k):
        pa, pc = m.pinned[a], m.pinned[c]
        if pa and pc:
            continue
        d = projection(m.positions[a], m.positions[c], rest)
        if not pa:
            b[a] += k * d + (k * m.pin_positions[c] if pc else 0.0)
        if not pc:
            b[c] += -k * d + (k * m.pin_positions[a] if pa else 0.0)
    return b


def test_colour_ordered_scatter_matches_the_edge_order_sum(oracle):
    m = perturbed_grid(oracle)
    assert m.edges.shape[0] >= 256
    s = oracle.OracleSim(m, oracle.Config())
    got = s.rhs(np.zeros((m.n, 3)), overwrite_pins=False)
    ref = edge_order_scatter(m)
    assert np.max(np.abs(got - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))
    col = s.coloring()
    assert col["count"] >= 2


# ------------------------------- bend stencil rows (test_distance_term.cpp:961-1012)
def test_bend_stencil_matrix_rows_and_constant_rhs(oracle):
    """Three points (0,0,0), (0.1, ε, 0), (0.2, 0, 0), outer two pinned, k = 2000: pinned rows are
    exact identity rows with the pinned columns removed from the free row, the free diagonal is
    m/h² + 4k (w_b² = 4), and the middle vertex's constant right-hand side is −k·w_b·(q_a + q_c):
    +800 in x, 0 in y and z; pinned rows take none."""
    spacing, k, eps, h, mass = 0.1, 2.0e3, 0.01, 1.0 / 120.0, 0.05
    pos = np.array([[0.0, 0.0, 0.0], [spacing, eps, 0.0], [2 * spacing, 0.0, 0.0]])
    mesh = oracle.Mesh(positions=pos, masses=np.full(3, mass), pinned=np.array([1, 0, 1], np.uint8),
                       edges=np.zeros((0, 2), np.int32), edge_rest=np.zeros(0), edge_k=np.zeros(0),
                       bends=np.array([[0, 1, 2]], np.int32), bend_k=np.array([k]),
                       pin_positions=np.array([[0.0, 0.0, 0.0], [spacing, eps, 0.0], [2 * spacing, 0.0, 0.0]]))
    s = oracle.OracleSim(mesh, oracle.Config(dt=h))
    rp, ci, val = s.matrix()
    A = np.zeros((3, 3))
    for r in range(3):
        A[r, ci[rp[r]:rp[r + 1]]] = val[rp[r]:rp[r + 1]]
    assert A[0, 0] == 1.0 and A[0, 1] == 0.0 and A[0, 2] == 0.0 and A[1, 0] == 0.0
    assert A[2, 2] == 1.0 and A[1, 2] == 0.0
    assert abs(A[1, 1] - (mass / (h * h) + 4.0 * k)) <= 1e-9
    rhs = s.bend_rhs()
    assert abs(rhs[1, 0] - 800.0) <= 1e-9 and rhs[1, 1] == 0.0 and rhs[1, 2] == 0.0
    assert not np.any(rhs[[0, 2]])


# ----------------------------------------- translation invariance (_verify/translation_invariance.cpp)
def spring_at(O, pin, free, gravity):
    pos = np.array([pin, free], np.float64)
    mesh = O.Mesh(positions=pos, masses=np.array([0.05, 0.05]), pinned=np.array([1, 0], np.uint8),
                  edges=np.array([[0, 1]], np.int32), edge_rest=np.array([0.1]), edge_k=np.array([1.0e4]),
                  velocities=np.zeros((2, 3)), pin_positions=pos.copy())
    return O.OracleSim(mesh, O.Config(dt=1.0 / 120.0, gravity=gravity, velocity_damping=0.0, max_iterations=40,
                                      rel_tolerance=0.0, abs_tolerance=1e-18))


@pytest.mark.parametrize("pin", [(0, 0, 0), (1, 0, 0), (0, 5, 0), (3, -2, 7)])
def test_spring_at_rest_length_without_gravity_stays_put(oracle, pin):
    """At rest length with no gravity the free end does not move (< 1e-12 over 50 substeps),
    wherever the pin is: a missing κ·q term would pull it toward the origin."""
    free = np.asarray(pin, np.float64) + [0.0, 0.0, 0.1]
    s = spring_at(oracle, pin, free, (0.0, 0.0, 0.0))
    worst = 0.0
    for _ in range(50):
        s.step(1)
        worst = max(worst, float(np.linalg.norm(s.state()[0][1] - free)))
    assert worst < 1e-12


def test_spring_motion_is_translation_invariant(oracle):
    a = spring_at(oracle, (0, 0, 0), (0, 0.12, 0), (0.0, -9.81, 0.0))
    b = spring_at(oracle, (10, 20, 30), (10, 20.12, 30), (0.0, -9.81, 0.0))
    a.step(200)
    b.step(200)
    xa, xb = a.state()[0], b.state()[0]
    assert np.linalg.norm((xa[1] - xa[0]) - (xb[1] - xb[0])) < 1e-9


def test_cloth_shape_is_translation_invariant(oracle):
    """An 8×8 cloth shifted by (5, 7, −3): after 300 substeps every edge length agrees to 1e-6."""
    runs = []
    for shift in ((0.0, 0.0, 0.0), (5.0, 7.0, -3.0)):
        m = oracle.make_grid(oracle.GridSpec(nx=8, ny=8, spacing=0.05, stiffness=1.0e4))
        m.positions = m.positions + np.asarray(shift)
        m.pin_positions = m.positions.copy()
        s = oracle.OracleSim(m, oracle.Config(dt=1.0 / 120.0, max_iterations=20, rel_tolerance=1e-8))
        s.step(300)
        x = s.state()[0]
        runs.append(np.linalg.norm(x[m.edges[:, 0]] - x[m.edges[:, 1]], axis=1))
    assert np.max(np.abs(runs[0] - runs[1]) / np.maximum(runs[0], 1e-12)) < 1e-6


# --------------------------------------------------- hanging chain (_verify/chain_test.cpp)
def chain(O, n, k, pinned, damping):
    ell, mass = 0.05, 0.005
    pos = np.zeros((n, 3))
    pos[:, 1] = np.arange(n) * ell
    pin = np.zeros(n, np.uint8)
    if pinned:
        pin[0] = 1
    edges = np.stack([np.arange(n - 1), np.arange(1, n)], axis=1).astype(np.int32)
    mesh = O.Mesh(positions=pos, masses=np.full(n, mass), pinned=pin, edges=edges, edge_rest=np.full(n - 1, ell),
                  edge_k=np.full(n - 1, k), velocities=np.zeros((n, 3)), pin_positions=pos.copy())
    return O.OracleSim(mesh, O.Config(dt=1.0 / 120.0, velocity_damping=damping, max_iterations=40,
                                      rel_tolerance=0.0, abs_tolerance=1e-16)), edges


def chain_length(x, edges):
    return float(np.sum(np.linalg.norm(x[edges[:, 0]] - x[edges[:, 1]], axis=1)))


@pytest.mark.parametrize("n", [5, 20, 100])
def test_free_chain_falls_without_stretching(oracle, n):
    s, edges = chain(oracle, n, 1.0e4, False, 0.0)
    s.step(400)
    want = (n - 1) * 0.05
    assert abs(chain_length(s.state()[0], edges) - want) / want < 1e-3


@pytest.mark.parametrize("n,k", [(5, 1e4), (5, 1e5), (20, 1e4), (20, 1e5), (100, 1e4), (100, 1e5)])
def test_pinned_chain_length_matches_the_analytic_sum(oracle, n, k):
    """The k-th segment from the free end carries k vertices' weight, so the segments change length
    by m·g·n(n − 1)/(2κ) in total. The chain starts straight above its pin along +y and nothing
    perturbs it sideways, so it stays a column standing on the pin, compressed by that amount
    rather than stretched; the reference's 5 % bound on the total length holds either way, and the
    change itself matches the analytic sum to 1e-6 after 8000 damped substeps."""
    s, edges = chain(oracle, n, k, True, 0.5)
    s.step(8000)
    length = chain_length(s.state()[0], edges)
    change = 0.005 * 9.81 * n * (n - 1) / (2.0 * k)
    assert abs(length - ((n - 1) * 0.05 + change)) / ((n - 1) * 0.05 + change) < 0.05
    assert abs(((n - 1) * 0.05 - length) - change) <= 1e-6 * change


# ------------------------------------------------ projection direction (_verify/direction_audit.cpp)
def test_projection_direction_follows_the_endpoint_order(oracle):
    """A: d lies along x_a − x_b (a at the origin, b above ⇒ −ŷ), flips when the order is swapped,
    and has length ℓ either way (the oracle's projection takes no pin flags, so no pin case can flip it)."""
    ell = 0.1
    d1 = oracle.project_one([0.0, 0.0, 0.0], [0.0, 0.15, 0.0], ell)
    d2 = oracle.project_one([0.0, 0.15, 0.0], [0.0, 0.0, 0.0], ell)
    assert abs(d1[1] + ell) < 1e-14 and abs(d2[1] - ell) < 1e-14
    assert abs(np.linalg.norm(d1) - ell) < 1e-15 and abs(np.linalg.norm(d2) - ell) < 1e-15


@pytest.mark.parametrize("y", [0.06, 0.08, 0.0999, 0.1001, 0.12, 0.15])
def test_net_elastic_term_is_the_negative_energy_gradient(oracle, y):
    """B: with the pin at the origin, the free end's row is (m/h²)·y + κ·y = (m/h²)·ŷ + scatter, so
    scatter − κ·y must equal −dU/dx = −κ(r − ℓ)·(x_free − x_pin)/r, in stretch and in compression and
    for both endpoint orders."""
    k, ell = 1.0e4, 0.1
    for free_index, pos in ((1, [[0.0, 0.0, 0.0], [0.0, y, 0.0]]), (0, [[0.0, y, 0.0], [0.0, 0.0, 0.0]])):
        pinned = [1, 0] if free_index == 1 else [0, 1]
        s = two_vertices(oracle, pos, pinned, pos, k, ell)
        b = s.rhs(np.zeros((2, 3)), overwrite_pins=False)
        xf, xp = np.asarray(pos[free_index]), np.asarray(pos[1 - free_index])
        r = np.linalg.norm(xf - xp)
        want = (xf - xp) * (-k * (r - ell) / r)
        assert abs((b[free_index] - k * xf)[1] - want[1]) <= 1e-6


def test_scatter_matches_an_independent_standard_pd(oracle):
    """C: eight arbitrary configurations: b_a = κ·d and b_b = −κ·d with d = ℓ·unit(x_a − x_b)."""
    k, ell = 1.0e4, 0.1
    for t in range(8):
        xa = np.array([0.01 * t, 0.02 + 0.03 * t, -0.015 * t])
        xb = np.array([-0.005 * t, 0.0, 0.01 * t])
        s = two_vertices(oracle, [xa, xb], [0, 0], [xa, xb], k, ell)
        b = s.rhs(np.zeros((2, 3)), overwrite_pins=False)
        raw = xa - xb
        d = raw * (ell / np.linalg.norm(raw))
        assert np.linalg.norm(b[0] - k * d) <= 1e-9 and np.linalg.norm(b[1] + k * d) <= 1e-9


# ------------------------------------------------------ bend audit (_verify/bend_audit.cpp:100-186)
def test_bend_chain_one_implicit_euler_step(oracle):
    """A three-point chain with only a bend stencil (k = 1000, unit masses, h = 1/120), ends pinned,
    the middle raised to ŷ = 0.03: pinned rows are exact identity rows (A0), and the solve gives
    y = ŷ·(m/h²)/(m/h² + 4k) = 0.03·14400/18400 to 1e-12 (A2) with ‖Lx − b‖∞/max(1, ‖b‖∞) < 1e-12 (B)."""
    k, h, spacing, eps = 1000.0, 1.0 / 120.0, 0.1, 0.03
    pos = np.array([[0.0, 0.0, 0.0], [spacing, eps, 0.0], [2 * spacing, 0.0, 0.0]])
    mesh = oracle.Mesh(positions=pos, masses=np.ones(3), pinned=np.array([1, 0, 1], np.uint8),
                       edges=np.zeros((0, 2), np.int32), edge_rest=np.zeros(0), edge_k=np.zeros(0),
                       bends=np.array([[0, 1, 2]], np.int32), bend_k=np.array([k]), pin_positions=pos.copy())
    s = oracle.OracleSim(mesh, oracle.Config(dt=h, gravity=(0.0, 0.0, 0.0)))
    rp, ci, val = s.matrix()
    A = np.zeros((3, 3))
    for r in range(3):
        A[r, ci[rp[r]:rp[r + 1]]] = val[rp[r]:rp[r + 1]]
    for v in (0, 2):
        assert A[v, v] == 1.0 and np.count_nonzero(A[v]) == 1 and A[1, v] == 0.0
    assert A[1, 1] == 1.0 / (h * h) + 4.0 * k
    b = s.rhs(pos / (h * h), overwrite_pins=True)
    x = s.solve(b)
    assert abs(x[1, 1] - 0.03 * (14400.0 / (14400.0 + 4.0 * k))) < 1e-12
    assert np.max(np.abs(A @ x - b)) / max(1.0, np.max(np.abs(b))) < 1e-12


# ------------------------------------------ projection definition (test_distance_term.cpp:44-99)
def test_projection_is_collinear_forward_exact_at_rest_and_zero_when_degenerate(oracle):
    a, b = np.array([0.1, -0.2, 0.3]), np.array([-0.4, 0.5, -0.6])
    d = oracle.project_one(a, b, 0.25)
    raw = a - b
    assert abs(float(raw @ d) / (np.linalg.norm(raw) * np.linalg.norm(d)) - 1.0) <= 1e-14
    # at rest length the projection is the edge vector itself, component for component
    a, b = np.array([1.0, 0.0, 0.0]), np.array([0.63, 0.0, 0.0])
    assert np.array_equal(oracle.project_one(a, b, 0.37), a - b)
    # a degenerate edge has no direction: the projection is the zero vector
    p = np.array([1.0, 2.0, 3.0])
    assert not np.any(oracle.project_one(p, p, 0.1))


def test_projection_energy_gradient_matches_finite_differences(oracle):
    """E = κ/2·(r − ℓ)² has ∂E/∂x_a = κ(r − ℓ)·(x_a − x_b)/r = κ·((x_a − x_b) − d): the projection
    d is the point the gradient pulls toward."""
    k, rest = 1234.0, 0.2
    pa, pb = np.array([0.1, 0.3, -0.2]), np.array([-0.4, 0.25, 0.35])

    def energy(a):
        return 0.5 * k * (np.linalg.norm(a - pb) - rest) ** 2

    grad = k * ((pa - pb) - oracle.project_one(pa, pb, rest))
    for c in range(3):
        e = np.zeros(3)
        e[c] = 1e-7
        fd = (energy(pa + e) - energy(pa - e)) / 2e-7
        assert abs(grad[c] - fd) <= 1e-6 * abs(fd) + 1e-9


# ------------------------------------- refactorization stamp (test_distance_term.cpp:293-330)
def test_only_left_hand_side_changes_refactorize(oracle):
    """Pin drags and damping leave Ã alone (no refactorization); stiffness and dt changes refactorize."""
    pos = np.array([[0.0, 0.0, 0.0], [0.4, 0.1, 0.0]])
    mesh = oracle.Mesh(positions=pos, masses=np.array([0.1, 0.1]), pinned=np.array([1, 0], np.uint8),
                       edges=np.array([[0, 1]], np.int32), edge_rest=np.array([0.1]), edge_k=np.array([400.0]),
                       pin_positions=pos.copy())
    cfg = oracle.Config(dt=1.0 / 120.0)
    s = oracle.OracleSim(mesh, cfg)
    s.step(1)
    count = s.stats()["factorize_count"]
    s.set_pin_positions(np.array([[0.7, -0.3, 2.0], [0.4, 0.1, 0.0]]))
    s.step(1)
    s.set_config(oracle.Config(dt=1.0 / 120.0, velocity_damping=0.35))
    s.step(1)
    assert s.stats()["factorize_count"] == count
    s.set_edge_stiffness(np.array([401.0]))
    s.step(1)
    assert s.stats()["factorize_count"] == count + 1
    s.set_config(oracle.Config(dt=1.0 / 240.0, velocity_damping=0.35))
    s.step(1)
    assert s.stats()["factorize_count"] == count + 2


# ------------------------------------------ grid construction (test_distance_term.cpp:769-935)
def test_shear_diagonals_are_added_once(oracle):
    nx = ny = 20
    base = oracle.make_grid(oracle.GridSpec(nx=nx, ny=ny, spacing=0.05))
    sheared = oracle.make_grid(oracle.GridSpec(nx=nx, ny=ny, spacing=0.05, shear_stiffness=1.0e3))
    assert base.edges.shape[0] == 2 * nx * ny - nx - ny
    assert sheared.edges.shape[0] == base.edges.shape[0] + (nx - 1) * (ny - 1)
    pairs = {tuple(sorted(map(int, e))) for e in sheared.edges}
    assert len(pairs) == sheared.edges.shape[0]
    assert np.array_equal(sheared.edges[:base.edges.shape[0]], base.edges)


def test_bend_stencils_have_the_exact_vertex_triples(oracle):
    """Rows first (centre i = 1..nx−2 of every row j, in order), then columns (centre j = 1..ny−2
    of every column i); every stencil carries the given stiffness; none without a grid bend knob."""
    nx, ny, k = 20, 14, 777.0
    assert oracle.make_grid(oracle.GridSpec(nx=nx, ny=ny, spacing=0.05)).bends.shape[0] == 0
    m = oracle.make_grid(oracle.GridSpec(nx=nx, ny=ny, spacing=0.05, bend_stiffness=k))
    rows = [(j * nx + i - 1, j * nx + i, j * nx + i + 1) for j in range(ny) for i in range(1, nx - 1)]
    cols = [((j - 1) * nx + i, j * nx + i, (j + 1) * nx + i) for i in range(nx) for j in range(1, ny - 1)]
    assert m.bends.shape[0] == (nx - 2) * ny + (ny - 2) * nx
    assert [tuple(map(int, b)) for b in m.bends] == rows + cols
    assert np.all(m.bend_k == k)


def test_strided_bend_sampling_cannot_see_coarse_bending(oracle):
    """Stride 2 on a 9×2 grid keeps only the odd row centres (8 stencils); putting every odd vertex
    at the midpoint of its even neighbours zeroes every sampled A_s·x exactly, however strongly the
    even sub-grid bends (test_distance_term.cpp:1274-1330): the counterexample for which the
    reference rejects strided sampling."""
    nx, ny = 9, 2
    m = oracle.make_grid(oracle.GridSpec(nx=nx, ny=ny, spacing=1.0, bend_stiffness=1000.0, bend_stride=2,
                                         pin_mode=4))
    assert m.bends.shape[0] == 8 and all((int(b[1]) % nx) % 2 == 1 for b in m.bends)
    even = np.array([0.0, 1.0, 4.0, 9.0, 16.0])
    y = np.zeros(nx)
    y[0::2] = even
    y[1::2] = 0.5 * (even[:-1] + even[1:])
    x = m.positions.copy()
    for j in range(ny):
        x[j * nx:(j + 1) * nx, 1] = y
    second = x[m.bends[:, 0]] - 2.0 * x[m.bends[:, 1]] + x[m.bends[:, 2]]
    assert not np.any(second)
    assert np.all(even[:-2] - 2.0 * even[1:-1] + even[2:] == 2.0)  # the even sub-grid bends throughout


# ------------------------------------------------------ spring fixed points (spring_vertical.cpp)
def test_iteration_count_does_not_change_the_fixed_point(oracle):
    """One spring: the projection is −ℓŷ whatever x is and the matrix already holds κ, so one
    iteration lands on the fixed point: 1, 5 and 50 iterations agree to 1e-15·ℓ and match the
    closed form to 1e-12 (spring_vertical.cpp:130-152)."""
    from tests.test_oracle import ELL, H, K, M, closed_form, spring
    ys = []
    for iters in (1, 5, 50):
        s = spring(oracle, 0.12, iters=iters)
        s.step(1)
        ys.append(s.state()[0][1, 1])
    assert abs(ys[2] - closed_form(0.12 - H * H * 9.81, M, K, H)) / ELL <= 1e-12
    assert abs(ys[1] - ys[2]) / ELL <= 1e-15 and abs(ys[0] - ys[2]) / ELL <= 1e-15


@pytest.mark.parametrize("h", [1.0 / 240.0, 1.0 / 480.0, 1.0 / 960.0])
def test_damped_spring_settles_at_the_energy_minimum(oracle, h):
    """E(y) = κ/2·(y − ℓ)² + m·g·y is least at y = ℓ − m·g/κ, below the rest length, for every h
    (spring_vertical.cpp:231-252; κ = 20, damping 0.5, 40 s)."""
    from tests.test_oracle import ELL, M, spring
    k = 20.0
    s = spring(oracle, 0.12, kd=0.5, k=k, h=h)
    s.step(int(40.0 / h))
    assert abs(s.state()[0][1, 1] - (ELL - M * 9.81 / k)) / ELL <= 1e-3


def test_free_chain_iterates_to_rest_lengths_without_gravity(oracle):
    """Twelve unpinned vertices on a slanted line, spaced wider than ℓ, one PD iteration a substep,
    no gravity, damping or early exit: the substep change falls to 1e-12 and every edge returns to
    its rest length to 1e-9 (spring_vertical.cpp:442-512)."""
    n, ell, k = 12, 0.1, 1.0e3
    pos = np.array([[0.03 * i, 0.11 * i, 0.0] for i in range(n)])
    edges = np.stack([np.arange(n - 1), np.arange(1, n)], axis=1).astype(np.int32)
    mesh = oracle.Mesh(positions=pos, masses=np.full(n, 0.05), pinned=np.zeros(n, np.uint8), edges=edges,
                       edge_rest=np.full(n - 1, ell), edge_k=np.full(n - 1, k), velocities=np.zeros((n, 3)),
                       pin_positions=pos.copy())
    s = oracle.OracleSim(mesh, oracle.Config(dt=1.0 / 120.0, gravity=(0.0, 0.0, 0.0), velocity_damping=0.0,
                                             max_iterations=1, rel_tolerance=0.0, abs_tolerance=0.0))
    x = pos
    for _ in range(50000):
        s.step(1)
        nxt = s.state()[0]
        change = float(np.max(np.abs(nxt - x)))
        x = nxt
        if change <= 1e-12:
            break
    assert change <= 1e-12
    lengths = np.linalg.norm(x[edges[:, 0]] - x[edges[:, 1]], axis=1)
    assert np.max(np.abs(lengths - ell)) / ell < 1e-9
    assert abs(lengths.sum() - (n - 1) * ell) <= 1e-9
