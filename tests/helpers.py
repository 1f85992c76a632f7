"""Shared helpers: build the oracle twin of a GPU scene (same arrays, same elimination order)."""
import numpy as np

from oracle import oracle as O


def oracle_config(cfg, threads=0):
    return O.Config(dt=cfg.dt, gravity=tuple(cfg.gravity), velocity_damping=cfg.velocity_damping,
                    max_iterations=cfg.max_iterations, rel_tolerance=cfg.rel_tolerance,
                    abs_tolerance=cfg.abs_tolerance, residual_tolerance=cfg.residual_tolerance,
                    threads=threads, cheb_mode=cfg.cheb_mode, cheb_rho=cfg.cheb_rho,
                    cheb_start=cfg.cheb_start, cheb_m=cfg.cheb_m, cheb_d=cfg.cheb_d)


def oracle_twin(scene, cfg, perm=None, threads=0):
    mesh = O.Mesh(positions=np.asarray(scene.positions, np.float64), masses=scene.masses,
                  pinned=scene.pinned, edges=np.asarray(scene.edges, np.int32).reshape(-1, 2),
                  edge_rest=scene.edge_rest, edge_k=scene.edge_stiffness,
                  bends=np.asarray(scene.bends, np.int32).reshape(-1, 3), bend_k=scene.bend_stiffness,
                  velocities=scene.velocities, pin_positions=scene.pin_positions)
    return O.OracleSim(mesh, oracle_config(cfg, threads), perm=perm)


def bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def max_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)


def obj_sheet(nx=9, ny=7, seed=0, curved=True):
    """OBJ text of a triangulated nx×ny sheet (two triangles per quad, alternating diagonals),
    vertices listed in a seeded random order and faces written in mixed token styles."""
    rng = np.random.default_rng(seed)
    order = rng.permutation(nx * ny)          # file position of grid vertex g
    inv = np.empty_like(order)
    inv[order] = np.arange(nx * ny)
    lines = ["# sheet", "o sheet"]
    for p in range(nx * ny):
        g = int(inv[p])
        i, j = g % nx, g // nx
        x, y = i / (nx - 1), j / (ny - 1)
        z = 0.08 * np.sin(3.0 * x) * np.cos(2.0 * y) if curved else 0.0
        lines.append(f"v {x:.9f} {z:.9f} {y:.9f}")
    styles = ["{}", "{}/{}", "{}/{}/{}", "{}//{}"]
    f = 0
    for j in range(ny - 1):
        for i in range(nx - 1):
            a, b, c, d = j * nx + i, j * nx + i + 1, (j + 1) * nx + i + 1, (j + 1) * nx + i
            tris = [(a, b, c), (a, c, d)] if (i + j) % 2 == 0 else [(a, b, d), (b, c, d)]
            for t in tris:
                st = styles[f % 4]
                f += 1
                lines.append("f " + " ".join(st.format(*([int(order[v]) + 1] * st.count("{}"))) for v in t))
    return "\n".join(lines) + "\n"
