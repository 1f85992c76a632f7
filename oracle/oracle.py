"""ctypes wrapper around the CPU oracle (``oracle/pd_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: the oracle is the checker for the CUDA path. Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline / reference arm may import this
module. The product package (``pd_gb300``) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libpd_oracle.so")
_lib = None


def build() -> str:
    """Compiles the oracle with its Makefile (no reference sources are used)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class _Config(C.Structure):
    _fields_ = [
        ("dt", C.c_double),
        ("gravity", C.c_double * 3),
        ("velocity_damping", C.c_double),
        ("max_iterations", C.c_int),
        ("rel_tolerance", C.c_double),
        ("abs_tolerance", C.c_double),
        ("residual_tolerance", C.c_double),
        ("threads", C.c_int),
        ("cheb_mode", C.c_int),
        ("cheb_rho", C.c_double),
        ("cheb_start", C.c_int),
        ("cheb_m", C.c_double),
        ("cheb_d", C.c_double),
    ]


class _GridSpec(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("spacing", C.c_double), ("stiffness", C.c_double),
        ("density", C.c_double), ("shear_stiffness", C.c_double), ("bend_stiffness", C.c_double),
        ("bend_sampling", C.c_int), ("bend_stride", C.c_int), ("mass_mode", C.c_int),
        ("total_mass", C.c_double), ("pin_mode", C.c_int),
    ]


class _Stats(C.Structure):
    _fields_ = [
        ("last_residual", C.c_double), ("iterations_used", C.c_int), ("converged", C.c_int),
        ("early_exit_count", C.c_int), ("factorize_count", C.c_int), ("analyze_count", C.c_int),
        ("color_count", C.c_int), ("matrix_nnz", C.c_int64), ("factor_nnz", C.c_int64),
        ("max_strain", C.c_double), ("mean_strain", C.c_double), ("elastic_energy", C.c_double),
        ("total_energy", C.c_double), ("max_speed", C.c_double),
    ]


def _P(t):
    return C.POINTER(t)


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        build()
    L = C.CDLL(_LIB_PATH)
    dp, ip, u8p, u32p = _P(C.c_double), _P(C.c_int32), _P(C.c_uint8), _P(C.c_uint32)
    L.oracle_grid_counts.argtypes = [_P(_GridSpec), _P(C.c_int), _P(C.c_int), _P(C.c_int)]
    L.oracle_make_grid.argtypes = [_P(_GridSpec), dp, dp, u8p, ip, dp, dp, ip, dp]
    L.oracle_make_grid.restype = C.c_int
    L.oracle_sim_step_traced.argtypes = [C.c_void_p, C.c_int, dp]
    L.oracle_sim_step_traced.restype = C.c_int
    L.oracle_obj_counts.argtypes = [C.c_char_p, _P(C.c_int), _P(C.c_int)]
    L.oracle_obj_counts.restype = C.c_int
    L.oracle_make_obj.argtypes = [C.c_char_p, C.c_double, C.c_double, dp, dp, u8p, ip, dp, dp]
    L.oracle_make_obj.restype = C.c_int
    L.oracle_sim_create.argtypes = [C.c_int, dp, dp, dp, u8p, dp, C.c_int, ip, dp, dp, C.c_int, ip, dp,
                                    _P(_Config), ip]
    L.oracle_sim_create.restype = C.c_void_p
    L.oracle_sim_destroy.argtypes = [C.c_void_p]
    L.oracle_sim_step.argtypes = [C.c_void_p, C.c_int, ip, u8p]
    L.oracle_sim_step.restype = C.c_int
    L.oracle_sim_get_state.argtypes = [C.c_void_p, dp, dp]
    L.oracle_sim_set_state.argtypes = [C.c_void_p, dp, dp]
    L.oracle_sim_set_pin_positions.argtypes = [C.c_void_p, dp]
    L.oracle_sim_set_config.argtypes = [C.c_void_p, _P(_Config)]
    L.oracle_sim_set_edge_stiffness.argtypes = [C.c_void_p, dp]
    L.oracle_sim_stats.argtypes = [C.c_void_p, _P(_Stats)]
    L.oracle_sim_nonlinear_residual.argtypes = [C.c_void_p]
    L.oracle_sim_nonlinear_residual.restype = C.c_double
    L.oracle_sim_factor.argtypes = [C.c_void_p, ip, ip, ip, dp, dp]
    L.oracle_sim_factor.restype = C.c_int64
    L.oracle_sim_matrix.argtypes = [C.c_void_p, ip, ip, dp]
    L.oracle_sim_matrix.restype = C.c_int64
    L.oracle_sim_solve.argtypes = [C.c_void_p, dp, dp]
    L.oracle_sim_solve.restype = C.c_int
    L.oracle_sim_rhs.argtypes = [C.c_void_p, dp, dp, C.c_int]
    L.oracle_sim_rhs.restype = C.c_int
    L.oracle_sim_coloring.argtypes = [C.c_void_p, u32p, u32p, u32p, u32p, u32p]
    L.oracle_sim_coloring.restype = C.c_int
    L.oracle_sim_bend_rhs.argtypes = [C.c_void_p, dp]
    L.oracle_project_one.argtypes = [dp, dp, C.c_double, dp]
    L.oracle_sim_gradient.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp, dp, dp]
    L.oracle_sim_gradient.restype = C.c_int
    L.oracle_sim_spectrum.argtypes = [C.c_void_p, C.c_int, dp]
    L.oracle_sim_spectrum.restype = C.c_int
    _lib = L
    return L


def _ptr(a, t):
    if a is None:
        return None
    return a.ctypes.data_as(_P(t))


@dataclass
class Config:
    """Mirror of the reference ``SceneConfig`` knobs used by ``stepOnce`` (core/sim/Scene.h:14-137)."""
    dt: float = 1.0 / 120.0
    gravity: tuple = (0.0, -9.81, 0.0)
    velocity_damping: float = 0.02
    max_iterations: int = 10
    rel_tolerance: float = 1.0e-3
    abs_tolerance: float = 1.0e-12
    residual_tolerance: float = 1.0e-3
    threads: int = 0
    cheb_mode: int = 0        # 0 off, 1 ρ recurrence (PD_CHEB=1), 2 roots over [m−δ, m+δ] (interval)
    cheb_rho: float = 0.98
    cheb_start: int = 10
    cheb_m: float = 1.0
    cheb_d: float = 1.0

    def c(self):
        c = _Config()
        c.dt = self.dt
        for i in range(3):
            c.gravity[i] = self.gravity[i]
        c.velocity_damping = self.velocity_damping
        c.max_iterations = self.max_iterations
        c.rel_tolerance = self.rel_tolerance
        c.abs_tolerance = self.abs_tolerance
        c.residual_tolerance = self.residual_tolerance
        c.threads = self.threads
        c.cheb_mode = self.cheb_mode
        c.cheb_rho = self.cheb_rho
        c.cheb_start = self.cheb_start
        c.cheb_m = self.cheb_m
        c.cheb_d = self.cheb_d
        return c


@dataclass
class GridSpec:
    """Regular grid scene (reference ``makeScene`` on a grid, core/sim/Scene.cpp:39-177)."""
    nx: int = 40
    ny: int = 40
    spacing: float = 0.025
    stiffness: float = 2.3e3
    density: float = 1.0
    shear_stiffness: float = 0.0
    bend_stiffness: float = 0.0
    bend_sampling: int = 0
    bend_stride: int = 1
    mass_mode: int = 0       # 0 edge-lumped (reference), 1 uniform total_mass
    total_mass: float = 1.0
    pin_mode: int = 0        # 0 corners of row ny-1, 1 corners of row 0, 2 row ny-1, 3 one corner, 4 none


@dataclass
class Mesh:
    positions: np.ndarray
    masses: np.ndarray
    pinned: np.ndarray
    edges: np.ndarray
    edge_rest: np.ndarray
    edge_k: np.ndarray
    bends: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    bend_k: np.ndarray = field(default_factory=lambda: np.zeros(0))
    velocities: np.ndarray | None = None
    pin_positions: np.ndarray | None = None

    @property
    def n(self):
        return int(self.positions.shape[0])


def make_grid(spec: GridSpec) -> Mesh:
    L = lib()
    g = _GridSpec(spec.nx, spec.ny, spec.spacing, spec.stiffness, spec.density, spec.shear_stiffness,
                  spec.bend_stiffness, spec.bend_sampling, spec.bend_stride, spec.mass_mode,
                  spec.total_mass, spec.pin_mode)
    nv, ne, nb = C.c_int(), C.c_int(), C.c_int()
    L.oracle_grid_counts(C.byref(g), C.byref(nv), C.byref(ne), C.byref(nb))
    nv, ne, nb = nv.value, ne.value, nb.value
    pos = np.zeros((nv, 3))
    mass = np.zeros(nv)
    pinned = np.zeros(nv, np.uint8)
    eab = np.zeros((ne, 2), np.int32)
    er = np.zeros(ne)
    ek = np.zeros(ne)
    babc = np.zeros((max(nb, 0), 3), np.int32)
    bk = np.zeros(max(nb, 0))
    rc = L.oracle_make_grid(C.byref(g), _ptr(pos, C.c_double), _ptr(mass, C.c_double),
                            _ptr(pinned, C.c_uint8), _ptr(eab, C.c_int32), _ptr(er, C.c_double),
                            _ptr(ek, C.c_double), _ptr(babc, C.c_int32), _ptr(bk, C.c_double))
    if rc != 0:
        raise ValueError("invalid grid spec")
    return Mesh(pos, mass, pinned, eab, er, ek, babc, bk)


def make_obj(text: str, stiffness: float = 2.3e3, density: float = 1.0) -> Mesh:
    """The OBJ triangle mesh of ``makeScene`` (Mesh::loadObj + surface masses)."""
    L = lib()
    raw = text.encode()
    nv, ne = C.c_int(), C.c_int()
    if L.oracle_obj_counts(raw, C.byref(nv), C.byref(ne)) != 0:
        raise ValueError("OBJ text the reference cannot load")
    nv, ne = nv.value, ne.value
    pos = np.zeros((nv, 3))
    mass = np.zeros(nv)
    pinned = np.zeros(nv, np.uint8)
    eab = np.zeros((ne, 2), np.int32)
    er = np.zeros(ne)
    ek = np.zeros(ne)
    L.oracle_make_obj(raw, stiffness, density, _ptr(pos, C.c_double), _ptr(mass, C.c_double),
                      _ptr(pinned, C.c_uint8), _ptr(eab, C.c_int32), _ptr(er, C.c_double), _ptr(ek, C.c_double))
    return Mesh(pos, mass, pinned, eab, er, ek)


class OracleSim:
    """A ``SimContext`` restated on the CPU; ``step`` runs the reference ``stepOnce``."""

    def __init__(self, mesh: Mesh, cfg: Config, perm=None):
        self._L = lib()
        self.n = mesh.n
        self.cfg = cfg
        pos = np.ascontiguousarray(mesh.positions, np.float64)
        vel = None if mesh.velocities is None else np.ascontiguousarray(mesh.velocities, np.float64)
        q = None if mesh.pin_positions is None else np.ascontiguousarray(mesh.pin_positions, np.float64)
        self._keep = [pos, vel, q]
        ccfg = cfg.c()
        p = None if perm is None else np.ascontiguousarray(perm, np.int32)
        self._h = self._L.oracle_sim_create(
            self.n, _ptr(pos, C.c_double), _ptr(vel, C.c_double),
            _ptr(np.ascontiguousarray(mesh.masses, np.float64), C.c_double),
            _ptr(np.ascontiguousarray(mesh.pinned, np.uint8), C.c_uint8), _ptr(q, C.c_double),
            int(mesh.edges.shape[0]), _ptr(np.ascontiguousarray(mesh.edges, np.int32), C.c_int32),
            _ptr(np.ascontiguousarray(mesh.edge_rest, np.float64), C.c_double),
            _ptr(np.ascontiguousarray(mesh.edge_k, np.float64), C.c_double),
            int(mesh.bends.shape[0]), _ptr(np.ascontiguousarray(mesh.bends, np.int32), C.c_int32),
            _ptr(np.ascontiguousarray(mesh.bend_k, np.float64), C.c_double), C.byref(ccfg),
            _ptr(p, C.c_int32))
        if not self._h:
            raise ValueError("oracle_sim_create rejected the scene")
        self.n_edges = int(mesh.edges.shape[0])

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.oracle_sim_destroy(h)
            self._h = None

    def step(self, substeps=1):
        it = np.zeros(substeps, np.int32)
        cv = np.zeros(substeps, np.uint8)
        rc = self._L.oracle_sim_step(self._h, substeps, _ptr(it, C.c_int32), _ptr(cv, C.c_uint8))
        if rc != 0:
            raise RuntimeError("oracle factorization failed")
        return it, cv

    def step_traced(self, substeps):
        """Steps, returning the gate residual after every iteration: (substeps, K) with NaN past
        each substep's last iteration."""
        K = max(1, self.cfg.max_iterations)
        out = np.zeros((substeps, K))
        if self._L.oracle_sim_step_traced(self._h, substeps, _ptr(out, C.c_double)) != 0:
            raise RuntimeError("oracle step failed")
        return out

    def state(self):
        x = np.zeros((self.n, 3))
        v = np.zeros((self.n, 3))
        self._L.oracle_sim_get_state(self._h, _ptr(x, C.c_double), _ptr(v, C.c_double))
        return x, v

    def set_state(self, x=None, v=None):
        xs = None if x is None else np.ascontiguousarray(x, np.float64)
        vs = None if v is None else np.ascontiguousarray(v, np.float64)
        self._L.oracle_sim_set_state(self._h, _ptr(xs, C.c_double), _ptr(vs, C.c_double))

    def set_pin_positions(self, q):
        q = np.ascontiguousarray(q, np.float64)
        self._L.oracle_sim_set_pin_positions(self._h, _ptr(q, C.c_double))

    def set_config(self, cfg: Config):
        self.cfg = cfg
        c = cfg.c()
        self._L.oracle_sim_set_config(self._h, C.byref(c))

    def set_edge_stiffness(self, k):
        k = np.ascontiguousarray(k, np.float64)
        self._L.oracle_sim_set_edge_stiffness(self._h, _ptr(k, C.c_double))

    def stats(self) -> dict:
        s = _Stats()
        self._L.oracle_sim_stats(self._h, C.byref(s))
        return {f: getattr(s, f) for f, _ in _Stats._fields_}

    def nonlinear_residual(self):
        return self._L.oracle_sim_nonlinear_residual(self._h)

    def factor(self):
        nnz = self._L.oracle_sim_factor(self._h, None, None, None, None, None)
        perm = np.zeros(self.n, np.int32)
        cp = np.zeros(self.n + 1, np.int32)
        ri = np.zeros(nnz, np.int32)
        val = np.zeros(nnz)
        dinv = np.zeros(self.n)
        self._L.oracle_sim_factor(self._h, _ptr(perm, C.c_int32), _ptr(cp, C.c_int32),
                                  _ptr(ri, C.c_int32), _ptr(val, C.c_double), _ptr(dinv, C.c_double))
        return dict(perm=perm, colptr=cp, rowidx=ri, val=val, dinv=dinv)

    def matrix(self):
        nnz = self._L.oracle_sim_matrix(self._h, None, None, None)
        rp = np.zeros(self.n + 1, np.int32)
        ci = np.zeros(nnz, np.int32)
        val = np.zeros(nnz)
        self._L.oracle_sim_matrix(self._h, _ptr(rp, C.c_int32), _ptr(ci, C.c_int32), _ptr(val, C.c_double))
        return rp, ci, val

    def solve(self, b):
        b = np.ascontiguousarray(b, np.float64).reshape(-1)
        x = np.zeros_like(b)
        if self._L.oracle_sim_solve(self._h, _ptr(b, C.c_double), _ptr(x, C.c_double)) != 0:
            raise RuntimeError("factorization failed")
        return x.reshape(-1, 3)

    def gradient(self, substeps, targets, force=None, grad=True):
        """Loss (mean over free vertices of |x − target|² after `substeps` substeps with the
        iteration count fixed) and, if `grad`, its gradient w.r.t. per-edge stiffness, initial
        velocities and an external per-vertex force; the state is left unchanged."""
        t = np.ascontiguousarray(targets, np.float64).reshape(-1)
        f = None if force is None else np.ascontiguousarray(force, np.float64).reshape(-1)
        loss = C.c_double()
        dk = np.zeros(self.n_edges) if grad else None
        dv = np.zeros((self.n, 3)) if grad else None
        df = np.zeros((self.n, 3)) if grad else None
        rc = self._L.oracle_sim_gradient(self._h, int(substeps), _ptr(t, C.c_double), _ptr(f, C.c_double),
                                         C.byref(loss), _ptr(dk, C.c_double), _ptr(dv, C.c_double),
                                         _ptr(df, C.c_double))
        if rc != 0:
            raise RuntimeError("oracle gradient failed")
        return dict(loss=loss.value, dkappa=dk, dv0=dv, dforce=df)

    def spectrum(self, iters=400):
        """Power-iteration estimates at the current positions: rho_plain (ρ(T)) and lambda_max
        (λ_max(B)) with the estimates one iteration earlier (iteration_spectrum.cpp)."""
        out = np.zeros(4)
        if self._L.oracle_sim_spectrum(self._h, int(iters), _ptr(out, C.c_double)) != 0:
            raise RuntimeError("factorization failed")
        return dict(rho_plain=out[0], rho_plain_prev=out[1], lambda_max=out[2], lambda_max_prev=out[3])

    def rhs(self, base, overwrite_pins=True):
        base = np.ascontiguousarray(base, np.float64).reshape(-1)
        b = np.zeros_like(base)
        self._L.oracle_sim_rhs(self._h, _ptr(base, C.c_double), _ptr(b, C.c_double), int(overwrite_pins))
        return b.reshape(-1, 3)

    def coloring(self):
        cc = self._L.oracle_sim_coloring(self._h, None, None, None, None, None)
        color_of = np.zeros(self.n_edges, np.uint32)
        start = np.zeros(cc + 1, np.uint32)
        order = np.zeros(self.n_edges, np.uint32)
        vstart = np.zeros(self.n + 1, np.uint32)
        vedges = np.zeros(2 * self.n_edges, np.uint32)
        self._L.oracle_sim_coloring(self._h, _ptr(color_of, C.c_uint32), _ptr(start, C.c_uint32),
                                    _ptr(order, C.c_uint32), _ptr(vstart, C.c_uint32), _ptr(vedges, C.c_uint32))
        return dict(count=cc, color_of=color_of, start=start, order=order, vstart=vstart, vedges=vedges)

    def bend_rhs(self):
        out = np.zeros(3 * self.n)
        self._L.oracle_sim_bend_rhs(self._h, _ptr(out, C.c_double))
        return out.reshape(-1, 3)


def project_one(pa, pb, rest):
    out = np.zeros(3)
    a = np.ascontiguousarray(pa, np.float64)
    b = np.ascontiguousarray(pb, np.float64)
    lib().oracle_project_one(_ptr(a, C.c_double), _ptr(b, C.c_double), float(rest), _ptr(out, C.c_double))
    return out
