"""ctypes bindings of ``include/pd_gb300.h`` and a thin Python mirror of the reference surface.

Mirrors, by name and argument meaning:
  * ``SceneConfig``        — core/sim/Scene.h:14-137
  * ``make_grid``          — Mesh::makeGrid + makeScene (core/mesh/Mesh.cpp:12-54, core/sim/Scene.cpp:39-177)
  * ``Simulator.step_once``— stepOnce (core/sim/Integrator.cpp:312-797), on the GPU
  * ``GpuDirectSolver``    — IGlobalSolver / EigenDirectSolver (core/solver/IGlobalSolver.h:45-127)
Every call raises ``PdError`` carrying the library's status code and message on failure.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field, fields

import numpy as np

PD_OK = 0
PD_ERR_INVALID_ARGUMENT = 1       # PdError.code values (PD_ERR_* in include/pd_gb300.h)
PD_ERR_STATE = 2
PD_ERR_FACTORIZATION = 3
PD_ERR_CUDA = 4
PD_ERR_UNSUPPORTED = 5
PD_ERR_NO_MEMORY = 6
PD_PRECISION_FP64_EXACT = 0       # FP64 in the reference's operation order (bit-identical)
PD_PRECISION_FP64 = 1             # FP64, supernodal solve (matches to rounding)
PD_PRECISION_FP32_PROJECTION = 2  # FP32 projection, FP64 supernodal solve
PD_PRECISION_FP32_SOLVE = 3       # FP32 solve + one FP64 refinement step
PD_PRECISION_MIXED = 4            # FP32 projection + FP32 solve + FP64 refinement
PD_SOLVE_LEVELS = 0               # solve kinds reported by Simulator.info()["solve_kind"]
PD_SOLVE_SUPERNODAL = 1
PD_SOLVE_SUPERNODAL32 = 2
PD_SOLVE_DENSE32 = 3
PD_SOLVE_DENSE32_TEAM = 4
PD_SOLVE_SUPERNODAL32_CORRECTION = 5
PD_SOLVE_DENSE64_TEAM = 6         # FP64 team kernel: explicit inverse in double-float arithmetic
PD_HOST_STATE_NONE = 0            # Simulator.info()["host_state"]: no host arrays bound
PD_HOST_STATE_COPIES = 1          # step_host copies each pageable array with its own copy
PD_HOST_STATE_GRAPH = 2           # step_host: gather/scatter kernels in one CUDA graph
PD_CHEB_OFF = 0                   # SceneConfig.cheb_mode: plain PD iterations
PD_CHEB_RHO = 1                   # ω recurrence from ρ after cheb_start plain iterations (PD_CHEB=1)
PD_CHEB_INTERVAL = 2              # Chebyshev roots over [m − δ, m + δ] (PD_CHEB_MODE=interval)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libpd_gb300.so")


class PdError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"pd_gb300 error {code}: {message}")
        self.code = code


class _Cfg(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("substeps_per_frame", C.c_int32), ("gravity", C.c_double * 3),
        ("stiffness", C.c_double), ("density", C.c_double), ("velocity_damping", C.c_double),
        ("max_iterations", C.c_int32), ("rel_tolerance", C.c_double), ("abs_tolerance", C.c_double),
        ("residual_tolerance", C.c_double), ("grid_nx", C.c_int32), ("grid_ny", C.c_int32),
        ("grid_spacing", C.c_double), ("shear_stiffness", C.c_double), ("bend_stiffness", C.c_double),
        ("bend_sampling", C.c_int32), ("bend_stride", C.c_int32), ("mass_mode", C.c_int32),
        ("total_mass", C.c_double), ("pin_mode", C.c_int32), ("precision", C.c_int32),
        ("cluster_ctas", C.c_int32), ("dense_max_vertices", C.c_int32),
        ("cheb_mode", C.c_int32), ("cheb_rho", C.c_double), ("cheb_start", C.c_int32),
        ("cheb_m", C.c_double), ("cheb_d", C.c_double),
    ]


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)


class _Mesh(C.Structure):
    _fields_ = [
        ("n_vertices", C.c_int32), ("positions", _dp), ("velocities", _dp), ("masses", _dp),
        ("pinned", _u8p), ("pin_positions", _dp), ("n_edges", C.c_int32), ("edges", _ip),
        ("edge_rest", _dp), ("edge_stiffness", _dp), ("n_bends", C.c_int32), ("bends", _ip),
        ("bend_stiffness", _dp),
    ]


class _SimInfo(C.Structure):
    _fields_ = [
        ("n_vertices", C.c_int32), ("n_edges", C.c_int32), ("n_bends", C.c_int32),
        ("color_count", C.c_int32), ("matrix_nnz", C.c_int64), ("factor_nnz", C.c_int64),
        ("forward_levels", C.c_int32), ("backward_levels", C.c_int32),
        ("factorize_count", C.c_int32), ("analyze_count", C.c_int32), ("device_bytes", C.c_int64),
        ("cluster_ctas", C.c_int32), ("solve_kind", C.c_int32), ("host_state", C.c_int32),
        ("device_factorize_count", C.c_int32),
    ]


class _Plan(C.Structure):
    _fields_ = [("team_ctas", C.c_int32), ("big_min_vertices", C.c_int32), ("big_cluster_ctas", C.c_int32),
                ("work_threads", C.c_int32), ("latency_scale", C.c_double)]


PD_TUNE_MAX_CANDIDATES = 32


class _Spectrum(C.Structure):
    _fields_ = [("rho_plain", C.c_double), ("rho_plain_prev", C.c_double), ("lambda_max", C.c_double),
                ("lambda_max_prev", C.c_double), ("lambda_min", C.c_double), ("rho_cheb", C.c_double)]


class _StageTimes(C.Structure):
    _fields_ = [(f, C.c_double) for f in ("predict", "local_step", "scatter", "assemble", "solve", "unpack_scan",
                                           "velocity", "total")]


class _SimStats(C.Structure):
    _fields_ = [("iterations_used", C.c_int32), ("converged", C.c_int32),
                ("early_exit_count", C.c_int32), ("last_residual", C.c_double)]


class _SolverStats(C.Structure):
    _fields_ = [
        ("analyze_calls", C.c_int32), ("factorize_calls", C.c_int32), ("solve_calls", C.c_int32),
        ("last_analyze_seconds", C.c_double), ("last_factorize_seconds", C.c_double),
        ("last_solve_seconds", C.c_double), ("total_factorize_seconds", C.c_double),
        ("total_solve_seconds", C.c_double), ("nnz", C.c_int64), ("factor_nnz", C.c_int64),
    ]


_lib = None

# name -> (argtypes, restype); every function returns an int status unless noted
_SIGS = {
    "pd_last_error": ([], C.c_char_p),
    "pd_scene_config_default": ([C.POINTER(_Cfg)], None),
    "pd_grid_counts": ([C.POINTER(_Cfg), _ip, _ip, _ip], C.c_int),
    "pd_make_grid": ([C.POINTER(_Cfg), _dp, _dp, _u8p, _ip, _dp, _dp, _ip, _dp], C.c_int),
    "pd_obj_counts": ([C.c_char_p, _ip, _ip], C.c_int),
    "pd_make_obj": ([C.POINTER(_Cfg), C.c_char_p, _dp, _dp, _u8p, _ip, _dp, _dp], C.c_int),
    "pd_solver_create": ([C.POINTER(C.c_void_p)], C.c_int),
    "pd_solver_destroy": ([C.c_void_p], C.c_int),
    "pd_solver_analyze": ([C.c_void_p, C.c_int32, _ip, _ip], C.c_int),
    "pd_solver_factorize": ([C.c_void_p, C.c_int32, _ip, _ip, _dp], C.c_int),
    "pd_solver_analyzed": ([C.c_void_p], C.c_int),
    "pd_solver_solve": ([C.c_void_p, _dp, _dp], C.c_int),
    "pd_solver_parallel_components": ([C.c_void_p], C.c_int),
    "pd_solver_solve_component": ([C.c_void_p, C.c_int32, _dp, _dp], C.c_int),
    "pd_solver_note_solve_stage": ([C.c_void_p, C.c_double], C.c_int),
    "pd_solver_stats_get": ([C.c_void_p, C.POINTER(_SolverStats)], C.c_int),
    "pd_sim_create": ([C.POINTER(_Mesh), C.POINTER(_Cfg), C.POINTER(C.c_void_p)], C.c_int),
    "pd_sim_create_batch": ([C.c_int32, C.POINTER(_Mesh), C.POINTER(_Cfg), C.POINTER(C.c_void_p)], C.c_int),
    "pd_sim_destroy": ([C.c_void_p], C.c_int),
    "pd_sim_instance_count": ([C.c_void_p], C.c_int),
    "pd_sim_step": ([C.c_void_p, C.c_int32], C.c_int),
    "pd_sim_synchronize": ([C.c_void_p], C.c_int),
    "pd_sim_set_stream": ([C.c_void_p, C.c_void_p], C.c_int),
    "pd_sim_get_state": ([C.c_void_p, C.c_int32, _dp, _dp], C.c_int),
    "pd_sim_set_state": ([C.c_void_p, C.c_int32, _dp, _dp], C.c_int),
    "pd_sim_device_state": ([C.c_void_p, C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)], C.c_int),
    "pd_sim_bind_host": ([C.c_void_p, C.POINTER(_dp), C.POINTER(_dp)], C.c_int),
    "pd_sim_set_stage_timing": ([C.c_void_p, C.c_int32], C.c_int),
    "pd_sim_get_stage_times": ([C.c_void_p, C.c_int32, C.POINTER(_StageTimes)], C.c_int),
    "pd_sim_reset_stage_times": ([C.c_void_p], C.c_int),
    "pd_sim_spectrum": ([C.c_void_p, C.c_int32, C.c_int32, C.POINTER(_Spectrum)], C.c_int),
    "pd_sim_autotune": ([C.c_void_p, C.c_int32, C.POINTER(_Plan), _dp, _ip, _ip], C.c_int),
    "pd_sim_set_plan": ([C.c_void_p, C.POINTER(_Plan)], C.c_int),
    "pd_sim_get_plan": ([C.c_void_p, C.POINTER(_Plan)], C.c_int),
    "pd_sim_step_host": ([C.c_void_p, C.c_int32], C.c_int),
    "pd_sim_set_pin_positions": ([C.c_void_p, C.c_int32, _dp], C.c_int),
    "pd_sim_set_edge_stiffness": ([C.c_void_p, C.c_int32, _dp], C.c_int),
    "pd_sim_set_pinned": ([C.c_void_p, C.c_int32, _u8p, _dp], C.c_int),
    "pd_sim_set_config": ([C.c_void_p, C.POINTER(_Cfg)], C.c_int),
    "pd_sim_get_info": ([C.c_void_p, C.c_int32, C.POINTER(_SimInfo)], C.c_int),
    "pd_sim_get_stats": ([C.c_void_p, C.c_int32, C.POINTER(_SimStats)], C.c_int),
    "pd_sim_set_residual_trace": ([C.c_void_p, C.c_int32], C.c_int),
    "pd_sim_get_residual_trace": ([C.c_void_p, C.c_int32, _dp, C.c_int32], C.c_int),
    "pd_sim_iteration_log": ([C.c_void_p, C.c_int32, _ip, _u8p, C.c_int32], C.c_int),
    "pd_sim_get_factor": ([C.c_void_p, C.c_int32, _ip, _ip, _ip, _dp, _dp, C.POINTER(C.c_int64)], C.c_int),
    "pd_sim_solve": ([C.c_void_p, C.c_int32, _dp, _dp], C.c_int),
    "pd_sim_gradient": ([C.c_void_p, C.c_int32, C.POINTER(_dp), C.POINTER(_dp), _dp, C.POINTER(_dp),
                         C.POINTER(_dp), C.POINTER(_dp)], C.c_int),
    "pd_scene_factor": ([C.POINTER(_Mesh), C.POINTER(_Cfg), _ip, _ip, _ip, _dp, _dp, C.POINTER(C.c_int64),
                         C.POINTER(_SimInfo)], C.c_int),
    "pd_scene_coloring": ([C.POINTER(_Mesh), C.POINTER(C.c_uint32), C.POINTER(C.c_int32)], C.c_int),
}


def scene_factor(scene: "GridScene", cfg: "SceneConfig"):
    """Host-only preparation of pd_sim_create: returns (factor dict, info dict); no GPU work."""
    lib = load_library()
    m, keep = scene._c()
    c = cfg.c()
    nnz = C.c_int64()
    info = _SimInfo()
    _check(lib.pd_scene_factor(C.byref(m), C.byref(c), None, None, None, None, None, C.byref(nnz), C.byref(info)))
    n = scene.n
    perm = np.zeros(n, np.int32)
    cp = np.zeros(n + 1, np.int32)
    ri = np.zeros(nnz.value, np.int32)
    val = np.zeros(nnz.value)
    dinv = np.zeros(n)
    _check(lib.pd_scene_factor(C.byref(m), C.byref(c), _ptr(perm, C.c_int32), _ptr(cp, C.c_int32),
                               _ptr(ri, C.c_int32), _ptr(val, C.c_double), _ptr(dinv, C.c_double),
                               C.byref(nnz), None))
    del keep
    return dict(perm=perm, colptr=cp, rowidx=ri, val=val, dinv=dinv), {f: getattr(info, f) for f, _ in _SimInfo._fields_}


def scene_coloring(scene: "GridScene"):
    """Edge colouring of the scene (host only): (color_of, colour count)."""
    lib = load_library()
    m, keep = scene._c()
    out = np.zeros(int(np.asarray(scene.edges).reshape(-1, 2).shape[0]), np.uint32)
    cc = C.c_int32()
    _check(lib.pd_scene_coloring(C.byref(m), _ptr(out, C.c_uint32), C.byref(cc)))
    del keep
    return out, cc.value


def load_library(path: str | None = None):
    """Loads the CUDA library; raises if it has not been built (no CPU fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"pd_gb300 CUDA library not found at {p}; build it with "
                          "`python -m pd_gb300.build` (or __graft_entry__.build())")
    lib = C.CDLL(p)
    for name, (args, res) in _SIGS.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def _check(rc):
    if rc != PD_OK:
        raise PdError(rc, _lib.pd_last_error().decode())


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


@dataclass
class SceneConfig:
    """``SceneConfig`` (core/sim/Scene.h:14-137) with the reference defaults."""
    dt: float = 1.0 / 120.0
    substeps_per_frame: int = 2
    gravity: tuple = (0.0, -9.81, 0.0)
    stiffness: float = 2.3e3
    density: float = 1.0
    velocity_damping: float = 0.02
    max_iterations: int = 10
    rel_tolerance: float = 1.0e-3
    abs_tolerance: float = 1.0e-12
    residual_tolerance: float = 1.0e-3
    grid_nx: int = 40
    grid_ny: int = 40
    grid_spacing: float = 0.025
    shear_stiffness: float = 0.0
    bend_stiffness: float = 0.0
    bend_sampling: int = 0
    bend_stride: int = 1
    mass_mode: int = 0
    total_mass: float = 1.0
    pin_mode: int = 0
    precision: int = PD_PRECISION_FP64_EXACT
    cluster_ctas: int = 0
    dense_max_vertices: int = 0
    # over-relaxed iterates (Integrator.cpp:476-645; the reference's PD_CHEB* variables)
    cheb_mode: int = 0        # PD_CHEB_OFF, PD_CHEB_RHO, PD_CHEB_INTERVAL
    cheb_rho: float = 0.98
    cheb_start: int = 10
    cheb_m: float = 1.0
    cheb_d: float = 1.0

    def c(self) -> _Cfg:
        c = _Cfg()
        for f in fields(self):
            v = getattr(self, f.name)
            if f.name == "gravity":
                for i in range(3):
                    c.gravity[i] = v[i]
            else:
                setattr(c, f.name, v)
        return c


@dataclass
class GridScene:
    """Raw arrays of one cloth (vectors [x, y, z] per vertex)."""
    positions: np.ndarray
    masses: np.ndarray
    pinned: np.ndarray
    edges: np.ndarray
    edge_rest: np.ndarray
    edge_stiffness: np.ndarray
    bends: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    bend_stiffness: np.ndarray = field(default_factory=lambda: np.zeros(0))
    velocities: np.ndarray | None = None
    pin_positions: np.ndarray | None = None

    @property
    def n(self):
        return int(self.positions.shape[0])

    def _c(self):
        """Returns a pd_mesh view plus the arrays that must stay alive while it is used."""
        keep = [np.ascontiguousarray(self.positions, np.float64),
                None if self.velocities is None else np.ascontiguousarray(self.velocities, np.float64),
                np.ascontiguousarray(self.masses, np.float64),
                np.ascontiguousarray(self.pinned, np.uint8),
                None if self.pin_positions is None else np.ascontiguousarray(self.pin_positions, np.float64),
                np.ascontiguousarray(self.edges, np.int32).reshape(-1, 2),
                np.ascontiguousarray(self.edge_rest, np.float64),
                np.ascontiguousarray(self.edge_stiffness, np.float64),
                np.ascontiguousarray(self.bends, np.int32).reshape(-1, 3),
                np.ascontiguousarray(self.bend_stiffness, np.float64)]
        m = _Mesh(self.n, _ptr(keep[0], C.c_double), _ptr(keep[1], C.c_double), _ptr(keep[2], C.c_double),
                  _ptr(keep[3], C.c_uint8), _ptr(keep[4], C.c_double), int(keep[5].shape[0]),
                  _ptr(keep[5], C.c_int32), _ptr(keep[6], C.c_double), _ptr(keep[7], C.c_double),
                  int(keep[8].shape[0]), _ptr(keep[8], C.c_int32), _ptr(keep[9], C.c_double))
        return m, keep


def make_grid(cfg: SceneConfig) -> GridScene:
    """The grid cloth of ``makeScene`` for this config, built by the library (pd_make_grid)."""
    lib = load_library()
    c = cfg.c()
    nv, ne, nb = C.c_int32(), C.c_int32(), C.c_int32()
    _check(lib.pd_grid_counts(C.byref(c), C.byref(nv), C.byref(ne), C.byref(nb)))
    nv, ne, nb = nv.value, ne.value, nb.value
    pos = np.zeros((nv, 3))
    mass = np.zeros(nv)
    pin = np.zeros(nv, np.uint8)
    e = np.zeros((ne, 2), np.int32)
    er = np.zeros(ne)
    ek = np.zeros(ne)
    b = np.zeros((nb, 3), np.int32)
    bk = np.zeros(nb)
    _check(lib.pd_make_grid(C.byref(c), _ptr(pos, C.c_double), _ptr(mass, C.c_double), _ptr(pin, C.c_uint8),
                            _ptr(e, C.c_int32), _ptr(er, C.c_double), _ptr(ek, C.c_double),
                            _ptr(b, C.c_int32), _ptr(bk, C.c_double)))
    return GridScene(pos, mass, pin, e, er, ek, b, bk)


def make_obj(obj, cfg: SceneConfig) -> GridScene:
    """The triangle mesh of ``makeScene`` with a mesh path (``Mesh::loadObj`` + surface masses,
    core/mesh/Mesh.cpp:56-153), built by the library (pd_make_obj). ``obj`` is the path of an OBJ
    file or its text; cfg supplies stiffness and density. No pins: set ``scene.pinned``."""
    lib = load_library()
    if "\n" not in obj and os.path.exists(obj):
        with open(obj) as f:
            obj = f.read()
    text = obj.encode()
    c = cfg.c()
    nv, ne = C.c_int32(), C.c_int32()
    _check(lib.pd_obj_counts(text, C.byref(nv), C.byref(ne)))
    nv, ne = nv.value, ne.value
    pos = np.zeros((nv, 3))
    mass = np.zeros(nv)
    pin = np.zeros(nv, np.uint8)
    e = np.zeros((ne, 2), np.int32)
    er = np.zeros(ne)
    ek = np.zeros(ne)
    _check(lib.pd_make_obj(C.byref(c), text, _ptr(pos, C.c_double), _ptr(mass, C.c_double), _ptr(pin, C.c_uint8),
                           _ptr(e, C.c_int32), _ptr(er, C.c_double), _ptr(ek, C.c_double)))
    return GridScene(pos, mass, pin, e, er, ek)


class Simulator:
    """One or more cloths stepped on the GPU (``SimContext`` + ``stepOnce``)."""

    def __init__(self, scenes, cfgs):
        lib = load_library()
        if isinstance(scenes, GridScene):
            scenes = [scenes]
        if isinstance(cfgs, SceneConfig):
            cfgs = [cfgs] * len(scenes)
        self._lib = lib
        self.n = [s.n for s in scenes]
        self.n_edges = [int(np.asarray(s.edges).reshape(-1, 2).shape[0]) for s in scenes]
        meshes = (_Mesh * len(scenes))()
        keep = []
        for i, s in enumerate(scenes):
            m, k = s._c()
            meshes[i] = m
            keep.append(k)
        ccfg = (_Cfg * len(cfgs))()
        for i, cf in enumerate(cfgs):
            ccfg[i] = cf.c()
        h = C.c_void_p()
        _check(lib.pd_sim_create_batch(len(scenes), meshes, ccfg, C.byref(h)))
        self._h = h
        self.count = len(scenes)
        self._last = 0
        self._cfgs = list(cfgs)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pd_sim_destroy(self._h)
            self._h = None

    __del__ = close

    def step(self, substeps: int = 1, sync: bool = True):
        _check(self._lib.pd_sim_step(self._h, int(substeps)))
        self._last = int(substeps)
        if sync:
            _check(self._lib.pd_sim_synchronize(self._h))

    step_once = step

    def synchronize(self):
        _check(self._lib.pd_sim_synchronize(self._h))

    def set_stream(self, stream_ptr: int | None):
        _check(self._lib.pd_sim_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def _index(self, i: int) -> int:
        if not 0 <= i < self.count:
            raise PdError(1, f"instance index {i} out of range (batch of {self.count})")
        return i

    def state(self, i: int = 0, out_x=None, out_v=None):
        """Positions and velocities of instance i (waits for queued work); optional out arrays."""
        self._index(i)
        x = np.zeros((self.n[i], 3)) if out_x is None else out_x
        v = np.zeros((self.n[i], 3)) if out_v is None else out_v
        for a in (x, v):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != 3 * self.n[i]:
                raise ValueError("state arrays must be contiguous float64 of shape (n, 3)")
        _check(self._lib.pd_sim_get_state(self._h, i, _ptr(x, C.c_double), _ptr(v, C.c_double)))
        return x, v

    def set_state(self, i: int = 0, x=None, v=None):
        xs = None if x is None else np.ascontiguousarray(x, np.float64)
        vs = None if v is None else np.ascontiguousarray(v, np.float64)
        _check(self._lib.pd_sim_set_state(self._h, i, _ptr(xs, C.c_double), _ptr(vs, C.c_double)))
        self._keep = (xs, vs)  # host memory must outlive the queued copy

    def bind_host(self, xs, vs):
        """Binds one positions and one velocities array ((n, 3) contiguous float64) per instance for
        step_host; None, None unbinds. Arrays in page-locked memory (e.g. numpy views of pinned
        torch tensors) are moved by kernels inside one CUDA graph; they are kept referenced here."""
        if xs is None and vs is None:
            _check(self._lib.pd_sim_bind_host(self._h, None, None))
            self._host = None
            return
        if isinstance(xs, np.ndarray):
            xs, vs = [xs], [vs]
        if len(xs) != self.count or len(vs) != self.count:
            raise ValueError("one positions and one velocities array per instance")
        for i, (x, v) in enumerate(zip(xs, vs)):
            for a in (x, v):
                if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != 3 * self.n[i]:
                    raise ValueError("host state arrays must be contiguous float64 of shape (n, 3)")
        px = (_dp * self.count)(*[_ptr(x, C.c_double) for x in xs])
        pv = (_dp * self.count)(*[_ptr(v, C.c_double) for v in vs])
        _check(self._lib.pd_sim_bind_host(self._h, px, pv))
        self._host = (list(xs), list(vs))

    def step_host(self, substeps: int = 1):
        """Copies the bound arrays in, runs `substeps` substeps and copies them back (blocking)."""
        _check(self._lib.pd_sim_step_host(self._h, int(substeps)))
        if substeps > 0:
            self._last = int(substeps)

    def set_stage_timing(self, enable: bool = True):
        """StageTimes (core/sim/Scene.h:140-149) on the device: see pd_sim_set_stage_timing."""
        _check(self._lib.pd_sim_set_stage_timing(self._h, int(bool(enable))))

    def stage_times(self, i: int = 0) -> dict:
        out = _StageTimes()
        _check(self._lib.pd_sim_get_stage_times(self._h, i, C.byref(out)))
        return {f: getattr(out, f) for f, _ in _StageTimes._fields_}

    def reset_stage_times(self):
        _check(self._lib.pd_sim_reset_stage_times(self._h))

    def spectrum(self, i: int = 0, iters: int = 400) -> dict:
        """Power-iteration spectrum of the linearised PD map of instance i at its current positions
        (pd_sim_spectrum; the reference's _verify/iteration_spectrum.cpp)."""
        out = _Spectrum()
        _check(self._lib.pd_sim_spectrum(self._h, i, int(iters), C.byref(out)))
        return {f: getattr(out, f) for f, _ in _Spectrum._fields_}

    def autotune(self, substeps: int = 10) -> dict:
        """Times candidate launch plans on this batch and keeps the fastest (pd_sim_autotune); the
        simulation state is unchanged. Returns {"tried": [plan dicts], "ms": [...], "chosen": k}."""
        plans = (_Plan * PD_TUNE_MAX_CANDIDATES)()
        ms = np.zeros(PD_TUNE_MAX_CANDIDATES)
        n, k = C.c_int32(), C.c_int32()
        _check(self._lib.pd_sim_autotune(self._h, int(substeps), plans, _ptr(ms, C.c_double), C.byref(n), C.byref(k)))
        tried = [{f: getattr(plans[i], f) for f, _ in _Plan._fields_} for i in range(n.value)]
        self._last = 0
        return {"tried": tried, "ms": ms[:n.value].tolist(), "chosen": k.value}

    def plan(self) -> dict:
        p = _Plan()
        _check(self._lib.pd_sim_get_plan(self._h, C.byref(p)))
        return {f: getattr(p, f) for f, _ in _Plan._fields_}

    def set_plan(self, plan: dict):
        p = _Plan(**{f: plan.get(f, 0) for f, _ in _Plan._fields_})
        _check(self._lib.pd_sim_set_plan(self._h, C.byref(p)))
        self._last = 0

    def device_state(self, i: int = 0):
        x, v = C.c_void_p(), C.c_void_p()
        _check(self._lib.pd_sim_device_state(self._h, i, C.byref(x), C.byref(v)))
        return x.value, v.value

    def set_pin_positions(self, q, i: int = 0):
        q = np.ascontiguousarray(q, np.float64)
        _check(self._lib.pd_sim_set_pin_positions(self._h, i, _ptr(q, C.c_double)))

    def set_edge_stiffness(self, k, i: int = 0):
        k = np.ascontiguousarray(k, np.float64)
        _check(self._lib.pd_sim_set_edge_stiffness(self._h, i, _ptr(k, C.c_double)))

    def set_pinned(self, pinned, q=None, i: int = 0):
        p = np.ascontiguousarray(pinned, np.uint8)
        qq = None if q is None else np.ascontiguousarray(q, np.float64)
        _check(self._lib.pd_sim_set_pinned(self._h, i, _ptr(p, C.c_uint8), _ptr(qq, C.c_double)))

    def set_config(self, cfg: SceneConfig):
        c = cfg.c()
        _check(self._lib.pd_sim_set_config(self._h, C.byref(c)))
        self._cfgs = [cfg] * self.count

    def info(self, i: int = 0) -> dict:
        s = _SimInfo()
        _check(self._lib.pd_sim_get_info(self._h, i, C.byref(s)))
        return {f: getattr(s, f) for f, _ in _SimInfo._fields_}

    def stats(self, i: int = 0) -> dict:
        s = _SimStats()
        _check(self._lib.pd_sim_get_stats(self._h, i, C.byref(s)))
        return {f: getattr(s, f) for f, _ in _SimStats._fields_}

    def gradient(self, substeps: int, targets, forces=None, grad=True):
        """Loss and adjoint gradients of every instance (pd_sim_gradient): targets / forces are one
        (n, 3) array per instance (or one array for a single cloth; forces may be None). Returns one
        dict per instance with loss, dkappa (per edge), dv0 and dforce ((n, 3)), or a single dict."""
        count = self.count
        single = not isinstance(targets, (list, tuple))
        tl = [targets] if single else list(targets)
        fl = [forces] * count if (forces is None or single) else list(forces)
        if single and forces is not None:
            fl = [forces]
        if len(tl) != count or len(fl) != count:
            raise PdError(1, "one target (and force) array per instance")
        keep = []
        def arr(a):
            a = np.ascontiguousarray(a, np.float64)
            keep.append(a)
            return _ptr(a, C.c_double)
        tp = (_dp * count)(*[arr(t) for t in tl])
        fp = (_dp * count)(*[(arr(f) if f is not None else _dp()) for f in fl])
        loss = np.zeros(count)
        outs = []
        for i in range(count):
            outs.append(dict(dkappa=np.zeros(self.n_edges[i]), dv0=np.zeros((self.n[i], 3)),
                             dforce=np.zeros((self.n[i], 3))) if grad else {})
        def ptrs(key):
            if not grad:
                return (_dp * count)()
            return (_dp * count)(*[_ptr(o[key], C.c_double) for o in outs])
        _check(self._lib.pd_sim_gradient(self._h, int(substeps), tp, fp, _ptr(loss, C.c_double), ptrs("dkappa"),
                                         ptrs("dv0"), ptrs("dforce")))
        for i, o in enumerate(outs):
            o["loss"] = float(loss[i])
        return outs[0] if single else outs

    def iteration_log(self, i: int = 0):
        it = np.zeros(self._last, np.int32)
        cv = np.zeros(self._last, np.uint8)
        _check(self._lib.pd_sim_iteration_log(self._h, i, _ptr(it, C.c_int32), _ptr(cv, C.c_uint8), self._last))
        return it, cv

    def set_residual_trace(self, enable: bool = True):
        """Record the gate residual after every iteration of every substep (pd_sim_set_residual_trace)."""
        _check(self._lib.pd_sim_set_residual_trace(self._h, 1 if enable else 0))

    def residual_trace(self, i: int = 0):
        """(substeps of the last step, max_iterations) residuals, NaN past each substep's last iteration."""
        k = max(1, self._cfgs[i].max_iterations)
        out = np.zeros((self._last, k))
        _check(self._lib.pd_sim_get_residual_trace(self._h, i, _ptr(out, C.c_double), self._last))
        return out

    def factor(self, i: int = 0) -> dict:
        nnz = C.c_int64()
        _check(self._lib.pd_sim_get_factor(self._h, i, None, None, None, None, None, C.byref(nnz)))
        n = self.n[i]
        perm = np.zeros(n, np.int32)
        cp = np.zeros(n + 1, np.int32)
        ri = np.zeros(nnz.value, np.int32)
        val = np.zeros(nnz.value)
        dinv = np.zeros(n)
        _check(self._lib.pd_sim_get_factor(self._h, i, _ptr(perm, C.c_int32), _ptr(cp, C.c_int32),
                                           _ptr(ri, C.c_int32), _ptr(val, C.c_double), _ptr(dinv, C.c_double),
                                           C.byref(nnz)))
        return dict(perm=perm, colptr=cp, rowidx=ri, val=val, dinv=dinv)

    def solve(self, b, i: int = 0):
        b = np.ascontiguousarray(b, np.float64).reshape(-1)
        x = np.zeros_like(b)
        _check(self._lib.pd_sim_solve(self._h, i, _ptr(b, C.c_double), _ptr(x, C.c_double)))
        return x.reshape(-1, 3)


class GpuDirectSolver:
    """``IGlobalSolver`` drop-in (analyze / factorize / solve / solveComponent / stats).

    Matrices are given in compressed-column form (Eigen's SparseMatrix layout): ``col_ptr``,
    ``row_idx`` and ``values`` of the 3n × 3n matrix L.
    """

    def __init__(self):
        self._lib = load_library()
        h = C.c_void_p()
        _check(self._lib.pd_solver_create(C.byref(h)))
        self._h = h
        self.n = 0

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pd_solver_destroy(self._h)
            self._h = None

    __del__ = close

    def analyze(self, n, col_ptr, row_idx):
        self._cp = np.ascontiguousarray(col_ptr, np.int32)
        self._ri = np.ascontiguousarray(row_idx, np.int32)
        _check(self._lib.pd_solver_analyze(self._h, int(n), _ptr(self._cp, C.c_int32), _ptr(self._ri, C.c_int32)))
        self.n = int(n)

    def analyzed(self) -> bool:
        return bool(self._lib.pd_solver_analyzed(self._h))

    def factorize(self, n, col_ptr, row_idx, values):
        cp = np.ascontiguousarray(col_ptr, np.int32)
        ri = np.ascontiguousarray(row_idx, np.int32)
        v = np.ascontiguousarray(values, np.float64)
        _check(self._lib.pd_solver_factorize(self._h, int(n), _ptr(cp, C.c_int32), _ptr(ri, C.c_int32),
                                             _ptr(v, C.c_double)))

    def solve(self, b):
        b = np.ascontiguousarray(b, np.float64).reshape(-1)
        x = np.zeros_like(b)
        _check(self._lib.pd_solver_solve(self._h, _ptr(b, C.c_double), _ptr(x, C.c_double)))
        return x

    def parallel_components(self) -> int:
        return int(self._lib.pd_solver_parallel_components(self._h))

    def solve_component(self, c, b, x):
        b = np.ascontiguousarray(b, np.float64).reshape(-1)
        assert x.dtype == np.float64 and x.flags.c_contiguous and x.size == b.size
        _check(self._lib.pd_solver_solve_component(self._h, int(c), _ptr(b, C.c_double), _ptr(x, C.c_double)))

    def note_solve_stage(self, seconds: float):
        _check(self._lib.pd_solver_note_solve_stage(self._h, float(seconds)))

    def stats(self) -> dict:
        s = _SolverStats()
        _check(self._lib.pd_solver_stats_get(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in _SolverStats._fields_}
