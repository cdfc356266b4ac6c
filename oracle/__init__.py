"""ctypes wrapper of the CPU FP64 oracle (oracle.c).

TEST INFRASTRUCTURE ONLY. Only the tests, the smoke check and bench.py's CPU
baseline may import this package; the shipped library and its Python mirror never
do. Parity status: partially pinned (see oracle.h).

Arrays follow the reference's Julia layout: markers are (N, 2) column-major
(numpy order='F'), so the flat buffer is [v1(1..N); v2(1..N)].
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build() -> str:
    """Compile the oracle (make -C oracle); returns the library path."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
        os.path.join(_HERE, "oracle.c")
    ):
        build()
    lib = C.CDLL(_LIB_PATH)
    lib.om_create.restype = C.c_void_p
    lib.om_create.argtypes = [_dp, C.c_int, _dp, C.c_int, C.c_int, C.c_int]
    lib.om_destroy.argtypes = [C.c_void_p]
    lib.om_n_dofs.argtypes = [C.c_void_p]
    lib.om_nd1.argtypes = [C.c_void_p]
    for name in ("om_mass_matrix_dense",):
        getattr(lib, name).argtypes = [C.c_void_p, _dp]
    lib.om_extraction.argtypes = [C.c_void_p, C.c_int, _dp]
    lib.om_quadrature.argtypes = [C.c_void_p, _dp, _dp]
    lib.om_mass_solve.argtypes = [C.c_void_p, _dp, _dp]
    lib.om_set_mass_solver.argtypes = [C.c_void_p, C.c_int]
    lib.om_l2_project.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _dp]
    lib.om_l2_rhs.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _dp]
    lib.om_compute_r.argtypes = [C.c_void_p, _dp, _dp]
    lib.om_entropy.argtypes = [C.c_void_p, _dp]
    lib.om_entropy.restype = C.c_double
    lib.om_compute_G.argtypes = [C.c_void_p, _dp, C.c_int, _dp, _dp]
    lib.om_hessian_L.argtypes = [C.c_void_p, _dp, C.c_int, _dp, _dp]
    lib.om_diagnostics.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _dp]
    lib.om_loggrad.argtypes = [C.c_void_p, _dp, C.c_int, _dp, _dp]
    lib.om_eval_field.argtypes = [C.c_void_p, _dp, C.c_double, C.c_double]
    lib.om_eval_field.restype = C.c_double
    lib.om_collision.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int, _dp, C.c_int]
    lib.om_collision_rows.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int, _ip, C.c_int, _dp, C.c_int]
    lib.om_collision_metric.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int, _dp, _dp, C.c_int]
    lib.om_moments.argtypes = [_dp, _dp, C.c_int, _dp]
    lib.om_drift_multipliers.argtypes = [_dp, _dp, _dp, C.c_int, C.c_double, C.c_double,
                                         C.c_double, C.c_double, _dp]
    lib.om_lb_velocity.argtypes = [_dp, _dp, _dp, C.c_int, C.c_double, C.c_double,
                                   C.c_double, C.c_double]
    lib.om_picard_map.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp, _dp, _dp, C.c_int,
                                  C.c_double, C.c_double]
    lib.om_step_anderson.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp, _dp, C.c_int,
                                     C.c_double, C.c_double, _dp]
    lib.om_step_defect.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_int,
                                   C.c_int, _dp,
                                   _dp, _dp, C.c_int, C.c_double, C.c_double, _dp]
    lib.om_predictor.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp, _dp, C.c_int, C.c_double]
    lib.om_step_newton.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double,
                                   _dp, _dp, _dp, C.c_int, C.c_double, C.c_double, _dp]
    _lib = lib
    return lib


class _Opts(C.Structure):
    _fields_ = [
        ("model", C.c_int), ("nu", C.c_double), ("use_gonzalez", C.c_int),
        ("use_anderson", C.c_int), ("exit_picard_step", C.c_int), ("m", C.c_int),
        ("max_iter", C.c_int), ("tol", C.c_double), ("abs_floor", C.c_double),
        ("stag_window", C.c_int), ("stag_rel_tol", C.c_double),
        ("damp_decay_start", C.c_int), ("damp_decay_factor", C.c_double),
        ("restart_factor", C.c_double), ("damping", C.c_double),
        ("reg_factor", C.c_double), ("nthreads", C.c_int),
    ]


@dataclass
class Opts:
    """Solver switches of SimParameters (Parameters.jl:50-106) that the oracle reads."""
    model: str = "landau"
    nu: float = 1.0
    use_gonzalez: bool = True
    use_anderson: bool = True
    exit_picard_step: bool = True
    m: int = 5
    max_iter: int = 1000
    tol: float = 1e-12
    abs_floor: float = 1e-7
    stag_window: int = 50
    stag_rel_tol: float = 0.01
    damp_decay_start: int = 200
    damp_decay_factor: float = 0.5
    restart_factor: float = float("inf")
    damping: float = 0.5
    reg_factor: float = 1e-10
    nthreads: int = 0

    def c(self) -> _Opts:
        return _Opts(1 if self.model == "lb" else 0, self.nu, int(self.use_gonzalez),
                     int(self.use_anderson), int(self.exit_picard_step), self.m,
                     self.max_iter, self.tol, self.abs_floor, self.stag_window,
                     self.stag_rel_tol, self.damp_decay_start, self.damp_decay_factor,
                     self.restart_factor if np.isfinite(self.restart_factor) else -1.0,
                     self.damping, self.reg_factor, self.nthreads)


def _d(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _mk(a, n=None) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    return np.asfortranarray(a)


class OracleMesh:
    """Workspace analogue on the CPU (MantisWrappers.jl:90-158)."""

    def __init__(self, bp1, bp2, nquad: int = 6, use_logsq: bool = False):
        self.lib = _load()
        self.bp1 = np.ascontiguousarray(bp1, dtype=np.float64)
        self.bp2 = np.ascontiguousarray(bp2, dtype=np.float64)
        self.h = self.lib.om_create(_d(self.bp1), len(self.bp1), _d(self.bp2), len(self.bp2),
                                    nquad, int(use_logsq))
        if not self.h:
            raise ValueError("bad mesh")
        self.n_dofs = self.lib.om_n_dofs(self.h)
        self.nd1 = self.lib.om_nd1(self.h)
        self.nquad = nquad

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.om_destroy(self.h)
            self.h = None

    # --- FEM layer -------------------------------------------------------
    def mass_matrix(self) -> np.ndarray:
        out = np.zeros((self.n_dofs, self.n_dofs))
        self.lib.om_mass_matrix_dense(self.h, _d(out))
        return out

    def extraction(self, dim: int) -> np.ndarray:
        n = (len(self.bp1) if dim == 1 else len(self.bp2)) - 1
        out = np.zeros((n, 3, 3))
        self.lib.om_extraction(self.h, dim, _d(out))
        return out

    def quadrature(self):
        x = np.zeros(self.nquad)
        w = np.zeros(self.nquad)
        self.lib.om_quadrature(self.h, _d(x), _d(w))
        return x, w

    def set_mass_solver(self, kind: int) -> None:
        """0: 2D banded Cholesky (default); 1: tensor-product solve with the 1D
        Cholesky factors -- a second correct FP64 solve for round-off studies."""
        self.lib.om_set_mass_solver(self.h, int(kind))

    def mass_solve(self, rhs) -> np.ndarray:
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        out = np.zeros(self.n_dofs)
        self.lib.om_mass_solve(self.h, _d(rhs), _d(out))
        return out

    def l2_project(self, v, w) -> np.ndarray:
        v, w = _mk(v), np.ascontiguousarray(w, dtype=np.float64)
        out = np.zeros(self.n_dofs)
        self.lib.om_l2_project(self.h, _d(v), _d(w), v.shape[0], _d(out))
        return out

    def l2_rhs(self, v, w) -> np.ndarray:
        v, w = _mk(v), np.ascontiguousarray(w, dtype=np.float64)
        out = np.zeros(self.n_dofs)
        self.lib.om_l2_rhs(self.h, _d(v), _d(w), v.shape[0], _d(out))
        return out

    def compute_r(self, f) -> np.ndarray:
        f = np.ascontiguousarray(f, dtype=np.float64)
        out = np.zeros(self.n_dofs)
        self.lib.om_compute_r(self.h, _d(f), _d(out))
        return out

    def entropy(self, f) -> float:
        f = np.ascontiguousarray(f, dtype=np.float64)
        return self.lib.om_entropy(self.h, _d(f))

    def compute_G(self, v, L) -> np.ndarray:
        v, L = _mk(v), np.ascontiguousarray(L, dtype=np.float64)
        out = np.zeros((v.shape[0], 2), order="F")
        self.lib.om_compute_G(self.h, _d(v), v.shape[0], _d(L), _d(out))
        return out

    def diagnostics(self, v, w) -> np.ndarray:
        """(S, energy, P1, P2, ||f_s - f_p||_2, negative-part L1) of markers v."""
        v = _mk(v)
        w = np.ascontiguousarray(w, dtype=np.float64)
        out = np.zeros(6)
        self.lib.om_diagnostics(self.h, _d(v), _d(w), v.shape[0], _d(out))
        return out

    def hessian_L(self, v, L) -> np.ndarray:
        """(H11, H12, H22) of the spline field L at markers v, shape (N, 3)."""
        v, L = _mk(v), np.ascontiguousarray(L, dtype=np.float64)
        out = np.zeros((v.shape[0], 3), order="F")
        self.lib.om_hessian_L(self.h, _d(v), v.shape[0], _d(L), _d(out))
        return out

    def loggrad(self, v, f) -> np.ndarray:
        v, f = _mk(v), np.ascontiguousarray(f, dtype=np.float64)
        out = np.zeros((v.shape[0], 2), order="F")
        self.lib.om_loggrad(self.h, _d(v), v.shape[0], _d(f), _d(out))
        return out

    def eval_field(self, c, x1: float, x2: float) -> float:
        c = np.ascontiguousarray(c, dtype=np.float64)
        return self.lib.om_eval_field(self.h, _d(c), float(x1), float(x2))

    # --- pair sums -------------------------------------------------------
    def collision(self, v, w, G, nthreads: int = 0) -> np.ndarray:
        v, G = _mk(v), _mk(G)
        w = np.ascontiguousarray(w, dtype=np.float64)
        out = np.zeros((v.shape[0], 2), order="F")
        self.lib.om_collision(self.h, _d(v), _d(w), _d(G), v.shape[0], _d(out), nthreads)
        return out

    def collision_rows(self, v, w, G, rows, nthreads: int = 0) -> np.ndarray:
        v, G = _mk(v), _mk(G)
        w = np.ascontiguousarray(w, dtype=np.float64)
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        out = np.zeros((len(rows), 2), order="F")
        self.lib.om_collision_rows(self.h, _d(v), _d(w), _d(G), v.shape[0],
                                   rows.ctypes.data_as(_ip), len(rows), _d(out), nthreads)
        return out

    def collision_metric(self, v, w, G, nthreads: int = 0):
        v, G = _mk(v), _mk(G)
        w = np.ascontiguousarray(w, dtype=np.float64)
        out = np.zeros((v.shape[0], 2), order="F")
        A = np.zeros((v.shape[0], 3), order="F")
        self.lib.om_collision_metric(self.h, _d(v), _d(w), _d(G), v.shape[0], _d(out),
                                     _d(A), nthreads)
        return out, A

    # --- solver ------------------------------------------------------------
    def picard_map(self, opts: Opts, v_in, v0, w, S0: float, dt: float) -> np.ndarray:
        v_in, v0 = _mk(v_in), _mk(v0)
        w = np.ascontiguousarray(w, dtype=np.float64)
        out = np.zeros_like(v0, order="F")
        o = opts.c()
        self.lib.om_picard_map(self.h, C.byref(o), _d(out), _d(v_in), _d(v0), _d(w),
                               v0.shape[0], S0, dt)
        return out

    def step_anderson(self, opts: Opts, v1, v0, w, S0: float, dt: float):
        v1 = np.array(v1, dtype=np.float64, order="F", copy=True)
        v0 = _mk(v0)
        w = np.ascontiguousarray(w, dtype=np.float64)
        out4 = np.zeros(4)
        o = opts.c()
        self.lib.om_step_anderson(self.h, C.byref(o), _d(v1), _d(v0), _d(w), v0.shape[0],
                                  S0, dt, _d(out4))
        return v1, (int(out4[0]), out4[1], int(out4[2]), out4[3])

    def step_defect(self, opts: Opts, v1, v0, w, S0: float, dt: float, eta: float = 0.05,
                    max_inner: int = 60, stag_window: int = 5, outer_m: int = 0,
                    precond: int = 0):
        """step_defect! (solver.jl:569-634) -> (v, (outer, residual, inner, r0));
        outer_m > 0 adds Anderson mixing of the outer iterates, precond = 1 the
        block-Newton preconditioner of the inner iteration."""
        v1 = np.array(v1, dtype=np.float64, order="F", copy=True)
        v0 = _mk(v0)
        w = np.ascontiguousarray(w, dtype=np.float64)
        out4 = np.zeros(4)
        o = opts.c()
        self.lib.om_step_defect(self.h, C.byref(o), eta, max_inner, stag_window, outer_m,
                                int(precond), _d(v1), _d(v0),
                                _d(w), v0.shape[0], S0, dt, _d(out4))
        return v1, (int(out4[0]), out4[1], int(out4[2]), out4[3])

    def step_newton(self, opts: Opts, v1, v0, w, S0: float, dt: float, krylov_max: int = 30,
                    fd_h: float = 1e-6, eta_max: float = 0.9):
        """step_newton! (solver.jl:460-486) -> (v, (evals, ||F||, newton steps, ||F_0||,
        status)); status 0 converged, 1 stalled, 2 budget."""
        v1 = np.array(v1, dtype=np.float64, order="F", copy=True)
        v0 = _mk(v0)
        w = np.ascontiguousarray(w, dtype=np.float64)
        out5 = np.zeros(5)
        o = opts.c()
        self.lib.om_step_newton(self.h, C.byref(o), krylov_max, fd_h, eta_max, _d(v1), _d(v0),
                                _d(w), v0.shape[0], S0, dt, _d(out5))
        return v1, (int(out5[0]), out5[1], int(out5[2]), out5[3], int(out5[4]))

    def predictor(self, opts: Opts, v, w, dt: float) -> np.ndarray:
        v = _mk(v)
        w = np.ascontiguousarray(w, dtype=np.float64)
        out = np.zeros_like(v, order="F")
        o = opts.c()
        self.lib.om_predictor(self.h, C.byref(o), _d(out), _d(v), _d(w), v.shape[0], dt)
        return out


def moments(v, w):
    """compute_moments (functions.jl:68-83) -> (n, U1, U2, Q)."""
    lib = _load()
    v, w = _mk(v), np.ascontiguousarray(w, dtype=np.float64)
    out = np.zeros(4)
    lib.om_moments(_d(v), _d(w), v.shape[0], _d(out))
    return tuple(out)


def drift_multipliers(v, w, g, n, U1, U2, Q):
    """compute_drift_multipliers (functions.jl:91-107) -> (A1, A2, B)."""
    lib = _load()
    v, g, w = _mk(v), _mk(g), np.ascontiguousarray(w, dtype=np.float64)
    out = np.zeros(3)
    lib.om_drift_multipliers(_d(v), _d(w), _d(g), v.shape[0], n, U1, U2, Q, _d(out))
    return tuple(out)


def lb_velocity(v, g, A1, A2, B, nu):
    """compute_LB_velocity! (functions.jl:110-116)."""
    lib = _load()
    v, g = _mk(v), _mk(g)
    out = np.zeros_like(v, order="F")
    lib.om_lb_velocity(_d(out), _d(v), _d(g), v.shape[0], A1, A2, B, nu)
    return out


def momentum(v, w):
    """compute_momentum (functions.jl:349-353)."""
    v = np.asarray(v)
    return float(np.sum(w * v[:, 0])), float(np.sum(w * v[:, 1]))


def energy(v, w):
    """compute_energy (functions.jl:355-358)."""
    v = np.asarray(v)
    return 0.5 * float(np.sum(w * (v[:, 0] ** 2 + v[:, 1] ** 2)))
