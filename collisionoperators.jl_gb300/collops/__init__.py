"""collops -- host-side mirror of CollisionOperators.jl's hot-loop API over the
GB300 C-ABI library (libcollops.so, sm_103a).

The reference repoints five hooks at run time (solver.jl:30-34, main.jl:390-423):
COLLISION_FN, L2PROJ_FN, COMPG_FN, LOGGRAD_FN and COLLMETRIC_FN. This module
offers the same operations with the same argument meaning: every hook writes
into its first array argument and returns None; arrays use the reference's
Julia layout (markers are N x 2 column-major, i.e. numpy order='F'). A non-zero
status from the library raises CollopsError; there is no CPU fallback -- if the
library or a GPU is missing, the call fails.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
from dataclasses import dataclass, field
from typing import Any

import numpy as np

__all__ = [
    "CollopsError", "SimParameters", "parse_overrides", "Workspace", "build_workspace",
    "compute_collision_gpu", "compute_collision_gpu32", "compute_collision_metric_gpu",
    "l2_project_gpu", "compute_G_gpu", "eval_loggrad_gpu", "compute_r_gpu",
    "compute_entropy_gpu", "mass_solve_gpu", "picard_map", "step_anderson", "step_defect",
    "step_newton",
    "predictor", "save_checkpoint", "load_checkpoint", "checkpoint_path",
    "enable_gpu", "Hooks", "library_path", "load_library",
]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_lib", "libcollops.so")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

CO_MODEL_LANDAU, CO_MODEL_LB = 0, 1
CO_PREC_FP64, CO_PREC_MIXED, CO_PREC_MIXED_DS = 0, 1, 2
_PREC = {"fp64": CO_PREC_FP64, "mixed": CO_PREC_MIXED, "mixed_ds": CO_PREC_MIXED_DS}
CO_FLAG_LOGSQ, CO_FLAG_FP32_PAIR, CO_FLAG_ONESIDED = 1, 2, 4


class CollopsError(RuntimeError):
    """Raised for a non-zero library status (the Julia shim raises `error`)."""

    def __init__(self, status: int, where: str):
        msg = load_library().co_strerror(status).decode() if _lib is not None else str(status)
        super().__init__(f"{where}: status {status} ({msg})")
        self.status = status


class CoOpts(C.Structure):
    """co_opts of include/collops.h."""
    _fields_ = [
        ("model", C.c_int), ("nu", C.c_double), ("use_gonzalez", C.c_int),
        ("use_anderson", C.c_int), ("exit_picard_step", C.c_int), ("m", C.c_int),
        ("max_iter", C.c_int), ("tol", C.c_double), ("abs_floor", C.c_double),
        ("stag_window", C.c_int), ("stag_rel_tol", C.c_double),
        ("damp_decay_start", C.c_int), ("damp_decay_factor", C.c_double),
        ("restart_factor", C.c_double), ("damping", C.c_double),
        ("reg_factor", C.c_double), ("precision", C.c_int), ("mixed_floor", C.c_double),
    ]


class CoProfile(C.Structure):
    """co_profile_t of include/collops.h."""
    _fields_ = [("pair64_ms", C.c_double), ("pair64_launches", C.c_ulonglong),
                ("pair64_pairs", C.c_double), ("pair32_ms", C.c_double),
                ("pair32_launches", C.c_ulonglong), ("pair32_pairs", C.c_double),
                ("maps64", C.c_ulonglong), ("maps32", C.c_ulonglong),
                ("pairds_ms", C.c_double), ("pairds_launches", C.c_ulonglong),
                ("pairds_pairs", C.c_double), ("mapsds", C.c_ulonglong)]


class CoDefectOpts(C.Structure):
    """co_defect_opts of include/collops.h."""
    _fields_ = [("eta", C.c_double), ("max_inner", C.c_int), ("stag_window", C.c_int),
                ("fp32_stall", C.c_double), ("metric64", C.c_int), ("outer_m", C.c_int),
                ("precond", C.c_int), ("metric_freeze", C.c_double), ("fp32_window", C.c_int),
                ("cap_refresh", C.c_int), ("cap_abort", C.c_int)]


class CoNewtonOpts(C.Structure):
    """co_newton_opts of include/collops.h."""
    _fields_ = [("krylov_max", C.c_int), ("fd_h", C.c_double), ("eta_max", C.c_double)]


class CoStepInfo(C.Structure):
    """co_step_info of include/collops.h."""
    _fields_ = [("outer", C.c_int), ("inner", C.c_int), ("res", C.c_double),
                ("r0", C.c_double), ("converged", C.c_int), ("exit", C.c_int),
                ("start", C.c_int), ("attempts", C.c_int), ("r_start", C.c_double * 3),
                ("S_new", C.c_double)]

    START_NAMES = ("predictor", "learned", "previous")

    def as_dict(self) -> dict:
        return dict(outer=self.outer, inner=self.inner, res=self.res, r0=self.r0,
                    converged=bool(self.converged), exit=self.exit,
                    start=self.START_NAMES[self.start], attempts=self.attempts,
                    r_start=list(self.r_start), S_new=self.S_new)


class CoBatchInstance(C.Structure):
    """co_batch_instance of include/collops.h."""
    _fields_ = [("bp1", C.POINTER(C.c_double)), ("nb1", C.c_int), ("bp2", C.POINTER(C.c_double)),
                ("nb2", C.c_int), ("model", C.c_int), ("nu", C.c_double), ("N", C.c_int)]


# (name, restype, argtypes) of every entry point in include/collops.h
_SIGNATURES = {
    "co_version": (C.c_int, []),
    "co_strerror": (C.c_char_p, [C.c_int]),
    "co_ctx_create": (C.c_int, [_dp, C.c_int, _dp, C.c_int, C.c_int, C.c_int, C.c_uint,
                                C.c_int, C.POINTER(C.c_void_p)]),
    "co_ctx_destroy": (C.c_int, [C.c_void_p]),
    "co_ctx_n_dofs": (C.c_int, [C.c_void_p, _ip]),
    "co_collision": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, C.c_int]),
    "co_collision_metric": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp, _dp, C.c_int]),
    "co_l2_project": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_int]),
    "co_grad_L": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_int]),
    "co_loggrad": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_int]),
    "co_compute_r": (C.c_int, [C.c_void_p, _dp, _dp]),
    "co_entropy": (C.c_int, [C.c_void_p, _dp, _dp]),
    "co_mass_solve": (C.c_int, [C.c_void_p, _dp, _dp]),
    "co_picard_map": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), _dp, _dp, _dp, _dp, C.c_int,
                                C.c_double, C.c_double]),
    "co_step_anderson": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), _dp, _dp, _dp, C.c_int,
                                   C.c_double, C.c_double, _ip, _dp, _ip, _dp]),
    "co_step_anderson_dev": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_int, C.c_double, C.c_double, _ip, _dp,
                                       _ip, _dp]),
    "co_step_defect": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), C.POINTER(CoDefectOpts), _dp,
                                 _dp, _dp, C.c_int, C.c_double, C.c_double, _ip, _dp, _ip, _dp]),
    "co_step_defect_dev": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), C.POINTER(CoDefectOpts),
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double,
                                     C.c_double, _ip, _dp, _ip, _dp]),
    "co_step_newton": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), C.POINTER(CoNewtonOpts), _dp,
                                 _dp, _dp, C.c_int, C.c_double, C.c_double, _ip, _dp, _ip, _dp,
                                 _ip]),
    "co_step_newton_dev": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), C.POINTER(CoNewtonOpts),
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double,
                                     C.c_double, _ip, _dp, _ip, _dp, _ip]),
    "co_predictor": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), _dp, _dp, _dp, C.c_int,
                               C.c_double]),
    "co_predictor_dev": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_int, C.c_double]),
    "co_entropy_of_markers_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, _dp]),
    "co_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_ulonglong)]),
    "co_ctx_set_wait_limit": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "co_ctx_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "co_profile": (C.c_int, [C.c_void_p, C.c_int]),
    "co_profile_read": (C.c_int, [C.c_void_p, C.POINTER(CoProfile)]),
    "co_measure_fma_peak": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "co_batch_create": (C.c_int, [C.POINTER(CoBatchInstance), C.c_int, C.c_int, C.c_uint,
                                  C.c_int, C.POINTER(C.c_void_p)]),
    "co_batch_destroy": (C.c_int, [C.c_void_p]),
    "co_batch_tune": (C.c_int, [C.c_void_p, _ip, _ip, _ip, _dp]),
    "co_batch_step_dev": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), C.c_void_p, C.c_void_p,
                                    C.c_void_p, _dp, C.c_double, C.c_int, _ip, _dp]),
    "co_batch_predictor_dev": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_double]),
    "co_batch_entropy_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, _dp]),
    "co_batch_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_ulonglong)]),
    "co_mlp_create": (C.c_int, [C.c_int, C.c_int, C.c_uint, C.c_int, C.POINTER(C.c_void_p)]),
    "co_mlp_destroy": (C.c_int, [C.c_void_p]),
    "co_mlp_num_params": (C.c_int, [C.c_void_p, _ip]),
    "co_mlp_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "co_mlp_get_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "co_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "co_mlp_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                   C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "co_mlp_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float,
                                    C.POINTER(C.c_float)]),
    "co_diagnostics": (C.c_int, [C.c_void_p, _dp, _dp, C.c_int, _dp]),
    "co_diagnostics_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, _dp]),
    "co_warmstart_features_dev": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), C.c_void_p,
                                            C.c_void_p, C.c_int, C.c_double, C.c_double,
                                            C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "co_warmstart_apply_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                         C.c_double, _dp, _dp, C.c_void_p]),
    "co_picard_residual_dev": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_int, C.c_double, C.c_double, _dp]),
    "co_mlp_set_normalization": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp]),
    "co_step_learned": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), C.POINTER(CoDefectOpts),
                                  C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_int, C.c_double,
                                  C.c_double, C.POINTER(CoStepInfo)]),
    "co_step_learned_dev": (C.c_int, [C.c_void_p, C.POINTER(CoOpts), C.POINTER(CoDefectOpts),
                                      C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_int, C.c_double, C.c_double, C.POINTER(CoStepInfo)]),
    "co_collision_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_void_p]),
}


def library_path() -> str:
    return _LIB_PATH


def load_library():
    """Load libcollops.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise RuntimeError(
            f"libcollops.so not found at {_LIB_PATH}: build it first "
            "(python collisionoperators.jl_gb300/build.py)")
    lib = C.CDLL(_LIB_PATH)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(status: int, where: str) -> None:
    if status != 0:
        raise CollopsError(status, where)


# ------------------------------------------------------------------ params

@dataclass
class SimParameters:
    """The SimParameters fields the hot path reads (Parameters.jl:18-140).

    Defaults follow the reference. `bp1`/`bp2` are the breakpoint vectors.
    """
    bp1: Any = field(default_factory=lambda: np.concatenate(
        [[-6.0, -5.0], np.linspace(-4.0, 4.0, 17), [5.0, 6.0]]))
    bp2: Any = field(default_factory=lambda: np.concatenate(
        [[-6.0], np.linspace(-2.5, 2.5, 13), [6.0]]))
    P_DEG: int = 2
    K_REG: int = 1
    N_QUAD: int = 6
    N_PARTICLES: int = 10_000
    σ1: float = 4 / 3
    σ2: float = 0.5
    DT: float = 0.001
    N_STEPS: int = 400
    collision_model: str = "landau"
    nu: float = 1.0
    use_gonzalez: bool = True
    use_logsq: bool = False
    use_anderson: bool = True
    damping: float = 0.7
    m_anderson: int = 8
    tol: float = 1e-12
    max_iter: int = 2000
    abs_floor: float = 1e-7
    stag_window: int = 50
    stag_rel_tol: float = 0.01
    damp_decay_start: int = 200
    damp_decay_factor: float = 0.5
    exit_picard_step: bool = True
    v1_peak: float = 0.0
    use_gpu: bool = False
    gpu_fp32: bool = False
    suffix: str = "anderson"
    seed: int = 42
    # build-specific: precision form of the implicit solve ("fp64" | "mixed"),
    # and the one-sided pair kernels in place of the symmetric ones
    precision: str = "fp64"
    mixed_floor: float = 0.0
    pair_onesided: bool = False

    def opts(self, **kw) -> CoOpts:
        """co_opts for step_anderson!/picard_map! from these parameters."""
        d = dict(model=CO_MODEL_LB if self.collision_model == "lb" else CO_MODEL_LANDAU,
                 nu=self.nu, use_gonzalez=int(self.use_gonzalez),
                 use_anderson=int(self.use_anderson), exit_picard_step=int(self.exit_picard_step),
                 m=self.m_anderson, max_iter=self.max_iter, tol=self.tol,
                 abs_floor=self.abs_floor, stag_window=self.stag_window,
                 stag_rel_tol=self.stag_rel_tol, damp_decay_start=self.damp_decay_start,
                 damp_decay_factor=self.damp_decay_factor, restart_factor=-1.0,
                 damping=self.damping, reg_factor=1e-10,
                 precision=_PREC[self.precision],
                 mixed_floor=self.mixed_floor)
        d.update(kw)
        return CoOpts(**d)


def _coerce(tp, s: str):
    """_coerce of Parameters.jl:157-171."""
    if tp is bool:
        if s in ("true", "1"):
            return True
        if s in ("false", "0"):
            return False
        raise ValueError(f"Cannot parse {s} as Bool")
    if tp in ("Any",) or tp is Any:
        raise ValueError("Vector parameters (`bp1`, `bp2`) are not CLI-overridable; "
                         "edit the preset file")
    if tp is str:
        return s
    return tp(s)


def parse_overrides(p: SimParameters, args) -> SimParameters:
    """parse_overrides (Parameters.jl:179-192): apply --key=value tokens."""
    if not args:
        return p
    types = {f.name: f.type for f in dataclasses.fields(SimParameters)}
    resolved = {"int": int, "float": float, "bool": bool, "str": str, "Any": Any}
    over = {}
    for tok in args:
        if not tok.startswith("--"):
            continue
        if "=" not in tok:
            raise ValueError(f"CLI override {tok} must use --key=value form")
        key, val = tok[2:].split("=", 1)
        if key not in types:
            raise ValueError(f"Unknown parameter: {key}")
        tp = types[key]
        tp = resolved.get(tp, tp) if isinstance(tp, str) else tp
        over[key] = _coerce(tp, val)
    return dataclasses.replace(p, **over)


# ------------------------------------------------------------------ arrays

def _markers(a, N=None, name="array", ncol=2) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    if a.ndim != 2 or a.shape[1] != ncol or (N is not None and a.shape[0] != N):
        raise ValueError(f"{name}: expected shape (N, {ncol})")
    return np.asfortranarray(a)


def _out(a, shape, name) -> np.ndarray:
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.shape == shape and
            (a.flags.f_contiguous or len(shape) == 1 and a.flags.c_contiguous)):
        raise ValueError(f"{name}: output must be a float64 array of shape {shape} in "
                         "column-major (order='F') layout")
    return a


def _vec(a, n=None, name="vector") -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.ndim != 1 or (n is not None and a.shape[0] != n):
        raise ValueError(f"{name}: expected length {n}")
    return a


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


# ------------------------------------------------------------------ workspace

class Workspace:
    """Device workspace of one mesh (build_workspace, MantisWrappers.jl:90-158)."""

    def __init__(self, p: SimParameters, device: int = 0):
        self.lib = load_library()
        if p.P_DEG != 2:
            # the reference keeps the CPU projection for P_DEG != 2 (main.jl:396-404);
            # the library reports the configuration as unsupported
            pass
        self.p = p
        self.bp1 = np.ascontiguousarray(p.bp1, dtype=np.float64)
        self.bp2 = np.ascontiguousarray(p.bp2, dtype=np.float64)
        flags = ((CO_FLAG_LOGSQ if p.use_logsq else 0) | (CO_FLAG_FP32_PAIR if p.gpu_fp32 else 0)
                 | (CO_FLAG_ONESIDED if p.pair_onesided else 0))
        h = C.c_void_p()
        self.h = None
        _check(self.lib.co_ctx_create(_p(self.bp1), len(self.bp1), _p(self.bp2), len(self.bp2),
                                      p.P_DEG, p.N_QUAD, flags, device, C.byref(h)),
               "co_ctx_create")
        self.h = h
        n = C.c_int()
        _check(self.lib.co_ctx_n_dofs(self.h, C.byref(n)), "co_ctx_n_dofs")
        self.n_dofs = n.value
        self.n_dofs_1d_1 = len(self.bp1) + 1
        self.n_dofs_1d_2 = len(self.bp2) + 1

    def close(self):
        if self.h is not None:
            self.lib.co_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def launch_count(self) -> int:
        n = C.c_ulonglong()
        _check(self.lib.co_launch_count(self.h, C.byref(n)), "co_launch_count")
        return n.value

    def set_wait_limit(self, spins: int = 0, phantom_blocks: int = 0) -> None:
        """Bounded device-side waits (co_ctx_set_wait_limit): the LB grid
        barrier polls at most `spins` times (0: the default) and waits for
        `phantom_blocks` arrivals beyond the grid (0 in normal use)."""
        _check(self.lib.co_ctx_set_wait_limit(self.h, int(spins), int(phantom_blocks)),
               "co_ctx_set_wait_limit")

    def stream(self) -> int:
        """cudaStream_t (as an int) on which the context enqueues all its work."""
        s = C.c_void_p()
        _check(self.lib.co_ctx_stream(self.h, C.byref(s)), "co_ctx_stream")
        return s.value or 0


def build_workspace(p: SimParameters, device: int = 0) -> Workspace:
    return Workspace(p, device)


# ------------------------------------------------------------------ hooks

def compute_collision_gpu(ws: Workspace, dot_v, v_parts, w_parts, G) -> None:
    """COLLISION_FN (functions.jl:205-237; collision_gpu.jl:258-280)."""
    v = _markers(v_parts, name="v_parts")
    N = v.shape[0]
    _check(ws.lib.co_collision(ws.h, _p(v), _p(_vec(w_parts, N, "w_parts")),
                               _p(_markers(G, N, "G")), _p(_out(dot_v, (N, 2), "dot_v")), N),
           "co_collision")


def compute_collision_gpu32(ws: Workspace, dot_v, v_parts, w_parts, G) -> None:
    """COLLISION_FN under gpu_fp32 (collision_gpu.jl:233-256): the mixed FP32 pair sum.

    The workspace must have been built with gpu_fp32=True.
    """
    if not ws.p.gpu_fp32:
        raise ValueError("compute_collision_gpu32 needs a workspace built with gpu_fp32=true")
    compute_collision_gpu(ws, dot_v, v_parts, w_parts, G)


def compute_collision_metric_gpu(ws: Workspace, dot_v, A, v_parts, w_parts, G) -> None:
    """COLLMETRIC_FN (functions.jl:249-290; collision_gpu.jl:377-402)."""
    v = _markers(v_parts, name="v_parts")
    N = v.shape[0]
    _check(ws.lib.co_collision_metric(ws.h, _p(v), _p(_vec(w_parts, N, "w_parts")),
                                      _p(_markers(G, N, "G")), _p(_out(dot_v, (N, 2), "dot_v")),
                                      _p(_out(A, (N, 3), "A")), N), "co_collision_metric")


def l2_project_gpu(ws: Workspace, f_coeffs, v_parts, w_parts) -> None:
    """L2PROJ_FN (functions.jl:121-134; projection_gpu.jl:213-226), mass solve included."""
    v = _markers(v_parts, name="v_parts")
    N = v.shape[0]
    _check(ws.lib.co_l2_project(ws.h, _p(v), _p(_vec(w_parts, N, "w_parts")),
                                _p(_out(f_coeffs, (ws.n_dofs,), "f_coeffs")), N),
           "co_l2_project")


def compute_G_gpu(ws: Workspace, G, v_parts, L_vec) -> None:
    """COMPG_FN (functions.jl:182-202; projection_gpu.jl:228-246)."""
    v = _markers(v_parts, name="v_parts")
    N = v.shape[0]
    _check(ws.lib.co_grad_L(ws.h, _p(v), _p(_vec(L_vec, ws.n_dofs, "L_vec")),
                            _p(_out(G, (N, 2), "G")), N), "co_grad_L")


def eval_loggrad_gpu(ws: Workspace, g, v_parts, f_coeffs) -> None:
    """LOGGRAD_FN (functions.jl:37-64; projection_gpu.jl:251-269)."""
    v = _markers(v_parts, name="v_parts")
    N = v.shape[0]
    _check(ws.lib.co_loggrad(ws.h, _p(v), _p(_vec(f_coeffs, ws.n_dofs, "f_coeffs")),
                             _p(_out(g, (N, 2), "g")), N), "co_loggrad")


def compute_r_gpu(ws: Workspace, r, f_coeffs) -> None:
    """compute_r! (functions.jl:158-179) from coefficients."""
    _check(ws.lib.co_compute_r(ws.h, _p(_vec(f_coeffs, ws.n_dofs, "f_coeffs")),
                               _p(_out(r, (ws.n_dofs,), "r"))), "co_compute_r")


def compute_entropy_gpu(ws: Workspace, f_coeffs) -> float:
    """compute_entropy (functions.jl:137-155) from coefficients."""
    S = np.zeros(1)
    _check(ws.lib.co_entropy(ws.h, _p(_vec(f_coeffs, ws.n_dofs, "f_coeffs")), _p(S)),
           "co_entropy")
    return float(S[0])


def mass_solve_gpu(ws: Workspace, out, rhs) -> None:
    """ldiv!(out, ws.M_lu, rhs) (solver.jl:67)."""
    _check(ws.lib.co_mass_solve(ws.h, _p(_vec(rhs, ws.n_dofs, "rhs")),
                                _p(_out(out, (ws.n_dofs,), "out"))), "co_mass_solve")


def _opts(ws: Workspace, use_gonzalez=None, **kw) -> CoOpts:
    o = ws.p.opts(**kw)
    if use_gonzalez is not None:
        o.use_gonzalez = int(use_gonzalez)
    return o


def picard_map(ws: Workspace, v_out, v_in, v0, w_parts, S0: float, dt: float, *,
               use_gonzalez: bool = True, precision: str | None = None) -> None:
    """picard_map! (solver.jl:176-227); model from ws.p.collision_model."""
    v0 = _markers(v0, name="v0")
    N = v0.shape[0]
    kw = {}
    if precision is not None:
        kw["precision"] = _PREC[precision]
    o = _opts(ws, use_gonzalez, **kw)
    _check(ws.lib.co_picard_map(ws.h, C.byref(o), _p(_out(v_out, (N, 2), "v_out")),
                                _p(_markers(v_in, N, "v_in")), _p(v0),
                                _p(_vec(w_parts, N, "w_parts")), N, S0, dt), "co_picard_map")


def step_anderson(ws: Workspace, v1, v0, w_parts, S0: float, dt: float, *, m: int = 5,
                  max_iter: int = 1000, tol: float = 1e-12, abs_floor: float = 1e-7,
                  stag_window: int = 50, stag_rel_tol: float = 0.01,
                  damp_decay_start: int = 200, damp_decay_factor: float = 0.5,
                  restart_factor: float = float("inf"), damping: float = 0.5,
                  reg_factor: float = 1e-10, use_anderson: bool = True,
                  use_gonzalez: bool = True, exit_picard_step: bool = True,
                  precision: str = "fp64", mixed_floor: float = 0.0):
    """step_anderson! (solver.jl:300-423) on the device; v1 (guess) is overwritten
    with the solution. Returns (iterations, residual, n_restarts, initial_residual)."""
    v0 = _markers(v0, name="v0")
    N = v0.shape[0]
    v1 = _out(v1, (N, 2), "v1")
    o = ws.p.opts(m=m, max_iter=max_iter, tol=tol, abs_floor=abs_floor, stag_window=stag_window,
                  stag_rel_tol=stag_rel_tol, damp_decay_start=damp_decay_start,
                  damp_decay_factor=damp_decay_factor,
                  restart_factor=restart_factor if np.isfinite(restart_factor) else -1.0,
                  damping=damping, reg_factor=reg_factor, use_anderson=int(use_anderson),
                  use_gonzalez=int(use_gonzalez), exit_picard_step=int(exit_picard_step),
                  precision=_PREC[precision], mixed_floor=mixed_floor)
    it, nrs = C.c_int(), C.c_int()
    res, r0 = C.c_double(), C.c_double()
    _check(ws.lib.co_step_anderson(ws.h, C.byref(o), _p(v1), _p(v0),
                                   _p(_vec(w_parts, N, "w_parts")), N, S0, dt, C.byref(it),
                                   C.byref(res), C.byref(nrs), C.byref(r0)), "co_step_anderson")
    return it.value, res.value, nrs.value, r0.value


def step_defect(ws: Workspace, v1, v0, w_parts, S0: float, dt: float, *, m: int = 8,
                max_iter: int = 2000, tol: float = 1e-12, abs_floor: float = 1e-7,
                damping: float = 0.7, eta: float = 0.05, max_inner: int = 60,
                stag_window: int = 5, stag_rel_tol: float = 0.1, use_gonzalez: bool = True,
                precision: str = "fp64", metric64: bool = True, fp32_stall: float = 0.5,
                outer_m: int = 0, precond: int = 0, metric_freeze: float = 0.0,
                fp32_window: int = 0, cap_refresh: int = 0, cap_abort: int = 0):
    """step_defect! (solver.jl:569-634) on the device; v1 (guess) is overwritten with
    the solution. Returns (outer_iterations, residual, inner_iterations, initial_residual).
    outer_m > 0 mixes the outer iterates by Anderson and precond = 1 preconditions the
    inner iteration per marker (0, 0 = the reference's algorithm); metric_freeze > 0
    stops rebuilding the FP32 metric once ||r|| < metric_freeze ||r_1||; cap_refresh
    rebuilds it after an inner solve that hit max_inner; cap_abort = K leaves through
    the stagnation exit once K FP64-stage outer maps in a row ended in a capped inner
    solve without a new best outer residual."""
    v0 = _markers(v0, name="v0")
    N = v0.shape[0]
    v1 = _out(v1, (N, 2), "v1")
    o = ws.p.opts(m=m, max_iter=max_iter, tol=tol, abs_floor=abs_floor, damping=damping,
                  stag_rel_tol=stag_rel_tol, use_gonzalez=int(use_gonzalez),
                  precision=_PREC[precision])
    d = CoDefectOpts(eta, max_inner, stag_window, fp32_stall, int(metric64), int(outer_m),
                     int(precond), float(metric_freeze), int(fp32_window), int(cap_refresh),
                     int(cap_abort))
    it, inner = C.c_int(), C.c_int()
    res, r0 = C.c_double(), C.c_double()
    _check(ws.lib.co_step_defect(ws.h, C.byref(o), C.byref(d), _p(v1), _p(v0),
                                 _p(_vec(w_parts, N, "w_parts")), N, S0, dt, C.byref(it),
                                 C.byref(res), C.byref(inner), C.byref(r0)), "co_step_defect")
    return it.value, res.value, inner.value, r0.value


def step_newton(ws: Workspace, v1, v0, w_parts, S0: float, dt: float, *, max_iter: int = 1000,
                tol: float = 1e-12, abs_floor: float = 1e-7, krylov_max: int = 30,
                fd_h: float = 1e-6, eta_max: float = 0.9, use_gonzalez: bool = True,
                exit_picard_step: bool = True, precision: str = "fp64"):
    """step_newton! (solver.jl:460-486) on the device; v1 (guess) is overwritten with
    the solution. Returns (evaluations, ||F||, newton_steps, ||F_0||, status) with
    status 0 converged, 1 stalled (line search failed), 2 budget."""
    v0 = _markers(v0, name="v0")
    N = v0.shape[0]
    v1 = _out(v1, (N, 2), "v1")
    o = ws.p.opts(max_iter=max_iter, tol=tol, abs_floor=abs_floor,
                  use_gonzalez=int(use_gonzalez), exit_picard_step=int(exit_picard_step),
                  precision=_PREC[precision])
    k = CoNewtonOpts(krylov_max, fd_h, eta_max)
    ev, nn, stt = C.c_int(), C.c_int(), C.c_int()
    res, r0 = C.c_double(), C.c_double()
    _check(ws.lib.co_step_newton(ws.h, C.byref(o), C.byref(k), _p(v1), _p(v0),
                                 _p(_vec(w_parts, N, "w_parts")), N, S0, dt, C.byref(ev),
                                 C.byref(res), C.byref(nn), C.byref(r0), C.byref(stt)),
           "co_step_newton")
    return ev.value, res.value, nn.value, r0.value, stt.value


def diagnostics(ws: Workspace, v_parts, w_parts) -> dict:
    """Post-step diagnostics of main.jl:298-307 on the device: entropy, energy,
    momentum, ||f_s - f_p||_2 and the negative-part L1 norm of f_s."""
    v = _markers(v_parts, name="v_parts")
    N = v.shape[0]
    out = np.zeros(6)
    _check(ws.lib.co_diagnostics(ws.h, _p(v), _p(_vec(w_parts, N, "w_parts")), N, _p(out)),
           "co_diagnostics")
    return dict(entropy=out[0], energy=out[1], momentum=(out[2], out[3]), fs_minus_fp_l2=out[4],
                negative_part_l1=out[5])


# columns of the reference's per-step conservation CSV (io.jl CONS_COLS)
CONS_COLS = ("step", "time", "entropy", "energy", "momentum_1", "momentum_2", "iter",
             "residual", "fp_minus_fs", "neg_part", "r0", "dt")


def conservation_row(step: int, time: float, diag: dict, iters: int, residual: float,
                     r0: float, dt: float) -> str:
    """One row of the conservation CSV the reference's time loop appends after
    each step (main.jl:309-317; columns io.jl CONS_COLS), from `diagnostics()`
    and the step's solver record, so the reference's dashboards read it."""
    vals = (step, time, diag["entropy"], diag["energy"], diag["momentum"][0],
            diag["momentum"][1], iters, residual, diag["fs_minus_fp_l2"],
            diag["negative_part_l1"], r0, dt)
    return ",".join(repr(float(x)) if isinstance(x, float) else str(x) for x in vals)


# ------------------------------------------------------------------ checkpoint

# Fields of the reference's checkpoint NamedTuple (io.jl:53-86), in its order.
CHECKPOINT_FIELDS = ("step", "t", "v_particles", "w_particles", "f_coeffs", "entropy_history",
                     "energy_history", "momentum_history", "iter_history", "res_history",
                     "fp_l2_history", "neg_history", "rng_state")


def checkpoint_path(suffix: str, step: int) -> str:
    """checkpoint_path (io.jl:65-67) with the .npz extension of this export."""
    return f"checkpoint_{suffix}_step{step:04d}.npz"


def save_checkpoint(suffix: str, step: int, t: float, v_particles, w_particles, f_coeffs,
                    entropy_history, energy_history, momentum_history, iter_history,
                    res_history, fp_l2_history, neg_history, directory: str = ".") -> str:
    """save_checkpoint (io.jl:70-86) as a NumPy archive with the same fields: the
    markers (N x 2, the Julia layout), weights, spline coefficients and the seven
    diagnostic histories. The device holds no other state between steps (the
    solver re-derives everything from v and w), so this is the whole state.
    rng_state is left empty: the reference only keeps it for forward
    compatibility (io.jl:60-61), and a Julia RNG cannot be written from here;
    the conversion in INTEGRATION.md substitutes Random.default_rng()."""
    v = _markers(v_particles, name="v_particles")
    N = v.shape[0]
    arrays = dict(step=np.int64(step), t=np.float64(t), v_particles=v,
                  w_particles=_vec(w_particles, N, "w_particles"),
                  f_coeffs=_vec(f_coeffs, None, "f_coeffs"),
                  entropy_history=np.asarray(entropy_history, dtype=np.float64),
                  energy_history=np.asarray(energy_history, dtype=np.float64),
                  momentum_history=np.asarray(momentum_history, dtype=np.float64).reshape(-1, 2),
                  iter_history=np.asarray(iter_history, dtype=np.int64),
                  res_history=np.asarray(res_history, dtype=np.float64),
                  fp_l2_history=np.asarray(fp_l2_history, dtype=np.float64),
                  neg_history=np.asarray(neg_history, dtype=np.float64),
                  rng_state=np.zeros(0, dtype=np.uint8))
    path = os.path.join(directory, checkpoint_path(suffix, step))
    # v_particles is stored transposed-free: np.save keeps the array's own
    # (Fortran) order flag, so a Julia reader sees the column-major N x 2 matrix
    with open(path, "wb") as fh:
        np.savez(fh, **arrays)
    return path


def load_checkpoint(suffix: str, step, directory: str = ".") -> dict:
    """load_checkpoint (io.jl:169-182): step = "auto" (or <= 0) picks the
    highest-step archive of the suffix. Returns the fields as a dict."""
    if step == "auto" or (isinstance(step, int) and step <= 0):
        files = sorted(f for f in os.listdir(directory)
                       if f.startswith(f"checkpoint_{suffix}_step") and f.endswith(".npz"))
        if not files:
            raise FileNotFoundError(f"No checkpoint files for suffix={suffix}")
        path = os.path.join(directory, files[-1])
    else:
        path = os.path.join(directory, checkpoint_path(suffix, int(step)))
    if not os.path.exists(path):
        raise FileNotFoundError(f"Checkpoint not found: {path}")
    with np.load(path) as z:
        d = {k: z[k] for k in CHECKPOINT_FIELDS}
    d["step"] = int(d["step"])
    d["t"] = float(d["t"])
    d["v_particles"] = np.asfortranarray(d["v_particles"])
    return d


def predictor(ws: Workspace, v1, v_parts, w_parts, dt: float, precision: str = "fp64") -> None:
    """Explicit predictor of the time loop (main.jl:233-245): v1 = v + dt vdot(v)."""
    v = _markers(v_parts, name="v_parts")
    N = v.shape[0]
    o = ws.p.opts(precision=_PREC[precision])
    _check(ws.lib.co_predictor(ws.h, C.byref(o), _p(_out(v1, (N, 2), "v1")), _p(v),
                               _p(_vec(w_parts, N, "w_parts")), N, dt), "co_predictor")


@dataclass
class Hooks:
    """The five hook slots of solver.jl:30-34 after enable_gpu! (main.jl:390-423)."""
    COLLISION_FN: Any = None
    L2PROJ_FN: Any = None
    COMPG_FN: Any = None
    LOGGRAD_FN: Any = None
    COLLMETRIC_FN: Any = None


def enable_gpu(p: SimParameters) -> Hooks:
    """Repoint the hooks at the GB300 library, keyed like enable_gpu! on
    collision_model and gpu_fp32. P_DEG != 2 raises (unsupported), where the
    reference would keep its CPU projection."""
    if p.P_DEG != 2:
        raise CollopsError(3, "enable_gpu")
    h = Hooks(L2PROJ_FN=l2_project_gpu, COMPG_FN=compute_G_gpu)
    if p.collision_model == "lb":
        h.LOGGRAD_FN = eval_loggrad_gpu
    else:
        if p.gpu_fp32:
            h.COLLISION_FN = compute_collision_gpu32
        else:
            h.COLLISION_FN = compute_collision_gpu
            h.COLLMETRIC_FN = compute_collision_metric_gpu
    return h


class Batch:
    """Many independent ensembles advanced together (co_batch_*): one engine,
    one stream, one batched pair-sum launch per Picard iteration for all Landau
    instances, CUDA-graph replay of the iteration. `instances` is a list of
    dicts with keys bp1, bp2, model ("landau" | "lb"), nu, N. Marker arrays are
    torch CUDA tensors of the concatenated per-instance (2, N_i) blocks."""

    def __init__(self, instances, n_quad: int = 6, device: int = 0):
        self.lib = load_library()
        self._keep = []
        arr = (CoBatchInstance * len(instances))()
        for k, d in enumerate(instances):
            b1 = np.ascontiguousarray(d["bp1"], dtype=np.float64)
            b2 = np.ascontiguousarray(d["bp2"], dtype=np.float64)
            self._keep += [b1, b2]
            arr[k] = CoBatchInstance(_p(b1), len(b1), _p(b2), len(b2),
                                     CO_MODEL_LB if d.get("model") == "lb" else CO_MODEL_LANDAU,
                                     float(d.get("nu", 1.0)), int(d["N"]))
        h = C.c_void_p()
        self.h = None
        _check(self.lib.co_batch_create(arr, len(instances), n_quad, 0, device, C.byref(h)),
               "co_batch_create")
        self.h = h
        self.n = len(instances)
        self.N = [int(d["N"]) for d in instances]
        self.offsets = np.concatenate([[0], np.cumsum(self.N)]).astype(np.int64)

    def close(self):
        if self.h is not None:
            self.lib.co_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tune(self):
        W, KC, grid = C.c_int(), C.c_int(), C.c_int()
        ms = C.c_double()
        _check(self.lib.co_batch_tune(self.h, C.byref(W), C.byref(KC), C.byref(grid),
                                      C.byref(ms)), "co_batch_tune")
        return dict(warps=W.value, chunk=KC.value, grid=grid.value, pair_ms=ms.value)

    def entropy(self, v, w):
        S = np.zeros(self.n)
        _check(self.lib.co_batch_entropy_dev(self.h, v.data_ptr(), w.data_ptr(), _p(S)),
               "co_batch_entropy_dev")
        return S

    def predictor(self, opts: CoOpts, v1, v, w, dt: float):
        _check(self.lib.co_batch_predictor_dev(self.h, C.byref(opts), v1.data_ptr(), v.data_ptr(),
                                               w.data_ptr(), dt), "co_batch_predictor_dev")

    def step(self, opts: CoOpts, v1, v0, w, S0, dt: float, use_graph: bool = True):
        S0 = np.ascontiguousarray(S0, dtype=np.float64)
        it = (C.c_int * self.n)()
        res = np.zeros(self.n)
        _check(self.lib.co_batch_step_dev(self.h, C.byref(opts), v1.data_ptr(), v0.data_ptr(),
                                          w.data_ptr(), _p(S0), dt, int(use_graph), it, _p(res)),
               "co_batch_step_dev")
        return list(it), res

    def launch_count(self) -> int:
        n = C.c_ulonglong()
        _check(self.lib.co_batch_launch_count(self.h, C.byref(n)), "co_batch_launch_count")
        return n.value
