"""CPU tests of the C-ABI boundary and the host-side mirror (no GPU needed).

- the library builds for sm_103a, loads, and exports every entry point that
  include/collops.h declares (no compute calls);
- status codes come back as statuses (no device: CO_ERR_NODEVICE; bad
  arguments: CO_ERR_ARG; P_DEG != 2: CO_ERR_UNSUPPORTED) rather than crashes;
- parse_overrides behaves like the reference's (main_helpers.jl:63-72).
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, cuda_available

HEADER = os.path.join(ROOT, "include", "collops.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(co_[A-Za-z0-9_]+)\s*\(", txt)))


def test_header_declares_hooks():
    syms = declared_symbols()
    for s in ("co_ctx_create", "co_collision", "co_collision_metric", "co_l2_project",
              "co_grad_L", "co_loggrad", "co_step_anderson", "co_picard_map"):
        assert s in syms


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_mirror_binds_every_symbol(built_lib, collops_mod):
    lib = collops_mod.load_library()
    assert lib.co_version() == 1
    for s in declared_symbols():
        assert s in collops_mod._SIGNATURES, f"{s} not bound in collops"


def test_strerror_and_status_codes(built_lib, collops_mod):
    lib = collops_mod.load_library()
    assert lib.co_strerror(0) == b"ok"
    assert b"P_DEG" in lib.co_strerror(3)
    h = C.c_void_p()
    bp = np.linspace(-6, 6, 17)
    dp = bp.ctypes.data_as(C.POINTER(C.c_double))
    # invalid arguments are rejected before any device work
    assert lib.co_ctx_create(dp, 1, dp, 17, 2, 6, 0, 0, C.byref(h)) == 1
    assert lib.co_ctx_create(dp, 17, dp, 17, 2, 0, 0, 0, C.byref(h)) == 1
    assert lib.co_ctx_create(dp, 17, dp, 17, 3, 6, 0, 0, C.byref(h)) == 3
    bad = np.array([0.0, 1.0, 1.0, 2.0])  # non-increasing breakpoints
    bdp = bad.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.co_ctx_create(bdp, 4, dp, 17, 2, 6, 0, 0, C.byref(h)) == 1
    assert lib.co_collision(None, None, None, None, None, 0) == 1
    if not cuda_available():
        assert lib.co_ctx_create(dp, 17, dp, 17, 2, 6, 0, 0, C.byref(h)) == 7


def test_opts_struct_layout(collops_mod):
    # co_opts: 18 fields, natural alignment (x86-64 and aarch64 LP64): 128 bytes
    assert C.sizeof(collops_mod.CoOpts) == 128
    o = collops_mod.SimParameters().opts()
    assert o.m == 8 and o.tol == 1e-12 and o.model == 0


def test_parse_overrides(collops_mod):
    """main_helpers.jl:63-72 restated on the Python mirror."""
    base = collops_mod.SimParameters(suffix="base")
    p = collops_mod.parse_overrides(base, ["--suffix=run2", "--DT=0.004", "--N_STEPS=300"])
    assert p.suffix == "run2" and p.DT == 0.004 and p.N_STEPS == 300
    assert p.N_PARTICLES == base.N_PARTICLES
    assert collops_mod.parse_overrides(base, []) is base
    with pytest.raises(ValueError):
        collops_mod.parse_overrides(base, ["--no_such_field=1"])
    with pytest.raises(ValueError):
        collops_mod.parse_overrides(base, ["--bp1=1"])
    q = collops_mod.parse_overrides(base, ["--use_gonzalez=0", "--gpu_fp32=true",
                                           "--collision_model=lb"])
    assert q.use_gonzalez is False and q.gpu_fp32 is True and q.collision_model == "lb"


def test_enable_gpu_hook_selection(collops_mod):
    """enable_gpu! (main.jl:390-423): which hooks are repointed."""
    h = collops_mod.enable_gpu(collops_mod.SimParameters())
    assert h.COLLISION_FN is collops_mod.compute_collision_gpu
    assert h.COLLMETRIC_FN is collops_mod.compute_collision_metric_gpu
    assert h.L2PROJ_FN is collops_mod.l2_project_gpu and h.COMPG_FN is collops_mod.compute_G_gpu
    h = collops_mod.enable_gpu(collops_mod.SimParameters(gpu_fp32=True))
    assert h.COLLISION_FN is collops_mod.compute_collision_gpu32 and h.COLLMETRIC_FN is None
    h = collops_mod.enable_gpu(collops_mod.SimParameters(collision_model="lb"))
    assert h.LOGGRAD_FN is collops_mod.eval_loggrad_gpu and h.COLLISION_FN is None
    with pytest.raises(collops_mod.CollopsError):
        collops_mod.enable_gpu(collops_mod.SimParameters(P_DEG=3))


def test_output_layout_checked(collops_mod):
    """Outputs must be column-major float64 (Julia layout); checked before any call."""
    with pytest.raises(ValueError):
        collops_mod._out(np.zeros((4, 2)), (4, 2), "dot_v")   # C order
    collops_mod._out(np.zeros((4, 2), order="F"), (4, 2), "dot_v")


def test_conservation_row_layout(collops_mod):
    """conservation_row writes the reference's CONS_COLS in order (io.jl)."""
    assert collops_mod.CONS_COLS == ("step", "time", "entropy", "energy", "momentum_1",
                                     "momentum_2", "iter", "residual", "fp_minus_fs",
                                     "neg_part", "r0", "dt")
    d = dict(entropy=2.5, energy=0.625, momentum=(1e-17, -2e-17), fs_minus_fp_l2=0.1,
             negative_part_l1=0.002)
    row = collops_mod.conservation_row(3, 0.06, d, 18, 3e-10, 6.5, 0.02)
    fields = row.split(",")
    assert len(fields) == len(collops_mod.CONS_COLS)
    assert fields[0] == "3" and fields[6] == "18"
    assert float(fields[2]) == 2.5 and float(fields[5]) == -2e-17 and float(fields[11]) == 0.02


def test_checkpoint_roundtrip(collops_mod, tmp_path):
    """save_checkpoint / load_checkpoint keep the reference's fields (io.jl:53-86,
    169-182) and the Julia N x 2 column-major marker layout; step="auto" picks
    the highest step."""
    rng = np.random.default_rng(3)
    N = 257
    v = np.asfortranarray(rng.standard_normal((N, 2)))
    w = np.full(N, 1.0 / N)
    f = rng.standard_normal(324)
    hist = dict(entropy_history=[1.0, 1.1], energy_history=[0.6, 0.6],
                momentum_history=[(0.0, 0.1), (0.0, 0.1)], iter_history=[0, 17],
                res_history=[0.0, 3e-10], fp_l2_history=[0.1, 0.09], neg_history=[0.0, 1e-5])
    for step in (25, 50):
        collops_mod.save_checkpoint("run", step, 0.02 * step, v, w, f, directory=str(tmp_path),
                                    **hist)
    d = collops_mod.load_checkpoint("run", "auto", directory=str(tmp_path))
    assert d["step"] == 50 and d["t"] == 1.0
    assert tuple(d) == collops_mod.CHECKPOINT_FIELDS
    assert np.array_equal(d["v_particles"], v) and d["v_particles"].flags.f_contiguous
    assert np.array_equal(d["f_coeffs"], f) and d["momentum_history"].shape == (2, 2)
    assert list(d["iter_history"]) == [0, 17]
    assert collops_mod.load_checkpoint("run", 25, directory=str(tmp_path))["step"] == 25


def _header_structs():
    """{typedef name: [(C type, field name, array length or 0)]} of the plain
    typedef structs in include/collops.h (comments stripped)."""
    import re
    src = open(os.path.join(ROOT, "include", "collops.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    out = {}
    for body, name in re.findall(r"typedef struct\s*\{(.*?)\}\s*(\w+)\s*;", src, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"(.*?)(\w+)\s*(?:\[(\d+)\])?$", decl)
            ctype, fname, n = m.group(1).strip(), m.group(2), int(m.group(3) or 0)
            fields.append((ctype, fname, n))
        out[name] = fields
    return out


@pytest.mark.parametrize("cname,pyname", [("co_opts", "CoOpts"),
                                          ("co_defect_opts", "CoDefectOpts"),
                                          ("co_newton_opts", "CoNewtonOpts"),
                                          ("co_step_info", "CoStepInfo")])
def test_ctypes_mirrors_match_header(collops_mod, cname, pyname):
    """The Python mirrors of the option and record structs have the header's
    fields, in its order, with its types (a field added on one side only would
    shift every later field across the C ABI)."""
    ctypes_of = {"int": C.c_int, "double": C.c_double, "unsigned": C.c_uint,
                 "unsigned long long": C.c_ulonglong}
    hdr = _header_structs()[cname]
    py = getattr(collops_mod, pyname)._fields_
    assert [f for _, f, _ in hdr] == [f for f, _ in py]
    for (ctype, fname, n), (_, pytype) in zip(hdr, py):
        want = ctypes_of[ctype] * n if n else ctypes_of[ctype]
        assert C.sizeof(pytype) == C.sizeof(want) and (
            pytype == want or getattr(pytype, "_type_", None) == getattr(want, "_type_", None)), fname
