"""GPU parity of every hook and of the Picard map / Anderson step against the
CPU FP64 oracle, called through the C ABI (ctypes).

Tolerances:
  - FP64 stage outputs (coefficients, r, S, G, g, vdot): max-abs error
    <= 1e-12 * max-abs of the oracle value (normwise relative).
  - Picard map velocities: ||v_out^gpu - v_out^oracle||_inf /
    ||v_out^oracle||_inf <= 1e-12 (the per-RHS bar of the FP64 form).
  - LB velocities: the same 1e-12. g = grad f_s / f_s (functions.jl:37-64)
    multiplies the FP64 round-off of f_s by 1/f_s in the tails; two correct
    FP64 mass solves in the oracle (2D banded Cholesky and the tensor-product
    1D solve) move the LB map by 8e-14 (C1) and 4e-15 (C2) relative, so the
    per-RHS bar holds with room (test_oracle.py::test_two_mass_solves_spread).
  - Mixed FP32 pair sum: normwise relative 1e-5 on vdot.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import gaussian_markers, uniform_bp

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL_LB = TOL64


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    s = np.max(np.abs(b))
    return np.max(np.abs(a - b)) / (s if s > 0 else 1.0)


CASES = {
    "c1": dict(lo=-6.0, hi=6.0, n=16, N=2048, sx=1.0, sy=0.5, peak=0.0),
    "c2": dict(lo=-8.0, hi=8.0, n=32, N=16384, sx=np.sqrt(0.5), sy=np.sqrt(0.5), peak=2.0),
}


@pytest.fixture(scope="module", params=["c1", "c2"])
def setup(request, built_lib, oracle_mod, collops_mod):
    c = CASES[request.param]
    bp = uniform_bp(c["lo"], c["hi"], c["n"])
    p = collops_mod.SimParameters(bp1=bp, bp2=bp)
    ws = collops_mod.build_workspace(p)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    v, w = gaussian_markers(c["N"], c["sx"], c["sy"], seed=11, peak=c["peak"])
    yield dict(ws=ws, om=om, v=v, w=w, bp=bp, name=request.param, p=p)
    ws.close()


def test_l2_project(setup, collops_mod):
    ws, om, v, w = setup["ws"], setup["om"], setup["v"], setup["w"]
    f = np.zeros(ws.n_dofs)
    collops_mod.l2_project_gpu(ws, f, v, w)
    assert rel(f, om.l2_project(v, w)) < TOL64


def test_projection_deterministic(setup, collops_mod):
    ws, v, w = setup["ws"], setup["v"], setup["w"]
    f1 = np.zeros(ws.n_dofs)
    f2 = np.zeros(ws.n_dofs)
    collops_mod.l2_project_gpu(ws, f1, v, w)
    collops_mod.l2_project_gpu(ws, f2, v, w)
    assert np.array_equal(f1, f2)


def test_r_entropy_mass(setup, collops_mod):
    ws, om, v, w = setup["ws"], setup["om"], setup["v"], setup["w"]
    f = om.l2_project(v, w)
    r = np.zeros(ws.n_dofs)
    collops_mod.compute_r_gpu(ws, r, f)
    r_ref = om.compute_r(f)
    assert rel(r, r_ref) < TOL64
    S = collops_mod.compute_entropy_gpu(ws, f)
    assert abs(S - om.entropy(f)) < TOL64 * abs(om.entropy(f))
    L = np.zeros(ws.n_dofs)
    collops_mod.mass_solve_gpu(ws, L, r_ref)
    assert rel(L, om.mass_solve(r_ref)) < TOL64


def test_grad_and_loggrad(setup, collops_mod):
    ws, om, v, w = setup["ws"], setup["om"], setup["v"], setup["w"]
    f = om.l2_project(v, w)
    L = om.mass_solve(om.compute_r(f))
    G = np.zeros((v.shape[0], 2), order="F")
    collops_mod.compute_G_gpu(ws, G, v, L)
    assert rel(G, om.compute_G(v, L)) < TOL64
    g = np.zeros((v.shape[0], 2), order="F")
    collops_mod.eval_loggrad_gpu(ws, g, v, f)
    assert rel(g, om.loggrad(v, f)) < TOL64


def _G(om, v, w):
    f = om.l2_project(v, w)
    return om.compute_G(v, om.mass_solve(om.compute_r(f)))


def test_collision_fp64(setup, collops_mod):
    ws, om, v, w = setup["ws"], setup["om"], setup["v"], setup["w"]
    G = _G(om, v, w)
    dv = np.zeros((v.shape[0], 2), order="F")
    collops_mod.compute_collision_gpu(ws, dv, v, w, G)
    ref = om.collision(v, w, G)
    assert rel(dv, ref) < TOL64
    # conservation of momentum and energy (exact identities of the pair sum)
    scale = np.max(np.abs(dv))
    assert abs(np.sum(w * dv[:, 0])) < 1e-12 * scale
    assert abs(np.sum(w * dv[:, 1])) < 1e-12 * scale
    assert abs(np.sum(w * (v[:, 0] * dv[:, 0] + v[:, 1] * dv[:, 1]))) < 1e-12 * scale * np.max(np.abs(v))


def test_collision_metric(setup, collops_mod):
    ws, om, v, w = setup["ws"], setup["om"], setup["v"], setup["w"]
    G = _G(om, v, w)
    N = v.shape[0]
    F = np.zeros((N, 2), order="F")
    A = np.zeros((N, 3), order="F")
    collops_mod.compute_collision_metric_gpu(ws, F, A, v, w, G)
    Fr, Ar = om.collision_metric(v, w, G)
    assert rel(F, Fr) < TOL64
    assert rel(A, Ar) < TOL64
    # F of the metric kernel agrees with the plain kernel to round-off
    F0 = np.zeros((N, 2), order="F")
    collops_mod.compute_collision_gpu(ws, F0, v, w, G)
    assert rel(F, F0) < 1e-14


@pytest.mark.parametrize("fp32", [False, True])
def test_symmetric_vs_onesided(setup, collops_mod, fp32):
    """Newton's-third-law kernels against the one-sided kernels (same inputs)."""
    om, v, w = setup["om"], setup["v"], setup["w"]
    G = _G(om, v, w)
    out = {}
    for ones in (False, True):
        p = collops_mod.SimParameters(bp1=setup["bp"], bp2=setup["bp"], gpu_fp32=fp32,
                                      pair_onesided=ones)
        ws = collops_mod.build_workspace(p)
        dv = np.zeros((v.shape[0], 2), order="F")
        collops_mod.compute_collision_gpu(ws, dv, v, w, G)
        dv2 = np.zeros((v.shape[0], 2), order="F")
        collops_mod.compute_collision_gpu(ws, dv2, v, w, G)
        ws.close()
        assert np.array_equal(dv, dv2)            # deterministic
        out[ones] = dv
    assert rel(out[False], out[True]) < (1e-6 if fp32 else 1e-14)
    if not fp32:
        # conservation is exact in the symmetric form up to summation round-off
        s = out[False]
        assert abs(np.sum(w * s[:, 0])) < 1e-13 * np.max(np.abs(s))


def test_picard_map_double_single(setup, collops_mod, oracle_mod):
    """One Landau Picard map with the double-single pair kernel (FP32 head+tail
    arithmetic, ~44 bits) against the FP64 oracle: 1e-11 relative on v_out."""
    om, v, w = setup["om"], setup["v"], setup["w"]
    p = collops_mod.SimParameters(bp1=setup["bp"], bp2=setup["bp"])
    ws = collops_mod.build_workspace(p)
    o = oracle_mod.Opts()
    dt = 0.05
    S0 = om.entropy(om.l2_project(v, w))
    v_in = om.predictor(o, v, w, dt)
    out = np.zeros_like(v, order="F")
    collops_mod.picard_map(ws, out, v_in, v, w, S0, dt, precision="mixed_ds")
    ws.close()
    ref = om.picard_map(o, v_in, v, w, S0, dt)
    assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) < 1e-11
    # the vdot error itself, relative to max |vdot|
    assert np.max(np.abs(out - ref)) / (dt * np.max(np.abs(ref - v))) < 1e-9


def test_collision_mixed(setup, collops_mod, oracle_mod):
    om, v, w = setup["om"], setup["v"], setup["w"]
    p = collops_mod.SimParameters(bp1=setup["bp"], bp2=setup["bp"], gpu_fp32=True)
    ws32 = collops_mod.build_workspace(p)
    G = _G(om, v, w)
    dv = np.zeros((v.shape[0], 2), order="F")
    collops_mod.compute_collision_gpu32(ws32, dv, v, w, G)
    ws32.close()
    assert rel(dv, om.collision(v, w, G)) < 1e-5


@pytest.mark.parametrize("model", ["landau", "lb"])
@pytest.mark.parametrize("gonzalez", [True, False])
def test_picard_map(setup, collops_mod, oracle_mod, model, gonzalez):
    om, v, w = setup["om"], setup["v"], setup["w"]
    p = collops_mod.SimParameters(bp1=setup["bp"], bp2=setup["bp"], collision_model=model)
    ws = collops_mod.build_workspace(p)
    o = oracle_mod.Opts(model=model, use_gonzalez=gonzalez)
    dt = 0.05
    S0 = om.entropy(om.l2_project(v, w))
    v_in = om.predictor(o, v, w, dt)
    out = np.zeros_like(v, order="F")
    collops_mod.picard_map(ws, out, v_in, v, w, S0, dt, use_gonzalez=gonzalez)
    ref = om.picard_map(o, v_in, v, w, S0, dt)
    ws.close()
    tol = TOL_LB if model == "lb" else TOL64
    assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) < tol


def lb_predictor_sensitivity(oracle_mod, om, v, w, dt, trials=3):
    """How far the oracle's LB predictor moves (relative to max|v1|) when the
    projection coefficients f_s move by one unit round-off of max|f_s| -- the
    error model of any FP64 scatter and mass solve. g = grad f_s / f_s divides
    by f_s, so at a marker where f_s undershoots to ~0 this is far above 1e-16."""
    f = om.l2_project(v, w)

    def pred(fc):
        g = om.loggrad(v, fc)
        n, U1, U2, Q = oracle_mod.moments(v, w)
        A1, A2, B = oracle_mod.drift_multipliers(v, w, g, n, U1, U2, Q)
        return v + dt * oracle_mod.lb_velocity(v, g, A1, A2, B, 1.0)
    p0 = pred(f)
    rng = np.random.default_rng(0)
    eps = np.finfo(np.float64).eps * np.max(np.abs(f))
    return max(np.max(np.abs(pred(f + eps * rng.choice([-1.0, 1.0], f.size)) - p0)) /
               np.max(np.abs(p0)) for _ in range(trials))


@pytest.mark.parametrize("model", ["landau", "lb"])
def test_predictor(setup, collops_mod, oracle_mod, model):
    """Explicit predictor v1 = v + dt vdot(v) (main.jl:233-245). Landau: 1e-12.
    LB evaluates g = grad f_s / f_s at the markers themselves, where a Gibbs
    undershoot of f_s can sit next to a marker: its tolerance is
    max(1e-12, 8 x the predictor's change under a one-ulp perturbation of f_s),
    i.e. a scatter-plus-solve round-off budget of 8 ulps of max|f_s| (measured
    sensitivity 5e-13 at C2, GPU error 1.7e-12)."""
    om, v, w = setup["om"], setup["v"], setup["w"]
    p = collops_mod.SimParameters(bp1=setup["bp"], bp2=setup["bp"], collision_model=model)
    ws = collops_mod.build_workspace(p)
    o = oracle_mod.Opts(model=model)
    v1 = np.zeros_like(v, order="F")
    collops_mod.predictor(ws, v1, v, w, 0.05)
    ws.close()
    ref = om.predictor(o, v, w, 0.05)
    tol = TOL64
    if model == "lb":
        tol = max(TOL64, 8.0 * lb_predictor_sensitivity(oracle_mod, om, v, w, 0.05))
    err = np.max(np.abs(v1 - ref)) / np.max(np.abs(ref))
    assert err < tol, (err, tol)


@pytest.mark.parametrize("model", ["landau", "lb"])
def test_step_anderson_c1(built_lib, oracle_mod, collops_mod, model):
    """One implicit step against the oracle's step_anderson!: configuration 1
    (16x16, N=2048, Anderson depth 5, tol 1e-12). Landau with Gonzalez at
    dt=0.02; at the configuration's dt=0.05 Anderson stagnates for some seeds
    in the oracle as well, and two stagnating trajectories are chaotic. LB at
    dt=0.01 without Gonzalez (with Gonzalez, LB stagnates on this mesh in the
    reference formulation as well: lambda jumps where the entropy integrand's
    f_s -> 0+ quadrature points move)."""
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=5)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    gz = model == "landau"
    dt = 0.02 if model == "landau" else 0.01
    o = oracle_mod.Opts(model=model, m=5, tol=1e-12, abs_floor=0.0, damping=0.7,
                        max_iter=400, use_gonzalez=gz)
    S0 = om.entropy(om.l2_project(v, w))
    v1 = om.predictor(o, v, w, dt)
    ref, info_ref = om.step_anderson(o, v1, v, w, S0, dt)
    p = collops_mod.SimParameters(bp1=bp, bp2=bp, collision_model=model)
    ws = collops_mod.build_workspace(p)
    x = np.array(v1, order="F", copy=True)
    info = collops_mod.step_anderson(ws, x, v, w, S0, dt, m=5, tol=1e-12, abs_floor=0.0,
                                     damping=0.7, max_iter=400, use_gonzalez=gz)
    ws.close()
    # both solves converge (not a stagnation exit) to the same fixed point
    assert info_ref[0] < 400 and info[0] < 400
    assert info[1] < 1e-12 * np.linalg.norm(x) and info_ref[1] < 1e-12 * np.linalg.norm(ref)
    assert abs(info[0] - info_ref[0]) <= max(3, info_ref[0] // 10)
    assert np.max(np.abs(x - ref)) / np.max(np.abs(ref)) < 1e-10
    # conservation across the step (exit_picard_step = true)
    p0 = np.array([np.sum(w * v[:, 0]), np.sum(w * v[:, 1])])
    p1 = np.array([np.sum(w * x[:, 0]), np.sum(w * x[:, 1])])
    E0 = 0.5 * np.sum(w * (v ** 2).sum(1))
    E1 = 0.5 * np.sum(w * (x ** 2).sum(1))
    assert np.max(np.abs(p1 - p0)) < 1e-12
    assert abs(E1 - E0) < 1e-12 * E0


@pytest.mark.parametrize("precision", ["mixed", "mixed_ds"])
def test_step_anderson_mixed_c1(built_lib, oracle_mod, collops_mod, precision):
    """Mixed-precision step_anderson!: FP32 pair maps, then Anderson on the
    FP64-accurate (FP64 or double-single) map to the same tolerance. The result
    is a fixed point of the oracle's FP64 map and conserves momentum and energy."""
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=5)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    dt = 0.02
    o = oracle_mod.Opts(model="landau", m=5, tol=1e-12, abs_floor=0.0, damping=0.7,
                        max_iter=400)
    S0 = om.entropy(om.l2_project(v, w))
    v1 = om.predictor(o, v, w, dt)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp))
    x = np.array(v1, order="F", copy=True)
    info = collops_mod.step_anderson(ws, x, v, w, S0, dt, m=5, tol=1e-12, abs_floor=0.0,
                                     damping=0.7, max_iter=400, precision=precision)
    ws.close()
    assert info[0] < 400 and info[1] < 1e-12 * np.linalg.norm(x)
    assert np.linalg.norm(om.picard_map(o, x, v, w, S0, dt) - x) < 1e-9
    E0 = 0.5 * np.sum(w * (v ** 2).sum(1))
    assert np.max(np.abs((w[:, None] * (x - v)).sum(0))) < 1e-12
    assert abs(0.5 * np.sum(w * (x ** 2).sum(1)) - E0) < 1e-12 * E0


@pytest.mark.parametrize("precision,precond", [("fp64", 0), ("fp64", 1), ("mixed_ds", 1)])
def test_step_defect_outer_anderson_c1(built_lib, oracle_mod, collops_mod, precision, precond):
    """Defect correction with Anderson mixing of the outer iterates (outer_m = 5),
    with and without the block-Newton inner preconditioner. FP64 with the FP64
    metric follows the oracle's same algorithm to the same fixed point; the
    mixed form converges to an FP64 fixed point."""
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=5)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    dt = 0.02
    o = oracle_mod.Opts(model="landau", m=8, tol=1e-12, abs_floor=0.0, damping=0.7,
                        max_iter=200, stag_rel_tol=0.1)
    S0 = om.entropy(om.l2_project(v, w))
    v1 = om.predictor(o, v, w, dt)
    ref, info_ref = om.step_defect(o, v1, v, w, S0, dt, outer_m=5, precond=precond)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp))
    x = np.array(v1, order="F", copy=True)
    info = collops_mod.step_defect(ws, x, v, w, S0, dt, m=8, tol=1e-12, abs_floor=0.0,
                                   damping=0.7, max_iter=200, metric64=precision == "fp64",
                                   precision=precision, outer_m=5, precond=precond)
    ws.close()
    assert info[0] < 200 and info[1] < 1e-12 * np.linalg.norm(x)
    if precision == "fp64":
        assert abs(info[0] - info_ref[0]) <= 2
        assert np.max(np.abs(x - ref)) / np.max(np.abs(ref)) < 1e-10
    assert np.linalg.norm(om.picard_map(o, x, v, w, S0, dt) - x) < 1e-9
    E0 = 0.5 * np.sum(w * (v ** 2).sum(1))
    assert np.max(np.abs((w[:, None] * (x - v)).sum(0))) < 1e-12
    assert abs(0.5 * np.sum(w * (x ** 2).sum(1)) - E0) < 1e-12 * E0


def test_step_defect_metric_freeze_c1(built_lib, oracle_mod, collops_mod):
    """Freezing the FP32 frozen metric once the outer residual has fallen 100x
    changes only the inner model: the mixed-precision step still converges to a
    fixed point of the oracle's FP64 map and conserves momentum and energy."""
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=5)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    dt = 0.02
    o = oracle_mod.Opts(model="landau", m=8, tol=1e-12, abs_floor=0.0, damping=0.7,
                        max_iter=200, stag_rel_tol=0.1)
    S0 = om.entropy(om.l2_project(v, w))
    v1 = om.predictor(o, v, w, dt)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp))
    for freeze in (0.0, 1e-2):
        x = np.array(v1, order="F", copy=True)
        info = collops_mod.step_defect(ws, x, v, w, S0, dt, m=8, tol=1e-12, abs_floor=0.0,
                                       damping=0.7, max_iter=200, metric64=False,
                                       precision="mixed_ds", metric_freeze=freeze)
        assert info[0] < 200 and info[1] < 1e-12 * np.linalg.norm(x)
        assert np.linalg.norm(om.picard_map(o, x, v, w, S0, dt) - x) < 1e-9
        E0 = 0.5 * np.sum(w * (v ** 2).sum(1))
        assert np.max(np.abs((w[:, None] * (x - v)).sum(0))) < 1e-12
        assert abs(0.5 * np.sum(w * (x ** 2).sum(1)) - E0) < 1e-12 * E0
    ws.close()


@pytest.mark.parametrize("logsq", [False, True])
def test_diagnostics_c2(built_lib, oracle_mod, collops_mod, logsq):
    """Post-step diagnostics (entropy, energy, momentum, ||f_s - f_p||_2,
    negative-part L1) against the oracle, bimodal markers on [-8,8]^2 with a
    32x32 mesh (the tails give a nonzero negative part)."""
    bp = uniform_bp(-8.0, 8.0, 32)
    rng = np.random.default_rng(21)
    N = 16384
    v = np.zeros((N, 2), order="F")
    v[:, 0] = np.where(np.arange(N) < N // 2, -2.0, 2.0) + np.sqrt(0.5) * rng.standard_normal(N)
    v[:, 1] = np.sqrt(0.5) * rng.standard_normal(N)
    w = np.full(N, 1.0 / N)
    om = oracle_mod.OracleMesh(bp, bp, 6, use_logsq=logsq)
    ref = om.diagnostics(v, w)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp, use_logsq=logsq))
    d = collops_mod.diagnostics(ws, v, w)
    ws.close()
    got = np.array([d["entropy"], d["energy"], *d["momentum"], d["fs_minus_fp_l2"],
                    d["negative_part_l1"]])
    assert ref[5] > 0.0
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-15)


def test_step_defect_c1(built_lib, oracle_mod, collops_mod):
    """step_defect! against the oracle's (same algorithm, FP64 metric): the same
    fixed point. The implicit step can have several fixed points (two solvers
    from the same guess may land on different ones), so the comparison is
    between runs of the same algorithm."""
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=5)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    dt = 0.02
    o = oracle_mod.Opts(model="landau", m=8, tol=1e-12, abs_floor=0.0, damping=0.7,
                        max_iter=200, stag_rel_tol=0.1)
    S0 = om.entropy(om.l2_project(v, w))
    v1 = om.predictor(o, v, w, dt)
    ref, info_ref = om.step_defect(o, v1, v, w, S0, dt)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp))
    x = np.array(v1, order="F", copy=True)
    info = collops_mod.step_defect(ws, x, v, w, S0, dt, m=8, tol=1e-12, abs_floor=0.0,
                                   damping=0.7, max_iter=200, metric64=True)
    # GB300 form: FP32 metric (changes only the inner model)
    x32 = np.array(v1, order="F", copy=True)
    info32 = collops_mod.step_defect(ws, x32, v, w, S0, dt, m=8, tol=1e-12, abs_floor=0.0,
                                     damping=0.7, max_iter=200, metric64=False)
    # mixed: FP32 outer maps first, then FP64 outer maps to the same stopping rule
    xm = np.array(v1, order="F", copy=True)
    infom = collops_mod.step_defect(ws, xm, v, w, S0, dt, m=8, tol=1e-12, abs_floor=0.0,
                                    damping=0.7, max_iter=200, metric64=False, precision="mixed")
    ws.close()
    assert info_ref[0] < 200 and info[0] < 200
    assert abs(info[0] - info_ref[0]) <= 2
    assert np.max(np.abs(x - ref)) / np.max(np.abs(ref)) < 1e-10
    E0 = 0.5 * np.sum(w * (v ** 2).sum(1))
    xd = np.array(v1, order="F", copy=True)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp))
    infod = collops_mod.step_defect(ws, xd, v, w, S0, dt, m=8, tol=1e-12, abs_floor=0.0,
                                    damping=0.7, max_iter=200, metric64=False,
                                    precision="mixed_ds")
    ws.close()
    for xx, inf in ((x32, info32), (xm, infom), (xd, infod)):
        assert inf[0] < 200 and inf[1] < 1e-12 * np.linalg.norm(xx)
        # an FP64 fixed point of the map (exit Picard update included)
        assert np.linalg.norm(om.picard_map(o, xx, v, w, S0, dt) - xx) < 1e-9
        assert np.max(np.abs((w[:, None] * (xx - v)).sum(0))) < 1e-12
        assert abs(0.5 * np.sum(w * (xx ** 2).sum(1)) - E0) < 1e-12 * E0


def test_step_deterministic(built_lib, collops_mod, oracle_mod):
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=7)
    p = collops_mod.SimParameters(bp1=bp, bp2=bp)
    ws = collops_mod.build_workspace(p)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    S0 = om.entropy(om.l2_project(v, w))
    outs = []
    for _ in range(2):
        x = np.zeros_like(v, order="F")
        collops_mod.predictor(ws, x, v, w, 0.05)
        info = collops_mod.step_anderson(ws, x, v, w, S0, 0.05, m=5, tol=1e-12, abs_floor=0.0,
                                         damping=0.7, max_iter=400)
        outs.append((x, info))
    ws.close()
    assert np.array_equal(outs[0][0], outs[1][0])
    assert outs[0][1] == outs[1][1]


def test_edge_cases(built_lib, collops_mod, oracle_mod):
    bp = uniform_bp(-6.0, 6.0, 16)
    p = collops_mod.SimParameters(bp1=bp, bp2=bp)
    ws = collops_mod.build_workspace(p)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    # N = 0
    e = np.zeros((0, 2), order="F")
    collops_mod.compute_collision_gpu(ws, e.copy(order="F"), e, np.zeros(0), e)
    f = np.zeros(ws.n_dofs)
    collops_mod.l2_project_gpu(ws, f, e, np.zeros(0))
    assert np.all(f == 0)
    # N = 1 and markers on / outside the boundary, plus an exact duplicate pair
    v = np.array([[0.1, 0.2], [6.0, 0.0], [-7.0, 1.0], [0.3, -0.2], [0.3, -0.2], [1.0, 1.0]],
                 order="F")
    w = np.array([0.1, 0.2, 0.3, 0.15, 0.15, 0.1])
    G = np.array([[1.0, -2.0], [0.5, 0.5], [3.0, 1.0], [0.2, 0.1], [-0.4, 0.7], [0.0, 1.0]],
                 order="F")
    for n in (1, 6):
        dv = np.zeros((n, 2), order="F")
        collops_mod.compute_collision_gpu(ws, dv, v[:n], w[:n], G[:n])
        ref = om.collision(v[:n], w[:n], G[:n])
        assert np.allclose(dv, ref, rtol=1e-13, atol=1e-15)
    assert np.all(dv[1] == 0) and np.all(dv[2] == 0)   # out-of-domain markers
    f = np.zeros(ws.n_dofs)
    collops_mod.l2_project_gpu(ws, f, v, w)
    assert rel(f, om.l2_project(v, w)) < TOL64
    # NaN input -> status CO_ERR_NONFINITE, no trap
    bad = v.copy(order="F")
    bad[0, 0] = np.nan
    with pytest.raises(collops_mod.CollopsError) as ei:
        collops_mod.compute_collision_gpu(ws, np.zeros((6, 2), order="F"), bad, w, G)
    assert ei.value.status == 4
    ws.close()
    # P_DEG != 2 -> unsupported
    with pytest.raises(collops_mod.CollopsError) as ei:
        collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp, P_DEG=3))
    assert ei.value.status == 3


def test_launch_counter_moves(built_lib, collops_mod):
    bp = uniform_bp(-6.0, 6.0, 16)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp))
    v, w = gaussian_markers(512, seed=1)
    n0 = ws.launch_count()
    f = np.zeros(ws.n_dofs)
    collops_mod.l2_project_gpu(ws, f, v, w)
    assert ws.launch_count() > n0
    ws.close()


@pytest.mark.parametrize("precision,outer_m,precond", [("fp64", 0, 0), ("mixed_ds", 5, 1)])
def test_step_defect_device_loop_matches_host_loop(built_lib, collops_mod, monkeypatch,
                                                   precision, outer_m, precond):
    """The inner Anderson loop of step_defect! runs on the device (one CUDA graph
    whose body repeats under a conditional node) unless COLLOPS_INNER_LOOP=host
    selects the host-driven loop. Both launch the same kernels on the same data
    in the same order, so the steps agree bit for bit, with the same outer and
    inner iteration counts."""
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=5)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp))
    f = np.zeros(ws.n_dofs)
    collops_mod.l2_project_gpu(ws, f, v, w)
    S0 = collops_mod.compute_entropy_gpu(ws, f)
    dt = 0.02
    v1 = np.zeros((2048, 2), order="F")
    collops_mod.predictor(ws, v1, v, w, dt)
    out = {}
    for mode in ("device", "host"):
        if mode == "host":
            monkeypatch.setenv("COLLOPS_INNER_LOOP", "host")
        else:
            monkeypatch.delenv("COLLOPS_INNER_LOOP", raising=False)
        x = np.array(v1, order="F", copy=True)
        info = collops_mod.step_defect(ws, x, v, w, S0, dt, m=8, tol=1e-12, abs_floor=0.0,
                                       damping=0.7, max_iter=200,
                                       metric64=precision == "fp64", precision=precision,
                                       outer_m=outer_m, precond=precond)
        out[mode] = (x, info)
    ws.close()
    (xd, infod), (xh, infoh) = out["device"], out["host"]
    print(f"device {infod} host {infoh}")
    assert infod[0] == infoh[0] and infod[2] == infoh[2] and infod[1] == infoh[1]
    assert np.array_equal(xd, xh)
