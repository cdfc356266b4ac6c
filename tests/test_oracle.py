"""CPU tests of the FP64 oracle: the reference's own known-answer tests
(test/integration/main_helpers.jl:13-61) plus exact identities of the method,
and the committed golden vectors.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import gaussian_markers, uniform_bp

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


# ---------------------------------------------------- reference known answers

def test_momentum_energy_known_answer(oracle_mod):
    """main_helpers.jl:13-26."""
    v = np.array([[1.0, 2.0], [-3.0, 0.5]])
    w = np.array([0.25, 0.75])
    p = oracle_mod.momentum(v, w)
    assert np.allclose(p, (0.25 * 1.0 + 0.75 * -3.0, 0.25 * 2.0 + 0.75 * 0.5))
    assert np.isclose(oracle_mod.energy(v, w),
                      0.5 * (0.25 * (1.0 ** 2 + 2.0 ** 2) + 0.75 * ((-3.0) ** 2 + 0.5 ** 2)))
    rng = np.random.default_rng(3)
    vr = rng.standard_normal((100, 2))
    wr = np.full(100, 1 / 100)
    assert np.isclose(oracle_mod.energy(vr, wr), np.sum(0.5 * (vr ** 2).sum(1)) / 100)


def test_compute_moments_known_answer(oracle_mod):
    """main_helpers.jl:28-38."""
    v = np.array([[1.0, 2.0], [-3.0, 0.5], [0.0, -1.0]])
    w = np.array([0.2, 0.3, 0.5])
    n, U1, U2, Q = oracle_mod.moments(v, w)
    assert np.isclose(n, 1.0)
    assert np.isclose(U1, 0.2 * 1.0 + 0.3 * -3.0)
    assert np.isclose(U2, 0.2 * 2.0 + 0.3 * 0.5 + 0.5 * -1.0)
    assert np.isclose(Q, 0.2 * 5.0 + 0.3 * 9.25 + 0.5 * 1.0)
    assert np.isclose(oracle_mod.energy(v, w), 0.5 * Q)


@pytest.mark.parametrize("N", [16, 257])
def test_lb_drift_conservation(oracle_mod, N):
    """main_helpers.jl:40-61 (seeded numpy RNG in place of MersenneTwister(2024))."""
    rng = np.random.default_rng(2024)
    v = np.asfortranarray(rng.standard_normal((N, 2)))
    w = rng.random(N)
    w /= w.sum()
    g = np.asfortranarray(rng.standard_normal((N, 2)))
    n, U1, U2, Q = oracle_mod.moments(v, w)
    A1, A2, B = oracle_mod.drift_multipliers(v, w, g, n, U1, U2, Q)
    dv = oracle_mod.lb_velocity(v, g, A1, A2, B, 1.0)
    scale = np.max(np.abs(dv))
    assert abs(np.sum(w * dv[:, 0])) < 1e-12 * scale
    assert abs(np.sum(w * dv[:, 1])) < 1e-12 * scale
    assert abs(np.sum(w * (v * dv).sum(1))) < 1e-12 * scale * np.max(np.abs(v))


# ---------------------------------------------------- FEM identities

@pytest.fixture(scope="module")
def mesh16(oracle_mod):
    bp = uniform_bp(-6.0, 6.0, 16)
    return oracle_mod.OracleMesh(bp, bp, 6), bp


def _mass1d(bp):
    """Independent 1D mass matrix of the clamped C1 quadratic B-splines via
    Cox-de Boor recursion and a 5-point Gauss rule per element."""
    n = len(bp) - 1
    t = np.concatenate([[bp[0]] * 3, bp[1:-1], [bp[-1]] * 3])
    nb = n + 2

    def basis(x):
        # degree-0 on the span containing x
        out = np.zeros(len(t) - 1)
        k = min(np.searchsorted(t, x, side="right") - 1, len(t) - 4)
        out[k] = 1.0
        for p in (1, 2):
            new = np.zeros(len(t) - 1 - p)
            for i in range(len(new)):
                a = (x - t[i]) / (t[i + p] - t[i]) * out[i] if t[i + p] > t[i] else 0.0
                b = (t[i + p + 1] - x) / (t[i + p + 1] - t[i + 1]) * out[i + 1] \
                    if t[i + p + 1] > t[i + 1] else 0.0
                new[i] = a + b
            out = new
        return out[:nb]

    xg, wg = np.polynomial.legendre.leggauss(5)
    M = np.zeros((nb, nb))
    for e in range(n):
        a, b = bp[e], bp[e + 1]
        for xq, wq in zip(xg, wg):
            x = a + (b - a) * (xq + 1) / 2
            phi = basis(x)
            M += np.outer(phi, phi) * wq * (b - a) / 2
    return M


def test_mass_matrix_is_kronecker_spd(oracle_mod):
    bp1 = np.array([-6.0, -5.0, -3.0, -2.5, 0.0, 1.0, 4.0, 6.0])   # non-uniform
    bp2 = uniform_bp(-4.0, 4.0, 5)
    om = oracle_mod.OracleMesh(bp1, bp2, 6)
    M = om.mass_matrix()
    M1, M2 = _mass1d(bp1), _mass1d(bp2)
    K = np.kron(M2, M1)          # first index fastest: gid = i1 + i2 * nd1
    assert np.max(np.abs(M - K)) < 1e-14 * np.max(np.abs(K))
    assert np.allclose(M, M.T)
    assert np.linalg.eigvalsh(M).min() > 0
    area = (bp1[-1] - bp1[0]) * (bp2[-1] - bp2[0])
    assert abs(M.sum() - area) < 1e-12 * area


def test_partition_of_unity(mesh16):
    om, bp = mesh16
    ones = np.ones(om.n_dofs)
    rng = np.random.default_rng(1)
    for x, y in rng.uniform(-5.99, 5.99, (50, 2)):
        assert abs(om.eval_field(ones, x, y) - 1.0) < 1e-14


def test_projection_reproduces_moments(mesh16):
    """int f_s q = sum_a w_a q(v_a) for q in the spline space (L2 projection)."""
    om, bp = mesh16
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=0)
    f = om.l2_project(v, w)
    xq, wq = np.polynomial.legendre.leggauss(6)
    tot = np.zeros(6)
    for i in range(16):
        for j in range(16):
            a, b, c, d = bp[i], bp[i + 1], bp[j], bp[j + 1]
            for qi in range(6):
                for qj in range(6):
                    x = a + (b - a) * (xq[qi] + 1) / 2
                    y = c + (d - c) * (xq[qj] + 1) / 2
                    ww = wq[qi] * wq[qj] * (b - a) * (d - c) / 4
                    tot += ww * om.eval_field(f, x, y) * np.array([1, x, y, x * x, x * y, y * y])
    ref = np.array([w.sum(), (w * v[:, 0]).sum(), (w * v[:, 1]).sum(), (w * v[:, 0] ** 2).sum(),
                    (w * v[:, 0] * v[:, 1]).sum(), (w * v[:, 1] ** 2).sum()])
    assert np.max(np.abs(tot - ref)) < 1e-13


def test_entropy_chain_rule(mesh16):
    """dS_h/dv_a = -w_a G_a (solver.jl:43-61) by central differences."""
    om, bp = mesh16
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=0)
    f = om.l2_project(v, w)
    G = om.compute_G(v, om.mass_solve(om.compute_r(f)))
    h = 3e-4
    for a in (5, 100, 1000):
        for comp in (0, 1):
            vp = v.copy(order="F")
            vp[a, comp] += h
            vm = v.copy(order="F")
            vm[a, comp] -= h
            fd = (om.entropy(om.l2_project(vp, w)) - om.entropy(om.l2_project(vm, w))) / (2 * h)
            assert abs(fd - (-w[a] * G[a, comp])) < 1e-5 * abs(w[a] * G[a, comp]) + 1e-12


def test_gaussian_entropy_normalisation(oracle_mod):
    """S_h of a resolved Gaussian approaches 1 + log(2 pi s1 s2) (per-element
    weights normalised to the element area)."""
    bp = uniform_bp(-6.0, 6.0, 48)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    v, w = gaussian_markers(200_000, 1.0, 1.0, seed=2)
    S = om.entropy(om.l2_project(v, w))
    assert abs(S - (1 + np.log(2 * np.pi))) < 2e-2


# ---------------------------------------------------- pair sum / solver

def test_pair_sum_conservation(mesh16):
    om, bp = mesh16
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=4)
    f = om.l2_project(v, w)
    G = om.compute_G(v, om.mass_solve(om.compute_r(f)))
    dv = om.collision(v, w, G)
    scale = np.max(np.abs(dv))
    assert abs(np.sum(w * dv[:, 0])) < 1e-12 * scale
    assert abs(np.sum(w * dv[:, 1])) < 1e-12 * scale
    assert abs(np.sum(w * (v * dv).sum(1))) < 1e-12 * scale * np.max(np.abs(v))
    F, A = om.collision_metric(v, w, G)
    assert np.array_equal(F, dv)    # same loop, bit-identical (functions.jl:245-247)
    # vdot = B - A G with B = sum w U(d) G_a (docs: the metric split)
    rows = np.array([0, 17, 1000])
    dvr = om.collision_rows(v, w, G, rows)
    assert np.array_equal(dvr, dv[rows])


def test_gonzalez_identity(mesh16, oracle_mod):
    """G_eff . dv reproduces S(v_in) - S0 exactly (discrete-gradient identity)."""
    om, bp = mesh16
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=6)
    o = oracle_mod.Opts()
    S0 = om.entropy(om.l2_project(v, w))
    v_in = om.predictor(o, v, w, 0.05)
    vm = 0.5 * (v + v_in)
    dv = v_in - v
    G = om.compute_G(vm, om.mass_solve(om.compute_r(om.l2_project(vm, w))))
    dS = -w[:, None] * G
    S1 = om.entropy(om.l2_project(v_in, w))
    lam = (S1 - S0 - np.sum(dv * dS)) / np.sum(dv * dv)
    assert abs(np.sum((dS + lam * dv) * dv) - (S1 - S0)) < 1e-13 * abs(S1 - S0) + 1e-16


@pytest.mark.parametrize("model", ["landau", "lb"])
def test_oracle_step_conserves(oracle_mod, model):
    """Landau with Gonzalez at dt=0.05; LB without Gonzalez at dt=0.01 (LB with
    Gonzalez stagnates on this coarse mesh: lambda is not smooth where entropy
    quadrature points have f_s -> 0+)."""
    bp = uniform_bp(-6.0, 6.0, 16)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    v, w = gaussian_markers(1024, 1.0, 0.5, seed=8)
    gz = model == "landau"
    dt = 0.05 if gz else 0.01
    o = oracle_mod.Opts(model=model, m=5, abs_floor=0.0, damping=0.7, max_iter=400,
                        use_gonzalez=gz)
    S0 = om.entropy(om.l2_project(v, w))
    v1 = om.predictor(o, v, w, dt)
    x, (it, res, nrs, r0) = om.step_anderson(o, v1, v, w, S0, dt)
    assert it < 400 and res < 1e-12 * np.linalg.norm(x)
    assert np.max(np.abs(np.array(oracle_mod.momentum(x, w)) - oracle_mod.momentum(v, w))) < 1e-13
    E0 = oracle_mod.energy(v, w)
    assert abs(oracle_mod.energy(x, w) - E0) < 1e-12 * E0
    # the returned G(v) is a fixed point of the map to the solve tolerance
    Gx = om.picard_map(o, x, v, w, S0, dt)
    assert np.linalg.norm(Gx - x) < 1e-9
    if gz:
        # Gonzalez: entropy is non-decreasing over the step
        assert om.entropy(om.l2_project(x, w)) >= S0 - 1e-14


# ---------------------------------------------------- golden vectors

def test_diagnostics_known_answers(mesh16, oracle_mod):
    """om_diagnostics: momentum and energy are the reference's known answers
    (test/integration/main_helpers.jl:13-19), the entropy equals the projection's
    S, and for markers spread uniformly over a cell-aligned block the histogram
    error is small against the density itself while a concentrated clump shows
    a Gibbs negative lobe."""
    om, bp = mesh16
    v = np.asfortranarray([[1.0, 2.0], [-3.0, 0.5]])
    w = np.array([0.25, 0.75])
    d = om.diagnostics(v, w)
    assert np.isclose(d[2], 0.25 * 1.0 + 0.75 * -3.0) and np.isclose(d[3], 0.25 * 2.0 + 0.75 * 0.5)
    assert np.isclose(d[1], 0.5 * (0.25 * (1.0 + 4.0) + 0.75 * (9.0 + 0.25)))
    rng = np.random.default_rng(8)
    vg, wg = gaussian_markers(4096, 1.0, 0.5, seed=8)
    dg = om.diagnostics(vg, wg)
    assert np.isclose(dg[0], om.entropy(om.l2_project(vg, wg)), rtol=1e-14)
    # uniform markers on [-3,3]^2 (cell-aligned): f_s ~ f_p ~ 1/36 in the block
    vu = np.asfortranarray(rng.uniform(-3.0, 3.0, size=(200000, 2)))
    du = om.diagnostics(vu, np.full(200000, 1 / 200000))
    assert du[4] < 0.2 * np.sqrt(1 / 36.0)
    # a tight clump: the projection rings and has a negative part
    vc = np.asfortranarray(0.01 * rng.standard_normal((2000, 2)))
    dc = om.diagnostics(vc, np.full(2000, 1 / 2000))
    assert dc[5] > 0.0


def test_hessian_matches_gradient_differences(mesh16, oracle_mod):
    """The Hessian gather of the block preconditioner equals central differences
    of the gradient gather compute_G on the same field (away from cell edges)."""
    om, bp = mesh16
    rng = np.random.default_rng(3)
    L = rng.standard_normal(om.n_dofs)
    h = bp[1] - bp[0]
    # markers well inside cells so that +-eps stays in the same cell
    cells = rng.integers(1, len(bp) - 2, size=(64, 2))
    v = np.asfortranarray(bp[cells] + h * rng.uniform(0.2, 0.8, size=(64, 2)))
    H = om.hessian_L(v, L)
    eps = 1e-6
    for k, (c1, c2) in enumerate(((0, 0), (1, 1))):
        e = np.zeros(2)
        e[k] = eps
        dG = (om.compute_G(v + e, L) - om.compute_G(v - e, L)) / (2 * eps)
        np.testing.assert_allclose(H[:, 0 if k == 0 else 2], dG[:, k], rtol=1e-6, atol=1e-6)
        np.testing.assert_allclose(H[:, 1], dG[:, 1 - k], rtol=1e-6, atol=1e-6)


def test_oracle_defect_precond(oracle_mod):
    """step_defect! with the block-Newton inner preconditioner converges to a
    fixed point of the FP64 map that conserves momentum and energy, with no more
    inner maps than the reference's inner iteration."""
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=5)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    dt = 0.02
    o = oracle_mod.Opts(model="landau", m=8, tol=1e-12, abs_floor=0.0, damping=0.7,
                        max_iter=200, stag_rel_tol=0.1)
    S0 = om.entropy(om.l2_project(v, w))
    v1 = om.predictor(o, v, w, dt)
    _x0, info0 = om.step_defect(o, v1, v, w, S0, dt)
    x, info = om.step_defect(o, v1, v, w, S0, dt, outer_m=5, precond=1)
    assert info[1] < 1e-12 * np.linalg.norm(x)
    assert info[2] <= info0[2]
    assert np.linalg.norm(om.picard_map(o, x, v, w, S0, dt) - x) < 1e-10
    assert np.max(np.abs((w[:, None] * (x - v)).sum(0))) < 1e-14
    E0 = 0.5 * np.sum(w * (v ** 2).sum(1))
    assert abs(0.5 * np.sum(w * (x ** 2).sum(1)) - E0) < 1e-13 * E0


def test_oracle_defect_outer_anderson(oracle_mod):
    """step_defect! with Anderson mixing of the outer iterates: fewer outer maps
    than the reference's plain outer iteration on the same step, and the result
    is a fixed point of the FP64 map that conserves momentum and energy."""
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=5)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    dt = 0.02
    o = oracle_mod.Opts(model="landau", m=8, tol=1e-12, abs_floor=0.0, damping=0.7,
                        max_iter=200, stag_rel_tol=0.1)
    S0 = om.entropy(om.l2_project(v, w))
    v1 = om.predictor(o, v, w, dt)
    _x0, info0 = om.step_defect(o, v1, v, w, S0, dt, outer_m=0)
    x, info = om.step_defect(o, v1, v, w, S0, dt, outer_m=5)
    assert info0[1] < 1e-12 * np.linalg.norm(_x0) and info[1] < 1e-12 * np.linalg.norm(x)
    assert info[0] < info0[0]
    assert np.linalg.norm(om.picard_map(o, x, v, w, S0, dt) - x) < 1e-10
    assert np.max(np.abs((w[:, None] * (x - v)).sum(0))) < 1e-14
    E0 = 0.5 * np.sum(w * (v ** 2).sum(1))
    assert abs(0.5 * np.sum(w * (x ** 2).sum(1)) - E0) < 1e-13 * E0


def test_golden_vectors(oracle_mod):
    """The oracle reproduces the committed fixture (tests/golden/make_golden.py)."""
    path = os.path.join(GOLDEN, "c1_small.npz")
    if not os.path.exists(path):
        pytest.skip("golden fixture not generated")
    z = np.load(path)
    bp = z["bp"]
    om = oracle_mod.OracleMesh(bp, bp, 6)
    v, w = np.asfortranarray(z["v"]), z["w"]
    f = om.l2_project(v, w)
    assert np.max(np.abs(f - z["f"])) <= 1e-13 * np.max(np.abs(z["f"]))
    r = om.compute_r(f)
    assert np.max(np.abs(r - z["r"])) <= 1e-13 * np.max(np.abs(z["r"]))
    assert abs(om.entropy(f) - float(z["S"])) <= 1e-13 * abs(float(z["S"]))
    G = om.compute_G(v, om.mass_solve(r))
    assert np.max(np.abs(G - z["G"])) <= 1e-12 * np.max(np.abs(z["G"]))
    dv = om.collision(v, w, G)
    assert np.max(np.abs(dv - z["dotv"])) <= 1e-12 * np.max(np.abs(z["dotv"]))
    for k in ("mom_v", "mom_w", "mom_out"):
        assert k in z.files
    n, U1, U2, Q = oracle_mod.moments(z["mom_v"], z["mom_w"])
    assert np.allclose([n, U1, U2, Q], z["mom_out"], rtol=1e-15, atol=1e-15)


@pytest.mark.parametrize("case", ["c1", "c2"])
def test_two_mass_solves_spread(oracle_mod, case):
    """Two correct FP64 mass solves -- the 2D banded Cholesky of the assembled
    matrix and the tensor-product solve with 1D Cholesky factors -- give
    coefficients within a few ulps of max|f| and Picard maps within the per-RHS
    bar: the LB map's 1/f_s amplification of solve round-off stays far below
    1e-12 relative at C1 and C2 (measured 8e-14 and 4e-15), which is what lets
    the GPU LB map be held to 1e-12 against the oracle."""
    lo, n, N, sx, sy, peak = {"c1": (6.0, 16, 2048, 1.0, 0.5, 0.0),
                              "c2": (8.0, 32, 16384, np.sqrt(0.5), np.sqrt(0.5), 2.0)}[case]
    bp = uniform_bp(-lo, lo, n)
    v, w = gaussian_markers(N, sx, sy, seed=11, peak=peak)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    b = om.l2_rhs(v, w)
    f0 = om.mass_solve(b)
    om.set_mass_solver(1)
    f1 = om.mass_solve(b)
    om.set_mass_solver(0)
    assert np.max(np.abs(f0 - f1)) < 1e-14 * np.max(np.abs(f0))
    S0 = om.entropy(om.l2_project(v, w))
    for model in ("lb", "landau"):
        o = oracle_mod.Opts(model=model)
        vin = om.predictor(o, v, w, 0.05)
        r0 = om.picard_map(o, vin, v, w, S0, 0.05)
        om.set_mass_solver(1)
        r1 = om.picard_map(o, vin, v, w, S0, 0.05)
        om.set_mass_solver(0)
        assert np.max(np.abs(r0 - r1)) < 2e-13 * np.max(np.abs(r0)), model
