"""Parity over consecutive time steps at the stated configurations.

Every step is started from the ORACLE's state of that step (its markers and the
entropy S0 of their projection), so a difference in one step cannot carry into
the next; the GPU runs the predictor and the implicit solve through the C ABI
and is compared with the oracle's same step:

- the Picard map at the oracle's predictor point, per step: 1e-12 relative on
  v_out (the per-RHS bar of the FP64 form), both Landau and LB;
- the exit of step_anderson! (converged, or the stagnation exit of
  solver.jl:357-367 with its best iterate) and the returned state. When both
  converge, the iteration counts agree within 10 % and the fixed points to
  1e-10. When both stagnate, both leave on a window boundary with best
  residuals within 5x (the iteration does not contract there, so round-off
  differences grow and the best iterates differ at the scale of that
  residual). A step where one side converges and the other stagnates is that
  same amplification deciding the exit (both started within 1e-15); it passes
  only if the converged result, run through the OTHER side's map, has a
  residual below the other side's best -- i.e. it is the better answer by the
  other implementation's own measure.

Configurations (uniform meshes, uniform weights 1/N, Gonzalez on, tol 1e-12,
abs_floor 0 so that tol*||v|| binds):
  C1: 16x16 on [-6,6]^2, N = 2048 anisotropic Gaussian (T_x 1, T_y 0.25),
      dt 0.05, Anderson depth 5, 10 steps (Landau);
  C2: 32x32 on [-8,8]^2, N = 16384 bimodal at (+-2, 0), T = 0.5, dt 0.05,
      depth 8, 5 steps, Landau and LB (nu = 1).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import gaussian_markers, uniform_bp

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _run(oracle_mod, collops_mod, *, lo, n, N, sx, sy, peak, model, dt, m, steps, seed=5):
    bp = uniform_bp(-lo, lo, n)
    v, w = gaussian_markers(N, sx, sy, seed=seed, peak=peak)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    kw = dict(m=m, tol=1e-12, abs_floor=0.0, damping=0.7, max_iter=400, stag_window=50,
              stag_rel_tol=0.01)
    o = oracle_mod.Opts(model=model, **kw)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp,
                                                               collision_model=model))
    rows = []
    x = v
    for k in range(steps):
        S0 = om.entropy(om.l2_project(x, w))
        v1 = om.predictor(o, x, w, dt)
        # one Picard map at the oracle's predictor point
        ref_map = om.picard_map(o, v1, x, w, S0, dt)
        out = np.zeros_like(x, order="F")
        collops_mod.picard_map(ws, out, v1, x, w, S0, dt)
        map_err = _rel(out, ref_map)
        # the whole step: the GPU's predictor and solve from the oracle's state
        ref, info_ref = om.step_anderson(o, v1, x, w, S0, dt)
        y = np.zeros_like(x, order="F")
        collops_mod.predictor(ws, y, x, w, dt)
        info = collops_mod.step_anderson(ws, y, x, w, S0, dt, **kw)
        conv = info[1] < 1e-12 * np.linalg.norm(y)
        conv_ref = info_ref[1] < 1e-12 * np.linalg.norm(ref)
        cross = None
        if conv and not conv_ref:        # the GPU result through the oracle's map
            cross = np.linalg.norm(om.picard_map(o, y, x, w, S0, dt) - y)
        elif conv_ref and not conv:      # the oracle result through the GPU's map
            g = np.zeros_like(x, order="F")
            collops_mod.picard_map(ws, g, ref, x, w, S0, dt)
            cross = np.linalg.norm(g - ref)
        rows.append(dict(k=k, map_err=map_err, it=info[0], it_ref=info_ref[0], res=info[1],
                         res_ref=info_ref[1], conv=conv, conv_ref=conv_ref, cross=cross,
                         diff=_rel(y, ref), x=x, y=y))
        x = ref
    ws.close()
    return rows, w


def _check(rows, w):
    report = "\n".join(f"step {r['k']}: map {r['map_err']:.2e} it {r['it']}/{r['it_ref']} "
                       f"res {r['res']:.2e}/{r['res_ref']:.2e} conv {r['conv']}/{r['conv_ref']} "
                       f"diff {r['diff']:.2e}" +
                       (f" cross-residual {r['cross']:.2e}" if r["cross"] is not None else "")
                       for r in rows)
    flips = 0
    for r in rows:
        assert r["map_err"] < TOL64, report
        if r["conv"] and r["conv_ref"]:
            assert abs(r["it"] - r["it_ref"]) <= max(3, r["it_ref"] // 10), report
            assert r["diff"] < 1e-10, report
        elif not r["conv"] and not r["conv_ref"]:
            # stagnation exits leave on a window boundary (solver.jl:357-367)
            assert r["it"] % 50 == 0 and r["it_ref"] % 50 == 0, report
            assert 0.2 < r["res"] / r["res_ref"] < 5.0, report
        else:
            flips += 1
            other_best = r["res_ref"] if r["conv"] else r["res"]
            assert r["cross"] < other_best, report
        # the returned state is a Picard update: momentum is conserved
        dp = np.abs((w[:, None] * (r["y"] - r["x"])).sum(0)).max()
        assert dp < 1e-12, report
    assert flips <= max(1, len(rows) // 4), report
    return report


def test_c1_ten_steps_landau(built_lib, oracle_mod, collops_mod):
    rows, w = _run(oracle_mod, collops_mod, lo=6.0, n=16, N=2048, sx=1.0, sy=0.5, peak=0.0,
                   model="landau", dt=0.05, m=5, steps=10)
    print(_check(rows, w))
    assert any(r["conv_ref"] for r in rows)


@pytest.mark.parametrize("model", ["landau", "lb"])
def test_c2_five_steps(built_lib, oracle_mod, collops_mod, model):
    rows, w = _run(oracle_mod, collops_mod, lo=8.0, n=32, N=16384, sx=np.sqrt(0.5),
                   sy=np.sqrt(0.5), peak=2.0, model=model, dt=0.05, m=8, steps=5)
    print(_check(rows, w))


@pytest.mark.parametrize("logsq", [True, False])
def test_c3_picard_maps_full_size(built_lib, oracle_mod, collops_mod, logsq):
    """C3 at full size (N = 131,072, 64x64 on [-6,6]^2, dt 0.02): one FP64 and one
    double-single Picard map at the oracle's predictor point against the
    oracle's full FP64 map (every pair evaluated). FP64 holds the per-RHS bar of
    1e-12; the double-single map (the FP64-accurate stage of the mixed form)
    holds 1e-11."""
    bp = uniform_bp(-6.0, 6.0, 64)
    rng = np.random.default_rng(42)
    N = 131072
    v = np.zeros((N, 2), order="F")
    v[:, 0] = rng.standard_normal(N)
    v[:, 1] = 0.5 * rng.standard_normal(N)
    w = np.full(N, 1.0 / N)
    dt = 0.02
    om = oracle_mod.OracleMesh(bp, bp, 6, use_logsq=logsq)
    o = oracle_mod.Opts(model="landau")
    S0 = om.entropy(om.l2_project(v, w))
    v1 = om.predictor(o, v, w, dt)
    ref = om.picard_map(o, v1, v, w, S0, dt)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp, use_logsq=logsq))
    errs = {}
    for prec in ("fp64", "mixed_ds"):
        out = np.zeros_like(v, order="F")
        collops_mod.picard_map(ws, out, v1, v, w, S0, dt, precision=prec)
        errs[prec] = _rel(out, ref)
    ws.close()
    print(f"C3 map errors (logsq={logsq}): {errs}")
    assert errs["fp64"] < TOL64, errs
    assert errs["mixed_ds"] < 1e-11, errs
