"""Failure paths of the device solver, made without a GPU fault.

- The LB drift kernel's grid barrier is a bounded wait: a barrier that cannot
  complete (one phantom arrival) with a short poll limit must end the kernel and
  return CO_ERR_TIMEOUT, and the context must stay usable afterwards.
- The step's exits other than convergence follow step_anderson!
  (solver.jl:357-367 stagnation, :419-422 max_iter): both return the best
  iterate's Picard update, which is compared with the oracle's same exit on the
  same inputs.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import gaussian_markers, uniform_bp

pytestmark = pytest.mark.gpu

CO_ERR_TIMEOUT = 5


def _c1(oracle_mod, dt=0.05):
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=5)
    om = oracle_mod.OracleMesh(bp, bp, 6)
    S0 = om.entropy(om.l2_project(v, w))
    return bp, v, w, om, S0


def test_lb_barrier_timeout_returns_status(built_lib, oracle_mod, collops_mod):
    bp, v, w, om, S0 = _c1(oracle_mod)
    dt = 0.05
    o = oracle_mod.Opts(model="lb")
    v_in = om.predictor(o, v, w, dt)
    ref = om.picard_map(o, v_in, v, w, S0, dt)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp,
                                                               collision_model="lb"))
    out = np.zeros_like(v, order="F")
    ws.set_wait_limit(spins=1000, phantom_blocks=1)
    with pytest.raises(collops_mod.CollopsError) as ei:
        collops_mod.picard_map(ws, out, v_in, v, w, S0, dt)
    assert ei.value.status == CO_ERR_TIMEOUT
    # the kernel ended and the context still works with the default limits
    ws.set_wait_limit(0, 0)
    collops_mod.picard_map(ws, out, v_in, v, w, S0, dt)
    ws.close()
    assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) < 1e-11


def _exit_case(oracle_mod, collops_mod, **kw):
    bp, v, w, om, S0 = _c1(oracle_mod)
    dt = 0.05
    o = oracle_mod.Opts(model="landau", m=5, tol=1e-12, abs_floor=0.0, damping=0.7, **kw)
    v1 = om.predictor(o, v, w, dt)
    ref, info_ref = om.step_anderson(o, v1, v, w, S0, dt)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp))
    x = np.array(v1, order="F", copy=True)
    info = collops_mod.step_anderson(ws, x, v, w, S0, dt, m=5, tol=1e-12, abs_floor=0.0,
                                     damping=0.7, **kw)
    ws.close()
    return x, info, ref, info_ref, v, w


def test_max_iter_exit_returns_best_iterate(built_lib, oracle_mod, collops_mod):
    """max_iter = 3: not converged, the best of the three iterates' Picard
    updates comes back (solver.jl:419-422), as in the oracle."""
    x, info, ref, info_ref, v, w = _exit_case(oracle_mod, collops_mod, max_iter=3)
    assert info[0] == info_ref[0] == 3
    assert info[1] > 1e-12 * np.linalg.norm(x)          # a non-converged exit
    assert abs(info[1] - info_ref[1]) <= 1e-9 * info_ref[1]
    # a few Anderson iterations of the same algorithm: the per-map 1e-12 bar
    # with room for the window's amplification of round-off
    assert np.max(np.abs(x - ref)) / np.max(np.abs(ref)) < 1e-11
    # the returned state is a Picard update: momentum conserved
    assert np.max(np.abs((w[:, None] * (x - v)).sum(0))) < 1e-12


def test_stagnation_exit_returns_best_iterate(built_lib, oracle_mod, collops_mod):
    """stag_window = 2 with stag_rel_tol = 0.99: the window test at k = 6 finds
    less than a 99 % drop of the best residual and exits with the best iterate
    (solver.jl:357-367), as the oracle does."""
    x, info, ref, info_ref, v, w = _exit_case(oracle_mod, collops_mod, max_iter=200,
                                              stag_window=2, stag_rel_tol=0.99)
    assert info_ref[0] == info[0]
    assert info[0] < 200 and info[0] % 2 == 0
    assert info[1] > 1e-12 * np.linalg.norm(x)
    assert abs(info[1] - info_ref[1]) <= 1e-9 * info_ref[1]
    assert np.max(np.abs(x - ref)) / np.max(np.abs(ref)) < 1e-11
    assert np.max(np.abs((w[:, None] * (x - v)).sum(0))) < 1e-12


def test_cap_abort_leaves_early_with_best_iterate(built_lib, collops_mod):
    """cap_abort (the library's extension of step_defect!): with max_inner = 1 and
    an inner tolerance no single inner map can meet, every inner solve hits the
    cap, so once two FP64-stage outer maps in a row bring no new best outer
    residual the step leaves through the stagnation exit, far below max_iter,
    with a state that conserves momentum (the best iterate's Picard update).
    Without cap_abort the same step runs until the stagnation window exits or it
    converges, and never with fewer outer maps. A negative cap_abort is refused."""
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=5)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp))
    f = np.zeros(ws.n_dofs)
    collops_mod.l2_project_gpu(ws, f, v, w)
    S0 = collops_mod.compute_entropy_gpu(ws, f)
    dt = 0.05
    v1 = np.zeros((2048, 2), order="F")
    collops_mod.predictor(ws, v1, v, w, dt)
    kw = dict(m=8, tol=1e-12, abs_floor=0.0, damping=0.7, max_iter=200, eta=1e-6, max_inner=1,
              stag_window=10, stag_rel_tol=1e-3, metric64=True)
    x_on = np.array(v1, order="F", copy=True)
    info_on = collops_mod.step_defect(ws, x_on, v, w, S0, dt, cap_abort=2, **kw)
    x_off = np.array(v1, order="F", copy=True)
    info_off = collops_mod.step_defect(ws, x_off, v, w, S0, dt, cap_abort=0, **kw)
    with pytest.raises(collops_mod.CollopsError) as ei:
        collops_mod.step_defect(ws, np.array(v1, order="F", copy=True), v, w, S0, dt,
                                cap_abort=-1, **kw)
    ws.close()
    print(f"cap_abort=2: {info_on}  cap_abort=0: {info_off}")
    assert ei.value.status == 1
    assert info_on[0] < 200 and info_on[0] <= info_off[0]
    for x in (x_on, x_off):
        assert np.all(np.isfinite(x))
        assert np.max(np.abs((w[:, None] * (x - v)).sum(0))) < 1e-12
