"""step_newton! on the device (co_step_newton: JFNK with matrix-free GMRES,
newton_krylov.jl:74-303, solver.jl:460-486) against the oracle's restatement of
the same algorithm, on C1's mesh and markers (16x16 on [-6,6]^2, N = 2048) in
two settings where the reference's Newton converges.

GMRES's dot products are summed in a different order on the two sides, and the
forward-difference products (fd_h 1e-6) amplify that round-off by ~1e6, so the
Newton directions differ at ~1e-10; the counts of map evaluations may differ by
a few and the fixed points agree to 1e-10 (the tolerance of the other step
tests). A double-single solve must land on a fixed point of the oracle's FP64
map."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import gaussian_markers, uniform_bp

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("logsq,dt", [(True, 0.02), (False, 0.005)])
def test_step_newton_matches_oracle(built_lib, oracle_mod, collops_mod, logsq, dt):
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=5)
    om = oracle_mod.OracleMesh(bp, bp, 6, use_logsq=logsq)
    S0 = om.entropy(om.l2_project(v, w))
    o = oracle_mod.Opts(model="landau", m=5, tol=1e-12, abs_floor=0.0, damping=0.7,
                        max_iter=400)
    v1 = om.predictor(o, v, w, dt)
    ref, info_ref = om.step_newton(o, v1, v, w, S0, dt)
    assert info_ref[4] == 0                       # the oracle converges here
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp, use_logsq=logsq))
    x = np.array(v1, order="F", copy=True)
    info = collops_mod.step_newton(ws, x, v, w, S0, dt, max_iter=400, tol=1e-12, abs_floor=0.0)
    xd = np.array(v1, order="F", copy=True)
    info_ds = collops_mod.step_newton(ws, xd, v, w, S0, dt, max_iter=400, tol=1e-12,
                                      abs_floor=0.0, precision="mixed_ds")
    ws.close()
    print(f"newton logsq={logsq} dt={dt}: gpu {info} oracle {info_ref} ds {info_ds}")
    assert info[4] == 0 and info[1] < 1e-12 * np.linalg.norm(v1)
    assert abs(info[0] - info_ref[0]) <= max(4, info_ref[0] // 5)
    assert np.max(np.abs(x - ref)) / np.max(np.abs(ref)) < 1e-10
    # the exit Picard update conserves momentum and energy (exit_picard_step)
    E0 = 0.5 * np.sum(w * (v ** 2).sum(1))
    for xx in (x, xd):
        assert np.max(np.abs((w[:, None] * (xx - v)).sum(0))) < 1e-12
        assert abs(0.5 * np.sum(w * (xx ** 2).sum(1)) - E0) < 1e-12 * E0
    assert info_ds[4] == 0
    assert np.linalg.norm(om.picard_map(o, xd, v, w, S0, dt) - xd) < 1e-9


def test_step_newton_rejects_bad_options(built_lib, collops_mod):
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(256, 1.0, 0.5, seed=1)
    ws = collops_mod.build_workspace(collops_mod.SimParameters(bp1=bp, bp2=bp))
    x = np.array(v, order="F", copy=True)
    with pytest.raises(collops_mod.CollopsError) as ei:
        collops_mod.step_newton(ws, x, v, w, 1.0, 0.01, krylov_max=0)
    assert ei.value.status == 1
    ws.close()
