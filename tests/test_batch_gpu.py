"""The batched form: independent ensembles (Landau and LB, different N and
meshes) advanced by one engine -- one batched pair-sum launch per Picard
iteration for all Landau instances, the iteration captured as a CUDA graph.
Each instance must reach the same fixed point as the single-ensemble solver
(step_anderson! through a context) and conserve momentum and energy."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import gaussian_markers, uniform_bp

pytestmark = pytest.mark.gpu

INSTANCES = [
    dict(n=16, N=2048, model="landau", sx=1.0, sy=0.5, seed=1),
    dict(n=20, N=3000, model="lb", nu=1.0, sx=0.8, sy=0.9, seed=2),
    dict(n=24, N=4096, model="landau", sx=0.7, sy=1.1, seed=3),
    dict(n=16, N=1500, model="lb", nu=0.7, sx=1.0, sy=0.6, seed=4),
]


def _setup():
    import torch
    vs, ws, descs = [], [], []
    for d in INSTANCES:
        bp = uniform_bp(-6.0, 6.0, d["n"])
        v, w = gaussian_markers(d["N"], d["sx"], d["sy"], seed=d["seed"])
        vs.append(v)
        ws.append(w)
        descs.append(dict(bp1=bp, bp2=bp, model=d["model"], nu=d.get("nu", 1.0), N=d["N"]))
    vcat = torch.cat([torch.from_numpy(np.ascontiguousarray(v.T)).reshape(-1) for v in vs]).cuda()
    wcat = torch.cat([torch.from_numpy(w) for w in ws]).cuda()
    return vs, ws, descs, vcat, wcat


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_matches_single(built_lib, collops_mod, use_graph):
    import torch
    vs, ws, descs, vcat, wcat = _setup()
    batch = collops_mod.Batch(descs)
    dt = 0.005   # every instance converges here in the oracle (no stagnation exits)
    p = collops_mod.SimParameters(m_anderson=5, damping=0.7, tol=1e-12, abs_floor=0.0,
                                  max_iter=400, use_gonzalez=False)
    o = p.opts()
    S0 = batch.entropy(vcat, wcat)
    v1 = torch.empty_like(vcat)
    batch.predictor(o, v1, vcat, wcat, dt)
    iters, res = batch.step(o, v1, vcat, wcat, S0, dt, use_graph=use_graph)
    out = v1.cpu().numpy()
    batch.close()
    off = 0
    for k, d in enumerate(descs):
        N = d["N"]
        x = out[2 * off: 2 * off + 2 * N].reshape(2, N).T
        off += N
        ps = collops_mod.SimParameters(bp1=d["bp1"], bp2=d["bp2"], collision_model=d["model"],
                                       nu=d["nu"], use_gonzalez=False)
        ws_ = collops_mod.build_workspace(ps)
        f = np.zeros(ws_.n_dofs)
        collops_mod.l2_project_gpu(ws_, f, vs[k], ws[k])
        S0k = collops_mod.compute_entropy_gpu(ws_, f)
        assert abs(S0k - S0[k]) < 1e-13 * abs(S0k)
        y = np.zeros((N, 2), order="F")
        collops_mod.predictor(ws_, y, vs[k], ws[k], dt)
        info = collops_mod.step_anderson(ws_, y, vs[k], ws[k], S0k, dt, m=5, tol=1e-12,
                                         abs_floor=0.0, damping=0.7, max_iter=400,
                                         use_gonzalez=False)
        ws_.close()
        assert iters[k] < 400 and info[0] < 400
        assert res[k] < 1e-12 * np.linalg.norm(x)
        assert np.max(np.abs(x - y)) / np.max(np.abs(y)) < 1e-10
        w = ws[k]
        v = vs[k]
        assert np.max(np.abs((w[:, None] * (x - v)).sum(0))) < 1e-12
        E0 = 0.5 * np.sum(w * (v ** 2).sum(1))
        assert abs(0.5 * np.sum(w * (x ** 2).sum(1)) - E0) < 1e-12 * E0


def test_batch_tuner_choices(built_lib, collops_mod):
    _, _, descs, vcat, wcat = _setup()
    batch = collops_mod.Batch(descs)
    t = batch.tune()
    batch.close()
    assert t["warps"] in (4, 8) and t["chunk"] in (4, 16) and t["pair_ms"] > 0
