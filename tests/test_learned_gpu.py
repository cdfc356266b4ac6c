"""GPU: the warm-start MLP kernels (BF16 weights, FP32 accumulation) against the
FP64 NumPy oracle, training, and the learned warm start on a small workload.

Tolerances: forward outputs 1e-4 relative (FP32 accumulation of 64-term sums),
gradients 2e-3 relative in the 2-norm (FP32 per-sample backward and FP32
minibatch reduction against FP64)."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import PKG, gaussian_markers, uniform_bp

pytestmark = pytest.mark.gpu


def test_mlp_forward_and_gradients_match_oracle(built_lib, collops_mod):
    import torch
    from collops import learned
    from oracle import mlp as om
    net = learned.MLP(seed=3, n_in=9)
    p = net.get_params()
    rng = np.random.default_rng(1)
    X = rng.standard_normal((1000, 9)).astype(np.float32)
    T = rng.standard_normal((1000, 2)).astype(np.float32)
    Xd, Td = torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda()
    Y = torch.empty((1000, 2), dtype=torch.float32, device="cuda")
    net.forward(Xd, Y)
    y_ref, _ = om.forward(p, X.astype(np.float64))
    assert np.max(np.abs(Y.cpu().numpy() - y_ref)) <= 1e-4 * max(1.0, np.max(np.abs(y_ref)))
    g, loss = net.gradients(Xd, Td)
    loss_ref, g_ref = om.loss_and_grad(p, X, T)
    assert abs(loss - loss_ref) <= 1e-5 * loss_ref
    assert np.linalg.norm(g - g_ref) <= 2e-3 * np.linalg.norm(g_ref)
    net.close()


def test_mlp_training_reduces_loss(built_lib, collops_mod):
    import torch
    from collops import learned
    rng = np.random.default_rng(2)
    X = rng.standard_normal((16384, 9)).astype(np.float32)
    W = rng.standard_normal((9, 2)).astype(np.float32)
    T = np.tanh(X @ W).astype(np.float32)
    ws = learned.WarmStart(mlp=learned.MLP(n_in=9))
    hist = ws.fit(X, T, epochs=12, batch=2048, lr=3e-3)
    ws.mlp.close()
    assert hist[-1] < 0.2 * hist[0]


def test_learned_warm_start_small(built_lib, collops_mod, tmp_path):
    """Generate solver pairs on a small Landau workload, train, and compare the
    first residual and the iteration count of the next step with and without
    the learned proposal. The proposal is used only when its first residual is
    smaller (the fallback rule), so the chosen start is never worse; the gain
    itself is recorded, not required (the reference measured none)."""
    import torch
    from collops import learned
    bp = uniform_bp(-6.0, 6.0, 16)
    v, w = gaussian_markers(2048, 1.0, 0.5, seed=9)
    p = collops_mod.SimParameters(bp1=bp, bp2=bp, m_anderson=5, damping=0.7, tol=1e-12,
                                  abs_floor=0.0, max_iter=400)
    ws = collops_mod.build_workspace(p)
    o = p.opts()
    dt = 0.02
    vd = torch.from_numpy(np.ascontiguousarray(v.T)).cuda()
    wd = torch.from_numpy(w).cuda()
    lib = ws.lib
    import ctypes as C

    def solve(v1, x, S0):
        it, nrs = C.c_int(), C.c_int()
        res, r0 = C.c_double(), C.c_double()
        collops_mod._check(lib.co_step_anderson_dev(ws.h, C.byref(o), v1.data_ptr(), x.data_ptr(),
                                                    wd.data_ptr(), 2048, S0, dt, C.byref(it),
                                                    C.byref(res), C.byref(nrs), C.byref(r0)),
                           "step")
        return it.value
    X, T, x = learned.generate_pairs(ws, o, vd, wd, dt, 6, solve)
    assert X.shape == (6 * 2048, learned.N_IN) and np.all(np.isfinite(X)) and np.all(np.isfinite(T))
    wsn = learned.WarmStart()
    hist = wsn.fit(X, T, epochs=30, batch=1024, lr=2e-3)
    assert hist[-1] < hist[0]
    path = tmp_path / "ws.npz"
    wsn.save(str(path))
    wsn2 = learned.WarmStart.load(str(path))
    S0 = learned.entropy_of(ws, x, wd)
    v1 = torch.empty_like(x)
    used, rl, rp = wsn2.propose(ws, o, x, wd, S0, dt, v1)
    assert np.isfinite(rl) and np.isfinite(rp)
    it_learned = solve(v1.clone(), x, S0)
    Xf, vp, _rp = learned.features(ws, o, x, wd, S0, dt)
    it_plain = solve(vp.clone(), x, S0)
    print(f"learned warm start: used={used} r_learned={rl:.3e} r_predictor={rp:.3e} "
          f"iterations learned-start={it_learned} predictor-start={it_plain}")
    assert min(rl, rp) <= rp
    wsn.mlp.close()
    wsn2.mlp.close()
    ws.close()


def test_trained_warm_start_gain(built_lib, collops_mod):
    """The committed network (trained by collops.train_warmstart on >= 1M pairs
    from converged steps of the N = 131,072 workload and the batched family,
    use_logsq = true) on held-out Landau instances of that family: its proposal's
    first residual is well below both fallbacks -- the explicit predictor and the
    plain previous-step guess -- so the step starts from it, and the step
    converges (a solve from the learned start that stagnates on the stiff map is
    retried once from the next start). The first residuals come from one
    co_step_learned call (r_start: predictor, learned, previous state)."""
    import torch
    from collops import learned
    path = os.path.join(PKG, "collops", "warmstart_c3.npz")
    warm = learned.WarmStart.load(path)
    gains = []
    for N, n, sx, sy, seed in ((16384, 32, 0.9, 0.6, 501), (32768, 40, 1.1, 0.7, 502)):
        bp = uniform_bp(-6.0, 6.0, n)
        v, w = gaussian_markers(N, sx, sy, seed=seed)
        p = collops_mod.SimParameters(bp1=bp, bp2=bp, m_anderson=8, damping=0.7, tol=1e-12,
                                      abs_floor=1e-10, max_iter=400, precision="mixed_ds",
                                      use_logsq=True)
        ws = collops_mod.build_workspace(p)
        o = p.opts()
        dt = 0.02
        x = torch.from_numpy(np.ascontiguousarray(v.T)).cuda()
        wd = torch.from_numpy(w).cuda()
        S0 = learned.entropy_of(ws, x, wd)
        v1 = torch.empty_like(x)
        d = collops_mod.CoDefectOpts(0.02, 100, 5, 0.9, 0, 5, 0, 1e-3, 0)
        rec = warm.step(ws, o, d, x, wd, S0, dt, v1)
        ws.close()
        r_pred, r_learn, r_prev = rec["r_start"]
        print(f"N={N}: first residual learned {r_learn:.3e} predictor {r_pred:.3e} "
              f"previous {r_prev:.3e}; start {rec['start']}, outer {rec['outer']}, "
              f"inner {rec['inner']}, converged {rec['converged']}")
        assert r_learn < min(r_pred, r_prev) and rec["converged"]
        # the first attempt starts from the learned proposal; a different final
        # start means that attempt stagnated and the retry converged
        assert rec["start"] == "learned" or rec["attempts"] == 2
        gains.append(min(r_pred, r_prev) / r_learn)
    warm.mlp.close()
    assert min(gains) > 1.25


def test_step_defect_warm(built_lib, collops_mod):
    """The learned-start step helper: proposal, defect-correction solve (retry from
    the other start only on stagnation), result a converged step that conserves
    momentum and energy."""
    import torch
    from collops import learned
    warm = learned.WarmStart.load(os.path.join(PKG, "collops", "warmstart_c3.npz"))
    N, n = 16384, 32
    bp = uniform_bp(-6.0, 6.0, n)
    v, w = gaussian_markers(N, 0.9, 0.6, seed=503)
    p = collops_mod.SimParameters(bp1=bp, bp2=bp, m_anderson=8, damping=0.7, tol=1e-12,
                                  abs_floor=0.0, max_iter=400, precision="mixed_ds")
    ws = collops_mod.build_workspace(p)
    o = p.opts()
    o.stag_rel_tol = 0.1
    x = torch.from_numpy(np.ascontiguousarray(v.T)).cuda()
    wd = torch.from_numpy(w).cuda()
    S0 = learned.entropy_of(ws, x, wd)
    v1 = torch.empty_like(x)
    d = collops_mod.CoDefectOpts(0.05, 60, 5, 0.5, 0, 0, 0, 1e-2)
    info, rec = learned.step_defect_warm(ws, warm, o, d, x, wd, S0, 0.02, v1)
    ws.close()
    warm.mlp.close()
    x1 = v1.cpu().numpy().T
    assert rec["attempts"] in (1, 2) and info[1] < 1e-12 * np.linalg.norm(x1)
    assert np.max(np.abs((w[:, None] * (x1 - v)).sum(0))) < 1e-12
    E0 = 0.5 * np.sum(w * (v ** 2).sum(1))
    assert abs(0.5 * np.sum(w * (x1 ** 2).sum(1)) - E0) < 1e-12 * E0
