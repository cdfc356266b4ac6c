"""Train the learned warm start on solver-generated pairs.

Pairs (features at a step start, delta = (v_converged - v_Euler)/dt^2 of the
converged step; steps whose solve did not converge are advanced but not kept)
come from the solver itself, with use_logsq = true as in the benchmark, on
  - the N = 131,072 Landau workload (anisotropic Gaussian sigma = (1, 0.5),
    64x64 mesh on [-6,6]^2, dt = 0.02), 20 consecutive steps;
  - Landau instances of the batched workload family (N log-uniform in
    [4096, 65536], meshes 24..48 cells on [-6,6]^2, anisotropic Gaussians with
    T_x, T_y uniform in [0.2, 1.5]), a few steps each;
until at least `--pairs` pairs are collected. The network is trained on the
GPU by the library's own kernels (co_mlp_train_step) and saved with its
normalisation to `--out`.

Usage: python -m collops.train_warmstart --out <file.npz> [--pairs 1000000]
(run from the collisionoperators.jl_gb300 directory or with it on sys.path).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np


def _markers(N, sx, sy, seed, peak=0.0):
    rng = np.random.default_rng(seed)
    v = np.zeros((N, 2), order="F")
    if peak:
        half = N // 2
        v[:, 0] = np.concatenate([np.full(half, -peak), np.full(N - half, peak)]) + \
            sx * rng.standard_normal(N)
    else:
        v[:, 0] = sx * rng.standard_normal(N)
    v[:, 1] = sy * rng.standard_normal(N)
    return v, np.full(N, 1.0 / N)


def collect(pairs: int, seed: int = 0, precision: str = "mixed_ds", log=print):
    import torch

    import collops as co
    from collops import learned

    Xs, Ts = [], []
    total = 0
    rng = np.random.default_rng(seed)
    jobs = [dict(N=131072, n=64, sx=1.0, sy=0.5, dt=0.02, steps=20, seed=1000)]
    for k in range(64):
        N = int(np.exp(rng.uniform(np.log(4096), np.log(65536))))
        jobs.append(dict(N=N, n=int(rng.integers(24, 49)), sx=float(np.sqrt(rng.uniform(0.2, 1.5))),
                         sy=float(np.sqrt(rng.uniform(0.2, 1.5))), dt=0.02, steps=3,
                         seed=2000 + k))
    for job in jobs:
        if total >= pairs:
            break
        bp = np.linspace(-6.0, 6.0, job["n"] + 1)
        p = co.SimParameters(bp1=bp, bp2=bp, m_anderson=8, damping=0.7, tol=1e-12,
                             abs_floor=1e-10, max_iter=2000, precision=precision,
                             use_logsq=True)
        ws = co.build_workspace(p)
        o = p.opts()
        v, w = _markers(job["N"], job["sx"], job["sy"], job["seed"])
        vd = torch.from_numpy(np.ascontiguousarray(v.T)).cuda()
        wd = torch.from_numpy(w).cuda()
        d = co.CoDefectOpts(0.02, 100, 5, 0.9, 0, 5, 0, 1e-3, 0)
        N, dt = job["N"], job["dt"]

        def solve(v1, x, S0):
            oo = p.opts()
            oo.stag_rel_tol = 0.1
            it, inner = C.c_int(), C.c_int()
            res, r0 = C.c_double(), C.c_double()
            co._check(ws.lib.co_step_defect_dev(ws.h, C.byref(oo), C.byref(d), v1.data_ptr(),
                                                x.data_ptr(), wd.data_ptr(), N, S0, dt,
                                                C.byref(it), C.byref(res), C.byref(inner),
                                                C.byref(r0)), "co_step_defect_dev")
            return res.value < max(1e-12 * float(torch.linalg.vector_norm(v1)), 1e-10)
        t0 = time.time()
        X, T, _ = learned.generate_pairs(ws, o, vd, wd, dt, job["steps"], solve)
        ws.close()
        Xs.append(X)
        Ts.append(T)
        total += X.shape[0]
        log(f"  N={N} mesh={job['n']} steps={job['steps']}: {X.shape[0]} pairs "
            f"({time.time() - t0:.1f} s), total {total}")
    return np.concatenate(Xs), np.concatenate(Ts)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--pairs", type=int, default=1_000_000)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=2e-3)
    a = ap.parse_args(argv)
    from collops import learned
    t0 = time.time()
    X, T = collect(a.pairs)
    t1 = time.time()
    # hold out every 20th pair for a validation loss
    rng = np.random.default_rng(5)
    held = rng.random(X.shape[0]) < 0.05
    ws = learned.WarmStart()
    hist = ws.fit(X[~held], T[~held], epochs=a.epochs, batch=a.batch, lr=a.lr)
    val = ws.validation_loss(X[held], T[held])
    t2 = time.time()
    ws.save(a.out)
    print(json.dumps({"pairs": int(X.shape[0]), "held_out": int(held.sum()),
                      "collect_s": round(t1 - t0, 1), "train_s": round(t2 - t1, 1),
                      "loss_first": hist[0], "loss_last": hist[-1], "val_loss": val,
                      "epochs": a.epochs}))


if __name__ == "__main__":
    main()
