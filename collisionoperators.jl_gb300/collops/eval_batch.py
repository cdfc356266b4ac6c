"""Evaluate the batched engine on the many-ensemble workload.

Workload: 64 independent instances with seeded parameters -- N log-uniform in
[4096, 65536], uniform meshes of 24..48 cells per dimension on [-6,6]^2,
alternately Landau and LB (nu uniform in [0.5, 2]), anisotropic Gaussian
markers with T_x, T_y uniform in [0.2, 1.5], uniform weights 1/N. FP64 pair
sums, Anderson depth 5, damping 0.7, tol 1e-12, abs_floor 0, dt = 0.005, and
Gonzalez off: with Gonzalez on, the LB step on these coarse meshes stagnates in
the FP64 oracle as well.

Reported: the batched step (all 64 instances; predictor + implicit solve; one
batched pair-sum launch per Picard iteration, iterations replayed as a CUDA
graph, tile shapes from the autotuner) against the same step taken by the
single-ensemble solver instance after instance (one context each), from the
same state. Wall time around synchronised calls.

Usage (from the collisionoperators.jl_gb300 directory):
  python -m collops.eval_batch [--steps 2] [--instances 64]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np


def workload(n_inst: int = 64, seed: int = 11):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_inst):
        N = int(np.exp(rng.uniform(np.log(4096), np.log(65536))))
        n = int(rng.integers(24, 49))
        tx, ty = rng.uniform(0.2, 1.5, size=2)
        model = "landau" if k % 2 == 0 else "lb"
        nu = float(rng.uniform(0.5, 2.0)) if model == "lb" else 1.0
        v = np.zeros((N, 2), order="F")
        v[:, 0] = np.sqrt(tx) * rng.standard_normal(N)
        v[:, 1] = np.sqrt(ty) * rng.standard_normal(N)
        out.append(dict(N=N, n=n, model=model, nu=nu, v=v, w=np.full(N, 1.0 / N)))
    return out


def run(steps: int = 2, n_inst: int = 64, dt: float = 0.005, log=print):
    import torch

    import collops as co

    inst = workload(n_inst)
    descs = []
    for d in inst:
        bp = np.linspace(-6.0, 6.0, d["n"] + 1)
        descs.append(dict(bp1=bp, bp2=bp, model=d["model"], nu=d["nu"], N=d["N"]))
    v = torch.cat([torch.from_numpy(np.ascontiguousarray(d["v"].T)).reshape(-1)
                   for d in inst]).cuda()
    w = torch.cat([torch.from_numpy(d["w"]) for d in inst]).cuda()
    p = co.SimParameters(m_anderson=5, damping=0.7, tol=1e-12, abs_floor=0.0, max_iter=2000,
                         use_gonzalez=False)
    o = p.opts()
    batch = co.Batch(descs)
    tune = batch.tune()
    log(f"autotuner: {tune}")

    def batched_step(x, use_graph):
        S0 = batch.entropy(x, w)
        x1 = torch.empty_like(x)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        batch.predictor(o, x1, x, w, dt)
        it, res = batch.step(o, x1, x, w, S0, dt, use_graph=use_graph)
        torch.cuda.synchronize()
        return x1, (time.perf_counter() - t0) * 1e3, it, res

    # the state after one untimed step, then the timed steps
    x, _, _, _ = batched_step(v, True)
    x_start = x.clone()
    times, iters, ress = [], [], []
    n0 = batch.launch_count()
    for _ in range(steps):
        x, ms, it, res = batched_step(x, True)
        times.append(ms)
        iters.append(it)
        ress.append(res)
    launches = (batch.launch_count() - n0) / steps
    _, ms_nograph, it_ng, _ = batched_step(x_start, False)
    batch.close()

    # the same step from x_start, instance after instance
    xs = x_start.cpu().numpy()
    off = 0
    seq_ms = 0.0
    seq_it = []
    for d in inst:
        N = d["N"]
        xi = torch.from_numpy(xs[2 * off:2 * off + 2 * N].copy()).cuda()
        wi = w[off:off + N].contiguous()
        off += N
        bp = np.linspace(-6.0, 6.0, d["n"] + 1)
        ps = co.SimParameters(bp1=bp, bp2=bp, collision_model=d["model"], nu=d["nu"],
                              m_anderson=5, damping=0.7, tol=1e-12, abs_floor=0.0,
                              max_iter=2000, use_gonzalez=False)
        ws = co.build_workspace(ps)
        oi = ps.opts()
        S = C.c_double()
        co._check(ws.lib.co_entropy_of_markers_dev(ws.h, xi.data_ptr(), wi.data_ptr(), N,
                                                   C.byref(S)), "co_entropy_of_markers_dev")
        v1 = torch.empty_like(xi)
        it, nrs = C.c_int(), C.c_int()
        res, r0 = C.c_double(), C.c_double()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        co._check(ws.lib.co_predictor_dev(ws.h, C.byref(oi), v1.data_ptr(), xi.data_ptr(),
                                          wi.data_ptr(), N, dt), "co_predictor_dev")
        co._check(ws.lib.co_step_anderson_dev(ws.h, C.byref(oi), v1.data_ptr(), xi.data_ptr(),
                                              wi.data_ptr(), N, S.value, dt, C.byref(it),
                                              C.byref(res), C.byref(nrs), C.byref(r0)),
                  "co_step_anderson_dev")
        torch.cuda.synchronize()
        seq_ms += (time.perf_counter() - t0) * 1e3
        seq_it.append(it.value)
        ws.close()
    Ns = [d["N"] for d in inst]
    return {
        "workload": f"batch{n_inst}_landau_lb_n4096-65536_mesh24-48_dt{dt}",
        "instances": n_inst, "markers_total": int(sum(Ns)),
        "ordered_pairs_landau_per_map": float(sum(n * (n - 1) for n, d in zip(Ns, inst)
                                                  if d["model"] == "landau")),
        "autotuner": tune,
        "batched_ms_per_step": [round(t, 1) for t in times],
        "batched_iterations_max": [int(max(i)) for i in iters],
        "batched_residual_max": [float(max(r)) for r in ress],
        "batched_launches_per_step": launches,
        "batched_no_graph_ms": round(ms_nograph, 1),
        "sequential_ms_same_step": round(seq_ms, 1),
        "sequential_iterations_max": int(max(seq_it)),
        "speedup_batched_vs_sequential": round(seq_ms / times[0], 2),
    }


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--dt", type=float, default=0.005)
    a = ap.parse_args(argv)
    print(json.dumps(run(a.steps, a.instances, a.dt)))


if __name__ == "__main__":
    main()
