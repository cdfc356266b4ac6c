"""Evaluate the batched engine on the many-ensemble workload.

Workload: 64 independent instances with seeded parameters -- N log-uniform in
[4096, 65536], uniform meshes of 24..48 cells per dimension on [-6,6]^2,
alternately Landau and LB (nu uniform in [0.5, 2]), anisotropic Gaussian
markers with T_x, T_y uniform in [0.2, 1.5], uniform weights 1/N. FP64 pair
sums, Gonzalez on, Anderson depth 5, damping 0.7, tol 1e-12, abs_floor 0 and,
as the batched configuration states no time step, dt = 0.001 (the DT of the
reference's Landau and LB presets). The LB instances stagnate at this setting in
the FP64 oracle as well (the Gonzalez-corrected LB map does not contract on
these coarse meshes) and leave through the stagnation exit.

Reported: `--steps` consecutive batched steps (all instances; predictor +
implicit solve; one batched pair-sum launch per Picard iteration; the iteration
runs as a CUDA graph whose conditional WHILE node repeats it on the device until
an instance finishes; tile shapes from the autotuner), against step 0 taken by
the single-ensemble solver instance after instance (one context each) from the
same state. Wall time around synchronised calls. The comparison of batched
instances with the CPU oracle is a test (tests/test_batch_gpu.py).

Usage (from the collisionoperators.jl_gb300 directory):
  python -m collops.eval_batch [--steps 20] [--instances 64]
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


def _single_step(co, d, xi, wi, dt, gonzalez):
    """step 0 of one instance through its own context; returns (ms, iterations,
    residual, result)."""
    import torch
    N = d["N"]
    bp = np.linspace(-6.0, 6.0, d["n"] + 1)
    ps = co.SimParameters(bp1=bp, bp2=bp, collision_model=d["model"], nu=d["nu"],
                          m_anderson=5, damping=0.7, tol=1e-12, abs_floor=0.0,
                          max_iter=2000, use_gonzalez=gonzalez)
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
    ms = (time.perf_counter() - t0) * 1e3
    ws.close()
    return ms, it.value, res.value, v1


def run(steps: int = 20, n_inst: int = 64, dt: float = 0.001, gonzalez: bool = True,
        log=print):
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
                         use_gonzalez=gonzalez)
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
        return x1, (time.perf_counter() - t0) * 1e3, np.array(it), np.array(res)

    Ns = [d["N"] for d in inst]
    offs = np.concatenate([[0], np.cumsum(Ns)]).astype(int)

    def converged(x, res):
        xs = x.cpu().numpy()
        return [bool(res[k] < 1e-12 * np.linalg.norm(xs[2 * offs[k]:2 * offs[k + 1]]))
                for k in range(n_inst)]

    x = v.clone()
    times, iters_max, conv_counts = [], [], []
    first = None
    n0 = batch.launch_count()
    for s in range(steps):
        x, ms, it, res = batched_step(x, True)
        times.append(ms)
        iters_max.append(int(it.max()))
        cv = converged(x, res)
        conv_counts.append(int(sum(cv)))
        if s == 0:
            first = (x.clone(), it, res, cv)
        log(f"step {s}: {ms:.1f} ms, max iterations {it.max()}, converged {sum(cv)}/{n_inst}")
    launches = (batch.launch_count() - n0) / steps
    _, ms_nograph, _, _ = batched_step(v, False)
    batch.close()

    # step 0 from the initial state, instance after instance, against the batch
    seq_ms = 0.0
    seq_it = []
    diffs = []
    x0b = first[0].cpu().numpy()
    for k, d in enumerate(inst):
        xi = v[2 * offs[k]:2 * offs[k + 1]].clone()
        wi = w[offs[k]:offs[k + 1]].contiguous()
        ms, itk, resk, y = _single_step(co, d, xi, wi, dt, gonzalez)
        seq_ms += ms
        seq_it.append(itk)
        if first[3][k]:
            got = x0b[2 * offs[k]:2 * offs[k + 1]]
            yy = y.reshape(-1).cpu().numpy()
            diffs.append(float(np.max(np.abs(got - yy)) / np.max(np.abs(yy))))
    out = {
        "workload": f"batch{n_inst}_landau_lb_n4096-65536_mesh24-48_dt{dt}_gonzalez{int(gonzalez)}",
        "instances": n_inst, "markers_total": int(sum(Ns)),
        "ordered_pairs_landau_per_map": float(sum(n * (n - 1) for n, d in zip(Ns, inst)
                                                  if d["model"] == "landau")),
        "autotuner": tune, "steps": steps,
        "batched_ms_per_step": [round(t, 1) for t in times],
        "batched_ms_per_step_mean": round(float(np.mean(times)), 1),
        "batched_iterations_max": iters_max,
        "converged_instances_per_step": conv_counts,
        "batched_launches_per_step": launches,
        "batched_no_graph_ms_step0": round(ms_nograph, 1),
        "batched_ms_step0": round(times[0], 1),
        "sequential_ms_step0": round(seq_ms, 1),
        "sequential_iterations_max_step0": int(max(seq_it)),
        "speedup_batched_vs_sequential_step0": round(seq_ms / times[0], 2),
        "converged_batched_vs_single_max_rel_diff": max(diffs) if diffs else None,
    }
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--dt", type=float, default=0.001)
    ap.add_argument("--no-gonzalez", dest="gonzalez", action="store_false")
    a = ap.parse_args(argv)
    print(json.dumps(run(a.steps, a.instances, a.dt, a.gonzalez)))


if __name__ == "__main__":
    main()
