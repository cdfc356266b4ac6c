"""Evaluate the learned warm start against the methods without it.

Workload: Landau, N = 262,144 markers, a bimodal initial condition (two
Gaussians at (+-2.5, 0) with temperature T = 0.4 in both directions, 50/50
split as in main.jl:96-98), uniform weights 1/N, [-8,8]^2 with a 64x64 P_DEG=2
mesh, dt = 0.02, Gonzalez on, Anderson depth 8, damping 0.7, tol 1e-12,
abs_floor 0; defect correction with the benchmark's settings. Markers are seeded synthetic data (numpy default_rng).

The same state sequence is advanced `--steps` times; at each step the implicit
solve is started from
  - learned:    the headline rule (co_step_learned, no retry): whichever of
                the network's proposal v_pred + dt^2 * delta, the predictor and
                the previous state has the smallest first residual;
  - predictor:  the explicit step v0 + dt * vdot(v0) of main.jl:233-245;
  - previous:   the previous step's state v0 itself;
and solved to the same tolerance by the same solver. The trajectory follows the
learned run; the other starts are solved from the same v0 for comparison.
Reported per start: solver iterations, ms per step (CUDA events on the library
stream, warm-start work included) and the final residual.

Usage (from the collisionoperators.jl_gb300 directory):
  python -m collops.eval_warmstart --weights <file.npz> [--steps 3] [--solver anderson]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import statistics

import numpy as np

WORKLOAD = dict(name="landau_bimodal_n262144_mesh64_dt0.02", N=262144, n_el=64, lo=-8.0,
                hi=8.0, peak=2.5, T=0.4, dt=0.02, m=8, damping=0.7, tol=1e-12,
                abs_floor=1e-10, max_iter=2000, stag_window=50, stag_rel_tol=0.01,
                use_logsq=True, seed=7)


def bimodal_markers(N: int, peak: float, T: float, seed: int):
    rng = np.random.default_rng(seed)
    half = N // 2
    v = np.zeros((N, 2), order="F")
    v[:, 0] = np.concatenate([np.full(half, -peak), np.full(N - half, peak)])
    v += np.sqrt(T) * rng.standard_normal((N, 2))
    return v, np.full(N, 1.0 / N)


def run(weights: str, steps: int = 3, solver: str = "anderson", form: str = "mixed_ds",
        N: int | None = None, device: int = 0, log=print):
    import torch

    import collops as co
    from collops import learned

    cfg = dict(WORKLOAD)
    if N:
        cfg["N"] = N
    torch.cuda.set_device(device)
    bp = np.linspace(cfg["lo"], cfg["hi"], cfg["n_el"] + 1)
    p = co.SimParameters(bp1=bp, bp2=bp, m_anderson=cfg["m"], damping=cfg["damping"],
                         tol=cfg["tol"], abs_floor=cfg["abs_floor"], max_iter=cfg["max_iter"],
                         stag_window=cfg["stag_window"], stag_rel_tol=cfg["stag_rel_tol"],
                         use_logsq=cfg["use_logsq"], precision=form)
    ws = co.build_workspace(p, device=device)
    lib, h = ws.lib, ws.h
    stream = torch.cuda.ExternalStream(ws.stream(), device=device)
    # the benchmark's under-relaxed proposal (v_pred + 0.75 dt^2 delta)
    warm = learned.WarmStart.load(weights, device=device, relax=0.75)
    N, dt = cfg["N"], cfg["dt"]
    v_np, w_np = bimodal_markers(N, cfg["peak"], cfg["T"], cfg["seed"])
    dev = torch.device("cuda", device)
    x = torch.from_numpy(np.ascontiguousarray(v_np.T)).to(dev)
    w = torch.from_numpy(w_np).to(dev)
    v1 = torch.empty_like(x)
    # the benchmark's defect-correction settings: eta 0.02, 100 inner maps, stagnation
    # window 5 (stag_rel_tol from the workload), FP32 stage left below a 0.9 cut, no
    # outer mixing, no inner preconditioner, FP32 metric frozen after a 1000x residual
    # drop, stagnation exit after 2 capped inner solves without a new best
    dopt = co.CoDefectOpts(0.02, 100, 5, 0.9, 0, 0, 0, 1e-3, 0, 0, 2)

    def entropy(xx):
        S = C.c_double()
        co._check(lib.co_entropy_of_markers_dev(h, xx.data_ptr(), w.data_ptr(), N, C.byref(S)),
                  "co_entropy_of_markers_dev")
        return S.value

    def step(x0, S0, start):
        o = p.opts()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        used = None
        it, nrs = C.c_int(), C.c_int()
        res, r0 = C.c_double(), C.c_double()
        if start == "learned":
            rec = warm.step(ws, o, dopt if solver == "defect" else None, x0, w, S0, dt, v1,
                            retry=False)
            used = rec["start"]
            it.value, res.value, r0.value = rec["outer"], rec["res"], rec["r0"]
        else:
            if start == "predictor":
                co._check(lib.co_predictor_dev(h, C.byref(o), v1.data_ptr(), x0.data_ptr(),
                                               w.data_ptr(), N, dt), "co_predictor_dev")
            else:
                with torch.cuda.stream(stream):
                    v1.copy_(x0)
            if solver == "defect":
                co._check(lib.co_step_defect_dev(h, C.byref(o), C.byref(dopt), v1.data_ptr(),
                                                 x0.data_ptr(), w.data_ptr(), N, S0, dt,
                                                 C.byref(it), C.byref(res), C.byref(nrs),
                                                 C.byref(r0)), "co_step_defect_dev")
            else:
                co._check(lib.co_step_anderson_dev(h, C.byref(o), v1.data_ptr(), x0.data_ptr(),
                                                   w.data_ptr(), N, S0, dt, C.byref(it),
                                                   C.byref(res), C.byref(nrs), C.byref(r0)),
                          "co_step_anderson_dev")
        e1.record(stream)
        torch.cuda.synchronize()
        conv = res.value < max(cfg["tol"] * float(torch.linalg.vector_norm(v1)),
                                cfg["abs_floor"])
        return v1.clone(), dict(iterations=it.value, residual=res.value, first_residual=r0.value,
                                ms=e0.elapsed_time(e1), start=used, converged=bool(conv))

    starts = ("learned", "predictor", "previous")
    rec = {s: [] for s in starts}
    S0 = entropy(x)
    for k in range(steps):
        out = {}
        for s in starts:
            out[s] = step(x, S0, s)
            rec[s].append(out[s][1])
        log(f"step {k}: " + ", ".join(f"{s} {out[s][1]['iterations']} it "
                                      f"{out[s][1]['ms']:.0f} ms" for s in starts))
        x = out["learned"][0]
        S0 = entropy(x)
    summary = {s: dict(iterations_mean=statistics.mean(r["iterations"] for r in rec[s]),
                       ms_per_step=statistics.mean(r["ms"] for r in rec[s]),
                       converged_steps=sum(r["converged"] for r in rec[s]),
                       ms_per_converged_step=(statistics.mean(r["ms"] for r in rec[s]
                                                              if r["converged"])
                                              if any(r["converged"] for r in rec[s]) else None),
                       residual_max=max(r["residual"] for r in rec[s]),
                       first_residual_mean=statistics.mean(r["first_residual"] for r in rec[s]))
               for s in starts}
    summary["learned"]["starts_chosen"] = {k: sum(r["start"] == k for r in rec["learned"])
                                           for k in ("learned", "predictor", "previous")}
    ws.close()
    return {"workload": cfg["name"], "N": N, "solver": solver, "form": form, "steps": steps,
            "tol": cfg["tol"], "summary": summary, "per_step": rec}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--weights", required=True)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--solver", choices=["anderson", "defect"], default="anderson")
    ap.add_argument("--form", choices=["fp64", "mixed", "mixed_ds"], default="mixed_ds")
    ap.add_argument("--N", type=int, default=None)
    a = ap.parse_args(argv)
    r = run(a.weights, a.steps, a.solver, a.form, a.N)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
