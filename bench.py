#!/usr/bin/env python3
"""Benchmark: ms per converged implicit step, Landau N = 131,072.

Workload (the precision-form configuration): Landau, N = 131,072 markers from an
anisotropic Gaussian (T_x = 1.0, T_y = 0.25, i.e. sigma = (1, 0.5)), uniform
weights 1/N, [-6,6]^2 with a 64x64 P_DEG=2 mesh, dt = 0.02, Gonzalez on,
N_QUAD 6, tol 1e-12. use_logsq = true and abs_floor 1e-10 (below tol*||v|| =
4e-10, so tol binds) are the settings of the reference's production Landau
presets (parameters_sq_d04.jl, parameters_bimodal_v1.jl); the solver knobs
are the SimParameters defaults (Parameters.jl:66-91): Anderson depth 8, damping
0.7, stagnation window 50 with stag_rel_tol 0.01, and the defect correction's
window of 5 outer maps. Markers are seeded synthetic data (numpy
default_rng(42)).

One "step" = one time step of the reference's loop (main.jl:226-300): the warm
start, the implicit solve, and the entropy S0 of the new state for the next
step. `--steps K` times K CONSECUTIVE time steps from the initial markers, each
starting from the state the previous one returned. A step either converges
(||G(v) - v|| < max(tol*||v||, abs_floor)) or leaves through the reference's
stagnation exit with its best iterate (solver.jl:357-367) and the trajectory
continues from there, as the reference's time loop does. `value` is the mean ms
over the converged steps; stagnated steps are counted and timed separately.

The headline form is one C-ABI call per step (co_step_learned_dev): features,
the learned proposal (BF16 MLP), the explicit predictor and the previous-step
state as starts, the solve from the start with the smallest first residual --
mixed precision (FP32 pair maps, then double-single pair maps) under defect
correction around a frozen metric -- one retry from the next start if the solve
does not converge, and the new state's entropy. Inputs are resident in HBM;
W warm-up steps repeat step 0. `plain_fp64` times the plain FP64 form (Anderson
on FP64 pair maps from the FP64 explicit predictor: the reference's GPU
configuration) on the first `--plain-steps` states of the same trajectory. `e2e`
runs the same steps through the host-pointer call co_step_learned from pinned
host arrays, copies inside the timed region. Each timed step is bracketed by
CUDA events on the library's stream; a 256 MB buffer is written before each
timed step to flush L2.

--impl reference times the CPU FP64 oracle (the reference's CPU algorithm,
OpenMP over all host cores) on the same workload: each timed sample is one
complete Picard map with every pair evaluated, scaled to a converged step by
the FP64 maps per step of this workload (measured by the plain FP64 GPU step,
the same algorithm, see FP64_MAPS_PER_STEP).
"""
from __future__ import annotations

import argparse
import csv
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "collisionoperators.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "ms/converged implicit step, Landau N=131k: mixed+learned vs plain FP64 GPU"
UNIT = "ms/step"
WORKLOAD = dict(name="landau_n131072_mesh64_dt0.02", N=131072, n_el=64, lo=-6.0, hi=6.0,
                sx=1.0, sy=0.5, dt=0.02, m=8, damping=0.7, tol=1e-12, abs_floor=1e-10,
                max_iter=2000, stag_window=50, stag_rel_tol=0.01, use_logsq=True, seed=42)
# FP64 Picard maps of a converged plain FP64 step of this workload (Anderson
# iterations + the explicit predictor), measured by the plain_fp64 leg of this
# benchmark on GB300 (step 0 from the initial markers). The reference arm
# scales its measured per-map time by it: a converged CPU step takes far longer
# than the few minutes a benchmark run may take.
FP64_MAPS_PER_STEP = 284
FP64_MAPS_SOURCE = ("plain FP64 step 0 of this workload on GB300 (plain_fp64.iterations + 1 of "
                    "python bench.py)")
C1 = dict(name="landau_n2048_mesh16_dt0.05", N=2048, n_el=16, lo=-6.0, hi=6.0, sx=1.0, sy=0.5,
          dt=0.05, m=5, damping=0.7, tol=1e-12, abs_floor=0.0, max_iter=400, stag_window=50,
          stag_rel_tol=0.01, use_logsq=False, seed=42)


def markers(cfg, seed):
    rng = np.random.default_rng(seed)
    N = cfg["N"]
    v = np.zeros((N, 2), order="F")
    v[:, 0] = cfg["sx"] * rng.standard_normal(N)
    v[:, 1] = cfg["sy"] * rng.standard_normal(N)
    w = np.full(N, 1.0 / N)
    return v, w


def bp_of(cfg):
    return np.linspace(cfg["lo"], cfg["hi"], cfg["n_el"] + 1)


# ---------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for r in csv.reader(f):
                if len(r) >= 9:
                    rows.append([x.strip() for x in r])
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------- multi-GPU

def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def aggregate(elapsed_ms: float, steps: int, world: int, group=None):
    """Replicas: every rank runs the same workload on its own GPU; the job time
    is the max over ranks, and the job's ms per step is that time over all
    ranks' steps (weak scaling). Returns (job_ms_per_step, max_elapsed_ms)."""
    t = elapsed_ms
    if world > 1:
        import torch
        import torch.distributed as dist
        x = torch.tensor([elapsed_ms], dtype=torch.float64,
                         device="cuda" if dist.get_backend(group) == "nccl" else "cpu")
        dist.all_reduce(x, op=dist.ReduceOp.MAX, group=group)
        t = float(x.item())
    return t / (steps * world), t


def converged_mean(times, flags):
    """(ms per converged step, its sample count); the mean over all steps when
    none converged (then flagged by count 0)."""
    sel = [t for t, f in zip(times, flags) if f]
    if sel:
        return statistics.mean(sel), len(sel)
    return (statistics.mean(times) if times else 0.0), 0


# ---------------------------------------------------------------- CPU side

def oracle_full_map_ms(cfg, threads: int, reps: int = 1):
    """One complete Picard map of the CPU FP64 oracle on the workload (every
    ordered pair, the projection, quadrature, mass solves and G): wall ms per
    map over `reps` maps."""
    import oracle
    oracle.build()
    bp = bp_of(cfg)
    om = oracle.OracleMesh(bp, bp, 6, use_logsq=cfg["use_logsq"])
    o = oracle.Opts(model="landau", nthreads=threads)
    v, w = markers(cfg, cfg["seed"])
    S0 = om.entropy(om.l2_project(v, w))
    N = cfg["N"]
    # v_in: a perturbed state standing in for an iterate (same cost as any other)
    v_in = np.asfortranarray(v + 1e-3 * np.sin(np.arange(2 * N)).reshape(N, 2, order="F"))
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        om.picard_map(o, v_in, v, w, S0, cfg["dt"])
        ts.append((time.perf_counter() - t0) * 1e3)
    return statistics.mean(ts), ts


def c1_cpu_steps(threads: int, steps: int = 3):
    """The C1 workload (N = 2048, 16x16, dt 0.05, Anderson depth 5) solved by the
    CPU oracle's step_anderson! for `steps` consecutive steps, each timed in
    full. Returns (ms per step list, states list, S0 list, iteration list)."""
    import oracle
    oracle.build()
    cfg = C1
    bp = bp_of(cfg)
    om = oracle.OracleMesh(bp, bp, 6, use_logsq=cfg["use_logsq"])
    o = oracle.Opts(model="landau", m=cfg["m"], tol=cfg["tol"], abs_floor=cfg["abs_floor"],
                    damping=cfg["damping"], max_iter=cfg["max_iter"],
                    stag_window=cfg["stag_window"], stag_rel_tol=cfg["stag_rel_tol"],
                    nthreads=threads)
    v, w = markers(cfg, cfg["seed"])
    ms, states, S0s, its = [], [], [], []
    x = v
    for _ in range(steps):
        t0 = time.perf_counter()
        S0 = om.entropy(om.l2_project(x, w))
        v1 = om.predictor(o, x, w, cfg["dt"])
        xn, info = om.step_anderson(o, v1, x, w, S0, cfg["dt"])
        ms.append((time.perf_counter() - t0) * 1e3)
        states.append(x)
        S0s.append(S0)
        its.append(info[0])
        x = xn
    return ms, states, S0s, its, w


def cpu_baseline(cfg, maps_per_step, maps_src, c1_gpu=None):
    threads = os.cpu_count() or 1
    per_map, _ = oracle_full_map_ms(cfg, threads)
    value = per_map * maps_per_step
    out = dict(value=round(value, 1), unit=UNIT, cores=threads, kind="port",
               extrapolated=True, per_map_ms=round(per_map, 1),
               maps_per_step=round(maps_per_step, 1), maps_source=maps_src,
               sample=(f"one complete FP64 oracle Picard map at N={cfg['N']} (every pair, "
                       f"projection, quadrature, mass solves, grad L) timed: "
                       f"{per_map:.0f} ms; scaled by {maps_per_step:.0f} maps per converged "
                       f"FP64 step ({maps_src})"),
               measured="per_map_ms (one full map); the maps per step come from the plain "
                        "FP64 GPU step of the same algorithm")
    if c1_gpu is not None:
        cpu_ms, _states, _s0, its, _w = c1_gpu["cpu"]
        out["c1_full_steps"] = dict(
            workload=C1["name"], steps=len(cpu_ms),
            cpu_ms_per_step=round(statistics.mean(cpu_ms), 1),
            cpu_iterations=its, gpu_fp64_ms_per_step=round(statistics.mean(c1_gpu["gpu_ms"]), 2),
            gpu_iterations=c1_gpu["gpu_its"],
            ratio=round(statistics.mean(cpu_ms) / statistics.mean(c1_gpu["gpu_ms"]), 1),
            note="both sides run step_anderson! in FP64 on the same states, every step "
                 "timed in full (predictor + solve), CPU on all host cores")
    return out


# ---------------------------------------------------------------- GPU side

def run_gpu(args, cfg):
    import torch

    world, rank, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import collops as co
    lib = co.load_library()
    N, dt = cfg["N"], cfg["dt"]
    bp = bp_of(cfg)
    p = co.SimParameters(bp1=bp, bp2=bp, m_anderson=cfg["m"], damping=cfg["damping"],
                         tol=cfg["tol"], abs_floor=cfg["abs_floor"], max_iter=cfg["max_iter"],
                         stag_window=cfg["stag_window"], stag_rel_tol=cfg["stag_rel_tol"],
                         use_logsq=cfg["use_logsq"])
    ws = co.build_workspace(p, device=local)
    h = ws.h
    sptr = C.c_void_p()
    lib.co_ctx_stream(h, C.byref(sptr))
    stream = torch.cuda.ExternalStream(sptr.value)

    peak32, peak64 = C.c_double(), C.c_double()
    lib.co_measure_fma_peak(local, 0, C.byref(peak32))
    lib.co_measure_fma_peak(local, 1, C.byref(peak64))

    v_np, w_np = markers(cfg, cfg["seed"] + rank)
    dev = torch.device("cuda", local)
    v = torch.from_numpy(np.ascontiguousarray(v_np.T)).to(dev)      # (2, N) = Julia N x 2
    w = torch.from_numpy(w_np).to(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def opts(prec):
        return p.opts(precision=co._PREC[prec], mixed_floor=args.mixed_floor)

    # the defect correction's outer stagnation test uses stag_rel_tol over
    # dc_stag_window outer maps (Parameters.jl:89-91)
    dopt = co.CoDefectOpts(args.dc_eta, args.dc_max_inner, args.dc_stag_window,
                           args.dc_fp32_stall, 0, args.dc_outer_m, args.dc_precond,
                           args.dc_metric_freeze, args.dc_fp32_window, args.dc_cap_refresh,
                           args.dc_cap_abort)
    dptr = C.byref(dopt) if args.solver == "defect" else None

    from collops import learned
    warm = None
    if args.warmstart == "learned":
        if not os.path.exists(args.warmstart_file):
            raise SystemExit(f"warm-start weights not found: {args.warmstart_file}")
        warm = learned.WarmStart.load(args.warmstart_file, device=local, relax=args.warm_relax)
    mlp_h = warm.mlp.h if warm is not None else None
    o_head = opts(args.form)

    def step_dev(x, S0, out):
        """the headline step through co_step_learned_dev; returns its record"""
        info = co.CoStepInfo()
        co._check(lib.co_step_learned_dev(h, C.byref(o_head), dptr, mlp_h, int(args.retry),
                                          out.data_ptr(), x.data_ptr(), w.data_ptr(), N, S0, dt,
                                          C.byref(info)), "co_step_learned_dev")
        return info.as_dict()

    def fp64_residual(x_new, x_old, S_old):
        """||G64(x) - x|| of a returned state (one FP64 Picard map, untimed)."""
        r = C.c_double()
        o = opts("fp64")
        co._check(lib.co_picard_residual_dev(h, C.byref(o), x_new.data_ptr(), x_old.data_ptr(),
                                             w.data_ptr(), N, S_old, dt, C.byref(r)),
                  "co_picard_residual_dev")
        return r.value

    diag6 = np.zeros(6)

    def energy_momentum(x):
        co._check(lib.co_diagnostics_dev(h, x.data_ptr(), w.data_ptr(), N, co._p(diag6)),
                  "co_diagnostics_dev")
        return float(diag6[1]), float(diag6[2]), float(diag6[3])

    S_ic = learned.entropy_of(ws, v, w)
    x_ic = v.clone()
    out = torch.empty_like(v)

    # warm-up: W steps from the initial markers (the state is not advanced)
    for _ in range(args.warmup):
        step_dev(x_ic, S_ic, out)
    torch.cuda.synchronize()

    # ---- timed headline form: K consecutive steps
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    lib.co_profile(h, 1)
    n_launch0 = ws.launch_count()
    states, S0s, recs, times = [x_ic], [S_ic], [], []
    launches = 0
    cur, S_cur = x_ic, S_ic
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        n0 = ws.launch_count()
        e0.record(stream)
        nxt = torch.empty_like(v)
        rec = step_dev(cur, S_cur, nxt)
        e1.record(stream)
        torch.cuda.synchronize()
        launches += ws.launch_count() - n0
        times.append(e0.elapsed_time(e1))
        recs.append(rec)
        states.append(nxt)
        S0s.append(rec["S_new"])
        cur, S_cur = nxt, rec["S_new"]
    prof = co.CoProfile()
    lib.co_profile_read(h, C.byref(prof))
    lib.co_profile(h, 0)
    clk = clocks.stop()
    del n_launch0
    # untimed per-step checks: the FP64 map residual of each returned state and
    # its momentum / energy drift from the step's start
    for k, rec in enumerate(recs):
        x0, x1 = states[k], states[k + 1]
        rec["fp64_residual"] = fp64_residual(x1, x0, S0s[k])
        rec["tol_norm"] = max(cfg["tol"] * float(torch.linalg.vector_norm(x1)), cfg["abs_floor"])
        E0, P10, P20 = energy_momentum(x0)
        E1, P11, P21 = energy_momentum(x1)
        rec["momentum_drift"] = max(abs(P11 - P10), abs(P21 - P20))
        rec["energy_drift_rel"] = abs(E1 - E0) / E0
    conv = [bool(r["converged"]) for r in recs]
    value, n_conv = converged_mean(times, conv)
    if world > 1:
        dist.barrier()
    job_ms, _ = aggregate(value, 1, world)
    stag_t = [t for t, f in zip(times, conv) if not f]

    # ---- the plain FP64 form on the first states of the same trajectory
    plain = None
    x64_step0 = None
    if args.plain_steps > 0:
        lib.co_profile(h, 1)
        o64 = opts("fp64")
        tp, ip, cp, rp, fr = [], [], [], [], []
        for k in range(min(args.plain_steps, args.steps)):
            x0, S0 = states[k], S0s[k]
            v1 = torch.empty_like(v)
            with torch.cuda.stream(stream):
                flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            co._check(lib.co_predictor_dev(h, C.byref(o64), v1.data_ptr(), x0.data_ptr(),
                                           w.data_ptr(), N, dt), "co_predictor_dev")
            it, nrs = C.c_int(), C.c_int()
            res, r0 = C.c_double(), C.c_double()
            co._check(lib.co_step_anderson_dev(h, C.byref(o64), v1.data_ptr(), x0.data_ptr(),
                                               w.data_ptr(), N, S0, dt, C.byref(it),
                                               C.byref(res), C.byref(nrs), C.byref(r0)),
                      "co_step_anderson_dev")
            e1.record(stream)
            torch.cuda.synchronize()
            tp.append(e0.elapsed_time(e1))
            ip.append(it.value)
            rp.append(res.value)
            cp.append(res.value < max(cfg["tol"] * float(torch.linalg.vector_norm(v1)),
                                      cfg["abs_floor"]))
            if k == 0:
                x64_step0 = v1.clone()
            fr.append(fp64_residual(v1, x0, S0))
        prof64 = co.CoProfile()
        lib.co_profile_read(h, C.byref(prof64))
        lib.co_profile(h, 0)
        pm, pn = converged_mean(tp, cp)
        plain = dict(ms_per_step=round(pm, 1), steps=len(tp), converged_steps=pn,
                     step_ms=[round(t, 1) for t in tp], converged=cp, iterations=ip,
                     residuals=rp, maps=[i + 1 for i in ip], fp64_residual_returned=fr,
                     pair64_ms_avg=(prof64.pair64_ms / max(1, prof64.pair64_launches)),
                     solver="step_anderson! on FP64 pair maps from the FP64 explicit predictor")
    else:
        prof64 = co.CoProfile()

    # ---- accuracy of the headline step 0 against FP64
    acc = None
    if args.accuracy:
        xh = states[1]
        # the FP64 fixed point nearest the headline result: plain FP64 Anderson
        # started from it
        o64 = opts("fp64")
        xp = xh.clone()
        it, nrs = C.c_int(), C.c_int()
        res, r0 = C.c_double(), C.c_double()
        co._check(lib.co_step_anderson_dev(h, C.byref(o64), xp.data_ptr(), x_ic.data_ptr(),
                                           w.data_ptr(), N, S_ic, dt, C.byref(it), C.byref(res),
                                           C.byref(nrs), C.byref(r0)), "co_step_anderson_dev")
        ah, ap = xh.cpu().numpy(), xp.cpu().numpy()
        acc = dict(
            step=0,
            fp64_polish=dict(iterations=it.value, residual=res.value),
            vel_err_rel_vs_fp64_polish=float(np.abs(ah - ap).max() / np.abs(ap).max()),
            fp64_map_residual_headline=recs[0]["fp64_residual"],
            tol_times_norm=recs[0]["tol_norm"],
            note="the implicit Gonzalez step can have several roots; the polish measures "
                 "the distance from the headline result to the FP64 fixed point it sits on")
        if x64_step0 is not None:
            a64 = x64_step0.cpu().numpy()
            acc["root_diff_rel_vs_plain_fp64"] = float(np.abs(ah - a64).max() /
                                                        np.abs(a64).max())
            acc["plain_fp64_map_residual"] = fp64_residual(x64_step0, x_ic, S_ic)

    # ---- e2e: host arrays in pinned memory through co_step_learned
    e2e = None
    if args.e2e_steps > 0:
        ke = min(args.e2e_steps, args.steps)
        vh = torch.empty((2, N), dtype=torch.float64).pin_memory()
        wh = torch.from_numpy(w_np).pin_memory()
        vout = torch.empty((2, N), dtype=torch.float64).pin_memory()
        dp = C.POINTER(C.c_double)
        ets, econv = [], []
        for k in range(ke):
            vh.copy_(states[k].cpu())
            with torch.cuda.stream(stream):
                flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            info = co.CoStepInfo()
            co._check(lib.co_step_learned(h, C.byref(o_head), dptr, mlp_h, int(args.retry),
                                          C.cast(vout.data_ptr(), dp), C.cast(vh.data_ptr(), dp),
                                          C.cast(wh.data_ptr(), dp), N, S0s[k], dt,
                                          C.byref(info)), "co_step_learned")
            e1.record(stream)
            torch.cuda.synchronize()
            ets.append(e0.elapsed_time(e1))
            econv.append(bool(info.converged))
        em, en = converged_mean(ets, econv)
        e2e_job, _ = aggregate(em, 1, world)
        e2e = dict(value=round(e2e_job, 2), unit=UNIT, h2d_bytes_per_step=8 * 3 * N,
                   d2h_bytes_per_step=8 * 2 * N, steps=ke, converged_steps=en,
                   step_ms=[round(t, 1) for t in ets],
                   path="pinned host arrays -> co_step_learned (C ABI: copies in, whole step "
                        "on the device, copies out) -> host")

    # ---- roofline of the pair kernels
    def roof(ms, launches_, pairs, peak, kind, kernel):
        if launches_ == 0:
            return None
        avg_ms = ms / launches_
        flops = 23.0 * pairs / launches_            # 23 algorithmic flops per ordered pair
        achieved = flops / (avg_ms * 1e-3) / 1e12
        pk = peak / 1e12
        return {"bound": kind,
                "bound_note": "SIMT pipe bound (FP32 FMA or FP64): an N-body pair sum, no "
                              "tensor-core contraction; inputs are L2-resident, so not HBM",
                "achieved": round(achieved, 3), "peak": round(pk, 3),
                "unit": "TFLOP/s", "frac": round(achieved / pk, 4), "traffic": None,
                "kernel": kernel, "avg_launch_ms": round(avg_ms, 3), "launches": launches_,
                "pairs_per_launch": pairs / launches_,
                "peak_source": "measured in this run: FMA-chain kernel (co_measure_fma_peak), "
                               "2 flops per FMA; no FP32/FP64 SIMT figure in MEASURED_PEAKS.json"}

    r32 = roof(prof.pair32_ms, prof.pair32_launches, prof.pair32_pairs, peak32.value, "fp32",
               "k_pair32_sym")
    rds = roof(prof.pairds_ms, prof.pairds_launches, prof.pairds_pairs, peak32.value, "fp32",
               "k_pair_ds_sym")
    r64 = roof(prof64.pair64_ms, prof64.pair64_launches, prof64.pair64_pairs, peak64.value,
               "fp64", "k_pair64_sym")
    if rds:
        rds["fp64_equivalent_frac"] = round(rds["achieved"] / (peak64.value / 1e12), 3)
        rds["note"] = ("double-single (FP32 head+tail) arithmetic: 23 FP64-equivalent flops per "
                       "ordered pair; frac is against the FP32 peak by the 23-flop count, "
                       "fp64_equivalent_frac against the measured FP64 peak")
    cands = [(prof.pair32_ms, r32), (prof.pairds_ms, rds)]
    dominant = max((c for c in cands if c[1]), key=lambda c: c[0], default=(0, None))[1]
    traffic = load_traffic()
    for rr in (r32, r64, rds):
        if rr:
            if traffic.get(rr["kernel"]) is not None:
                rr["traffic"] = traffic[rr["kernel"]]
            for key in ("ncu_issue_active", "ncu_fma_pipe", "ncu_fp64_pipe"):
                val = load_profile_lines(key).get(rr["kernel"])
                if val is not None:
                    rr[key] = val

    # ---- CPU baseline (rank 0, one GPU)
    cpu = None
    if rank == 0 and world == 1 and args.cpu_baseline:
        maps = FP64_MAPS_PER_STEP
        src = FP64_MAPS_SOURCE
        if plain and plain["converged"][0]:
            maps, src = plain["maps"][0], "the plain FP64 GPU step 0 of this run"
        c1 = c1_compare(args, co, torch)
        cpu = cpu_baseline(cfg, maps, src, c1)

    line = {
        "metric": METRIC, "value": round(job_ms, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(job_ms, 2),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": {"mixed": "fp32 pair maps + fp64 pair maps",
                  "mixed_ds": "fp32 pair maps + double-single (fp32x2) pair maps",
                  "fp64": "fp64"}[args.form] + "; fp64 projection, mass solve, Gonzalez, solver",
        "data": "synthetic: seeded anisotropic Gaussian markers (numpy default_rng)",
        "config": {"workload": cfg["name"], "form": args.form, "solver": args.solver, "N": N,
                   "mesh": f"{cfg['n_el']}x{cfg['n_el']} P2 on [{cfg['lo']},{cfg['hi']}]^2",
                   "dt": dt, "anderson_m": cfg["m"], "damping": cfg["damping"],
                   "tol": cfg["tol"], "abs_floor": cfg["abs_floor"], "gonzalez": True,
                   "use_logsq": cfg["use_logsq"], "stag_window": cfg["stag_window"],
                   "stag_rel_tol": cfg["stag_rel_tol"], "dc_stag_window": args.dc_stag_window,
                   "defect": {"eta": args.dc_eta, "max_inner": args.dc_max_inner,
                              "fp32_stall": args.dc_fp32_stall, "outer_m": args.dc_outer_m,
                              "precond": args.dc_precond,
                              "metric_freeze": args.dc_metric_freeze,
                              "cap_abort": args.dc_cap_abort,
                              "cap_refresh": args.dc_cap_refresh},
                   "warmstart": args.warmstart, "warm_relax": args.warm_relax,
                   "retry": bool(args.retry),
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "256 MB buffer written before each timed step"},
        "timed_steps": f"{args.steps} consecutive time steps from the initial markers; a "
                       "stagnated step returns its best iterate and the trajectory continues",
        "value_over": f"the {n_conv} converged steps" if n_conv else "all steps (none converged)",
        "steps_converged": n_conv, "steps_stagnated": len(stag_t),
        "stagnated_ms_mean": round(statistics.mean(stag_t), 1) if stag_t else None,
        "ms_per_step_all": round(statistics.mean(times), 2),
        "step_ms": [round(t, 1) for t in times], "converged": conv,
        "per_step": recs,
        "maps": {"fp32": prof.maps32, "double_single": prof.mapsds, "fp64": prof.maps64},
        "plain_fp64": plain, "accuracy": acc,
        "warmstart": ({"kind": "learned MLP (BF16, own kernels)", "file": os.path.relpath(
            args.warmstart_file, ROOT),
            "starts": {s: sum(1 for r in recs if r["start"] == s)
                       for s in ("learned", "predictor", "previous")},
            "retries": sum(1 for r in recs if r["attempts"] > 1),
            "relax": args.warm_relax,
            "rule": "start with the smallest first residual among the learned proposal "
                    "(v_pred + relax dt^2 delta), the explicit predictor and the previous-step "
                    "state; a solve that does not converge is repeated once from the next "
                    "start"}
            if warm is not None else {"kind": "explicit predictor or previous-step state"}),
        "roofline": dominant, "roofline_fp64": r64, "roofline_fp32": r32, "roofline_ds": rds,
        "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": int(launches),
    }
    if plain:
        line["speedup_vs_plain_fp64"] = round(plain["ms_per_step"] / job_ms, 2)
        line["speedup_step0_vs_plain_fp64_step0"] = round(plain["step_ms"][0] / times[0], 2)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def c1_compare(args, co, torch):
    """The C1 workload fully timed on both sides: the CPU oracle's FP64
    step_anderson! and the library's FP64 step (predictor + solve) on the same
    states."""
    threads = os.cpu_count() or 1
    cpu = c1_cpu_steps(threads, steps=args.c1_steps)
    cpu_ms, states, S0s, _its, w = cpu
    cfg = C1
    bp = bp_of(cfg)
    p = co.SimParameters(bp1=bp, bp2=bp, m_anderson=cfg["m"], damping=cfg["damping"],
                         tol=cfg["tol"], abs_floor=cfg["abs_floor"], max_iter=cfg["max_iter"],
                         stag_window=cfg["stag_window"], stag_rel_tol=cfg["stag_rel_tol"],
                         use_logsq=cfg["use_logsq"])
    ws = co.build_workspace(p)
    gpu_ms, gpu_its = [], []
    for x, S0 in zip(states, S0s):
        y = np.zeros_like(x, order="F")
        t0 = time.perf_counter()
        co.predictor(ws, y, x, w, cfg["dt"])
        info = co.step_anderson(ws, y, x, w, S0, cfg["dt"], m=cfg["m"], tol=cfg["tol"],
                                abs_floor=cfg["abs_floor"], damping=cfg["damping"],
                                max_iter=cfg["max_iter"], stag_window=cfg["stag_window"],
                                stag_rel_tol=cfg["stag_rel_tol"])
        gpu_ms.append((time.perf_counter() - t0) * 1e3)
        gpu_its.append(info[0])
    ws.close()
    return dict(cpu=cpu, gpu_ms=gpu_ms, gpu_its=gpu_its)


def load_profile_lines(key: str = "traffic_bytes_per_launch"):
    """Per-kernel figures from the committed ncu summaries: profiles/*.md lines
    '<key> <kernel>: <value>' (DRAM bytes per launch, pipe fractions)."""
    out = {}
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return out
    for fn in sorted(os.listdir(d)):
        if not fn.endswith(".md"):
            continue
        for line in open(os.path.join(d, fn)):
            if line.startswith(key + " "):
                k, val = line[len(key) + 1:].split(":")
                try:
                    out[k.strip()] = float(val)
                except ValueError:
                    pass
    return out


def load_traffic():
    return load_profile_lines("traffic_bytes_per_launch")


def run_reference(args, cfg):
    """The reference's CPU algorithm (the FP64 oracle port, all host cores): K
    timed samples, each one complete Picard map on the workload, scaled to a
    converged step by FP64_MAPS_PER_STEP."""
    world, rank, _ = dist_info()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    maps = args.ref_maps or FP64_MAPS_PER_STEP
    src = "--ref-maps" if args.ref_maps else FP64_MAPS_SOURCE
    if args.warmup > 0:
        oracle_full_map_ms(cfg, threads, reps=min(args.warmup, 1))
    t0 = time.perf_counter()
    per_map, samples = oracle_full_map_ms(cfg, threads, reps=args.steps)
    timed_s = time.perf_counter() - t0
    value = per_map * maps
    # the K timed maps are K / maps of one converged step: `steps` says so, so that
    # ms_per_step x steps is the timed region
    steps_timed = round(args.steps / maps, 4)
    line = {"metric": METRIC, "value": round(value, 1), "unit": UNIT, "impl": "reference",
            "n_gpus": world, "steps": steps_timed, "maps_timed": args.steps,
            "steps_note": (f"{args.steps} complete FP64 Picard maps timed = {steps_timed} of a "
                           f"converged step of {maps} maps"),
            "warmup": args.warmup,
            "ms_per_step": round(value, 1), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64",
            "data": "synthetic: seeded anisotropic Gaussian markers (numpy default_rng)",
            "config": {"workload": cfg["name"], "form": "reference CPU FP64 (oracle port)",
                       "N": cfg["N"], "use_logsq": cfg["use_logsq"]},
            "timed_unit": "one complete FP64 Picard map per timed sample",
            "timed_region_s": round(timed_s, 2),
            "per_map_ms": round(per_map, 1), "map_ms": [round(t, 1) for t in samples],
            "maps_per_step": maps, "maps_source": src, "extrapolated": True,
            "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": threads,
                             "kind": "port", "extrapolated": True,
                             "sample": (f"{args.steps} complete FP64 oracle Picard maps at "
                                        f"N={cfg['N']} (every pair evaluated), "
                                        f"{per_map:.0f} ms each, x {maps} maps per converged "
                                        f"FP64 step ({src})")},
            "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_profile_maps(args, cfg):
    """One Picard map per pair precision (FP32, double-single, FP64) on the
    workload's initial markers, for kernel captures (ncu -k regex:k_pair -c 3);
    prints the event-timed pair-kernel milliseconds of each map."""
    import torch

    import collops as co
    lib = co.load_library()
    N, dt = cfg["N"], cfg["dt"]
    bp = bp_of(cfg)
    p = co.SimParameters(bp1=bp, bp2=bp, m_anderson=cfg["m"], damping=cfg["damping"],
                         tol=cfg["tol"], abs_floor=cfg["abs_floor"], max_iter=cfg["max_iter"],
                         use_logsq=cfg["use_logsq"])
    ws = co.build_workspace(p)
    h = ws.h
    v_np, w_np = markers(cfg, cfg["seed"])
    v = np.asfortranarray(v_np)
    out = np.zeros_like(v, order="F")
    f = np.zeros(ws.n_dofs)
    co._check(lib.co_l2_project(h, co._p(v), co._p(w_np), co._p(f), N), "co_l2_project")
    Sb = np.zeros(1)
    co._check(lib.co_entropy(h, co._p(f), co._p(Sb)), "co_entropy")
    rec = {}
    for name, prec in (("fp32", 1), ("ds", 2), ("fp64", 0)):
        if name not in args.profile_maps_kinds.split(","):
            continue
        lib.co_profile(h, 1)
        o = p.opts(precision=prec)
        co._check(lib.co_picard_map(h, C.byref(o), co._p(out), co._p(v), co._p(v), co._p(w_np),
                                    N, float(Sb[0]), dt), "co_picard_map")
        pr = co.CoProfile()
        lib.co_profile_read(h, C.byref(pr))
        lib.co_profile(h, 0)
        rec[name] = {"fp32": pr.pair32_ms, "ds": pr.pairds_ms, "fp64": pr.pair64_ms}[name]
    torch.cuda.synchronize()
    print(json.dumps({"profile_maps": cfg["name"], "pair_ms": rec}), flush=True)
    ws.close()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--form", choices=["mixed_ds", "mixed", "fp64"], default="mixed_ds")
    ap.add_argument("--solver", choices=["defect", "anderson"], default="defect")
    ap.add_argument("--warmstart", choices=["learned", "euler"], default="learned")
    ap.add_argument("--warmstart-file", default=os.path.join(
        PKG, "collops", "warmstart_c3.npz"))
    ap.add_argument("--warm-relax", type=float, default=0.75,
                    help="under-relaxation of the learned proposal: v_pred + relax dt^2 delta")
    ap.add_argument("--no-retry", dest="retry", action="store_false",
                    help="do not repeat a non-converged solve from the next start")
    ap.add_argument("--logsq", type=int, choices=[0, 1], default=None,
                    help="override use_logsq of the workload")
    ap.add_argument("--dc-eta", type=float, default=0.02)
    ap.add_argument("--dc-max-inner", type=int, default=100)
    ap.add_argument("--dc-stag-window", type=int, default=5)
    ap.add_argument("--dc-fp32-stall", type=float, default=0.9,
                    help="the mixed forms leave FP32 outer maps once a map cuts the residual "
                         "by less than this factor")
    ap.add_argument("--dc-fp32-window", type=int, default=0,
                    help="leave FP32 outer maps after this many maps without a new best "
                         "residual (0: after the first map below the stall cut)")
    ap.add_argument("--dc-outer-m", type=int, default=0,
                    help="Anderson depth over the defect correction's outer iterates")
    ap.add_argument("--dc-cap-refresh", type=int, default=0, choices=[0, 1],
                    help="rebuild the FP32 metric after an inner solve that hit max_inner")
    ap.add_argument("--dc-cap-abort", type=int, default=2,
                    help="stagnation exit after this many FP64-stage outer maps in a row whose "
                         "inner solve hit max_inner without a new best (0: off)")
    ap.add_argument("--dc-precond", type=int, default=0, choices=[0, 1, 2],
                    help="block-Newton preconditioner of the inner iteration")
    ap.add_argument("--no-accuracy", dest="accuracy", action="store_false")
    ap.add_argument("--dc-metric-freeze", type=float, default=1e-3,
                    help="stop rebuilding the FP32 frozen metric once ||r|| < this x ||r_1||")
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=None,
                    help="steps of the e2e leg (default: all timed steps)")
    ap.add_argument("--mixed-floor", type=float, default=0.0)
    ap.add_argument("--c1-steps", type=int, default=3)
    ap.add_argument("--ref-maps", type=float, default=None,
                    help="reference arm: maps per converged FP64 step (default the measured "
                         "FP64_MAPS_PER_STEP)")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--N", type=int, default=None, help="override the marker count (tests)")
    ap.add_argument("--seed", type=int, default=None,
                    help="marker seed (default 42; other seeds give other trajectories of "
                         "the same workload, for solver-setting comparisons)")
    ap.add_argument("--profile-maps", action="store_true",
                    help="run one Picard map per pair precision and exit (kernel captures)")
    ap.add_argument("--profile-maps-kinds", default="fp32,ds,fp64")
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 0)
    if args.e2e_steps is None:
        args.e2e_steps = args.steps
    cfg = dict(WORKLOAD)
    if args.logsq is not None:
        cfg["use_logsq"] = bool(args.logsq)
    if args.N:
        cfg["N"] = args.N
        cfg["name"] = f"landau_n{args.N}_mesh64_dt0.02"
    if args.seed is not None:
        cfg["seed"] = args.seed
        cfg["name"] += f"_seed{args.seed}"
    if args.profile_maps:
        run_profile_maps(args, cfg)
    elif args.impl == "reference":
        run_reference(args, cfg)
    else:
        run_gpu(args, cfg)


if __name__ == "__main__":
    main()
