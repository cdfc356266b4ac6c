#!/usr/bin/env python3
"""Benchmark: ms per converged implicit step, Landau N = 131,072.

Workload (the precision-form configuration): Landau, N = 131,072 markers from an
anisotropic Gaussian (T_x = 1.0, T_y = 0.25, i.e. sigma = (1, 0.5)), uniform
weights 1/N, [-6,6]^2 with a 64x64 P_DEG=2 mesh, dt = 0.02, Gonzalez on,
Anderson depth 8, damping 0.7, tol 1e-12, abs_floor 0 (so tol*||v|| binds),
N_QUAD 6. Markers are seeded synthetic data (numpy default_rng(42)).

One "step" = one time step of the reference's loop (main.jl:226-300): the
warm start, the implicit solve to convergence (tol 1e-12 on ||G(v) - v||), and
the entropy S0 of the new state for the next step. `value` times the headline
form -- mixed precision (FP32 pair maps, then double-single pair maps for the
FP64-accurate stage), defect correction around a frozen metric, and the
learned warm start (kept only when its first residual is below the explicit
predictor's) -- with inputs resident in HBM. The timed steps walk the
workload's first three time steps from its initial markers, cycled (step k
starts from state k mod 3 of the headline's own trajectory); W warm-up steps
repeat step 0. `plain_fp64` times the plain FP64 form (Anderson on FP64 pair
maps from the explicit predictor, the reference's GPU configuration) on the
same steps; `accuracy` compares step 0 with the same solver run on FP64 pair
maps from the same guess; `e2e` runs the headline form from pinned host arrays
with the copies inside the timed region. Each timed step is bracketed by CUDA
events on the library's stream; a 256 MB buffer is written before each timed
step to flush L2.

--impl reference times the CPU FP64 oracle (the reference's CPU algorithm,
OpenMP over all host cores) on the same workload: one Picard map per step with
the pair sum evaluated on a seeded sample of target rows and scaled to all rows,
times the number of maps of a converged FP64 step.
"""
from __future__ import annotations

import argparse
import csv
import ctypes as C
import io
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
                sx=1.0, sy=0.5, dt=0.02, m=8, damping=0.7, tol=1e-12, abs_floor=0.0,
                max_iter=2000, seed=42)
# maps per converged FP64 step of this workload, measured by the plain FP64
# GPU solve (profiles/c3_fp64_step.md); used only when this run does not
# measure it itself
FP64_MAPS_FILE = os.path.join(ROOT, "profiles", "c3_fp64_step.md")


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


# ---------------------------------------------------------------- CPU side

def oracle_map_sample(cfg, v, w, rows_sample: int, threads: int):
    """One Picard map of the CPU oracle at the full workload with the pair sum on
    a seeded sample of target rows; returns (estimated ms per map, details)."""
    import oracle
    oracle.build()
    bp = bp_of(cfg)
    om = oracle.OracleMesh(bp, bp, 6)
    o = oracle.Opts(model="landau", nthreads=threads)
    dt = cfg["dt"]
    N = cfg["N"]
    # v_in: a perturbed state standing in for the predictor (same cost)
    v_in = np.asfortranarray(v + 1e-3 * np.sin(np.arange(2 * N)).reshape(N, 2, order="F"))
    t0 = time.perf_counter()
    S0 = om.entropy(om.l2_project(v, w))
    t_s0 = time.perf_counter() - t0
    t0 = time.perf_counter()
    f_in = om.l2_project(v_in, w)          # Gonzalez projection of v_in
    S1 = om.entropy(f_in)
    vm = np.asfortranarray(0.5 * (v + v_in))
    f = om.l2_project(vm, w)
    L = om.mass_solve(om.compute_r(f))
    G = om.compute_G(vm, L)
    t_on = time.perf_counter() - t0
    inside = np.all((vm > cfg["lo"]) & (vm < cfg["hi"]), axis=1)
    n_in = int(inside.sum())
    rng = np.random.default_rng(7)
    rows = np.sort(rng.choice(np.flatnonzero(inside), size=min(rows_sample, n_in), replace=False))
    t0 = time.perf_counter()
    om.collision_rows(vm, w, G, rows, nthreads=threads)
    t_pairs = time.perf_counter() - t0
    per_map = (t_on + t_pairs * n_in / len(rows)) * 1e3
    _ = (S0, S1, t_s0)
    return per_map, dict(t_on_ms=t_on * 1e3, t_pairs_sample_ms=t_pairs * 1e3, rows=len(rows),
                         n_in=n_in)


def fp64_maps_from_profile():
    try:
        for line in open(FP64_MAPS_FILE):
            if line.startswith("maps_per_step:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def cpu_baseline(cfg, maps_per_step, maps_src, rows_sample=32768):
    threads = os.cpu_count() or 1
    v, w = markers(cfg, cfg["seed"])
    per_map, d = oracle_map_sample(cfg, v, w, rows_sample, threads)
    value = per_map * maps_per_step
    sample = (f"one Picard map of the FP64 oracle at N={cfg['N']}: projection, quadrature, "
              f"mass solves and grad-L in full ({d['t_on_ms']:.0f} ms), pair sum on "
              f"{d['rows']} seeded target rows ({d['t_pairs_sample_ms']:.0f} ms) scaled to "
              f"{d['n_in']} rows; x {maps_per_step:.1f} maps per converged FP64 step "
              f"({maps_src})")
    return dict(value=round(value, 1), unit=UNIT, cores=threads, kind="port", sample=sample,
                per_map_ms=round(per_map, 1))


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
                         tol=cfg["tol"], abs_floor=cfg["abs_floor"], max_iter=cfg["max_iter"])
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
    v1 = torch.empty_like(v)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def opts(prec):
        return p.opts(precision=co._PREC[prec], mixed_floor=args.mixed_floor)

    def entropy(x):
        S = C.c_double()
        co._check(lib.co_entropy_of_markers_dev(h, x.data_ptr(), w.data_ptr(), N, C.byref(S)),
                  "co_entropy_of_markers_dev")
        return S.value

    dopt = co.CoDefectOpts(args.dc_eta, args.dc_max_inner, args.dc_stag_window, args.dc_fp32_stall, 0,
                           args.dc_outer_m, args.dc_precond, args.dc_metric_freeze,
                           args.dc_fp32_window)

    warm = None
    if args.warmstart == "learned":
        from collops import learned
        if not os.path.exists(args.warmstart_file):
            raise SystemExit(f"warm-start weights not found: {args.warmstart_file}")
        warm = learned.WarmStart.load(args.warmstart_file, device=local)
    ws_stats = {"used": 0, "steps": 0, "mlp_launches": 0, "retries": 0}

    def initial_guess(x, S0, prec, learned_start):
        """v1 <- the warm start of the step from x: the learned proposal (kept only
        when its first residual is below the predictor's) or the explicit predictor."""
        o = opts(prec)
        if warm is not None and learned_start:
            used, _rl, _rp = warm.propose(ws, o, x, w, S0, dt, v1)
            ws_stats["used"] += int(used)
            ws_stats["steps"] += 1
            ws_stats["mlp_launches"] += 1
        else:
            co._check(lib.co_predictor_dev(h, C.byref(o), v1.data_ptr(), x.data_ptr(),
                                           w.data_ptr(), N, dt), "co_predictor_dev")

    def solve(x, S0, prec, solver):
        """the implicit solve from the guess in v1 (in place); returns its info tuple"""
        o = opts(prec)
        it, nrs = C.c_int(), C.c_int()
        res, r0 = C.c_double(), C.c_double()
        if solver == "defect":
            o.stag_rel_tol = 0.1
            co._check(lib.co_step_defect_dev(h, C.byref(o), C.byref(dopt), v1.data_ptr(),
                                             x.data_ptr(), w.data_ptr(), N, S0, dt, C.byref(it),
                                             C.byref(res), C.byref(nrs), C.byref(r0)),
                      "co_step_defect_dev")
        else:
            co._check(lib.co_step_anderson_dev(h, C.byref(o), v1.data_ptr(), x.data_ptr(),
                                               w.data_ptr(), N, S0, dt, C.byref(it),
                                               C.byref(res), C.byref(nrs), C.byref(r0)),
                      "co_step_anderson_dev")
        return (it.value, res.value, nrs.value, r0.value)

    def one_step(x, S0, prec, solver=None, learned_start=True):
        """warm start + implicit solve + S of the new state; returns (x1, S1, info).
        The headline form (learned start, defect correction) retries a stagnated
        solve once from the other start candidate (collops.learned.step_defect_warm)."""
        solver = solver or args.solver
        headline = learned_start and solver == args.solver and prec == args.form
        if headline and warm is not None and solver == "defect":
            o = opts(prec)
            o.stag_rel_tol = 0.1
            info, rec = learned.step_defect_warm(ws, warm, o, dopt, x, w, S0, dt, v1)
            ws_stats["used"] += int(rec["used_learned"])
            ws_stats["steps"] += 1
            ws_stats["mlp_launches"] += 1
            ws_stats["retries"] += rec["attempts"] - 1
        else:
            initial_guess(x, S0, prec, headline)
            info = solve(x, S0, prec, solver)
        S1 = entropy(v1)
        return v1.clone(), S1, info

    def converged(info, x):
        return info[1] < cfg["tol"] * float(torch.linalg.vector_norm(x)) * 1.0000001

    def fp64_residual(x_new, x_old, S_old):
        """||G64(x) - x|| of a returned state (one FP64 Picard map, untimed)."""
        r = C.c_double()
        o = opts("fp64")
        co._check(lib.co_picard_residual_dev(h, C.byref(o), x_new.data_ptr(), x_old.data_ptr(),
                                             w.data_ptr(), N, S_old, dt, C.byref(r)),
                  "co_picard_residual_dev")
        return r.value

    # The timed steps walk the workload's first CYCLE time steps from its initial
    # markers (step k starts from state k mod CYCLE of the headline's own
    # trajectory): every solver of this library and the reference's plain FP64
    # Anderson converge there. Later steps of this workload stagnate for every
    # solver (the quadrature's f > 1e-30 guard makes the discrete map jump).
    CYCLE = 3
    S_ic = entropy(v)
    x_ic = v.clone()

    def run_steps(k, prec, solver=None, flush_l2=True, record=None):
        cur = (x_ic, S_ic)
        times, infos, flags = [], [], []
        for i in range(k):
            if flush_l2:
                with torch.cuda.stream(stream):
                    flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            x1, S1, info = one_step(cur[0], cur[1], prec, solver)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
            infos.append(info)
            flags.append(bool(converged(info, x1)))
            if record is not None:
                record.append((cur, x1))
            cur = (x1, S1) if (i + 1) % CYCLE else (x_ic, S_ic)
        return times, infos, flags

    # warm-up: W steps from the initial markers (the state is not advanced)
    for _ in range(args.warmup):
        one_step(x_ic, S_ic, args.form)
    torch.cuda.synchronize()

    # ---- timed headline form
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    lib.co_profile(h, 1)
    n_launch0 = ws.launch_count()
    mlp0 = ws_stats["mlp_launches"]
    times, infos, conv = run_steps(args.steps, args.form)
    n_launch = ws.launch_count() - n_launch0 + ws_stats["mlp_launches"] - mlp0
    prof = co.CoProfile()
    lib.co_profile_read(h, C.byref(prof))
    lib.co_profile(h, 0)
    clk = clocks.stop()
    elapsed = float(sum(times))
    if world > 1:
        dist.barrier()
    job_ms, max_elapsed = aggregate(elapsed, args.steps, world)

    # ---- the plain FP64 form (Anderson, FP64 pair maps, explicit predictor)
    plain = None
    if args.plain_steps > 0:
        lib.co_profile(h, 1)
        tp, ip, cp = run_steps(args.plain_steps, "fp64", solver="anderson")
        prof64 = co.CoProfile()
        lib.co_profile_read(h, C.byref(prof64))
        lib.co_profile(h, 0)
        plain = dict(ms_per_step=round(statistics.mean(tp), 1), steps=len(tp),
                     step_ms=[round(t, 1) for t in tp], converged=cp,
                     iterations=[i[0] for i in ip], residuals=[i[1] for i in ip],
                     pair64_ms_avg=(prof64.pair64_ms / max(1, prof64.pair64_launches)))

    # ---- accuracy of the headline step 0 against the same algorithm in FP64
    acc = None
    if args.accuracy:
        initial_guess(x_ic, S_ic, args.form, True)
        guess = v1.clone()
        info_h = solve(x_ic, S_ic, args.form, args.solver)
        xh = v1.clone()
        # the FP64 fixed point nearest the headline result: the same solver on
        # FP64 pair maps, started from the headline result
        v1.copy_(xh)
        info_p = solve(x_ic, S_ic, "fp64", args.solver)
        xp = v1.clone()
        # the same solver on FP64 pair maps from the headline's own guess (the
        # implicit step has several roots; this one may land on another)
        v1.copy_(guess)
        info_64 = solve(x_ic, S_ic, "fp64", args.solver)
        x64 = v1.clone()
        x0 = x_ic.cpu().numpy()
        ah, a64, ap = xh.cpu().numpy(), x64.cpu().numpy(), xp.cpu().numpy()
        wn = w.cpu().numpy()
        E0 = 0.5 * (wn * (x0 ** 2).sum(0)).sum()

        def drift(a):
            return (float(np.abs((wn * (a - x0)).sum(1)).max()),
                    float(abs(0.5 * (wn * (a ** 2).sum(0)).sum() - E0) / E0))
        acc = dict(
            reference="the FP64 fixed point reached by the same solver on FP64 pair maps "
                      "started from the headline result",
            headline=dict(iterations=info_h[0], residual=info_h[1], inner=info_h[2]),
            fp64_polish=dict(iterations=info_p[0], residual=info_p[1], inner=info_p[2]),
            vel_err_rel_vs_fp64=float(np.abs(ah - ap).max() / np.abs(ap).max()),
            fp64_same_guess=dict(iterations=info_64[0], residual=info_64[1], inner=info_64[2],
                                 root_diff_rel=float(np.abs(ah - a64).max() /
                                                     np.abs(a64).max())),
            fp64_map_residual_headline=fp64_residual(xh, x_ic, S_ic),
            fp64_map_residual_fp64=fp64_residual(x64, x_ic, S_ic),
            tol_times_norm=cfg["tol"] * float(torch.linalg.vector_norm(xh)),
            momentum_drift=drift(ah)[0], energy_drift_rel=drift(ah)[1],
            momentum_drift_fp64=drift(a64)[0], energy_drift_rel_fp64=drift(a64)[1])

    # ---- e2e: host arrays in pinned memory, copied in and out inside the timed
    # region, through the public API (WarmStart.propose + co_step_defect_dev)
    e2e = None
    if args.e2e_steps > 0:
        vh = torch.empty((2, N), dtype=torch.float64).pin_memory()
        wh = torch.from_numpy(w_np).pin_memory()
        vout = torch.empty((2, N), dtype=torch.float64).pin_memory()
        xd = torch.empty_like(x_ic)
        cur_h, S_h = x_ic.cpu(), S_ic
        ets = []
        for i in range(args.e2e_steps):
            vh.copy_(cur_h)
            with torch.cuda.stream(stream):
                flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            with torch.cuda.stream(stream):
                xd.copy_(vh, non_blocking=True)
                w.copy_(wh, non_blocking=True)
            x1, S1, _info = one_step(xd, S_h, args.form)
            with torch.cuda.stream(stream):
                vout.copy_(x1, non_blocking=True)
            e1.record(stream)
            torch.cuda.synchronize()
            ets.append(e0.elapsed_time(e1))
            if (i + 1) % CYCLE:
                cur_h, S_h = vout.clone(), S1
            else:
                cur_h, S_h = x_ic.cpu(), S_ic
        h2d = 8 * (2 * N + N)     # markers + weights
        d2h = 8 * (2 * N + 1)     # new markers + S of the new state
        e2e_job, _ = aggregate(float(sum(ets)), len(ets), world)
        e2e = dict(value=round(e2e_job, 2), unit=UNIT, h2d_bytes_per_step=h2d,
                   d2h_bytes_per_step=d2h, steps=len(ets),
                   path="pinned host arrays -> WarmStart.propose + co_step_defect_dev -> host")

    # ---- roofline of the dominant pair kernel
    def roof(ms, launches, pairs, peak, kind):
        if launches == 0:
            return None
        avg_ms = ms / launches
        flops = 23.0 * pairs / launches            # 23 algorithmic flops per ordered pair
        achieved = flops / (avg_ms * 1e-3) / 1e12
        pk = peak / 1e12
        return {"bound": kind,
                "bound_note": "SIMT pipe bound (FP32 FMA or FP64): an N-body pair sum, no "
                              "tensor-core contraction; inputs are L2-resident, so not HBM",
                "achieved": round(achieved, 3), "peak": round(pk, 3),
                "unit": "TFLOP/s", "frac": round(achieved / pk, 4), "traffic": None,
                "kernel": "k_pair32" if kind == "fp32" else "k_pair64<false>",
                "avg_launch_ms": round(avg_ms, 3), "launches": launches,
                "pairs_per_launch": pairs / launches,
                "peak_source": "measured in this run: FMA-chain kernel (co_measure_fma_peak), "
                               "2 flops per FMA; no FP32/FP64 SIMT figure in MEASURED_PEAKS.json"}

    r32 = roof(prof.pair32_ms, prof.pair32_launches, prof.pair32_pairs, peak32.value, "fp32")
    r64 = roof(prof.pair64_ms, prof.pair64_launches, prof.pair64_pairs, peak64.value, "fp64")
    rds = roof(prof.pairds_ms, prof.pairds_launches, prof.pairds_pairs, peak32.value, "fp32")
    if rds:
        rds["kernel"] = "k_pair_ds_sym"
        rds["fp64_equivalent_frac"] = round(rds["achieved"] / (peak64.value / 1e12), 3)
        rds["note"] = ("double-single (FP32 head+tail) arithmetic: 23 FP64-equivalent flops per "
                       "ordered pair, executed as ~210 FP32-pipe instructions per unordered pair "
                       "(ncu); frac is against the FP32 peak by the 23-flop count, "
                       "fp64_equivalent_frac against the measured FP64 peak, ncu_issue_active the "
                       "fraction of issue slots the kernel keeps busy")
    if r32:
        r32["kernel"] = "k_pair32_sym"
    if r64:
        r64["kernel"] = "k_pair64_sym"
    cands = [(prof.pair32_ms, r32), (prof.pair64_ms, r64), (prof.pairds_ms, rds)]
    dominant = max((c for c in cands if c[1]), key=lambda c: c[0], default=(0, None))[1]
    traffic = load_traffic()
    if dominant and traffic.get(dominant["kernel"]) is not None:
        dominant["traffic"] = traffic[dominant["kernel"]]
    for rr in (r32, r64, rds):
        if rr:
            for key in ("ncu_issue_active", "ncu_fma_pipe", "ncu_fp64_pipe"):
                val = load_profile_lines(key).get(rr["kernel"])
                if val is not None:
                    rr[key] = val

    maps_fp64 = None
    maps_src = None
    if plain:
        maps_fp64 = statistics.mean(plain["iterations"]) + 1
        maps_src = "measured by the plain FP64 GPU step in this run (iterations + predictor)"
    else:
        mf = fp64_maps_from_profile()
        if mf:
            maps_fp64, maps_src = mf, "from " + os.path.relpath(FP64_MAPS_FILE, ROOT)
    cpu = None
    if rank == 0 and world == 1 and args.cpu_baseline and maps_fp64:
        cpu = cpu_baseline(cfg, maps_fp64, maps_src, rows_sample=args.cpu_rows)

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
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "256 MB buffer written between timed steps"},
        "step_ms": [round(t, 1) for t in times], "converged": conv,
        "steps_converged": int(sum(conv)),
        "iterations": [i[0] for i in infos], "residuals": [i[1] for i in infos],
        "inner_or_restarts": [i[2] for i in infos],
        "timed_steps": f"time steps 0..{CYCLE - 1} of the workload from its initial markers, "
                       f"cycled (step k starts from state k mod {CYCLE})",
        "maps": {"fp32": prof.maps32, "fp64": prof.maps64, "double_single": prof.mapsds},
        "plain_fp64": plain, "accuracy": acc,
        "warmstart": ({"kind": "learned MLP (BF16, own kernels)", "file": os.path.relpath(
            args.warmstart_file, ROOT), "learned_start_used": ws_stats["used"],
            "steps": ws_stats["steps"], "retries_from_other_start": ws_stats["retries"],
            "rule": "learned proposal when its first residual is below the predictor's; a "
                    "stagnated solve is repeated once from the other start"}
            if warm is not None else {"kind": "explicit predictor"}),
        "roofline": dominant, "roofline_fp64": r64, "roofline_fp32": r32, "roofline_ds": rds,
        "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": int(n_launch),
    }
    if plain:
        line["speedup_vs_plain_fp64"] = round(plain["ms_per_step"] / job_ms, 2)
        line["speedup_step0_vs_plain_fp64_step0"] = round(plain["step_ms"][0] / times[0], 2)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


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
    world, rank, _ = dist_info()
    if rank != 0:
        return
    maps = fp64_maps_from_profile()
    src = "from " + os.path.relpath(FP64_MAPS_FILE, ROOT)
    if maps is None:
        print(json.dumps({"impl": "reference", "metric": METRIC,
                          "unavailable": "maps per converged FP64 step not yet measured"}))
        return
    vals = []
    info = None
    for k in range(args.warmup + args.steps):
        info = cpu_baseline(cfg, maps, src, rows_sample=args.cpu_rows)
        if k >= args.warmup:
            vals.append(info["value"])
    value = statistics.mean(vals)
    line = {"metric": METRIC, "value": round(value, 1), "unit": UNIT, "impl": "reference",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(value, 1), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64",
            "data": "synthetic: seeded anisotropic Gaussian markers (numpy default_rng)",
            "config": {"workload": cfg["name"], "form": "reference CPU FP64 (oracle port)",
                       "N": cfg["N"]},
            "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": info["cores"],
                             "kind": "port", "sample": info["sample"]},
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
                         tol=cfg["tol"], abs_floor=cfg["abs_floor"], max_iter=cfg["max_iter"])
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
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--form", choices=["mixed_ds", "mixed", "fp64"], default="mixed_ds")
    ap.add_argument("--solver", choices=["defect", "anderson"], default="defect")
    ap.add_argument("--warmstart", choices=["learned", "euler"], default="learned")
    ap.add_argument("--warmstart-file", default=os.path.join(
        PKG, "collops", "warmstart_c3.npz"))
    ap.add_argument("--dc-eta", type=float, default=0.02)
    ap.add_argument("--dc-max-inner", type=int, default=100)
    ap.add_argument("--dc-stag-window", type=int, default=5)
    ap.add_argument("--dc-fp32-stall", type=float, default=0.9,
                    help="the mixed forms leave FP32 outer maps once a map cuts the residual "
                         "by less than this factor")
    ap.add_argument("--dc-fp32-window", type=int, default=0,
                    help="leave FP32 outer maps after this many maps without a new best "
                         "residual (0: after the first map below the stall cut)")
    ap.add_argument("--dc-outer-m", type=int, default=5,
                    help="Anderson depth over the defect correction's outer iterates")
    ap.add_argument("--dc-precond", type=int, default=0, choices=[0, 1, 2],
                    help="block-Newton preconditioner of the inner iteration")
    ap.add_argument("--no-accuracy", dest="accuracy", action="store_false")
    ap.add_argument("--dc-metric-freeze", type=float, default=1e-3,
                    help="stop rebuilding the FP32 frozen metric once ||r|| < this x ||r_1||")
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--mixed-floor", type=float, default=0.0)
    ap.add_argument("--cpu-rows", type=int, default=32768)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--N", type=int, default=None, help="override the marker count (tests)")
    ap.add_argument("--profile-maps", action="store_true",
                    help="run one Picard map per pair precision and exit (kernel captures)")
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 0)
    cfg = dict(WORKLOAD)
    if args.N:
        cfg["N"] = args.N
        cfg["name"] = f"landau_n{args.N}_mesh64_dt0.02"
    if args.profile_maps:
        run_profile_maps(args, cfg)
    elif args.impl == "reference":
        run_reference(args, cfg)
    else:
        run_gpu(args, cfg)


if __name__ == "__main__":
    main()
