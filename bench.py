"""Benchmark: residual + RK4 throughput of the shock-fitted CPG cylinder at 800 x 400.

One step = one explicit RK4 step (ADVECT_FLOW_EXPLICIT: 4 residual stages, shock
fitting, CFL dt on the device) over the 800 x 400 cylinder = 1.28 M cell-stages.
Metric: Mcell-stage/s (cells x 4 stages x steps / time), FP64.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Device timing: CUDA events on the library's stream around each step; every step is
preceded (outside its timed window) by a 512 MiB write that evicts the 129 MB L2.
e2e: the same metric through the public API with host buffers: per step, one
hymor_advect call uploads the state from pinned host memory, advances it one step and
writes it back, timed on the host clock.
With --gpus N > 1 (torchrun) every rank advances its own replica of the case (the
path has no cross-GPU exchange); value = all ranks' cell-stages / max rank time.
--impl reference times the CPU restatement of the reference path (the oracle,
OpenMP over every host core) on the same workload.

The line also carries "matvec": the second benchmark of the 800 x 400 case, the
linearised-residual (stencil-block Jacobian) matvec applied to 64 seeded unit-norm
vectors, batched in one launch and as 64 one-vector launches, against the FP64 and the
HBM roofline, with the Jacobian assembly time and the oracle's matvec beside it.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NCHI, NETA = 800, 400
CELLS = NCHI * NETA
STAGES = 4
BYTES_PER_CELL_STAGE = 216   # algorithmic bytes of residual + RK4 stage (2-D CPG)
FLUSH_BYTES = 512 << 20
MATVEC_VECTORS = 64          # seeded unit-norm perturbation vectors of the matvec benchmark
MATVEC_FLOP = 288            # 144 FMA per cell-matvec (9 neighbour blocks of 4 x 4)
METRIC = "Mcell-RK4-stages/s"
UNIT = "Mcell-stage/s"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_numbers():
    """DRAM traffic and FP64 work of the flux kernel over one RK stage (its two tile-class
    launches) from the committed ncu summary (profiles/k_flux_cylinder_800x400.md)."""
    path = os.path.join(ROOT, "profiles", "k_flux_cylinder_800x400.md")
    out = {}
    try:
        for line in open(path):
            for key in ("traffic_bytes_per_stage", "fp64_flop_per_stage", "fp64_inst_per_stage"):
                if line.strip().startswith(key + ":"):
                    out[key] = float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def init_dist(world, backend):
    if world <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(dist, value: float) -> float:
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def make_case():
    from hymor_gb300 import case as C
    cfg = C.cylinder_config(NCHI, NETA)
    return cfg, C.initial_state(cfg)


def cpu_baseline_sample(cs, budget_s: float = 12.0):
    """Oracle (CPU restatement of the reference path, OpenMP) on a bounded sample of the
    same workload: whole RK4 steps of the 800 x 400 cylinder until ~budget_s."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.lib().orc_set_threads(threads)
    o = O.Oracle(cs)
    o.advect(1)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while True:
        o.advect(1)
        steps += 1
        el = time.perf_counter() - t0
        if el > budget_s or steps >= 200:
            break
    return {"value": CELLS * STAGES * steps / el / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} RK4 steps of the {NCHI}x{NETA} cylinder ({el:.1f} s)"}


def matvec_bytes(k: int) -> float:
    """Algorithmic bytes per cell-matvec with k vectors per launch: the 144 coefficients
    (1152 B) once per launch, x and y (64 B) per vector."""
    return (1152 + 64 * k) / k


def matvec_numbers(sol, cs, fp64_peak_tflops: float, hbm_gbs: float, cpu: bool, reps: int = 3):
    """The linearised-residual matvec of the 800 x 400 case on 64 seeded unit-norm vectors
    (numpy PCG64, seed 2): one batched launch against 64 one-vector launches (device time,
    CUDA events on the library stream; the 369 MB of Jacobian blocks and the 655 MB of
    vectors exceed L2, so no flush is needed), the device Jacobian assembly it needs
    (hymor_linearize: 37 residual evaluations and the scatter, host clock), and the
    oracle's single-vector matvec on the host."""
    import torch
    from hymor_gb300._lib import dp
    L, h = sol.ctx.L, sol.ctx.h
    t0 = time.perf_counter()
    sol.ctx.check(L.hymor_linearize(h))
    jac_s = time.perf_counter() - t0
    k, n = MATVEC_VECTORS, 4 * CELLS
    rng = np.random.Generator(np.random.PCG64(2))
    X = rng.standard_normal((k, n))
    X /= np.linalg.norm(X, axis=1, keepdims=True)
    dX = torch.from_numpy(X.reshape(-1)).cuda()
    dY = torch.empty_like(dX)
    torch.cuda.synchronize()
    xp, yp = ctypes.c_void_p(dX.data_ptr()), ctypes.c_void_p(dY.data_ptr())
    ms = ctypes.c_float()
    sol.ctx.check(L.hymor_bench_matvec(h, k, xp, yp, 0, 0, 1, ctypes.byref(ms)))  # warm-up
    sol.ctx.check(L.hymor_bench_matvec(h, k, xp, yp, 0, 0, reps, ctypes.byref(ms)))
    t_b = ms.value / 1e3 / reps
    sol.ctx.check(L.hymor_bench_matvec(h, k, xp, yp, 0, 1, reps, ctypes.byref(ms)))
    t_p = ms.value / 1e3 / reps
    sol.ctx.check(L.hymor_bench_matvec(h, k, xp, yp, 1, 0, reps, ctypes.byref(ms)))
    t_t = ms.value / 1e3 / reps
    cell_mv = CELLS * k

    def roof(t, kk):
        fl = cell_mv * MATVEC_FLOP / t / 1e12
        gbs = cell_mv * matvec_bytes(kk) / t / 1e9
        return {"bound": "fp64", "achieved_tflops": fl, "peak_tflops": fp64_peak_tflops,
                "frac": fl / fp64_peak_tflops, "hbm_algorithmic_gbs": gbs, "hbm_peak_gbs": hbm_gbs,
                "hbm_frac": gbs / hbm_gbs, "bytes_per_cell_matvec": matvec_bytes(kk),
                "flop_per_cell_matvec": MATVEC_FLOP}

    out = {"workload": f"linearised-residual matvec, {k} seeded unit-norm vectors x {n} ({NCHI}x{NETA})",
           "vectors": k, "batched_ms": t_b * 1e3, "plain_ms": t_p * 1e3, "transpose_batched_ms": t_t * 1e3,
           "batched_speedup": t_p / t_b,
           "per_vector_us": {"batched": t_b / k * 1e6, "plain": t_p / k * 1e6},
           "roofline": roof(t_b, k), "plain_roofline": roof(t_p, 1),
           "jacobian_assembly_s": jac_s, "gpu_launches": {"batched": reps, "plain": reps * k}}
    if cpu:
        from oracle import oracle as O
        coef = np.empty(CELLS * 144)
        sol.ctx.check(L.hymor_jacobian_get(h, dp(coef)))
        o = O.Oracle(cs)
        o.matvec(coef, X[0])  # warm-up
        t0, nv = time.perf_counter(), 0
        while nv < 3:
            o.matvec(coef, X[nv])
            nv += 1
        el = (time.perf_counter() - t0) / nv
        out["cpu_baseline"] = {"ms_per_vector": el * 1e3, "cores": 1, "kind": "port",
                               "sample": f"{nv} vectors through the oracle's stencil matvec"}
    del dX, dY
    out["propagator"] = propagator_numbers(fp64_peak_tflops)
    try:
        out["shock_unknowns"] = extended_numbers(cs)
    except Exception as e:  # reported, never fatal to the bench line
        out["shock_unknowns"] = {"error": str(e)}
    return out


def extended_numbers(cs, reps: int = 10):
    """The same 800 x 400 case linearised with the shock-position unknowns (perturb_shock):
    the device assembly (36 + 8 + Nchi residuals, host clock), the matvec on one vector of
    4N + Nchi unknowns forward and transposed (device time, CUDA events), and LINEARIZE_B
    (13 residuals, host clock)."""
    import dataclasses
    import torch
    from hymor_gb300 import solver as S
    case = dataclasses.replace(cs, cfg=dataclasses.replace(cs.cfg, perturb_shock=True))
    sol = S.Solution(case)
    try:
        S.ADVECT_FLOW(sol, 20)
        L, h = sol.ctx.L, sol.ctx.h
        sol.ctx.check(L.hymor_linearize(h))  # warm-up
        t0 = time.perf_counter()
        sol.ctx.check(L.hymor_linearize(h))
        asm = time.perf_counter() - t0
        n = sol.operator_size()
        x = torch.from_numpy(np.random.Generator(np.random.PCG64(2)).standard_normal(n)).cuda()
        y = torch.empty_like(x)
        torch.cuda.synchronize()
        xp, yp = ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr())
        ms = ctypes.c_float()
        res = {"workload": f"perturb_shock, {NCHI}x{NETA}: {n} unknowns", "assembly_s": asm}
        for tr, key in ((0, "matvec_ms"), (1, "transpose_matvec_ms")):
            sol.ctx.check(L.hymor_bench_matvec(h, 1, xp, yp, tr, 0, 1, ctypes.byref(ms)))
            sol.ctx.check(L.hymor_bench_matvec(h, 1, xp, yp, tr, 0, reps, ctypes.byref(ms)))
            res[key] = ms.value / reps
        sol.ctx.check(L.hymor_linearize_b(h))  # warm-up
        t0 = time.perf_counter()
        sol.ctx.check(L.hymor_linearize_b(h))
        res["linearize_b_ms"] = (time.perf_counter() - t0) * 1e3
        del x, y
        return res
    finally:
        sol.close()


def propagator_numbers(fp64_peak_tflops: float, nchi: int = 100, neta: int = 80, k: int = 64,
                       nsteps: int = 50, order: int = 5):
    """Batched against one-vector propagation on the small cylinder (100 x 80, where one
    matvec is ~2 us of FP64 work and the one-vector path is bound by latency): 50 Taylor
    steps of degree 5 (250 matvecs) of exp(L dt), the building block of the Krylov solves,
    for 64 seeded vectors (seed 3) in one call against 64 one-vector calls; host clock
    around a device synchronisation."""
    import torch
    from hymor_gb300 import case as C
    from hymor_gb300 import solver as S
    cfg = C.cylinder_config(nchi, neta)
    sol = S.Solution(C.initial_state(cfg))
    L, h = sol.ctx.L, sol.ctx.h
    sol.ctx.check(L.hymor_linearize(h))
    dt = ctypes.c_double()
    sol.ctx.check(L.hymor_cfl_timestep(h, ctypes.byref(dt)))
    n = 4 * nchi * neta
    rng = np.random.Generator(np.random.PCG64(3))
    X = rng.standard_normal((k, n))
    X /= np.linalg.norm(X, axis=1, keepdims=True)
    dX = torch.from_numpy(X.reshape(-1)).cuda()
    dY = torch.empty_like(dX)
    xp, yp = dX.data_ptr(), dY.data_ptr()

    def batched():
        sol.ctx.check(L.hymor_expm_apply_dev(h, k, dt.value, nsteps, order, ctypes.c_void_p(xp),
                                             ctypes.c_void_p(yp), 0))

    def plain():
        for v in range(k):
            sol.ctx.check(L.hymor_expm_apply_dev(h, 1, dt.value, nsteps, order, ctypes.c_void_p(xp + 8 * n * v),
                                                 ctypes.c_void_p(yp + 8 * n * v), 0))

    res = {}
    for name, fn in (("batched", batched), ("plain", plain)):
        fn()  # warm-up (scratch allocation)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        res[name] = time.perf_counter() - t0
    sol.close()
    flop = float(nsteps * order) * nchi * neta * MATVEC_FLOP * k
    return {"workload": f"exp(L dt): {nsteps} Taylor steps of degree {order}, {k} vectors x {n} ({nchi}x{neta})",
            "batched_s": res["batched"], "plain_s": res["plain"],
            "batched_speedup": res["plain"] / res["batched"],
            "per_vector_ms": {"batched": res["batched"] / k * 1e3, "plain": res["plain"] / k * 1e3},
            "fp64_frac": {"batched": flop / res["batched"] / 1e12 / fp64_peak_tflops,
                          "plain": flop / res["plain"] / 1e12 / fp64_peak_tflops},
            "gpu_launches": {"batched": 1, "plain": k}}


def solve_numbers(nchi: int = 100, neta: int = 80, n_modes: int = 4, T_ref: float = 0.5, tol: float = 1e-8,
                  block: int = 8, steps: int = 20, maxit: int = 200):
    """Solve level (--solve, minutes): the n_modes eigenvalues of largest magnitude of
    exp(L T_ref) on the cylinder (after `steps` RK4 steps of the synthetic start), by the
    block Krylov-Schur (`block` vectors per batched propagation) and by the one-vector
    Krylov-Schur, both to Ritz residual tol or maxit restarts, from start vectors on the
    flow cells (the masked operator's other directions only carry the trivial eigenvalue
    0); host clock around each solve. Reports the residuals reached: on a clustered
    spectrum neither solve may reach tol within maxit."""
    from hymor_gb300 import case as C
    from hymor_gb300 import solver as S
    cfg = C.cylinder_config(nchi, neta)
    sol = S.Solution(C.initial_state(cfg))
    S.ADVECT_FLOW(sol, steps)
    _, Lop = S.LINEARIZE_L(sol)
    lam_b, info_b = S.EIGENVALUES(Lop, sol, n_modes, T_ref=T_ref, tol=tol, block=block, flow_start=True,
                                  maxit=maxit, keep_unconverged=True)
    lam_p, info_p = S.EIGENVALUES(Lop, sol, n_modes, T_ref=T_ref, tol=tol, flow_start=True, maxit=maxit,
                                  keep_unconverged=True)
    scale = float(np.max(np.abs(lam_p)))
    agree = max(float(np.min(np.abs(lam_p - a))) for a in lam_b) / scale
    sol.close()
    rel = {k: [float(r) for r in i["resid"] / np.abs(i["mu"])] for k, i in (("batched", info_b), ("plain", info_p))}
    return {"workload": f"EIGENVALUES, {n_modes} modes of exp(L {T_ref}) ({info_p['timesteps']} Taylor steps of "
                        f"degree 5), cylinder {nchi}x{neta}, Ritz residual {tol:g}",
            "batched_s": info_b["seconds"], "plain_s": info_p["seconds"],
            "batched_speedup": info_p["seconds"] / info_b["seconds"], "block": block,
            "propagations": {"batched": info_b["nops"], "plain": info_p["nops"]},
            "s_per_vector_propagation": {"batched": info_b["seconds"] / info_b["nops"],
                                         "plain": info_p["seconds"] / info_p["nops"]},
            "resid_rel": rel, "converged": {k: bool(max(v) <= tol) for k, v in rel.items()},
            "eigenvalues_agree_rel": agree,
            "eigenvalues": [[float(np.real(a)), float(np.imag(a))] for a in lam_p]}


def run_reference(args, world, rank):
    """--impl reference: the reference's CPU path (restated, the oracle) on host cores."""
    if rank != 0:
        return 0
    cfg, cs = make_case()
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.lib().orc_set_threads(threads)
    o = O.Oracle(cs)
    for _ in range(min(args.warmup, 3)):
        o.advect(1)
    # a bounded sample: the requested steps, or as many as fit in ~60 s of host time
    t0, done = time.perf_counter(), 0
    while done < args.steps:
        o.advect(1)
        done += 1
        if time.perf_counter() - t0 > 60.0:
            break
    el = time.perf_counter() - t0
    v = CELLS * STAGES * done / el / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el / done * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"shock-fitted CPG cylinder {NCHI}x{NETA}, M5 Re1e4, residual + RK4 step",
                   "cells": CELLS, "stages_per_step": STAGES, "parallelism": "cpu"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{done} of the {args.steps} requested RK4 steps of the {NCHI}x{NETA} "
                                   f"cylinder ({el:.1f} s)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Julia (not installable here); its hot path restated in C++ "
                "(oracle/hymor_oracle.cpp) is timed instead",
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # 1000 timed steps (~0.6 s of device time) let the clock sampler see the timed region
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="hymor", choices=["hymor", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--no-matvec", action="store_true")
    ap.add_argument("--solve", action="store_true", help="add the solve-level timing (minutes)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    dist = init_dist(world, "nccl")
    import torch
    torch.cuda.set_device(local)
    from hymor_gb300 import solver as S
    from hymor_gb300._lib import dp, ip

    cfg, cs = make_case()
    sol = S.Solution(cs)
    L, h = sol.ctx.L, sol.ctx.h
    fp64_peak = ctypes.c_double()
    sol.ctx.check(L.hymor_fp64_peak(h, ctypes.byref(fp64_peak)))
    # warm-up (graph capture happens on the first step)
    ms = ctypes.c_float()
    sol.ctx.check(L.hymor_bench_steps(h, args.warmup, FLUSH_BYTES, ctypes.byref(ms)))
    # timed region: K steps, flux-kernel events on
    sol.ctx.check(L.hymor_profile_flux(h, 1, None, None))
    torch.cuda.synchronize()
    barrier(dist)
    with ClockSampler(local) as clk:
        sol.ctx.check(L.hymor_bench_steps(h, args.steps, FLUSH_BYTES, ctypes.byref(ms)))
    torch.cuda.synchronize()
    barrier(dist)
    flux_ms, flux_n = ctypes.c_float(), ctypes.c_int32()
    phases = (ctypes.c_float * 18)()
    sol.ctx.check(L.hymor_profile_phases(h, phases))
    sol.ctx.check(L.hymor_profile_flux(h, 0, ctypes.byref(flux_ms), ctypes.byref(flux_n)))
    step_kernels = sol.step_kernels()
    t_dev = max_over_ranks(dist, ms.value / 1e3)
    total_cell_stages = CELLS * STAGES * args.steps * world
    value = total_cell_stages / t_dev / 1e6

    # end-to-end through the public API with pinned host buffers
    G = (NCHI + 2) * (NETA + 2)
    q_host = torch.empty(4 * G, dtype=torch.float64, pin_memory=True)
    q_host.numpy()[:] = cs.q_flat()
    st = sol.get_state()
    pts = [np.ascontiguousarray(st[k]) for k in ("pts_x", "pts_y", "pts_chi", "pts_eta")]
    ci = np.ascontiguousarray(st["cell_idx"])
    qp = ctypes.cast(q_host.data_ptr(), ctypes.POINTER(ctypes.c_double))
    sol.set_state(q_host.numpy(), *pts, ci, st["t"])
    torch.cuda.synchronize()
    barrier(dist)
    # the host buffers' pointers, made once as a caller holding its state would
    t_state = ctypes.c_double(st["t"])
    adv_args = (qp, dp(pts[0]), dp(pts[1]), dp(pts[2]), dp(pts[3]), ip(ci), ctypes.byref(t_state))
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        # ADVECT_FLOW on the host-resident state: upload, one step, download (hymor_advect)
        sol.ctx.check(L.hymor_advect(h, 1, *adv_args))
    t_e2e = max_over_ranks(dist, time.perf_counter() - t0)
    e2e_value = CELLS * STAGES * args.e2e_steps * world / t_e2e / 1e6
    h2d = 4 * G * 8 + 4 * NCHI * 8 + NCHI * 4
    d2h = h2d

    if rank == 0:
        hbm, kind = peaks()
        flux_avg_s = flux_ms.value / 1e3 / max(flux_n.value, 1)
        achieved = BYTES_PER_CELL_STAGE * CELLS / flux_avg_s / 1e9
        prof = profile_numbers()
        # one "launch" of the roofline = the flux of one RK stage (its two tile-class
        # launches), timed by CUDA events on the library stream inside the step graph
        roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                    "frac": achieved / hbm, "traffic": prof.get("traffic_bytes_per_stage"),
                    "kernel": "k_flux (residual of one RK stage, both tile classes)", "peak_kind": kind,
                    "stage_flux_ms": flux_avg_s * 1e3, "stages_timed": flux_n.value}
        if "fp64_flop_per_stage" in prof:
            # the binding roof on GB300: FP64 FLOPs (DADD + DMUL + 2 DFMA, ncu) per stage
            fp = prof["fp64_flop_per_stage"] / flux_avg_s / 1e12
            roofline["fp64"] = {"achieved_tflops": fp, "peak_tflops": fp64_peak.value, "unit": "TFLOP/s",
                                "frac": fp / fp64_peak.value,
                                "peak_kind": "DFMA throughput kernel timed in this run (hymor_fp64_peak)"}
            if "fp64_inst_per_stage" in prof:
                # the pipe issues one FP64 instruction (DFMA, DADD or DMUL) per lane-slot:
                # instruction rate against the DFMA peak's instruction rate
                roofline["fp64"]["inst_frac"] = (prof["fp64_inst_per_stage"] / flux_avg_s) / (fp64_peak.value * 1e12 / 2)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"shock-fitted CPG cylinder {NCHI}x{NETA}, M5 Re1e4, residual + RK4 step",
                       "cells": CELLS, "stages_per_step": STAGES, "parallelism": f"replicas x{world}",
                       "l2": "512 MiB flush before every timed step"},
            "roofline": roofline,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": step_kernels * args.steps,
            # main-stream phases of one step (us, averaged over the timed steps)
            "step_phases_us": {"start": round(phases[0] * 1e3, 1),
                               "stages": [[round(phases[1 + 4 * k + q] * 1e3, 1) for q in range(4)]
                                          for k in range(4)],
                               "stage_fields": ["update", "flux_interior", "start_shock_bc_after_interior", "flux_shock_bc"],
                               "end": round(phases[17] * 1e3, 1)},
            "clocks": clk.summary(),
        }
        if not args.no_cpu_baseline and world == 1:
            line["cpu_baseline"] = cpu_baseline_sample(cs)
        elif world > 1:
            line["cpu_baseline"] = None
        if not args.no_matvec:
            line["matvec"] = matvec_numbers(sol, cs, fp64_peak.value, hbm,
                                            cpu=not args.no_cpu_baseline and world == 1)
        if args.solve:
            line["solve"] = solve_numbers()
        print(json.dumps(line), flush=True)
    sol.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
