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
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,clocks.mem,"
              "clocks.max.mem")

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
        sm, mx, reasons, mem, mem_max = [], None, set(), [], None
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            try:  # the memory clock, which latency-bound kernels follow too
                mem.append(float(parts[9]))
                mem_max = float(parts[10])
            except (ValueError, IndexError):
                pass
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}
        if mem:
            out["mem_mhz"] = statistics.median(mem)
            out["mem_max_mhz"] = mem_max
        return out


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
    from hymor_gb300 import baseflow as B
    base, rec = B.solution("cylinder_800x400"), B.load("cylinder_800x400")
    state = "synthetic start (no converged base flow cached)"
    if base is not None:
        # the Jacobian of the converged base flow (its own, taller domain); the matvec's
        # work per cell does not depend on the state
        sol, cs = base, B.case_of(rec, "cylinder_800x400")
        state = f"converged base flow, step residual {float(rec['residual']):.2e} at t = {float(rec['t']):.1f}"
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
           "state": state, "vectors": k, "batched_ms": t_b * 1e3, "plain_ms": t_p * 1e3, "transpose_batched_ms": t_t * 1e3,
           "batched_speedup": t_p / t_b,
           "per_vector_us": {"batched": t_b / k * 1e6, "plain": t_p / k * 1e6},
           "roofline": roof(t_b, k), "plain_roofline": roof(t_p, 1),
           "jacobian_assembly_s": jac_s, "gpu_launches": {"batched": reps, "plain": reps * k}}
    if cpu:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        O.lib().orc_set_threads(threads)
        coef = np.empty(CELLS * 144)
        sol.ctx.check(L.hymor_jacobian_get(h, dp(coef)))
        o = O.Oracle(cs)
        o.matvec(coef, X[0])  # warm-up
        t0, nv = time.perf_counter(), 0
        while nv < 3:
            o.matvec(coef, X[nv])
            nv += 1
        el = (time.perf_counter() - t0) / nv
        out["cpu_baseline"] = {"ms_per_vector": el * 1e3, "cores": threads, "kind": "port",
                               "sample": f"{nv} vectors through the oracle's stencil matvec (OpenMP)"}
    del dX, dY
    out["propagator_800x400"] = propagator_large(sol, fp64_peak_tflops)
    if base is not None:
        base.close()
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
    for arith in (1, 0):  # float-float (the default), then FP64
        sol.ctx.check(L.hymor_set_expm_arith(h, arith))
        for name, fn in (("batched", batched), ("plain", plain)):
            fn()  # warm-up (scratch allocation, the float-float copy of the blocks)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            res[(arith, name)] = time.perf_counter() - t0
    sol.close()
    flop = float(nsteps * order) * nchi * neta * MATVEC_FLOP * k
    return {"workload": f"exp(L dt): {nsteps} Taylor steps of degree {order}, {k} vectors x {n} ({nchi}x{neta})",
            "arithmetic": "float-float matvecs on the FP32 pipe (default); the fp64 object times the same in FP64",
            "batched_s": res[(1, "batched")], "plain_s": res[(1, "plain")],
            "batched_speedup": res[(1, "plain")] / res[(1, "batched")],
            "per_vector_ms": {"batched": res[(1, "batched")] / k * 1e3, "plain": res[(1, "plain")] / k * 1e3},
            "fp64_equivalent_tflops": {"batched": flop / res[(1, "batched")] / 1e12,
                                       "plain": flop / res[(1, "plain")] / 1e12},
            "fp64": {"batched_s": res[(0, "batched")], "plain_s": res[(0, "plain")],
                     "fp64_frac": {"batched": flop / res[(0, "batched")] / 1e12 / fp64_peak_tflops,
                                   "plain": flop / res[(0, "plain")] / 1e12 / fp64_peak_tflops}},
            "float_float_speedup": {"batched": res[(0, "batched")] / res[(1, "batched")],
                                    "plain": res[(0, "plain")] / res[(1, "plain")]},
            "gpu_launches": {"batched": 1, "plain": k}}


def propagator_large(sol, fp64_peak_tflops: float, k: int = 8, nsteps: int = 50, order: int = 4):
    """The propagation on the bench case's own Jacobian (800 x 400, 1.28 M unknowns): 50
    Taylor steps of degree 4 of one vector, and of 8 vectors in one call, in float-float
    (the default) and in FP64; CUDA-synchronised host clock."""
    import torch
    L, h = sol.ctx.L, sol.ctx.h
    dt = ctypes.c_double()
    sol.ctx.check(L.hymor_cfl_timestep(h, ctypes.byref(dt)))
    n = 4 * NCHI * NETA
    rng = np.random.Generator(np.random.PCG64(5))
    X = rng.standard_normal((k, n))
    dX = torch.from_numpy(X.reshape(-1)).cuda()
    dY = torch.empty_like(dX)
    out = {"workload": f"exp(L dt): {nsteps} Taylor steps of degree {order}, 1 and {k} vectors x {n} "
                       f"({NCHI}x{NETA})"}
    for arith, name in ((1, "float_float"), (0, "fp64")):
        sol.ctx.check(L.hymor_set_expm_arith(h, arith))
        row = {}
        for kk in (1, k):
            call = lambda: sol.ctx.check(L.hymor_expm_apply_dev(h, kk, dt.value, nsteps, order,
                                                               ctypes.c_void_p(dX.data_ptr()),
                                                               ctypes.c_void_p(dY.data_ptr()), 0))
            call()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            call()
            torch.cuda.synchronize()
            el = time.perf_counter() - t0
            flop = float(nsteps * order) * CELLS * MATVEC_FLOP * kk
            row[f"{kk}_vectors"] = {"s": el, "ms_per_matvec_vector": el / (nsteps * order * kk) * 1e3,
                                    "fp64_equivalent_tflops": flop / el / 1e12}
        out[name] = row
    sol.ctx.check(L.hymor_set_expm_arith(h, 1))
    out["float_float_speedup"] = {key: out["fp64"][key]["s"] / out["float_float"][key]["s"] for key in out["fp64"]}
    return out


def _base_solution(name: str):
    """The converged base flow of `name` (hymor_gb300/_cache, made by `python -m
    hymor_gb300.baseflow name`), or None."""
    from hymor_gb300 import baseflow as B
    return B.solution(name), B.load(name)


def solve_eigen(n_modes: int = 12, ncv: int = 60, substeps: int = 50, order: int = 4, tol: float = 1e-8,
                block: int = 6, maxit: int = 300, arms=("plain", "batched")):
    """Solve level, modal analysis (sphere-cone 1200 x 400, M 6, Re 2e4, on its converged
    base flow): the n_modes eigenvalues of largest modulus of exp(L dt_50), built from
    `substeps` Taylor steps of degree `order` of the CFL dt, Krylov basis ncv, Ritz residual
    tol, start vectors on the flow cells; the one-vector Krylov-Schur against the block
    Krylov-Schur (`block` vectors per batched propagation), both through hymor_eigs. Host
    clock around each solve."""
    from hymor_gb300 import solver as S
    sol, rec = _base_solution("sphere_cone_1200x400")
    if sol is None:
        return {"unavailable": "no converged sphere-cone base flow: run python -m hymor_gb300.baseflow "
                               "sphere_cone_1200x400"}
    _, Lop = S.LINEARIZE_L(sol)
    dt = S.CFL_TIMESTEP(sol)
    out = {"workload": f"EIGENVALUES: {n_modes} eigenvalues of exp(L {substeps} dt), {substeps} Taylor steps of "
                       f"degree {order}, Krylov {ncv}, sphere-cone 1200x400 M6 Re2e4, Ritz residual {tol:g}",
           "base_flow": {"residual": float(rec["residual"]), "t": float(rec["t"]),
                         "levels": rec["levels"].tolist()},
           "n": Lop.n, "dt": dt}
    res = {}
    for name, b in (("plain", 1), ("batched", block)):
        if name not in arms:
            continue
        lam, info = S.EIGENVALUES(Lop, sol, n_modes, T_ref=substeps * dt, ncv=ncv, tol=tol, order=order,
                                  block=b, flow_start=True, maxit=maxit, keep_unconverged=True)
        rel = info["resid"] / np.abs(info["mu"])
        res[name] = dict(seconds=info["seconds"], block=b, converged=info["converged"], restarts=info["restarts"],
                         vector_propagations=info["nops"], max_resid_rel=float(np.max(rel)),
                         s_per_vector_propagation=info["seconds"] / max(info["nops"], 1),
                         eigenvalues=[[float(np.real(a)), float(np.imag(a))] for a in lam])
    out.update(res)
    if len(res) == 2:
        la = np.array([complex(*e) for e in res["plain"]["eigenvalues"]])
        lb = np.array([complex(*e) for e in res["batched"]["eigenvalues"]])
        out["batched_speedup"] = res["plain"]["seconds"] / res["batched"]["seconds"]
        out["eigenvalues_agree_rel"] = float(max(np.min(np.abs(la - x)) for x in lb) / np.max(np.abs(la)))
    sol.close()
    return out


def solve_tg(Ts=(0.0625, 0.125, 0.25, 0.5), n_modes: int = 2, tol: float = 1e-8, maxit: int = 300):
    """Solve level, transient growth (cylinder 600 x 300, M 5, on its converged base flow):
    the optimal gains of the horizons Ts, solved together (hymor_tg_gain with every horizon:
    one batched forward and one batched adjoint propagation per round) against one horizon
    after another, gains matched to 1e-6. Host clock around each solve."""
    from hymor_gb300 import solver as S
    sol, rec = _base_solution("cylinder_600x300")
    if sol is None:
        return {"unavailable": "no converged 600x300 cylinder base flow: run python -m hymor_gb300.baseflow "
                               "cylinder_600x300"}
    _, Lop = S.LINEARIZE_L(sol)
    dt = S.CFL_TIMESTEP(sol)
    Gb, infos = S.TRANSIENT_GROWTH_HORIZONS(Lop, sol, n_modes, Ts, tol=tol, maxit=maxit, keep_unconverged=True)
    t_batched = infos[0]["seconds"]
    t_plain, Gp, conv_p = 0.0, [], []
    for T in Ts:
        g, info = S.TRANSIENT_GROWTH_DOWNSTREAM(Lop, sol, n_modes, T, tol=tol, maxit=maxit, keep_unconverged=True)
        t_plain += info["seconds"]
        Gp.append(g)
        conv_p.append(info["converged"])
    Gp = np.array(Gp)
    sol.close()
    return {"workload": f"TRANSIENT_GROWTH_DOWNSTREAM: {n_modes} gains for T in {list(Ts)}, cylinder 600x300 M5 "
                        f"Re1e4, Ritz residual {tol:g}",
            "base_flow": {"residual": float(rec["residual"]), "t": float(rec["t"]), "levels": rec["levels"].tolist()},
            "dt_cfl": dt, "taylor_steps": [inf["n_t"] for inf in infos],
            "batched": {"seconds": t_batched, "converged": [inf["converged"] for inf in infos],
                        "vector_applications": [inf["nops"] for inf in infos]},
            "plain": {"seconds": t_plain, "converged": conv_p},
            "batched_speedup": t_plain / t_batched,
            "gains": Gb.tolist(),
            "gains_agree_rel": float(np.max(np.abs(Gb - Gp) / np.abs(Gp)))}


def solve_receptivity(ncases: int = 16, nw: int = 24, T: float = 0.01, n_modes: int = 1, tol: float = 1e-8,
                      steps: int = 200, seed: int = 6, grid_lo=(80, 40), grid_hi=(240, 96)):
    """Batched receptivity over uneven grids (the fifth benchmark configuration, at reduced
    sizes): `ncases` shock-fitted CPG cases, blunt wedge (cylinder nose) and axisymmetric
    blunt cone alternately, grids drawn by seed between grid_lo and grid_hi, Mach uniform in
    4-6, Re log-uniform in 5e3-5e4, `steps` RK4 steps from the synthetic start (above Mach 6 the
    coarser of these grids reach negative pressure during the start-up transient, in the
    oracle as on the device), each with nw
    freestream wavenumbers k in logspace(-1, 1.5, nw) (convected at the freestream speed:
    w = k). The optimal freestream disturbances of every case: FREESTREAM_RECEPTIVITY_BATCH
    (all cases in lockstep, their propagations concurrent) against one FREESTREAM_RECEPTIVITY
    after another, gains matched."""
    from hymor_gb300 import baseflow as B
    from hymor_gb300 import case as C
    from hymor_gb300 import receptivity as R
    from hymor_gb300 import solver as S
    rng = np.random.Generator(np.random.PCG64(seed))
    w = np.logspace(-1, 1.5, nw)
    cases, meta = [], []
    t_setup = time.perf_counter()
    for i in range(ncases):
        nchi = int(rng.integers(grid_lo[0], grid_hi[0] + 1)) // 2 * 2
        neta = int(rng.integers(grid_lo[1], grid_hi[1] + 1))
        M, Re = float(rng.uniform(4, 6)), float(10 ** rng.uniform(np.log10(5e3), np.log10(5e4)))
        # the cylinders on the taller domain of the base-flow cases (the bow shock of a slow
        # case stands off further than the default domain reaches); first-order extrapolation
        # above the shock through the start-up transient, as the base-flow marches
        make = B.cylinder if i % 2 == 0 else C.blunt_cone_config
        sol = S.Solution(C.initial_state(make(nchi, neta, Mach=M, Re=Re, shock_interp="1st")))
        S.ADVECT_FLOW(sol, steps)
        _, L = S.LINEARIZE_L(sol)
        _, Lr = R.LINEARIZE_L_(L, sol, w)
        cases.append((Lr, sol))
        meta.append({"geometry": "blunt wedge" if i % 2 == 0 else "blunt cone", "grid": [nchi, neta],
                     "Mach": round(M, 3), "Re": round(Re, 1), "unknowns": Lr.n})
    t_setup = time.perf_counter() - t_setup
    batch = R.FREESTREAM_RECEPTIVITY_BATCH(cases, n_modes, T, tol=tol, keep_unconverged=True)
    t_batched = batch[0][1]["seconds"]
    t_plain, worst = 0.0, 0.0
    for (Lr, sol), (G, info), m in zip(cases, batch, meta):
        _, G1, _, info1 = R.FREESTREAM_RECEPTIVITY(Lr, sol, n_modes, T, tol=tol, keep_unconverged=True)
        t_plain += info1["seconds"]
        worst = max(worst, float(np.max(np.abs(G - G1) / np.abs(G1))))
        m.update(gain=float(G[0]), converged=info["converged"], taylor_steps=info["n_t"], applications=info["nops"])
    for _, sol in cases:
        sol.close()
    return {"workload": f"FREESTREAM_RECEPTIVITY of {ncases} uneven cases x {nw} wavenumbers, T = {T:g}, "
                        f"{n_modes} gain each, tol {tol:g}",
            "cases": meta, "setup_s": t_setup, "batched_s": t_batched, "plain_s": t_plain,
            "batched_speedup": t_plain / t_batched, "gains_agree_rel": worst,
            "note": f"synthetic states after {steps} RK4 steps (no converged base flows for these grids); "
                    "grids reduced from 200x100..1000x400 so that both arms finish in minutes"}


def solve_numbers(which: str):
    out = {}
    if which in ("all", "eigen"):
        out["eigen"] = solve_eigen()
    if which in ("all", "eigen4"):
        # the same operator over a ten times longer horizon (500 degree-4 steps), 4 eigenvalues:
        # exp(L 50 dt) puts the whole stable spectrum within ~1 % of |mu| = 1
        out["eigen_4_modes_500_steps"] = solve_eigen(n_modes=4, substeps=500, maxit=60)
    if which == "eigen12":
        # the sphere-cone solve's 12 eigenvalues and Krylov 60 over the ten times longer horizon, one-vector
        out["eigen_12_modes_500_steps"] = solve_eigen(n_modes=12, substeps=500, maxit=80, arms=("plain",))
    if which in ("all", "tg"):
        out["transient_growth"] = solve_tg()
    if which in ("all", "recept"):
        out["receptivity"] = solve_receptivity()
    return out


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
    ap.add_argument("--solve", nargs="?", const="all", default=None, choices=["all", "eigen", "eigen4", "eigen12", "tg", "recept"],
                    help="add the solve-level timing on the converged base flows (minutes)")
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
    # the flux configuration picked by the library's autotuner on this case (state restored after)
    choice = np.zeros(3, dtype=np.int32)
    tune_ms = (ctypes.c_float * 18)()
    sol.ctx.check(L.hymor_autotune(h, 20, ip(choice), tune_ms))
    tiles = {8: "31x8", 16: "31x16", 4: "31x4+31x8"}  # 4: interior tiles 31x4, shock/boundary 31x8
    autotune = {"flux_tile": tiles[int(choice[0])], "interior_spare_blocks_per_sm": int(choice[1]),
                "halo": "TMA" if choice[2] else "thread loads",
                "candidates_ms_per_step": {f"{'tma' if t else 'ld'}/{tiles[r]}/spare{sp}":
                                           round(tune_ms[9 * t + 3 * ri + sp], 4)
                                           for t in (0, 1) for ri, r in enumerate((8, 16, 4))
                                           for sp in (0, 1, 2)}}
    sol.ctx.check(L.hymor_bench_steps(h, 2, FLUSH_BYTES, ctypes.byref(ms)))
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
    # the same steps with the viscous terms in FP64 instead of float-float (a reported
    # comparison; the state marches on from where the timed steps left it)
    n64 = max(50, args.steps // 4)
    sol.set_step_viscous(0)
    sol.ctx.check(L.hymor_bench_steps(h, 3, FLUSH_BYTES, ctypes.byref(ms)))
    sol.ctx.check(L.hymor_bench_steps(h, n64, FLUSH_BYTES, ctypes.byref(ms)))
    value_fp64_viscous = CELLS * STAGES * n64 * world / max_over_ranks(dist, ms.value / 1e3) / 1e6
    sol.set_step_viscous(1)

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
            "viscous_arithmetic": "float-float (FP32 pairs, ~48-bit) for the viscous gradients, stresses and "
                                  "heat flux of the step; FP64 everywhere else",
            "value_fp64_viscous": value_fp64_viscous,
            "autotune": autotune,
        }
        if not args.no_cpu_baseline and world == 1:
            line["cpu_baseline"] = cpu_baseline_sample(cs)
        elif world > 1:
            line["cpu_baseline"] = None
        if not args.no_matvec:
            line["matvec"] = matvec_numbers(sol, cs, fp64_peak.value, hbm,
                                            cpu=not args.no_cpu_baseline and world == 1)
        if args.solve:
            line["solve"] = solve_numbers(args.solve)
        print(json.dumps(line), flush=True)
    sol.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
