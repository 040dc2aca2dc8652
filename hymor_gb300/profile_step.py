"""A short, deterministic run of the RK step for profilers (ncu).

    python -m hymor_gb300.profile_step [--nchi 800 --neta 400] [--steps 3] [--warmup 2]
        [--viscous ff|fp64] [--tiling ROWS,SPARE,TMA] [--linearize]
        [--expm K [--expm-steps 50 --expm-order 5 --expm-arith ff|fp64]]

Builds the shock-fitted cylinder of the given size (the benchmark case at 800 x 400),
marches `warmup` steps, then `steps` more; with --linearize it also assembles the Jacobian
once; with --expm K it linearises and propagates K seeded vectors once through the Taylor
propagator (one cooperative launch, k_expm_coop_ff or k_expm_coop). Launches per step: hymor_step_kernels (46 for the cylinder). A capture of the flux
kernel skips the warm-up's launches, e.g. `ncu -k regex:k_flux -s 16 -c 2 ...` (two flux
launches per RK stage, four stages per step).
"""
from __future__ import annotations

import argparse
import time

from . import case as C
from . import solver as S


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--nchi", type=int, default=800)
    ap.add_argument("--neta", type=int, default=400)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--viscous", choices=["ff", "fp64"], default="ff")
    ap.add_argument("--tiling", default=None, help="rows,spare,tma (rows 4: the split tiling; default: the library's)")
    ap.add_argument("--linearize", action="store_true")
    ap.add_argument("--expm", type=int, default=0, help="vectors to propagate after linearising")
    ap.add_argument("--expm-steps", type=int, default=50)
    ap.add_argument("--expm-order", type=int, default=5)
    ap.add_argument("--expm-arith", choices=["ff", "fp64"], default="ff")
    a = ap.parse_args(argv)
    sol = S.Solution(C.initial_state(C.cylinder_config(a.nchi, a.neta)))
    sol.set_step_viscous(1 if a.viscous == "ff" else 0)
    if a.tiling:
        rows, spare, tma = (int(x) for x in a.tiling.split(","))
        sol.ctx.check(sol.ctx.L.hymor_set_flux_tiling(sol.ctx.h, rows, spare, tma))
    S.ADVECT_FLOW(sol, a.warmup)
    sol.ctx.check(sol.ctx.L.hymor_synchronize(sol.ctx.h))
    t0 = time.perf_counter()
    S.ADVECT_FLOW(sol, a.steps)
    sol.ctx.check(sol.ctx.L.hymor_synchronize(sol.ctx.h))
    el = time.perf_counter() - t0
    if a.linearize or a.expm:
        _, L = S.LINEARIZE_L(sol)
    if a.expm:
        import numpy as np
        sol.set_expm_arith(1 if a.expm_arith == "ff" else 0)
        X = np.random.Generator(np.random.PCG64(3)).standard_normal((L.n, a.expm))
        dt = S.CFL_TIMESTEP(sol)
        t1 = time.perf_counter()
        Y = L.expm(X, dt, a.expm_steps, order=a.expm_order)
        print(f"expm: {a.expm} vectors, {a.expm_steps} steps of degree {a.expm_order} ({a.expm_arith}) in "
              f"{(time.perf_counter() - t1) * 1e3:.2f} ms, |Y| = {np.linalg.norm(Y):.6e}")
    print(f"{a.nchi}x{a.neta}: {a.steps} steps in {el * 1e3:.2f} ms, {sol.step_kernels()} launches per step")
    sol.close()


if __name__ == "__main__":
    main()
