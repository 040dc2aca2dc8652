"""Converged base flows of the large benchmark cases, marched on the GPU.

The reference obtains its base flow by RUN_SIMULATION's explicit time marching
(utils/Time_marching/RUN_SIMULATION.jl:77-80) and judges convergence by the step
residual of ADVECT_FLOW_EXPLICIT.m:92-110 (RESIDUAL: rms change of each conserved
variable over the flow cells per step, relative to its rms). This module marches a
case on the device until that residual falls below a tolerance and caches the state
under hymor_gb300/_cache/ (not committed: regenerate with
`python -m hymor_gb300.baseflow <case>`).

Large grids start from a coarser converged solution (grid sequencing): the coarse
state is interpolated linearly in physical space onto the fine cell centres, the shock
line in element space, and the fine grid is then marched to the tolerance. Only the
start differs; the converged state is a fixed point of the fine-grid march.
"""
from __future__ import annotations

import argparse
import os
import time

import numpy as np

from . import case as C
from . import mesh as meshmod
from . import solver as S

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(HERE, "_cache")

# The cylinder's domain reaches 0.75 R above the stagnation point and 2.2 R above the
# shoulder instead of the default 0.5 R and 1.5 R: marched to a steady state, the M 5 bow
# shock stands ~0.5 R off the stagnation point and ~1.4 R off the shoulder, and the
# reference re-meshes its domain to 1.3 times the shock distance before marching on
# (remesh_shock_distance, tutorials/hypersonic_cylinder/input_file.jl:110), which this hot
# path does not do during a march.
CYLINDER_DRS, CYLINDER_DRE = 0.75, 2.2
# The march extrapolates the two cells above the shocked cell with first order
# (shock.interpolate "1st", EXTRAPOLATE_CELLS_SHOCK.jl): during the start-up transient the
# second-order extrapolation drives those cells to negative pressure, where the reference's
# UPDATE_SOUND_SPEED (sqrt over every cell) stops with an error. The extrapolated cells
# enter the flow only through shocked rows that change and the CFL sound-speed maximum, so
# the steady state is the same fixed point for either order; the cases' configurations
# (config()) keep "2nd".
MARCH_KW = dict(shock_interp="1st")


def cylinder(nchi: int, neta: int, **kw):
    from .mesh import Mapping
    kw.setdefault("mapping", Mapping(dRs=CYLINDER_DRS, dRe=CYLINDER_DRE))
    return C.cylinder_config(nchi, neta, **kw)


# name -> (config factory (nchi, neta, **kw), grid, coarse levels marched first)
CASES = {
    "cylinder_800x400": (cylinder, (800, 400), [(200, 100), (400, 200)]),
    "cylinder_600x300": (cylinder, (600, 300), [(150, 75), (300, 150)]),
    "sphere_cone_1200x400": (C.blunt_cone_config, (1200, 400), [(240, 80), (600, 200)]),
}


def config(name: str, **kw):
    make, (nchi, neta), _ = CASES[name]
    return make(nchi, neta, **kw)


def _level_config(name: str, nchi: int, neta: int, **kw):
    return CASES[name][0](nchi, neta, **kw)


def path(name: str) -> str:
    return os.path.join(CACHE, f"{name}.npz")


def load(name: str) -> dict | None:
    """The cached converged state of `name` (q, shock points, cell_idx, t, residual,
    steps), or None."""
    p = path(name)
    if not os.path.exists(p):
        return None
    with np.load(p) as z:
        return {k: z[k] for k in z.files}


def prolongate(cs_coarse: C.Case, st: dict, cfg_fine: C.Config) -> C.Case:
    """The coarse state st (Solution.get_state() of cs_coarse's grid) on the fine grid of
    cfg_fine: conserved variables interpolated linearly in physical space (nearest value
    outside the coarse hull), the shock line interpolated in element space."""
    from scipy.interpolate import LinearNDInterpolator, NearestNDInterpolator
    fine = C.initial_state(cfg_fine, noise=0.0)
    mc, mf = cs_coarse.mesh, fine.mesh
    pts_c = np.column_stack([np.ravel(mc["x_ext"], order="F"), np.ravel(mc["y_ext"], order="F")])
    pts_f = np.column_stack([np.ravel(mf["x_ext"], order="F"), np.ravel(mf["y_ext"], order="F")])
    qc = np.asarray(st["q"]).reshape(4, -1)
    shape_f = (cfg_fine.nchi + 2, cfg_fine.neta + 2)
    q = np.empty((4,) + shape_f, order="F")
    lin = LinearNDInterpolator(pts_c, qc.T)
    vals = lin(pts_f)
    bad = ~np.isfinite(vals).all(axis=1)
    if bad.any():
        vals[bad] = NearestNDInterpolator(pts_c, qc.T)(pts_f[bad])
    for v in range(4):
        q[v] = vals[:, v].reshape(shape_f, order="F")
    mp = cfg_fine.mapping
    chi_c = np.asarray(st["pts_chi"])
    eta_c = np.asarray(st["pts_eta"])
    chi_f = np.asarray(mf["chi1"])
    eta_f = np.interp(chi_f, chi_c, eta_c)
    px, py = meshmod.physical_space(mp, chi_f, eta_f)
    if mp.boundary_type != "circle":
        chi_s, eta_s = meshmod.element_space(mp, px, py)
    else:
        chi_s, eta_s = chi_f.copy(), eta_f.copy()
    fine.q = q
    fine.pts_x = np.ascontiguousarray(px, dtype=np.float64)
    fine.pts_y = np.ascontiguousarray(py, dtype=np.float64)
    fine.pts_chi = np.ascontiguousarray(chi_s, dtype=np.float64)
    fine.pts_eta = np.ascontiguousarray(eta_s, dtype=np.float64)
    fine.cell_idx = np.ascontiguousarray(C.detect_cells(mf, px, py), dtype=np.int32)
    fine.t = float(st["t"])
    fine.a = C.thermo_sound_speed(cfg_fine, q)
    return fine


def march(name: str, tol: float = 1e-10, coarse_tol: float = 1e-7, max_seconds: float = 3600.0,
          check_every: int = 5000, log=print, level_seconds: float = 300.0) -> dict:
    """Marches `name` to RESIDUAL < tol through its coarse levels (each to coarse_tol or
    level_seconds), saves the state to the cache and returns the record."""
    t0 = time.perf_counter()
    levels = CASES[name][2]
    cs = None
    st = None
    hist = []
    for lev in list(levels) + [None]:
        final = lev is None
        cfg = config(name, **MARCH_KW) if final else _level_config(name, lev[0], lev[1], **MARCH_KW)
        cs_new = C.initial_state(cfg) if cs is None else prolongate(cs, st, cfg)
        sol = S.Solution(cs_new)
        left = max_seconds - (time.perf_counter() - t0)
        if not final:
            left = min(left, level_seconds)
        r = S.MARCH_TO_RESIDUAL(sol, tol if final else coarse_tol, check_every=check_every, max_seconds=left,
                                log=(lambda m, g=(cfg.nchi, cfg.neta): log(f"{name} {g[0]}x{g[1]}: {m}")))
        hist.append(dict(grid=[cfg.nchi, cfg.neta], steps=r["steps"], residual=float(np.max(r["residual"])),
                         seconds=r["seconds"]))
        st = sol.get_state()
        sol.close()
        cs = cs_new
        if final:
            break
    os.makedirs(CACHE, exist_ok=True)
    rec = dict(q=st["q"], pts_x=st["pts_x"], pts_y=st["pts_y"], pts_chi=st["pts_chi"], pts_eta=st["pts_eta"],
               cell_idx=st["cell_idx"], t=st["t"], residual=hist[-1]["residual"], tol=tol,
               converged=hist[-1]["residual"] < tol, levels=np.array([h["grid"] + [h["steps"]] for h in hist]),
               seconds=time.perf_counter() - t0)
    tmp = path(name) + ".tmp.npz"
    np.savez(tmp, **rec)
    os.replace(tmp, path(name))
    return rec


def case_of(rec: dict, name: str, **cfg_kw) -> C.Case:
    """A Case (host arrays) holding the cached state rec of `name`."""
    cfg = config(name, **cfg_kw)
    cs = C.initial_state(cfg, noise=0.0)
    G = (cfg.nchi + 2) * (cfg.neta + 2)
    q = np.asarray(rec["q"]).reshape(4, G)
    cs.q = np.stack([q[v].reshape(cfg.nchi + 2, cfg.neta + 2, order="F") for v in range(4)])
    cs.pts_x, cs.pts_y = np.array(rec["pts_x"]), np.array(rec["pts_y"])
    cs.pts_chi, cs.pts_eta = np.array(rec["pts_chi"]), np.array(rec["pts_eta"])
    cs.cell_idx = np.ascontiguousarray(rec["cell_idx"], dtype=np.int32)
    cs.t = float(rec["t"])
    cs.a = C.thermo_sound_speed(cfg, cs.q)
    return cs


def solution(name: str, **cfg_kw):
    """A Solution of `name` holding its cached converged state (None if not cached)."""
    rec = load(name)
    if rec is None:
        return None
    cfg = config(name, **cfg_kw)
    cs = C.initial_state(cfg, noise=0.0)
    sol = S.Solution(cs)
    sol.set_state(rec["q"], rec["pts_x"], rec["pts_y"], rec["pts_chi"], rec["pts_eta"], rec["cell_idx"],
                  float(rec["t"]))
    return sol


def main(argv=None):
    ap = argparse.ArgumentParser(description="march a benchmark case to a converged base flow (GPU)")
    ap.add_argument("case", choices=sorted(CASES))
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--coarse-tol", type=float, default=1e-7)
    ap.add_argument("--max-seconds", type=float, default=3600.0)
    ap.add_argument("--check-every", type=int, default=5000)
    ap.add_argument("--level-seconds", type=float, default=300.0)
    ap.add_argument("--copy-to", default=None, help="also copy the cached file to this directory")
    a = ap.parse_args(argv)
    rec = march(a.case, a.tol, a.coarse_tol, a.max_seconds, a.check_every, log=lambda m: print(m, flush=True),
                level_seconds=a.level_seconds)
    if a.copy_to:
        import shutil
        os.makedirs(a.copy_to, exist_ok=True)
        shutil.copy(path(a.case), a.copy_to)
    print(f"{a.case}: residual {rec['residual']:.3e} (tol {a.tol:g}), converged {bool(rec['converged'])}, "
          f"levels {rec['levels'].tolist()}, {rec['seconds']:.0f} s -> {path(a.case)}")


if __name__ == "__main__":
    main()
