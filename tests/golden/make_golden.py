"""Generates the golden fixtures of tests/golden (run from the repository root):

    python tests/golden/make_golden.py

The reference (Julia) ships no golden vectors and cannot run here, so the fixtures are
of four kinds, each recorded with where it comes from:

- spline.npz: smoothing-spline values and slopes from scipy.interpolate's
  make_smoothing_spline, which minimises the objective of BSplineKit 0.19.2's
  fit(BSplineOrder(4), x, y, lambda) used by LEAST_SQUARES_SHOCK_POINTS.jl:52-58
  (the reference's spline library is not vendored);
- known_answers.json: the channel-flow leading eigenvalue printed in
  tutorials/channel_flow/README.md:164-168, and the CPG normal-shock ratios at M 5
  (Rankine-Hugoniot, as INITIAL_SOLUTION_POST_SHOCK.jl:64-92 uses them);
- oracle_*.npz: outputs of the C++ restatement (oracle/) for small seeded cases:
  the residual (PDE) and the state after ten RK4 steps (ADVECT_FLOW). These are
  regression vectors: they pin the oracle and the CUDA path to the outputs the
  oracle produced when the fixtures were made;
- oracle_linear_cylinder_24x20.npz: the oracle's finite-difference operators that
  the reference assembles beside the stencil Jacobian, on the 24 x 20 cylinder after
  five RK4 steps: the shock-position blocks of perturb_shock
  (LINEARIZE_EQUATIONS_NO_DISCONTINUITY.jl:140-274) and the upstream-boundary operator B
  (LINEARIZE_B.jl:40-296). Regression vectors as well.

Each part can be made on its own: python tests/golden/make_golden.py linear
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# small cases of the regression vectors: (file stem, case builder, RK4 steps)
ORACLE_CASES = {
    "oracle_cylinder_40x30": ("cylinder_config", dict(nchi=40, neta=30), 10),
    "oracle_channel_36x20": ("channel_config", dict(nchi=36, neta=20), 10),
    "oracle_blunt_cone_48x24": ("blunt_cone_config", dict(nchi=48, neta=24), 10),
}
SPLINE_LAMBDAS = (1e-3, 1e-6, 1e-9)


def spline_fixture():
    from scipy import interpolate

    rng = np.random.Generator(np.random.PCG64(7))
    x = np.sort(rng.uniform(0, 1, 60))
    y = np.sin(3 * x) + 0.01 * rng.standard_normal(60)
    t = np.concatenate([x, 0.5 * (x[1:] + x[:-1])])
    out = {"x": x, "y": y, "t": t, "lam": np.array(SPLINE_LAMBDAS)}
    for k, lam in enumerate(SPLINE_LAMBDAS):
        f = interpolate.make_smoothing_spline(x, y, lam=lam)
        out[f"val{k}"] = f(t)
        out[f"der{k}"] = f.derivative()(t)
    np.savez_compressed(os.path.join(HERE, "spline.npz"), **out)


def known_answers():
    g, M = 1.4, 5.0
    rho_ratio = (g + 1) * M**2 / ((g - 1) * M**2 + 2)
    p_ratio = 1 + 2 * g / (g + 1) * (M**2 - 1)
    data = {
        "channel_eigenvalue": {"re": 0.000247, "im": 0.248408,
                               "source": "tutorials/channel_flow/README.md:164-168",
                               "grid": [180, 60], "Re": 7500, "Mach": 0.05},
        "normal_shock_M5": {"gamma": g, "Mach": M, "rho2_rho1": rho_ratio, "p2_p1": p_ratio,
                            "source": "Rankine-Hugoniot, INITIAL_SOLUTION_POST_SHOCK.jl:64-92"},
    }
    assert abs(rho_ratio - 5.0) < 1e-12 and abs(p_ratio - 29.0) < 1e-12
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(data, f, indent=1)


def oracle_fixtures():
    from hymor_gb300 import case as C
    from oracle import oracle as O

    for stem, (builder, kw, steps) in ORACLE_CASES.items():
        kw = dict(kw)
        nchi, neta = kw.pop("nchi"), kw.pop("neta")
        cfg = getattr(C, builder)(nchi, neta, **kw)
        cs = C.initial_state(cfg, seed=1, noise=1e-6)
        o = O.Oracle(cs)
        flux = o.residual()
        o2 = O.Oracle(cs)
        o2.advect(steps)
        st = o2.get_state()
        np.savez_compressed(os.path.join(HERE, stem + ".npz"), flux=flux, q=st["q"], t=st["t"],
                            pts_x=st["pts_x"], pts_y=st["pts_y"], cell_idx=st["cell_idx"], steps=steps)


def linear_fixture():
    from hymor_gb300 import case as C
    from oracle import oracle as O

    cfg = C.cylinder_config(24, 20, perturb_shock=True)
    cs = C.initial_state(cfg, seed=1, noise=1e-6)
    o = O.Oracle(cs)
    o.advect(5)
    o.linearize()
    rows, a21f, a12, a22 = o.shock_blocks()
    brows, bq, bs = o.linearize_b()
    np.savez_compressed(os.path.join(HERE, "oracle_linear_cylinder_24x20.npz"), steps=5, rows=rows,
                        a21=O.compact_a21(rows, a21f), a12=a12, a22=a22, b_rows=brows, bq=bq, bs=bs)


if __name__ == "__main__":
    parts = sys.argv[1:] or ["spline", "known", "oracle", "linear"]
    if "spline" in parts:
        spline_fixture()
    if "known" in parts:
        known_answers()
    if "oracle" in parts:
        oracle_fixtures()
    if "linear" in parts:
        linear_fixture()
    print("fixtures written to", HERE)
