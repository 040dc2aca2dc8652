"""The committed golden fixtures (tests/golden, made by tests/golden/make_golden.py):
the oracle against them on the CPU, and the CUDA path against them on the GPU."""
import json
import os

import numpy as np
import pytest

from hymor_gb300 import case as C
from oracle import oracle as O
from tests.golden.make_golden import ORACLE_CASES
from tests.helpers import rel_err, residual_rel, state_rel

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RES_TOL = 1e-12     # residual, relative to the face-flux scale (as the parity tests)
STATE_TOL = 1e-11   # state after ten RK4 steps


def _case(stem):
    builder, kw, steps = ORACLE_CASES[stem]
    kw = dict(kw)
    nchi, neta = kw.pop("nchi"), kw.pop("neta")
    cs = C.initial_state(getattr(C, builder)(nchi, neta, **kw), seed=1, noise=1e-6)
    return cs, steps, np.load(os.path.join(GOLDEN, stem + ".npz"))


def test_spline_fixture():
    """The oracle's Reinsch smoothing spline against scipy's make_smoothing_spline values
    stored in spline.npz (the objective of the reference's BSplineKit fit)."""
    g = np.load(os.path.join(GOLDEN, "spline.npz"))
    for k, lam in enumerate(g["lam"]):
        val, der = O.spline(g["x"], g["y"], float(lam), g["t"])
        assert np.max(np.abs(val - g[f"val{k}"])) < 1e-9
        assert np.max(np.abs(der - g[f"der{k}"])) < 1e-7


def test_normal_shock_known_answer():
    """The stagnation-line state behind the initial shock is the CPG normal-shock state:
    rho2/rho1 = 5 and p2/p1 = 29 at M 5 (known_answers.json)."""
    ka = json.load(open(os.path.join(GOLDEN, "known_answers.json")))["normal_shock_M5"]
    cfg = C.cylinder_config(24, 24)
    cs = C.initial_state(cfg, noise=0.0)
    fs = C.freestream_cpg(cfg)
    rho, ru, rv, rE = cs.q[:, 1, 1]
    p = (rE - 0.5 * (ru**2 + rv**2) / rho) * (cfg.gamma - 1)
    assert abs(rho / fs["rho_0"] - ka["rho2_rho1"]) < 1e-12 * ka["rho2_rho1"]
    assert abs(p / fs["p_0"] - ka["p2_p1"]) < 1e-12 * ka["p2_p1"]


@pytest.mark.parametrize("stem", list(ORACLE_CASES))
def test_oracle_reproduces_fixtures(stem):
    cs, steps, g = _case(stem)
    o = O.Oracle(cs)
    assert max(residual_rel(o.residual(), g["flux"], cs)) < RES_TOL
    o2 = O.Oracle(cs)
    o2.advect(steps)
    st = o2.get_state()
    assert max(state_rel(st["q"], g["q"])) < STATE_TOL
    assert np.array_equal(st["cell_idx"], g["cell_idx"])
    assert rel_err(st["pts_x"], g["pts_x"]) < STATE_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("stem", list(ORACLE_CASES))
def test_cuda_path_reproduces_fixtures(require_gpu, stem):
    """PDE and ten ADVECT_FLOW steps through the C ABI against the stored vectors."""
    from hymor_gb300 import solver as S

    cs, steps, g = _case(stem)
    sol = S.Solution(cs)
    assert max(residual_rel(S.PDE(sol), g["flux"], cs)) < RES_TOL
    sol.close()
    sol = S.Solution(cs)
    S.ADVECT_FLOW(sol, steps)
    st = sol.get_state()
    assert max(state_rel(st["q"], g["q"])) < STATE_TOL
    assert np.array_equal(st["cell_idx"], g["cell_idx"])
    assert rel_err(st["pts_x"], g["pts_x"]) < STATE_TOL
    assert abs(st["t"] - float(g["t"])) < 1e-13 * max(1.0, abs(float(g["t"])))
    sol.close()


def _linear_case():
    g = np.load(os.path.join(GOLDEN, "oracle_linear_cylinder_24x20.npz"))
    cs = C.initial_state(C.cylinder_config(24, 20, perturb_shock=True), seed=1, noise=1e-6)
    return cs, int(g["steps"]), g


def test_oracle_reproduces_linear_fixture():
    """The oracle's shock-position blocks and upstream-boundary operator B against the
    stored ones (finite differences: 1e-9 of each block's scale)."""
    cs, steps, g = _linear_case()
    o = O.Oracle(cs)
    o.advect(steps)
    o.linearize()
    rows, a21f, a12, a22 = o.shock_blocks()
    brows, bq, bs = o.linearize_b()
    assert np.array_equal(rows, g["rows"]) and np.array_equal(brows, g["b_rows"])
    for got, key in ((O.compact_a21(rows, a21f), "a21"), (a12, "a12"), (a22, "a22"), (bq, "bq"), (bs, "bs")):
        assert rel_err(got, g[key]) < 1e-9, key


@pytest.mark.gpu
def test_cuda_path_reproduces_linear_fixture(require_gpu):
    """The device's shock-position blocks and B against the stored vectors (1e-5, the FD
    agreement of the device and the oracle)."""
    from hymor_gb300 import receptivity as R
    from hymor_gb300 import solver as S

    cs, steps, g = _linear_case()
    sol = S.Solution(cs)
    S.ADVECT_FLOW(sol, steps)
    _, L = S.LINEARIZE_L(sol)
    rows, a21, a12, a22 = L.shock_blocks()
    brows, bq, bs = R.LINEARIZE_B(sol)
    assert np.array_equal(rows, g["rows"]) and np.array_equal(brows, g["b_rows"])
    for got, key in ((a21, "a21"), (a12, "a12"), (a22, "a22"), (bq, "bq"), (bs, "bs")):
        assert rel_err(got, g[key]) < 1e-5, key
    sol.close()
