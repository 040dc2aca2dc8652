"""CPU tests: the oracle against the known answers of the reference (its pins), and
the mesh / case set-up it shares with the GPU path."""
import json
import math
import os

import numpy as np
import pytest

from hymor_gb300 import case as C
from hymor_gb300 import mesh as M
from oracle import oracle as O


@pytest.mark.parametrize("make", [
    lambda: C.cylinder_config(40, 30),
    lambda: C.channel_config(24, 16),
    lambda: C.blunt_cone_config(48, 24, pde_dimension="2D"),
])
def test_mesh_closure(make):
    """CHECK_MESH.jl:40-60: face area * normal sums vanish on every 2-D cell."""
    cfg = make()
    msh = M.generate_mesh(cfg.mapping, cfg.nchi, cfg.neta, False, cfg.eta_stretch_ratio)
    assert M.check_mesh_closure(msh) < 1e-13


def test_element_space_roundtrip():
    """GO_TO_ELEMENT_SPACE inverts GO_TO_PHYSICAL_SPACE (circle and blunt cone)."""
    for mp in (M.Mapping(), C.blunt_cone_config(10, 10).mapping):
        chi = np.linspace(0.02, 0.98, 23)
        eta = np.linspace(0.05, 0.9, 23)
        x, y = M.physical_space(mp, chi, eta)
        c2, e2 = M.element_space(mp, x, y)
        assert np.max(np.abs(c2 - chi)) < 1e-12
        assert np.max(np.abs(e2 - eta)) < 1e-12
        # the oracle's own restatement agrees with the host mapping
        cs = C.config_struct(C.Config(mapping=mp))
        import ctypes
        ch = np.empty_like(x)
        et = np.empty_like(x)
        O.lib().orc_element_space(ctypes.byref(cs), len(x), O.dptr(x), O.dptr(y), O.dptr(ch), O.dptr(et))
        assert np.max(np.abs(ch - chi)) < 1e-12 and np.max(np.abs(et - eta)) < 1e-12


@pytest.mark.parametrize("lam", [1e-3, 1e-6, 1e-9])
def test_spline_matches_scipy(lam):
    """The smoothing spline minimises Σ (y_i - f(x_i))² + λ ∫ f''² — the objective of
    BSplineKit's fit(BSplineOrder(4), x, y, λ) and of scipy's make_smoothing_spline."""
    interp = pytest.importorskip("scipy.interpolate")
    rng = np.random.Generator(np.random.PCG64(7))
    x = np.sort(rng.uniform(0, 1, 60))
    y = np.sin(3 * x) + 0.01 * rng.standard_normal(60)
    ref = interp.make_smoothing_spline(x, y, lam=lam)
    t = np.concatenate([x, 0.5 * (x[1:] + x[:-1])])
    val, der = O.spline(x, y, lam, t)
    assert np.max(np.abs(val - ref(t))) < 1e-9
    assert np.max(np.abs(der - ref.derivative()(t))) < 1e-7


def test_spline_linear_extrapolation():
    x = np.linspace(0, 1, 20)
    y = x**3
    val, der = O.spline(x, y, 1e-6, np.array([-0.2, 1.3]))
    v0, d0 = O.spline(x, y, 1e-6, np.array([0.0, 1.0]))
    assert abs(val[0] - (v0[0] - 0.2 * d0[0])) < 1e-14
    assert abs(val[1] - (v0[1] + 0.3 * d0[1])) < 1e-14
    assert der[0] == d0[0] and der[1] == d0[1]


def test_uniform_freestream_is_fixed_point():
    """A uniform freestream on a closed curvilinear mesh has zero residual."""
    cfg = C.cylinder_config(24, 16, shock_enabled=False, bc_chi0="outflow_supersonic_1st",
                            bc_chi1="outflow_supersonic_1st", bc_eta0="outflow_supersonic_1st",
                            bc_eta1="outflow_supersonic_1st")
    cs = C.initial_state(cfg, noise=0.0)
    o = O.Oracle(cs)
    f = o.residual().reshape(4, -1)
    scale = np.array([1.0, 1.0, 1.0, cs.fs["rho_E_0"]]) / cs.mesh["vol"].min()
    assert np.max(np.abs(f) / scale[:, None]) < 1e-12


def test_normal_shock_is_stationary():
    """CPG Rankine-Hugoniot (UPDATE_SHOCK_JUMP_PROPERTIES.jl:453-471): behind a normal
    shock at M 5 the state is rho2/rho1 = 5, p2/p1 = 29 and the shock speed is zero."""
    cfg = C.cylinder_config(24, 20)
    cs = C.initial_state(cfg, noise=0.0)
    g, Mn = cfg.gamma, cfg.Mach
    rho2 = (g + 1) * Mn**2 / ((g - 1) * Mn**2 + 2)
    p2 = (2 * g * Mn**2 - (g - 1)) / (g + 1)
    assert abs(rho2 - 5.0) < 1e-14 and abs(p2 - 29.0) < 1e-13
    col = cs.q[:, 1, 1:cs.cell_idx[0]]
    p = (col[3] - (col[1] ** 2 + col[2] ** 2) / col[0] / 2) * (g - 1)
    assert np.allclose(col[0], 5.0, rtol=1e-14)
    assert np.allclose(p / cs.fs["p_0"], 29.0, rtol=1e-13)
    o = O.Oracle(cs)
    o.residual()
    d = o.derived()
    assert abs(d["beta"][0] - math.pi / 2) == 0
    assert abs(d["speed_x"][0]) < 1e-12


@pytest.mark.slow
def test_channel_eigenvalue_pin():
    """tutorials/channel_flow/README.md:164-168: the leading eigenvalue of the FD Jacobian
    of plane Poiseuille flow (180 x 60, Re 7500, M 0.05) is 0.000247 + 0.248408i. The FD
    Jacobian's rounding noise at M 0.05 moves this eigenvalue by ~1e-5 (compare eps =
    3e-9 .. 1e-7), so the pin holds to 5e-6."""
    sla = pytest.importorskip("scipy.sparse.linalg")
    cfg = C.channel_config()
    cs = C.initial_state(cfg, noise=0.0)
    o = O.Oracle(cs)
    L = O.stencil_to_csr(cfg, o.linearize())
    lam = sla.eigs(L.astype(complex), k=1, sigma=0.25j, return_eigenvectors=False)[0]
    ka = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))
    pin = ka["channel_eigenvalue"]
    assert abs(lam.real - pin["re"]) < 5e-6
    assert abs(lam.imag - pin["im"]) < 5e-6


def test_linearization_consistency():
    """CHECK_LINEARIZATION_L.jl:33-130: A q matches f(x + q) - f(x) for a small random q."""
    cfg = C.cylinder_config(30, 24)
    cs = C.initial_state(cfg)
    o = O.Oracle(cs)
    o.advect(5)
    st = o.get_state()
    coef = o.linearize()
    st = o.get_state()
    base = O.Oracle(cs)
    base.set_state(st["q"], st["pts_x"], st["pts_y"], st["pts_chi"], st["pts_eta"], st["cell_idx"], st["t"])
    f0 = base.residual()
    rng = np.random.Generator(np.random.PCG64(11))
    N = cfg.nchi * cfg.neta
    G = (cfg.nchi + 2) * (cfg.neta + 2)
    dq = 1e-7 * rng.standard_normal(4 * N)
    flow = (np.arange(1, cfg.neta + 1)[None, :] < st["cell_idx"][:, None]).ravel(order="F")
    dq *= np.tile(flow, 4)
    q = st["q"].copy().reshape(4, cfg.nchi + 2, cfg.neta + 2, order="C")
    q = st["q"].copy().reshape(4, -1)
    for v in range(4):
        blk = q[v].reshape(cfg.nchi + 2, cfg.neta + 2, order="F")
        blk[1:-1, 1:-1] += dq[v * N:(v + 1) * N].reshape(cfg.nchi, cfg.neta, order="F")
        q[v] = blk.ravel(order="F")
    pert = O.Oracle(cs)
    pert.set_state(q.ravel(), st["pts_x"], st["pts_y"], st["pts_chi"], st["pts_eta"], st["cell_idx"], st["t"])
    f1 = pert.residual()
    Aq = o.matvec(coef, dq)
    df = f1 - f0
    assert np.linalg.norm(Aq - df) / np.linalg.norm(df) < 1e-3


def test_dot_product_identity():
    """<L x, y> = <x, Lᵀ y> for the stencil-block matvec and its transpose."""
    cfg = C.channel_config(12, 9)
    cs = C.initial_state(cfg)
    o = O.Oracle(cs)
    coef = o.linearize()
    rng = np.random.Generator(np.random.PCG64(4))
    x = rng.standard_normal(4 * cfg.nchi * cfg.neta)
    y = rng.standard_normal(4 * cfg.nchi * cfg.neta)
    lhs = np.dot(o.matvec(coef, x), y)
    rhs = np.dot(x, o.matvec(coef, y, transpose=True))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)
    # and against the scattered CSR matrix
    L = O.stencil_to_csr(cfg, coef)
    assert np.max(np.abs(L @ x - o.matvec(coef, x))) < 1e-10 * np.max(np.abs(L @ x))


def test_shock_leaving_the_mesh_raises():
    """A shocked row outside 2..Neta-1 is a BoundsError in the reference's shock chain;
    the oracle raises it instead of indexing past its arrays. Heavy smoothing (p = 0.9)
    straightens the bow shock until its ends leave the 100 x 80 cylinder mesh."""
    cfg = C.cylinder_config(100, 80, spline_param=0.9)
    orc = O.Oracle(C.initial_state(cfg))
    with pytest.raises(RuntimeError, match="outside 2..79"):
        orc.advect(10)
