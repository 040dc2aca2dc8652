"""Shock-position unknowns of the linearised operator (stability_analysis.perturb_shock,
LINEARIZE_EQUATIONS_NO_DISCONTINUITY.jl:140-274): the oracle's restatement against the
reference's own consistency measure (CHECK_LINEARIZATION_L.jl:33-130) on the CPU, and the
device blocks, operator, propagator and solvers against the oracle on the GPU."""
import numpy as np
import pytest

from hymor_gb300 import case as C
from oracle import oracle as O

from helpers import rel_err


def _oracle_case(nchi=30, neta=24, steps=5, **kw):
    cfg = C.cylinder_config(nchi, neta, perturb_shock=True, **kw)
    cs = C.initial_state(cfg)
    orc = O.Oracle(cs)
    orc.advect(steps)
    co = orc.linearize()
    return cfg, cs, orc, co


def _perturbed_residuals(cs, orc, dq, dr):
    """f and the shock speeds of the prepared state and of the state raised by dq (cells)
    with every shock point moved by dr along PERTURB_SHOCK's direction
    (CHECK_LINEARIZATION_L.jl:92-100), each on a fresh copy."""
    cfg = cs.cfg
    N = cfg.nchi * cfg.neta
    st = orc.get_state()
    q = st["q"].copy().reshape(4, -1)
    for v in range(4):
        blk = q[v].reshape(cfg.nchi + 2, cfg.neta + 2, order="F")
        blk[1:-1, 1:-1] += dq[v * N:(v + 1) * N].reshape(cfg.nchi, cfg.neta, order="F")
        q[v] = blk.ravel(order="F")
    ang = orc.derived()["beta"] - np.pi / 2 - np.arctan2(orc.cs.rho_v_0, orc.cs.rho_u_0)
    out = []
    for qq, px, py in ((st["q"], st["pts_x"], st["pts_y"]),
                       (q.ravel(), st["pts_x"] + np.cos(ang) * dr, st["pts_y"] + np.sin(ang) * dr)):
        o = O.Oracle(cs)
        o.set_state(qq, px, py, st["pts_chi"], st["pts_eta"], st["cell_idx"], st["t"])
        out.append((o.residual(), o.rel_vel()))
    return out


def test_a21_is_column_local():
    """The reference assembles A21 one perturbed cell per residual (spline_param != 1,
    :143-205), each a full column over the Nchi shock speeds. The speed of point idx reads
    only the cells of its own column (UPDATE_SHOCK_JUMP_PROPERTIES.jl:354-405), so every
    entry idx != i is an exact zero: raising the cell (i, sc_i - j) of every column in one
    residual, as the device assembly does, gives the same column entries."""
    cfg, cs, orc, co = _oracle_case()
    rows, a21f, a12, a22 = orc.shock_blocks()
    n = cfg.nchi
    F = a21f.reshape(4, 2, n, n)
    diag = F[:, :, np.arange(n), np.arange(n)].copy()
    F[:, :, np.arange(n), np.arange(n)] = 0
    assert np.max(np.abs(F)) == 0.0
    assert np.max(np.abs(diag)) > 0.1
    assert a12.shape == (4 * n, n) and a22.shape == (n, n)
    assert np.all(rows == orc.get_state()["cell_idx"])


@pytest.mark.parametrize("spline_param", [None, 1.0])
def test_shock_linearization_consistency(spline_param):
    """CHECK_LINEARIZATION_L with the shock unknowns: [A11 A12; A21 A22] [q; r] matches the
    change of the masked residual and of the shock speeds when the cells move by q and the
    shock points by r along their normals, with the smoothing spline (A21 one cell per
    residual) and without it (spline_param = 1: all columns at once, :207-258). Without A12
    the flux response misses the shock's share by orders of magnitude more."""
    cfg, cs, orc, co = _oracle_case(**({} if spline_param is None else {"spline_param": spline_param}))
    rows, a21f, a12, a22 = orc.shock_blocks()
    blocks = (rows, O.compact_a21(rows, a21f), a12, a22)
    n, N = cfg.nchi, cfg.nchi * cfg.neta
    st = orc.get_state()
    flow = np.tile((np.arange(1, cfg.neta + 1)[None, :] < st["cell_idx"][:, None]).ravel(order="F"), 4)
    rng = np.random.Generator(np.random.PCG64(11))
    dq = 1e-7 * rng.standard_normal(4 * N) * flow
    dr = 1e-7 * rng.standard_normal(n)
    (f0, r0), (f1, r1) = _perturbed_residuals(cs, orc, dq, dr)
    df, dsp = (f1 - f0) * flow, r1 - r0
    Ax = orc.matvec_ext(co, blocks, np.concatenate([dq, dr]))
    assert np.linalg.norm(Ax[:4 * N] - df) < 1e-4 * np.linalg.norm(df)
    assert np.linalg.norm(Ax[4 * N:] - dsp) < 1e-4 * np.linalg.norm(dsp)
    assert np.linalg.norm(orc.matvec(co, dq) - df) > 1e-2 * np.linalg.norm(df)


def test_shock_operator_adjoint_identity():
    cfg, cs, orc, co = _oracle_case(24, 20)
    rows, a21f, a12, a22 = orc.shock_blocks()
    blocks = (rows, O.compact_a21(rows, a21f), a12, a22)
    rng = np.random.Generator(np.random.PCG64(4))
    n = 4 * cfg.nchi * cfg.neta + cfg.nchi
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    lhs = np.dot(orc.matvec_ext(co, blocks, x), y)
    rhs = np.dot(x, orc.matvec_ext(co, blocks, y, transpose=True))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


# ---------------------------------------------------------------------------
# GPU, through the C ABI


def _gpu_case(nchi=30, neta=24, steps=5, cone=False):
    from hymor_gb300 import solver as S
    make = C.blunt_cone_config if cone else C.cylinder_config
    cfg = make(nchi, neta, perturb_shock=True)
    cs = C.initial_state(cfg)
    sol, orc = S.Solution(cs), O.Oracle(cs)
    S.ADVECT_FLOW(sol, steps)
    orc.advect(steps)
    _, L = S.LINEARIZE_L(sol)
    co = orc.linearize()
    rows, a21f, a12, a22 = orc.shock_blocks()
    return cfg, cs, sol, orc, L, co, (rows, O.compact_a21(rows, a21f), a12, a22)


@pytest.mark.gpu
@pytest.mark.parametrize("cone", [False, True])
def test_shock_blocks_parity(require_gpu, cone):
    """The device's shock blocks against the oracle's per-point restatement, on the
    cylinder and the axisymmetric sphere-cone (shocked rows varying between columns).
    Entries are finite differences with eps = 1e-8 of residuals that agree to ~1e-13, so
    they agree to the FD rounding, as the A11 blocks do."""
    cfg, cs, sol, orc, L, co, ob = _gpu_case(48, 24, cone=True) if cone else _gpu_case()
    assert L.n == 4 * cfg.nchi * cfg.neta + cfg.nchi
    rows, a21, a12, a22 = L.shock_blocks()
    assert np.array_equal(rows, ob[0])
    for g, o in zip((a21, a12, a22), ob[1:]):
        assert rel_err(g, o) < 1e-5
    assert rel_err(L.blocks(), co) < 1e-5


@pytest.mark.gpu
def test_shock_operator_parity(require_gpu):
    """With the oracle's blocks on the device: matvec and transpose to 1e-13, the adjoint
    identity to 1e-12, the Taylor propagator (forward and adjoint) to 1e-12."""
    cfg, cs, sol, orc, L, co, ob = _gpu_case()
    L.set_blocks(co)
    L.set_shock_blocks(ob)
    n = L.n
    rng = np.random.Generator(np.random.PCG64(2))
    X = rng.standard_normal((n, 5))
    Y, YT = L @ X, L.T @ X
    for j in range(5):
        assert rel_err(Y[:, j], orc.matvec_ext(co, ob, X[:, j])) < 1e-13
        assert rel_err(YT[:, j], orc.matvec_ext(co, ob, X[:, j], transpose=True)) < 1e-13
    lhs, rhs = np.dot(L @ X[:, 0], X[:, 1]), np.dot(X[:, 0], L.T @ X[:, 1])
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    dt = 0.2 * sol.cfg.CFL * 1e-2
    for tr in (False, True):
        P = L.T if tr else L
        Pg = P.expm(X[:, :3], dt, 12)
        for j in range(3):
            assert rel_err(Pg[:, j], orc.expm_ext(co, ob, dt, 12, X[:, j], transpose=tr)) < 1e-12
    L.set_shock_blocks(None)
    assert L.n == 4 * cfg.nchi * cfg.neta


@pytest.mark.gpu
def test_shock_check_linearization(require_gpu):
    """CHECK_LINEARIZATION_L on the device operator with the shock unknowns: the reference's
    error measure stays below its 1e-3 threshold."""
    from hymor_gb300 import solver as S
    cfg, cs, sol, orc, L, co, ob = _gpu_case()
    err = S.CHECK_LINEARIZATION_L(L, sol, seed=5, verbose=False)
    assert err < 1e-3


@pytest.mark.gpu
def test_shock_eigenvalues_vs_oracle(require_gpu):
    """EIGENVALUES on the extended operator (device Krylov-Schur) against ARPACK on the
    oracle's extended propagator, same blocks."""
    sla = pytest.importorskip("scipy.sparse.linalg")
    from hymor_gb300 import solver as S
    cfg, cs, sol, orc, L, co, ob = _gpu_case(30, 20, steps=20)
    L.set_blocks(co)
    L.set_shock_blocks(ob)
    lam, info = S.EIGENVALUES(L, sol, 4, T_ref=0.02, ncv=24, tol=1e-11)
    dt, nt = info["dt"], info["timesteps"]
    n = L.n
    op = sla.LinearOperator((n, n), dtype=np.float64,
                            matvec=lambda x: orc.expm_ext(co, ob, dt, nt, np.ascontiguousarray(x).ravel()))
    mu = sla.eigs(op, k=4, which="LM", tol=1e-13, ncv=24, return_eigenvectors=False)
    lam_o = np.log(mu.astype(complex)) / (dt * nt)
    for a in lam:
        assert np.min(np.abs(lam_o - a)) <= 1e-8 * np.max(np.abs(lam_o))


@pytest.mark.gpu
def test_shock_transient_growth_vs_oracle(require_gpu):
    """TRANSIENT_GROWTH_DOWNSTREAM with the shock unknowns (R identity and M^ = bt_area / 2
    on them, M zero there) against eigsh on the same operator built from the oracle."""
    sla = pytest.importorskip("scipy.sparse.linalg")
    from hymor_gb300 import solver as S
    cfg, cs, sol, orc, L, co, ob = _gpu_case(24, 24, steps=20)
    L.set_blocks(co)
    L.set_shock_blocks(ob)
    T = 0.01
    G, info = S.TRANSIENT_GROWTH_DOWNSTREAM(L, sol, 2, T, ncv=16, tol=1e-11)
    st = sol.get_state()
    C0, D = S.chu_blocks_from_state(cfg, cs.mesh["vol"], st["q"], st["cell_idx"])
    Ki = np.linalg.inv(np.linalg.cholesky(D))
    N, n = cfg.nchi * cfg.neta, L.n
    kt = 1 / np.sqrt(np.asarray(cs.mesh["bt_a"])[np.arange(cfg.nchi), st["cell_idx"] - 1] / 2)

    def blk(B, x, tail):
        X = x[:4 * N].reshape(4, N).T
        return np.concatenate([np.einsum("nij,nj->ni", B, X).T.ravel(), tail * x[4 * N:]])
    dt, nt = info["dt"], info["n_t"]

    def mv(y):
        x = blk(np.transpose(Ki, (0, 2, 1)), np.ascontiguousarray(y).ravel(), kt)
        z = orc.expm_ext(co, ob, dt, nt, x)
        z = blk(C0, z, 0.0)
        z = orc.expm_ext(co, ob, dt, nt, z, transpose=True)
        return blk(Ki, z, kt)
    op = sla.LinearOperator((n, n), matvec=mv, dtype=np.float64)
    Go = np.sort(sla.eigsh(op, k=2, which="LA", tol=1e-13, return_eigenvectors=False))[::-1]
    assert np.allclose(np.sort(G)[::-1], Go, rtol=1e-6, atol=0)
