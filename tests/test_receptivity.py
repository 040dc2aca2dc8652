"""Freestream receptivity (utils/Stability_analysis/Freestream_receptivity): the oracle's
LINEARIZE_B against the reference's own consistency measure (CHECK_LINEARIZATION_B.jl) on
the CPU; on the GPU the device B against the oracle's, the extended operator L_ and its
propagation against a sparse restatement built from the same blocks, and
FREESTREAM_RECEPTIVITY's gains against eigsh on that restatement."""
import numpy as np
import pytest

from hymor_gb300 import case as C
from oracle import oracle as O

from helpers import rel_err


def _oracle_case(nchi=30, neta=24, steps=5):
    cfg = C.cylinder_config(nchi, neta)
    cs = C.initial_state(cfg)
    orc = O.Oracle(cs)
    orc.advect(steps)
    co = orc.linearize()
    return cfg, cs, orc, co


def b_apply(cfg, rows, bq, P):
    """B P on the flux rows (m, sc_m - 1): P (4, Nchi) per-column upstream perturbation."""
    nchi, N = cfg.nchi, cfg.nchi * cfg.neta
    y = np.zeros(4 * N)
    for m in range(nchi):
        cell = m + (rows[m] - 2) * nchi
        for d in (-1, 0, 1):
            n = m + d
            if 0 <= n < nchi:
                y[np.arange(4) * N + cell] += bq[m, d + 1] @ P[:, n]
    return y


def test_linearize_b_consistency():
    """CHECK_LINEARIZATION_B: B q matches the change of the masked residual when the
    per-column upstream state moves by q (every column at once, 1e-7 * randn)."""
    cfg, cs, orc, co = _oracle_case()
    rows, bq, bs = orc.linearize_b()
    st = orc.get_state()
    fs = np.array([orc.cs.rho_0, orc.cs.rho_u_0, orc.cs.rho_v_0, orc.cs.rho_E_0])
    base_cols = np.repeat(fs[:, None], cfg.nchi, axis=1)
    P = 1e-7 * np.random.Generator(np.random.PCG64(12)).standard_normal((4, cfg.nchi))
    f = []
    for cols in (base_cols, base_cols + P):
        o = O.Oracle(cs)
        o.set_state(st["q"], st["pts_x"], st["pts_y"], st["pts_chi"], st["pts_eta"], st["cell_idx"], st["t"])
        o.set_upstream(cols)
        f.append(o.residual())
    flow = np.tile((np.arange(1, cfg.neta + 1)[None, :] < st["cell_idx"][:, None]).ravel(order="F"), 4)
    df = (f[1] - f[0]) * flow
    Bq = b_apply(cfg, rows, bq, P)
    assert np.linalg.norm(df) > 0
    assert np.linalg.norm(Bq - df) < 1e-4 * np.linalg.norm(df)
    # B couples each column to its neighbours only, and the uniform state is a no-op
    assert np.all(bq[0, 0] == 0) and np.all(bq[-1, 2] == 0)


# ---------------------------------------------------------------------------
# GPU, through the C ABI


def _gpu_case(nchi=24, neta=20, steps=20, cone=False):
    from hymor_gb300 import solver as S
    cfg = (C.blunt_cone_config if cone else C.cylinder_config)(nchi, neta)
    cs = C.initial_state(cfg)
    sol, orc = S.Solution(cs), O.Oracle(cs)
    S.ADVECT_FLOW(sol, steps)
    orc.advect(steps)
    _, L = S.LINEARIZE_L(sol)
    co = orc.linearize()
    return cfg, cs, sol, orc, L, co


def _sparse_recept(cfg, coef, rows, bq, w):
    """L_ = [L, B ... B; 0, diag(-i w_k I)] as a scipy sparse matrix from the blocks."""
    import scipy.sparse as sp
    nchi, N = cfg.nchi, cfg.nchi * cfg.neta
    L = O.stencil_to_csr(cfg, coef)
    r, c, v = [], [], []
    for m in range(nchi):
        cell = m + (rows[m] - 2) * nchi
        for d in (-1, 0, 1):
            n = m + d
            if 0 <= n < nchi:
                for vo in range(4):
                    for vi in range(4):
                        r.append(vo * N + cell)
                        c.append(vi * nchi + n)
                        v.append(bq[m, d + 1, vo, vi])
    B = sp.csr_matrix((v, (r, c)), shape=(4 * N, 4 * nchi))
    p = 4 * nchi
    top = sp.hstack([L] + [B] * len(w))
    bot = sp.hstack([sp.csr_matrix((len(w) * p, 4 * N)), sp.kron(sp.diags(-1j * np.asarray(w)), sp.eye(p))])
    return sp.vstack([top, bot]).tocsr().astype(complex)


def _exponential(A, x, dt, n_t, order=5):
    """EXPONENTIAL!'s Taylor recurrence (CONSTRUCT_C.jl:78-111) with the matrix A dt."""
    Adt = A * dt
    vout = x.copy()
    for _ in range(n_t):
        term = vout.copy()
        for j in range(1, order + 1):
            term = (Adt @ term) * (1.0 / j)
            vout = vout + term
    return vout


@pytest.mark.gpu
@pytest.mark.parametrize("cone", [False, True])
def test_b_parity(require_gpu, cone):
    """The device's LINEARIZE_B against the oracle's (finite differences with eps = 1e-8 of
    residuals that agree to ~1e-13: agreement to the FD rounding), on the cylinder and the
    axisymmetric sphere-cone."""
    from hymor_gb300 import receptivity as R
    cfg, cs, sol, orc, L, co = _gpu_case(48, 24, steps=5, cone=True) if cone else _gpu_case()
    rows, bq, bs = R.LINEARIZE_B(sol)
    rows_o, bq_o, bs_o = orc.linearize_b()
    assert np.array_equal(rows, rows_o)
    assert rel_err(bq, bq_o) < 1e-5
    assert rel_err(bs, bs_o) < 1e-5


@pytest.mark.gpu
def test_receptivity_operator_parity(require_gpu):
    """L_ and L_^H (hymor_recept_apply_dev) and their Taylor propagation against the sparse
    restatement from the device's own blocks: 1e-12."""
    from hymor_gb300 import receptivity as R
    cfg, cs, sol, orc, L, co = _gpu_case()
    w = [0.0, 1.5, 4.0]
    _, Lr = R.LINEARIZE_L_(L, sol, w)
    rows, bq, _ = R.LINEARIZE_B(sol)
    A = _sparse_recept(cfg, L.blocks(), rows, bq, w)
    assert A.shape == (Lr.n, Lr.n)
    rng = np.random.Generator(np.random.PCG64(6))
    X = rng.standard_normal((Lr.n, 2)) + 1j * rng.standard_normal((Lr.n, 2))
    for adj, M in ((False, A), (True, A.conj().T.tocsr())):
        Y = Lr.apply(X, adjoint=adj)
        for j in range(2):
            ref = M @ X[:, j]
            assert np.max(np.abs(Y[:, j] - ref)) <= 1e-12 * np.max(np.abs(ref))
        P = Lr.expm(X[:, 0], 2e-3, 7, adjoint=adj)
        ref = _exponential(M, X[:, 0], 2e-3, 7)
        assert np.max(np.abs(P - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.gpu
def test_freestream_receptivity_vs_eigsh(require_gpu):
    """FREESTREAM_RECEPTIVITY (device Krylov-Schur on the real form of the reduced Hermitian
    problem) against eigsh on the complex Hermitian operator composed from the sparse
    restatement, the same weights and the same propagation: gains to 1e-6."""
    sla = pytest.importorskip("scipy.sparse.linalg")
    from hymor_gb300 import receptivity as R
    from hymor_gb300 import solver as S
    cfg, cs, sol, orc, L, co = _gpu_case()
    w = [0.0, 2.0]
    _, Lr = R.LINEARIZE_L_(L, sol, w)
    V, G, T_opt, info = R.FREESTREAM_RECEPTIVITY(Lr, sol, 2, 0.01, ncv=16, tol=1e-10, modes=True)
    rows, bq, _ = R.LINEARIZE_B(sol)
    A = _sparse_recept(cfg, L.blocks(), rows, bq, w)
    AH = A.conj().T.tocsr()
    N, p = cfg.nchi * cfg.neta, 4 * cfg.nchi
    C0, _ = S.chu_blocks(sol)
    Ki = np.linalg.inv(np.linalg.cholesky(R.freestream_weights(sol, w)))   # (Nw, Nchi, 4, 4)
    dt, nt = info["dt"], info["n_t"]

    def mv(y):
        y = np.asarray(y).ravel()
        x = np.einsum("knji,kjn->kin", Ki, y.reshape(len(w), 4, cfg.nchi)).ravel()
        z = np.concatenate([np.zeros(4 * N, dtype=complex), x])
        z = _exponential(A, z, dt, nt)
        q = z[:4 * N].reshape(4, N).T
        z = np.concatenate([np.einsum("nij,nj->ni", C0, q).T.ravel(), np.zeros(len(w) * p)])
        z = _exponential(AH, z, dt, nt)
        return np.einsum("knij,kjn->kin", Ki, z[4 * N:].reshape(len(w), 4, cfg.nchi)).ravel()
    nf = len(w) * p
    op = sla.LinearOperator((nf, nf), matvec=mv, dtype=complex)
    lam = np.sort(np.real(sla.eigsh(op, k=2, which="LA", tol=1e-12, return_eigenvectors=False)))[::-1] / 2
    assert np.allclose(np.sort(G)[::-1], lam, rtol=1e-6, atol=0)
    assert info["converged"] and V.shape == (Lr.n, 2)
    assert np.all(V[:4 * N] == 0)


@pytest.mark.gpu
def test_residual_with_upstream_state(require_gpu):
    """hymor_set_upstream: the residual with a prescribed per-column upstream state against
    the oracle's (rho_0_upstream_p), to 1e-12 of the flux scale; and the device B passes
    the reference's CHECK_LINEARIZATION_B measure (< 1e-3)."""
    from hymor_gb300 import receptivity as R
    from hymor_gb300 import solver as S
    from hymor_gb300._lib import dp
    from helpers import residual_rel
    cfg, cs, sol, orc, L, co = _gpu_case()
    st = sol.get_state()
    fs = np.array([orc.cs.rho_0, orc.cs.rho_u_0, orc.cs.rho_v_0, orc.cs.rho_E_0])
    cols = np.ascontiguousarray(fs[:, None] * (1 + 1e-3 * np.random.Generator(np.random.PCG64(9)).standard_normal(
        (4, cfg.nchi))))
    pts = (st["pts_x"], st["pts_y"], st["pts_chi"], st["pts_eta"])
    o = O.Oracle(cs)
    o.set_state(st["q"], *pts, st["cell_idx"], st["t"])
    o.set_upstream(cols)
    s2 = S.Solution(cs)
    s2.set_state(np.asarray(st["q"]), *pts, st["cell_idx"], st["t"])
    s2.ctx.check(s2.ctx.L.hymor_set_upstream(s2.ctx.h, dp(cols.ravel())))
    assert max(residual_rel(S.PDE(s2), o.residual(), cs)) < 1e-12
    s2.close()
    err = R.CHECK_LINEARIZATION_B(R.LINEARIZE_B(sol), sol, seed=3, verbose=False)
    assert err < 1e-3


@pytest.mark.gpu
def test_receptivity_operator_with_shock_unknowns(require_gpu):
    """L_ with the shock-position unknowns (perturb_shock): the downstream part is the
    extended operator [A11 A12; A21 A22] and B has speed rows; apply and adjoint against the
    sparse restatement from the device's own blocks, 1e-12."""
    import scipy.sparse as sp
    from hymor_gb300 import receptivity as R
    from hymor_gb300 import solver as S
    cfg = C.cylinder_config(24, 20, perturb_shock=True)
    cs = C.initial_state(cfg)
    sol = S.Solution(cs)
    S.ADVECT_FLOW(sol, 5)
    _, L = S.LINEARIZE_L(sol)
    w = [0.0, 3.0]
    _, Lr = R.LINEARIZE_L_(L, sol, w)
    rows_b, bq, bs = R.LINEARIZE_B(sol)
    rows, a21, a12, a22 = L.shock_blocks()
    nchi, N = cfg.nchi, cfg.nchi * cfg.neta
    n_down = 4 * N + nchi
    assert Lr.n == n_down + len(w) * 4 * nchi
    A11 = O.stencil_to_csr(cfg, L.blocks())
    r, c, v = [], [], []
    for i in range(nchi):
        for vv in range(4):
            for p in range(nchi):
                r.append(vv * N + i + (rows[i] - 2) * nchi); c.append(4 * N + p); v.append(a12[vv * nchi + i, p])
            for j in (1, 2):
                r.append(4 * N + i); c.append(vv * N + i + (rows[i] - 1 - j) * nchi); v.append(a21[i, (j - 1) * 4 + vv])
        for p in range(nchi):
            r.append(4 * N + i); c.append(4 * N + p); v.append(a22[i, p])
    Ld = sp.csr_matrix((v, (r, c)), shape=(n_down, n_down)) + sp.block_diag([A11, sp.csr_matrix((nchi, nchi))])
    r, c, v = [], [], []
    for m in range(nchi):
        cell = m + (rows_b[m] - 2) * nchi
        for d in (-1, 0, 1):
            n = m + d
            if 0 <= n < nchi:
                for vi in range(4):
                    for vo in range(4):
                        r.append(vo * N + cell); c.append(vi * nchi + n); v.append(bq[m, d + 1, vo, vi])
                    r.append(4 * N + m); c.append(vi * nchi + n); v.append(bs[m, d + 1, vi])
    B = sp.csr_matrix((v, (r, c)), shape=(n_down, 4 * nchi))
    p4 = 4 * nchi
    A = sp.vstack([sp.hstack([Ld] + [B] * len(w)),
                   sp.hstack([sp.csr_matrix((len(w) * p4, n_down)),
                              sp.kron(sp.diags(-1j * np.asarray(w)), sp.eye(p4))])]).tocsr().astype(complex)
    rng = np.random.Generator(np.random.PCG64(7))
    x = rng.standard_normal(Lr.n) + 1j * rng.standard_normal(Lr.n)
    for adj, M in ((False, A), (True, A.conj().T.tocsr())):
        ref = M @ x
        assert np.max(np.abs(Lr.apply(x, adjoint=adj) - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_linearize_b_axisymmetric_first_column():
    """On an axisymmetric case the reference zeroes rho_v of the first column's upstream
    state (COMPUTE_UPSTREAM_CONDITIONS.jl:105-108), so B has no entries for that input;
    the other inputs of the first column act."""
    cfg = C.blunt_cone_config(48, 24)
    cs = C.initial_state(cfg)
    orc = O.Oracle(cs)
    orc.advect(2)
    orc.linearize()
    rows, bq, bs = orc.linearize_b()
    # input column n = 0 is reached from output columns m = 0 (d = 0) and m = 1 (d = -1)
    assert np.all(bq[0, 1, :, 2] == 0) and np.all(bq[1, 0, :, 2] == 0)
    assert np.all(bs[0, 1, 2] == 0) and np.all(bs[1, 0, 2] == 0)
    assert np.max(np.abs(bq[0, 1, :, 0])) > 0 and np.max(np.abs(bq[2, 1, :, 2])) > 0


@pytest.mark.gpu
def test_receptivity_batch_uneven_grids(require_gpu):
    """FREESTREAM_RECEPTIVITY_BATCH: three cases of different grids, Mach numbers and
    frequency sets solved together (lockstep Krylov-Schur, the cases' propagations enqueued
    together on their own streams) give each case's own FREESTREAM_RECEPTIVITY gains: the
    same operations in the same order, so to rounding of nothing (1e-12 allowed)."""
    from hymor_gb300 import receptivity as R
    from hymor_gb300 import solver as S
    specs = [(24, 20, 5.0, 1e4, [0.0, 2.0]), (36, 24, 6.0, 2e4, [0.5, 1.0, 3.0]), (28, 28, 4.0, 5e3, [1.0])]
    cases, sols = [], []
    for nchi, neta, M, Re, w in specs:
        cs = C.initial_state(C.cylinder_config(nchi, neta, Mach=M, Re=Re))
        sol = S.Solution(cs)
        S.ADVECT_FLOW(sol, 20)
        _, L = S.LINEARIZE_L(sol)
        _, Lr = R.LINEARIZE_L_(L, sol, w)
        cases.append((Lr, sol))
        sols.append(sol)
    batch = R.FREESTREAM_RECEPTIVITY_BATCH(cases, 2, 0.01, ncv=16, tol=1e-10)
    for (Lr, sol), (G, info) in zip(cases, batch):
        _, G1, _, info1 = R.FREESTREAM_RECEPTIVITY(Lr, sol, 2, 0.01, ncv=16, tol=1e-10)
        assert info["converged"] and info1["converged"]
        assert np.allclose(G, G1, rtol=1e-12, atol=0), (G, G1)
        assert info["nops"] == info1["nops"]
    for sol in sols:
        sol.close()
