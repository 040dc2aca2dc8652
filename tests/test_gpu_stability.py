"""GPU stability drivers: the exponential-transform eigen solver and transient growth
(device-resident Krylov-Schur) against ARPACK on the oracle's propagator, with the same
Jacobian blocks, plus the adjoint identities of the propagator and the FD check of the
linearisation."""
import numpy as np
import pytest

from hymor_gb300 import case as C
from hymor_gb300 import solver as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _setup(nchi, neta, steps=20):
    cfg = C.cylinder_config(nchi, neta)
    cs = C.initial_state(cfg)
    sol, orc = S.Solution(cs), O.Oracle(cs)
    S.ADVECT_FLOW(sol, steps)
    orc.advect(steps)
    return cfg, cs, sol, orc


def test_eigenvalues_device_vs_oracle(require_gpu):
    sla = pytest.importorskip("scipy.sparse.linalg")
    cfg, cs, sol, orc = _setup(30, 20)
    _, L = S.LINEARIZE_L(sol)
    co = orc.linearize()
    L.set_blocks(co)
    lam, info = S.EIGENVALUES(L, sol, 4, T_ref=0.02, ncv=24, tol=1e-11)
    dt, nt = info["dt"], info["timesteps"]
    n = 4 * cfg.nchi * cfg.neta
    op = sla.LinearOperator((n, n), matvec=lambda x: orc.expm(co, dt, nt, np.ascontiguousarray(x).ravel()),
                            dtype=np.float64)
    mu = sla.eigs(op, k=4, which="LM", tol=1e-13, ncv=24, return_eigenvectors=False)
    mu = mu[np.argsort(-np.abs(mu))]
    lam_o = np.log(mu.astype(complex)) / (dt * nt)
    for a in lam:
        assert np.min(np.abs(lam_o - a)) <= 1e-8 * np.max(np.abs(lam_o))
    assert np.all(info["resid"] <= 1e-11 * np.abs(info["mu"]))
    # the reference's structure (host ARPACK, one GPU propagation per vector) agrees
    lam_h, _ = S.EIGENVALUES(L, sol, 4, T_ref=0.02, ncv=24, tol=1e-12, method="host")
    for a in lam:
        assert np.min(np.abs(lam_h - a)) <= 1e-8 * np.max(np.abs(lam_o))


def test_transient_growth_device_vs_oracle(require_gpu):
    sla = pytest.importorskip("scipy.sparse.linalg")
    cfg, cs, sol, orc = _setup(24, 24)
    _, L = S.LINEARIZE_L(sol)
    co = orc.linearize()
    L.set_blocks(co)
    T = 0.01
    G, info = S.TRANSIENT_GROWTH_DOWNSTREAM(L, sol, 2, T, ncv=16, tol=1e-11)
    st = sol.get_state()
    C0, D = S.chu_blocks_from_state(cfg, cs.mesh["vol"], st["q"], st["cell_idx"])
    K = np.linalg.cholesky(D)
    Ki = np.linalg.inv(K)
    N = cfg.nchi * cfg.neta

    def blk(B, x):
        X = x.reshape(4, N).T
        return np.einsum("nij,nj->ni", B, X).T.ravel()
    dt, nt = info["dt"], info["n_t"]

    def mv(y):
        x = blk(np.transpose(Ki, (0, 2, 1)), np.ascontiguousarray(y).ravel())
        z = orc.expm(co, dt, nt, x)
        z = blk(C0, z)
        z = orc.expm(co, dt, nt, z, transpose=True)
        return blk(Ki, z)
    op = sla.LinearOperator((4 * N, 4 * N), matvec=mv, dtype=np.float64)
    Go = np.sort(sla.eigsh(op, k=2, which="LA", tol=1e-13, return_eigenvectors=False))[::-1]
    assert np.allclose(np.sort(G)[::-1], Go, rtol=1e-6, atol=0)


def test_eigenvalue_modes_and_nonconvergence(require_gpu):
    """modes=True returns the eigenvectors (the reference's V): exp(L T) x = mu x for each;
    a solve that stops short of tol warns and returns NaN, as the reference does, unless
    keep_unconverged."""
    cfg, cs, sol, orc = _setup(30, 20)
    _, L = S.LINEARIZE_L(sol)
    for block in (1, 4):
        lam, info = S.EIGENVALUES(L, sol, 4, T_ref=0.02, ncv=28, tol=1e-10, block=block, modes=True)
        X, mu = info["modes"], info["mu"]
        assert X.shape == (4 * cfg.nchi * cfg.neta, 4)
        dt, nt = info["dt"], info["timesteps"]
        for i in range(4):
            x = X[:, i]
            Px = L.expm(np.ascontiguousarray(x.real), dt, nt) + 1j * L.expm(np.ascontiguousarray(x.imag), dt, nt)
            assert np.linalg.norm(Px - mu[i] * x) <= 1e-8 * abs(mu[i])
    with pytest.warns(UserWarning):
        lam, info = S.EIGENVALUES(L, sol, 4, T_ref=0.02, ncv=24, tol=1e-15, maxit=2, modes=True)
    assert np.all(np.isnan(lam)) and np.all(np.isnan(info["modes"])) and not info["converged"]
    lam, info = S.EIGENVALUES(L, sol, 4, T_ref=0.02, ncv=24, tol=1e-15, maxit=2, keep_unconverged=True)
    assert np.all(np.isfinite(lam)) and not info["converged"]


def test_transient_growth_modes(require_gpu):
    """modes=True returns the optimal initial conditions x (the reference's V), D-normalised
    (x' R'M^R x = 1) with Rayleigh quotient (P x)' R'MR (P x) = G."""
    cfg, cs, sol, orc = _setup(24, 24)
    _, L = S.LINEARIZE_L(sol)
    G, info = S.TRANSIENT_GROWTH_DOWNSTREAM(L, sol, 2, 0.01, ncv=16, tol=1e-11, modes=True)
    X = info["modes"]
    C0, D = S.chu_blocks(sol)
    N = cfg.nchi * cfg.neta

    def blk(B, x):
        return np.einsum("nij,nj->ni", B, x.reshape(4, N).T).T.ravel()
    for i in range(2):
        x = np.ascontiguousarray(X[:, i])
        assert abs(x @ blk(D, x) - 1) < 1e-10
        Px = L.expm(x, info["dt"], info["n_t"])
        assert abs(Px @ blk(C0, Px) - G[i]) <= 1e-8 * abs(G[i])


def test_block_eigenvalues_match_single_vector(require_gpu):
    """Block Krylov-Schur (4 vectors per batched propagation) finds the same eigenvalues
    as the single-vector Krylov-Schur, to 1e-8 of the spectrum's scale."""
    cfg, cs, sol, orc = _setup(30, 20)
    _, L = S.LINEARIZE_L(sol)
    lam1, info1 = S.EIGENVALUES(L, sol, 4, T_ref=0.02, ncv=24, tol=1e-11)
    lam4, info4 = S.EIGENVALUES(L, sol, 4, T_ref=0.02, ncv=28, tol=1e-10, block=4)
    scale = np.max(np.abs(lam1))
    for a in lam4:
        assert np.min(np.abs(lam1 - a)) <= 1e-8 * scale
    assert np.all(info4["resid"] <= 1e-10 * np.abs(info4["mu"]))
    assert info4["nops"] % 4 == 0


def test_block_transient_growth_matches_single_vector(require_gpu):
    """Block Lanczos (Krylov-Schur, symmetric) on the transient-growth operator gives the
    single-vector gains to 1e-6."""
    cfg, cs, sol, orc = _setup(24, 24)
    _, L = S.LINEARIZE_L(sol)
    G1, _ = S.TRANSIENT_GROWTH_DOWNSTREAM(L, sol, 2, 0.01, ncv=16, tol=1e-11)
    G4, _ = S.TRANSIENT_GROWTH_DOWNSTREAM(L, sol, 2, 0.01, ncv=20, tol=1e-10, block=4)
    assert np.allclose(np.sort(G4)[::-1], np.sort(G1)[::-1], rtol=1e-6, atol=0)


def test_propagator_adjoint_identity(require_gpu):
    """<P x, y> = <x, Pᵀ y> for the Taylor propagator and its adjoint (the dot-product test)."""
    cfg, cs, sol, orc = _setup(30, 20, steps=5)
    _, L = S.LINEARIZE_L(sol)
    rng = np.random.Generator(np.random.PCG64(4))
    n = 4 * cfg.nchi * cfg.neta
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    dt = S.CFL_TIMESTEP(sol)
    Px = L.expm(x, dt, 25)
    Pty = L.T.expm(y, dt, 25)
    lhs, rhs = np.dot(Px, y), np.dot(x, Pty)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_adjoint_identities_at_600x300(require_gpu):
    """The transient-growth case's checks at its size (600 x 300 cylinder, 720 000
    unknowns): the seeded dot-product test <L x, y> = <x, Lᵀ y> for the matvec and for the
    Taylor propagator (50 steps of the CFL dt), to 1e-12."""
    cfg = C.cylinder_config(600, 300)
    sol = S.Solution(C.initial_state(cfg))
    S.ADVECT_FLOW(sol, 5)
    _, L = S.LINEARIZE_L(sol)
    rng = np.random.Generator(np.random.PCG64(4))
    n = 4 * cfg.nchi * cfg.neta
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    lhs, rhs = np.dot(L @ x, y), np.dot(x, L.T @ y)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    dt = S.CFL_TIMESTEP(sol)
    lhs, rhs = np.dot(L.expm(x, dt, 50), y), np.dot(x, L.T.expm(y, dt, 50))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    sol.close()


def test_check_linearization_l(require_gpu):
    """CHECK_LINEARIZATION_L, the reference's own consistency measure (below ~1e-3 means a
    consistent linearisation), on the GPU operator and residual."""
    cfg, cs, sol, orc = _setup(30, 20, steps=10)
    _, L = S.LINEARIZE_L(sol)
    err = S.CHECK_LINEARIZATION_L(L, sol, seed=7)
    assert err < 1e-3


def test_linearisation_matches_residual_differences(require_gpu):
    """CHECK_LINEARIZATION_L.jl:33-130 on the GPU: L q ~ f(x + q) - f(x) (central, h = 1e-7)."""
    cfg, cs, sol, orc = _setup(30, 20, steps=10)
    _, L = S.LINEARIZE_L(sol)
    st = sol.get_state()
    N = cfg.nchi * cfg.neta
    rng = np.random.Generator(np.random.PCG64(5))
    flow = (np.arange(1, cfg.neta + 1)[None, :] < st["cell_idx"][:, None]).ravel(order="F")
    dq = rng.standard_normal(4 * N) * np.tile(flow, 4)
    h = 1e-7

    def residual_at(sign):
        q = st["q"].copy().reshape(4, -1)
        for v in range(4):
            blk = q[v].reshape(cfg.nchi + 2, cfg.neta + 2, order="F")
            blk[1:-1, 1:-1] += sign * h * dq[v * N:(v + 1) * N].reshape(cfg.nchi, cfg.neta, order="F")
            q[v] = blk.ravel(order="F")
        s2 = S.Solution(cs)
        s2.set_state(q.ravel(), st["pts_x"], st["pts_y"], st["pts_chi"], st["pts_eta"], st["cell_idx"], st["t"])
        return S.PDE(s2)
    df = (residual_at(+1) - residual_at(-1)) / (2 * h)
    Lq = L @ dq
    assert np.linalg.norm(Lq - df) / np.linalg.norm(df) < 1e-3


def test_expm_multi_matches_single_propagations(require_gpu):
    """hymor_expm_apply_multi_dev: k propagations with their own dt and step counts in one
    batched call equal the k one-vector propagations (the same FMA chains per output)."""
    import ctypes
    from hymor_gb300.krylov import DeviceBuffer
    cfg, cs, sol, orc = _setup(30, 20, steps=5)
    _, L = S.LINEARIZE_L(sol)
    n = L.n
    rng = np.random.Generator(np.random.PCG64(8))
    X = rng.standard_normal((3, n))
    dts = np.array([1.1e-3, 0.9e-3, 1.3e-3])
    steps = np.array([40, 25, 7], dtype=np.int32)
    bx, by = DeviceBuffer(sol.ctx, 8 * n * 3), DeviceBuffer(sol.ctx, 8 * n * 3)
    bx.upload(X.ravel())
    Lh, h = sol.ctx.L, sol.ctx.h
    for tr in (0, 1):
        sol.ctx.check(Lh.hymor_expm_apply_multi_dev(h, 3, dts.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                    steps.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 5,
                                                    bx.ptr, by.ptr, tr))
        Y = by.download(3 * n).reshape(3, n)
        P = L.T if tr else L
        for c in range(3):
            ref = P.expm(X[c], dts[c], int(steps[c]))
            assert np.max(np.abs(Y[c] - ref)) <= 1e-14 * np.max(np.abs(ref))
    bx.free()
    by.free()


def test_transient_growth_horizons_batched(require_gpu):
    """TRANSIENT_GROWTH_HORIZONS (the horizons of one solve propagated together, lockstep
    Krylov-Schur) gives each horizon's TRANSIENT_GROWTH_DOWNSTREAM gains."""
    cfg, cs, sol, orc = _setup(24, 24)
    _, L = S.LINEARIZE_L(sol)
    Ts = [0.004, 0.016, 0.008]
    G, infos = S.TRANSIENT_GROWTH_HORIZONS(L, sol, 2, Ts, ncv=16, tol=1e-11)
    for h, T in enumerate(Ts):
        g1, info1 = S.TRANSIENT_GROWTH_DOWNSTREAM(L, sol, 2, T, ncv=16, tol=1e-11)
        assert np.allclose(G[h], g1, rtol=1e-9, atol=0)
        assert infos[h]["n_t"] == info1["n_t"] and infos[h]["converged"]
