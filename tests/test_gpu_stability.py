"""GPU stability drivers: the exponential-transform eigen solver and transient growth
(device-resident Krylov-Schur) against ARPACK on the oracle's propagator, with the same
Jacobian blocks, plus the adjoint identities of the propagator and the FD check of the
linearisation."""
import numpy as np
import pytest

from hymor_gb300 import case as C
from hymor_gb300 import solver as S
from helpers import rel_err
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


def test_expm_float_float_against_fp64(require_gpu):
    """The cooperative propagator in float-float arithmetic (the default) against the same
    propagator in FP64 on the same Jacobian: 200 Taylor steps of degree 4 and 5, forward and
    adjoint, one vector and a batch of 8; then, after the Jacobian is linearised again on a
    later state, the float-float copy of the blocks follows it."""
    cfg, cs, sol, orc = _setup(60, 40, steps=5)
    _, L = S.LINEARIZE_L(sol)
    rng = np.random.Generator(np.random.PCG64(31))
    X = rng.standard_normal((L.n, 8))
    dt = S.CFL_TIMESTEP(sol)
    worst = 0.0
    for order in (4, 5):
        for P in (L, L.T):
            for x in (X[:, 0], X):
                sol.set_expm_arith(1)
                yf = P.expm(x, dt, 200, order=order)
                sol.set_expm_arith(0)
                yd = P.expm(x, dt, 200, order=order)
                assert np.isfinite(yf).all()
                e = rel_err(yf, yd)
                worst = max(worst, e)
                assert e < 1e-10, (order, e)
    print(f"\nfloat-float against FP64, 200 steps: {worst:.2e}")
    sol.set_expm_arith(1)
    S.ADVECT_FLOW(sol, 10)
    _, L2 = S.LINEARIZE_L(sol)
    yf = L2.expm(X[:, 1], dt, 50)
    sol.set_expm_arith(0)
    yd = L2.expm(X[:, 1], dt, 50)
    assert rel_err(yf, yd) < 1e-10
    sol.close()


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


@pytest.mark.slow
def test_channel_eigenvalue_pin_device(require_gpu):
    """tutorials/channel_flow/README.md:164-168, through the device: the channel (180 x 60,
    Re 7500, M 0.05) linearised by LINEARIZE_L on the GPU has the leading eigenvalue
    0.000247 + 0.248408i, the reference's printed answer, held to the oracle's 5e-6 (the FD
    Jacobian's rounding moves it by ~1e-5 at M 0.05). Shift-invert on the host, as the
    tutorial's main.jl:69-81."""
    import json
    import os
    sla = pytest.importorskip("scipy.sparse.linalg")
    cfg = C.channel_config()
    cs = C.initial_state(cfg, noise=0.0)
    sol = S.Solution(cs)
    _, L = S.LINEARIZE_L(sol)
    A = O.stencil_to_csr(cfg, L.blocks())
    lam = sla.eigs(A.astype(complex), k=1, sigma=0.25j, return_eigenvectors=False)[0]
    ka = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))
    pin = ka["channel_eigenvalue"]
    assert abs(lam.real - pin["re"]) < 5e-6, lam
    assert abs(lam.imag - pin["im"]) < 5e-6, lam
    sol.close()


@pytest.mark.slow
def test_eigenvalues_sphere_cone_degree4(require_gpu):
    """The batched-modal-analysis configuration's shape at reduced size: the axisymmetric
    7-degree sphere-cone (M 6, Re 2e4) at 240 x 80, exp(L dt_50) built from 50 Taylor steps
    of degree 4 (the RK4-substep form of the propagator), start vector on the flow cells.
    The device Krylov-Schur eigenvalues match ARPACK on the oracle's propagator to 1e-8 of
    the spectrum's scale, with the same Jacobian blocks."""
    sla = pytest.importorskip("scipy.sparse.linalg")
    cfg = C.blunt_cone_config(240, 80)
    cs = C.initial_state(cfg)
    sol, orc = S.Solution(cs), O.Oracle(cs)
    S.ADVECT_FLOW(sol, 20)
    orc.advect(20)
    _, L = S.LINEARIZE_L(sol)
    co = orc.linearize()
    L.set_blocks(co)
    dt = S.CFL_TIMESTEP(sol)
    lam, info = S.EIGENVALUES(L, sol, 4, T_ref=50 * dt, order=4, ncv=30, tol=1e-11, flow_start=True)
    assert info["timesteps"] == 50 and info["converged"]
    n = 4 * cfg.nchi * cfg.neta
    st = sol.get_state()
    flow = (np.arange(1, cfg.neta + 1)[None, :] < st["cell_idx"][:, None]).ravel(order="F")
    v0 = np.random.Generator(np.random.PCG64(3)).standard_normal(n) * np.tile(flow, 4)
    op = sla.LinearOperator((n, n), matvec=lambda x: orc.expm(co, info["dt"], 50, np.ascontiguousarray(x).ravel(),
                                                             order=4), dtype=np.float64)
    mu = sla.eigs(op, k=4, which="LM", tol=1e-12, ncv=30, v0=v0, return_eigenvectors=False)
    lam_o = np.log(mu.astype(complex)) / (info["dt"] * 50)
    scale = np.max(np.abs(lam_o))
    for a in lam:
        assert np.min(np.abs(lam_o - a)) <= 1e-8 * scale, (lam, lam_o)
    sol.close()


@pytest.mark.slow
def test_transient_growth_cylinder_T1(require_gpu):
    """The transient-growth configuration's family at reduced size: the cylinder with the
    same wall-normal stretch at 80 x 40 and a horizon of one freestream time unit (T = 1,
    1126 Taylor steps of the CFL dt). The device gains match eigsh on the oracle's forward
    and adjoint propagators to 1e-6, with the same Jacobian blocks."""
    sla = pytest.importorskip("scipy.sparse.linalg")
    cfg, cs, sol, orc = _setup(80, 40)
    _, L = S.LINEARIZE_L(sol)
    co = orc.linearize()
    L.set_blocks(co)
    G, info = S.TRANSIENT_GROWTH_DOWNSTREAM(L, sol, 2, 1.0, ncv=16, tol=1e-11)
    assert info["n_t"] > 1000 and info["converged"]
    st = sol.get_state()
    C0, D = S.chu_blocks_from_state(cfg, cs.mesh["vol"], st["q"], st["cell_idx"])
    Ki = np.linalg.inv(np.linalg.cholesky(D))
    N = cfg.nchi * cfg.neta

    def blk(B, x):
        return np.einsum("nij,nj->ni", B, x.reshape(4, N).T).T.ravel()
    dt, nt = info["dt"], info["n_t"]

    def mv(y):
        x = blk(np.transpose(Ki, (0, 2, 1)), np.ascontiguousarray(y).ravel())
        z = blk(C0, orc.expm(co, dt, nt, x))
        return blk(Ki, orc.expm(co, dt, nt, z, transpose=True))
    op = sla.LinearOperator((4 * N, 4 * N), matvec=mv, dtype=np.float64)
    Go = np.sort(sla.eigsh(op, k=2, which="LA", tol=1e-12, ncv=16, return_eigenvectors=False))[::-1]
    assert np.allclose(np.sort(G)[::-1], Go, rtol=1e-6, atol=0), (G, Go)
    sol.close()


def test_cabi_solvers_match_python_driver(require_gpu):
    """hymor_eigs and hymor_tg_gain (the Krylov-Schur solvers behind the C ABI, with their own
    dense steps) give the eigenvalues and gains of the same Krylov-Schur driven from Python
    with LAPACK's dense steps (krylov.py), on the same device operator and start vectors:
    the two differ only in the rounding of the projected-matrix steps."""
    cfg, cs, sol, orc = _setup(30, 20)
    _, L = S.LINEARIZE_L(sol)
    for block in (1, 3):
        lam_c, ic = S.EIGENVALUES(L, sol, 4, T_ref=0.02, ncv=24, tol=1e-11, block=block)
        lam_p, ip_ = S.EIGENVALUES(L, sol, 4, T_ref=0.02, ncv=24, tol=1e-11, block=block, method="python")
        assert ic["converged"] and ip_["converged"]
        scale = np.max(np.abs(lam_p))
        for a in lam_c:
            assert np.min(np.abs(lam_p - a)) <= 1e-9 * scale, (block, lam_c, lam_p)
    G_c, ic = S.TRANSIENT_GROWTH_DOWNSTREAM(L, sol, 2, 0.01, ncv=16, tol=1e-11, modes=True)
    G_p, ip_ = S.TRANSIENT_GROWTH_DOWNSTREAM(L, sol, 2, 0.01, ncv=16, tol=1e-11, modes=True, method="python")
    assert np.allclose(G_c, G_p, rtol=1e-9, atol=0), (G_c, G_p)
    for i in range(2):  # the same optimal initial conditions up to sign
        a, b = ic["modes"][:, i], ip_["modes"][:, i]
        assert min(np.linalg.norm(a - b), np.linalg.norm(a + b)) <= 1e-7 * np.linalg.norm(b)
    Ts = [0.004, 0.016, 0.008]
    Gh_c, _ = S.TRANSIENT_GROWTH_HORIZONS(L, sol, 2, Ts, ncv=16, tol=1e-11)
    Gh_p, _ = S.TRANSIENT_GROWTH_HORIZONS(L, sol, 2, Ts, ncv=16, tol=1e-11, method="python")
    assert np.allclose(Gh_c, Gh_p, rtol=1e-9, atol=0)


def test_cabi_eigs_seeded_start_and_errors(require_gpu):
    """hymor_eigs called as a C caller would: no start vector (the library's seeded normal
    start, masked to the flow cells), the converged flag, and the errors before a Jacobian
    exists or with inconsistent options."""
    import ctypes
    from hymor_gb300 import _lib
    from hymor_gb300._lib import dp, ip
    cfg, cs, sol, orc = _setup(30, 20)
    Lh, h = sol.ctx.L, sol.ctx.h
    o = S._krylov_opts(4, 24, 1e-10, 300, 1, 5, seed=11, flow_start=True)
    mr, mi, res = np.empty(4), np.empty(4), np.empty(4)
    info = np.zeros(3, dtype=np.int32)
    dt = S.CFL_TIMESTEP(sol)
    assert Lh.hymor_eigs(h, ctypes.byref(o), dt, 40, None, dp(mr), dp(mi), dp(res), ip(info), None) == -6
    _, L = S.LINEARIZE_L(sol)
    sol.ctx.check(Lh.hymor_eigs(h, ctypes.byref(o), dt, 40, None, dp(mr), dp(mi), dp(res), ip(info), None))
    assert info[2] == 1 and info[0] > 0
    assert np.all(res <= 1e-10 * np.abs(mr + 1j * mi))
    lam_ref, _ = S.EIGENVALUES(L, sol, 4, T_ref=40 * dt, ncv=24, tol=1e-10, flow_start=True)
    lam = np.log((mr + 1j * mi).astype(complex)) / (dt * 40)
    for a in lam:
        assert np.min(np.abs(lam_ref - a)) <= 1e-8 * np.max(np.abs(lam_ref))
    bad = S._krylov_opts(10, 11, 1e-10, 300, 1, 5)
    assert Lh.hymor_eigs(h, ctypes.byref(bad), dt, 40, None, dp(mr), dp(mi), None, None, None) == -1
    assert "nev + 2 block <= ncv" in Lh.hymor_last_error(h).decode()
