"""Freestream receptivity over libhymor (utils/Stability_analysis/Freestream_receptivity).

The reference extends the linearised operator with the upstream state of every column and
one block of freestream unknowns per disturbance frequency (LINEARIZE_L_.jl:36-71),

    L_ = [L,  B, ..., B;  0, diag(-i w_k I_{4 Nchi})],

and finds the freestream disturbances of largest energy gain over a horizon T: the
generalised Hermitian eigenproblem C x = G D x with C = Z exp(L_ T)^H R'MR exp(L_ T) Z (Z
zeroes the downstream cells, CONSTRUCT_C.jl:55-76) and D = R_' M_infty_ R_
(FREESTREAM_RECEPTIVITY.jl:37-162). Here B is assembled on the device (hymor_linearize_b),
L_ and its conjugate transpose act on the device (hymor_recept_apply_dev / _expm_dev), and
the eigenproblem is solved by the device Krylov-Schur on the real form of the unknowns the
initial condition may carry (the shock displacements and the freestream blocks), reduced
with the per-block Cholesky factor of D. The weights (R, M, M_infty, a handful of 4 x 4
blocks per column) are host-side set-up, as in the reference.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import dp, ip
from .krylov import DeviceBuffer, krylov_schur
from .solver import CFL_TIMESTEP, LinearOperatorGPU, Solution, chu_blocks


def GET_T_REF(s: Solution) -> float:
    """GET_T_REF (GET_T_REF.jl:20-48): the downstream mass over the mass flux through the
    shock, sum(rho flow vol) / sum_i bt_area(i, sc_i) |rho_u_0 n_x + rho_v_0 n_y|."""
    st = s.get_state()
    c, m = s._cs, s.case.mesh
    nchi, neta = s.nchi, s.neta
    rho = np.asarray(st["q"]).reshape(4, -1)[0].reshape(nchi + 2, neta + 2, order="F")[1:-1, 1:-1]
    ci = st["cell_idx"]
    flow = (np.arange(1, neta + 1)[None, :] < ci[:, None]).astype(float)
    mass = float(np.sum(rho * flow * np.asarray(m["vol"])))
    i = np.arange(nchi)
    j = ci - 1
    flux = np.abs(c.rho_u_0 * np.asarray(m["bt_xn"])[i, j] + c.rho_v_0 * np.asarray(m["bt_yn"])[i, j])
    return mass / float(np.sum(np.asarray(m["bt_a"])[i, j] * flux))


def freestream_blocks(s: Solution) -> np.ndarray:
    """R_infty (CONSTRUCT_R_.jl:59-142): the 4 x 4 map from the conserved freestream
    perturbation to (p, u, v, S) at the uniform freestream state."""
    c = s._cs
    g = c.gamma
    rho, u, v, p = c.rho_0, c.rho_u_0 / c.rho_0, c.rho_v_0 / c.rho_0, c.p_0
    return np.array([
        [(g - 1) * (u**2 + v**2) / 2, -u * (g - 1), -v * (g - 1), g - 1],
        [-u / rho, 1 / rho, 0, 0],
        [-v / rho, 0, 1 / rho, 0],
        [(u**2 + v**2) / (2 * p) - g / (g - 1) / rho, -u / p, -v / p, 1 / p]])


def freestream_weights(s: Solution, w_infty, norms=(1, 1, 1, 1)) -> np.ndarray:
    """The freestream blocks of D = R_' M_infty_ R_ (CONSTRUCT_M_INFTY_.jl:31-52 and
    :63-160 with scaling_non_temporal, i.e. scaled by GET_T_REF): per frequency k and
    column i, R_inf' diag(m) R_inf with the Chu weights of the freestream times the
    column's shock arc length bt_area |n . V_inf / |V_inf||, halved for w_k != 0.
    Returns (Nw, Nchi, 4, 4)."""
    c, m = s._cs, s.case.mesh
    g, rho, p = c.gamma, c.rho_0, c.p_0
    a = s.case.fs["a_0"]
    ci = s.get_state()["cell_idx"]
    i, j = np.arange(s.nchi), ci - 1
    vm = np.hypot(c.rho_u_0, c.rho_v_0)
    proj = np.asarray(m["bt_xn"])[i, j] * (c.rho_u_0 / vm) + np.asarray(m["bt_yn"])[i, j] * (c.rho_v_0 / vm)
    arc = np.asarray(m["bt_a"])[i, j] * np.abs(proj)
    wv = np.array([rho * a**2 / (2 * (g * p) ** 2), rho / 2, rho / 2, (g - 1) * p / (2 * g)]) * np.asarray(norms)
    Rinf = freestream_blocks(s)
    T_ref = GET_T_REF(s)
    out = np.empty((len(w_infty), s.nchi, 4, 4))
    for k, w in enumerate(w_infty):
        f = 1.0 if w == 0 else 0.5
        mw = wv[None, :] * arc[:, None] * T_ref * f                    # (Nchi, 4)
        out[k] = np.einsum("vi,nv,vj->nij", Rinf, mw, Rinf)
    return out


class ReceptivityOperator:
    """L_ of LINEARIZE_L_ on the device for the frequencies w_infty: ``apply`` and ``expm``
    on complex host vectors of n = hymor_recept_size unknowns [q; r; u_1; ...; u_Nw]."""

    def __init__(self, L: LinearOperatorGPU, s: Solution, w_infty):
        self.L, self.s = L, s
        self.w = np.ascontiguousarray(w_infty, dtype=np.float64)
        n = ctypes.c_int64()
        s.ctx.check(s.ctx.L.hymor_recept_size(s.ctx.h, len(self.w), ctypes.byref(n)))
        self.n = n.value
        self.n_down = 4 * s.N

    def _run(self, fn, x, *args):
        X = np.asarray(x, dtype=complex).reshape(self.n, -1)
        k = X.shape[1]
        buf = np.empty((k, 2, self.n))
        buf[:, 0], buf[:, 1] = X.real.T, X.imag.T
        bx, by = DeviceBuffer(self.s.ctx, buf.nbytes), DeviceBuffer(self.s.ctx, buf.nbytes)
        try:
            bx.upload(buf.ravel())
            fn(k, bx.ptr, by.ptr, *args)
            out = by.download(buf.size).reshape(k, 2, self.n)
        finally:
            bx.free()
            by.free()
        Y = (out[:, 0] + 1j * out[:, 1]).T
        return Y[:, 0] if np.ndim(x) == 1 else Y

    def apply(self, x, adjoint: bool = False, scale: float = 1.0):
        """scale L_ x, or scale L_^H x."""
        c = self.s.ctx

        def fn(k, src, dst):
            c.check(c.L.hymor_recept_apply_dev(c.h, k, len(self.w), dp(self.w), float(scale), src, dst,
                                               int(adjoint)))
        return self._run(fn, x)

    def expm(self, x, dt: float, nsteps: int, adjoint: bool = False, order: int = 5):
        """EXPONENTIAL!'s Taylor propagation of x by nsteps steps of L_ dt (or L_^H dt)."""
        c = self.s.ctx

        def fn(k, src, dst):
            c.check(c.L.hymor_recept_expm_dev(c.h, k, len(self.w), dp(self.w), float(dt), int(nsteps), int(order),
                                              src, dst, int(adjoint)))
        return self._run(fn, x)


def LINEARIZE_B(s: Solution):
    """LINEARIZE_B (LINEARIZE_B.jl:40-296) on the device; returns (rows, bq, bs) as
    hymor_b_get lays them out: bq (Nchi, 3, 4, 4), bs (Nchi, 3, 4)."""
    s.ctx.check(s.ctx.L.hymor_linearize_b(s.ctx.h))
    n = s.nchi
    rows = np.empty(n, dtype=np.int32)
    bq, bs = np.empty(48 * n), np.empty(12 * n)
    s.ctx.check(s.ctx.L.hymor_b_get(s.ctx.h, ip(rows), dp(bq), dp(bs)))
    return rows, bq.reshape(n, 3, 4, 4), bs.reshape(n, 3, 4)


def CHECK_LINEARIZATION_B(B, s: Solution, seed: int | None = None, verbose: bool = True) -> float:
    """CHECK_LINEARIZATION_B (CHECK_LINEARIZATION_B.jl:20-89): B q against the change of the
    masked residual (and of the shock speeds with the shock unknowns) when the per-column
    upstream state moves by q = perturbation_magnitude * randn, both residuals on copies of
    `s` with a prescribed upstream state. B = (rows, bq, bs) of LINEARIZE_B. Returns (and
    prints) the reference's measure ||(B q - dq) / (|B q| + 1e-8)|| / sqrt(48 Nchi)."""
    rows, bq, bs = B
    c, nchi, N = s._cs, s.nchi, s.N
    eps = c.perturbation_magnitude
    rng = np.random.default_rng(seed)
    P = eps * rng.standard_normal((4, nchi))
    fs = np.array([c.rho_0, c.rho_u_0, c.rho_v_0, c.rho_E_0])
    cols0 = np.ascontiguousarray(np.repeat(fs[:, None], nchi, axis=1))
    st = s.get_state()
    pts = (st["pts_x"], st["pts_y"], st["pts_chi"], st["pts_eta"])
    shock_rows = s.operator_size() > 4 * N
    out = []
    for cols in (cols0, np.ascontiguousarray(cols0 + P)):
        x = Solution(s.case)
        try:
            x.set_state(np.asarray(st["q"]), *pts, st["cell_idx"], st["t"])
            x.ctx.check(x.ctx.L.hymor_set_upstream(x.ctx.h, dp(cols.ravel())))
            from .solver import PDE
            out.append((PDE(x), x.shock_fields()[1]))
        finally:
            x.close()
    flow = np.tile((np.arange(1, s.neta + 1)[None, :] < st["cell_idx"][:, None]).ravel(order="F"), 4)
    dq = (out[1][0] - out[0][0]) * flow
    Bq = np.zeros(4 * N)
    Bs = np.zeros(nchi)
    for m in range(nchi):
        cell = m + (rows[m] - 2) * nchi
        for d in (-1, 0, 1):
            n = m + d
            if 0 <= n < nchi:
                Bq[np.arange(4) * N + cell] += bq[m, d + 1] @ P[:, n]
                Bs[m] += bs[m, d + 1] @ P[:, n]
    if shock_rows:
        dq = np.concatenate([dq, out[1][1] - out[0][1]])
        Bq = np.concatenate([Bq, Bs])
    err = float(np.linalg.norm((Bq - dq) / (np.abs(Bq) + 1e-8)) / np.sqrt(3 * 4 * 4 * nchi))
    if verbose:
        print(f"Error of linearization: {err:e} .")
    return err


def LINEARIZE_L_(L: LinearOperatorGPU, s: Solution, w_infty):
    """LINEARIZE_L_ (LINEARIZE_L_.jl:36-71): B on the device and the extended operator L_
    for the frequencies w_infty. Call after LINEARIZE_L. Returns (s, L_)."""
    s.ctx.check(s.ctx.L.hymor_linearize_b(s.ctx.h))
    return s, ReceptivityOperator(L, s, w_infty)


class _ReceptivityProblem:
    """The reduced receptivity operator of one case, y -> K^-1 Z P^H R'MR P Z K^-H y on the
    real form of the free unknowns (FREESTREAM_RECEPTIVITY.jl:80-116), split into the host
    step that stages the input (begin), the device propagations, which it only enqueues on
    the case's stream (launch), and the host step that reads the result (end)."""

    def __init__(self, L_: ReceptivityOperator, s: Solution, T: float, order: int):
        dt_cfl = CFL_TIMESTEP(s)
        self.n_t = int(round(T / dt_cfl))
        self.dt = T / self.n_t
        self.L_, self.s, self.order = L_, s, order
        self.n, self.n4 = L_.n, L_.n_down
        self.nr = L_.L.n - self.n4                # shock displacements (0 without the shock unknowns)
        self.nw, self.p = len(L_.w), 4 * s.nchi
        # D on the free unknowns: the shock tail, then per frequency and column a 4 x 4 block
        ci = s.get_state()["cell_idx"]
        d_r = np.asarray(s.case.mesh["bt_a"])[np.arange(s.nchi), ci - 1] / 2 if self.nr else np.zeros(0)
        Dk = freestream_weights(s, L_.w)                               # (Nw, Nchi, 4, 4)
        self.Kinv = np.linalg.inv(np.linalg.cholesky(Dk))
        self.kr = 1 / np.sqrt(d_r)
        self.nf = self.nr + self.nw * self.p      # free unknowns (complex)
        C0, _ = chu_blocks(s)
        self.bC0 = DeviceBuffer(s.ctx, 8 * s.N * 16)
        self.bC0.upload(np.ascontiguousarray(C0.reshape(-1)))
        self.tail0 = DeviceBuffer(s.ctx, 8 * (self.n - self.n4))
        self.tail0.upload(np.zeros(self.n - self.n4))
        self.bz = [DeviceBuffer(s.ctx, 8 * 2 * self.n) for _ in range(2)]
        self.count = 0

    def k_inv_t(self, y):   # x = K^-H y on the free unknowns (K real)
        x = np.empty_like(y)
        nr = self.nr
        x[:nr] = self.kr * y[:nr]
        U = y[nr:].reshape(self.nw, 4, self.s.nchi)
        x[nr:] = np.einsum("knji,kjn->kin", self.Kinv, U).reshape(-1)
        return x

    def k_inv(self, y):     # K^-1 y
        x = np.empty_like(y)
        nr = self.nr
        x[:nr] = self.kr * y[:nr]
        U = y[nr:].reshape(self.nw, 4, self.s.nchi)
        x[nr:] = np.einsum("knij,kjn->kin", self.Kinv, U).reshape(-1)
        return x

    def begin(self, src):
        c = self.s.ctx
        self.count += 1
        y = np.empty(2 * self.nf)
        c.check(c.L.hymor_memcpy_d2h(c.h, y.ctypes.data, src, y.nbytes))
        x = self.k_inv_t(y[:self.nf] + 1j * y[self.nf:])
        z = np.zeros((2, self.n))
        z[0, self.n4:], z[1, self.n4:] = x.real, x.imag
        self.bz[0].upload(z.ravel())

    def launch(self):
        """Enqueues P, R'MR and P^H on the case's stream (returns before they run)."""
        c, w, n, n4 = self.s.ctx, self.L_.w, self.n, self.n4
        nw, dt, n_t, order = len(w), self.dt, self.n_t, self.order
        c.check(c.L.hymor_recept_expm_dev(c.h, 1, nw, dp(w), dt, n_t, order, self.bz[0].ptr, self.bz[1].ptr, 0))
        c.check(c.L.hymor_block4_apply_ext_dev(c.h, 2, n - n4, self.bC0.ptr, self.tail0.ptr, self.bz[1].ptr,
                                               self.bz[0].ptr))
        c.check(c.L.hymor_recept_expm_dev(c.h, 1, nw, dp(w), dt, n_t, order, self.bz[0].ptr, self.bz[1].ptr, 1))

    def end(self, dst):
        c, n, n4 = self.s.ctx, self.n, self.n4
        out = self.bz[1].download(2 * n).reshape(2, n)
        r = self.k_inv(out[0, n4:] + 1j * out[1, n4:])
        res = np.concatenate([r.real, r.imag])
        c.check(c.L.hymor_memcpy_h2d(c.h, dst, res.ctypes.data, res.nbytes))

    def modes(self, Y, n_modes):
        V = np.zeros((self.n, n_modes), dtype=complex)
        for m_ in range(n_modes):
            V[self.n4:, m_] = self.k_inv_t(Y[:self.nf, m_] + 1j * Y[self.nf:, m_])
        return V

    def free(self):
        for b in [self.bC0, self.tail0] + self.bz:
            b.free()


def FREESTREAM_RECEPTIVITY(L_: ReceptivityOperator, s: Solution, n_modes: int, T: float, ncv: int | None = None,
                           tol: float = 1e-8, order: int = 5, seed: int = 5, maxit: int = 300,
                           modes: bool = False, keep_unconverged: bool = False):
    """FREESTREAM_RECEPTIVITY (FREESTREAM_RECEPTIVITY.jl:37-162): the n_modes largest gains
    G of Z P^H R'MR P Z x = G D x over the horizon T_opt = n_t dt (dt = T / round(T /
    dt_CFL)), P the Taylor propagation of L_ (EXPONENTIAL!). The initial condition carries
    no downstream cells (Z); its unknowns are the shock displacements (with the shock
    unknowns, D = bt_area / 2 there) and the freestream blocks (D = R_inf' M_infty R_inf,
    halved for w != 0). The problem is reduced with the block Cholesky factor K of D and
    solved by the device Krylov-Schur on the real form (real and imaginary parts) of the
    reduced complex Hermitian operator, which has the same eigenvalues; as the reference,
    the gains are the eigenvalues / 2 (FREESTREAM_RECEPTIVITY.jl:113-116).

    Returns (V, D, T_opt) like the reference: V the modes (n x n_modes complex, with modes
    True, else None), D the gains; NaN with a warning when tol is not reached (:136-140),
    unless keep_unconverged."""
    import time
    import warnings
    pb = _ReceptivityProblem(L_, s, T, order)

    def apply_op(src, dst):
        pb.begin(src)
        pb.launch()
        pb.end(dst)
    ncv = ncv or max(2 * n_modes + 1, 16)
    t0 = time.perf_counter()
    try:
        lam, resid, nops, Y = krylov_schur(s.ctx, 2 * pb.nf, apply_op, n_modes, ncv, tol=tol, maxit=maxit,
                                           seed=seed, symmetric=True, want_vectors=True)
        elapsed = time.perf_counter() - t0
        lam = np.real(lam)
        converged = bool(np.all(resid <= tol * np.abs(lam)))
        gains = lam / 2
        V = pb.modes(Y, n_modes) if (modes and Y is not None) else None
    finally:
        pb.free()
    if not converged and not keep_unconverged:
        warnings.warn(f"receptivity solve did not reach tol {tol:g} in {maxit} restarts; returning NaN")
        gains = np.full(n_modes, np.nan)
        V = np.full((pb.n, n_modes), np.nan + 0j) if modes else None
    info = dict(resid=resid, dt=pb.dt, n_t=pb.n_t, nops=nops, seconds=elapsed, converged=converged,
                applications=pb.count)
    return V, gains, pb.n_t * pb.dt, info


def FREESTREAM_RECEPTIVITY_BATCH(cases, n_modes: int, T: float, ncv: int | None = None, tol: float = 1e-8,
                                 order: int = 5, seed: int = 5, maxit: int = 300, keep_unconverged: bool = False):
    """FREESTREAM_RECEPTIVITY for several cases at once: cases = [(L_, s), ...], each its own
    context and grid (sizes may differ), each L_ with its own frequencies. One Krylov-Schur
    solve per case in lockstep (each makes the operations of its own FREESTREAM_RECEPTIVITY
    with the same seed, so the gains are the same): every round stages each unfinished case's
    vector, then enqueues all their propagations before waiting for any, so the cases'
    propagations run concurrently on their streams, then reads the results. The reference
    solves one case per FREESTREAM_RECEPTIVITY call. Returns [(gains, info)] per case (info
    seconds: the whole batched solve)."""
    import time
    import warnings
    from .krylov import krylov_schur_steps
    probs = [_ReceptivityProblem(L_, s, T, order) for (L_, s) in cases]
    ncv = ncv or max(2 * n_modes + 1, 16)
    gens = [krylov_schur_steps(s.ctx, 2 * pb.nf, n_modes, ncv, tol, maxit, seed, True, None, False)
            for pb, (_, s) in zip(probs, cases)]
    results: list = [None] * len(gens)
    pending = {}
    t0 = time.perf_counter()
    try:
        for i, g in enumerate(gens):
            try:
                pending[i] = next(g)
            except StopIteration as done:
                results[i] = done.value
        while pending:
            idx = sorted(pending)
            for i in idx:
                probs[i].begin(pending[i][0])
            for i in idx:
                probs[i].launch()
            for i in idx:
                probs[i].end(pending[i][1])
            for i in idx:
                try:
                    pending[i] = gens[i].send(None)
                except StopIteration as done:
                    results[i] = done.value
                    del pending[i]
        elapsed = time.perf_counter() - t0
    finally:
        for pb in probs:
            pb.free()
    out = []
    for pb, res in zip(probs, results):
        lam, resid, nops = res
        lam = np.real(lam)
        converged = bool(np.all(resid <= tol * np.abs(lam)))
        gains = lam / 2
        if not converged and not keep_unconverged:
            warnings.warn(f"receptivity solve did not reach tol {tol:g}; its gains are NaN")
            gains = np.full(n_modes, np.nan)
        out.append((gains, dict(resid=resid, dt=pb.dt, n_t=pb.n_t, nops=nops, seconds=elapsed, converged=converged,
                                applications=pb.count)))
    return out
