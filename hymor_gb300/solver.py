"""Reference-shaped host API over libhymor.

The reference drives its hot path through Julia functions on a solution Dict
(utils/Operators/PDE.jl:1, utils/Time_marching/ADVECT_FLOW.jl:30,
utils/Stability_analysis/Modal_stability_analysis/LINEARIZE_L.jl:34, ...). This
module keeps those names and argument meanings: a :class:`Solution` plays the
Dict (its arrays live on the GPU), and the functions mutate it in place and
return it, exactly as the reference mutates and returns `s`.

Every hot-path call goes through the C ABI (include/hymor.h). The host side only
assembles small set-up data, as the reference's host code does: the Chu-norm weight
blocks of transient growth and the projected Krylov matrices (<= ncv x ncv).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .case import Case, config_struct
from ._lib import HymorError, dp, ip


class Solution:
    """A solution Dict resident on one GPU (one libhymor context)."""

    def __init__(self, case: Case):
        self.case = case
        self.cfg = case.cfg
        self.nchi, self.neta = case.cfg.nchi, case.cfg.neta
        self._cs = config_struct(case.cfg)
        self._ms, self._keep = case.mesh_struct()
        self.ctx = _lib.Context(self._cs, self._ms)
        self.set_state(case.q_flat(), case.pts_x, case.pts_y, case.pts_chi, case.pts_eta,
                       case.cell_idx, case.t, case.a)

    # -- sizes
    @property
    def G(self) -> int:
        return (self.nchi + 2) * (self.neta + 2)

    @property
    def N(self) -> int:
        return self.nchi * self.neta

    # -- state transfer
    def set_state(self, qflat, px, py, pchi, peta, cell_idx, t, a=None):
        qflat = np.ascontiguousarray(qflat, dtype=np.float64)
        if qflat.size != 4 * self.G:
            raise HymorError(-1, f"state has {qflat.size} values, expected 4 x {self.G}")
        arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in (px, py, pchi, peta)]
        ci = np.ascontiguousarray(cell_idx, dtype=np.int32)
        aa = None if a is None else np.asfortranarray(a, dtype=np.float64)
        self.ctx.check(self.ctx.L.hymor_set_state(
            self.ctx.h, dp(qflat), *[dp(v) for v in arrs], ip(ci), float(t),
            dp(aa) if aa is not None else None))

    def get_state(self) -> dict:
        q = np.empty(4 * self.G)
        px, py, pc, pe = (np.empty(self.nchi) for _ in range(4))
        ci = np.empty(self.nchi, dtype=np.int32)
        t, dt = ctypes.c_double(), ctypes.c_double()
        self.ctx.check(self.ctx.L.hymor_get_state(self.ctx.h, dp(q), dp(px), dp(py), dp(pc), dp(pe),
                                                  ip(ci), ctypes.byref(t), ctypes.byref(dt)))
        return dict(q=q, pts_x=px, pts_y=py, pts_chi=pc, pts_eta=pe, cell_idx=ci, t=t.value,
                    dt=dt.value)

    def advect_host(self, q, px, py, pchi, peta, cell_idx, t: float, nsteps: int) -> float:
        """ADVECT_FLOW of a host-resident state in one call (hymor_advect): the arrays are
        uploaded, advanced `nsteps` steps and overwritten with the result; returns t."""
        arrs = (q, px, py, pchi, peta)
        for v in arrs:
            if v.dtype != np.float64 or not v.flags.c_contiguous:
                raise HymorError(-1, "advect_host needs contiguous float64 arrays (updated in place)")
        if cell_idx.dtype != np.int32 or not cell_idx.flags.c_contiguous:
            raise HymorError(-1, "advect_host needs contiguous int32 cell indices (updated in place)")
        tt = ctypes.c_double(t)
        self.ctx.check(self.ctx.L.hymor_advect(self.ctx.h, int(nsteps), *[dp(v) for v in arrs], ip(cell_idx),
                                               ctypes.byref(tt)))
        return tt.value

    def var(self) -> dict:
        """s["var"]: the four ghosted conserved arrays, (Nchi+2, Neta+2) column-major."""
        q = self.get_state()["q"].reshape(4, -1)
        shape = (self.nchi + 2, self.neta + 2)
        return {k: q[v].reshape(shape, order="F") for v, k in enumerate(("rho", "rho_u", "rho_v", "rho_E"))}

    def counters(self) -> tuple[int, int]:
        a, b = ctypes.c_int32(), ctypes.c_int32()
        self.ctx.check(self.ctx.L.hymor_counters(self.ctx.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def shock_fields(self) -> tuple[np.ndarray, np.ndarray]:
        """(s["shock"]["beta"] of the last shock update of the solution, the relative shock
        speeds of the last shock update), Nchi each."""
        beta, rel = np.empty(self.nchi), np.empty(self.nchi)
        self.ctx.check(self.ctx.L.hymor_shock_fields(self.ctx.h, dp(beta), dp(rel)))
        return beta, rel

    def operator_size(self) -> int:
        """Unknowns of the linearised operator: 4 Nchi Neta, plus Nchi with the shock-position
        blocks (perturb_shock)."""
        n = ctypes.c_int64()
        self.ctx.check(self.ctx.L.hymor_operator_size(self.ctx.h, ctypes.byref(n)))
        return n.value

    def set_step_viscous(self, mode: int):
        """Arithmetic of the viscous terms in the RK step's flux: 1 float-float (default),
        0 FP64 (hymor_set_step_viscous). PDE and the Jacobian always use FP64."""
        self.ctx.check(self.ctx.L.hymor_set_step_viscous(self.ctx.h, int(mode)))

    def set_cfl_screen(self, on: int):
        """Reduction of the RK step's CFL maxima: 1 through the exact FP32 screen (default),
        0 FP64 over every cell (hymor_set_cfl_screen); dt is the same bit for bit."""
        self.ctx.check(self.ctx.L.hymor_set_cfl_screen(self.ctx.h, int(on)))

    def set_expm_arith(self, mode: int):
        """Arithmetic of the cooperative Taylor propagator's matvecs: 1 float-float on the
        FP32 pipe (default), 0 FP64 (hymor_set_expm_arith)."""
        self.ctx.check(self.ctx.L.hymor_set_expm_arith(self.ctx.h, int(mode)))

    def step_kernels(self) -> int:
        """Kernel launches one ADVECT_FLOW step makes (the kernel nodes of its graph)."""
        n = ctypes.c_int32()
        self.ctx.check(self.ctx.L.hymor_step_kernels(self.ctx.h, ctypes.byref(n)))
        return n.value

    def close(self):
        self.ctx.close()


# ---------------------------------------------------------------------------
# Reference entry points


def PDE(s: Solution, flux_out: np.ndarray | None = None) -> np.ndarray:
    """NON_LINEAR_DYNAMICS_NO_DISCONTINUITY / PDE (utils/Operators/PDE.jl:1-47): the
    residual of `s`, flux = 4 x Nchi*Neta ([rho; rho_u; rho_v; rho_E], chi fastest).
    Mutates `s` (ghost cells, shocked cells, shock points) like the reference."""
    f = flux_out if flux_out is not None else np.empty(4 * s.N)
    s.ctx.check(s.ctx.L.hymor_residual(s.ctx.h, dp(f)))
    return f


NON_LINEAR_DYNAMICS_NO_DISCONTINUITY = PDE


def ADVECT_FLOW(s: Solution, nsteps: int = 1) -> Solution:
    """ADVECT_FLOW (utils/Time_marching/ADVECT_FLOW.jl:30-39), explicit RK4, `nsteps` times."""
    s.ctx.check(s.ctx.L.hymor_step(s.ctx.h, int(nsteps)))
    return s


def RUN_SIMULATION(s: Solution, N_iter: int) -> Solution:
    """RUN_SIMULATION's time loop (utils/Time_marching/RUN_SIMULATION.jl:77-80), without
    plotting and remeshing."""
    return ADVECT_FLOW(s, N_iter)


def RESIDUAL(s: Solution, q_save: np.ndarray, cell_idx: np.ndarray | None = None) -> np.ndarray:
    """RESIDUAL of the MATLAB twin (utils/Time_marching/ADVECT_FLOW_EXPLICIT.m:92-110): per
    conserved variable, rms of the change since q_save over the flow cells divided by the rms
    of the variable there (interior cells; flow cells j < cell_idx[i] with shock fitting).
    q_save is a state as Solution.get_state()["q"] returns it."""
    st = s.get_state()
    shape = (s.nchi + 2, s.neta + 2)
    qa = st["q"].reshape(4, -1)
    qb = np.asarray(q_save).reshape(4, -1)
    ci = st["cell_idx"] if cell_idx is None else cell_idx
    if s.cfg.shock_enabled:
        mask = (np.arange(1, s.neta + 1)[None, :] < np.asarray(ci)[:, None])
    else:
        mask = np.ones((s.nchi, s.neta), dtype=bool)
    out = np.empty(4)
    for v in range(4):
        a = qa[v].reshape(shape, order="F")[1:-1, 1:-1][mask]
        b = qb[v].reshape(shape, order="F")[1:-1, 1:-1][mask]
        out[v] = np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(a**2))
    return out


def MARCH_TO_RESIDUAL(s: Solution, tol: float = 1e-10, max_steps: int = 10**7, check_every: int = 2000,
                      max_seconds: float | None = None, log=None) -> dict:
    """RUN_SIMULATION's time loop (RUN_SIMULATION.jl:77-80) until the step residual of the
    MATLAB twin (RESIDUAL, max over the four variables) falls below tol. The residual of
    one step is measured every check_every steps; the march stops at tol, at max_steps or
    after max_seconds of wall time. Returns the step count, the last residual and the
    history [(step, t, residual)]."""
    import time
    t0 = time.perf_counter()
    steps, hist = 0, []
    res = np.full(4, np.inf)
    while steps < max_steps:
        q_save = s.get_state()["q"]
        ADVECT_FLOW(s, 1)
        steps += 1
        res = RESIDUAL(s, q_save)
        st_t = s.get_state()["t"]
        hist.append((steps, st_t, float(np.max(res))))
        if log:
            log(f"step {steps} t {st_t:.4f} residual {np.max(res):.3e} ({time.perf_counter() - t0:.0f} s)")
        if np.max(res) < tol:
            break
        if max_seconds is not None and time.perf_counter() - t0 > max_seconds:
            break
        n = min(check_every - 1, max_steps - steps)
        if n > 0:
            ADVECT_FLOW(s, n)
            steps += n
    return dict(steps=steps, residual=res, converged=bool(np.max(res) < tol), history=hist,
                seconds=time.perf_counter() - t0)


def UPDATE_FLOW_CELLS(s: Solution) -> Solution:
    s.ctx.check(s.ctx.L.hymor_update_flow_cells(s.ctx.h))
    return s


def CFL_TIMESTEP(s: Solution) -> float:
    dt = ctypes.c_double()
    s.ctx.check(s.ctx.L.hymor_cfl_timestep(s.ctx.h, ctypes.byref(dt)))
    return dt.value


class LinearOperatorGPU:
    """The linearised operator L (a Nchi*Neta*144 stencil-block Jacobian on the GPU, plus the
    shock-position blocks when linearised with perturb_shock).

    Stands in for the reference's SparseMatrixCSC `L` of LINEARIZE_L: ``L @ x``,
    ``L.T @ x`` and the Taylor propagator act on n-vectors (or n x k blocks), n = 4N, or
    4N + Nchi with the shock unknowns (the reference's 4*Nchi*Neta + Nchi)."""

    def __init__(self, s: Solution, transpose: bool = False):
        self.s = s
        self.n = s.operator_size()
        self.shape = (self.n, self.n)
        self.dtype = np.float64
        self._t = transpose

    @property
    def T(self):
        return LinearOperatorGPU(self.s, not self._t)

    def _block(self, x):
        x = np.asarray(x, dtype=np.float64)
        vec = x.ndim == 1
        X = np.asfortranarray(x.reshape(self.n, -1))
        return X, vec

    def __matmul__(self, x):
        X, vec = self._block(x)
        k = X.shape[1]
        Y = np.empty((self.n, k), order="F")
        self.s.ctx.check(self.s.ctx.L.hymor_matvec(self.s.ctx.h, k, dp(X), dp(Y), int(self._t)))
        return Y[:, 0] if vec else Y

    matvec = __matmul__

    def expm(self, x, dt: float, nsteps: int, order: int = 5):
        """(Σ_{j<=order} (L dt)^j / j!)^nsteps x (POWER_METHOD!, ARNOLDI_POWER_GPU.jl:64-82)."""
        X, vec = self._block(x)
        k = X.shape[1]
        Y = np.empty((self.n, k), order="F")
        self.s.ctx.check(self.s.ctx.L.hymor_expm_apply(self.s.ctx.h, k, float(dt), int(nsteps), int(order),
                                                       dp(X), dp(Y), int(self._t)))
        return Y[:, 0] if vec else Y

    def blocks(self) -> np.ndarray:
        c = np.empty(self.s.N * 144)
        self.s.ctx.check(self.s.ctx.L.hymor_jacobian_get(self.s.ctx.h, dp(c)))
        return c

    def set_blocks(self, coef: np.ndarray):
        coef = np.ascontiguousarray(coef, dtype=np.float64)
        self.s.ctx.check(self.s.ctx.L.hymor_jacobian_set(self.s.ctx.h, dp(coef)))

    def shock_blocks(self):
        """(rows, a21, a12, a22) of the shock-position unknowns (include/hymor.h layouts:
        Nchi; Nchi x 8; 4 Nchi x Nchi; Nchi x Nchi)."""
        n = self.s.nchi
        rows = np.empty(n, dtype=np.int32)
        a21, a12, a22 = np.empty((n, 8)), np.empty((4 * n, n)), np.empty((n, n))
        self.s.ctx.check(self.s.ctx.L.hymor_shock_blocks_get(self.s.ctx.h, ip(rows), dp(a21), dp(a12), dp(a22)))
        return rows, a21, a12, a22

    def set_shock_blocks(self, blocks):
        """Sets the shock-position blocks (None turns the shock unknowns off)."""
        L, h = self.s.ctx.L, self.s.ctx.h
        if blocks is None:
            self.s.ctx.check(L.hymor_shock_blocks_set(h, None, None, None, None))
        else:
            rows, a21, a12, a22 = blocks
            rows = np.ascontiguousarray(rows, dtype=np.int32)
            a21, a12, a22 = (np.ascontiguousarray(b, dtype=np.float64) for b in (a21, a12, a22))
            self.s.ctx.check(L.hymor_shock_blocks_set(h, ip(rows), dp(a21), dp(a12), dp(a22)))
        self.n = self.s.operator_size()


def LINEARIZE_L(s: Solution):
    """LINEARIZE_L (LINEARIZE_L.jl:34-69): coloured finite-difference Jacobian of the
    residual, assembled on the GPU. Returns (s, L)."""
    s.ctx.check(s.ctx.L.hymor_linearize(s.ctx.h))
    return s, LinearOperatorGPU(s)


# ---------------------------------------------------------------------------
# Stability drivers over the device-resident Krylov solver


def CHECK_LINEARIZATION_L(L: LinearOperatorGPU, s: Solution, seed: int | None = None, verbose: bool = True) -> float:
    """CHECK_LINEARIZATION_L (Modal_stability_analysis/CHECK_LINEARIZATION_L.jl:33-130):
    the linearised response L q against the finite difference f(x + q) - f(x) of the
    nonlinear residual, for a random perturbation q of every conserved variable (scaled by
    perturbation_magnitude, masked by the flow cells like the reference), both residuals on
    copies of `s`; with the shock unknowns the shock points move too and the shock speeds
    are compared as well. Returns (and prints) the reference's error measure
    ||(L q - dq) / (|L q| + 1e-8)|| / sqrt(144 N); below ~1e-3 means consistent."""
    cfg, N = s.cfg, s.N
    nchi, neta = cfg.nchi, cfg.neta
    eps = cfg.perturbation_magnitude
    st = s.get_state()
    rng = np.random.default_rng(seed)
    shock = bool(cfg.shock_enabled)
    flow = ((np.arange(1, neta + 1)[None, :] < st["cell_idx"][:, None]).astype(np.float64)
            if shock else np.ones((nchi, neta)))  # (nchi, neta), chi fastest when raveled "F"
    q = np.zeros(4 * N)
    qs = np.asarray(st["q"], dtype=np.float64).reshape(4, -1).copy()
    for v in range(4):
        P = rng.standard_normal((nchi, neta))
        dv = (flow * P if shock else P) * eps
        blk = qs[v].reshape(nchi + 2, neta + 2, order="F")
        blk[1:-1, 1:-1] += dv
        qs[v] = blk.ravel(order="F")
        # the reference masks q for rho only (:52-96); the masked Jacobian ignores the rest
        q[v * N:(v + 1) * N] = (dv if v == 0 else P * eps).ravel(order="F")
    pts = (st["pts_x"], st["pts_y"], st["pts_chi"], st["pts_eta"])
    pts_p = pts
    shock_unknowns = L.n > 4 * N
    if shock_unknowns:
        # the shock points move along PERTURB_SHOCK's direction by eps * randn (:92-100)
        vp = rng.standard_normal(nchi)
        beta, _ = s.shock_fields()
        ang = beta - np.pi / 2 - np.arctan2(s._cs.rho_v_0, s._cs.rho_u_0)
        pts_p = (st["pts_x"] + eps * np.cos(ang) * vp, st["pts_y"] + eps * np.sin(ang) * vp,
                 st["pts_chi"], st["pts_eta"])
        q = np.concatenate([q, eps * vp])
    base, pert = Solution(s.case), Solution(s.case)
    try:
        base.set_state(np.asarray(st["q"]), *pts, st["cell_idx"], st["t"])
        pert.set_state(qs.ravel(), *pts_p, st["cell_idx"], st["t"])
        f0, f1 = PDE(base), PDE(pert)
        mask = np.tile(flow.ravel(order="F"), 4) if shock else 1.0
        dq = (f1 - f0) * mask
        if shock_unknowns:
            dq = np.concatenate([dq, pert.shock_fields()[1] - base.shock_fields()[1]])
    finally:
        base.close()
        pert.close()
    dq_lin = L @ q
    err = float(np.linalg.norm((dq_lin - dq) / (np.abs(dq_lin) + 1e-8)) / np.sqrt(9 * 4 * 4 * N))
    if verbose:
        print(f"Error of linearization: {err:e} .")
    return err


def _expm_op(s: Solution, dt: float, nsteps: int, order: int, transpose: int = 0):
    L, h = s.ctx.L, s.ctx.h

    def apply(src, dst):
        s.ctx.check(L.hymor_expm_apply_dev(h, 1, float(dt), int(nsteps), int(order), src, dst, int(transpose)))
    return apply


def _expm_block_op(s: Solution, dt: float, nsteps: int, order: int, transpose: int = 0):
    """The propagator over k contiguous device vectors in one batched call."""
    L, h = s.ctx.L, s.ctx.h

    def apply(src, dst, k):
        s.ctx.check(L.hymor_expm_apply_dev(h, int(k), float(dt), int(nsteps), int(order), src, dst, int(transpose)))
    return apply


def _krylov_opts(nev: int, ncv: int, tol: float, maxit: int, block: int, order: int, seed: int = 0,
                 flow_start: bool = False):
    o = _lib.KrylovOpts()
    o.nev, o.ncv, o.maxit, o.block, o.order = int(nev), int(ncv), int(maxit), int(block), int(order)
    o.flow_start, o.seed, o.tol = int(flow_start), int(seed), float(tol)
    return o


def EIGENVALUES(L: LinearOperatorGPU, s: Solution, n_modes: int, T_ref: float = 0.5, ncv: int | None = None,
                tol: float = 1e-8, order: int = 5, method: str = "device", seed: int = 3, maxit: int = 300,
                block: int = 1, flow_start: bool = False, modes: bool = False, keep_unconverged: bool = False):
    """EIGENVALUES_GPU_ARNOLDI (Eigenvalues/EIGENVALUES.jl:112-205): the n_modes eigenvalues of
    largest magnitude of exp(L T_ref) (Taylor-`order` steps of the CFL dt), mapped back as
    lambda = log(mu) / (dt * timesteps).

    modes: also the eigenvectors (info["modes"], n x n_modes, complex, unit norm; the
    reference's V). When the solve does not reach tol, the reference warns and returns NaN
    (EIGENVALUES.jl:184-204); so does this, unless keep_unconverged, which returns the last
    Ritz values (and no modes) with info["converged"] False.

    method "device": hymor_eigs, the Krylov-Schur solver behind the C ABI (basis in HBM;
                     block > 1: `block` vectors propagated per batched call).
    method "python": the same Krylov-Schur restart driven from Python (hymor_gb300/krylov.py)
                     over the device building blocks, with LAPACK's dense steps.
    method "host":   the reference's structure, ARPACK on the host calling one GPU
                     propagation per Krylov vector with a host round trip.
    flow_start: random start vectors that vanish outside the flow cells. The residual is
    masked by the flow cells, so the operator has zero rows there and leaves the flow-cell
    subspace invariant (with the shock unknowns too, which read and write only flow cells);
    the other cells only add the trivial eigenvalue mu = 1 (lambda = 0), which this excludes
    exactly."""
    import time
    dt = CFL_TIMESTEP(s)
    timesteps = int(round(T_ref / dt))
    n = L.n
    ncv = ncv or max(2 * n_modes + 1, 20, n_modes + 4 * block)
    mask = None
    if flow_start and s.cfg.shock_enabled and s.cfg.shock_feedback:
        st = s.get_state()
        flow = (np.arange(1, s.cfg.neta + 1)[None, :] < st["cell_idx"][:, None]).ravel(order="F")
        mask = np.concatenate([np.tile(flow.astype(np.float64), 4), np.ones(n - 4 * s.N)])
    rng = np.random.Generator(np.random.PCG64(seed))
    t0 = time.perf_counter()
    X = None
    restarts = None
    if method == "device":
        from .krylov import DeviceBuffer
        x0 = rng.standard_normal((block, n))
        if mask is not None:
            x0 *= mask[None, :]
        x0 = np.ascontiguousarray(x0.ravel())
        mr, mi, resid = np.empty(n_modes), np.empty(n_modes), np.empty(n_modes)
        info3 = np.zeros(3, dtype=np.int32)
        want = modes and 2 * n_modes <= ncv
        vb = DeviceBuffer(s.ctx, 8 * n * 2 * n_modes) if want else None
        o = _krylov_opts(n_modes, ncv, tol, maxit, block, order)
        s.ctx.check(s.ctx.L.hymor_eigs(s.ctx.h, ctypes.byref(o), float(dt), int(timesteps), dp(x0), dp(mr), dp(mi),
                                       dp(resid), ip(info3), vb.ptr if vb else None))
        mu = mr + 1j * mi
        if vb is not None:
            Xr = vb.download(2 * n * n_modes).reshape(2 * n_modes, n).T
            X = Xr[:, :n_modes] + 1j * Xr[:, n_modes:]
            vb.free()
        nops, converged, restarts = int(info3[0]), bool(info3[2]), int(info3[1])
    elif method == "python" and block > 1:
        from .krylov import block_krylov_schur
        mu, resid, nops, X = block_krylov_schur(s.ctx, n, _expm_block_op(s, dt, timesteps, order), n_modes, ncv,
                                                block, tol=tol, maxit=maxit, seed=seed, start_mask=mask,
                                                want_vectors=True)
        converged = bool(np.all(resid <= tol * np.abs(mu)))
    elif method == "python":
        from .krylov import krylov_schur
        v0 = rng.standard_normal(n)
        if mask is not None:
            v0 = v0 * mask
        mu, resid, nops, X = krylov_schur(s.ctx, n, _expm_op(s, dt, timesteps, order), n_modes, ncv, tol=tol,
                                          maxit=maxit, v0=v0, want_vectors=True)
        converged = bool(np.all(resid <= tol * np.abs(mu)))
    elif method == "host":
        from scipy.sparse.linalg import ArpackNoConvergence, LinearOperator, eigs
        count = [0]

        def mv(x):
            count[0] += 1
            return L.expm(np.ascontiguousarray(x, dtype=np.float64).ravel(), dt, timesteps, order)
        try:
            mu, X = eigs(LinearOperator((n, n), matvec=mv, dtype=np.float64), k=n_modes, which="LM", tol=tol,
                         ncv=ncv, v0=rng.standard_normal(n), maxiter=maxit * n_modes, return_eigenvectors=True)
            order_ = np.argsort(-np.abs(mu))
            mu, X = mu[order_], X[:, order_]
            converged = True
        except ArpackNoConvergence as e:
            mu, X, converged = np.asarray(e.eigenvalues), None, False
        resid = np.full(len(mu), np.nan)
        nops = count[0]
    else:
        raise HymorError(-1, f"unknown method {method!r}")
    elapsed = time.perf_counter() - t0
    lam = np.log(mu.astype(complex)) / (dt * timesteps)
    if not converged and not keep_unconverged:
        import warnings
        warnings.warn(f"eigen solve did not reach tol {tol:g} in {maxit} restarts; returning NaN")
        lam = np.full(n_modes, np.nan + 1j * np.nan)
        mu = np.full(n_modes, np.nan + 1j * np.nan)
        X = np.full((n, n_modes), np.nan + 1j * np.nan) if modes else None
    info = dict(mu=mu, resid=resid, dt=dt, timesteps=timesteps, nops=nops, seconds=elapsed, converged=converged,
                restarts=restarts)
    if modes:
        info["modes"] = X
    return lam, info


def chu_blocks(s: Solution, norms=(1, 1, 1, 1)):
    """Per-cell 4x4 blocks of C0 = R'MR and D = R'M^R for the current state of `s`."""
    st = s.get_state()
    return chu_blocks_from_state(s.cfg, s.case.mesh["vol"], st["q"], st["cell_idx"], norms)


def chu_blocks_from_state(cfg, vol, qflat, cell_idx, norms=(1, 1, 1, 1)):
    """CONSTRUCT_R.jl:24-133 (conserved -> (p, u, v, S)), CONSTRUCT_M.jl:27-94 (Chu weights
    masked by the flow cells) and CONSTRUCT_M_HAT.jl:25-105 (unmasked), as per-cell 4x4
    blocks of C0 = R'MR and D = R'M^R. Host-side set-up of the transient-growth operator,
    like the reference's sparse constructions."""
    nchi, neta = cfg.nchi, cfg.neta
    g = cfg.gamma
    q = np.asarray(qflat).reshape(4, nchi + 2, neta + 2, order="C")
    q = np.asarray(qflat).reshape(4, -1)
    shape = (nchi + 2, neta + 2)
    rho_G, ru_G, rv_G, rE_G = (q[k].reshape(shape, order="F")[1:-1, 1:-1].ravel(order="F") for k in range(4))
    rho = rho_G
    u = ru_G / rho
    w = rv_G / rho
    p = (rE_G - (ru_G**2 + rv_G**2) / rho / 2) * (g - 1)
    a = np.sqrt(g * p / rho)
    N = nchi * neta
    R = np.zeros((N, 4, 4))
    R[:, 0, 0] = (g - 1) * (u**2 + w**2) / 2
    R[:, 0, 1] = -u * (g - 1)
    R[:, 0, 2] = -w * (g - 1)
    R[:, 0, 3] = g - 1
    R[:, 1, 0] = -u / rho
    R[:, 1, 1] = 1.0 / rho
    R[:, 2, 0] = -w / rho
    R[:, 2, 2] = 1.0 / rho
    R[:, 3, 0] = (u**2 + w**2) / (2 * p) - g / (g - 1) / rho
    R[:, 3, 1] = -u / p
    R[:, 3, 2] = -w / p
    R[:, 3, 3] = 1.0 / p
    v = np.asarray(vol).ravel(order="F")
    if cfg.shock_enabled:
        flow = (np.arange(1, neta + 1)[None, :] < np.asarray(cell_idx)[:, None]).ravel(order="F").astype(float)
    else:
        flow = np.ones(N)
    mh = np.stack([rho * a**2 / (2 * (g * p) ** 2), rho / 2, rho / 2, (g - 1) * p / (2 * g)], axis=1) * v[:, None]
    mh = mh * np.asarray(norms, dtype=float)[None, :]
    m = mh * flow[:, None]
    C0 = np.einsum("nki,nk,nkj->nij", R, m, R)
    D = np.einsum("nki,nk,nkj->nij", R, mh, R)
    return C0, D


class _ChuWeights:
    """The weight operators of transient growth on the device: C0 = R'MR, K^-1 and K^-T with
    D = R'M^R = K Kᵀ per cell (CONSTRUCT_R/M/M_HAT), and their shock-position tails: R is
    the identity on those unknowns (CONSTRUCT_R.jl:109-118), M has no entries there
    (CONSTRUCT_M.jl:88-92) and M^ weighs them by bt_area[i, sc_i] / 2
    (CONSTRUCT_M_HAT.jl:77-90), so C0 is 0 and K is sqrt(bt_area / 2) on the tail."""

    def __init__(self, L: LinearOperatorGPU, s: Solution):
        from .krylov import DeviceBuffer
        self.s, self.N = s, s.N
        C0, D = chu_blocks(s)
        Kinv = np.linalg.inv(np.linalg.cholesky(D))
        self.KinvT = np.transpose(Kinv, (0, 2, 1))
        self.ntail = L.n - 4 * s.N
        self.tail_k = np.ones(1)
        if self.ntail:
            ci = s.get_state()["cell_idx"]
            self.tail_k = 1.0 / np.sqrt(np.asarray(s.case.mesh["bt_a"])[np.arange(s.nchi), ci - 1] / 2)
        self.blocks = [DeviceBuffer(s.ctx, 8 * s.N * 16) for _ in range(3)]
        for b, arr in zip(self.blocks, (C0, Kinv, self.KinvT)):
            b.upload(np.ascontiguousarray(arr.reshape(-1)))
        self.tails = [DeviceBuffer(s.ctx, 8 * max(self.ntail, 1)) for _ in range(2)]
        self.tails[0].upload(np.zeros(max(self.ntail, 1)))
        self.tails[1].upload(np.ascontiguousarray(self.tail_k))

    def apply(self, which: str, k: int, src, dst):
        """which: "C0", "Kinv" or "KinvT", on k contiguous device vectors."""
        b, t = {"C0": (0, 0), "Kinv": (1, 1), "KinvT": (2, 1)}[which]
        self.s.ctx.check(self.s.ctx.L.hymor_block4_apply_ext_dev(self.s.ctx.h, int(k), self.ntail, self.blocks[b].ptr,
                                                                 self.tails[t].ptr, src, dst))

    def initial_conditions(self, Y: np.ndarray) -> np.ndarray:
        """x = K^-T y per cell (and on the tail), y as [rho; rho_u; rho_v; rho_E; r] columns."""
        N = self.N
        Yc = Y[:4 * N].reshape(4, N, -1).transpose(1, 0, 2)            # (N, 4, k)
        X = np.einsum("nij,njk->nik", self.KinvT, Yc).transpose(1, 0, 2).reshape(4 * N, -1)
        if self.ntail:
            X = np.concatenate([X, Y[4 * N:] * self.tail_k[:, None]])
        return X

    def free(self):
        for b in self.blocks + self.tails:
            b.free()


def TRANSIENT_GROWTH_DOWNSTREAM(L: LinearOperatorGPU, s: Solution, n_modes: int, T: float, ncv: int | None = None,
                                tol: float = 1e-8, order: int = 5, seed: int = 4, maxit: int = 300,
                                block: int = 1, modes: bool = False, keep_unconverged: bool = False,
                                method: str = "device"):
    """TRANSIENT_GROWTH_DOWNSTREAM (TRANSIENT_GROWTH_DOWNSTREAM.jl:34-153): optimal energy gains
    G(T), the largest eigenvalues of exp(Lᵀ T) R'MR exp(L T) x = G R'M^R x. The generalised
    symmetric problem is reduced with the per-cell Cholesky factor of R'M^R (D = K Kᵀ) to
    K^{-1} Pᵀ C0 P K^{-ᵀ} y = G y and solved by Krylov-Schur (Lanczos with full
    reorthogonalisation) on the device; the forward propagation P and its adjoint Pᵀ are
    Taylor-`order` steps of dt = T / round(T / dt_CFL). block > 1: block Krylov-Schur, the
    operator applied to `block` vectors per batched call. modes: also the optimal initial
    conditions x = K^-T y (info["modes"], n x n_modes, x' R'M^R x = 1; the reference's V).
    Non-convergence warns and returns NaN, as the reference
    (TRANSIENT_GROWTH_DOWNSTREAM.jl:131-135), unless keep_unconverged.

    method "device": hymor_tg_gain (the solver behind the C ABI, weights built on the device
    context's state); "python": the Krylov-Schur driven from Python (krylov.py) with the
    weights built by numpy."""
    ncv = ncv or max(2 * n_modes + 1, 16, n_modes + 4 * block)
    if method == "python":
        return _tg_python(L, s, n_modes, T, ncv, tol, order, seed, maxit, block, modes, keep_unconverged)
    import time
    from .krylov import DeviceBuffer
    n = L.n
    rng = np.random.Generator(np.random.PCG64(seed))
    x0 = np.ascontiguousarray(rng.standard_normal((block, n)).ravel())
    G = np.empty(n_modes)
    resid = np.empty(n_modes)
    info3 = np.zeros(3, dtype=np.int32)
    dt_o, nt_o = np.empty(1), np.zeros(1, dtype=np.int32)
    vb = DeviceBuffer(s.ctx, 8 * n * n_modes) if modes else None
    o = _krylov_opts(n_modes, ncv, tol, maxit, block, order)
    Ts = np.array([float(T)])
    t0 = time.perf_counter()
    s.ctx.check(s.ctx.L.hymor_tg_gain(s.ctx.h, ctypes.byref(o), 1, dp(Ts), dp(x0), dp(G), dp(resid), ip(info3),
                                      dp(dt_o), ip(nt_o), vb.ptr if vb else None))
    elapsed = time.perf_counter() - t0
    X = None
    if vb is not None:
        X = vb.download(n * n_modes).reshape(n_modes, n).T.copy()
        vb.free()
    converged = bool(info3[2])
    if not converged and not keep_unconverged:
        import warnings
        warnings.warn(f"transient-growth solve did not reach tol {tol:g} in {maxit} restarts; returning NaN")
        G = np.full(n_modes, np.nan)
        X = np.full((n, n_modes), np.nan) if modes else None
    dt, n_t = float(dt_o[0]), int(nt_o[0])
    info = dict(resid=resid, dt=dt, n_t=n_t, T_opt=n_t * dt, nops=int(info3[0]), seconds=elapsed,
                converged=converged, restarts=int(info3[1]))
    if modes:
        info["modes"] = X
    return G, info


def _tg_python(L, s, n_modes, T, ncv, tol, order, seed, maxit, block, modes, keep_unconverged):
    """TRANSIENT_GROWTH_DOWNSTREAM with the Krylov-Schur driven from Python (krylov.py)."""
    import time
    from .krylov import DeviceBuffer, block_krylov_schur, krylov_schur
    dt_cfl = CFL_TIMESTEP(s)
    n_t = int(round(T / dt_cfl))
    dt = T / n_t
    n = L.n
    W = _ChuWeights(L, s)
    t1, t2 = DeviceBuffer(s.ctx, 8 * n * block), DeviceBuffer(s.ctx, 8 * n * block)
    Lh, h = s.ctx.L, s.ctx.h

    def apply_k(src, dst, k):
        W.apply("KinvT", k, src, t1.ptr)                                                   # x = K^-T y
        s.ctx.check(Lh.hymor_expm_apply_dev(h, k, dt, n_t, order, t1.ptr, t2.ptr, 0))      # P x
        W.apply("C0", k, t2.ptr, t1.ptr)                                                   # C0 P x
        s.ctx.check(Lh.hymor_expm_apply_dev(h, k, dt, n_t, order, t1.ptr, t2.ptr, 1))      # Pᵀ C0 P x
        W.apply("Kinv", k, t2.ptr, dst)                                                    # K^-1 (...)
    t0 = time.perf_counter()
    if block > 1:
        gains, resid, nops, Y = block_krylov_schur(s.ctx, n, apply_k, n_modes, ncv, block, tol=tol, maxit=maxit,
                                                   seed=seed, symmetric=True, want_vectors=True)
    else:
        gains, resid, nops, Y = krylov_schur(s.ctx, n, lambda a, b: apply_k(a, b, 1), n_modes, ncv, tol=tol,
                                             maxit=maxit, seed=seed, symmetric=True, want_vectors=True)
    elapsed = time.perf_counter() - t0
    for b in (t1, t2):
        b.free()
    gains = np.real(gains)
    converged = bool(np.all(resid <= tol * np.abs(gains)))
    X = W.initial_conditions(Y) if (modes and Y is not None) else None
    W.free()
    if not converged and not keep_unconverged:
        import warnings
        warnings.warn(f"transient-growth solve did not reach tol {tol:g} in {maxit} restarts; returning NaN")
        gains = np.full(n_modes, np.nan)
        X = np.full((n, n_modes), np.nan) if modes else None
    info = dict(resid=resid, dt=dt, n_t=n_t, T_opt=n_t * dt, nops=nops, seconds=elapsed, converged=converged)
    if modes:
        info["modes"] = X
    return gains, info


def TRANSIENT_GROWTH_HORIZONS(L: LinearOperatorGPU, s: Solution, n_modes: int, Ts, ncv: int | None = None,
                              tol: float = 1e-8, order: int = 5, seed: int = 4, maxit: int = 300,
                              keep_unconverged: bool = False, method: str = "device"):
    """TRANSIENT_GROWTH_DOWNSTREAM for several time horizons at once: one Krylov-Schur solve
    per horizon, run in lockstep, so that each round propagates one vector per unfinished
    horizon in one batched call (hymor_expm_apply_multi_dev: each vector with its own
    dt = T / round(T / dt_CFL) and step count, the longer horizons first). Each horizon's
    solve makes the same operations as TRANSIENT_GROWTH_DOWNSTREAM(T) with the same seed.
    Returns (gains, infos): gains[h] the n_modes gains of Ts[h], infos[h] as
    TRANSIENT_GROWTH_DOWNSTREAM's info (seconds: the whole batched solve).

    method "device": hymor_tg_gain with nh horizons (the lockstep behind the C ABI);
    "python": krylov_schur_many driven from Python."""
    ncv = ncv or max(2 * n_modes + 1, 16)
    if method == "python":
        return _tg_horizons_python(L, s, n_modes, Ts, ncv, tol, order, seed, maxit, keep_unconverged)
    import time
    Ts = np.array([float(T) for T in Ts])
    H, n = len(Ts), L.n
    x0 = np.ascontiguousarray(np.random.Generator(np.random.PCG64(seed)).standard_normal(n))
    G = np.empty((H, n_modes))
    resid = np.empty((H, n_modes))
    info3 = np.zeros(3 * H, dtype=np.int32)
    dts, nts = np.empty(H), np.zeros(H, dtype=np.int32)
    o = _krylov_opts(n_modes, ncv, tol, maxit, 1, order)
    t0 = time.perf_counter()
    s.ctx.check(s.ctx.L.hymor_tg_gain(s.ctx.h, ctypes.byref(o), H, dp(Ts), dp(x0), dp(G), dp(resid), ip(info3),
                                      dp(dts), ip(nts), None))
    elapsed = time.perf_counter() - t0
    infos = []
    for h in range(H):
        converged = bool(info3[3 * h + 2])
        if not converged and not keep_unconverged:
            G[h] = np.nan
        infos.append(dict(resid=resid[h], dt=float(dts[h]), n_t=int(nts[h]), T_opt=int(nts[h]) * float(dts[h]),
                          nops=int(info3[3 * h]), seconds=elapsed, converged=converged,
                          restarts=int(info3[3 * h + 1])))
    if not all(inf["converged"] for inf in infos) and not keep_unconverged:
        import warnings
        warnings.warn(f"transient-growth solves of some horizons did not reach tol {tol:g}; their gains are NaN")
    return G, infos


def _tg_horizons_python(L, s, n_modes, Ts, ncv, tol, order, seed, maxit, keep_unconverged):
    """TRANSIENT_GROWTH_HORIZONS with the lockstep Krylov-Schur driven from Python."""
    import time
    from .krylov import DeviceBuffer, krylov_schur_many
    Ts = [float(T) for T in Ts]
    dt_cfl = CFL_TIMESTEP(s)
    steps = [int(round(T / dt_cfl)) for T in Ts]
    dts = [T / nt for T, nt in zip(Ts, steps)]
    order_h = sorted(range(len(Ts)), key=lambda h: -steps[h])        # longest horizon first
    H, n = len(Ts), L.n
    W = _ChuWeights(L, s)
    bufs = [DeviceBuffer(s.ctx, 8 * n * H) for _ in range(4)]
    Lh, h = s.ctx.L, s.ctx.h

    def apply_many(idx, srcs, dsts):
        k = len(idx)
        hs = [order_h[i] for i in idx]
        dt_k = np.array([dts[j] for j in hs])
        st_k = np.array([steps[j] for j in hs], dtype=np.int32)
        for c, src in enumerate(srcs):
            s.ctx.check(Lh.hymor_memcpy_d2d(h, bufs[0].addr(c * n), src, 8 * n))
        def expm(src, dst, transpose):
            s.ctx.check(Lh.hymor_expm_apply_multi_dev(h, k, dp(dt_k), ip(st_k), int(order), src, dst, transpose))
        W.apply("KinvT", k, bufs[0].ptr, bufs[1].ptr)       # x = K^-T y
        expm(bufs[1].ptr, bufs[2].ptr, 0)                  # P x
        W.apply("C0", k, bufs[2].ptr, bufs[3].ptr)          # C0 P x
        expm(bufs[3].ptr, bufs[2].ptr, 1)                  # Pᵀ C0 P x
        W.apply("Kinv", k, bufs[2].ptr, bufs[0].ptr)        # K^-1 (...)
        for c, dst in enumerate(dsts):
            s.ctx.check(Lh.hymor_memcpy_d2d(h, dst, bufs[0].addr(c * n), 8 * n))
    problems = [dict(nev=n_modes, ncv=ncv, tol=tol, maxit=maxit, seed=seed, symmetric=True) for _ in Ts]
    t0 = time.perf_counter()
    res = krylov_schur_many(s.ctx, n, apply_many, problems)
    elapsed = time.perf_counter() - t0
    for b in bufs:
        b.free()
    W.free()
    gains = np.full((H, n_modes), np.nan)
    infos: list = [None] * H
    for i, j in enumerate(order_h):
        g, resid, nops = res[i]
        g = np.real(g)
        converged = bool(np.all(resid <= tol * np.abs(g)))
        if converged or keep_unconverged:
            gains[j] = g
        infos[j] = dict(resid=resid, dt=dts[j], n_t=steps[j], T_opt=steps[j] * dts[j], nops=nops, seconds=elapsed,
                        converged=converged)
    if not all(inf["converged"] for inf in infos) and not keep_unconverged:
        import warnings
        warnings.warn(f"transient-growth solves of some horizons did not reach tol {tol:g}; their gains are NaN")
    return gains, infos
