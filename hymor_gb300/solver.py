"""Reference-shaped host API over libhymor.

The reference drives its hot path through Julia functions on a solution Dict
(utils/Operators/PDE.jl:1, utils/Time_marching/ADVECT_FLOW.jl:30,
utils/Stability_analysis/Modal_stability_analysis/LINEARIZE_L.jl:34, ...). This
module keeps those names and argument meanings: a :class:`Solution` plays the
Dict (its arrays live on the GPU), and the functions mutate it in place and
return it, exactly as the reference mutates and returns `s`.

Every call goes through the C ABI (include/hymor.h); nothing here computes
flow quantities on the CPU.
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

    def var(self) -> dict:
        """s["var"]: the four ghosted conserved arrays, (Nchi+2, Neta+2) column-major."""
        q = self.get_state()["q"].reshape(4, -1)
        shape = (self.nchi + 2, self.neta + 2)
        return {k: q[v].reshape(shape, order="F") for v, k in enumerate(("rho", "rho_u", "rho_v", "rho_E"))}

    def counters(self) -> tuple[int, int]:
        a, b = ctypes.c_int32(), ctypes.c_int32()
        self.ctx.check(self.ctx.L.hymor_counters(self.ctx.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

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


def UPDATE_FLOW_CELLS(s: Solution) -> Solution:
    s.ctx.check(s.ctx.L.hymor_update_flow_cells(s.ctx.h))
    return s


def CFL_TIMESTEP(s: Solution) -> float:
    dt = ctypes.c_double()
    s.ctx.check(s.ctx.L.hymor_cfl_timestep(s.ctx.h, ctypes.byref(dt)))
    return dt.value


class LinearOperatorGPU:
    """The linearised operator L (a Nchi*Neta*144 stencil-block Jacobian on the GPU).

    Stands in for the reference's SparseMatrixCSC `L` of LINEARIZE_L: ``L @ x``,
    ``L.T @ x`` and the Taylor propagator act on 4N-vectors (or 4N x k blocks)."""

    def __init__(self, s: Solution, transpose: bool = False):
        self.s = s
        self.n = 4 * s.N
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


def LINEARIZE_L(s: Solution):
    """LINEARIZE_L (LINEARIZE_L.jl:34-69): coloured finite-difference Jacobian of the
    residual, assembled on the GPU. Returns (s, L)."""
    s.ctx.check(s.ctx.L.hymor_linearize(s.ctx.h))
    return s, LinearOperatorGPU(s)
