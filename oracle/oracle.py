"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module. It never serves the product path.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from oracle import build_oracle  # noqa: E402
from hymor_gb300.case import Case, config_struct, dptr  # noqa: E402

_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        L = build_oracle.load()
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [vp, vp]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_state.argtypes = [vp, dp, dp, dp, dp, dp, ip, ctypes.c_double, dp]
        L.orc_get_state.argtypes = [vp, dp, dp, dp, dp, dp, ip, dp, dp]
        L.orc_get_derived.argtypes = [vp, dp, dp, dp, dp, dp, dp]
        L.orc_residual.argtypes = [vp, dp]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_set_flux.argtypes = [vp, dp]
        L.orc_update_flow_cells.argtypes = [vp]
        L.orc_update_shock_bc.argtypes = [vp]
        L.orc_cfl_timestep.argtypes = [vp]
        L.orc_cfl_timestep.restype = ctypes.c_double
        L.orc_advect.argtypes = [vp, ctypes.c_int]
        L.orc_counters.argtypes = [vp, ip, ip]
        L.orc_spline.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_int, dp, dp, dp]
        L.orc_element_space.argtypes = [vp, ctypes.c_int, dp, dp, dp, dp]
        L.orc_linearize.argtypes = [vp, dp]
        L.orc_jacobian.argtypes = [vp, dp]
        L.orc_matvec.argtypes = [vp, dp, dp, dp, ctypes.c_int]
        L.orc_expm.argtypes = [vp, dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, dp, dp,
                               ctypes.c_int]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_shock_blocks.argtypes = [vp, ip, dp, dp, dp]
        L.orc_get_rel_vel.argtypes = [vp, dp]
        L.orc_linearize_b.argtypes = [vp, ip, dp, dp]
        L.orc_set_upstream.argtypes = [vp, dp]
        L.orc_matvec_ext.argtypes = [vp, dp, ip, dp, dp, dp, dp, dp, ctypes.c_int]
        L.orc_expm_ext.argtypes = [vp, dp, ip, dp, dp, dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, dp, dp,
                                   ctypes.c_int]
        _lib = L
    return _lib


def _check(rc: int):
    if rc != 0:
        raise RuntimeError(lib().orc_last_error().decode())


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class Oracle:
    """One reference solution Dict held by the C++ restatement."""

    def __init__(self, case: Case):
        self.case = case
        self.cfg = case.cfg
        self.cs = config_struct(case.cfg)
        self._ms, self._keep = case.mesh_struct()
        self.h = lib().orc_create(ctypes.byref(self.cs), ctypes.byref(self._ms))
        self.nchi, self.neta = case.cfg.nchi, case.cfg.neta
        self.set_state(case.q_flat(), case.pts_x, case.pts_y, case.pts_chi, case.pts_eta,
                       case.cell_idx, case.t, case.a)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    @property
    def G(self):
        return (self.nchi + 2) * (self.neta + 2)

    @property
    def N(self):
        return self.nchi * self.neta

    def set_state(self, qflat, px, py, pchi, peta, cell_idx, t, a=None):
        qflat = np.ascontiguousarray(qflat, dtype=np.float64)
        arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in (px, py, pchi, peta)]
        ci = np.ascontiguousarray(cell_idx, dtype=np.int32)
        aa = None if a is None else np.asfortranarray(a, dtype=np.float64)
        lib().orc_set_state(self.h, dptr(qflat), *[dptr(v) for v in arrs], _ip(ci), float(t),
                            dptr(aa) if aa is not None else None)

    def get_state(self):
        q = np.empty(4 * self.G)
        px, py, pc, pe = (np.empty(self.nchi) for _ in range(4))
        ci = np.empty(self.nchi, dtype=np.int32)
        t, dt = ctypes.c_double(), ctypes.c_double()
        lib().orc_get_state(self.h, dptr(q), dptr(px), dptr(py), dptr(pc), dptr(pe), _ip(ci),
                            ctypes.byref(t), ctypes.byref(dt))
        return dict(q=q, pts_x=px, pts_y=py, pts_chi=pc, pts_eta=pe, cell_idx=ci, t=t.value,
                    dt=dt.value)

    def derived(self):
        p, T, a = (np.empty(self.G) for _ in range(3))
        beta, sx, sy = (np.empty(self.nchi) for _ in range(3))
        lib().orc_get_derived(self.h, dptr(p), dptr(T), dptr(a), dptr(beta), dptr(sx), dptr(sy))
        return dict(p=p, T=T, a=a, beta=beta, speed_x=sx, speed_y=sy)

    def residual(self) -> np.ndarray:
        f = np.empty(4 * self.N)
        _check(lib().orc_residual(self.h, dptr(f)))
        return f

    def set_flux(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        lib().orc_set_flux(self.h, dptr(f))

    def advect(self, nsteps: int):
        _check(lib().orc_advect(self.h, int(nsteps)))

    def update_flow_cells(self):
        _check(lib().orc_update_flow_cells(self.h))

    def cfl(self) -> float:
        return lib().orc_cfl_timestep(self.h)

    def counters(self):
        a, b = ctypes.c_int32(), ctypes.c_int32()
        lib().orc_counters(self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def linearize(self) -> np.ndarray:
        coef = np.empty(self.N * 144)
        _check(lib().orc_linearize(self.h, dptr(coef)))
        return coef

    def jacobian(self) -> np.ndarray:
        coef = np.empty(self.N * 144)
        lib().orc_jacobian(self.h, dptr(coef))
        return coef

    def matvec(self, coef, x, transpose=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(4 * self.N)
        lib().orc_matvec(ctypes.byref(self.cs), dptr(coef), dptr(x), dptr(y), int(transpose))
        return y

    def rel_vel(self) -> np.ndarray:
        """s["shock"]["relative_increase_velocity"] of the last shock update."""
        r = np.empty(self.cs.nchi)
        lib().orc_get_rel_vel(self.h, dptr(r))
        return r

    def linearize_b(self):
        """LINEARIZE_B of the prepared state: rows (Nchi), bq (Nchi x 3 x 4 x 4: output column,
        input column offset + 1, vout, vin), bs (Nchi x 3 x 4)."""
        n = self.cs.nchi
        rows = np.empty(n, dtype=np.int32)
        bq, bs = np.empty(48 * n), np.empty(12 * n)
        _check(lib().orc_linearize_b(self.h, _ip(rows), dptr(bq), dptr(bs)))
        return rows, bq.reshape(n, 3, 4, 4), bs.reshape(n, 3, 4)

    def set_upstream(self, cols):
        """Prescribed per-column upstream state (4 x Nchi), or None."""
        if cols is None:
            lib().orc_set_upstream(self.h, None)
        else:
            cols = np.ascontiguousarray(cols, dtype=np.float64).ravel()
            lib().orc_set_upstream(self.h, dptr(cols))

    def shock_blocks(self):
        """The shock-position blocks of the prepared state (after linearize()): rows (Nchi),
        a21_full (8 Nchi x Nchi: the reference's A21 columns, column (v*2 + j-1)*Nchi + i),
        a12 (4 Nchi x Nchi), a22 (Nchi x Nchi)."""
        n = self.cs.nchi
        rows = np.empty(n, dtype=np.int32)
        a21 = np.empty(8 * n * n)
        a12 = np.empty(4 * n * n)
        a22 = np.empty(n * n)
        _check(lib().orc_shock_blocks(self.h, _ip(rows), dptr(a21), dptr(a12), dptr(a22)))
        return rows, a21.reshape(8 * n, n), a12.reshape(4 * n, n), a22.reshape(n, n)

    def matvec_ext(self, coef, blocks, x, transpose=False):
        rows, a21, a12, a22 = (np.ascontiguousarray(b) for b in blocks)
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(4 * self.N + self.cs.nchi)
        lib().orc_matvec_ext(ctypes.byref(self.cs), dptr(coef), _ip(rows), dptr(a21), dptr(a12), dptr(a22),
                             dptr(x), dptr(y), int(transpose))
        return y

    def expm_ext(self, coef, blocks, dt, nsteps, x, order=5, transpose=False):
        rows, a21, a12, a22 = (np.ascontiguousarray(b) for b in blocks)
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(4 * self.N + self.cs.nchi)
        lib().orc_expm_ext(ctypes.byref(self.cs), dptr(coef), _ip(rows), dptr(a21), dptr(a12), dptr(a22),
                           float(dt), int(nsteps), int(order), dptr(x), dptr(y), int(transpose))
        return y

    def expm(self, coef, dt, nsteps, x, order=5, transpose=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(4 * self.N)
        lib().orc_expm(ctypes.byref(self.cs), dptr(coef), float(dt), int(nsteps), int(order),
                       dptr(x), dptr(y), int(transpose))
        return y


def compact_a21(rows, a21_full):
    """The stencil-compact A21 (Nchi x 8, entry (j-1)*4 + v) of the reference's columns: the
    column of cell (i, sc_i - j), variable v, contributes its entry for point i."""
    n = len(rows)
    F = np.asarray(a21_full).reshape(4, 2, n, n)       # (v, j-1, perturbed column i, point idx)
    out = np.empty((n, 8))
    for v in range(4):
        for j in range(2):
            out[:, j * 4 + v] = F[v, j, np.arange(n), np.arange(n)]
    return out


def spline(xs, ys, lam, t):
    xs, ys, t = (np.ascontiguousarray(v, dtype=np.float64) for v in (xs, ys, t))
    val, der = np.empty(len(t)), np.empty(len(t))
    lib().orc_spline(len(xs), dptr(xs), dptr(ys), float(lam), len(t), dptr(t), dptr(val), dptr(der))
    return val, der


def stencil_to_csr(cfg, coef):
    """Scatter the stencil blocks into a scipy CSR matrix (4N x 4N)."""
    import scipy.sparse as sp
    nchi, neta = cfg.nchi, cfg.neta
    N = nchi * neta
    per_chi = cfg.bc_chi0 == "periodic" and cfg.bc_chi1 == "periodic"
    per_eta = cfg.bc_eta0 == "periodic" and cfg.bc_eta1 == "periodic"
    B = coef.reshape(N, 9, 4, 4)
    ii, jj = np.meshgrid(np.arange(nchi), np.arange(neta), indexing="ij")
    m = (ii + jj * nchi).ravel(order="F")
    iif, jjf = ii.ravel(order="F"), jj.ravel(order="F")
    rows, cols, vals = [], [], []
    for b in (-1, 0, 1):
        for a in (-1, 0, 1):
            q = (b + 1) * 3 + (a + 1)
            ni, nj = iif + a, jjf + b
            wi = (ni < 0) | (ni >= nchi)
            wj = (nj < 0) | (nj >= neta)
            ok = (~wi | per_chi) & (~wj | per_eta) & ~(wi & wj)
            ni = np.mod(ni, nchi)
            nj = np.mod(nj, neta)
            n = ni + nj * nchi
            for vo in range(4):
                for vi in range(4):
                    rows.append(vo * N + m[ok])
                    cols.append(vi * N + n[ok])
                    vals.append(B[m[ok], q, vo, vi])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                         shape=(4 * N, 4 * N))
