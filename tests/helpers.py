"""Shared helpers of the parity tests."""
from __future__ import annotations

import numpy as np


def rel_err(a, b) -> float:
    """max |a - b| / max |b| (norm-wise relative error)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.max(np.abs(b))
    if scale == 0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b)) / scale)


def per_var_rel(a, b, nvar=4):
    a = np.asarray(a).reshape(nvar, -1)
    b = np.asarray(b).reshape(nvar, -1)
    return [rel_err(a[v], b[v]) for v in range(nvar)]


def flux_term_scale(case) -> np.ndarray:
    """Per-variable magnitude of the face fluxes that the residual sums, max over cells of
    Σ |F_face| A / vol with inviscid face fluxes of the initial state. Rounding errors of
    a residual scale with this, not with the (possibly cancelling) residual itself."""
    q = case.q
    g = case.cfg.gamma
    rho, ru, rv, rE = q
    p = (rE - (ru**2 + rv**2) / rho / 2) * (g - 1)
    u, v = ru / rho, rv / rho
    speed = np.sqrt(u**2 + v**2)
    inner = (slice(1, -1), slice(1, -1))
    m = case.mesh.arrays
    geo = ((m["lr_a"][1:] + m["lr_a"][:-1]) + (m["bt_a"][:, 1:] + m["bt_a"][:, :-1])) / m["vol"]
    terms = [rho * speed, ru * speed + p, rv * speed + p, (rE + p) * speed]
    return np.array([np.max(np.abs(t[inner]) * geo) for t in terms])


def residual_rel(fg, fo, case):
    """max |fg - fo| per variable over max(max |fo|, flux term scale)."""
    fg = np.asarray(fg).reshape(4, -1)
    fo = np.asarray(fo).reshape(4, -1)
    sc = flux_term_scale(case)
    return [float(np.max(np.abs(fg[v] - fo[v])) / max(np.max(np.abs(fo[v])), sc[v])) for v in range(4)]


def state_rel(qa, qb):
    """State error per variable; momentum components share the momentum scale."""
    a = np.asarray(qa).reshape(4, -1)
    b = np.asarray(qb).reshape(4, -1)
    mom = max(np.max(np.abs(b[1])), np.max(np.abs(b[2])))
    scales = [np.max(np.abs(b[0])), mom, mom, np.max(np.abs(b[3]))]
    return [float(np.max(np.abs(a[v] - b[v])) / scales[v]) for v in range(4)]
