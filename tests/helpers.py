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
