"""Shared helpers of the test suite: workload construction and the parity metrics."""
from __future__ import annotations

import numpy as np

from plens_gb300 import configs


def make(spec):
    return configs.make_case(spec)


def var_scales(X: np.ndarray) -> np.ndarray:
    """Per-equation scale of a [5][ndof] field: max |.| of rho, of the momentum vector (the three
    components jointly, so a component that is pure round-off noise in a quasi-1D flow is
    measured against the momentum it belongs to), and of rho E."""
    a = np.abs(X)
    m = a[1:4].max()
    return np.array([a[0].max(), m, m, m, a[4].max()])


def max_rel_err(X: np.ndarray, ref: np.ndarray) -> float:
    """max over equations of max_dof |X - ref| / scale(ref)."""
    s = var_scales(ref)
    s = np.where(s > 0, s, 1.0)
    return float(max(np.abs(X[v] - ref[v]).max() / s[v] for v in range(5)))


def rel_l1(X: np.ndarray, ref: np.ndarray) -> np.ndarray:
    """Relative L1 error of rho, momentum (jointly) and rho E."""
    d = np.abs(X - ref)
    a = np.abs(ref)
    return np.array([d[0].sum() / a[0].sum(), d[1:4].sum() / max(a[1:4].sum(), 1e-300), d[4].sum() / a[4].sum()])
