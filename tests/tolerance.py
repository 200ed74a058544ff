"""Per-cell error measures shared by the parity tests.

The FP64 tolerance is relative per cell, with a floor for fields that cross
zero (velocities, momenta): a cell passes when
    |got - want| <= tol * max(|want|, 1e-3 * max|want over the field|).
A field that is identically zero in the oracle must be identically zero.
"""
import numpy as np

FP64_TOL = 1e-12


def cell_rel_err(got, want, floor=1e-3):
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    scale = float(np.abs(want).max()) if want.size else 0.0
    if scale == 0.0:
        return 0.0 if not np.any(got) else float("inf")
    den = np.maximum(np.abs(want), floor * scale)
    return float((np.abs(got - want) / den).max())


def l1_rel(got, want):
    """sum |got - want| / sum |want| (the L1 error of a field)."""
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    s = float(np.abs(want).sum())
    return float(np.abs(got - want).sum() / s) if s > 0 else float(np.abs(got).sum())


def linf_rel(got, want):
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    s = float(np.abs(want).max())
    return float(np.abs(got - want).max() / s) if s > 0 else float(np.abs(got).max())
