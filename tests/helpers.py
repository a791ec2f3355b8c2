"""Shared checks for the parity tests."""
import numpy as np


def max_rel(a, b, floor=1e-300):
    """max over cells of |a-b| / max(|b|, floor)."""
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


def max_rel_scaled(a, b):
    """Max per-cell relative difference of primitive planes (rho, u, [v,] T): density and
    temperature (positive everywhere) relative to each cell's value; velocities, which pass
    through zero, relative to the field's largest magnitude."""
    a, b = np.asarray(a), np.asarray(b)
    nv = a.shape[0]
    out = 0.0
    for k in range(nv):
        if k in (0, nv - 1):
            scale = np.abs(b[k])
        else:
            scale = np.full_like(b[k], max(np.max(np.abs(b[k])), 1e-300))
        out = max(out, float(np.max(np.abs(a[k] - b[k]) / scale)))
    return out


def l1(a, b):
    return np.mean(np.abs(np.asarray(a) - np.asarray(b)), axis=-1)
