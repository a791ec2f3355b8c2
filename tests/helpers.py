"""Shared checks for the parity tests."""
import numpy as np


def max_rel(a, b, floor=1e-300):
    """max over cells of |a-b| / max(|b|, floor)."""
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


def max_rel_scaled(a, b):
    """max per-cell relative difference, with each field's difference taken relative to
    max(|b_cell|, 1e-12 * max|b|) so that cells where a velocity is ~0 do not divide by ~0."""
    a, b = np.asarray(a), np.asarray(b)
    out = 0.0
    for k in range(a.shape[0]):
        scale = np.maximum(np.abs(b[k]), 1e-12 * np.max(np.abs(b[k])) + 1e-300)
        out = max(out, float(np.max(np.abs(a[k] - b[k]) / scale)))
    return out


def l1(a, b):
    return np.mean(np.abs(np.asarray(a) - np.asarray(b)), axis=-1)
