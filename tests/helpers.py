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


def batch1d_draws(count=4096, seed=0):
    """The seeded batch of independent 1D shock tubes (4096 tubes, seed 0): per tube, in this draw
    order, cells round(exp(U(ln 256, ln 16384))), density ratio U(2, 100), temperature ratio
    U(0.5, 2), diaphragm position U(0.3, 0.7); first order for the first half, second order after.
    Returns (index, cells, density ratio, temperature ratio, diaphragm, order) tuples."""
    import math
    rng = np.random.default_rng(seed)
    out = []
    for t in range(count):
        n = int(round(math.exp(rng.uniform(math.log(256), math.log(16384)))))
        ratio = float(rng.uniform(2, 100))
        tr = float(rng.uniform(0.5, 2))
        xd = float(rng.uniform(0.3, 0.7))
        out.append((t, n, ratio, tr, xd, 1 if t < count // 2 else 2))
    return out


def tube_params(shll, draw, precision):
    t, n, ratio, tr, xd, order = draw
    return shll.params(1, order, nx=n, precision=precision, t_end=0.2, ic_x_d=xd, ic_rho_l=ratio, ic_T_l=tr,
                       ic_rho_r=1.0, ic_T_r=1.0, ic_u_l=0.0, ic_u_r=0.0)


def batch2d_draws(count=256, seed=1):
    """The seeded batch of independent 2D first-order domains (256 domains, seed 1): per domain, in
    this draw order, side uniform in {128, 256, 512, 1024}, diaphragm radius U(0.1, 0.35), inside /
    outside density ratio U(2, 50), temperature ratio U(0.5, 2); gas at rest, 400 steps.
    Returns (index, side, radius, density ratio, temperature ratio) tuples."""
    rng = np.random.default_rng(seed)
    out = []
    for t in range(count):
        n = int(rng.choice([128, 256, 512, 1024]))
        out.append((t, n, float(rng.uniform(0.1, 0.35)), float(rng.uniform(2, 50)), float(rng.uniform(0.5, 2))))
    return out


def circle_params(shll, n, radius, ratio, tr, steps, precision):
    return shll.params(2, 1, nx=n, ny=n, precision=precision, n_steps=steps, ic_kind=shll.IC_CIRCLE2D, ic_cx=0.5,
                       ic_cy=0.5, ic_radius=radius, ic_rho_l=ratio, ic_T_l=tr, ic_rho_r=1.0, ic_T_r=1.0)
