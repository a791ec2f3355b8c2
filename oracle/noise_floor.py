"""Noise floor of the reference scheme -- TEST INFRASTRUCTURE ONLY.

How far the FP64 solution of a shock tube moves when its initial state is perturbed at FP32
scale: the oracle's FP64 run (the reference scheme with float -> double) from the tube's initial
data, and again from the same data with density and temperature multiplied by 1 + eps*U(-1, 1)
(seeded).  The L1 distance between the two results is the spread that any arithmetic rounding at
FP32 scale must be expected to produce.  The second-order scheme (minmod on the split fluxes,
base-c/2nd_order_base_shll.c:191-201, 438-446) amplifies such perturbations strongly, so its
spread grows with the tube size; the first-order scheme on a Sod tube damps them.

spread_stepwise repeats the perturbation every few steps, as an arithmetic that rounds at FP32
scale in every step does; spread2d measures base-omp's 2D second-order problem.

Command line: python oracle/noise_floor.py [order] [cells ...]
(e.g. "python oracle/noise_floor.py 2 4096 16384 65536"; 65536 cells take a few minutes per run.)
"""
import concurrent.futures
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import oracle as O  # noqa: E402


def perturbed(prim, eps, seed):
    r = np.random.default_rng(seed)
    out = prim.copy()
    out[0] *= 1.0 + eps * r.uniform(-1.0, 1.0, prim.shape[1])
    out[2] *= 1.0 + eps * r.uniform(-1.0, 1.0, prim.shape[1])
    return out


def spread(n, order=2, x_d=0.5, rhoL=10.0, TL=1.0, eps=6e-8, seed=0):
    """L1 (rho, u, T) between the FP64 run from the Sod-type initial data and from its perturbation."""
    cfg = O.make_cfg(order=order, nx=n, real_bits=64)
    prim = O.ic_sod(n, x_d=x_d, rhoL=rhoL, TL=TL)
    with concurrent.futures.ThreadPoolExecutor(2) as ex:   # (the oracle runs outside the Python lock)
        a, b = ex.map(lambda p: O.run(cfg, p)[1], [prim, perturbed(prim, eps, seed)])
    return np.mean(np.abs(a - b), axis=1)


def spread_stepwise(n, order=2, x_d=0.5, rhoL=10.0, TL=1.0, eps=6e-8, every=10, seed=0):
    """The same distance when the perturbation is repeated every `every` steps (the run split into
    oracle runs of `every` steps, the state perturbed between them): the spread of an arithmetic that
    rounds at FP32 scale throughout the run, not only once."""
    cfg = O.make_cfg(order=order, nx=n, real_bits=64)
    total = O.count_steps(cfg)
    prim = O.ic_sod(n, x_d=x_d, rhoL=rhoL, TL=TL)
    ref = O.run(cfg, prim)[1]
    r = np.random.default_rng(seed)
    p, done = prim, 0
    while done < total:
        k = min(every, total - done)
        p = O.run(O.make_cfg(order=order, nx=n, real_bits=64, n_steps=k), p)[1]
        done += k
        p = perturbed(p, eps, int(r.integers(1 << 30)))
    return np.mean(np.abs(p - ref), axis=1)


def spread2d(n, eps=6e-8, seed=0):
    """The same distance for base-omp's 2D second-order problem (the quadrant initial data of
    base-omp/2nd_order_base_shll.c:147-172, MC limiter, t = 0.3) on n x n cells."""
    cfg = O.make_cfg(dim=2, order=2, nx=n, ny=n, real_bits=64, t_end=0.3, limiter=1, mc_alpha=1.25)
    prim = O.ic_quadrants2d(n, n, 64)
    r = np.random.default_rng(seed)
    pert = prim.copy()
    pert[0] *= 1.0 + eps * r.uniform(-1.0, 1.0, prim.shape[1])
    pert[3] *= 1.0 + eps * r.uniform(-1.0, 1.0, prim.shape[1])
    with concurrent.futures.ThreadPoolExecutor(2) as ex:
        a, b = ex.map(lambda p: O.run(cfg, p)[1], [prim, pert])
    return np.mean(np.abs(a - b), axis=1)


if __name__ == "__main__":
    order = int(sys.argv[1]) if len(sys.argv) > 1 else 2
    for n in [int(a) for a in sys.argv[2:]] or [4096, 16384]:
        s = spread(n, order)
        print(f"order {order}, {n} cells: L1 rho {s[0]:.2e}  u {s[1]:.2e}  T {s[2]:.2e}", flush=True)
