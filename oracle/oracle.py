"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only the tests, the smoke check and the CPU-baseline leg of bench.py import this module; it is
the checker the CUDA library is compared against, never part of the product path.  The C code
it loads (shll_oracle.c) restates the reference's solvers:
base-c/base_shll.c (1D first order), base-c/2nd_order_base_shll.c (second order, whose x sweep is
the 1D second-order scheme), base-c/base_shll_2d.c (2D first order) and the MC limiter of
base-omp/2nd_order_base_shll.c.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libshll_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")


class OracleCfg(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("order", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("real_bits", ctypes.c_int), ("limiter", ctypes.c_int), ("mc_alpha", ctypes.c_double),
        ("gamma", ctypes.c_double), ("R", ctypes.c_double), ("cfl", ctypes.c_double),
        ("lx", ctypes.c_double), ("ly", ctypes.c_double), ("t_end", ctypes.c_double),
        ("n_steps", ctypes.c_long),
    ]


_lib = None


def build():
    """Compiles the oracle library with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        L.oracle_run.argtypes = [ctypes.POINTER(OracleCfg), dp, dp, dp]
        L.oracle_run.restype = ctypes.c_long
        L.oracle_split_fluxes.argtypes = [ctypes.POINTER(OracleCfg), dp, dp, dp, dp, dp]
        L.oracle_split_fluxes.restype = ctypes.c_int
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_set_threads.restype = ctypes.c_int
        L.oracle_count_steps.argtypes = [ctypes.POINTER(OracleCfg)]
        L.oracle_count_steps.restype = ctypes.c_long
        L.oracle_ic_sod.argtypes = [ctypes.c_int] + [ctypes.c_double] * 7 + [dp]
        L.oracle_ic_ref_box2d.argtypes = [ctypes.c_int, ctypes.c_int, dp]
        L.oracle_ic_four_shock2d.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp]
        L.oracle_ic_quadrants2d.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp]
        L.oracle_ic_circle2d.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 9 + [dp]
        L.oracle_riemann_exact.argtypes = [ctypes.c_double] * 10 + [ctypes.c_int, ctypes.c_double, dp]
        L.oracle_riemann_exact.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_cfg(dim=1, order=1, nx=256, ny=1, real_bits=64, gamma=1.4, R=1.0, cfl=0.25,
             lx=1.0, ly=1.0, t_end=0.2, n_steps=0, limiter=0, mc_alpha=1.25):
    return OracleCfg(dim, order, nx, ny if dim == 2 else 1, real_bits, limiter, mc_alpha,
                     gamma, R, cfl, lx, ly, t_end, n_steps)


def nvar(cfg):
    return 4 if cfg.dim == 2 else 3


def run(cfg, prim_in):
    """Runs the oracle from primitive planes; returns (steps, prim_out, cons_out)."""
    n = cfg.nx * cfg.ny
    prim_in = np.ascontiguousarray(prim_in, dtype=np.float64).reshape(nvar(cfg), n)
    prim_out = np.zeros_like(prim_in)
    cons_out = np.zeros_like(prim_in)
    steps = lib().oracle_run(ctypes.byref(cfg), _p(prim_in), _p(prim_out), _p(cons_out))
    if steps < 0:
        raise ValueError("oracle rejected the configuration")
    return steps, prim_out, cons_out


def split_fluxes(cfg, cons):
    n = cfg.nx * cfg.ny
    cons = np.ascontiguousarray(cons, dtype=np.float64).reshape(nvar(cfg), n)
    fp, fm = np.zeros_like(cons), np.zeros_like(cons)
    hp, hm = np.zeros_like(cons), np.zeros_like(cons)
    rc = lib().oracle_split_fluxes(ctypes.byref(cfg), _p(cons), _p(fp), _p(fm), _p(hp), _p(hm))
    if rc != 0:
        raise ValueError("oracle rejected the configuration")
    return (fp, fm, hp, hm) if cfg.dim == 2 else (fp, fm)


def set_threads(n):
    """Threads of the stage loops (n <= 0: all processors); returns the count in use."""
    return lib().oracle_set_threads(n)


def count_steps(cfg):
    return lib().oracle_count_steps(ctypes.byref(cfg))


def ic_sod(n, x_d=0.5, rhoL=10.0, uL=0.0, TL=1.0, rhoR=1.0, uR=0.0, TR=1.0):
    prim = np.zeros((3, n))
    lib().oracle_ic_sod(n, x_d, rhoL, uL, TL, rhoR, uR, TR, _p(prim))
    return prim


def ic_ref_box2d(nx, ny):
    prim = np.zeros((4, nx * ny))
    lib().oracle_ic_ref_box2d(nx, ny, _p(prim))
    return prim


def ic_four_shock2d(nx, ny, real_bits, R=1.0):
    prim = np.zeros((4, nx * ny))
    lib().oracle_ic_four_shock2d(nx, ny, real_bits, R, _p(prim))
    return prim


def ic_quadrants2d(nx, ny, real_bits, R=1.0):
    prim = np.zeros((4, nx * ny))
    lib().oracle_ic_quadrants2d(nx, ny, real_bits, R, _p(prim))
    return prim


def ic_circle2d(nx, ny, cx=0.5, cy=0.5, r=0.25, rho_in=10.0, T_in=1.0, rho_out=1.0, T_out=1.0,
                lx=1.0, ly=1.0):
    prim = np.zeros((4, nx * ny))
    lib().oracle_ic_circle2d(nx, ny, lx, ly, cx, cy, r, rho_in, T_in, rho_out, T_out, _p(prim))
    return prim


def riemann_exact(n, t, x_d=0.5, rhoL=10.0, uL=0.0, TL=1.0, rhoR=1.0, uR=0.0, TR=1.0,
                  gamma=1.4, R=1.0, lx=1.0):
    prim = np.zeros((3, n))
    it = lib().oracle_riemann_exact(gamma, R, rhoL, uL, TL, rhoR, uR, TR, x_d, t, n, lx, _p(prim))
    if it < 0:
        raise ValueError("vacuum generated")
    return prim


def ref_available(name):
    return os.path.exists(os.path.join(REF_DIR, name))


def run_ref(name, cols, workdir):
    """Runs one executable built by make_ref.sh in workdir and parses its results.dat
    (columns: x, [y,] rho, u, [v,] T).  Returns (steps, prim planes)."""
    exe = os.path.join(REF_DIR, name)
    out = subprocess.run([exe], cwd=workdir, check=True, capture_output=True, text=True).stdout
    steps = None
    for line in out.splitlines():
        if line.startswith("Completed in"):
            steps = int(line.split()[2])
    data = np.loadtxt(os.path.join(workdir, "results.dat"), dtype=np.float64, ndmin=2)
    return steps, np.ascontiguousarray(data[:, cols].T)
