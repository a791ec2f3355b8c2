"""shll_tube_run_static: the entry point for callers that cannot allocate device memory.

It must give the same tube as the context API (shll_create + shll_step), within the tolerance of
the mixed-precision tests (L1 <= 1e-6 per variable), on two calls in a row with different tubes,
so that whatever the first call leaves in the library's static scratch cannot leak into the
second.  This file is collected last so that a run stopping at the first failure has already run
every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def conserved_from_primitives(p, prim):
    # the FP64 initial state exactly as the context API forms it (U from P)
    cv = p.R / (p.gamma - 1.0)
    rho, u, T = prim
    return np.stack([rho, rho * u, rho * (T * cv + 0.5 * u * u)])


def run_context(shll, p, prim, steps):
    ctx = shll.Context(p)
    ctx.set_primitives(prim[0], prim[1], prim[2])
    ctx.step(steps)
    out = ctx.conserved()
    ctx.close()
    return out


def run_static(shll, torch, p, prim, steps):
    U = torch.tensor(conserved_from_primitives(p, prim), dtype=torch.float64, device="cuda").contiguous()
    L = shll.lib()
    L.shll_tube_run_static.argtypes = [ctypes.POINTER(shll.Params), ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p]
    L.shll_tube_run_static.restype = ctypes.c_int
    rc = L.shll_tube_run_static(ctypes.byref(p), ctypes.c_void_p(U.data_ptr()), steps, None)
    torch.cuda.synchronize()
    return rc, U.cpu().numpy()


def sod(n, x_d, rho_l, T_l):
    x = np.arange(n)
    left = x < x_d * n
    return np.stack([np.where(left, rho_l, 1.0), np.zeros(n), np.where(left, T_l, 1.0)])


def test_static_entry_matches_context_api_twice(shll):
    torch = pytest.importorskip("torch")
    cases = [  # (order, cells, steps, diaphragm, rho_l, T_l): a chunked tube, then a small one
        (2, 3000, 700, 0.5, 10.0, 1.0),
        (1, 900, 500, 0.35, 4.0, 1.5),
    ]
    for order, n, steps, xd, rl, tl in cases:
        p = shll.params(1, order, nx=n, precision="mixed_f64", ic_kind=shll.IC_USER)
        prim = sod(n, xd, rl, tl)
        ref = run_context(shll, p, prim, steps)
        rc, got = run_static(shll, torch, p, prim, steps)
        assert rc == 0
        err = np.mean(np.abs(got - ref), axis=1)
        assert np.all(err <= 1e-6), (order, n, err)
        u0 = conserved_from_primitives(p, prim)
        if order == 1:  # reflective walls: mass is conserved exactly as by the context API
            assert abs(got[0].sum() - u0[0].sum()) / u0[0].sum() <= 1e-12


def test_static_entry_rejects_oversized_tube(shll):
    torch = pytest.importorskip("torch")
    p = shll.params(1, 1, nx=65537, precision="mixed_f64")
    buf = torch.zeros(3 * 8, dtype=torch.float64, device="cuda")
    L = shll.lib()
    L.shll_tube_run_static.argtypes = [ctypes.POINTER(shll.Params), ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p]
    L.shll_tube_run_static.restype = ctypes.c_int
    assert L.shll_tube_run_static(ctypes.byref(p), ctypes.c_void_p(buf.data_ptr()), 10, None) == shll.ERR_ARG


def test_static_entry_validates_parameters_with_explicit_steps(shll):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(3 * 1024, dtype=torch.float64, device="cuda")
    L = shll.lib()
    L.shll_tube_run_static.argtypes = [ctypes.POINTER(shll.Params), ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p]
    L.shll_tube_run_static.restype = ctypes.c_int
    for field, value in (("gamma", 1.0), ("cfl", 0.0), ("limiter", 3)):
        p = shll.params(1, 1, nx=1024, precision="mixed_f64")
        setattr(p, field, value)
        assert L.shll_tube_run_static(ctypes.byref(p), ctypes.c_void_p(buf.data_ptr()), 50, None) == shll.ERR_ARG
    assert torch.count_nonzero(buf).item() == 0   # refused before any work on the buffer
