"""The OpenMP calling pattern of base-omp/2nd_order_base_shll.c:615-653 over the C-ABI.

libshll_gb300_omp gives the reference's stage names team semantics (one thread of the team runs
the stage on the GPU, the others wait at the stage's implicit barrier); shll_omp is base-omp's
main() over it.  CPU tests check the library's exports; GPU tests run the driver with a team and
alone and compare both with the oracle (second order, MC limiter, quadrant initial data).
"""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import load_pkg

TEAM_STAGES = ["Compute_U_from_P", "Compute_P_from_U", "Compute_F_from_P", "Update_U_from_F", "shll_omp_status"]


def _paths():
    mod = load_pkg()
    build = os.path.dirname(mod.lib()._name)
    return os.path.join(build, "libshll_gb300_omp.so"), os.path.join(build, "shll_omp")


def test_omp_library_exports_the_team_stages():
    lib_path, drv = _paths()
    if not os.path.exists(lib_path):
        pytest.skip("built without OpenMP")
    lib = ctypes.CDLL(lib_path)
    for name in TEAM_STAGES:
        assert hasattr(lib, name), name
    assert lib.shll_omp_status() == 0
    assert os.access(drv, os.X_OK)


def _run_driver(drv, n, threads, prec, steps):
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([drv, str(n), str(threads), prec, str(steps)], cwd=d, capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr
        assert f"Completed in {steps} steps ({threads} threads)" in r.stdout, r.stdout
        return np.loadtxt(os.path.join(d, "results.dat"))


@pytest.mark.gpu
@pytest.mark.parametrize("prec,bits", [("f64_exact", 64), ("f32_exact", 32)])
def test_omp_team_matches_serial_and_oracle(oracle, prec, bits):
    lib_path, drv = _paths()
    if not os.path.exists(lib_path):
        pytest.skip("built without OpenMP")
    n, steps = 48, 30
    team = _run_driver(drv, n, 4, prec, steps)
    alone = _run_driver(drv, n, 1, prec, steps)
    assert np.array_equal(team, alone)
    cfg = oracle.make_cfg(dim=2, order=2, nx=n, ny=n, real_bits=bits, n_steps=steps, t_end=0.3, limiter=1,
                          mc_alpha=1.25)
    _, prim, _ = oracle.run(cfg, oracle.ic_quadrants2d(n, n, bits))
    # results.dat columns: x y rho u v T, printed with %e (7 significant digits)
    for c in range(4):
        ref = prim[c]
        got = team[:, 2 + c]
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-3)) < 1e-6, c
