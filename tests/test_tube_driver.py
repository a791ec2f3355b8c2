"""The reference-style C driver over the C-ABI (shll-sve-cfd_gb300/host/shll_tube.c): the time
loop of base-c/base_shll.c:198-225 with the reference's own stage names, its step-count line
and its results.dat (x rho u T per cell, "%e" tab-separated)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import load_pkg


def _driver():
    mod = load_pkg()
    return os.path.join(os.path.dirname(mod.lib()._name), "shll_tube")


def test_driver_is_built():
    assert os.access(_driver(), os.X_OK)


def _run(n, order, prec):
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([_driver(), str(n), str(order), prec], cwd=d, capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr
        return r.stdout, np.loadtxt(os.path.join(d, "results.dat"))


@pytest.mark.gpu
def test_driver_published_fp32_matches_oracle(oracle):
    # 1024 cells, first order, the published FP32 arithmetic: the reference's 1639 steps, and
    # results.dat equal to the oracle's FP32 run to the 7 significant digits that "%e" prints
    n = 1024
    out, res = _run(n, 1, "f32_exact")
    assert "Completed in 1639 steps" in out
    steps, ref, _ = oracle.run(oracle.make_cfg(nx=n, real_bits=32), oracle.ic_sod(n))
    assert steps == 1639
    assert res.shape == (n, 4)
    np.testing.assert_allclose(res[:, 0], (np.arange(n) + 0.5) / n, rtol=1e-6)
    for c in range(3):   # rho, u, T
        got, want = res[:, 1 + c], ref[c]
        assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-3)) < 1e-6, c


@pytest.mark.gpu
def test_driver_mixed_precision_run(oracle):
    n = 2048
    out, res = _run(n, 2, "mixed_f64")
    steps, ref, _ = oracle.run(oracle.make_cfg(order=2, nx=n), oracle.ic_sod(n))
    assert f"Completed in {steps} steps" in out
    assert np.mean(np.abs(res[:, 1] - ref[0])) < 1e-5
