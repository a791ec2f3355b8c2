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


def _ref_main():
    mod = load_pkg()
    return os.path.join(os.path.dirname(mod.lib()._name), "shll_ref_main")


@pytest.mark.gpu
def test_reference_style_main_runs_unchanged(oracle):
    # host/shll_ref_main.c: the reference program's globals and time loop (its own float clock, the
    # DT global set by the library's Compute_U_from_P), N = 1024: the published 1639 steps and the
    # published FP32 results
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([_ref_main()], cwd=d, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        res = np.loadtxt(os.path.join(d, "results.dat"))
    assert "Completed in 1639 steps" in r.stdout
    n = 1024
    _, ref, _ = oracle.run(oracle.make_cfg(nx=n, real_bits=32), oracle.ic_sod(n))
    for c in range(3):
        got, want = res[:, 1 + c], ref[c]
        assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-3)) < 1e-6, c


REF_SRC = os.environ.get("SHLL_REFERENCE_ROOT", "/root/reference")


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_SRC, "base-c", "base_shll.c")),
                    reason="the reference's sources are not present")
def test_reference_program_links_against_the_library():
    # the reference's own base-c/base_shll.c with only its stage-function definitions removed (its
    # globals and main() as published) links against libshll_gb300 (nothing runs: no GPU here)
    src = open(os.path.join(REF_SRC, "base-c", "base_shll.c")).read().replace("\r", "")
    stages = ("Allocate_and_Init_Memory", "Free_Memory", "Compute_U_from_P", "Update_U_from_F",
              "Compute_F_from_P", "Compute_P_from_U", "Save_Results")
    out, skip = [], False
    for line in src.split("\n"):
        if any(line.startswith(f"void {s}(") for s in stages):
            skip = True
            continue
        if skip:
            skip = line != "}"
            continue
        out.append(line)
    text = "\n".join(out)
    assert "int main()" in text and all(f"void {s}(" not in text for s in stages)
    lib = load_pkg().lib()._name
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "main.c")
        open(c, "w").write('#include "shll.h"\n' + text)
        inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
        r = subprocess.run(["gcc", "-O2", "-I", inc, c, "-o", os.path.join(d, "main"), "-L", os.path.dirname(lib),
                            "-lshll_gb300", "-lm"], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        syms = subprocess.run(["nm", "-D", os.path.join(d, "main")], capture_output=True, text=True).stdout
        # the program exports its DT (which the library writes) and its problem constants
        for name in ("DT", "N", "TOTAL_TIME"):
            assert any(l.split()[-1] == name for l in syms.splitlines() if l.strip()), name
