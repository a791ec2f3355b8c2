"""CPU tests of the oracle (test infrastructure): pinned to the reference's own solvers through
the committed golden fixtures (tests/golden, generated from the reference sources by
make_golden.py) and, when the reference executables are present (oracle/_ref), live."""
import glob
import os
import tempfile

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_cases():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def oracle_for(O, g):
    meta = {k: g[k].item() for k in ("dim", "order", "nx", "ny", "bits", "t_end")}
    lim = int(g["limiter"]) if "limiter" in g else 0
    cfg = O.make_cfg(dim=meta["dim"], order=meta["order"], nx=meta["nx"], ny=meta["ny"], real_bits=meta["bits"],
                     t_end=meta["t_end"], limiter=lim, mc_alpha=1.25)
    ic = str(g["ic"])
    nx, ny, bits = meta["nx"], meta["ny"], meta["bits"]
    prim = {"sod": lambda: O.ic_sod(nx), "box": lambda: O.ic_ref_box2d(nx, ny),
            "four_shock": lambda: O.ic_four_shock2d(nx, ny, bits), "quadrants": lambda: O.ic_quadrants2d(nx, ny, bits)}[ic]()
    return cfg, prim


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_reference_fixture_bitwise(oracle, path):
    g = np.load(path)
    cfg, prim = oracle_for(oracle, g)
    steps, out, _ = oracle.run(cfg, prim)
    assert steps == int(g["steps"])
    assert np.array_equal(out, g["prim"]), f"max diff {np.abs(out - g['prim']).max()}"


def test_golden_fixtures_present():
    assert len(golden_cases()) >= 10


@pytest.mark.parametrize("n,steps", [(256, 410), (512, 820), (1024, 1639), (2048, 3277), (4096, 6554),
                                     (8192, 13108), (16384, 26215), (32768, 52429), (65536, 104858)])
def test_step_counts_match_reference_readme(oracle, n, steps):
    # README.md tables 1-2: cells vs time steps of base-c/base_shll.c (float time loop)
    for bits in (32, 64):
        assert oracle.count_steps(oracle.make_cfg(nx=n, real_bits=bits)) == steps


@pytest.mark.parametrize("name,cols,kw", [
    ("base_shll_f32_n1024", [1, 2, 3], dict(dim=1, order=1, nx=1024, real_bits=32)),
    ("base_shll_f64_n2048", [1, 2, 3], dict(dim=1, order=1, nx=2048, real_bits=64)),
    ("base_shll_f64_n8", [1, 2, 3], dict(dim=1, order=1, nx=8, real_bits=64)),
    ("base_shll_2d_f32_64x64", [2, 3, 4, 5], dict(dim=2, order=1, nx=64, ny=64, real_bits=32, t_end=0.1)),
    ("o2_2d_f64_64x64", [2, 3, 4, 5], dict(dim=2, order=2, nx=64, ny=64, real_bits=64, t_end=0.2)),
])
def test_oracle_matches_reference_live(oracle, name, cols, kw):
    if not oracle.ref_available(name):
        pytest.skip("reference executables not built here (oracle/make_ref.sh)")
    cfg = oracle.make_cfg(**kw)
    with tempfile.TemporaryDirectory() as wd:
        steps, ref = oracle.run_ref(name, cols, wd)
    if cfg.dim == 1:
        prim = oracle.ic_sod(cfg.nx)
    elif cfg.order == 1:
        prim = oracle.ic_ref_box2d(cfg.nx, cfg.ny)
    else:
        prim = oracle.ic_four_shock2d(cfg.nx, cfg.ny, cfg.real_bits)
    s, out, _ = oracle.run(cfg, prim)
    assert s == steps
    assert np.array_equal(out, ref)


def test_riemann_exact_sod_structure(oracle):
    # Sod problem of base_shll.c at t = 0.2: left state, rarefaction, contact, shock, right state
    p = oracle.riemann_exact(1000, 0.2)
    rho, u, T = p
    assert rho[0] == pytest.approx(10.0) and rho[-1] == pytest.approx(1.0)
    assert np.all(u >= -1e-12)
    assert np.all(np.diff(rho[:480]) <= 1e-12)  # monotone through the rarefaction
    pstar = rho * T
    mid = pstar[(rho < 9.9) & (rho > 1.01)]
    assert mid.size > 0


@pytest.mark.parametrize("order,tol1024", [(1, 0.08), (2, 0.02)])
def test_scheme_converges_to_riemann_exact(oracle, order, tol1024):
    # SHLL on the Sod problem approaches the exact solution as N grows (measured here:
    # L1(rho) 0.059 / 0.023 at N = 1024 / 4096 for first order, 0.011 / 0.0033 for second order)
    errs = []
    for n in (1024, 4096):
        steps, out, _ = oracle.run(oracle.make_cfg(nx=n, order=order), oracle.ic_sod(n))
        ex = oracle.riemann_exact(n, steps * (0.125 / n))
        errs.append(np.mean(np.abs(out[0] - ex[0])))
    assert errs[0] < tol1024
    assert errs[1] < 0.6 * errs[0]


def test_oracle_conserves_mass_first_order(oracle):
    n = 512
    prim = oracle.ic_sod(n)
    _, _, cons = oracle.run(oracle.make_cfg(nx=n), prim)
    m0 = (prim[0]).sum()
    assert abs(cons[0].sum() - m0) / m0 < 1e-13


def test_oracle_rejects_bad_config(oracle):
    with pytest.raises(ValueError):
        oracle.run(oracle.make_cfg(nx=1), np.ones((3, 1)))


def test_threaded_stages_give_the_same_bits(oracle):
    # base-omp's calling pattern (a team running the stage loops) cannot change a result: every cell
    # of a stage is computed from the previous stage's arrays only
    cfg = oracle.make_cfg(dim=2, order=2, nx=96, ny=80, real_bits=32, limiter=1, mc_alpha=1.25, n_steps=40)
    prim = oracle.ic_quadrants2d(96, 80, 32)
    _, one, _ = oracle.run(cfg, prim)
    try:
        oracle.set_threads(4)
        _, four, _ = oracle.run(cfg, prim)
        cfg1 = oracle.make_cfg(dim=2, order=1, nx=64, ny=48, real_bits=64, n_steps=30)
        _, b4, _ = oracle.run(cfg1, oracle.ic_ref_box2d(64, 48))
    finally:
        oracle.set_threads(1)
    _, b1, _ = oracle.run(cfg1, oracle.ic_ref_box2d(64, 48))
    assert np.array_equal(one, four)
    assert np.array_equal(b1, b4)
