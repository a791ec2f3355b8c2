"""GPU parity of the plain (reference-arithmetic) kernels against the CPU oracle.

SHLL_PREC_F64_EXACT / F32_EXACT must equal the oracle bit for bit (the oracle is itself pinned
bit for bit to the reference's gcc builds, see test_oracle.py).  SHLL_PREC_F64 (fused
multiply-add allowed) must stay within a max per-cell relative difference of 1e-10."""
import glob
import os
import tempfile

import numpy as np
import pytest

from helpers import max_rel_scaled

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

CASES_1D = [(1, 2), (1, 3), (1, 33), (1, 256), (1, 1000), (2, 2), (2, 5), (2, 64), (2, 1024)]
CASES_2D = [(1, 16, 16), (1, 33, 7), (1, 64, 48), (2, 16, 16), (2, 32, 24), (2, 9, 40)]


def oracle_1d(O, order, n, bits, **kw):
    cfg = O.make_cfg(dim=1, order=order, nx=n, real_bits=bits, **kw)
    return O.run(cfg, O.ic_sod(n))


def oracle_2d(O, order, nx, ny, bits, **kw):
    t_end = 0.1 if order == 1 else 0.2
    cfg = O.make_cfg(dim=2, order=order, nx=nx, ny=ny, real_bits=bits, t_end=t_end, **kw)
    prim = O.ic_ref_box2d(nx, ny) if order == 1 else O.ic_four_shock2d(nx, ny, bits)
    return O.run(cfg, prim)


def gpu_run(shll, p):
    ctx = shll.Context(p)
    ctx.init_state()
    steps = ctx.run()
    out = ctx.primitives()
    cons = ctx.conserved()
    ctx.close()
    return steps, out, cons


@pytest.mark.parametrize("order,n", CASES_1D)
@pytest.mark.parametrize("prec,bits", [("f64_exact", 64), ("f32_exact", 32)])
def test_exact_1d_bitwise(shll, oracle, order, n, prec, bits):
    steps, ref, _ = oracle_1d(oracle, order, n, bits)
    s, out, _ = gpu_run(shll, shll.params(1, order, nx=n, precision=prec, t_end=0.2))
    assert s == steps
    assert np.array_equal(out, ref), f"max abs diff {np.abs(out - ref).max()}"


@pytest.mark.parametrize("order,nx,ny", CASES_2D)
@pytest.mark.parametrize("prec,bits", [("f64_exact", 64), ("f32_exact", 32)])
def test_exact_2d_bitwise(shll, oracle, order, nx, ny, prec, bits):
    steps, ref, _ = oracle_2d(oracle, order, nx, ny, bits)
    p = shll.params(2, order, nx=nx, ny=ny, precision=prec, t_end=0.1 if order == 1 else 0.2)
    s, out, _ = gpu_run(shll, p)
    assert s == steps
    assert np.array_equal(out, ref), f"max abs diff {np.abs(out - ref).max()}"


@pytest.mark.parametrize("prec,bits", [("f64_exact", 64), ("f32_exact", 32)])
def test_exact_mc_limiter_bitwise(shll, oracle, prec, bits):
    cfg = oracle.make_cfg(dim=2, order=2, nx=32, ny=32, real_bits=bits, t_end=0.05, limiter=1, mc_alpha=1.25)
    steps, ref, _ = oracle.run(cfg, oracle.ic_quadrants2d(32, 32, bits))
    p = shll.params(2, 2, nx=32, ny=32, precision=prec, t_end=0.05, limiter=1, mc_alpha=1.25,
                    ic_kind=shll.IC_QUADRANTS2D)
    s, out, _ = gpu_run(shll, p)
    assert s == steps and np.array_equal(out, ref)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_golden_fixture_on_gpu(shll, path):
    g = np.load(path)
    prec = "f32_exact" if int(g["bits"]) == 32 else "f64_exact"
    dim, order = int(g["dim"]), int(g["order"])
    ic = str(g["ic"])
    kind = {"sod": shll.IC_SOD, "box": shll.IC_REF_BOX2D, "four_shock": shll.IC_FOUR_SHOCK2D,
            "quadrants": shll.IC_QUADRANTS2D}[ic]
    p = shll.params(dim, order, nx=int(g["nx"]), ny=int(g["ny"]), precision=prec, t_end=float(g["t_end"]),
                    ic_kind=kind, limiter=int(g["limiter"]) if "limiter" in g else 0)
    if kind == shll.IC_SOD:
        p.ic.x_d, p.ic.rho_l, p.ic.T_l, p.ic.rho_r, p.ic.T_r = 0.5, 10.0, 1.0, 1.0, 1.0
    s, out, _ = gpu_run(shll, p)
    assert s == int(g["steps"])
    assert np.array_equal(out, g["prim"])


@pytest.mark.parametrize("dim,order,n", [(1, 1, 1024), (1, 2, 1024), (1, 1, 4096), (2, 1, 64), (2, 2, 48)])
def test_f64_fma_within_1e10(shll, oracle, dim, order, n):
    if dim == 1:
        steps, ref, _ = oracle_1d(oracle, order, n, 64)
        p = shll.params(1, order, nx=n, precision="f64")
    else:
        steps, ref, _ = oracle_2d(oracle, order, n, n, 64)
        p = shll.params(2, order, nx=n, ny=n, precision="f64", t_end=0.1 if order == 1 else 0.2)
    s, out, _ = gpu_run(shll, p)
    assert s == steps
    assert max_rel_scaled(out, ref) <= 1e-10


@pytest.mark.parametrize("dim,order,prec", [(1, 1, "f64_exact"), (1, 2, "f32_exact"), (2, 1, "f64_exact"),
                                            (2, 2, "f64_exact")])
def test_staged_reference_loop_equals_fused(shll, dim, order, prec):
    p = shll.params(dim, order, nx=40, ny=24, precision=prec, n_steps=30)
    a = shll.Context(p)
    a.init_state()
    for _ in range(30):
        a.compute_F_from_P()
        a.update_U_from_F()
        a.compute_P_from_U()
    staged = a.primitives()
    b = shll.Context(p)
    b.init_state()
    b.run()
    assert np.array_equal(staged, b.primitives())


@pytest.mark.parametrize("dim", [1, 2])
def test_split_fluxes_match_oracle(shll, oracle, dim):
    n, ny = (64, 1) if dim == 1 else (12, 10)
    p = shll.params(dim, 1, nx=n, ny=ny, precision="f64_exact", n_steps=3)
    ctx = shll.Context(p)
    ctx.init_state()
    ctx.step(3)
    cons = ctx.conserved()
    ctx.compute_F_from_P()
    got = ctx.fluxes()
    ref = oracle.split_fluxes(oracle.make_cfg(dim=dim, nx=n, ny=ny, real_bits=64), cons)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)


def test_reference_entry_point_names(shll, oracle):
    L = shll.lib()
    p = shll.params(1, 1, nx=128, precision="f64_exact")
    assert L.shll_ref_configure(p) == 0
    L.Allocate_and_Init_Memory()
    L.Compute_U_from_P()
    L.Compute_P_from_U()
    steps = shll.steps_for(p)
    for _ in range(steps):
        L.Compute_F_from_P()
        L.Update_U_from_F()
        L.Compute_P_from_U()
    ctx = L.shll_ref_context()
    out = np.zeros((3, 128))
    dp = lambda a: a.ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_double))
    assert L.shll_get_primitives(ctx, dp(out[0]), dp(out[1]), None, dp(out[2])) == 0
    L.Free_Memory()
    _, ref, _ = oracle_1d(oracle, 1, 128, 64)
    assert np.array_equal(out, ref)


def test_save_results_format(shll, oracle):
    n = 64
    ctx = shll.Context(shll.params(1, 1, nx=n, precision="f32_exact"))
    ctx.init_state()
    ctx.run()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "results.dat")
        ctx.save_results(path)
        lines = open(path).read().splitlines()
    assert len(lines) == n
    _, ref, _ = oracle_1d(oracle, 1, n, 32)
    dx = np.float32(1.0) / np.float32(n)
    for i in (0, 17, n - 1):
        cols = lines[i].split("\t")
        assert len(cols) == 4
        expect = [float(np.float32((i + 0.5) * dx)), ref[0][i], ref[1][i], ref[2][i]]
        assert cols == ["%e" % v for v in expect]


def test_totals_and_conservation(shll):
    ctx = shll.Context(shll.params(1, 1, nx=1000, precision="f64"))
    ctx.init_state()
    t0 = ctx.totals()
    ctx.run()
    t1 = ctx.totals()
    cons = ctx.conserved()
    assert np.allclose(t1, cons.sum(axis=1), rtol=1e-13, atol=1e-12)
    assert abs(t1[0] - t0[0]) / t0[0] < 1e-13  # reflective walls conserve mass
    assert abs(t1[2] - t0[2]) / t0[2] < 1e-13  # and energy


def test_user_primitives(shll, oracle):
    n = 300
    x = (np.arange(n) + 0.5) / n
    rho = 1.0 + 0.5 * np.sin(2 * np.pi * x)
    u = 0.1 * np.cos(2 * np.pi * x)
    T = 1.0 + 0.2 * x
    p = shll.params(1, 2, nx=n, precision="f64_exact", ic_kind=shll.IC_USER, n_steps=200)
    ctx = shll.Context(p)
    ctx.set_primitives(rho, u, T)
    ctx.run()
    _, ref, _ = oracle.run(oracle.make_cfg(order=2, nx=n, n_steps=200), np.stack([rho, u, T]))
    assert np.array_equal(ctx.primitives(), ref)


def test_call_order_errors(shll):
    ctx = shll.Context(shll.params(1, 1, nx=16))
    with pytest.raises(shll.ShllError) as e:
        ctx.compute_F_from_P()
    assert e.value.status == shll.ERR_STATE
    ctx.init_state()
    with pytest.raises(shll.ShllError) as e:
        ctx.update_U_from_F()
    assert e.value.status == shll.ERR_STATE
    m = shll.Context(shll.params(1, 1, nx=16, precision="mixed_f64"))
    m.init_state()
    with pytest.raises(shll.ShllError) as e:
        m.compute_F_from_P()
    assert e.value.status == shll.ERR_UNSUPPORTED
    with pytest.raises(shll.ShllError) as e:
        ctx.set_primitives(np.zeros(16), np.zeros(16), np.ones(16))
    assert e.value.status == shll.ERR_ARG


def test_plain_fp64_batch_1d_matches_oracle(shll, oracle):
    # the one-launch-per-step FP64 schedule over many tubes of different sizes, orders and data
    rng = np.random.default_rng(11)
    items, refs = [], []
    for k in range(10):
        n = int(rng.integers(3, 700))
        order = 1 + k % 2
        xd, rl, tl = float(rng.uniform(0.3, 0.7)), float(rng.uniform(2, 20)), float(rng.uniform(0.5, 2))
        items.append(shll.params(1, order, nx=n, precision="f64", ic_x_d=xd, ic_rho_l=rl, ic_T_l=tl))
        cfg = oracle.make_cfg(order=order, nx=n)
        refs.append(oracle.run(cfg, oracle.ic_sod(n, x_d=xd, rhoL=rl, TL=tl))[1])
    b = shll.Batch(items)
    b.run()
    for k in range(len(items)):
        assert max_rel_scaled(b.primitives(k), refs[k]) <= 1e-10, k
    assert b.cell_updates == sum(p.nx * shll.steps_for(p) for p in items)


def test_plain_fp64_batch_2d_matches_oracle(shll, oracle):
    items, refs = [], []
    for k, (n, r) in enumerate([(20, 0.2), (37, 0.3), (64, 0.15)]):
        items.append(shll.params(2, 1, nx=n, ny=n, precision="f64", n_steps=40 + 10 * k, ic_kind=shll.IC_CIRCLE2D,
                                 ic_cx=0.5, ic_cy=0.5, ic_radius=r, ic_rho_l=10.0, ic_T_l=1.0, ic_rho_r=1.0,
                                 ic_T_r=1.0))
        cfg = oracle.make_cfg(dim=2, order=1, nx=n, ny=n, n_steps=40 + 10 * k)
        refs.append(oracle.run(cfg, oracle.ic_circle2d(n, n, r=r))[1])
    b = shll.Batch(items)
    b.run()
    for k in range(len(items)):
        assert max_rel_scaled(b.primitives(k), refs[k]) <= 1e-10, k


@pytest.mark.parametrize("prec", ["f64", "mixed_f64"])
def test_batch_flags_the_items_that_break_down(shll, oracle, prec):
    # The reference's second-order scheme itself breaks down (NaN) on a Sod tube with density
    # ratio 100 and temperature ratio 2; the batch reports that item and finishes the others.
    specs = [(1, 300, 10.0, 1.0), (2, 512, 100.0, 2.0), (2, 200, 5.0, 1.0)]
    items = [shll.params(1, o, nx=n, precision=prec, ic_rho_l=rl, ic_T_l=tl) for o, n, rl, tl in specs]
    refs = [oracle.run(oracle.make_cfg(order=o, nx=n), oracle.ic_sod(n, rhoL=rl, TL=tl))[1] for o, n, rl, tl in specs]
    assert np.isnan(refs[1]).any() and not np.isnan(refs[0]).any()
    b = shll.Batch(items)
    assert b.run(allow_numeric=True) == shll.ERR_NUMERIC
    assert [b.item_status(i) for i in range(3)] == [shll.OK, shll.ERR_NUMERIC, shll.OK]
    tol = 1e-10 if prec == "f64" else 1e-6
    for i in (0, 2):
        got = b.primitives(i)
        err = max_rel_scaled(got, refs[i]) if prec == "f64" else np.max(np.mean(np.abs(got - refs[i]), axis=1))
        assert err <= tol, (i, err)


def test_results_file_reads_like_the_reference_plot_script(shll):
    # base-c/fetch_local.py: np.genfromtxt('./results.dat'), columns x y rho ux uy T, each reshaped
    # to (NX, NY); a non-square grid so that a transposed layout would show
    nx, ny = 40, 24
    ctx = shll.Context(shll.params(2, 1, nx=nx, ny=ny, precision="mixed_f64", n_steps=30))
    ctx.init_state()
    ctx.run()
    prim = ctx.primitives()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "results.dat")
        ctx.save_results(path)
        data = np.genfromtxt(path)
    ctx.close()
    assert data.shape == (nx * ny, 6)
    x_grid, y_grid, rho_grid = (data[:, k].reshape((nx, ny)) for k in (0, 1, 2))
    T_grid = data[:, 5].reshape((nx, ny))
    assert np.allclose(x_grid[:, 0], (np.arange(nx) + 0.5) / nx, rtol=1e-6)
    assert np.all(x_grid == x_grid[:, :1]) and np.all(y_grid == y_grid[:1, :])
    assert np.allclose(y_grid[0], (np.arange(ny) + 0.5) / ny, rtol=1e-6)
    assert np.allclose(rho_grid, prim[0].reshape(nx, ny), rtol=1e-6)
    assert np.allclose(T_grid, prim[3].reshape(nx, ny), rtol=1e-6)
