"""GPU tests of the 2D mixed-precision engine (first order with reflective walls, second order with
outflow walls) against the FP64 oracle (a restatement of base-c/base_shll_2d.c and
base-c/2nd_order_base_shll.c pinned bit for bit to the reference).

Tolerances: L1(rho, u, v, T) <= 1e-6 against the FP64 oracle; mass and energy conserved to
<= 1e-12 relative (reflective walls)."""
import numpy as np
import pytest

from helpers import l1

pytestmark = pytest.mark.gpu


def run(shll, p):
    ctx = shll.Context(p)
    ctx.init_state()
    t0 = ctx.totals()
    steps = ctx.run()
    out = ctx.primitives()
    t1 = ctx.totals()
    ctx.close()
    return steps, out, t0, t1


@pytest.mark.parametrize("prec", ["mixed_f64", "mixed_kahan"])
@pytest.mark.parametrize("nx,ny", [(16, 32), (40, 70), (64, 64), (100, 37), (2, 5)])
def test_box_vs_fp64_oracle(shll, oracle, prec, nx, ny):
    cfg = oracle.make_cfg(dim=2, order=1, nx=nx, ny=ny, t_end=0.1)
    steps, ref, _ = oracle.run(cfg, oracle.ic_ref_box2d(nx, ny))
    s, out, t0, t1 = run(shll, shll.params(2, 1, nx=nx, ny=ny, precision=prec, t_end=0.1))
    assert s == steps
    err = l1(out, ref)
    assert np.all(err <= 1e-6), err
    assert abs(t1[0] - t0[0]) / t0[0] <= 1e-12
    assert abs(t1[3] - t0[3]) / t0[3] <= 1e-12


@pytest.mark.parametrize("n,steps", [(96, 200), (130, 60)])
def test_circle_vs_fp64_oracle(shll, oracle, n, steps):
    cfg = oracle.make_cfg(dim=2, order=1, nx=n, ny=n, n_steps=steps)
    prim = oracle.ic_circle2d(n, n, r=0.25, rho_in=10.0, rho_out=1.0)
    _, ref, _ = oracle.run(cfg, prim)
    p = shll.params(2, 1, nx=n, ny=n, precision="mixed_f64", n_steps=steps, ic_kind=shll.IC_CIRCLE2D,
                    ic_cx=0.5, ic_cy=0.5, ic_radius=0.25, ic_rho_l=10.0, ic_T_l=1.0, ic_rho_r=1.0, ic_T_r=1.0)
    s, out, t0, t1 = run(shll, p)
    assert s == steps
    assert np.all(l1(out, ref) <= 1e-6)
    assert abs(t1[0] - t0[0]) / t0[0] <= 1e-12


def test_partial_steps(shll, oracle):
    nx, ny = 48, 40
    cfg = oracle.make_cfg(dim=2, order=1, nx=nx, ny=ny, n_steps=50)
    _, ref, _ = oracle.run(cfg, oracle.ic_ref_box2d(nx, ny))
    ctx = shll.Context(shll.params(2, 1, nx=nx, ny=ny, precision="mixed_f64", n_steps=50))
    ctx.init_state()
    ctx.step(1)
    ctx.step(20)
    ctx.run()
    assert ctx.steps_taken == 50
    assert np.all(l1(ctx.primitives(), ref) <= 1e-6)


def test_batch_of_domains(shll, oracle):
    rng = np.random.default_rng(5)
    items, refs = [], []
    for k in range(6):
        n = int(rng.choice([20, 33, 64, 80]))
        r = float(rng.uniform(0.1, 0.35))
        rin = float(rng.uniform(2, 50))
        tin = float(rng.uniform(0.5, 2))
        steps = int(rng.integers(10, 60))
        items.append(shll.params(2, 1, nx=n, ny=n, precision="mixed_f64", n_steps=steps,
                                 ic_kind=shll.IC_CIRCLE2D, ic_cx=0.5, ic_cy=0.5, ic_radius=r, ic_rho_l=rin,
                                 ic_T_l=tin, ic_rho_r=1.0, ic_T_r=1.0))
        cfg = oracle.make_cfg(dim=2, order=1, nx=n, ny=n, n_steps=steps)
        refs.append(oracle.run(cfg, oracle.ic_circle2d(n, n, r=r, rho_in=rin, T_in=tin))[1])
    b = shll.Batch(items)
    b.run()
    for k, p in enumerate(items):
        assert np.all(l1(b.primitives(k), refs[k]) <= 1e-6), k


# ---- second order (base-c/2nd_order_base_shll.c:203-459 in x and y, outflow walls; the MC limiter
# of base-omp/2nd_order_base_shll.c:316-325) ----

@pytest.mark.parametrize("prec", ["mixed_f64", "mixed_kahan"])
@pytest.mark.parametrize("limiter,ic", [(0, "four_shock"), (1, "quadrants")])
@pytest.mark.parametrize("nx,ny,steps", [(16, 32, 40), (40, 70, 120), (64, 64, 200), (100, 37, 90), (2, 5, 20),
                                         (33, 65, 60)])
def test_second_order_vs_fp64_oracle(shll, oracle, prec, limiter, ic, nx, ny, steps):
    cfg = oracle.make_cfg(dim=2, order=2, nx=nx, ny=ny, n_steps=steps, limiter=limiter, mc_alpha=1.25)
    prim = oracle.ic_four_shock2d(nx, ny, 64) if ic == "four_shock" else oracle.ic_quadrants2d(nx, ny, 64)
    _, ref, _ = oracle.run(cfg, prim)
    kind = shll.IC_FOUR_SHOCK2D if ic == "four_shock" else shll.IC_QUADRANTS2D
    p = shll.params(2, 2, nx=nx, ny=ny, precision=prec, n_steps=steps, limiter=limiter, mc_alpha=1.25, ic_kind=kind)
    s, out, _, _ = run(shll, p)
    assert s == steps
    err = l1(out, ref)
    assert np.all(err <= 1e-6), err


def test_second_order_conserves_away_from_the_walls(shll, oracle):
    # a diaphragm well inside the domain: no wave reaches the outflow walls within 8 steps (two cells
    # of reach per step), so mass, momentum and energy are conserved to the rounding of the state
    n, steps = 64, 8
    p = shll.params(2, 2, nx=n, ny=n, precision="mixed_f64", n_steps=steps, ic_kind=shll.IC_CIRCLE2D, ic_cx=0.5,
                    ic_cy=0.5, ic_radius=0.15, ic_rho_l=20.0, ic_T_l=1.5, ic_rho_r=1.0, ic_T_r=1.0)
    _, out, t0, t1 = run(shll, p)
    cfg = oracle.make_cfg(dim=2, order=2, nx=n, ny=n, n_steps=steps)
    _, ref, _ = oracle.run(cfg, oracle.ic_circle2d(n, n, r=0.15, rho_in=20.0, T_in=1.5))
    assert np.all(l1(out, ref) <= 1e-6)
    assert abs(t1[0] - t0[0]) / t0[0] <= 1e-12
    assert abs(t1[3] - t0[3]) / t0[3] <= 1e-12


def test_second_order_batch_and_replay(shll, oracle):
    # several second-order domains of different sizes in one batch, run twice from a checkpoint (the
    # second run replays a captured graph): each equals its single-domain oracle run
    rng = np.random.default_rng(11)
    items, refs = [], []
    for k in range(5):
        n = int(rng.choice([20, 33, 48, 64]))
        r = float(rng.uniform(0.1, 0.3))
        rin = float(rng.uniform(2, 20))
        steps = int(rng.integers(10, 50))
        items.append(shll.params(2, 2, nx=n, ny=n, precision="mixed_f64", n_steps=steps, ic_kind=shll.IC_CIRCLE2D,
                                 ic_cx=0.5, ic_cy=0.5, ic_radius=r, ic_rho_l=rin, ic_T_l=1.0, ic_rho_r=1.0,
                                 ic_T_r=1.0))
        cfg = oracle.make_cfg(dim=2, order=2, nx=n, ny=n, n_steps=steps)
        refs.append(oracle.run(cfg, oracle.ic_circle2d(n, n, r=r, rho_in=rin))[1])
    import torch
    st = torch.cuda.Stream()
    b = shll.Batch(items)
    b.set_stream(st.cuda_stream)
    b.checkpoint()
    outs = []
    for _ in range(3):
        b.restore()
        b.run()
        outs.append([b.primitives(k) for k in range(len(items))])
    b.close()
    for k in range(len(items)):
        assert np.all(l1(outs[0][k], refs[k]) <= 1e-6), k
        assert np.array_equal(outs[0][k], outs[2][k])


def test_second_order_batch_needs_one_limiter(shll):
    items = [shll.params(2, 2, nx=32, ny=32, precision="mixed_f64", limiter=lim, mc_alpha=1.25) for lim in (0, 1)]
    with pytest.raises(shll.ShllError):
        shll.Batch(items)


def test_checkpoint_restore_and_graph_replay(shll):
    # runs 2 and 3 from the same checkpoint replay a captured graph; all equal the direct launches
    items = [shll.params(2, 1, nx=n, ny=n, precision="mixed_f64", n_steps=70, ic_kind=shll.IC_CIRCLE2D, ic_cx=0.5,
                         ic_cy=0.5, ic_radius=0.3, ic_rho_l=9.0, ic_T_l=1.4, ic_rho_r=1.0, ic_T_r=1.0)
             for n in (48, 96)]
    import torch
    s = torch.cuda.Stream()
    b = shll.Batch(items)
    b.set_stream(s.cuda_stream)
    b.checkpoint()
    outs, launches = [], []
    for _ in range(3):
        b.restore()
        l0 = shll.kernel_launches()
        b.run()
        launches.append(shll.kernel_launches() - l0)
        outs.append([b.primitives(i) for i in range(len(items))])
    shll.set_graph_replay(False)
    try:
        b.restore()
        b.run()
        direct = [b.primitives(i) for i in range(len(items))]
    finally:
        shll.set_graph_replay(True)
    b.close()
    assert launches[0] == launches[1] == launches[2]
    for o in outs[1:] + [direct]:
        for x, y in zip(outs[0], o):
            assert np.array_equal(x, y)


def test_autotune_picks_a_fold_window_and_restores_the_state(shll, oracle):
    n, steps = 80, 120
    p = shll.params(2, 1, nx=n, ny=n, precision="mixed_f64", n_steps=steps, ic_kind=shll.IC_CIRCLE2D, ic_cx=0.5,
                    ic_cy=0.5, ic_radius=0.25, ic_rho_l=10.0, ic_T_l=1.0, ic_rho_r=1.0, ic_T_r=1.0)
    _, ref, _ = oracle.run(oracle.make_cfg(dim=2, order=1, nx=n, ny=n, n_steps=steps),
                           oracle.ic_circle2d(n, n, r=0.25, rho_in=10.0, rho_out=1.0))
    b = shll.Batch([p])
    cu0 = b.cell_updates
    b.autotune(64)
    sweep, fold, tile = b.tuning(0)
    # (the first value: time steps per step launch, one or two)
    assert sweep in (1, 2) and tile == 512 and fold in (16, 32, 64)
    assert b.cell_updates == cu0
    b.run()
    assert np.all(l1(b.primitives(0), ref) <= 1e-6)
    assert b.item_status(0) == 0
    b.close()



def _domains_run(shll, items, kstep, monkeypatch):
    # SHLL_2D_STEPS_PER_LAUNCH sets how many time steps a step launch takes for states created
    # while it is set (the fold window is given, so no tuned choice replaces it)
    monkeypatch.setenv("SHLL_2D_STEPS_PER_LAUNCH", str(kstep))
    b = shll.Batch(items)
    assert b.tuning(0)[0] == kstep
    t0 = [b.totals(i) for i in range(len(items))]
    b.run()
    out = [b.primitives(i) for i in range(len(items))]
    t1 = [b.totals(i) for i in range(len(items))]
    b.close()
    return out, t0, t1


@pytest.mark.parametrize("prec", ["mixed_f64", "mixed_kahan"])
@pytest.mark.parametrize("fold", [16, 64])
def test_two_steps_per_launch_vs_fp64_oracle(shll, oracle, monkeypatch, prec, fold):
    # the two-step kernel (a 20x36 window, the halo cells' first step taken in the tile's own frame,
    # the edge corrections of both steps applied by the next launch) rounds differently from one
    # step per launch; both stay within the tolerance of the FP64 oracle and conserve mass and
    # energy.  Domains smaller and larger than a window, odd step counts (a last single step), a
    # fold window cut by the run's end.
    rng = np.random.default_rng(fold)
    items, refs = [], []
    for nx, ny, k in ((7, 5, 33), (20, 36, 40), (93, 61, 101), (160, 144, 77), (2, 300, 64)):
        cx, cy = float(rng.uniform(0.3, 0.7)), float(rng.uniform(0.3, 0.7))
        r, rin = float(rng.uniform(0.1, 0.3)), float(rng.uniform(2, 10))
        items.append(shll.params(2, 1, nx=nx, ny=ny, precision=prec, n_steps=k, fold_steps=fold,
                                 ic_kind=shll.IC_CIRCLE2D, ic_cx=cx, ic_cy=cy, ic_radius=r, ic_rho_l=rin,
                                 ic_T_l=1.0, ic_rho_r=1.0, ic_T_r=1.0))
        cfg = oracle.make_cfg(dim=2, order=1, nx=nx, ny=ny, n_steps=k)
        refs.append(oracle.run(cfg, oracle.ic_circle2d(nx, ny, cx=cx, cy=cy, r=r, rho_in=rin))[1])
    outs = {}
    for kstep in (1, 2):
        out, t0, t1 = _domains_run(shll, items, kstep, monkeypatch)
        for i in range(len(items)):
            assert np.all(l1(out[i], refs[i]) <= 1e-6), (kstep, i)
            for q in (0, 3):
                assert abs(t1[i][q] - t0[i][q]) / t0[i][q] <= 1e-12, (kstep, i, q)
        outs[kstep] = out
    for a, b in zip(outs[1], outs[2]):
        assert np.all(l1(a, b) <= 1e-6)


@pytest.mark.parametrize("order,kstep", [(1, 1), (1, 2), (2, 1)])
def test_pair_accesses_equal_per_cell_accesses(shll, order, kstep, monkeypatch):
    # domains with even row lengths load and store their cell pairs with 8-byte accesses; the
    # per-cell accesses of the general path give the same bits (one and two steps per launch)
    monkeypatch.setenv("SHLL_2D_STEPS_PER_LAUNCH", str(kstep))

    def once():
        items = [shll.params(2, order, nx=n, ny=m, precision="mixed_f64", n_steps=37, ic_kind=shll.IC_CIRCLE2D,
                             ic_cx=0.45, ic_cy=0.55, ic_radius=0.3, ic_rho_l=8.0, ic_T_l=1.3, ic_rho_r=1.0,
                             ic_T_r=1.0, fold_steps=16)
                 for n, m in ((48, 40), (97, 64), (34, 34))]   # (ny <= nx: the y CFL number stays <= 0.25)
        b = shll.Batch(items)
        b.run()
        out = [b.primitives(k) for k in range(len(items))]
        b.close()
        return out
    pairs = once()
    monkeypatch.setenv("SHLL_2D_SCALAR_PAIRS", "1")
    cells = once()
    for x, y in zip(pairs, cells):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("limiter,ic", [(0, "four_shock"), (1, "quadrants")])
def test_second_order_many_tiles_vs_fp64_oracle(shll, oracle, limiter, ic):
    # 16 x 4 tiles (256 x 128 cells, 8-byte pair accesses), 150 steps: every interior tile edge and
    # its reconciliation in use
    nx, ny, steps = 256, 128, 150
    cfg = oracle.make_cfg(dim=2, order=2, nx=nx, ny=ny, n_steps=steps, limiter=limiter, mc_alpha=1.25)
    prim = oracle.ic_four_shock2d(nx, ny, 64) if ic == "four_shock" else oracle.ic_quadrants2d(nx, ny, 64)
    _, ref, _ = oracle.run(cfg, prim)
    kind = shll.IC_FOUR_SHOCK2D if ic == "four_shock" else shll.IC_QUADRANTS2D
    p = shll.params(2, 2, nx=nx, ny=ny, precision="mixed_f64", n_steps=steps, limiter=limiter, mc_alpha=1.25,
                    ic_kind=kind)
    s, out, _, _ = run(shll, p)
    assert s == steps
    assert np.all(l1(out, ref) <= 1e-6), l1(out, ref)
