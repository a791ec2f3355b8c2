"""Resident runs of the mixed 1D engine (one cooperative launch per run, each chunk waiting only
for its neighbours' previous sweep, frames and owned cells' pairs kept on chip within a fold
window) against the one-launch-per-sweep schedule: the results must be bit-identical, and the
launch counts show which schedule ran."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ctx_run(shll, p, calls, resident):
    """advances one context by the step counts in calls; returns primitives, totals, launches"""
    shll.set_resident(resident)
    try:
        c = shll.Context(p)
        c.init_state()
        n0 = shll.kernel_launches()
        for k in calls:
            c.step(k)
        launches = shll.kernel_launches() - n0
        out, tot = c.primitives(), c.totals()
        c.close()
    finally:
        shll.set_resident(True)
    return out, tot, launches


def _batch_run(shll, items, resident):
    shll.set_resident(resident)
    try:
        b = shll.Batch(items)
        n0 = shll.kernel_launches()
        b.run()
        launches = shll.kernel_launches() - n0
        out = [b.primitives(i) for i in range(len(items))]
        tot = [b.totals(i) for i in range(len(items))]
        b.close()
    finally:
        shll.set_resident(True)
    return out, tot, launches


CASES = [
    # (order, cells, precision, extra params); fold_steps given, so that no tuned choice applies
    (2, 65536, "mixed_f64", {"fold_steps": 64}),
    (2, 65536, "mixed_f64", {"fold_steps": 128}),
    (2, 20000, "mixed_kahan", {"fold_steps": 64}),
    (1, 30000, "mixed_f64", {"fold_steps": 64}),
    (1, 30000, "mixed_kahan", {"fold_steps": 32}),
    (2, 9000, "mixed_f64", {"fold_steps": 64, "cfl": 0.3, "limiter": 1, "mc_alpha": 1.25}),
    (1, 5000, "mixed_f64", {"fold_steps": 16, "cfl": 0.3}),
]


@pytest.mark.parametrize("order,n,prec,extra", CASES)
def test_resident_matches_launch_per_sweep(shll, order, n, prec, extra):
    p = shll.params(1, order, nx=n, precision=prec, **extra)
    calls = [16 * 37 + 5]   # a partial last sweep and a fold window cut by the run's end
    a, ta, la = _ctx_run(shll, p, calls, resident=False)
    b, tb, lb = _ctx_run(shll, p, calls, resident=True)
    # resident launch + fix-up (first order: + the start-of-run pair-flux flags), against one
    # launch per sweep
    assert lb == (3 if order == 1 else 2) and la > 30
    assert np.array_equal(a, b)
    assert np.array_equal(ta, tb)


def test_resident_run_sequence(shll):
    p = shll.params(1, 2, nx=40000, precision="mixed_f64", fold_steps=128)
    calls = [7, 100, 16, 333, 1]
    a, ta, _ = _ctx_run(shll, p, calls, resident=False)
    b, tb, lb = _ctx_run(shll, p, calls, resident=True)
    assert lb == 2 * len(calls)
    assert np.array_equal(a, b)
    assert np.array_equal(ta, tb)


def test_resident_batch_of_tubes(shll):
    # several tubes of one variant in one resident launch, of different sizes, initial states and
    # step counts (their blocks finish at different sweeps)
    rng = np.random.default_rng(5)
    items = [shll.params(1, 2, nx=int(n), precision="mixed_f64", n_steps=int(k), fold_steps=64,
                         ic_rho_l=float(rng.uniform(2, 10)), ic_x_d=float(rng.uniform(0.3, 0.7)))
             for n, k in ((3000, 700), (11000, 333), (7000, 1000), (20000, 517))]
    a, ta, la = _batch_run(shll, items, resident=False)
    b, tb, lb = _batch_run(shll, items, resident=True)
    assert lb == 2 and la > 30
    for i in range(len(items)):
        assert np.array_equal(a[i], b[i]), i
        assert np.array_equal(ta[i], tb[i])


def fp64_sod(shll, n, order=2):
    # the bit-exact FP64 path (the oracle's arithmetic) on the Sod tube
    c = shll.Context(shll.params(1, order, nx=n, precision="f64_exact"))
    c.init_state()
    c.run()
    out = c.primitives()
    c.close()
    return out


def test_resident_full_sod_run_vs_exact_riemann(shll, oracle):
    # the whole second-order run of a 16384-cell tube as one launch: mass conserved and the
    # solution at the exact Riemann solution's distance
    n = 16384
    c = shll.Context(shll.params(1, 2, nx=n, precision="mixed_f64", fold_steps=128))
    c.init_state()
    t0 = c.totals()
    n0 = shll.kernel_launches()
    steps = c.run()
    assert shll.kernel_launches() - n0 == 2
    t1 = c.totals()
    ex = oracle.riemann_exact(n, steps * (0.125 / n))
    e_mixed = np.mean(np.abs(c.primitives()[0] - ex[0]))
    e_fp64 = np.mean(np.abs(fp64_sod(shll, n)[0] - ex[0]))
    assert abs(e_mixed - e_fp64) <= 0.1 * e_fp64, (e_mixed, e_fp64)
    assert abs(t1[0] - t0[0]) / t0[0] <= 1e-12
    c.close()


def test_resident_wait_runs_out_and_is_reported(shll):
    # a chunk that never publishes its progress (test hook): its neighbours' bounded waits give
    # up, the other blocks follow as soon as they see the flag, the run reports SHLL_ERR_TIMEOUT
    # within seconds, and the device stays usable
    p = shll.params(1, 2, nx=20000, precision="mixed_f64", fold_steps=64)
    shll.debug_stall_chunk(3)
    try:
        c = shll.Context(p)
        c.init_state()
        t = time.time()
        with pytest.raises(shll.ShllError) as e:
            c.step(16 * 10)
        assert e.value.status == shll.ERR_TIMEOUT
        assert time.time() - t < 20
        c.close()
    finally:
        shll.debug_stall_chunk(-1)
    out, _, launches = _ctx_run(shll, p, [16 * 10], resident=True)
    assert launches == 2 and np.isfinite(out).all()


def test_tuned_sod_tube_resident_equals_launch_per_sweep(shll, oracle):
    # the benchmark's configuration: 65536 cells, second order, autotuned (the longest sweep whose
    # chunks fit one per SM); the resident run and the launch-per-sweep run of the same tuned
    # chunks give the same bits, close to the exact Riemann solution, with mass conserved
    n = 65536
    p = shll.params(1, 2, nx=n, precision="mixed_f64")
    a = shll.Context(p)
    a.init_state()
    a.autotune()
    choice = a.tuning()
    assert 8 <= choice[0] <= 32 and choice[2] > 0
    t0 = a.totals()
    n0 = shll.kernel_launches()
    steps = a.run()
    resident_launches = shll.kernel_launches() - n0
    t1 = a.totals()
    shll.set_resident(False)
    try:
        b = shll.Context(p)   # picks up the tuned choice of this size class
        b.init_state()
        assert b.tuning() == choice
        n0 = shll.kernel_launches()
        b.run()
        assert shll.kernel_launches() - n0 > 1000
    finally:
        shll.set_resident(True)
    if (n + choice[2] - 1) // choice[2] <= 152:   # (its chunks fit the 152 SMs at once: one launch + fix-up)
        assert resident_launches == 2
    assert np.array_equal(a.primitives(), b.primitives())
    ex = oracle.riemann_exact(n, steps * (0.125 / n))
    e_mixed = np.mean(np.abs(a.primitives()[0] - ex[0]))
    e_fp64 = np.mean(np.abs(fp64_sod(shll, n)[0] - ex[0]))
    assert abs(e_mixed - e_fp64) <= 0.1 * e_fp64, (e_mixed, e_fp64)
    assert abs(t1[0] - t0[0]) / t0[0] <= 1e-12
    a.close()
    b.close()


def _schedules_run(shll, items, cluster=False, resident=True):
    shll.set_cluster_runs(cluster)
    shll.set_resident(resident)
    try:
        b = shll.Batch(items)
        l0 = shll.kernel_launches()
        b.run()
        launches = shll.kernel_launches() - l0
        out = [b.primitives(i) for i in range(len(items))]
        b.close()
    finally:
        shll.set_cluster_runs(False)
        shll.set_resident(True)
    return out, launches


@pytest.mark.parametrize("order,n,count,prec", [(2, 3500, 19, "mixed_f64"), (1, 7000, 5, "mixed_f64"),
                                               (2, 7000, 3, "mixed_kahan")])
def test_cluster_runs_equal_the_other_schedules(shll, order, n, count, prec):
    # tubes of 8 and 16 chunks, each one thread-block cluster with the cluster barrier between
    # sweeps: the same bits as one launch per sweep and as the resident run
    rng = np.random.default_rng(order * 100 + count)
    items = [shll.params(1, order, nx=n, precision=prec, fold_steps=64, n_steps=16 * 40 + 7,
                         ic_x_d=float(rng.uniform(0.3, 0.7)), ic_rho_l=float(rng.uniform(2, 40)),
                         ic_T_l=float(rng.uniform(0.5, 2))) for _ in range(count)]
    a, la = _schedules_run(shll, items, cluster=False, resident=False)
    b, lb = _schedules_run(shll, items, cluster=True)
    c, _ = _schedules_run(shll, items, cluster=False, resident=True)
    assert la > 40 and lb <= 3   # (the cluster run: start-of-run flags, one launch, fix-up)
    for x, y, z in zip(a, b, c):
        assert np.array_equal(x, y) and np.array_equal(x, z)
