"""Parity of the 2D paths at the full sizes of the benchmark configurations.

  * the circular diaphragm on 4096 x 4096 cells, 500 first-order steps (rho 10 inside r = 0.25,
    1 outside, T 1, at rest): the plain FP64 path (fused multiply-add allowed) within a max
    per-cell relative difference of 1e-10 of the bit-exact FP64 path, the mixed FP32-flux /
    FP64-accumulate path within L1(rho, u, v, T) 1e-6 of it, mass conserved to 1e-12;
  * every 4th domain of the seeded batch of 256 domains (128^2 .. 1024^2, 400 steps each), the same
    bars per domain;
  * the bit-exact FP64 path is the oracle's arithmetic: pinned bit for bit to the CPU oracle here on
    the circular diaphragm at 256 x 256 cells and 500 steps (and at smaller sizes and the
    reference's own initial data in test_gpu_plain.py).
Reference being replaced: base-c/base_shll_2d.c:139-300 (flux, update) and :343-370 (time loop)."""
import numpy as np
import pytest

from helpers import batch2d_draws, circle_params, l1, max_rel_scaled

pytestmark = pytest.mark.gpu


def run_ctx(shll, p):
    c = shll.Context(p)
    c.init_state()
    t0 = c.totals()
    c.run()
    out, t1 = c.primitives(), c.totals()
    c.close()
    return out, t0, t1


def test_exact_path_is_the_oracle_on_the_circle_at_256(shll, oracle):
    n, steps = 256, 500
    _, ref, _ = oracle.run(oracle.make_cfg(dim=2, order=1, nx=n, ny=n, n_steps=steps),
                           oracle.ic_circle2d(n, n, r=0.25, rho_in=10.0, rho_out=1.0))
    out, _, _ = run_ctx(shll, circle_params(shll, n, 0.25, 10.0, 1.0, steps, "f64_exact"))
    assert np.array_equal(out, ref)


def test_circle_4096_fp64_and_mixed(shll):
    n, steps = 4096, 500
    exact, e0, e1 = run_ctx(shll, circle_params(shll, n, 0.25, 10.0, 1.0, steps, "f64_exact"))
    fused, _, _ = run_ctx(shll, circle_params(shll, n, 0.25, 10.0, 1.0, steps, "f64"))
    assert max_rel_scaled(fused, exact) <= 1e-10
    del fused
    mixed, m0, m1 = run_ctx(shll, circle_params(shll, n, 0.25, 10.0, 1.0, steps, "mixed_f64"))
    err = l1(mixed, exact)
    assert np.all(err <= 1e-6), err
    assert abs(m1[0] - m0[0]) / m0[0] <= 1e-12
    assert abs(e1[0] - e0[0]) / e0[0] <= 1e-12


def test_seeded_domain_batch(shll):
    draws = batch2d_draws()[::4]
    assert {d[1] for d in draws} == {128, 256, 512, 1024}

    def run_batch(prec):
        b = shll.Batch([circle_params(shll, d[1], d[2], d[3], d[4], 400, prec) for d in draws])
        b.run(allow_numeric=True)
        out = [(b.primitives(i), b.item_status(i), b.totals(i)) for i in range(len(draws))]
        b.close()
        return out

    exact, fused, mixed = run_batch("f64_exact"), run_batch("f64"), run_batch("mixed_f64")
    for d, (pe, se, _), (pf, sf, _), (pm, sm, tm) in zip(draws, exact, fused, mixed):
        assert se == 0 and sf == 0 and sm == 0, d
        assert max_rel_scaled(pf, pe) <= 1e-10, d
        assert np.all(l1(pm, pe) <= 1e-6), (d, l1(pm, pe))
        n, r, ratio = d[1], d[2], d[3]
        x = (np.arange(n) + 0.5) * (1.0 / n) - 0.5   # cell centres as the initial condition forms them
        inside = (x[:, None] ** 2 + x[None, :] ** 2 < r * r).sum()
        mass0 = ratio * inside + (n * n - inside)
        assert abs(tm[0] - mass0) <= 1e-12 * mass0, d
