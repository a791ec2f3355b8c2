"""The first-order tubes of the seeded batch of 1D shock tubes (4096 tubes, seed 0; density ratios
up to 100, temperature ratios up to 2, up to 16384 cells) in the mixed FP32-flux / FP64-accumulate
engine, against the FP64 oracle.

On strong tubes the reference's first-order scheme (base-c/base_shll.c:87-159) is very sensitive
to rounding: where the flow is supersonic its split gives the u - a wave a negative numerical
viscosity, and per-step perturbations grow by factors up to about 1e5 over a run.  On some tubes
this makes the FP64 result itself irreproducible: FP64 with fused multiply-adds and FP64 without
them (the only licensed difference between two FP64 builds) differ by up to 1e-3.  The bar is
therefore:
  * every sampled tube on which the two FP64 builds agree to 1e-8 (FP64-reproducible): the mixed
    result within L1 1e-6 of the oracle in rho, u and T;
  * every other tube that the FP64 scheme survives: within 50 times the FP64 builds' own
    difference (the mixed engine's rounding is larger than FP64's, which that difference
    measures).
The oracle's arithmetic runs on the GPU as the bit-exact FP64 batch (SHLL_PREC_F64_EXACT), which
the first test pins bit for bit to the CPU oracle."""
import numpy as np
import pytest

from helpers import batch1d_draws, tube_params

pytestmark = pytest.mark.gpu

DRAWS = batch1d_draws()
FIRST = [d for d in DRAWS if d[5] == 1]
# every 32nd first-order tube, the 8 strongest (density ratio x temperature ratio) and the 3 largest
SAMPLE = sorted({d[0] for d in FIRST[::32]} | {d[0] for d in sorted(FIRST, key=lambda d: -d[2] * d[3])[:8]}
                | {d[0] for d in sorted(FIRST, key=lambda d: -d[1])[:3]})


def run_batch(shll, precision, idx):
    b = shll.Batch([tube_params(shll, DRAWS[t], precision) for t in idx])
    b.run(allow_numeric=True)
    out = [(b.primitives(i), b.item_status(i), b.totals(i)) for i in range(len(idx))]
    b.close()
    return out


def test_exact_batch_is_the_oracle(shll, oracle):
    # small strong tubes of the sample: the bit-exact FP64 batch equals the CPU oracle bit for bit
    idx = [t for t in SAMPLE if DRAWS[t][1] <= 1400][:6]
    assert len(idx) >= 3
    got = run_batch(shll, "f64_exact", idx)
    for (prim, status, _), t in zip(got, idx):
        _, n, ratio, tr, xd, _ = DRAWS[t]
        _, ref, _ = oracle.run(oracle.make_cfg(nx=n, real_bits=64), oracle.ic_sod(n, x_d=xd, rhoL=ratio, TL=tr))
        assert status == 0
        assert np.array_equal(prim, ref), t


def test_first_order_tubes_match_fp64(shll):
    exact = run_batch(shll, "f64_exact", SAMPLE)
    fused = run_batch(shll, "f64", SAMPLE)
    mixed = run_batch(shll, "mixed_f64", SAMPLE)
    reproducible = 0
    for t, (pe, se, _), (pf, sf, _), (pm, sm, tot) in zip(SAMPLE, exact, fused, mixed):
        if se != 0:
            continue   # the reference scheme itself breaks down on this tube
        assert sm == 0, f"tube {t}: mixed engine broke down where FP64 did not"
        floor = float(np.max(np.mean(np.abs(pf - pe), axis=1))) if sf == 0 else np.inf
        err = np.mean(np.abs(pm - pe), axis=1)
        if floor <= 1e-8:
            reproducible += 1
            assert np.all(err <= 1e-6), (t, DRAWS[t], err)
        else:
            assert np.all(err <= max(1e-6, 50 * floor)), (t, DRAWS[t], err, floor)
        # reflective walls: mass conserved to FP64 rounding
        _, n, ratio, tr, xd, _ = DRAWS[t]
        left = sum(1 for i in range(n) if i < xd * n)
        mass0 = ratio * left + (n - left)
        assert abs(tot[0] - mass0) <= 1e-12 * mass0, t
    assert reproducible >= 60   # (the bar is tested on most of the sample)


def test_pair_flux_is_what_keeps_strong_tubes_accurate(shll):
    # the strongest FP64-reproducible tube of at most 5000 cells: with FP32 fluxes everywhere the
    # mixed engine misses the bar (or breaks down); with the pair flux it meets it, far closer
    cand = [d[0] for d in sorted(FIRST, key=lambda d: -d[2] * d[3]) if d[1] <= 5000][:6]
    exact = run_batch(shll, "f64_exact", cand)
    fused = run_batch(shll, "f64", cand)
    pick = [i for i in range(len(cand)) if exact[i][1] == 0 and fused[i][1] == 0
            and np.max(np.mean(np.abs(fused[i][0] - exact[i][0]), axis=1)) <= 1e-8]
    assert pick
    idx, ref = [cand[pick[0]]], exact[pick[0]][0]
    try:
        shll.set_pair_flux(0)
        fp32 = run_batch(shll, "mixed_f64", idx)[0]
    finally:
        shll.set_pair_flux(1)
    pair = run_batch(shll, "mixed_f64", idx)[0]
    e_pair = np.mean(np.abs(pair[0][0] - ref[0]))
    assert pair[1] == 0 and np.all(np.mean(np.abs(pair[0] - ref), axis=1) <= 1e-6)
    if fp32[1] == 0:
        e_fp32 = np.mean(np.abs(fp32[0][0] - ref[0]))
        assert e_fp32 > 1e-6 and e_fp32 > 100 * e_pair, (e_fp32, e_pair)
