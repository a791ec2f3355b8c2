"""The reference scheme's own sensitivity to FP32-scale perturbations (CPU oracle, FP64).

The second-order scheme (minmod slopes of the split fluxes with forward Euler,
base-c/2nd_order_base_shll.c:191-201, 438-446) amplifies a perturbation of the initial state by
6e-8 relative (the size of FP32 rounding) into an L1 spread that grows quickly with the tube size;
the first-order scheme damps it.  This spread is the floor below which no arithmetic that rounds at
FP32 scale can bring a second-order run against FP64, and the GPU tests of the mixed engine tie
their second-order bounds to it."""
from noise_floor import spread, spread2d, spread_stepwise


def test_second_order_spread_grows_with_the_tube():
    s4096 = spread(4096)[0]
    s16384 = spread(16384)[0]
    assert 5e-8 < s4096 < 5e-7
    assert 1e-6 < s16384 < 1e-5
    assert s16384 > 10 * s4096
    # rounding in every step (perturbations repeated every 10 steps) spreads further still
    assert spread_stepwise(4096)[0] > 3 * s4096


def test_first_order_sod_tube_damps_the_same_perturbation():
    assert spread(16384, order=1)[0] < 1e-7


def test_2d_second_order_spread():
    # base-omp's quadrant problem with the MC limiter on 256 x 256 cells (615 steps); the same
    # perturbation on 1024 x 1024 cells (2458 steps, measured with the FP64 GPU path) moves the
    # result by L1(rho) 2.3e-5
    s = spread2d(256)
    assert 1e-8 < s[0] < 1e-7
