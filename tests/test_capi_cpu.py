"""CPU tests of the C-ABI library: it loads, exports every entry point that include/shll.h
declares, and its host-side logic (defaults, step counts, parameter validation) is right.
No compute call is made here (there is no GPU in the CPU suite)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "shll.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s+\*?([A-Za-z_][A-Za-z0-9_]*)\s*\(", src, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "return")))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for ref in ("Allocate_and_Init_Memory", "Compute_U_from_P", "Compute_P_from_U", "Compute_F_from_P",
                "Update_U_from_F", "Save_Results", "Free_Memory"):
        assert ref in names
    assert len(names) >= 38


def test_library_exports_every_declared_symbol(shll):
    L = shll.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    assert set(shll.EXPORTS) <= set(declared_functions())


def test_params_default_matches_reference_constants(shll):
    p = shll.params(1, 1)
    assert (p.dim, p.order, p.nx, p.gamma, p.R, p.cfl, p.lx, p.t_end) == (1, 1, 256, 1.4, 1.0, 0.25, 1.0, 0.2)
    assert p.ic.kind == shll.IC_SOD and p.ic.rho_l == 10.0 and p.ic.rho_r == 1.0 and p.ic.x_d == 0.5
    p2 = shll.params(2, 1)
    assert p2.t_end == 0.1 and p2.ic.kind == shll.IC_REF_BOX2D
    p3 = shll.params(2, 2)
    assert p3.t_end == 0.8 and p3.ic.kind == shll.IC_FOUR_SHOCK2D


@pytest.mark.parametrize("n", [8, 256, 1000, 1024, 65536])
@pytest.mark.parametrize("bits", [32, 64])
def test_steps_for_matches_oracle(shll, oracle, n, bits):
    p = shll.params(1, 1, nx=n, clock_f32=1 if bits == 32 else 0)
    assert shll.steps_for(p) == oracle.count_steps(oracle.make_cfg(nx=n, real_bits=bits))


def test_steps_for_2d_and_fixed(shll, oracle):
    p = shll.params(2, 1, nx=48, ny=32)
    assert shll.steps_for(p) == oracle.count_steps(oracle.make_cfg(dim=2, nx=48, ny=32, t_end=0.1))
    p.n_steps = 500
    assert shll.steps_for(p) == 500


@pytest.mark.parametrize("field,value", [("nx", 1), ("dim", 3), ("order", 0), ("gamma", 1.0), ("cfl", 0.0),
                                         ("precision", 9), ("limiter", 2), ("fold_steps", -1)])
def test_create_rejects_bad_parameters_before_touching_the_gpu(shll, field, value):
    p = shll.params(1, 1)
    setattr(p, field, value)
    h = ctypes.c_void_p()
    assert shll.lib().shll_create(ctypes.byref(p), ctypes.byref(h)) == shll.ERR_ARG
    assert not h.value
    assert shll.steps_for(p) == -1


def test_create_rejects_mismatched_initial_condition(shll):
    p = shll.params(1, 1)
    p.ic.kind = shll.IC_CIRCLE2D
    h = ctypes.c_void_p()
    assert shll.lib().shll_create(ctypes.byref(p), ctypes.byref(h)) == shll.ERR_ARG


def test_status_strings(shll):
    L = shll.lib()
    assert L.shll_status_string(0) == b"ok"
    assert b"timed out" in L.shll_status_string(shll.ERR_TIMEOUT)
    assert L.shll_last_error(None) == b"no context"


def test_batch_rejects_empty(shll):
    h = ctypes.c_void_p()
    assert shll.lib().shll_batch_create(None, 0, ctypes.byref(h)) == shll.ERR_ARG


def test_initial_primitives_match_the_oracle(shll, oracle):
    # host-side initial conditions (what shll_init_state loads), no device involved
    import numpy as np
    p = shll.params(1, 1, nx=1000, precision="mixed_f64")
    assert np.array_equal(shll.initial_primitives(p), oracle.ic_sod(1000))
    p = shll.params(1, 2, nx=777, precision="f64", ic_x_d=0.37, ic_rho_l=4.5, ic_T_l=1.7)
    assert np.array_equal(shll.initial_primitives(p), oracle.ic_sod(777, x_d=0.37, rhoL=4.5, TL=1.7))
    p = shll.params(2, 1, nx=40, ny=24, precision="f64")
    assert np.array_equal(shll.initial_primitives(p), oracle.ic_ref_box2d(40, 24))
    p = shll.params(2, 1, nx=64, ny=48, precision="mixed_f64", ic_kind=shll.IC_CIRCLE2D, ic_cx=0.5, ic_cy=0.5,
                    ic_radius=0.3, ic_rho_l=7.0, ic_T_l=1.3, ic_rho_r=1.0, ic_T_r=1.0)
    assert np.array_equal(shll.initial_primitives(p),
                          oracle.ic_circle2d(64, 48, r=0.3, rho_in=7.0, T_in=1.3, rho_out=1.0, T_out=1.0))
    with pytest.raises(shll.ShllError):
        shll.initial_primitives(shll.params(1, 1, nx=0))


@pytest.mark.parametrize("field,value", [("gamma", 1.0), ("cfl", 0.0), ("R", 0.0), ("limiter", 2),
                                         ("mc_alpha", 0.0), ("fold_steps", -1), ("nx", 1)])
def test_static_tube_entry_validates_parameters_for_any_step_count(shll, field, value):
    # shll_tube_run_static applies shll_create's checks also when the caller gives the step count;
    # they come before any CUDA call, so a stand-in device pointer is never touched here
    L = shll.lib()
    L.shll_tube_run_static.argtypes = [ctypes.POINTER(shll.Params), ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p]
    L.shll_tube_run_static.restype = ctypes.c_int
    p = shll.params(1, 2, nx=1024, precision="mixed_f64", limiter=1, mc_alpha=1.25)
    setattr(p, field, value)
    for nsteps in (100, 0):
        assert L.shll_tube_run_static(ctypes.byref(p), ctypes.c_void_p(4096), nsteps, None) == shll.ERR_ARG


def test_mc_limiter_alpha_is_checked(shll):
    h = ctypes.c_void_p()
    p = shll.params(1, 2, limiter=1, mc_alpha=3.0)
    assert shll.lib().shll_create(ctypes.byref(p), ctypes.byref(h)) == shll.ERR_ARG
    p = shll.params(1, 2, limiter=1, mc_alpha=float("nan"))
    assert shll.steps_for(p) == -1
