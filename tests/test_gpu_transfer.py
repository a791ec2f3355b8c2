"""Host <-> device transfers of the mixed engines: primitive planes are copied as given and
converted on the device (Compute_U_from_P / Compute_P_from_U in FP64, base_shll.c:76-80,171-176,
base_shll_2d.c:126-136,312-318), bit for bit as a host FP64 evaluation of the same expressions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def host_primitives(U, CV):
    """Compute_P_from_U in FP64 on the host, same operation order as the library's kernel."""
    rho = U[0]
    u = U[1] / rho
    if U.shape[0] == 3:
        T = ((U[2] / rho) - 0.5 * u * u) / CV
        return np.stack([rho, u, T])
    v = U[2] / rho
    T = ((U[3] / rho) - 0.5 * (u * u + v * v)) / CV
    return np.stack([rho, u, v, T])


@pytest.mark.parametrize("prec", ["mixed_f64", "mixed_kahan"])
@pytest.mark.parametrize("dim", [1, 2])
def test_device_primitives_match_host_conversion(shll, prec, dim):
    p = shll.params(dim, 1, nx=3000 if dim == 1 else 96, ny=None if dim == 1 else 80, precision=prec, n_steps=100)
    c = shll.Context(p)
    c.init_state()
    c.step(100)
    CV = p.R / (p.gamma - 1.0)
    assert np.array_equal(c.primitives(), host_primitives(c.conserved(), CV))
    c.close()


@pytest.mark.parametrize("dim", [1, 2])
def test_set_primitives_equals_init_state(shll, oracle, dim):
    if dim == 1:
        p = shll.params(1, 2, nx=5000, precision="mixed_f64")
        prim = oracle.ic_sod(5000)
    else:
        p = shll.params(2, 1, nx=64, ny=48, precision="mixed_f64", n_steps=80, ic_kind=shll.IC_CIRCLE2D,
                        ic_cx=0.5, ic_cy=0.5, ic_radius=0.25, ic_rho_l=10.0, ic_T_l=1.0, ic_rho_r=1.0, ic_T_r=1.0)
    a = shll.Context(p)
    a.init_state()
    if dim == 2:
        prim = a.primitives()   # the descriptor's initial state, downloaded before any step
    a.run()
    b = shll.Context(p)
    if dim == 1:
        b.set_primitives(prim[0], prim[1], prim[2])
    else:
        b.set_primitives(prim[0], prim[1], prim[3], v=prim[2])
    b.run()
    assert np.array_equal(a.primitives(), b.primitives())
    a.close()
    b.close()


def test_set_primitives_rejects_bad_cell_and_keeps_state(shll, oracle):
    n = 2000
    c = shll.Context(shll.params(1, 1, nx=n, precision="mixed_f64"))
    c.init_state()
    c.step(32)
    before = c.primitives()
    prim = oracle.ic_sod(n)
    prim[0][1234] = -1.0
    prim[2][1500] = 0.0
    with pytest.raises(shll.ShllError) as e:
        c.set_primitives(prim[0], prim[1], prim[2])
    assert e.value.status == shll.ERR_ARG
    assert "cell 1234" in str(e.value)
    assert np.array_equal(c.primitives(), before)
    c.step(16)   # still usable
    c.close()


def test_batch_set_primitives_matches_single_context(shll, oracle):
    items = [shll.params(1, o, nx=n, precision="mixed_f64", n_steps=300) for o, n in ((1, 700), (2, 1900), (1, 2600))]
    b = shll.Batch(items)
    prim = oracle.ic_sod(1900, rhoL=4.0, TL=1.5)
    b.set_primitives(1, prim[0], prim[1], prim[2])
    b.run()
    single = shll.Context(items[1])
    single.set_primitives(prim[0], prim[1], prim[2])
    single.run()
    assert np.array_equal(b.primitives(1), single.primitives())
    # the other items kept their own initial data
    other = shll.Context(items[2])
    other.init_state()
    other.run()
    assert np.array_equal(b.primitives(2), other.primitives())
    for x in (b, single, other):
        x.close()


def test_primitives_into_caller_buffer(shll):
    c = shll.Context(shll.params(1, 1, nx=1000, precision="mixed_f64", n_steps=50))
    c.init_state()
    c.run()
    buf = np.empty((3, 1000))
    out = c.primitives(out=buf)
    assert out is buf
    assert np.array_equal(buf, c.primitives())
    c.close()


@pytest.mark.parametrize("dim", [1, 2])
def test_rerun_from_uploaded_initial_state_is_identical(shll, dim):
    # run; upload the descriptor's initial primitives again (shll_initial_primitives); run again:
    # nothing of the first run may carry over into the second
    if dim == 1:
        p = shll.params(1, 2, nx=9000, precision="mixed_f64", n_steps=400)
    else:
        p = shll.params(2, 1, nx=96, ny=64, precision="mixed_f64", n_steps=150, ic_kind=shll.IC_CIRCLE2D,
                        ic_cx=0.5, ic_cy=0.5, ic_radius=0.3, ic_rho_l=5.0, ic_T_l=1.2, ic_rho_r=1.0, ic_T_r=1.0)
    c = shll.Context(p)
    c.init_state()
    init = c.primitives()
    c.run()
    first = c.primitives()
    prim = shll.initial_primitives(p)
    assert np.allclose(prim, init, rtol=1e-14, atol=0)   # (U -> P on the device rounds)
    if dim == 1:
        c.set_primitives(prim[0], prim[1], prim[2])
    else:
        c.set_primitives(prim[0], prim[1], prim[3], v=prim[2])
    c.run()
    assert np.array_equal(c.primitives(), first)
    c.close()


@pytest.mark.parametrize("dim", [1, 2])
def test_batch_packed_transfers(shll, dim):
    if dim == 1:
        items = [shll.params(1, o, nx=n, precision="mixed_f64", n_steps=200, ic_rho_l=r)
                 for o, n, r in ((1, 700, 3.0), (2, 1900, 8.0), (1, 2600, 20.0))]
    else:
        items = [shll.params(2, 1, nx=n, ny=n, precision="mixed_f64", n_steps=60, ic_kind=shll.IC_CIRCLE2D,
                             ic_cx=0.5, ic_cy=0.5, ic_radius=0.2, ic_rho_l=r, ic_T_l=1.0, ic_rho_r=1.0, ic_T_r=1.0)
                 for n, r in ((64, 4.0), (32, 9.0))]
    b = shll.Batch(items)
    b.run()
    ref = [b.primitives(i) for i in range(len(items))]
    packed = b.get_all_primitives()
    off = 0
    for i, p in enumerate(items):
        size = ref[i].size
        assert np.array_equal(packed[off:off + size].reshape(ref[i].shape), ref[i])
        off += size
    # re-upload every item's initial state at once and run again: the same results
    init = np.concatenate([shll.initial_primitives(p).ravel() for p in items])
    b.set_all_primitives(init)
    b.run()
    assert np.array_equal(b.get_all_primitives(), packed)
    # a bad cell in the second item is refused before any state changes
    bad = init.copy()
    n0 = ref[0].size
    bad[n0 + 7] = -1.0
    with pytest.raises(shll.ShllError) as e:
        b.set_all_primitives(bad)
    assert e.value.status == shll.ERR_ARG and "item 1, cell 7" in str(e.value)
    assert np.array_equal(b.get_all_primitives(), packed)
    b.close()
