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
