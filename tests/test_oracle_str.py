"""The stretched-grid operator (rcsc.f) and its coefficient build (grid.f),
on the CPU:

* fdif's weights (grid.f:926-1115) differentiate polynomials of degree
  < nx exactly on arbitrary non-uniform points;
* the product's host generator (codesthesis_dir_gb300/grid.py) produces the
  oracle's spacings, levels and tables bit for bit, for grid.f's GEF grid,
  a tanh grid and a uniform grid;
* the multigrid (rcsc.f:1118-1444) solves psi_rr + psi_r/r - psi/r^2 +
  psi_zz = f to second order on wall-clustered grids;
* the reference's line order and the four-colour order converge to the
  same solution;
* corser clears row j = n1c of the coarse level (n1 for both directions),
  an interior row when n1 < n2;
* after the sweep limit psi is left as it was (the reference returns)."""
import math

import numpy as np
import pytest

from codesthesis_dir_gb300 import grid

R0, RMAX, ZMAX = 0.5, 1.0, 0.5


@pytest.mark.parametrize("nx,nref", [(3, 2), (4, 2), (4, 3), (3, 1), (3, 3), (5, 3)])
def test_fdif_exact_on_polynomials(oracle, nx, nref):
    rng = np.random.default_rng(nx * 10 + nref)
    x = np.sort(rng.uniform(0.0, 1.0, 12))
    k = 5
    w = oracle.str_fdif(nx, nref, k, x)
    pts = x[k - nref + 1:k - nref + 1 + nx]
    x0 = x[k]
    for deg in range(nx):
        f = pts ** deg
        for d in range(nx):
            exact = 0.0 if d > deg else math.factorial(deg) / math.factorial(deg - d) * x0 ** (deg - d)
            assert abs(w[d] @ f - exact) < 1e-9 * max(1.0, np.abs(w[d]).sum()), (deg, d)


def _spacings(kind, n1, n2):
    if kind == "gef":
        return (grid.spacing_gef(n1, R0, RMAX, 0.1, 1.15, 0.01), grid.spacing_gef(n2, 0.0, ZMAX, 0.1, 1.15, 0.01))
    if kind == "tanh":
        return grid.spacing_tanh(n1, R0, RMAX, 1.5), grid.spacing_tanh(n2, 0.0, ZMAX, 1.5)
    return grid.spacing_uniform(n1, R0, RMAX), grid.spacing_uniform(n2, 0.0, ZMAX)


@pytest.mark.parametrize("kind,n1,n2", [("gef", 16, 16), ("tanh", 32, 64), ("uni", 64, 32), ("tanh", 128, 128)])
def test_host_tables_equal_oracle(oracle, kind, n1, n2):
    hr, hz = _spacings(kind, n1, n2)
    L = grid.build(hr, hz, R0)
    o = oracle.OracleSTR(hr, hz, R0)
    assert L.nlev == o.nlev
    for l in range(1, L.nlev + 1):
        np.testing.assert_array_equal(np.array(L.r[l]), o.table("r", l))
        np.testing.assert_array_equal(np.array(L.z[l]), o.table("z", l))
        for name in ("cr", "crr", "cz", "czz"):
            np.testing.assert_array_equal(getattr(L, name)[l].ravel(), o.table(name, l), err_msg=(name, l))
    if kind == "gef":
        np.testing.assert_array_equal(np.array(hr), oracle.str_spacing_gef(n1, R0, RMAX, 0.1, 1.15, 0.01))
        assert abs(sum(hr) - (RMAX - R0)) < 1e-14 and hr[1:] == hr[1:][::-1]


def test_gef_stops_like_the_reference(oracle):
    with pytest.raises(ValueError):
        grid.spacing_gef(16, 0.0, 1.0, 10.0, 1.01, 0.001)     # too many points in the GEF region
    with pytest.raises(ValueError):
        oracle.str_spacing_gef(16, 0.0, 1.0, 10.0, 1.01, 0.001)


def manufactured(L):
    r = np.array(L.r[1])
    z = np.array(L.z[1])
    R, Z = np.meshgrid(r, z, indexing="ij")
    kr, kz = math.pi / (RMAX - R0), math.pi / ZMAX
    S, Cs, Sz = np.sin(kr * (R - R0)), np.cos(kr * (R - R0)), np.sin(kz * Z)
    exact = S * Sz
    f = (-(kr ** 2) * S + kr * Cs / R - S / R ** 2 - kz ** 2 * S) * Sz
    return exact, np.asfortranarray(f)


def test_second_order_on_stretched_grids(oracle):
    errs = []
    for n in (16, 32, 64):
        hr, hz = _spacings("tanh", n, n)
        L = grid.build(hr, hz, R0)
        o = oracle.OracleSTR(hr, hz, R0, mode=oracle.ORC_ZEBRA, tolcon=1e-10)
        exact, f = manufactured(L)
        st, sw, psi = o.poisson(np.zeros_like(f), f)
        assert st == 0, sw
        errs.append(np.max(np.abs(psi - exact)))
    assert errs[2] < 2e-3 and errs[0] / errs[1] > 3.0 and errs[1] / errs[2] > 3.0, errs


@pytest.mark.parametrize("n1,n2", [(32, 32), (16, 32), (32, 16)])
def test_orders_agree(oracle, n1, n2):
    hr, hz = _spacings("gef", n1, n2)
    L = grid.build(hr, hz, R0)
    exact, f = manufactured(L)
    a = oracle.OracleSTR(hr, hz, R0, mode=oracle.ORC_LEX, tolcon=1e-11).poisson(np.zeros_like(f), f)
    b = oracle.OracleSTR(hr, hz, R0, mode=oracle.ORC_ZEBRA, tolcon=1e-11).poisson(np.zeros_like(f), f)
    assert a[0] == 0 and b[0] == 0
    assert np.max(np.abs(a[2] - b[2])) < 1e-9 * max(1.0, np.max(np.abs(a[2])))


def test_corser_row_n1c_cleared(oracle):
    """With n1 < n2 the reference's clearing of row j = n1c (rcsc.f:1375-1380)
    hits an interior coarse row: its right-hand side is zero."""
    import ctypes as C
    hr, hz = _spacings("uni", 16, 32)
    o = oracle.OracleSTR(hr, hz, R0)
    m = o.m
    ld = m.ld
    rc = np.ctypeslib.as_array(m.rc, shape=(ld * ld,)).reshape(ld, ld).T
    rc[:, :] = np.random.default_rng(1).standard_normal(rc.shape)
    oracle.lib().orc_str_corser.argtypes = [C.POINTER(oracle.STRMG), C.c_int]
    oracle.lib().orc_str_corser(C.byref(m), 1)
    n1c, n2c = o.g.n1[2], o.g.n2[2]
    fc = np.ctypeslib.as_array(m.f[2], shape=((n1c + 1) * (n2c + 1),)).reshape(n2c + 1, n1c + 1).T
    assert n1c < n2c
    assert np.all(fc[:, n1c] == 0.0)
    assert np.all(fc[1:n1c, n1c + 1] != 0.0)


def test_sweep_limit_leaves_psi(oracle):
    hr, hz = _spacings("tanh", 16, 16)
    L = grid.build(hr, hz, R0)
    exact, f = manufactured(L)
    o = oracle.OracleSTR(hr, hz, R0, tolcon=1e-30, maxsweeps=3)
    psi0 = np.random.default_rng(0).standard_normal(f.shape)
    st, sw, psi = o.poisson(psi0, f)
    assert st == 1 and sw == 3
    np.testing.assert_array_equal(psi, psi0)
