"""Parity of the device stretched-grid streamfunction multigrid (rcsc.f) with
the oracle, bit for bit (psi and the sweep count), on grid.f's GEF grid and
on tanh grids, square and not (n1 < n2 makes corser's clearing of row n1
hit an interior coarse row), in the reference's line order and in the
four-colour order; and the sweep limit (psi untouched, no STOP)."""
import math

import numpy as np
import pytest

from codesthesis_dir_gb300 import grid

pytestmark = pytest.mark.gpu

R0, RMAX, ZMAX = 0.5, 1.0, 0.5


@pytest.fixture(scope="module")
def S(gblib):
    from codesthesis_dir_gb300 import stretched
    return stretched


def _case(kind, n1, n2):
    if kind == "gef":
        hr, hz = grid.spacing_gef(n1, R0, RMAX, 0.1, 1.15, 0.01), grid.spacing_gef(n2, 0.0, ZMAX, 0.1, 1.15, 0.01)
    else:
        hr, hz = grid.spacing_tanh(n1, R0, RMAX, 1.5), grid.spacing_tanh(n2, 0.0, ZMAX, 1.5)
    L = grid.build(hr, hz, R0)
    rng = np.random.default_rng(n1 + 3 * n2)
    f = np.asfortranarray(rng.standard_normal((n1 + 1, n2 + 1)))
    psi0 = np.zeros_like(f)
    psi0[1:n1, 1:n2] = 0.01 * rng.standard_normal((n1 - 1, n2 - 1))
    return hr, hz, L, f, psi0


@pytest.mark.parametrize("mode", [0, 1], ids=["lex", "four-colour"])
@pytest.mark.parametrize("kind,n1,n2", [("gef", 32, 32), ("tanh", 16, 32), ("tanh", 64, 32), ("tanh", 64, 64)])
def test_poisson_parity(oracle, S, mode, kind, n1, n2):
    hr, hz, L, f, psi0 = _case(kind, n1, n2)
    o = oracle.OracleSTR(hr, hz, R0, mode=mode)
    st_o, sw_o, psi_o = o.poisson(psi0, f)
    g = S.STR(L, smoother=mode)
    st_g, sw_g, psi_g = g.poisson(psi0, f)
    assert st_o == 0 and st_g == 0
    assert sw_g == sw_o
    np.testing.assert_array_equal(psi_g, psi_o)


def test_sweep_limit(oracle, S):
    hr, hz, L, f, psi0 = _case("tanh", 16, 16)
    g = S.STR(L, tolcon=1e-30, maxsweeps=4, smoother=1)
    st, sw, psi = g.poisson(psi0, f)
    o = oracle.OracleSTR(hr, hz, R0, mode=1, tolcon=1e-30, maxsweeps=4)
    st_o, sw_o, _ = o.poisson(psi0, f)
    assert st == 1 and st_o == 1 and sw == sw_o == 4
    np.testing.assert_array_equal(psi, psi0)
