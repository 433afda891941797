"""Parity of the device PRB path against the oracle, bit for bit.

The device kernels keep the reference's operation order with no fused
multiply-add, so every field, every Nusselt number and every multigrid
sweep count must be identical to the oracle's (the relative-L2 <= 1e-10
bar of the plain FP64 path is met with zero difference)."""
import numpy as np
import pytest

from prb_helpers import config0_params, diff_fields, make_pair

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gblib):
    from codesthesis_dir_gb300 import prb
    return prb


@pytest.mark.parametrize("smoother", [0, 1], ids=["lex", "zebra"])
@pytest.mark.parametrize("tolcon", [2e-6, 1e-10], ids=["tol2e-6", "tol1e-10"])
def test_routines_small(oracle, P, smoother, tolcon):
    """Routine-by-routine (the drop-in granularity) on a 16 x 32 grid."""
    o, g = make_pair(oracle, P, 16, 32, 1e-4, 1e5, 1.0, 0.0, 1.0, 2.0, smoother, tolcon, seed=3, amp=1e-2)
    for kt in range(1, 6):
        st, nu, sw = o.step()
        assert st == 0
        if kt == 1:
            g.cvorticity1()
            g.temperature1()
        else:
            g.cvorticity()
            g.temperature()
        t1, t2 = g.heat()
        g.rhsv()
        sv = g.poisson2()
        g.rhsu()
        su = g.poisson3()
        g.update()
        assert (sv, su) == (int(sw[0]), int(sw[1])), kt
        rmr0, xx = o.s.rmax - o.s.r0, o.s.xx
        assert t1 * rmr0 / xx == nu[0] and t2 * rmr0 / xx == nu[1], kt
        assert diff_fields(o, g) == {}, kt


@pytest.mark.parametrize("smoother", [0, 1], ids=["lex", "zebra"])
def test_graph_steps_config0(oracle, P, smoother):
    """Graph-replayed steps on the 129 x 65 layer (nr=64, np=128) with the
    1e-10 multigrid tolerance; the first step is the forward step."""
    prm = config0_params()
    o, g = make_pair(oracle, P, smoother=smoother, tolcon=1e-10, **prm)
    nsteps = 4 if smoother == 0 else 12
    nu_o, sw_o = [], []
    for _ in range(nsteps):
        st, nu, sw = o.step()
        assert st == 0
        nu_o.append(nu.copy())
        sw_o.append(sw.copy())
    nu_g, sw_g = g.step(nsteps)
    np.testing.assert_array_equal(np.array(sw_o), sw_g)
    np.testing.assert_array_equal(np.array(nu_o), nu_g)
    assert diff_fields(o, g) == {}


def test_zebra_matches_lex_at_convergence(oracle, P):
    """The two orderings converge to the same fields within the solver
    tolerance (the LEX path is the reference schedule)."""
    prm = config0_params(32, 64)
    _, glex = make_pair(oracle, P, smoother=0, tolcon=1e-12, **prm)
    _, gzeb = make_pair(oracle, P, smoother=1, tolcon=1e-12, **prm)
    glex.step(3)
    gzeb.step(3)
    for name in ("C", "th", "vel", "uel"):
        a, b = glex.get(name), gzeb.get(name)
        assert np.max(np.abs(a - b)) <= 1e-9 * max(1.0, np.max(np.abs(a))), name


def test_maxsweeps_status(oracle, P):
    """Where the reference STOPs the process (more than maxsweeps sweeps,
    PRB:1843) the device solve returns GB_MAXSWEEPS and leaves psi alone."""
    from codesthesis_dir_gb300 import lib
    o = oracle.OraclePRB(16, 32, 1e-4, 1e5, 1.0, r0=0.0, rmax=1.0, xx=2.0)
    o.initial(1, 1, 1e-2)
    g2 = P.PRB(16, 32, dt=1e-4, r0=0.0, rmax=1.0, xx=2.0, Ra=1e5, Pr=1.0, tolcon=1e-30, maxsweeps=3)
    for name in ("C", "Cp", "th", "thp"):
        g2.set(name, np.array(o.field(name), order="F"))
    g2.cvorticity1()
    g2.temperature1()
    g2.rhsv()
    before = g2.get("vel")
    with pytest.raises(lib.GBError) as ei:
        g2.poisson2()
    assert ei.value.status == lib.GB_MAXSWEEPS
    np.testing.assert_array_equal(before, g2.get("vel"))


@pytest.mark.parametrize("smoother", [0, 1], ids=["lex", "zebra"])
def test_graph_steps_oblique(oracle, P, smoother):
    """mpkoks.f (gravity along the diagonal, GB_PRB_OBLIQUE) through the same
    graph-replayed steps: fields, Nusselt numbers and sweep counts equal the
    oracle's bit for bit."""
    from prb_helpers import STATE_FIELDS
    from codesthesis_dir_gb300 import lib
    o = oracle.OraclePRB(16, 32, 1e-4, 1e5, 0.71, r0=0.5, rmax=1.0, xx=3.0, mode=smoother,
                         variant=oracle.ORC_OBLIQUE)
    o.initial(1, 7, 5e-2)
    g = P.PRB(16, 32, dt=1e-4, r0=0.5, rmax=1.0, xx=3.0, Ra=1e5, Pr=0.71, smoother=smoother,
              variant=lib.PRB_OBLIQUE)
    for name in STATE_FIELDS:
        g.set(name, np.array(o.field(name), order="F"))
    nu_o, sw_o = [], []
    for _ in range(6):
        st, nu, sw = o.step()
        assert st == 0
        nu_o.append(nu.copy())
        sw_o.append(sw.copy())
    nu_g, sw_g = g.step(6)
    np.testing.assert_array_equal(np.array(sw_o), sw_g)
    np.testing.assert_array_equal(np.array(nu_o), nu_g)
    assert diff_fields(o, g) == {}


@pytest.mark.parametrize("nr,np_", [(64, 128), (32, 64)])
def test_cluster_spread_solve_equals_one_cta(oracle, P, nr, np_):
    """The FP64 two-colour solve spread over a cluster of 8 CTAs gives
    exactly the bits of the one-CTA solve (the default) and of the oracle:
    fields, Nusselt numbers and sweep counts."""
    from codesthesis_dir_gb300 import lib
    L = lib.load()
    prm = config0_params(nr, np_)
    o, g8 = make_pair(oracle, P, smoother=1, tolcon=1e-10, **prm)
    _, g1 = make_pair(oracle, P, smoother=1, tolcon=1e-10, **prm)
    assert L.gb_prb_set_solve_spread(g1._h, 1) == 0
    assert L.gb_prb_set_solve_spread(g8._h, 8) == 0
    assert L.gb_prb_set_solve_spread(g8._h, 3) == lib.GB_ERR_INVALID
    nsteps = 8
    nu8, sw8 = g8.step(nsteps)
    nu1, sw1 = g1.step(nsteps)
    nu_o, sw_o = [], []
    for _ in range(nsteps):
        st, nu, sw = o.step()
        assert st == 0
        nu_o.append(nu.copy())
        sw_o.append(sw.copy())
    np.testing.assert_array_equal(sw8, sw1)
    np.testing.assert_array_equal(nu8, nu1)
    np.testing.assert_array_equal(np.array(sw_o), sw8)
    np.testing.assert_array_equal(np.array(nu_o), nu8)
    assert diff_fields(o, g8) == {}
    for name in ("C", "th", "vel", "uel"):
        np.testing.assert_array_equal(g8.get(name), g1.get(name))
