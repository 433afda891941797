"""Parity of the device horizontal-convection tank (GB_PRB_TANK,
monashubuntudir_velvor2dhorconvtankdir/velvor2dhorconvtank.f) against the
oracle, bit for bit: every field (np+2 columns), Nusselt number (with the
first step's httrans quirk) and multigrid sweep count, routine by routine
and over graph-replayed steps, in both line orders; the sweep limit stops
the run."""
import numpy as np
import pytest

from prb_helpers import COMPARED, STATE_FIELDS, diff_fields

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gblib):
    from codesthesis_dir_gb300 import prb
    return prb


def make_tank(O, P, nr, np_, dt, Ra, smoother, tolcon=None, maxsweeps=None):
    from codesthesis_dir_gb300 import lib
    o = O.OraclePRB(nr, np_, dt, Ra, 10.0, r0=0.5, rmax=1.5, xx=3.1, mode=smoother, tolcon=tolcon,
                    maxsweeps=maxsweeps, variant=O.ORC_TANK)
    o.initial()
    g = P.PRB(nr, np_, dt=dt, r0=0.5, rmax=1.5, xx=3.1, Ra=Ra, Pr=10.0, tolcon=tolcon, maxsweeps=maxsweeps,
              smoother=smoother, variant=lib.PRB_TANK)
    assert g.nlev == o.mgv.nlev and g.ncol == np_ + 2
    for name in STATE_FIELDS:
        g.set(name, np.array(o.field(name), order="F"))
    return o, g


@pytest.mark.parametrize("smoother", [0, 1], ids=["lex", "zebra"])
def test_tank_routines(oracle, P, smoother):
    o, g = make_tank(oracle, P, 16, 32, 1e-6, 1e6, smoother)
    for kt in range(1, 5):
        st, nu, sw = o.step()
        assert st == 0
        (g.cvorticity1 if kt == 1 else g.cvorticity)()
        (g.temperature1 if kt == 1 else g.temperature)()
        t1, t2 = g.heat()
        g.rhsv()
        sv = g.poisson2()
        g.rhsu()
        su = g.poisson3()
        g.update()
        assert (sv, su) == (int(sw[0]), int(sw[1])), kt
        want = (t2 * 2.0, 0.0) if kt == 1 else (t1 * 2.0, t2 * 2.0)
        assert want == (nu[0], nu[1]), kt
        assert diff_fields(o, g, STATE_FIELDS) == {}, kt


@pytest.mark.parametrize("smoother", [0, 1], ids=["lex", "zebra"])
def test_tank_graph_steps(oracle, P, smoother):
    o, g = make_tank(oracle, P, 32, 64, 1e-6, 1e6, smoother)
    nu_o, sw_o = [], []
    for _ in range(8):
        st, nu, sw = o.step()
        assert st == 0
        nu_o.append(nu.copy())
        sw_o.append(sw.copy())
    nu_g, sw_g = g.step(8)
    np.testing.assert_array_equal(np.array(sw_o), sw_g)
    np.testing.assert_array_equal(np.array(nu_o), nu_g)
    assert diff_fields(o, g, STATE_FIELDS) == {}
    th = g.get("th")
    np.testing.assert_array_equal(th[:, 65], 2.0 / 1.5 * th[:, 64] - 1.0 / 3.0 * th[:, 63])


def test_tank_sweep_limit_stops(oracle, P):
    from codesthesis_dir_gb300 import lib
    o, g = make_tank(oracle, P, 16, 32, 1e-6, 1e6, 0, tolcon=1e-30, maxsweeps=3)
    assert o.step()[0] == 0        # the start is at rest: zero right-hand sides converge at once
    st, nu, sw = o.step()
    assert st == 1 and sw[0] == 3
    with pytest.raises(lib.GBError) as ei:
        g.step(3)
    assert ei.value.status == lib.GB_MAXSWEEPS
