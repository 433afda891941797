"""Parity of the device horizontal-convection tank (GB_PRB_TANK,
monashubuntudir_velvor2dhorconvtankdir/velvor2dhorconvtank.f) and of the
differentially heated cavity (GB_PRB_DVD, velvor2ddvdbenchmark.f, the same
side-walled scheme) against the oracle, bit for bit: every field (np+2 columns), Nusselt number (with the
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


def make_tank(O, P, nr, np_, dt, Ra, smoother, tolcon=None, maxsweeps=None, dvd=False):
    from codesthesis_dir_gb300 import lib
    geo = dict(r0=0.0, rmax=1.0, xx=1.0, Pr=0.71) if dvd else dict(r0=0.5, rmax=1.5, xx=3.1, Pr=10.0)
    o = O.OraclePRB(nr, np_, dt, Ra, geo["Pr"], r0=geo["r0"], rmax=geo["rmax"], xx=geo["xx"], mode=smoother,
                    tolcon=tolcon, maxsweeps=maxsweeps, variant=O.ORC_DVD if dvd else O.ORC_TANK)
    o.initial()
    g = P.PRB(nr, np_, dt=dt, Ra=Ra, tolcon=tolcon, maxsweeps=maxsweeps, smoother=smoother,
              variant=lib.PRB_DVD if dvd else lib.PRB_TANK, **geo)
    assert g.nlev == o.mgv.nlev and g.ncol == np_ + 2
    for name in STATE_FIELDS:
        g.set(name, np.array(o.field(name), order="F"))
    return o, g


@pytest.mark.parametrize("dvd", [False, True], ids=["tank", "dvd"])
@pytest.mark.parametrize("smoother", [0, 1], ids=["lex", "zebra"])
def test_tank_routines(oracle, P, smoother, dvd):
    o, g = make_tank(oracle, P, 16, 32, 1e-6 if not dvd else 2e-5, 1e6 if not dvd else 1e5, smoother, dvd=dvd)
    c = 1.0 if dvd else 2.0
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
        want = (t2 * c, 0.0) if kt == 1 else (t1 * c, t2 * c)
        assert want == (nu[0], nu[1]), kt
        assert diff_fields(o, g, STATE_FIELDS) == {}, kt


@pytest.mark.parametrize("dvd", [False, True], ids=["tank", "dvd"])
@pytest.mark.parametrize("smoother", [0, 1], ids=["lex", "zebra"])
def test_tank_graph_steps(oracle, P, smoother, dvd):
    o, g = make_tank(oracle, P, 32, 64, 1e-6 if not dvd else 1e-5, 1e6 if not dvd else 1e5, smoother, dvd=dvd)
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
    if not dvd:
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
