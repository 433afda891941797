"""The time-loop diagnostics of the device step (PRB:404-493,
velvor2dnewsch3.4.f:404-493; after the update of the tank and the cavity,
velvor2dhorconvtank.f:424-513 and velvor2ddvdbenchmark.f:434-518) against
the oracle: the four running means and
every step's CFL maxima bit for bit, the zonal T variance bit for bit and the
zonal rms of u and v to an ulp (sqrt against libm pow), over a first block
and a "more iterations" block that starts the means again; the step's
fields are unchanged by the diagnostics."""
import numpy as np
import pytest

from prb_helpers import COMPARED, STATE_FIELDS, config0_params, diff_fields

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gblib):
    from codesthesis_dir_gb300 import prb
    return prb


def _pair(O, P, variant, smoother):
    if variant == "layer":
        p = config0_params(16, 32)
        o = O.OraclePRB(p["nr"], p["np_"], 2e-4, 1e6, p["Pr"], r0=p["r0"], rmax=p["rmax"], xx=p["xx"],
                        mode=smoother)
        g = P.PRB(p["nr"], p["np_"], dt=2e-4, r0=p["r0"], rmax=p["rmax"], xx=p["xx"], Ra=1e6, Pr=p["Pr"],
                  smoother=smoother)
    elif variant == "annulus":
        kw = dict(r0=0.5, rmax=1.0, Re=1.06148e5)
        o = O.OraclePRB(16, 32, 1e-6, 1e6, 0.71, mode=smoother, variant=O.ORC_ANNULUS, **kw)
        g = P.PRB(16, 32, dt=1e-6, Ra=1e6, Pr=0.71, smoother=smoother, variant=1, **kw)
    else:
        from codesthesis_dir_gb300 import lib
        dvd = variant == "dvd"
        geo = dict(r0=0.0, rmax=1.0, xx=1.0, Pr=0.71) if dvd else dict(r0=0.5, rmax=1.5, xx=3.1, Pr=10.0)
        dt, Ra = (2e-5, 1e5) if dvd else (1e-5, 1e6)
        o = O.OraclePRB(16, 32, dt, Ra, geo["Pr"], r0=geo["r0"], rmax=geo["rmax"], xx=geo["xx"], mode=smoother,
                        variant=O.ORC_DVD if dvd else O.ORC_TANK)
        g = P.PRB(16, 32, dt=dt, Ra=Ra, smoother=smoother, variant=lib.PRB_DVD if dvd else lib.PRB_TANK, **geo)
    if variant in ("tank", "dvd"):
        o.initial()
    else:
        o.initial(1, 5, 5e-2)
    for name in STATE_FIELDS:
        g.set(name, np.array(o.field(name), order="F"))
    o.enable_diagnostics()
    g.diagnostics(True)
    return o, g


def _check(o, g, cfl_o):
    for q in range(4):
        np.testing.assert_array_equal(g.running_mean(q), o.running_mean(q), err_msg="mean %d" % q)
    zo, zg = o.zmtm(), g.zonal()
    np.testing.assert_array_equal(zg[:, 0], zo[:, 0])
    np.testing.assert_allclose(zg[:, 1:], zo[:, 1:], rtol=4.5e-16, atol=0.0)
    assert diff_fields(o, g, COMPARED) == {}


@pytest.mark.parametrize("variant", ["layer", "annulus", "tank", "dvd"])
@pytest.mark.parametrize("smoother", [0, 1], ids=["lex", "zebra"])
def test_diagnostics_two_blocks(oracle, P, variant, smoother):
    o, g = _pair(oracle, P, variant, smoother)
    n1 = 7
    for _ in range(n1):
        assert o.step()[0] == 0
    g.step(n1)
    assert np.array_equal(g.cfl(n1), np.array(o.cfl_hist))
    assert o.cfl_hist[0] == (0.0, 0.0) and o.cfl_hist[-1][0] > 0.0 and o.cfl_hist[-1][1] > 0.0
    _check(o, g, o.cfl_hist)
    # a "more iterations" block: kt = 2.. again, the means start again
    o.new_block()
    g.new_block()
    o.cfl_hist = []
    n2 = 4
    for _ in range(n2):
        assert o.step()[0] == 0
    g.step(n2)
    assert np.array_equal(g.cfl(n2), np.array(o.cfl_hist))
    _check(o, g, o.cfl_hist)


def test_diagnostics_off_leave_the_step_alone(oracle, P):
    o, g = _pair(oracle, P, "layer", 1)
    g.diagnostics(False)
    for _ in range(5):
        assert o.step()[0] == 0
    g.step(5)
    assert diff_fields(o, g, COMPARED) == {}
