"""Parity of the device rotating-annulus path (velvor2dnewsch3.4.f of
iarchomedir_groke_storage_users_mpking_rotannconvvelvorplane_continueddir)
against the oracle, bit for bit: every field, Nusselt number and multigrid
sweep count, routine by routine and over graph-replayed steps, with the
reference's own initial profile and with seeded noise, in both smoother
orderings; and the driver's behaviour at the sweep limit (no STOP)."""
import math

import numpy as np
import pytest

from prb_helpers import COMPARED, STATE_FIELDS, diff_fields

pytestmark = pytest.mark.gpu

ANN = dict(r0=0.5, rmax=1.0, Re=1.06148e5, Pr=0.71)


@pytest.fixture(scope="module")
def P(gblib):
    from codesthesis_dir_gb300 import prb
    return prb


def make_annulus(O, P, nr, np_, dt, Ra, smoother, tolcon=None, maxsweeps=None, kind=1, seed=0, amp=1e-2):
    o = O.OraclePRB(nr, np_, dt, Ra, ANN["Pr"], r0=ANN["r0"], rmax=ANN["rmax"], mode=smoother,
                    tolcon=tolcon, maxsweeps=maxsweeps, variant=O.ORC_ANNULUS, Re=ANN["Re"])
    o.initial(kind, seed, amp)
    g = P.PRB(nr, np_, dt=dt, r0=ANN["r0"], rmax=ANN["rmax"], Ra=Ra, Pr=ANN["Pr"], tolcon=tolcon,
              maxsweeps=maxsweeps, smoother=smoother, variant=1, Re=ANN["Re"])
    assert g.nlev == o.mgv.nlev
    for name in STATE_FIELDS:
        g.set(name, np.array(o.field(name), order="F"))
    return o, g


def nu_annulus(o, t1, t2):
    L = math.log(o.s.r0 / o.s.rmax)
    return -o.s.r0 * L * t1 / (2.0 * math.acos(-1.0)), -o.s.rmax * L * t2 / (2.0 * math.acos(-1.0))


@pytest.mark.parametrize("smoother", [0, 1], ids=["lex", "zebra"])
def test_routines_small(oracle, P, smoother):
    """Routine-by-routine on a 16 x 32 annulus (3 multigrid levels)."""
    o, g = make_annulus(oracle, P, 16, 32, 1e-6, 1e6, smoother, seed=3)
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
        assert nu_annulus(o, t1, t2) == (nu[0], nu[1]), kt
        assert diff_fields(o, g) == {}, kt


@pytest.mark.parametrize("smoother,kind", [(0, 0), (1, 0), (1, 1)], ids=["lex-refinit", "zebra-refinit", "zebra-noise"])
def test_graph_steps_five_levels(oracle, P, smoother, kind):
    """Graph-replayed steps on a 64 x 128 annulus, five multigrid levels
    (the annulus cap), reference tolerance 1e-5."""
    o, g = make_annulus(oracle, P, 64, 128, 2e-7, 8e7, smoother, kind=kind, seed=11)
    assert o.mgv.nlev == 5
    nsteps = 3 if smoother == 0 else 8
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


def test_sweep_limit_continues(oracle, P):
    """At the sweep limit the annulus solves return with psi untouched and
    the run goes on (velvor2dnewsch3.4.f:1853); the device does the same,
    identically to the oracle."""
    o, g = make_annulus(oracle, P, 16, 32, 1e-6, 1e6, 0, tolcon=1e-30, maxsweeps=2, seed=4)
    nu_o, sw_o = [], []
    for _ in range(3):
        st, nu, sw = o.step()
        assert st == 0
        nu_o.append(nu.copy())
        sw_o.append(sw.copy())
    nu_g, sw_g = g.step(3)
    np.testing.assert_array_equal(np.array(sw_o), sw_g)
    assert np.all(sw_g == 2)
    np.testing.assert_array_equal(np.array(nu_o), nu_g)
    assert diff_fields(o, g) == {}


def test_fields_unchanged_by_layer_entry_points(oracle, P):
    """The layer (PRB) instance and the annulus instance share kernels; a
    layer run after an annulus run in the same process still matches its
    own oracle (no state leaks between the variants)."""
    from prb_helpers import make_pair
    o, g = make_annulus(oracle, P, 16, 32, 1e-6, 1e6, 1, seed=8)
    g.step(2)
    o2, g2 = make_pair(oracle, P, 16, 32, 1e-4, 1e5, 1.0, 0.0, 1.0, 2.0, 1, 2e-6, seed=9, amp=1e-2)
    for _ in range(2):
        o2.step()
    g2.step(2)
    assert diff_fields(o2, g2, COMPARED) == {}


def make_taycou(O, P, nr, np_, dt, Ra, Ta, smoother, kind=0, seed=0, amp=1e-2, tolcon=None, maxsweeps=None):
    o = O.OraclePRB(nr, np_, dt, Ra, ANN["Pr"], r0=ANN["r0"], rmax=ANN["rmax"], mode=smoother, tolcon=tolcon,
                    maxsweeps=maxsweeps, variant=O.ORC_TAYCOU, Re=9.1927e4, Ta=Ta)
    o.initial(kind, seed, amp)
    from codesthesis_dir_gb300 import lib
    g = P.PRB(nr, np_, dt=dt, r0=ANN["r0"], rmax=ANN["rmax"], Ra=Ra, Pr=ANN["Pr"], tolcon=tolcon,
              maxsweeps=maxsweeps, smoother=smoother, variant=lib.PRB_TAYCOU, Re=9.1927e4, Ta=Ta)
    assert g.nlev == o.mgv.nlev
    for name in STATE_FIELDS:
        g.set(name, np.array(o.field(name), order="F"))
    return o, g


@pytest.mark.parametrize("smoother", [0, 1], ids=["lex", "zebra"])
def test_taylor_couette_routines_and_steps(oracle, P, smoother):
    """velvor2dtaycouheat.f (GB_PRB_TAYCOU): the moving outer cylinder, its
    wall vorticity and rhsv term, Robert filter 0.01, PRB's multigrid with the
    polar operator; routine by routine and then graph-replayed, every field,
    Nusselt number and sweep count equal to the oracle's."""
    o, g = make_taycou(oracle, P, 16, 32, 1e-6, 1e6, 1e4, smoother)
    for kt in range(1, 4):
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
        assert nu_annulus(o, t1, t2) == (nu[0], nu[1]), kt
        assert diff_fields(o, g) == {}, kt
    g.kt = 3
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
    assert np.all(g.get("vel")[17] == -(1e4 ** 0.5) * ANN["Pr"] * 0.5 * ANN["rmax"])


def test_taylor_couette_four_levels_and_stop(oracle, P):
    """At most four levels where the annulus has five, and the sweep limit
    stops the run (the driver STOPs) on the device as in the oracle."""
    from codesthesis_dir_gb300 import lib
    o, g = make_taycou(oracle, P, 64, 64, 1e-6, 1e6, 1e4, 1)
    assert g.nlev == 4
    o, g = make_taycou(oracle, P, 16, 32, 1e-6, 1e6, 1e4, 0, tolcon=1e-30, maxsweeps=3)
    st, nu, sw = o.step()
    assert st == 1 and sw[0] == 3
    with pytest.raises(lib.GBError) as ei:
        g.step(2)
    assert ei.value.status == lib.GB_MAXSWEEPS
