"""Parity of the device 3D rotating annulus (rot3dmg.f) against the oracle,
bit for bit: every field, the heat flux and Nusselt numbers and the
multigrid sweep counts, routine by routine (the drop-in granularity) and
over whole steps, in the reference's line order (run as wavefronts) and in
the two-colour order, on grids with two and three multigrid levels and with
nr != nz; random fields large enough to switch on the hybrid upwinding
(cell Peclet number > 2) in every direction; and the sweep limit (the
reference STOPs)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ["An", "A", "Ap", "Bn", "B", "Bp", "Cn", "C", "Cp", "thn", "th", "thp",
          "uel", "vel", "wel", "uelp", "velp", "welp", "urh", "vrh", "wrh"]


@pytest.fixture(scope="module")
def R(gblib):
    from codesthesis_dir_gb300 import r3d
    return r3d


PRM = dict(dt=1e-5, r0=0.5, rmax=1.0, zmax=0.5, Ra=1e5, Re=100.0, Pr=0.7)


def make(O, R, nr, nz, np_, mode, prm=PRM, tolcon=None, maxsweeps=None, init="ref", seed=0, amp=1e-2, vscale=0.0):
    o = O.OracleR3D(nr, nz, np_, prm["dt"], prm["r0"], prm["rmax"], prm["zmax"], prm["Ra"], prm["Re"], prm["Pr"],
                    mode=mode, tolcon=tolcon, maxsweeps=maxsweeps)
    o.initial(3, amp)
    if init == "random":
        rng = np.random.default_rng(seed)
        for n in ("A", "Ap", "B", "Bp", "C", "Cp"):
            o.field(n)[...] = rng.standard_normal(o.shape)
        for n in ("uel", "vel", "wel", "uelp", "velp", "welp"):
            o.field(n)[...] = vscale * rng.standard_normal(o.shape)
        o.field("th")[...] += 0.1 * rng.standard_normal(o.shape)
        o.field("thp")[...] = np.array(o.field("th")) + 1e-3 * rng.standard_normal(o.shape)
    g = R.R3D(nr, nz, np_, smoother=mode, tolcon=tolcon, maxsweeps=maxsweeps, **prm)
    assert g.nlev == o.s.nlev
    for n in FIELDS:
        g.set(n, np.array(o.field(n)))
    return o, g


def wall_free_velocities(o, rng, scale):
    """Random velocities (both time levels) on each component's own interior,
    zero on its walls and with plane 0 equal to plane np, as the reference's
    solves leave them (rot3dmg.f:1291-1315): the z-line solves of relax1 and
    the r-line solves of relax3 take the walls as zero (the Thomas algorithm
    has no a(1) / c(n) term) while the residual reads them."""
    nr, nz = o.s.nr, o.s.nz
    for name, (i1, j1) in (("wel", (nr + 1, nz)), ("vel", (nr + 1, nz + 1)), ("uel", (nr, nz + 1))):
        for suffix in ("", "p"):
            a = np.zeros(o.shape)
            a[1:i1, 1:j1, :] = scale * rng.standard_normal((i1 - 1, j1 - 1, o.shape[2]))
            a[:, :, 0] = a[:, :, -1]
            o.field(name + suffix)[...] = a


def diff(o, g):
    bad = {}
    for n in FIELDS:
        a, b = np.array(o.field(n)), g.get(n)
        if not np.array_equal(a, b):
            bad[n] = float(np.max(np.abs(a - b)))
    return bad


@pytest.mark.parametrize("mode", [0, 1], ids=["lex", "zebra"])
@pytest.mark.parametrize("nr,nz,np_", [(8, 8, 16), (16, 8, 16), (8, 16, 32)])
def test_routines_random_fields(oracle, R, mode, nr, nz, np_):
    """Every routine once, from random fields with velocities up to ~100
    (upwinding active): transport, heat, right-hand sides, the three solves
    (with their sweep counts), update."""
    o, g = make(oracle, R, nr, nz, np_, mode, init="random", seed=nr + nz, vscale=40.0)
    for name in ("avorticity", "bvorticity", "cvorticity", "temperature"):
        o.call(name)
        getattr(g, name)()
        assert diff(o, g) == {}, name
    assert g.heat() == o.call("heat")
    # the solves from states the reference can reach: wall-free velocities
    # and vorticities small enough that the solve's residual stall (the
    # REAL*4 0.2 of relax1/2/3) stays below tolcon
    rng = np.random.default_rng(7)
    wall_free_velocities(o, rng, 1e-2)
    for n in ("An", "Bn", "Cn"):
        o.field(n)[...] *= 1e-3
    for n in ("An", "Bn", "Cn", "uel", "vel", "wel", "uelp", "velp", "welp"):
        g.set(n, np.array(o.field(n)))
    for which, rhs in ((1, "rhsw"), (2, "rhsv"), (3, "rhsu")):
        o.call(rhs)
        getattr(g, rhs)()
        assert diff(o, g) == {}, rhs
        st, sw = o.poisson(which)
        assert st == 0, (which, st, sw)
        assert g.poisson(which) == sw, which
        assert diff(o, g) == {}, "poisson%d" % which
    o.call("update")
    g.update()
    assert diff(o, g) == {}, "update"


@pytest.mark.parametrize("mode", [0, 1], ids=["lex", "zebra"])
def test_steps_three_levels(oracle, R, mode):
    """Whole steps on a 16 x 16 x 32 annulus (three levels) from the
    reference's initial state: fields, Nusselt numbers, sweep counts."""
    o, g = make(oracle, R, 16, 16, 32, mode, amp=5e-2)
    n = 4
    nu_o, sw_o = [], []
    for _ in range(n):
        st, nu, sw = o.step()
        assert st == 0
        nu_o.append(nu)
        sw_o.append(sw.copy())
    nu_g, sw_g = g.step(n)
    np.testing.assert_array_equal(np.array(sw_o), sw_g)
    np.testing.assert_array_equal(np.array(nu_o), nu_g)
    assert diff(o, g) == {}


def test_steps_two_levels_random(oracle, R):
    o, g = make(oracle, R, 8, 8, 16, 1, init="random", seed=3, vscale=1.0)
    wall_free_velocities(o, np.random.default_rng(5), 1e-2)
    for n in ("A", "Ap", "B", "Bp", "C", "Cp"):
        o.field(n)[...] *= 1e-2
    for n in FIELDS:
        g.set(n, np.array(o.field(n)))
    for _ in range(3):
        st, nu, sw = o.step()
        assert st == 0
    nu_g, sw_g = g.step(3)
    assert len(nu_g) == 3 and nu_g[-1] == nu
    assert diff(o, g) == {}


def test_sweep_limit_stops(oracle, R):
    """Beyond the sweep limit the reference STOPs; the device solve reports
    GB_MAXSWEEPS after the same number of sweeps and the step loop ends."""
    from codesthesis_dir_gb300 import lib
    o, g = make(oracle, R, 8, 8, 16, 1, tolcon=1e-30, maxsweeps=3)
    st, nu, sw = o.step()
    assert st == 1 and sw[0] == 3
    with pytest.raises(lib.GBError) as ei:
        g.step(2)
    assert ei.value.status == lib.GB_MAXSWEEPS
    assert g.steps_done == 0 and g.last_sweeps[0][0] == 3


@pytest.mark.parametrize("mode", [0, 1], ids=["lex", "zebra"])
def test_horizontal_annulus_steps(oracle, R, mode):
    """rot3dmghor.f (GB_R3D_HORIZONTAL) from its own start: gravity across
    the axis, both cylinders' Nusselt numbers, the plain V-cycle at tolcon
    1e-6; fields, httrans1, httrans2 and sweep counts equal the oracle's bit
    for bit, step by step and through the routines."""
    from codesthesis_dir_gb300 import lib
    prm = dict(dt=1e-5, r0=0.5, rmax=1.0, zmax=0.5, Ra=0.0, Re=0.0, Pr=7.0, Gr=1e4)
    o = oracle.OracleR3D(8, 8, 16, prm["dt"], prm["r0"], prm["rmax"], prm["zmax"], prm["Ra"], prm["Re"], prm["Pr"],
                         Gr=prm["Gr"], mode=mode, horizontal=True)
    o.initial(3, 5e-2)
    g = R.R3D(8, 8, 16, smoother=mode, variant=lib.R3D_HORIZONTAL, **prm)
    assert g.params.tolcon == 1e-6 and g.nlev == o.s.nlev
    for n in FIELDS:
        g.set(n, np.array(o.field(n)))
    nus, nu2s, sws = [], [], []
    for _ in range(3):
        st, nu, sw = o.step()
        assert st == 0
        nus.append(nu)
        nu2s.append(o.nu2)
        sws.append(sw.copy())
    nu_g, sw_g = g.step(3)
    assert list(nu_g) == nus and list(g.nu2) == nu2s
    np.testing.assert_array_equal(sw_g, np.array(sws))
    assert diff(o, g) == {}
    # one more step routine by routine, heat(trans1, trans2) included
    import ctypes as C
    o.call("avorticity")
    o.call("bvorticity")
    o.call("cvorticity")
    o.call("temperature")
    t2 = C.c_double()
    t1 = oracle.lib().orc_r3d_heat2(C.byref(o.s), C.byref(t2))
    g.avorticity()
    g.bvorticity()
    g.cvorticity()
    g.temperature()
    assert g.heat2() == (t1, t2.value)
    for which, rhs in ((1, "rhsw"), (2, "rhsv"), (3, "rhsu")):
        o.call(rhs)
        getattr(g, rhs)()
        st, sw = o.poisson(which)
        assert st == 0 and g.poisson(which) == sw
    o.call("update")
    g.update()
    assert diff(o, g) == {}
