"""Parity of the device axisymmetric annulus (rotann2.f) against the oracle,
bit for bit: every field, the heat flux and Nusselt numbers, the multigrid
sweep counts and the steady-state stop, routine by routine (the drop-in
granularity) and over graph-replayed steps, in both line orderings, on
grids with nr > nz and nr < nz (the second makes corser's use of n1 for
both directions clear an interior coarse row)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ["phi", "omegn", "omeg", "omegp", "veln", "vel", "velp", "thetan", "theta", "thetap"]


@pytest.fixture(scope="module")
def A(gblib):
    from codesthesis_dir_gb300 import axi
    return axi


def make(O, A, nr, nz, mode, kind=1, seed=0, amp=1e-2, tolcon=None, Ra=1e5, Re=1e2, dt=1e-5):
    prm = dict(dt=dt, r0=0.5, rmax=1.0, zmax=0.5, Ra=Ra, Re=Re, Pr=1.0)
    o = O.OracleAXI(nr, nz, prm["dt"], prm["r0"], prm["rmax"], prm["zmax"], prm["Ra"], prm["Re"], prm["Pr"],
                    mode=mode, tolcon=tolcon)
    o.initial(kind, seed, amp)
    g = A.AXI(nr, nz, smoother=mode, tolcon=tolcon, **prm)
    assert g.nlev == o.s.nlev
    for n in FIELDS:
        g.set(n, np.array(o.field(n)))
    return o, g


def diff(o, g):
    bad = {}
    for n in FIELDS:
        a, b = np.array(o.field(n)), g.get(n)
        if not np.array_equal(a, b):
            bad[n] = float(np.max(np.abs(a - b)))
    return bad


@pytest.mark.parametrize("mode", [0, 1], ids=["lex", "zebra"])
@pytest.mark.parametrize("nr,nz", [(32, 16), (16, 32)])
def test_routines(oracle, A, mode, nr, nz):
    import ctypes as C
    o, g = make(oracle, A, nr, nz, mode, seed=5)
    L = oracle.lib()
    for step in range(4):
        L.orc_axi_vorticity(C.byref(o.s))
        L.orc_axi_velocity(C.byref(o.s))
        L.orc_axi_temperature(C.byref(o.s))
        sw = C.c_int()
        st = L.orc_axi_poisson(C.byref(o.s), o.s.phi, o.s.omegn, C.byref(sw))
        L.orc_axi_update(C.byref(o.s))
        t_o = L.orc_axi_heat(C.byref(o.s))
        g.vorticity()
        g.velocity()
        g.temperature()
        sw_g = g.poisson()
        g.update()
        t_g = g.heat()
        assert st == 0 and sw_g == sw.value, (step, st, sw.value, sw_g)
        assert t_g == t_o, step
        assert diff(o, g) == {}, step


@pytest.mark.parametrize("mode,kind", [(0, 0), (1, 0), (1, 1)], ids=["lex-ref", "zebra-ref", "zebra-noise"])
def test_graph_steps(oracle, A, mode, kind):
    o, g = make(oracle, A, 64, 64, mode, kind=kind, seed=2, amp=1e-3, Ra=1e6)
    n = 6
    nu_o, sw_o = [], []
    for _ in range(n):
        st, nu, sw, conv = o.step()
        assert st == 0 and not conv
        nu_o.append(nu)
        sw_o.append(sw)
    nu_g, sw_g = g.step(n)
    assert len(nu_g) == n
    np.testing.assert_array_equal(np.array(sw_o), sw_g)
    np.testing.assert_array_equal(np.array(nu_o), nu_g)
    assert diff(o, g) == {}


def test_steady_state_stop(oracle, A):
    """From the conduction state with no perturbation the run is steady at
    once: the reference stops after the first step (rotann2.f:191), and so
    does the device loop."""
    o, g = make(oracle, A, 32, 32, 1, kind=1, amp=0.0, Ra=1e2)
    st, nu, sw, conv = o.step()
    nu_g, sw_g = g.step(5)
    assert conv and len(nu_g) == 1
    assert nu_g[0] == nu
    assert diff(o, g) == {}
