"""The rot3dmg.f drop-in symbols (libgb300r3d.so) driven as the reference's
main program drives its subroutines (rot3dmg.f:242-255), with the COMMON
blocks at the reference's PARAMETER bounds (kr = kz = 33, kp = 160) bound
from numpy: every field, the heat flux and every sweep count equal the
oracle's bit for bit, and the parts of the COMMON arrays outside the grid
come back untouched."""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KR, KZ, KP = 33, 33, 160
SOL1 = ["An", "A", "Ap", "Bn", "B", "Bp", "Cn", "C", "Cp"]
SOL2 = ["thn", "th", "thp"]
SOL3 = ["uel", "vel", "wel", "uelp", "velp", "welp"]
SENTINEL = 7.25


class Num(C.Structure):
    _fields_ = [("dt", C.c_double), ("dr", C.c_double), ("dz", C.c_double), ("dp", C.c_double),
                ("nr", C.c_int), ("nz", C.c_int), ("np", C.c_int)]


@pytest.fixture(scope="module")
def D(gblib):
    from codesthesis_dir_gb300 import lib
    return lib.load_r3d_dropin()


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.mark.parametrize("mode,horizontal", [(0, False), (1, False), (1, True)],
                         ids=["lex", "zebra", "horizontal-zebra"])
def test_main_loop_through_dropin(oracle, D, mode, horizontal):
    """horizontal: rot3dmghor.f's main loop through the same symbols with
    gb_r3d_bind_variant(GB_R3D_HORIZONTAL): heat(trans1, trans2) and both
    Nusselt numbers (rot3dmghor.f:255-267)."""
    nr, nz, np_ = 8, 8, 16
    prm = dict(dt=1e-5, r0=0.5, rmax=1.0, zmax=0.5, Ra=1e5, Re=100.0, Pr=0.7, Gr=0.0)
    if horizontal:
        prm.update(Ra=0.0, Re=0.0, Pr=7.0, Gr=1e4)
    o = oracle.OracleR3D(nr, nz, np_, prm["dt"], prm["r0"], prm["rmax"], prm["zmax"], prm["Ra"], prm["Re"],
                         prm["Pr"], Gr=prm["Gr"], mode=mode, horizontal=horizontal)
    o.initial(3, 5e-2)
    shp = (KR + 1, KZ + 1, KP + 1)
    S = int(np.prod(shp))
    ni, nj, nk = o.shape
    blocks = {"sol1": (SOL1, np.full(9 * S, SENTINEL)), "sol2": (SOL2, np.full(3 * S, SENTINEL)),
              "sol3": (SOL3, np.full(6 * S, SENTINEL))}

    def view(name):
        for names, buf in blocks.values():
            if name in names:
                q = names.index(name)
                return buf[q * S:(q + 1) * S].reshape(shp[::-1]).T
        raise KeyError(name)

    for name in SOL1 + SOL2 + SOL3:
        view(name)[:ni, :nj, :nk] = np.array(o.field(name))
    num = Num(prm["dt"], o.s.dr, o.s.dz, o.s.dp, nr, nz, np_)
    val = np.array([prm["Ra"], prm["Re"], prm["Pr"], prm["Gr"]])
    radius = np.array([prm["r0"], prm["rmax"]])
    rh = {n: np.full(S, SENTINEL) for n in ("wrh", "vrh", "urh")}
    for n in rh:
        rh[n].reshape(shp[::-1]).T[:ni, :nj, :nk] = 0.0
    D.gb_r3d_bind_bounds(KR, KZ, KP)
    D.gb_r3d_bind_common(_ptr(blocks["sol1"][1]), _ptr(blocks["sol2"][1]), _ptr(blocks["sol3"][1]),
                         C.cast(C.byref(num), C.c_void_p), _ptr(val), _ptr(radius))
    D.gb_r3d_bind_smoother(mode)
    D.gb_r3d_bind_variant(1 if horizontal else 0)
    ci = lambda v: C.byref(C.c_int(v))  # noqa: E731
    cd = lambda v: C.byref(C.c_double(v))  # noqa: E731
    nlev = C.c_int(0)
    D.poissoninit_(ci(nr), ci(nz), ci(np_), cd(o.s.dr), cd(o.s.dz), cd(o.s.dp), C.byref(nlev))
    assert D.gb_r3d_last_status() == 0 and nlev.value == o.s.nlev

    def vptr(name):
        for names, buf in blocks.values():
            if name in names:
                return C.c_void_p(buf.ctypes.data + 8 * S * names.index(name))

    args = (ci(nr), ci(nz), ci(np_), cd(o.s.dr), cd(o.s.dz), cd(o.s.dp), C.byref(nlev))
    pi = math.acos(-1.0)
    for step in range(3):
        st, nu_o, sw_o = o.step()
        assert st == 0
        D.avorticity_()
        D.bvorticity_()
        D.cvorticity_()
        D.temperature_()
        trans1, trans2 = C.c_double(), C.c_double()
        if horizontal:
            D.heat_(C.byref(trans1), C.byref(trans2))
        else:
            D.heat_(C.byref(trans1), None)   # rot3dmg.f's one-argument call: trans2 is not read
        sweeps = []
        for which, rhsn, fn, fnp, rfn in ((1, "wrh", "wel", "welp", D.rhsw_), (2, "vrh", "vel", "velp", D.rhsv_),
                                          (3, "urh", "uel", "uelp", D.rhsu_)):
            rfn(_ptr(rh[rhsn]))
            getattr(D, "poisson%d_" % which)(vptr(fn), vptr(fnp), _ptr(rh[rhsn]), *args)
            assert D.gb_r3d_last_status() == 0
            sweeps.append(D.gb_r3d_last_sweeps())
        D.update_()
        assert D.gb_r3d_last_status() == 0
        if horizontal:
            L = math.log(prm["r0"] / prm["rmax"])
            nu = nz / 6.0 * prm["r0"] * L * trans1.value / (prm["zmax"] * 2.0 * pi)
            nu2 = nz / 6.0 * prm["rmax"] * L * trans2.value / (prm["zmax"] * 2.0 * pi)
            assert nu2 == o.nu2, (step, nu2, o.nu2)
        else:
            nu = -prm["r0"] * math.log(prm["r0"] / prm["rmax"]) * trans1.value / (prm["zmax"] * 2.0 * pi)
        assert nu == nu_o, (step, nu, nu_o)
        assert sweeps == list(sw_o), (step, sweeps, sw_o)
        for name in SOL1 + SOL2 + SOL3:
            assert np.array_equal(view(name)[:ni, :nj, :nk], np.array(o.field(name))), (step, name)
        for n in ("wrh", "vrh", "urh"):
            assert np.array_equal(rh[n].reshape(shp[::-1]).T[:ni, :nj, :nk], np.array(o.field(n))), (step, n)
    for name in SOL1 + SOL2 + SOL3:
        a = view(name).copy()
        a[:ni, :nj, :nk] = SENTINEL
        assert np.all(a == SENTINEL), name
    D.gb_r3d_bind_common(None, None, None, None, None, None)
    D.gb_r3d_bind_variant(0)
