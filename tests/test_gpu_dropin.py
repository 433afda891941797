"""The gfortran-compatible drop-in symbols (poissoninit_, cvorticity1_, ...,
update_) driven the way the Fortran main program drives them (PRB:341-388),
with COMMON blocks laid out as gfortran lays them out, against the oracle.
The same symbols serve the rotating-annulus driver (velvor2dnewsch3.4.f,
main loop :341-387) once gb_prb_bind_variant selects it.
"""
import ctypes as C
import math

import numpy as np
import pytest

from prb_helpers import STATE_FIELDS

pytestmark = pytest.mark.gpu


class Num(C.Structure):  # COMMON /num/ dt,dr,dz,dp,nr,nz,np
    _fields_ = [("dt", C.c_double), ("dr", C.c_double), ("dz", C.c_double), ("dp", C.c_double),
                ("nr", C.c_int), ("nz", C.c_int), ("np", C.c_int)]


SOL1 = ["An", "A", "Ap", "Bn", "B", "Bp", "Cn", "C", "Cp"]
SOL2 = ["thn", "th", "thp"]
SOL3 = ["uel", "vel", "wel", "uelp", "velp", "welp"]


@pytest.mark.parametrize("kr,kp,variant", [(20, 40, 0), (290, 1610, 0), (20, 40, 1), (420, 3600, 1), (20, 40, 2),
                                           (20, 40, 3), (20, 40, 4), (20, 40, 5)],
                         ids=["small-bounds", "reference-bounds", "annulus-small-bounds", "annulus-reference-bounds",
                              "oblique-small-bounds", "taycou-small-bounds", "tank-small-bounds", "dvd-small-bounds"])
def test_dropin_main_loop(oracle, gblib, kr, kp, variant):
    """variant 0: PRB; 1: the annulus (velvor2dnewsch3.4.f); 2: mpkoks.f's
    oblique gravity (the same names, gb_prb_bind_variant(2)); 3: the
    Taylor-Couette driver (velvor2dtaycouheat.f, Ta in /val/'s Gr slot); 4:
    the tank (velvor2dhorconvtank.f: np+2 columns, Nu = 2 trans with the
    first step's swap)."""
    L = gblib
    nr, np_ = 16, 32
    dt, Ra, Pr, r0, rmax, xx, Re = 1e-4, 1e5, 0.71, 0.5, 1.0, 3.0, 1e4
    ann = variant in (1, 3)
    tank = variant in (4, 5)
    Ta = 1e4 if variant == 3 else 0.0
    if ann:
        dt, Ra = 1e-6, 1e6
    if variant == 4:
        dt, Ra, Pr, r0, rmax, xx = 1e-6, 1e6, 10.0, 0.5, 1.5, 3.1
    if variant == 5:
        dt, Ra, Pr, r0, rmax, xx = 2e-5, 1e5, 0.71, 0.0, 1.0, 1.0
    tol, maxsw = {1: (10e-6, 10000), 3: (1e-5, 500), 4: (5e-6, 500), 5: (5e-6, 500)}.get(variant, (2e-6, 500))
    ncol = np_ + 2 if tank else np_ + 1
    o = oracle.OraclePRB(nr, np_, dt, Ra, Pr, r0=r0, rmax=rmax, xx=xx, variant=variant, Re=Re, Ta=Ta)
    o.initial(0, 0, 0.0)  # the reference's own initial profile (PRB:137-186, annulus :130-178)
    S = (kr + 1) * (kp + 1)
    sol1 = np.zeros(9 * S)
    sol2 = np.zeros(3 * S)
    sol3 = np.zeros(6 * S)
    vrh = np.zeros(S)
    urh = np.zeros(S)

    def view(block, idx):
        return block[idx * S:(idx + 1) * S].reshape((kp + 1, kr + 1)).T

    for blk, names in ((sol1, SOL1), (sol2, SOL2), (sol3, SOL3)):
        for i, nm in enumerate(names):
            view(blk, i)[: nr + 2, : ncol] = np.array(o.field(nm))
    num = Num(dt, o.s.dr, 0.0, o.s.dp, nr, 1, np_)
    val = np.array([Ra, Re if ann else 0.0, Pr, Ta])
    radius = np.array([r0, rmax])
    L.gb_prb_bind_bounds(kr, kp)
    L.gb_prb_bind_tolerance(tol, maxsw)
    L.gb_prb_bind_smoother(0)
    L.gb_prb_bind_variant(variant)
    L.gb_prb_bind_radius(radius.ctypes.data)
    L.gb_prb_bind_common(sol1.ctypes.data, sol2.ctypes.data, sol3.ctypes.data, C.addressof(num), val.ctypes.data)
    try:
        nrc, nzc, npc = C.c_int(nr), C.c_int(1), C.c_int(np_)
        drc, dzc, dpc = C.c_double(o.s.dr), C.c_double(0.0), C.c_double(o.s.dp)
        nlev = C.c_int(0)
        L.poissoninit_(C.byref(nrc), C.byref(nzc), C.byref(npc), C.byref(drc), C.byref(dzc), C.byref(dpc),
                       C.byref(nlev))
        assert nlev.value == o.mgv.nlev
        vel, velp = view(sol3, 1), view(sol3, 4)
        uel, uelp = view(sol3, 0), view(sol3, 3)
        # the three arrays are views into the COMMON storage: pass raw addresses
        a_vel = sol3.ctypes.data + 1 * S * 8
        a_velp = sol3.ctypes.data + 4 * S * 8
        a_uel = sol3.ctypes.data + 0 * S * 8
        a_uelp = sol3.ctypes.data + 3 * S * 8
        for kt in range(1, 5):
            st, nu, sw = o.step()
            assert st == 0
            (L.cvorticity1_ if kt == 1 else L.cvorticity_)()
            (L.temperature1_ if kt == 1 else L.temperature_)()
            t1, t2 = C.c_double(), C.c_double()
            L.heat_(C.byref(t1), C.byref(t2))
            L.rhsv_(vrh.ctypes.data)
            L.poisson2_(a_vel, a_velp, vrh.ctypes.data, C.byref(nrc), C.byref(nzc), C.byref(npc), C.byref(drc),
                        C.byref(dzc), C.byref(dpc), C.byref(nlev))
            assert L.gb_prb_last_status() == 0
            assert L.gb_prb_last_sweeps() == sw[0]
            L.rhsu_(urh.ctypes.data)
            L.poisson3_(a_uel, a_uelp, urh.ctypes.data, C.byref(nrc), C.byref(nzc), C.byref(npc), C.byref(drc),
                        C.byref(dzc), C.byref(dpc), C.byref(nlev))
            assert L.gb_prb_last_status() == 0
            assert L.gb_prb_last_sweeps() == sw[1]
            L.update_()
            assert L.gb_prb_last_status() == 0
            if tank:
                c = 1.0 if variant == 5 else 2.0
                assert (t2.value * c if kt == 1 else t1.value * c) == nu[0]
            elif ann:
                assert -r0 * math.log(r0 / rmax) * t1.value / (2.0 * math.acos(-1.0)) == nu[0]
            else:
                assert t1.value * (rmax - r0) / xx == nu[0]
            for blk, names in ((sol1, SOL1), (sol2, SOL2), (sol3, SOL3)):
                for i, nm in enumerate(names):
                    np.testing.assert_array_equal(view(blk, i)[: nr + 2, : ncol], np.array(o.field(nm)),
                                                  err_msg="%s kt=%d" % (nm, kt))
        del vel, velp, uel, uelp
    finally:
        L.gb_prb_bind_common(None, None, None, None, None)
        L.gb_prb_bind_radius(None)
        L.gb_prb_bind_variant(0)
        L.gb_prb_bind_tolerance(2e-6, 500)
        L.gb_prb_bind_bounds(290, 1610)
