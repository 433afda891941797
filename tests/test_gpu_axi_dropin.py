"""The rotann2.f drop-in symbols (libgb300axi.so) driven as the reference's
main program drives its subroutines (rotann2.f:145-153: vorticity,
velocity, temperature, poisson(phi, omegn), update, heat), with the COMMON
blocks /sol1/ /sol2/ /num/ /val/ /radius/ laid out as gfortran lays them out
at the reference's PARAMETER bounds (nrmax = nzmax = 128) and at small
ones: every field, the heat flux and every sweep count equal the oracle's
bit for bit, and the parts of the arrays outside the grid come back
untouched."""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SOL1 = ["phi", "omegn", "omeg", "omegp", "veln", "vel", "velp"]
SOL2 = ["thetan", "theta", "thetap"]
SENTINEL = -3.5


class Num(C.Structure):   # COMMON /num/ dr,dz,nr,nz,dt (rotann2.f:22)
    _fields_ = [("dr", C.c_double), ("dz", C.c_double), ("nr", C.c_int), ("nz", C.c_int), ("dt", C.c_double)]


@pytest.fixture(scope="module")
def D(gblib):
    from codesthesis_dir_gb300 import lib
    return lib.load_axi_dropin()


@pytest.mark.parametrize("bounds,mode", [(128, 0), (40, 1)], ids=["reference-bounds-lex", "small-bounds-zebra"])
def test_main_loop_through_dropin(oracle, D, bounds, mode):
    nr, nz = 32, 16
    prm = dict(dt=1e-5, r0=0.5, rmax=1.0, zmax=0.5, Ra=1e5, Re=1e2, Pr=1.0)
    o = oracle.OracleAXI(nr, nz, prm["dt"], prm["r0"], prm["rmax"], prm["zmax"], prm["Ra"], prm["Re"], prm["Pr"],
                         mode=mode)
    o.initial(1, 5, 1e-2)
    S = (bounds + 1) * (bounds + 1)
    sol1 = np.full(7 * S, SENTINEL)
    sol2 = np.full(3 * S, SENTINEL)

    def view(name):
        buf, names = (sol1, SOL1) if name in SOL1 else (sol2, SOL2)
        q = names.index(name)
        return buf[q * S:(q + 1) * S].reshape(bounds + 1, bounds + 1).T

    for name in SOL1 + SOL2:
        view(name)[:nr + 1, :nz + 1] = np.array(o.field(name))
    s = o.s
    dt, Ptl, dr, dz = prm["dt"], prm["Pr"], s.dr, s.dz
    # /val/ as the main program forms it (rotann2.f:66-69)
    cf = [1.0 / (2.0 * Ptl * dt) + 1.0 / (dr * dr) + 1.0 / (dz * dz),
          1.0 / (2.0 * Ptl * dt) - 1.0 / (dr * dr) - 1.0 / (dz * dz),
          1.0 / (2.0 * dt) + 1.0 / (dr * dr) + 1.0 / (dz * dz),
          1.0 / (2.0 * dt) - 1.0 / (dr * dr) - 1.0 / (dz * dz)]
    val = np.array(cf + [prm["Ra"], prm["Re"], Ptl])
    num = Num(dr, dz, nr, nz, dt)
    radius = np.array([prm["r0"]])
    D.gb_axi_bind_bounds(bounds, bounds)
    D.gb_axi_bind_smoother(mode)
    D.gb_axi_bind_common(sol1.ctypes.data, sol2.ctypes.data, C.cast(C.byref(num), C.c_void_p), val.ctypes.data,
                         radius.ctypes.data)
    try:
        D.poissoninit_(C.byref(C.c_int(nr)), C.byref(C.c_int(nz)), C.byref(C.c_double(dr)), C.byref(C.c_double(dz)))
        assert D.gb_axi_last_status() == 0
        phi = C.c_void_p(sol1.ctypes.data + 8 * S * SOL1.index("phi"))
        omegn = C.c_void_p(sol1.ctypes.data + 8 * S * SOL1.index("omegn"))
        for step in range(4):
            st, nu_o, sw_o, conv = o.step()
            assert st == 0
            D.vorticity_()
            D.velocity_()
            D.temperature_()
            D.poisson_(phi, omegn)
            assert D.gb_axi_last_status() == 0 and D.gb_axi_last_sweeps() == sw_o, step
            D.update_()
            trans = C.c_double()
            D.heat_(C.byref(trans))
            assert D.gb_axi_last_status() == 0
            nu = -prm["r0"] * math.log(prm["r0"] / prm["rmax"]) * trans.value / (prm["zmax"] * prm["rmax"])
            assert nu == nu_o, (step, nu, nu_o)
            for name in SOL1 + SOL2:
                np.testing.assert_array_equal(view(name)[:nr + 1, :nz + 1], np.array(o.field(name)),
                                              err_msg="%s step %d" % (name, step))
        for name in SOL1 + SOL2:
            a = view(name).copy()
            a[:nr + 1, :nz + 1] = SENTINEL
            assert np.all(a == SENTINEL), name
    finally:
        D.gb_axi_bind_common(None, None, None, None, None)
        D.gb_axi_bind_bounds(128, 128)
