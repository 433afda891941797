"""Host-side mirror of rot3dmg.f's subroutines (the 3D rotating annulus).

`R3D` owns one device-resident instance (gb_r3d_create) and exposes the
reference's routines under their names: Avorticity (rot3dmg.f:341),
Bvorticity (:477), Cvorticity (:601), temperature (:736), heat (:882),
rhsw / rhsv / rhsu (:1026-1150), poisson1/2/3 (:1216-1540), update (:964);
`step` runs the main loop (:241-255).  Fields move as Fortran-ordered
(ld1, ld2, np+1) float64 arrays with ld1 >= nr+2 and ld2 >= nz+2.

variant=R3D_HORIZONTAL gives rot3dmghor.f, the annulus with its axis
horizontal (gravity Gr Ptl across the axis, both cylinders' heat flux,
the inner cylinder hot, plain V-cycles, tolcon 1e-6 by default); `heat2`
and the `nu2` of `step` are its outer-cylinder quantities.

Error behaviour: the reference STOPs when a solve passes 500 sweeps;
`poisson1/2/3` and `step` raise GBError with GB_MAXSWEEPS there (and on a
NaN residual), `step` after recording the steps completed.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lib as _L


class R3D:
    def __init__(self, nr, nz, np_, dt=1e-5, r0=0.5, rmax=1.0, zmax=0.5, Ra=1e6, Re=500.0, Pr=7.0, Gr=0.0,
                 tolcon=None, maxsweeps=None, nrel=None, sor=None, smoother=_L.SMOOTHER_LEX,
                 precision=_L.PRB_FP64, variant=_L.R3D_VERTICAL):
        L = _L.load()
        p = _L.R3dParams()
        L.gb_r3d_default_params(C.byref(p), nr, nz, np_)
        p.dt, p.r0, p.rmax, p.zmax, p.Ra, p.Re, p.Pr, p.Gr = dt, r0, rmax, zmax, Ra, Re, Pr, Gr
        p.smoother, p.precision, p.variant = smoother, precision, variant
        if variant == _L.R3D_HORIZONTAL:
            p.tolcon = 1e-6   # rot3dmghor.f:1599, :1798, :2051
        self.variant = variant
        for name, val in (("tolcon", tolcon), ("maxsweeps", maxsweeps), ("nrel", nrel), ("sor", sor)):
            if val is not None:
                setattr(p, name, val)
        self.params = p
        h = C.c_void_p()
        nlev = C.c_int(0)
        _L.check(L.gb_r3d_create(C.byref(p), C.byref(h), C.byref(nlev)), "gb_r3d_create")
        self._h = h
        self.nlev = nlev.value
        self.nr, self.nz, self.np = nr, nz, np_
        self.shape = (nr + 2, nz + 2, np_ + 1)
        self.steps_done = 0

    def set(self, name, arr):
        a = np.asfortranarray(arr, dtype=np.float64)
        assert a.shape[0] >= self.nr + 2 and a.shape[1] >= self.nz + 2 and a.shape[2] >= self.np + 1, a.shape
        _L.check(_L.load().gb_r3d_set_field(self._h, _L.R3D_FIELD_ID[name], a.ctypes.data, a.shape[0], a.shape[1]),
                 "set " + name)

    def get(self, name, ld1=None, ld2=None):
        ld1, ld2 = ld1 or self.shape[0], ld2 or self.shape[1]
        a = np.zeros((ld1, ld2, self.np + 1), order="F")
        _L.check(_L.load().gb_r3d_get_field(self._h, _L.R3D_FIELD_ID[name], a.ctypes.data, ld1, ld2), "get " + name)
        return a

    def _call(self, name):
        _L.check(getattr(_L.load(), "gb_r3d_" + name)(self._h), name)

    def avorticity(self):
        self._call("avorticity")

    def bvorticity(self):
        self._call("bvorticity")

    def cvorticity(self):
        self._call("cvorticity")

    def temperature(self):
        self._call("temperature")

    def rhsw(self):
        self._call("rhsw")

    def rhsv(self):
        self._call("rhsv")

    def rhsu(self):
        self._call("rhsu")

    def update(self):
        self._call("update")

    def heat(self):
        t = C.c_double()
        _L.check(_L.load().gb_r3d_heat(self._h, C.byref(t)), "heat")
        return t.value

    def heat2(self):
        """heat(trans1, trans2) of rot3dmghor.f:913-945."""
        t1, t2 = C.c_double(), C.c_double()
        _L.check(_L.load().gb_r3d_heat2(self._h, C.byref(t1), C.byref(t2)), "heat2")
        return t1.value, t2.value

    def poisson(self, which):
        """poisson1 (which=1, w), poisson2 (2, v), poisson3 (3, u); returns the sweep count."""
        sw = C.c_int()
        _L.check(_L.load().gb_r3d_poisson(self._h, which, C.byref(sw)), "poisson%d" % which)
        return sw.value

    def poisson1(self):
        return self.poisson(1)

    def poisson2(self):
        return self.poisson(2)

    def poisson3(self):
        return self.poisson(3)

    def step(self, nsteps=1):
        """Returns (nu[steps_done], sweeps[steps_done, 3])."""
        nu = np.zeros(nsteps)
        sw = np.zeros((nsteps, 3), dtype=np.int32)
        done = C.c_int()
        st = _L.load().gb_r3d_step(self._h, nsteps, nu.ctypes.data, sw.ctypes.data, C.byref(done))
        self.steps_done = done.value
        self.last_sweeps = sw[:min(nsteps, done.value + 1)]
        nu2 = np.zeros(nsteps)
        _L.load().gb_r3d_nu2(self._h, nsteps, nu2.ctypes.data)
        self.nu2 = nu2[:done.value]
        _L.check(st, "step")
        return nu[:done.value], sw[:done.value]

    def stream(self):
        return _L.load().gb_r3d_stream(self._h)

    def barrier_counts(self, reset=False):
        """Grid barriers passed by the w, v and u solves since creation or
        the last reset, and the block count of a solve launch."""
        c = (C.c_ulonglong * 3)()
        nb = C.c_int()
        _L.check(_L.load().gb_r3d_barrier_counts(self._h, c, C.byref(nb), 1 if reset else 0), "barrier_counts")
        return [int(x) for x in c], nb.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _L.load().gb_r3d_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
