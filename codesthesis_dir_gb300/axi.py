"""Host-side mirror of rotann2.f's subroutines (the axisymmetric rotating
annulus in the (r, z) plane).

`AXI` owns one device-resident instance (gb_axi_create) and exposes the
reference's routines under their names: vorticity (rotann2.f:268),
velocity (:324), temperature (:379), poisson(phi, omegn) (:598), update
(:497), heat (:468); `step` runs the main loop (:147-194) from a CUDA graph.
Fields move as Fortran-ordered (ld, nz+1) float64 arrays with ld >= nr+1.

Error behaviour: the reference returns from poisson silently after nvs
sweeps; `poisson` returns the sweep count and raises GBError only on a NaN
residual.  `step` stops at the reference's steady-state test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lib as _L


def stretched_grid(nr, nz, r0, rmax, zmax, factor):
    """grid.f's levels and weights for the tanh grid clustered toward all
    four walls with the given stretch factor (grid.spacing_tanh)."""
    from . import grid
    return grid.build(grid.spacing_tanh(nr, r0, rmax, factor), grid.spacing_tanh(nz, 0.0, zmax, factor), r0)


class AXI:
    def __init__(self, nr, nz, dt=1e-5, r0=0.5, rmax=1.0, zmax=0.5, Ra=1e5, Re=1e2, Pr=1.0,
                 tolcon=None, maxsweeps=None, nrel=None, smoother=_L.SMOOTHER_LEX, precision=_L.PRB_FP64,
                 grid=None):
        """grid: a grid.Levels (grid.build) for the stretched-grid mode
        (gb_axi_create_stretched); None for rotann2.f's uniform grid."""
        L = _L.load()
        p = _L.AxiParams()
        L.gb_axi_default_params(C.byref(p), nr, nz)
        p.dt, p.r0, p.rmax, p.zmax, p.Ra, p.Re, p.Pr = dt, r0, rmax, zmax, Ra, Re, Pr
        p.smoother, p.precision = smoother, precision
        if tolcon is not None:
            p.tolcon = tolcon
        if maxsweeps is not None:
            p.maxsweeps = maxsweeps
        if nrel is not None:
            p.nrel = nrel
        self.params = p
        h = C.c_void_p()
        nlev = C.c_int(0)
        if grid is None:
            _L.check(L.gb_axi_create(C.byref(p), C.byref(h), C.byref(nlev)), "gb_axi_create")
        else:
            from . import grid as G
            self._keep = []
            arr = (_L.StrLevel * grid.nlev)()
            for l in range(1, grid.nlev + 1):
                tabs = [np.ascontiguousarray(x, dtype=np.float64).ravel() for x in
                        (grid.r[l], grid.cr[l], grid.crr[l], grid.czz[l])]
                self._keep += tabs
                arr[l - 1] = _L.StrLevel(grid.n1[l], grid.n2[l], *(t.ctypes.data for t in tabs))
            z = np.ascontiguousarray(grid.z[1], dtype=np.float64)
            cz = np.ascontiguousarray(grid.cz[1], dtype=np.float64).ravel()
            hw = np.ascontiguousarray(G.fdif(5, 1, 0, grid.r[1])[1], dtype=np.float64)
            self._keep += [arr, z, cz, hw]
            g = _L.AxiGrid(grid.nlev, arr, z.ctypes.data, cz.ctypes.data, hw.ctypes.data)
            _L.check(L.gb_axi_create_stretched(C.byref(p), C.byref(g), C.byref(h), C.byref(nlev)),
                     "gb_axi_create_stretched")
        self._h = h
        self.nlev = nlev.value
        self.nr, self.nz = nr, nz
        self.ld = nr + 1

    def set(self, name, arr):
        a = np.asfortranarray(arr, dtype=np.float64)
        assert a.shape[0] >= self.nr + 1 and a.shape[1] >= self.nz + 1, a.shape
        _L.check(_L.load().gb_axi_set_field(self._h, _L.AXI_FIELD_ID[name], a.ctypes.data, a.shape[0]),
                 "set " + name)

    def get(self, name, ld=None):
        ld = ld or self.ld
        a = np.zeros((ld, self.nz + 1), order="F")
        _L.check(_L.load().gb_axi_get_field(self._h, _L.AXI_FIELD_ID[name], a.ctypes.data, ld), "get " + name)
        return a

    def vorticity(self):
        _L.check(_L.load().gb_axi_vorticity(self._h), "vorticity")

    def velocity(self):
        _L.check(_L.load().gb_axi_velocity(self._h), "velocity")

    def temperature(self):
        _L.check(_L.load().gb_axi_temperature(self._h), "temperature")

    def poisson(self):
        sw = C.c_int()
        st = _L.load().gb_axi_poisson(self._h, C.byref(sw))
        if st != _L.GB_MAXSWEEPS:
            _L.check(st, "poisson")
        return sw.value

    def update(self):
        _L.check(_L.load().gb_axi_update(self._h), "update")

    def heat(self):
        t = C.c_double()
        _L.check(_L.load().gb_axi_heat(self._h, C.byref(t)), "heat")
        return t.value

    def step(self, nsteps=1):
        """Returns (nu[steps_done], sweeps[steps_done])."""
        nu = np.zeros(nsteps)
        sw = np.zeros(nsteps, dtype=np.int32)
        done = C.c_int()
        _L.check(_L.load().gb_axi_step(self._h, nsteps, nu.ctypes.data, sw.ctypes.data, C.byref(done)), "step")
        return nu[:done.value], sw[:done.value]

    def stream(self):
        return _L.load().gb_axi_stream(self._h)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _L.load().gb_axi_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
