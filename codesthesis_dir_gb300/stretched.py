"""Host-side mirror of rcsc.f's stretched-grid streamfunction multigrid.

``STR(levels)`` owns one device instance (gb_str_create) built from the
coefficient tables of ``grid.build`` (grid.f's levels and finite-difference
weights); ``poisson(psi, rhs)`` is rcsc.f's poisson(psi, rhs, nlev, vel)
(rcsc.f:1118-1195): it returns the sweep count and the new psi, and leaves
psi as it was when the sweep limit passes (the reference returns silently
there).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lib as _L


class STR:
    def __init__(self, levels, tolcon=1e-6, maxsweeps=10000, nrel=2, smoother=_L.SMOOTHER_LEX):
        L = _L.load()
        self.n1, self.n2 = levels.n1[1], levels.n2[1]
        self.nlev = levels.nlev
        self._keep = []
        arr = (_L.StrLevel * levels.nlev)()
        for l in range(1, levels.nlev + 1):
            tabs = [np.ascontiguousarray(x, dtype=np.float64).ravel() for x in
                    (levels.r[l], levels.cr[l], levels.crr[l], levels.czz[l])]
            self._keep += tabs
            arr[l - 1] = _L.StrLevel(levels.n1[l], levels.n2[l], *(t.ctypes.data for t in tabs))
        h = C.c_void_p()
        _L.check(L.gb_str_create(levels.nlev, arr, tolcon, maxsweeps, nrel, smoother, C.byref(h)), "gb_str_create")
        self._h = h

    def poisson(self, psi, rhs):
        """psi, rhs: (n1+1, n2+1) arrays.  Returns (status, sweeps, psi)."""
        p = np.asfortranarray(psi, dtype=np.float64).copy(order="F")
        f = np.asfortranarray(rhs, dtype=np.float64)
        sw = C.c_int()
        st = _L.load().gb_str_poisson(self._h, p.ctypes.data, f.ctypes.data, p.shape[0], C.byref(sw))
        if st not in (_L.GB_OK, _L.GB_MAXSWEEPS):
            _L.check(st, "gb_str_poisson")
        return st, sw.value, p

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _L.load().gb_str_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
