"""Host-side mirror of the 2D periodic Rayleigh-Benard driver's subroutines
(monashubuntudir_velvor2dperiodicrbconvdir/velvor2dperiodicrbconv.f).

`PRB` owns one device-resident instance (gb_prb_create) and exposes the
reference's routines under their reference names, with the reference's
argument meaning: cvorticity1/cvorticity (PRB:584, 786), temperature1/
temperature (PRB:1056, 1220), heat (PRB:1452), rhsv/rhsu (PRB:1629, 1679),
poisson2/poisson3 (PRB:1796, 1930), update (PRB:1557).  Fields move in and
out as Fortran-ordered (ld, np+1) float64 arrays with ld >= nr+2.

variant=PRB_ANNULUS gives the rotating-annulus (r, phi) plane driver
(iarchomedir_groke_storage_users_mpking_rotannconvvelvorplane_continueddir/
velvor2dnewsch3.4.f), whose routines have the same names; tolcon and
maxsweeps then default to its 1e-5 and 10000.  variant=PRB_OBLIQUE is
mpkoks.f (the layer with gravity along the diagonal) and variant=PRB_TAYCOU
the Taylor-Couette driver (monashubuntudir_velvor2dtaycouheatdir/
velvor2dtaycouheat.f: the annulus with its outer cylinder moving at
-(Ta**0.5) Ptl rmax / 2, Taylor number Ta); variant=PRB_TANK the
horizontal-convection tank (monashubuntudir_velvor2dhorconvtankdir/
velvor2dhorconvtank.f), whose fields carry np+2 columns, and
variant=PRB_DVD the differentially heated cavity benchmark
(monashubuntudir_velvor2ddvdbenchmarkdir/velvor2ddvdbenchmark.f), likewise.

Error behaviour: where the reference STOPs after 500 multigrid sweeps
(PRB:1843), poisson2/poisson3 raise GBError with status GB_MAXSWEEPS.  The
annulus driver does not stop (velvor2dnewsch3.4.f:1853): its solves return
the sweep limit with psi untouched and step() carries on.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lib as _L


class PRB:
    def __init__(self, nr, np_, dt=1e-7, r0=0.5, rmax=1.0, xx=3.0, Ra=1e7, Pr=0.71,
                 tolcon=None, sor=1.2, maxsweeps=None, smoother=_L.SMOOTHER_LEX,
                 variant=_L.PRB_LAYER, Re=0.0, precision=_L.PRB_FP64, Ta=0.0):
        L = _L.load()
        p = _L.PrbParams()
        if variant == _L.PRB_ANNULUS:
            L.gb_prb_default_params_annulus(C.byref(p), nr, np_)
        elif variant == _L.PRB_TAYCOU:
            L.gb_prb_default_params_taycou(C.byref(p), nr, np_)
        elif variant == _L.PRB_TANK:
            L.gb_prb_default_params_tank(C.byref(p), nr, np_)
        elif variant == _L.PRB_DVD:
            L.gb_prb_default_params_dvd(C.byref(p), nr, np_)
        else:
            L.gb_prb_default_params(C.byref(p), nr, np_)
        p.Ta = Ta
        p.dt, p.r0, p.rmax, p.xx, p.Ra, p.Pr = dt, r0, rmax, xx, Ra, Pr
        p.sor, p.smoother, p.Re, p.precision, p.variant = sor, smoother, Re, precision, variant
        if tolcon is not None:
            p.tolcon = tolcon
        if maxsweeps is not None:
            p.maxsweeps = maxsweeps
        self.variant = variant
        self.params = p
        h = C.c_void_p()
        nlev = C.c_int(0)
        _L.check(L.gb_prb_create(C.byref(p), C.byref(h), C.byref(nlev)), "gb_prb_create")
        self._h = h
        self.nlev = nlev.value
        self.nr, self.np = nr, np_
        self.ld = nr + 2
        self.ncol = np_ + 2 if variant in (_L.PRB_TANK, _L.PRB_DVD) else np_ + 1
        self.kt = 0

    # -- fields ------------------------------------------------------------
    def set(self, name, arr):
        a = np.asfortranarray(arr, dtype=np.float64)
        assert a.shape[0] >= self.nr + 2 and a.shape[1] >= self.ncol, a.shape
        _L.check(_L.load().gb_prb_set_field(self._h, _L.FIELD_ID[name], a.ctypes.data, a.shape[0]),
                 "set_field " + name)

    def get(self, name, ld=None):
        ld = ld or self.ld
        a = np.zeros((ld, self.ncol), order="F")
        _L.check(_L.load().gb_prb_get_field(self._h, _L.FIELD_ID[name], a.ctypes.data, ld), "get_field " + name)
        return a

    def device_ptr(self, name):
        p = C.c_void_p()
        ld = C.c_int()
        _L.check(_L.load().gb_prb_field_device_ptr(self._h, _L.FIELD_ID[name], C.byref(p), C.byref(ld)), "ptr")
        return p.value, ld.value

    # -- the reference routines ---------------------------------------------
    def cvorticity1(self):
        _L.check(_L.load().gb_prb_cvorticity(self._h, 1), "cvorticity1")

    def cvorticity(self):
        _L.check(_L.load().gb_prb_cvorticity(self._h, 0), "cvorticity")

    def temperature1(self):
        _L.check(_L.load().gb_prb_temperature(self._h, 1), "temperature1")

    def temperature(self):
        _L.check(_L.load().gb_prb_temperature(self._h, 0), "temperature")

    def heat(self):
        t1, t2 = C.c_double(), C.c_double()
        _L.check(_L.load().gb_prb_heat(self._h, C.byref(t1), C.byref(t2)), "heat")
        return t1.value, t2.value

    def rhsv(self):
        _L.check(_L.load().gb_prb_rhsv(self._h), "rhsv")

    def rhsu(self):
        _L.check(_L.load().gb_prb_rhsu(self._h), "rhsu")

    def _poisson(self, which):
        sw = C.c_int()
        st = _L.load().gb_prb_poisson(self._h, which, C.byref(sw))
        if not (st == _L.GB_MAXSWEEPS and self.variant == _L.PRB_ANNULUS):
            _L.check(st, "poisson%d" % which)
        return sw.value

    def poisson2(self):
        return self._poisson(2)

    def poisson3(self):
        return self._poisson(3)

    def set_solve_spread(self, ctas):
        """CTAs sharing one two-colour solve (FP64 or mixed): 1 (the
        default, one CTA per equation) or 8 (a cluster).  Both give the same
        bits."""
        _L.check(_L.load().gb_prb_set_solve_spread(self._h, ctas), "set_solve_spread")

    def update(self):
        c = C.c_longlong()
        _L.check(_L.load().gb_prb_update(self._h, C.byref(c)), "update")
        return c.value

    def step(self, nsteps=1):
        """nsteps steps of the main loop from a CUDA graph; returns
        (nu[nsteps,2], sweeps[nsteps,2])."""
        nu = np.zeros((nsteps, 2))
        sw = np.zeros((nsteps, 2), dtype=np.int32)
        st = _L.load().gb_prb_step(self._h, self.kt + 1, nsteps, nu.ctypes.data, sw.ctypes.data)
        _L.check(st, "step")
        self.kt += nsteps
        return nu, sw

    def new_block(self):
        """A "more iterations" block of the main program: its steps run as
        kt = 2, 3, ... again (PRB:357-571)."""
        self.kt = 1

    # -- time-loop diagnostics (PRB:404-493) ----------------------------------
    def diagnostics(self, on=True):
        """Running means of T^2, T, u^2, v^2 and per-step CFL maxima, updated
        on the device by every step with kt >= 2."""
        _L.check(_L.load().gb_prb_diag_enable(self._h, 1 if on else 0), "diag_enable")

    def zonal(self):
        """(nr+2, 3): the rows of zmtmtempvar.dat (T variance, u rms, v rms)."""
        out = np.zeros(3 * (self.nr + 2))
        _L.check(_L.load().gb_prb_diag_zonal(self._h, out.ctypes.data), "diag_zonal")
        return out.reshape(-1, 3)

    def running_mean(self, q):
        """Running mean q (0: T^2, 1: T, 2: u^2, 3: v^2), (ld, np+1)."""
        a = np.zeros((self.ld, self.np + 1), order="F")
        _L.check(_L.load().gb_prb_diag_mean(self._h, q, a.ctypes.data, self.ld), "diag_mean")
        return a

    def cfl(self, nsteps):
        """(nsteps, 2): the u and v CFL maxima of each step of the last run."""
        out = np.zeros((nsteps, 2))
        _L.check(_L.load().gb_prb_diag_cfl(self._h, nsteps, out.ctypes.data), "diag_cfl")
        return out

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _L.load().gb_prb_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
