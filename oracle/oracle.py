"""ctypes access to the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
the CPU legs of bench.py, never by the product package.  PARITY PINNED:
the oracle restates the reference Fortran, which cannot be compiled here and
ships no outputs; its drivers run instead through the translator
tests/golden/f77.py, and the oracle reproduces those runs bit for bit
(tests/test_reference_runs.py).  The batched Poisson workload has no
reference program.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

ORC_LEX = 0
ORC_ZEBRA = 1
ORC_PRB = 0
ORC_ANNULUS = 1
ORC_OBLIQUE = 2   # mpkoks.f: the layer with gravity along the diagonal
ORC_TAYCOU = 3    # velvor2dtaycouheat.f: the annulus with a moving outer cylinder
ORC_TANK = 4      # velvor2dhorconvtank.f: the layer closed by side walls in x
ORC_DVD = 5       # velvor2ddvdbenchmark.f: the differentially heated cavity

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


class MG(C.Structure):
    _fields_ = [
        ("nr", C.c_int), ("np", C.c_int), ("ld", C.c_int), ("nlev", C.c_int),
        ("n1", C.c_int * 7), ("n3", C.c_int * 7),
        ("hr", C.c_double * 7), ("hp", C.c_double * 7),
        ("hhr", C.c_double * 7), ("hhp", C.c_double * 7),
        ("v", _dp * 7), ("f", _dp * 7),
        ("psic", _dp), ("psif", _dp), ("rc", _dp), ("rf", _dp), ("tempa", _dp),
        ("tolcon", C.c_double), ("sor", C.c_double),
        ("maxsweeps", C.c_int), ("mode", C.c_int), ("zero_scratch", C.c_int),
        ("mgen", C.c_long),
        ("scratch_v", _dp), ("scratch_f", _dp),
        ("last_sweeps", C.c_int), ("last_resmax", C.c_double),
        ("variant", C.c_int), ("r0", C.c_double), ("xwall", C.c_int),
    ]


_PRB_FIELDS = ["An", "A", "Ap", "Bn", "B", "Bp", "Cn", "C", "Cp", "thn", "th", "thp",
               "uel", "vel", "wel", "uelp", "velp", "welp", "urh", "vrh"]


class PRB(C.Structure):
    _fields_ = ([("nr", C.c_int), ("np", C.c_int), ("ld", C.c_int)] +
                [(n, C.c_double) for n in ("dt", "dr", "dp", "Ra", "Pr", "r0", "rmax", "xx")] +
                [(n, _dp) for n in _PRB_FIELDS] +
                [("clamp_count", C.c_long), ("variant", C.c_int), ("Re", C.c_double), ("Ta", C.c_double)])


_AXI_FIELDS = ["phi", "omegn", "omeg", "omegp", "veln", "vel", "velp", "thetan", "theta", "thetap"]


class AXI(C.Structure):
    _fields_ = ([("nr", C.c_int), ("nz", C.c_int), ("ld", C.c_int)] +
                [(n, C.c_double) for n in ("dt", "dr", "dz", "r0", "rmax", "zmax", "Ra", "Re", "Ptl",
                                           "cf1", "cf2", "cf3", "cf4")] +
                [(n, _dp) for n in _AXI_FIELDS] +
                [("nlev", C.c_int), ("n1", C.c_int * 8), ("n2", C.c_int * 8),
                 ("hr", C.c_double * 8), ("hz", C.c_double * 8), ("hhr", C.c_double * 8), ("hhz", C.c_double * 8),
                 ("rval", _dp), ("v", _dp * 8), ("f", _dp * 8),
                 ("psic", _dp), ("psif", _dp), ("rc", _dp), ("rf", _dp), ("tempa", _dp),
                 ("tolcon", C.c_double), ("nrel", C.c_int), ("maxsweeps", C.c_int), ("mode", C.c_int),
                 ("last_sweeps", C.c_int), ("last_resmax", C.c_double), ("sg", C.c_void_p), ("smg", C.c_void_p),
                 ("hw", C.c_double * 5)])


R3D_FIELDS = ["An", "A", "Ap", "Bn", "B", "Bp", "Cn", "C", "Cp", "thn", "th", "thp",
              "uel", "vel", "wel", "uelp", "velp", "welp", "urh", "vrh", "wrh"]
R3D_MAXLEV = 8


class R3D(C.Structure):
    _fields_ = ([(n, C.c_int) for n in ("nr", "nz", "np", "ni", "nj", "nk")] +
                [(n, C.c_double) for n in ("dt", "r0", "rmax", "zmax", "Ra", "Re", "Gr", "Ptl",
                                           "dr", "dz", "dp", "pi")] +
                [(n, _dp) for n in R3D_FIELDS] +
                [("nlev", C.c_int)] +
                [(n, C.c_int * R3D_MAXLEV) for n in ("n1", "n2", "n3")] +
                [(n, C.c_double * R3D_MAXLEV) for n in ("hr", "hz", "hp", "hhr", "hhz", "hhp")] +
                [(n, _dp * R3D_MAXLEV) for n in ("v", "f", "res")] +
                [("tolcon", C.c_double), ("sor", C.c_double), ("nrel", C.c_int), ("maxsweeps", C.c_int),
                 ("mode", C.c_int), ("last_resmax", C.c_double), ("last_sweeps", C.c_int),
                 ("horizontal", C.c_int), ("sinth", _dp), ("costh", _dp), ("nu2", C.c_double)])


STR_MAXLEV = 8


class STRGrid(C.Structure):
    _fields_ = [("nlev", C.c_int), ("n1", C.c_int * STR_MAXLEV), ("n2", C.c_int * STR_MAXLEV)] + \
               [(n, _dp * STR_MAXLEV) for n in ("hr", "hz", "r", "z", "cr", "crr", "cz", "czz")] + \
               [(n, C.c_double * 3) for n in ("cr0", "crn", "cz0", "czn")]


class STRMG(C.Structure):
    _fields_ = [("g", C.c_void_p), ("nlev", C.c_int), ("ld", C.c_int),
                ("v", _dp * STR_MAXLEV), ("f", _dp * STR_MAXLEV), ("psif", _dp), ("rc", _dp),
                ("tolcon", C.c_double), ("nrel", C.c_int), ("maxsweeps", C.c_int), ("mode", C.c_int),
                ("last_resmax", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        for nm in ("orc_tdma", "orc_ptdma"):
            getattr(L, nm).argtypes = [_dp] * 5 + [C.c_int]
        L.orc_pdma.argtypes = [_dp] * 7 + [C.c_int]
        L.orc_mg_init.argtypes = [C.POINTER(MG), C.c_int, C.c_int, C.c_double, C.c_double]
        L.orc_mg_init.restype = C.c_int
        L.orc_mg_init_variant.argtypes = [C.POINTER(MG), C.c_int, C.c_int, C.c_double, C.c_double,
                                          C.c_int, C.c_double]
        L.orc_mg_init_variant.restype = C.c_int
        L.orc_mg_free.argtypes = [C.POINTER(MG)]
        L.orc_poisson.argtypes = [C.POINTER(MG), C.c_int, _dp, _dp, _dp, C.c_int, _ip]
        L.orc_poisson.restype = C.c_int
        L.orc_relax.argtypes = [C.POINTER(MG), C.c_int, C.c_int, C.c_int, _ip]
        L.orc_corser.argtypes = [C.POINTER(MG), C.c_int]
        L.orc_finer.argtypes = [C.POINTER(MG), C.c_int]
        L.orc_prb_alloc.argtypes = [C.POINTER(PRB), C.c_int, C.c_int, C.c_int]
        L.orc_prb_alloc.restype = C.c_int
        L.orc_prb_free.argtypes = [C.POINTER(PRB)]
        for nm in ("orc_cvorticity1", "orc_cvorticity", "orc_temperature1", "orc_temperature",
                   "orc_update", "orc_rhsv", "orc_rhsu"):
            getattr(L, nm).argtypes = [C.POINTER(PRB)]
        L.orc_heat.argtypes = [C.POINTER(PRB), _dp, _dp]
        L.orc_prb_step.argtypes = [C.POINTER(PRB), C.POINTER(MG), C.POINTER(MG), C.c_int, _dp, _ip]
        L.orc_prb_step.restype = C.c_int
        L.orc_prb_initial.argtypes = [C.POINTER(PRB), C.c_int, C.c_ulonglong, C.c_double]
        L.orc_tank_initial.argtypes = [C.POINTER(PRB)]
        for nm in ("orc_tank_update", "orc_tank_rhsv", "orc_tank_rhsu"):
            getattr(L, nm).argtypes = [C.POINTER(PRB)]
        for nm in ("orc_tank_cvorticity", "orc_tank_temperature"):
            getattr(L, nm).argtypes = [C.POINTER(PRB), C.c_int]
        L.orc_tank_heat.argtypes = [C.POINTER(PRB), _dp, _dp]
        L.orc_prb_diag_accum.argtypes = [C.POINTER(PRB), C.c_int, _dp, _dp, _dp, _dp]
        L.orc_prb_cfl.argtypes = [C.POINTER(PRB), _dp, _dp]
        L.orc_prb_zmtm.argtypes = [C.POINTER(PRB), _dp, _dp, _dp, _dp, _dp]
        L.orc_axi_init.argtypes = [C.POINTER(AXI), C.c_int, C.c_int] + [C.c_double] * 7
        L.orc_axi_init.restype = C.c_int
        L.orc_axi_free.argtypes = [C.POINTER(AXI)]
        L.orc_axi_initial.argtypes = [C.POINTER(AXI), C.c_int, C.c_ulonglong, C.c_double]
        for nm in ("orc_axi_vorticity", "orc_axi_velocity", "orc_axi_temperature", "orc_axi_update"):
            getattr(L, nm).argtypes = [C.POINTER(AXI)]
        L.orc_axi_heat.argtypes = [C.POINTER(AXI)]
        L.orc_axi_heat.restype = C.c_double
        L.orc_axi_poisson.argtypes = [C.POINTER(AXI), _dp, _dp, _ip]
        L.orc_axi_poisson.restype = C.c_int
        L.orc_axi_step.argtypes = [C.POINTER(AXI), _dp, _ip, _ip]
        L.orc_axi_set_stretched.argtypes = [C.POINTER(AXI), C.POINTER(STRGrid), C.POINTER(STRMG)]
        L.orc_axi_set_stretched.restype = C.c_int
        L.orc_axi_step.restype = C.c_int
        L.orc_axi_arakawa.argtypes = [C.POINTER(AXI), _dp, _dp, _dp]
        L.orc_axi_relax.argtypes = [C.POINTER(AXI), C.c_int, C.c_int, _ip]
        L.orc_axi_corser.argtypes = [C.POINTER(AXI), C.c_int]
        L.orc_axi_finer.argtypes = [C.POINTER(AXI), C.c_int]
        L.orc_batch_solve.argtypes = [C.c_int, _ip, C.POINTER(C.c_longlong), _dp, _dp, C.c_int,
                                      C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, _ip, _dp]
        L.orc_batch_solve.restype = C.c_int
        for nm in ("orc_rb_sweep64",):
            getattr(L, nm).argtypes = [C.c_int, _dp, _dp]
        L.orc_residual64.argtypes = [C.c_int, _dp, _dp, _dp]
        L.orc_restrict64.argtypes = [C.c_int, _dp, _dp]
        L.orc_prolong_add64.argtypes = [C.c_int, _dp, _dp]
        L.orc_resnorm64.argtypes = [C.c_int, _dp, _dp]
        L.orc_resnorm64.restype = C.c_double
        L.orc_r3d_init.argtypes = [C.POINTER(R3D), C.c_int, C.c_int, C.c_int] + [C.c_double] * 8
        L.orc_r3d_init.restype = C.c_int
        L.orc_r3d_free.argtypes = [C.POINTER(R3D)]
        L.orc_r3d_initial.argtypes = [C.POINTER(R3D), C.c_int, C.c_double]
        for nm in ("avorticity", "bvorticity", "cvorticity", "temperature", "update", "rhsw", "rhsv", "rhsu"):
            getattr(L, "orc_r3d_" + nm).argtypes = [C.POINTER(R3D)]
        L.orc_r3d_heat.argtypes = [C.POINTER(R3D)]
        L.orc_r3d_heat.restype = C.c_double
        L.orc_r3d_heat2.argtypes = [C.POINTER(R3D), _dp]
        L.orc_r3d_heat2.restype = C.c_double
        L.orc_r3d_set_horizontal.argtypes = [C.POINTER(R3D)]
        L.orc_r3d_set_horizontal.restype = C.c_int
        L.orc_r3d_poisson.argtypes = [C.POINTER(R3D), C.c_int, _ip]
        L.orc_r3d_poisson.restype = C.c_int
        L.orc_r3d_relax.argtypes = [C.POINTER(R3D), C.c_int, C.c_int, C.c_int, _ip]
        L.orc_r3d_corser.argtypes = [C.POINTER(R3D), C.c_int]
        L.orc_r3d_finer.argtypes = [C.POINTER(R3D), C.c_int]
        L.orc_r3d_step.argtypes = [C.POINTER(R3D), _dp, _ip]
        L.orc_r3d_step.restype = C.c_int
        L.orc_str_spacing_gef.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, _dp]
        L.orc_str_spacing_gef.restype = C.c_int
        L.orc_str_levels.argtypes = [C.POINTER(STRGrid), C.c_int, C.c_int, _dp, _dp, C.c_double, C.c_double, C.c_int]
        L.orc_str_levels.restype = C.c_int
        L.orc_str_grid_free.argtypes = [C.POINTER(STRGrid)]
        L.orc_str_fdif.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp]
        L.orc_str_fdif.restype = C.c_int
        L.orc_str_coefficients.argtypes = [C.POINTER(STRGrid)]
        L.orc_str_coefficients.restype = C.c_int
        L.orc_str_mg_init.argtypes = [C.POINTER(STRMG), C.POINTER(STRGrid), C.c_int]
        L.orc_str_mg_init.restype = C.c_int
        L.orc_str_mg_free.argtypes = [C.POINTER(STRMG)]
        L.orc_str_poisson.argtypes = [C.POINTER(STRMG), _dp, _dp, _ip]
        L.orc_str_poisson.restype = C.c_int
        _lib = L
    return _lib


def ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32
    return a.ctypes.data_as(_ip)


# --------------------------------------------------------------------------
# banded solvers (copies made, the C routines destroy their inputs)
# --------------------------------------------------------------------------
def tdma(a, b, c, r):
    a, b, c, r = (np.array(x, dtype=np.float64) for x in (a, b, c, r))
    y = np.zeros_like(r)
    lib().orc_tdma(ptr(a), ptr(b), ptr(c), ptr(y), ptr(r), len(r))
    return y


def ptdma(a, b, c, r):
    a, b, c, r = (np.array(x, dtype=np.float64) for x in (a, b, c, r))
    y = np.zeros_like(r)
    lib().orc_ptdma(ptr(a), ptr(b), ptr(c), ptr(y), ptr(r), len(r))
    return y


def pdma(a, b, c, d, e, r):
    a, b, c, d, e, r = (np.array(x, dtype=np.float64) for x in (a, b, c, d, e, r))
    x = np.zeros_like(r)
    lib().orc_pdma(ptr(a), ptr(b), ptr(c), ptr(d), ptr(e), ptr(r), ptr(x), len(r))
    return x


# --------------------------------------------------------------------------
# PRB state
# --------------------------------------------------------------------------
class OraclePRB:
    """The PRB physical state plus the two multigrid contexts (v and u).

    variant ORC_PRB is the periodic plane layer (dp = xx/np); ORC_ANNULUS the
    rotating annulus (dp = 2 pi/np, rotational Reynolds number Re).  tolcon
    and maxsweeps default to each driver's own values."""

    def __init__(self, nr, np_, dt, Ra, Pr, r0=0.5, rmax=1.0, xx=3.0, mode=ORC_LEX,
                 tolcon=None, maxsweeps=None, sor=1.2, variant=ORC_PRB, Re=0.0, Ta=0.0):
        L = lib()
        self.s = PRB()
        assert L.orc_prb_alloc(C.byref(self.s), nr, np_, nr + 2) == 0
        s = self.s
        s.dt, s.Ra, s.Pr, s.r0, s.rmax, s.xx = dt, Ra, Pr, r0, rmax, xx
        s.variant, s.Re, s.Ta = variant, Re, Ta
        s.dr = (rmax - r0) / nr
        s.dp = 2.0 * math.acos(-1.0) / np_ if variant in (ORC_ANNULUS, ORC_TAYCOU) else xx / np_
        self.mgv, self.mgu = MG(), MG()
        for mg in (self.mgv, self.mgu):
            st = L.orc_mg_init_variant(C.byref(mg), nr, np_, s.dr, s.dp, variant, r0)
            if st != 0:
                raise ValueError("invalid multigrid size nr=%d np=%d" % (nr, np_))
            mg.mode = mode
            if tolcon is not None:
                mg.tolcon = tolcon
            if maxsweeps is not None:
                mg.maxsweeps = maxsweeps
            mg.sor = sor
        self.kt = 0
        self.diag = None
        self.cfl_hist = []

    def enable_diagnostics(self):
        """Running means (T^2, T, u^2, v^2) and per-step CFL maxima of
        PRB:404-459, updated by every later step with kt >= 2; a step with
        kt = 1 records CFL maxima (0, 0)."""
        n = self.s.ld * (self.s.np + 1)
        self.diag = [np.zeros(n) for _ in range(4)]
        self.cfl_hist = []

    def new_block(self):
        """A "more iterations" block: its steps run as kt = 2, 3, ... again."""
        self.kt = 1

    def zmtm(self) -> np.ndarray:
        """(nr+2, 3): the rows of zmtmtempvar.dat (PRB:474-493)."""
        out = np.zeros(3 * (self.s.nr + 2))
        lib().orc_prb_zmtm(C.byref(self.s), *[ptr(a) for a in self.diag], ptr(out))
        return out.reshape(-1, 3)

    def running_mean(self, q) -> np.ndarray:
        """Running mean q (0: T^2, 1: T, 2: u^2, 3: v^2) as a (ld, np+1) view."""
        return self.diag[q].reshape((self.s.np + 1, self.s.ld)).T

    @property
    def nr(self):
        return self.s.nr

    @property
    def np(self):
        return self.s.np

    @property
    def ncol(self):
        """Columns of a field: np+1, or np+2 in the tank (ghost column np+1)."""
        return self.s.np + (2 if self.s.variant in (ORC_TANK, ORC_DVD) else 1)

    def field(self, name) -> np.ndarray:
        """A (ld, ncol) Fortran-ordered view of a state field (i fastest)."""
        p = getattr(self.s, name)
        n = self.s.ld * self.ncol
        flat = np.ctypeslib.as_array(p, shape=(n,))
        return flat.reshape((self.ncol, self.s.ld)).T

    def initial(self, kind=1, seed=0, amp=1e-3):
        """kind 0: the driver's own start; 1: conduction plus seeded noise.
        The tank has only its own start (velvor2dhorconvtank.f:70-140)."""
        if self.s.variant in (ORC_TANK, ORC_DVD):
            lib().orc_tank_initial(C.byref(self.s))
        else:
            lib().orc_prb_initial(C.byref(self.s), kind, seed, amp)
        self.kt = 0

    def step(self):
        self.kt += 1
        nu = np.zeros(2)
        sw = np.zeros(2, dtype=np.int32)
        st = lib().orc_prb_step(C.byref(self.s), C.byref(self.mgv), C.byref(self.mgu), self.kt,
                                ptr(nu), iptr(sw))
        if self.diag is not None and st == 0:
            cu, cv = C.c_double(0.0), C.c_double(0.0)
            if self.kt >= 2:
                lib().orc_prb_diag_accum(C.byref(self.s), self.kt, *[ptr(a) for a in self.diag])
                lib().orc_prb_cfl(C.byref(self.s), C.byref(cu), C.byref(cv))
            self.cfl_hist.append((cu.value, cv.value))
        return st, nu, sw

    def close(self):
        if self.s.C:
            lib().orc_prb_free(C.byref(self.s))
            lib().orc_mg_free(C.byref(self.mgv))
            lib().orc_mg_free(C.byref(self.mgu))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OracleAXI:
    """The axisymmetric annulus state of rotann2.f with its multigrid."""

    def __init__(self, nr, nz, dt, r0, rmax, zmax, Ra, Re, Pr, mode=ORC_LEX, tolcon=None, maxsweeps=None):
        L = lib()
        self.s = AXI()
        if L.orc_axi_init(C.byref(self.s), nr, nz, dt, r0, rmax, zmax, Ra, Re, Pr) != 0:
            raise ValueError("invalid AXI size nr=%d nz=%d" % (nr, nz))
        self.s.mode = mode
        if tolcon is not None:
            self.s.tolcon = tolcon
        if maxsweeps is not None:
            self.s.maxsweeps = maxsweeps

    def field(self, name) -> np.ndarray:
        p = getattr(self.s, name)
        n = self.s.ld * (self.s.nz + 1)
        return np.ctypeslib.as_array(p, shape=(n,)).reshape((self.s.nz + 1, self.s.ld)).T

    def initial(self, kind=1, seed=0, amp=1e-3):
        lib().orc_axi_initial(C.byref(self.s), kind, seed, amp)

    def arakawa(self, psi, th) -> np.ndarray:
        """rotann2.f's arakawa(arak, psi, th) on (nr+1, nz+1) arrays indexed
        [i, j]; the interior points of the result are set, the rest zero."""
        ld, nz = self.s.ld, self.s.nz
        def col(a):
            b = np.zeros((nz + 1, ld))
            b[:, :a.shape[0]] = np.asarray(a, dtype=np.float64).T
            return np.ascontiguousarray(b)
        out = np.zeros((nz + 1, ld))
        pa, ta = col(psi), col(th)
        lib().orc_axi_arakawa(C.byref(self.s), out.ctypes.data_as(_dp), pa.ctypes.data_as(_dp),
                              ta.ctypes.data_as(_dp))
        return out.T[:self.s.nr + 1, :].copy()

    def stretch(self, hr1, hz1):
        """Puts the state on the non-uniform grid of level-1 spacings hr1,
        hz1 (1-based, index 0 unused; r from r0, z from 0): grid.f's levels
        and weights, rcsc.f's multigrid for the streamfunction.  Call before
        initial().  Returns the OracleSTR holding the grid."""
        st = OracleSTR(hr1, hz1, self.s.r0, 0.0, mode=self.s.mode)
        if lib().orc_axi_set_stretched(C.byref(self.s), C.byref(st.g), C.byref(st.m)) != 0:
            raise ValueError("stretched grid does not match nr x nz")
        self._str = st
        return st

    def step(self):
        nu = C.c_double()
        sw = C.c_int()
        conv = C.c_int()
        st = lib().orc_axi_step(C.byref(self.s), C.byref(nu), C.byref(sw), C.byref(conv))
        return st, nu.value, sw.value, bool(conv.value)

    def close(self):
        if self.s.phi:
            lib().orc_axi_free(C.byref(self.s))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OracleR3D:
    """The 3D rotating annulus state of rot3dmg.f with its multigrid.

    Fields are (nr+2, nz+2, np+1) Fortran-ordered views (i fastest)."""

    def __init__(self, nr, nz, np_, dt, r0, rmax, zmax, Ra, Re, Pr, Gr=0.0, mode=ORC_LEX, tolcon=None,
                 maxsweeps=None, horizontal=False):
        """horizontal: rot3dmghor.f, the annulus with its axis horizontal
        (gravity Gr Ptl across the axis, both walls' heat flux, the inner
        wall hot, plain V-cycle, tolcon 1e-6)."""
        L = lib()
        self.s = R3D()
        if L.orc_r3d_init(C.byref(self.s), nr, nz, np_, dt, r0, rmax, zmax, Ra, Re, Gr, Pr) != 0:
            L.orc_r3d_free(C.byref(self.s))
            raise ValueError("invalid R3D size nr=%d nz=%d np=%d" % (nr, nz, np_))
        if horizontal:
            assert L.orc_r3d_set_horizontal(C.byref(self.s)) == 0
        self.s.mode = mode
        if tolcon is not None:
            self.s.tolcon = tolcon
        if maxsweeps is not None:
            self.s.maxsweeps = maxsweeps

    @property
    def shape(self):
        return (self.s.ni, self.s.nj, self.s.nk)

    def field(self, name) -> np.ndarray:
        p = getattr(self.s, name)
        ni, nj, nk = self.shape
        return np.ctypeslib.as_array(p, shape=(ni * nj * nk,)).reshape((nk, nj, ni)).T

    def level(self, which, l) -> np.ndarray:
        """v, f or res of multigrid level l (1-based) as an (n1+1, n2+1, n3+1) view."""
        n1, n2, n3 = self.s.n1[l], self.s.n2[l], self.s.n3[l]
        p = getattr(self.s, which)[l]
        n = (n1 + 1) * (n2 + 1) * (n3 + 1)
        return np.ctypeslib.as_array(p, shape=(n,)).reshape((n3 + 1, n2 + 1, n1 + 1)).T

    def initial(self, nval=3, amp=1e-3):
        lib().orc_r3d_initial(C.byref(self.s), nval, amp)

    def call(self, name):
        return getattr(lib(), "orc_r3d_" + name)(C.byref(self.s))

    def poisson(self, which):
        sw = C.c_int()
        st = lib().orc_r3d_poisson(C.byref(self.s), which, C.byref(sw))
        return st, sw.value

    def step(self):
        """(status, nu, sweeps[3]); the horizontal annulus's outer-wall
        Nusselt number httrans2 is in self.nu2."""
        nu = C.c_double()
        sw = np.zeros(3, dtype=np.int32)
        st = lib().orc_r3d_step(C.byref(self.s), C.byref(nu), iptr(sw))
        return st, nu.value, sw

    @property
    def nu2(self):
        return self.s.nu2

    def close(self):
        if self.s.th:
            lib().orc_r3d_free(C.byref(self.s))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def str_spacing_gef(n, lo, hi, dist, gef, d1):
    """grid.f's wall-clustered spacings (1-based array of n+1, index 0 unused)."""
    h = np.zeros(n + 1)
    if lib().orc_str_spacing_gef(n, lo, hi, dist, gef, d1, ptr(h)) != 0:
        raise ValueError("grid.f would STOP for these GEF parameters")
    return h


def str_fdif(nx, nref, k, x):
    """Weights w[d, p] of point x[k-nref+1+p] for derivative d (grid.f fdif)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    w = np.zeros(nx * nx)
    assert lib().orc_str_fdif(nx, nref, k, ptr(x), ptr(w)) == 0
    return w.reshape(nx, nx)


class OracleSTR:
    """grid.f's levels and coefficient tables for level-1 spacings hr1, hz1
    (1-based, index 0 unused) and rcsc.f's multigrid on them."""

    def __init__(self, hr1, hz1, r0, zmin=0.0, mode=ORC_LEX, tolcon=None, maxsweeps=None, maxlev=0):
        L = lib()
        self.hr1 = np.ascontiguousarray(hr1, dtype=np.float64)
        self.hz1 = np.ascontiguousarray(hz1, dtype=np.float64)
        n1, n2 = len(self.hr1) - 1, len(self.hz1) - 1
        self.g = STRGrid()
        if L.orc_str_levels(C.byref(self.g), n1, n2, ptr(self.hr1), ptr(self.hz1), r0, zmin, maxlev) < 1:
            raise ValueError("no multigrid level for %d x %d" % (n1, n2))
        if L.orc_str_coefficients(C.byref(self.g)) != 0:
            raise ValueError("singular Taylor matrix")
        self.m = STRMG()
        assert L.orc_str_mg_init(C.byref(self.m), C.byref(self.g), 0) == 0
        self.m.mode = mode
        if tolcon is not None:
            self.m.tolcon = tolcon
        if maxsweeps is not None:
            self.m.maxsweeps = maxsweeps
        self.n1, self.n2 = n1, n2

    @property
    def nlev(self):
        return self.g.nlev

    def table(self, name, l):
        n1, n2 = self.g.n1[l], self.g.n2[l]
        size = {"r": n1 + 1, "z": n2 + 1, "hr": n1 + 1, "hz": n2 + 1, "cr": 3 * (n1 - 1), "crr": 4 * (n1 - 1),
                "cz": 3 * (n2 - 1), "czz": 4 * (n2 - 1)}[name]
        return np.ctypeslib.as_array(getattr(self.g, name)[l], shape=(size,)).copy()

    def poisson(self, psi, rhs):
        """psi, rhs: (n1+1, n2+1) arrays; returns (status, sweeps, psi)."""
        p = np.asfortranarray(psi, dtype=np.float64).copy(order="F")
        f = np.asfortranarray(rhs, dtype=np.float64)
        sw = C.c_int()
        st = lib().orc_str_poisson(C.byref(self.m), ptr(p), ptr(f), C.byref(sw))
        return st, sw.value, p

    def close(self):
        if self.m.psif:
            lib().orc_str_mg_free(C.byref(self.m))
            lib().orc_str_grid_free(C.byref(self.g))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson(which, psi, psip, rhs, nr, np_, dr, dp, mode=ORC_LEX, tolcon=None, maxsweeps=None,
            variant=ORC_PRB, r0=0.0):
    """Run one orc_poisson call on (nr+2, np+1) Fortran-ordered arrays; returns
    (status, sweeps).  psi and psip are updated in place."""
    L = lib()
    mg = MG()
    assert L.orc_mg_init_variant(C.byref(mg), nr, np_, dr, dp, variant, r0) == 0
    mg.mode = mode
    if tolcon is not None:
        mg.tolcon = tolcon
    if maxsweeps is not None:
        mg.maxsweeps = maxsweeps
    sw = C.c_int(0)
    for a in (psi, psip, rhs):
        assert a.flags["F_CONTIGUOUS"] and a.shape[0] == nr + 2
    st = L.orc_poisson(C.byref(mg), which, ptr(psi), ptr(psip), ptr(rhs), nr + 2, C.byref(sw))
    L.orc_mg_free(C.byref(mg))
    return st, sw.value


# --------------------------------------------------------------------------
# batched Poisson
# --------------------------------------------------------------------------
def batch_offsets(sizes):
    sizes = np.asarray(sizes, dtype=np.int32)
    off = np.zeros(len(sizes), dtype=np.int64)
    if len(sizes) > 1:
        off[1:] = np.cumsum(sizes.astype(np.int64) ** 2)[:-1]
    total = int(np.sum(sizes.astype(np.int64) ** 2))
    return sizes, off, total


def batch_solve(sizes, f, nu1=2, nu2=2, rtol=1e-10, max_cycles=100, precision=0, inner=1):
    sizes, off, total = batch_offsets(sizes)
    f = np.ascontiguousarray(f, dtype=np.float64)
    assert f.size == total
    psi = np.zeros(total)
    cyc = np.zeros(len(sizes), dtype=np.int32)
    rr = np.zeros(len(sizes))
    st = lib().orc_batch_solve(len(sizes), iptr(sizes), off.ctypes.data_as(C.POINTER(C.c_longlong)),
                               ptr(f), ptr(psi), nu1, nu2, rtol, max_cycles, precision, inner,
                               iptr(cyc), ptr(rr))
    return st, psi, cyc, rr
