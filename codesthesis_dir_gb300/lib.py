"""ctypes binding of the CUDA library libgb300conv.so (the C ABI declared in
include/gb300_convection.h).

The library is the only compute path: there is no CPU fallback.  Loading
fails with an exception when the shared object is missing or was not built
for this machine, and every call that returns a status other than GB_OK
raises GBError carrying the library's own error text.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgb300conv.so")

GB_OK = 0
GB_MAXSWEEPS = 1
GB_NAN = 2
GB_TIMEOUT = 3
GB_ERR_ALLOC = 4
GB_ERR_INVALID = 5
GB_ERR_CUDA = 6

STATUS_NAMES = {0: "GB_OK", 1: "GB_MAXSWEEPS", 2: "GB_NAN", 3: "GB_TIMEOUT", 4: "GB_ERR_ALLOC",
                5: "GB_ERR_INVALID", 6: "GB_ERR_CUDA"}

FIELDS = ["An", "A", "Ap", "Bn", "B", "Bp", "Cn", "C", "Cp", "thn", "th", "thp",
          "uel", "vel", "wel", "uelp", "velp", "welp", "urh", "vrh"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}

SMOOTHER_LEX = 0
SMOOTHER_ZEBRA = 1
PRB_LAYER = 0
PRB_ANNULUS = 1
PRB_OBLIQUE = 2   # mpkoks.f: the layer with gravity along the diagonal
PRB_TAYCOU = 3    # velvor2dtaycouheat.f: the annulus with a moving outer cylinder
PRB_TANK = 4      # velvor2dhorconvtank.f: the layer closed by side walls (fields have np+2 columns)
PRB_DVD = 5       # velvor2ddvdbenchmark.f: the differentially heated cavity (np+2 columns)
PRB_FP64 = 0
PRB_MIXED = 1
BATCH_FP64 = 0
BATCH_MIXED = 1            # float-pair outer residual
BATCH_MIXED_F64OUTER = 2   # FP64 outer residual, norm and update
BATCH_EXEC_GRAPH = 0
BATCH_EXEC_PERSISTENT = 1


class GBError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__("%s: %s (%s)" % (what, STATUS_NAMES.get(status, status), last_error()))
        self.status = status


AXI_FIELDS = ["phi", "omegn", "omeg", "omegp", "veln", "vel", "velp", "thetan", "theta", "thetap"]
AXI_FIELD_ID = {n: i for i, n in enumerate(AXI_FIELDS)}


class BatchTuning(C.Structure):
    """gb_batch_tuning: the tunables of a batched solve and, from the
    autotuner, the measured milliseconds per solve."""
    _fields_ = [("nu1", C.c_int), ("nu2", C.c_int), ("inner", C.c_int), ("local_n", C.c_int), ("fuse", C.c_int),
                ("exec", C.c_int), ("ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AxiParams(C.Structure):
    _fields_ = [("nr", C.c_int), ("nz", C.c_int),
                ("dt", C.c_double), ("r0", C.c_double), ("rmax", C.c_double), ("zmax", C.c_double),
                ("Ra", C.c_double), ("Re", C.c_double), ("Pr", C.c_double), ("tolcon", C.c_double),
                ("maxsweeps", C.c_int), ("nrel", C.c_int), ("smoother", C.c_int), ("precision", C.c_int)]


R3D_FIELDS = ["An", "A", "Ap", "Bn", "B", "Bp", "Cn", "C", "Cp", "thn", "th", "thp",
              "uel", "vel", "wel", "uelp", "velp", "welp", "urh", "vrh", "wrh"]
R3D_FIELD_ID = {n: i for i, n in enumerate(R3D_FIELDS)}


class R3dParams(C.Structure):
    _fields_ = [("nr", C.c_int), ("nz", C.c_int), ("np", C.c_int),
                ("dt", C.c_double), ("r0", C.c_double), ("rmax", C.c_double), ("zmax", C.c_double),
                ("Ra", C.c_double), ("Re", C.c_double), ("Gr", C.c_double), ("Pr", C.c_double),
                ("tolcon", C.c_double), ("sor", C.c_double), ("maxsweeps", C.c_int), ("nrel", C.c_int),
                ("smoother", C.c_int), ("precision", C.c_int), ("variant", C.c_int)]


R3D_VERTICAL = 0
R3D_HORIZONTAL = 1   # rot3dmghor.f


class StrLevel(C.Structure):
    _fields_ = [("n1", C.c_int), ("n2", C.c_int), ("r", C.c_void_p), ("cr", C.c_void_p), ("crr", C.c_void_p),
                ("czz", C.c_void_p)]


class AxiGrid(C.Structure):
    """gb_axi_grid: the stretched grid of gb_axi_create_stretched."""
    _fields_ = [("nlev", C.c_int), ("levels", C.POINTER(StrLevel)), ("z", C.c_void_p), ("cz", C.c_void_p),
                ("hw", C.c_void_p)]


class PrbParams(C.Structure):
    _fields_ = [("nr", C.c_int), ("np", C.c_int),
                ("dt", C.c_double), ("r0", C.c_double), ("rmax", C.c_double), ("xx", C.c_double),
                ("Ra", C.c_double), ("Pr", C.c_double), ("tolcon", C.c_double), ("sor", C.c_double),
                ("maxsweeps", C.c_int), ("smoother", C.c_int), ("variant", C.c_int), ("Re", C.c_double),
                ("precision", C.c_int), ("Ta", C.c_double)]


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p
_lib = None

# (name, restype, argtypes) of every exported entry point of the C ABI.
SIGNATURES = [
    ("gb_last_error", C.c_char_p, []),
    ("gb_version", C.c_char_p, []),
    ("gb_prb_default_params", None, [C.POINTER(PrbParams), C.c_int, C.c_int]),
    ("gb_prb_default_params_annulus", None, [C.POINTER(PrbParams), C.c_int, C.c_int]),
    ("gb_prb_default_params_taycou", None, [C.POINTER(PrbParams), C.c_int, C.c_int]),
    ("gb_prb_default_params_tank", None, [C.POINTER(PrbParams), C.c_int, C.c_int]),
    ("gb_prb_default_params_dvd", None, [C.POINTER(PrbParams), C.c_int, C.c_int]),
    ("gb_prb_create", C.c_int, [C.POINTER(PrbParams), C.POINTER(_vp), _ip]),
    ("gb_prb_destroy", C.c_int, [_vp]),
    ("gb_prb_set_field", C.c_int, [_vp, C.c_int, _vp, C.c_int]),
    ("gb_prb_get_field", C.c_int, [_vp, C.c_int, _vp, C.c_int]),
    ("gb_prb_field_device_ptr", C.c_int, [_vp, C.c_int, C.POINTER(_vp), _ip]),
    ("gb_prb_cvorticity", C.c_int, [_vp, C.c_int]),
    ("gb_prb_temperature", C.c_int, [_vp, C.c_int]),
    ("gb_prb_heat", C.c_int, [_vp, _dp, _dp]),
    ("gb_prb_rhsv", C.c_int, [_vp]),
    ("gb_prb_rhsu", C.c_int, [_vp]),
    ("gb_prb_poisson", C.c_int, [_vp, C.c_int, _ip]),
    ("gb_prb_update", C.c_int, [_vp, C.POINTER(C.c_longlong)]),
    ("gb_prb_step", C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp]),
    ("gb_prb_stream", _vp, [_vp]),
    ("gb_prb_run_begin", C.c_int, [_vp, C.c_int]),
    ("gb_prb_run_enqueue", C.c_int, [_vp, C.c_int, C.c_int]),
    ("gb_prb_run_query", C.c_int, [_vp]),
    ("gb_prb_run_end", C.c_int, [_vp, C.c_int, _vp, _vp, _ip]),
    ("gb_prb_diag_enable", C.c_int, [_vp, C.c_int]),
    ("gb_prb_diag_zonal", C.c_int, [_vp, _vp]),
    ("gb_prb_diag_mean", C.c_int, [_vp, C.c_int, _vp, C.c_int]),
    ("gb_prb_diag_cfl", C.c_int, [_vp, C.c_int, _vp]),
    ("gb_axi_default_params", None, [C.POINTER(AxiParams), C.c_int, C.c_int]),
    ("gb_axi_create", C.c_int, [C.POINTER(AxiParams), C.POINTER(_vp), _ip]),
    ("gb_axi_create_spacing", C.c_int, [C.POINTER(AxiParams), C.c_double, C.c_double, C.POINTER(_vp), _ip]),
    ("gb_axi_create_stretched", C.c_int, [C.POINTER(AxiParams), C.POINTER(AxiGrid), C.POINTER(_vp), _ip]),
    ("gb_axi_destroy", C.c_int, [_vp]),
    ("gb_axi_set_field", C.c_int, [_vp, C.c_int, _vp, C.c_int]),
    ("gb_axi_get_field", C.c_int, [_vp, C.c_int, _vp, C.c_int]),
    ("gb_axi_vorticity", C.c_int, [_vp]),
    ("gb_axi_velocity", C.c_int, [_vp]),
    ("gb_axi_temperature", C.c_int, [_vp]),
    ("gb_axi_poisson", C.c_int, [_vp, _ip]),
    ("gb_axi_update", C.c_int, [_vp]),
    ("gb_axi_heat", C.c_int, [_vp, _dp]),
    ("gb_axi_step", C.c_int, [_vp, C.c_int, _vp, _vp, _ip]),
    ("gb_axi_stream", _vp, [_vp]),
    ("gb_axi_run_begin", C.c_int, [_vp, C.c_int]),
    ("gb_axi_run_enqueue", C.c_int, [_vp, C.c_int]),
    ("gb_axi_run_query", C.c_int, [_vp]),
    ("gb_axi_run_end", C.c_int, [_vp, C.c_int, _vp, _vp, _ip]),
    ("gb_r3d_default_params", None, [C.POINTER(R3dParams), C.c_int, C.c_int, C.c_int]),
    ("gb_r3d_create", C.c_int, [C.POINTER(R3dParams), C.POINTER(_vp), _ip]),
    ("gb_r3d_create_spacing", C.c_int, [C.POINTER(R3dParams), C.c_double, C.c_double, C.c_double,
                                        C.POINTER(_vp), _ip]),
    ("gb_r3d_destroy", C.c_int, [_vp]),
    ("gb_r3d_set_field", C.c_int, [_vp, C.c_int, _vp, C.c_int, C.c_int]),
    ("gb_r3d_get_field", C.c_int, [_vp, C.c_int, _vp, C.c_int, C.c_int]),
    ("gb_r3d_avorticity", C.c_int, [_vp]),
    ("gb_r3d_bvorticity", C.c_int, [_vp]),
    ("gb_r3d_cvorticity", C.c_int, [_vp]),
    ("gb_r3d_temperature", C.c_int, [_vp]),
    ("gb_r3d_heat", C.c_int, [_vp, _dp]),
    ("gb_r3d_heat2", C.c_int, [_vp, _dp, _dp]),
    ("gb_r3d_nu2", C.c_int, [_vp, C.c_int, _vp]),
    ("gb_r3d_rhsw", C.c_int, [_vp]),
    ("gb_r3d_rhsv", C.c_int, [_vp]),
    ("gb_r3d_rhsu", C.c_int, [_vp]),
    ("gb_r3d_poisson", C.c_int, [_vp, C.c_int, _ip]),
    ("gb_r3d_update", C.c_int, [_vp]),
    ("gb_r3d_step", C.c_int, [_vp, C.c_int, _vp, _vp, _ip]),
    ("gb_r3d_stream", _vp, [_vp]),
    ("gb_r3d_set_wait_limit", C.c_int, [_vp, C.c_longlong]),
    ("gb_r3d_barrier_counts", C.c_int, [_vp, C.POINTER(C.c_ulonglong), C.POINTER(C.c_int), C.c_int]),
    ("gb_prb_bind_bounds", None, [C.c_int, C.c_int]),
    ("gb_prb_bind_smoother", None, [C.c_int]),
    ("gb_prb_bind_tolerance", None, [C.c_double, C.c_int]),
    ("gb_prb_bind_common", None, [_vp, _vp, _vp, _vp, _vp]),
    ("gb_prb_bind_variant", None, [C.c_int]),
    ("gb_prb_bind_radius", None, [_vp]),
    ("gb_prb_last_status", C.c_int, []),
    ("gb_prb_last_sweeps", C.c_int, []),
    ("poissoninit_", None, [_ip, _ip, _ip, _dp, _dp, _dp, _ip]),
    ("poisson2_", None, [_vp, _vp, _vp, _ip, _ip, _ip, _dp, _dp, _dp, _ip]),
    ("poisson3_", None, [_vp, _vp, _vp, _ip, _ip, _ip, _dp, _dp, _dp, _ip]),
    ("cvorticity1_", None, []),
    ("cvorticity_", None, []),
    ("temperature1_", None, []),
    ("temperature_", None, []),
    ("heat_", None, [_dp, _dp]),
    ("update_", None, []),
    ("rhsv_", None, [_vp]),
    ("rhsu_", None, [_vp]),
    ("gb_str_create", C.c_int, [C.c_int, C.POINTER(StrLevel), C.c_double, C.c_int, C.c_int, C.c_int,
                                C.POINTER(_vp)]),
    ("gb_str_poisson", C.c_int, [_vp, _vp, _vp, C.c_int, _ip]),
    ("gb_str_destroy", C.c_int, [_vp]),
    ("gb_tdma_batch", C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_longlong, C.c_longlong, _vp]),
    ("gb_ptdma_batch", C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_longlong, C.c_longlong, _vp]),
    ("gb_pdma_batch", C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_longlong, C.c_longlong, _vp]),
    ("gb_pdma_batch_noalloc", C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_longlong,
                                       C.c_longlong, _vp]),
    ("gb_prb_set_solve_spread", C.c_int, [_vp, C.c_int]),
    ("gb_prb_gang_create", C.c_int, [C.POINTER(_vp), _ip, C.c_int, C.POINTER(_vp)]),
    ("gb_prb_gang_enqueue", C.c_int, [_vp, C.c_int, _vp]),
    ("gb_prb_gang_query", C.c_int, [_vp]),
    ("gb_prb_gang_stream", _vp, [_vp]),
    ("gb_prb_gang_launches_per_step", C.c_longlong, [_vp]),
    ("gb_prb_gang_set_solve_spread", C.c_int, [_vp, C.c_int]),
    ("gb_prb_gang_destroy", C.c_int, [_vp]),
    ("gb_axi_gang_create", C.c_int, [C.POINTER(_vp), _ip, C.c_int, C.POINTER(_vp)]),
    ("gb_axi_gang_enqueue", C.c_int, [_vp, C.c_int, _vp]),
    ("gb_axi_gang_query", C.c_int, [_vp]),
    ("gb_axi_gang_stream", _vp, [_vp]),
    ("gb_axi_gang_destroy", C.c_int, [_vp]),
    ("gb_batch_create", C.c_int, [C.c_int, _ip, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.POINTER(_vp)]),
    ("gb_batch_create_tuned", C.c_int, [C.c_int, _ip, C.c_int, C.c_double, C.c_int, C.POINTER(BatchTuning),
                                        C.POINTER(_vp)]),
    ("gb_batch_autotune", C.c_int, [C.c_int, _ip, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, _vp, _vp,
                                    C.c_int, C.c_char_p, C.POINTER(BatchTuning), C.POINTER(BatchTuning), C.c_int,
                                    C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("gb_batch_destroy", C.c_int, [_vp]),
    ("gb_batch_total_points", C.c_longlong, [_vp]),
    ("gb_batch_set_inner_cycles", C.c_int, [_vp, C.c_int]),
    ("gb_batch_set_exec", C.c_int, [_vp, C.c_int]),
    ("gb_batch_set_wait_limit", C.c_int, [_vp, C.c_longlong]),
    ("gb_batch_solve_device", C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    ("gb_batch_solve_host", C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    ("gb_batch_submit_host", C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    ("gb_batch_drain", C.c_int, [_vp]),
    ("gb_batch_last_launches", C.c_longlong, [_vp]),
    ("gb_batch_profile", C.c_int, [_vp, C.c_int]),
    ("gb_batch_profile_read", C.c_int, [_vp, _dp, C.POINTER(C.c_longlong), _dp, C.c_int]),
    ("gb_batch_profile_read_kind", C.c_int, [_vp, C.c_int, _dp, C.POINTER(C.c_longlong), _dp]),
    ("gb_measure_issue_rates", C.c_int, [_dp, _dp]),
    ("gb_measure_grid_barrier", C.c_int, [C.c_int, C.c_int, C.c_int, _dp]),
    ("gb_check_division", C.c_int, [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)]),
    ("gb_check_conversions", C.c_int, [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
]


R3D_DROPIN_PATH = os.path.join(HERE, "_build", "libgb300r3d.so")
# (name, restype, argtypes) of libgb300r3d.so (include/gb300_r3d_fortran.h).
R3D_DROPIN_SIGNATURES = [
    ("poissoninit_", None, [_ip, _ip, _ip, _dp, _dp, _dp, _ip]),
    ("poisson1_", None, [_vp, _vp, _vp, _ip, _ip, _ip, _dp, _dp, _dp, _ip]),
    ("poisson2_", None, [_vp, _vp, _vp, _ip, _ip, _ip, _dp, _dp, _dp, _ip]),
    ("poisson3_", None, [_vp, _vp, _vp, _ip, _ip, _ip, _dp, _dp, _dp, _ip]),
    ("avorticity_", None, []),
    ("bvorticity_", None, []),
    ("cvorticity_", None, []),
    ("temperature_", None, []),
    ("heat_", None, [_dp, _dp]),
    ("update_", None, []),
    ("rhsw_", None, [_vp]),
    ("rhsv_", None, [_vp]),
    ("rhsu_", None, [_vp]),
    ("gb_r3d_bind_bounds", None, [C.c_int, C.c_int, C.c_int]),
    ("gb_r3d_bind_common", None, [_vp, _vp, _vp, _vp, _vp, _vp]),
    ("gb_r3d_bind_smoother", None, [C.c_int]),
    ("gb_r3d_bind_precision", None, [C.c_int]),
    ("gb_r3d_bind_variant", None, [C.c_int]),
    ("gb_r3d_bind_tolerance", None, [C.c_double, C.c_int]),
    ("gb_r3d_last_status", C.c_int, []),
    ("gb_r3d_last_sweeps", C.c_int, []),
]
_r3d_dropin = None

AXI_DROPIN_PATH = os.path.join(HERE, "_build", "libgb300axi.so")
# (name, restype, argtypes) of libgb300axi.so (include/gb300_axi_fortran.h).
AXI_DROPIN_SIGNATURES = [
    ("poissoninit_", None, [_ip, _ip, _dp, _dp]),
    ("vorticity_", None, []),
    ("velocity_", None, []),
    ("temperature_", None, []),
    ("poisson_", None, [_vp, _vp]),
    ("update_", None, []),
    ("heat_", None, [_dp]),
    ("gb_axi_bind_bounds", None, [C.c_int, C.c_int]),
    ("gb_axi_bind_common", None, [_vp, _vp, _vp, _vp, _vp]),
    ("gb_axi_bind_smoother", None, [C.c_int]),
    ("gb_axi_bind_precision", None, [C.c_int]),
    ("gb_axi_bind_tolerance", None, [C.c_double, C.c_int]),
    ("gb_axi_last_status", C.c_int, []),
    ("gb_axi_last_sweeps", C.c_int, []),
]
_axi_dropin = None


def load_axi_dropin(path: str = AXI_DROPIN_PATH):
    """Loads the rotann2.f drop-in library (its own handle: its symbols share
    names with the other drop-ins)."""
    global _axi_dropin
    if _axi_dropin is not None:
        return _axi_dropin
    load()
    if not os.path.exists(path):
        raise RuntimeError("libgb300axi.so not found at %s; run __graft_entry__.build() first" % path)
    L = C.CDLL(path, mode=C.RTLD_LOCAL)
    for name, res, args in AXI_DROPIN_SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _axi_dropin = L
    return L


def load_r3d_dropin(path: str = R3D_DROPIN_PATH):
    """Loads the rot3dmg.f drop-in library (its own handle: its symbols share
    names with the 2D drop-ins of the main library)."""
    global _r3d_dropin
    if _r3d_dropin is not None:
        return _r3d_dropin
    load()
    if not os.path.exists(path):
        raise RuntimeError("libgb300r3d.so not found at %s; run __graft_entry__.build() first" % path)
    L = C.CDLL(path, mode=C.RTLD_LOCAL)
    for name, res, args in R3D_DROPIN_SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _r3d_dropin = L
    return L


def load(path: str = LIB_PATH):
    """Loads the library (once).  Raises if it is missing: there is no
    fallback implementation."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libgb300conv.so not found at %s; run __graft_entry__.build() "
                           "(nvcc, sm_103a) first" % path)
    L = C.CDLL(path, mode=C.RTLD_GLOBAL)
    for name, res, args in SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    if _lib is None:
        return ""
    s = _lib.gb_last_error()
    return s.decode() if s else ""


def check(status: int, what: str):
    if status != GB_OK:
        raise GBError(status, what)
    return status
