"""The C-ABI library builds (nvcc cross-compiles without a GPU), loads, and
exports every entry point include/gb300_convection.h declares; the Python
binding's signature table covers the same set.  No compute call is made."""
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gb300_convection.h")


R3D_HEADER = os.path.join(ROOT, "include", "gb300_r3d_fortran.h")


def declared_functions(header=HEADER):
    src = open(header).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    src = "\n".join(l for l in src.splitlines() if not l.strip().startswith("#"))
    names = set()
    for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}]*)\)\s*;", src):
        name = m.group(1)
        if name in ("sizeof",):
            continue
        names.add(name)
    return names


def test_header_declares_the_dropin_symbols():
    names = declared_functions()
    for sym in ("poissoninit_", "poisson2_", "poisson3_", "cvorticity1_", "cvorticity_", "temperature1_",
                "temperature_", "heat_", "update_", "rhsv_", "rhsu_"):
        assert sym in names, sym


def test_library_exports_every_declared_symbol(gblib):
    from codesthesis_dir_gb300 import lib
    out = subprocess.run(["nm", "-D", "--defined-only", lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if l.strip()}
    missing = sorted(declared_functions() - exported)
    assert not missing, missing


def test_binding_table_matches_header(gblib):
    from codesthesis_dir_gb300 import lib
    bound = {n for n, _, _ in lib.SIGNATURES}
    assert declared_functions() == bound, declared_functions() ^ bound


def test_library_reports_version_without_gpu(gblib):
    v = gblib.gb_version().decode()
    assert "sm_103a" in v


def test_missing_library_fails_loudly(tmp_path):
    import importlib

    from codesthesis_dir_gb300 import lib
    mod = importlib.reload(lib)
    try:
        mod._lib = None
        try:
            mod.load(str(tmp_path / "nope.so"))
        except RuntimeError as e:
            assert "not found" in str(e)
        else:
            raise AssertionError("load() of a missing library must raise")
    finally:
        mod._lib = None
        mod.load()


def test_r3d_dropin_exports_its_header():
    """libgb300r3d.so (the rot3dmg.f drop-ins) exports every symbol its header
    declares, and the binding table covers the same set."""
    from codesthesis_dir_gb300 import _build, lib
    _build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib.R3D_DROPIN_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if l.strip()}
    declared = declared_functions(R3D_HEADER)
    assert {"avorticity_", "bvorticity_", "poisson1_", "rhsw_", "heat_", "update_"} <= declared
    assert not sorted(declared - exported), sorted(declared - exported)
    assert declared == {n for n, _, _ in lib.R3D_DROPIN_SIGNATURES}


def test_axi_dropin_exports_its_header():
    """libgb300axi.so (the rotann2.f drop-ins) exports every symbol its header
    declares, and the binding table covers the same set."""
    from codesthesis_dir_gb300 import _build, lib
    _build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib.AXI_DROPIN_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if l.strip()}
    declared = declared_functions(os.path.join(ROOT, "include", "gb300_axi_fortran.h"))
    assert {"vorticity_", "velocity_", "temperature_", "poisson_", "update_", "heat_", "poissoninit_"} <= declared
    assert not sorted(declared - exported), sorted(declared - exported)
    assert declared == {n for n, _, _ in lib.AXI_DROPIN_SIGNATURES}


def test_barrier_probe_checks_arguments_before_touching_the_device(gblib):
    """Argument errors come back without a device call (this runs without a GPU)."""
    import ctypes as C
    from codesthesis_dir_gb300 import lib
    t = C.c_double(-1.0)
    assert gblib.gb_measure_grid_barrier(0, 256, 10, C.byref(t)) == lib.GB_ERR_INVALID
    assert gblib.gb_measure_grid_barrier(8, 100, 10, C.byref(t)) == lib.GB_ERR_INVALID
    assert gblib.gb_measure_grid_barrier(8, 256, 0, C.byref(t)) == lib.GB_ERR_INVALID
    assert t.value == -1.0


def test_division_check_rejects_bad_arguments_without_a_device(gblib):
    import ctypes as C
    from codesthesis_dir_gb300 import lib
    bad = C.c_longlong(-1)
    assert gblib.gb_check_division(0, 1, C.byref(bad)) == lib.GB_ERR_INVALID
    assert bad.value == -1
