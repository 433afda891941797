"""Builds the in-tree CUDA library (sm_103a) with nvcc.

Every .cu file under csrc/ is compiled in parallel to an object file and
linked into codesthesis_dir_gb300/_build/libgb300conv.so.  The 3D annulus's
gfortran drop-in symbols (csrc_dropin/r3d_fortran.cpp, host code over the
context API) go into their own libgb300r3d.so, linked against it, because
their names clash with the 2D drivers' drop-ins.  Files whose
numerics must match the reference operation for operation are compiled with
-fmad=false (no contraction of multiply-add) and place fused multiply-adds
explicitly where they want them; host code is compiled with
-ffp-contract=off for the same reason, so the results are identical on
x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgb300conv.so")
DROPIN_SRC = os.path.join(HERE, "csrc_dropin", "r3d_fortran.cpp")
R3D_LIB = os.path.join(OUT, "libgb300r3d.so")
AXI_DROPIN_SRC = os.path.join(HERE, "csrc_dropin", "axi_fortran.cpp")
AXI_LIB = os.path.join(OUT, "libgb300axi.so")
# (source, library) of the drop-in libraries whose Fortran names clash with
# the main library's: rot3dmg.f's and rotann2.f's subroutines
DROPINS = [(DROPIN_SRC, R3D_LIB), (AXI_DROPIN_SRC, AXI_LIB)]
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "-fmad=false", "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build the library")
    return p


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + ARCH + COMMON + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-6000:]))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _sources() + _headers())


def _build_one_dropin(src: str, lib: str, force: bool) -> str:
    deps = [src, LIB] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= max(os.path.getmtime(f) for f in deps):
        return lib
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("no C++ compiler found for the drop-in library")
    tmp = lib + ".tmp"
    cmd = [cxx, "-O2", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off", "-Wall", "-I", INCLUDE, src,
           "-L", OUT, "-lgb300conv", "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("drop-in build failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(tmp, lib)
    return lib


def _build_dropin(force: bool) -> None:
    for src, lib in DROPINS:
        _build_one_dropin(src, lib, force)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        _build_dropin(False)
        return LIB
    os.makedirs(OUT, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(tmp, LIB)
    _build_dropin(True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
