"""Fortran file formats of the PRB driver: unformatted sequential records
(the restart/output files of velvor2dperiodicrbconv.f:253-312 and :500-549),
the ASCII dump of readoutput.f (format 1(1x,e16.8)) and the Nusselt history
(format 14(1x,e16.8), velvor2dperiodicrbconv.f:551-560); and those of the 3D
annulus driver: per field a header record nr,nz,np (default INTEGERs), a
header record rmax,r0,zmax,zmin and the field's own (i, j) extent over
k = 0..np (rot3dmg.f:157-216, 262-319), and the Nusselt history in format
2(1x,e16.8) (rot3dmg.f:321-326).

gfortran frames every unformatted sequential record with a 4-byte
little-endian length before and after the payload; records here are far
below the 2 GiB at which gfortran splits them into sub-records.
"""
from __future__ import annotations

import struct

import numpy as np

# Rows written per field (PRB:503-542): A, vel, wel, th use i = 0..nr+1; B, C, uel use i = 0..nr.
RESTART_ROWS = {"A": 2, "B": 1, "C": 1, "uel": 1, "vel": 2, "wel": 2, "th": 2}
RESTART_ORDER = ["A", "B", "C", "uel", "vel", "wel", "th"]


def write_record(fh, payload: bytes):
    n = len(payload)
    if n >= 2 ** 31:
        raise ValueError("record too large for a single gfortran record")
    fh.write(struct.pack("<i", n))
    fh.write(payload)
    fh.write(struct.pack("<i", n))


def read_record(fh) -> bytes:
    head = fh.read(4)
    if len(head) < 4:
        raise EOFError("end of unformatted file")
    (n,) = struct.unpack("<i", head)
    if n < 0:
        raise ValueError("sub-record files are not supported")
    data = fh.read(n)
    (tail,) = struct.unpack("<i", fh.read(4))
    if tail != n or len(data) != n:
        raise ValueError("corrupt record framing (%d vs %d)" % (n, tail))
    return data


def write_field(path, arr, nrows, np_):
    """arr: (ld, >= np+1) Fortran-ordered field; writes rows 0..nrows-1 of
    columns 0..np as one record, i fastest (the implied-do of PRB:503)."""
    a = np.asarray(arr)[:nrows, : np_ + 1]
    with open(path, "wb") as fh:
        write_record(fh, np.asfortranarray(a).ravel(order="F").astype("<f8").tobytes())


def read_field(path, nrows, np_, ld=None):
    with open(path, "rb") as fh:
        rec = read_record(fh)
    v = np.frombuffer(rec, dtype="<f8")
    if v.size != nrows * (np_ + 1):
        raise ValueError("%s holds %d values, expected %d x %d" % (path, v.size, nrows, np_ + 1))
    out = np.zeros((ld or nrows, np_ + 1), order="F")
    out[:nrows, :] = v.reshape((np_ + 1, nrows)).T
    return out


def fortran_e(x: float, w: int = 16, d: int = 8) -> str:
    """Fortran Ew.d edit descriptor (mantissa in [0.1, 1), two-digit
    exponent for |exp| < 100, three digits with no 'E' above)."""
    if x == 0.0:
        s = "0." + "0" * d + "E+00"
        return s.rjust(w)
    sign = "-" if x < 0 else ""
    m, e = ("%.*e" % (d - 1, abs(x))).split("e")
    e = int(e) + 1
    digits = m.replace(".", "")
    if len(digits) > d:
        digits = digits[:d]
    if abs(e) < 100:
        ex = "E%+03d" % e
    else:
        ex = "%+04d" % e
    s = "%s0.%s%s" % (sign, digits, ex)
    return s.rjust(w)


def write_dump(path, values):
    """readoutput.f's ASCII dump: one value per line, format (1x,e16.8)."""
    with open(path, "w") as fh:
        for v in np.ravel(values, order="F"):
            fh.write(" " + fortran_e(float(v)) + "\n")


def write_nu_history(path, dt, httrans, ssumc=None, ssums=None):
    """Nusselt history of PRB:551-560: (i-1)*dt, httrans(i), then six
    cos/sin Fourier integrals per line (zeros: the reference computes them in
    a routine that is commented out, so it writes the zero-initialised
    COMMON /grals/)."""
    n = len(httrans)
    with open(path, "w") as fh:
        for i in range(n):
            vals = [i * dt, httrans[i]] + [0.0] * 12
            fh.write("".join(" " + fortran_e(v) for v in vals) + "\n")


def write_zmtm(path, rows):
    """zmtmtempvar.dat of PRB:474-493: per row i = 0..nr+1 the zonal-mean
    time variance of T and the zonal rms of u and v, format 3(1x,e16.8)."""
    with open(path, "w") as fh:
        for r in np.asarray(rows).reshape(-1, 3):
            fh.write("".join(" " + fortran_e(float(v)) for v in r) + "\n")


def fortran_real(tok: str) -> float:
    """A value printed by an E edit descriptor, including the form without
    the letter E that a three-digit exponent takes (0.2+121)."""
    t = tok.strip()
    k = max(t.rfind("+"), t.rfind("-"))
    if k > 0 and t[k - 1] not in "eEdD":
        t = t[:k] + "E" + t[k:]
    return float(t.replace("D", "E").replace("d", "E"))


def read_zmtm(path):
    return np.array([[fortran_real(x) for x in ln.split()] for ln in open(path) if ln.strip()])


# (i, j) extents of the 3D fields in their files (rot3dmg.f:265-310): the last
# i and j index written, given nr and nz.
R3D_ORDER = ["A", "B", "C", "uel", "vel", "wel", "th"]


def r3d_extent(name, nr, nz):
    return {"A": (nr + 1, nz), "B": (nr, nz), "C": (nr, nz + 1), "uel": (nr, nz + 1), "vel": (nr + 1, nz + 1),
            "wel": (nr + 1, nz), "th": (nr + 1, nz + 1)}[name]


def write_r3d_field(path, arr, name, nr, nz, np_, rmax, r0, zmax, zmin=0.0):
    """arr: a (>= nr+2, >= nz+2, >= np+1) Fortran-ordered field."""
    im, jm = r3d_extent(name, nr, nz)
    a = np.asarray(arr)[: im + 1, : jm + 1, : np_ + 1]
    with open(path, "wb") as fh:
        write_record(fh, struct.pack("<3i", nr, nz, np_))
        write_record(fh, struct.pack("<4d", rmax, r0, zmax, zmin))
        write_record(fh, np.asfortranarray(a).ravel(order="F").astype("<f8").tobytes())


def read_r3d_field(path, name):
    """Returns ((nr, nz, np), (rmax, r0, zmax, zmin), field) with the field as
    a (nr+2, nz+2, np+1) Fortran-ordered array, zero outside its extent."""
    with open(path, "rb") as fh:
        nr, nz, np_ = struct.unpack("<3i", read_record(fh))
        geom = struct.unpack("<4d", read_record(fh))
        v = np.frombuffer(read_record(fh), dtype="<f8")
    im, jm = r3d_extent(name, nr, nz)
    if v.size != (im + 1) * (jm + 1) * (np_ + 1):
        raise ValueError("%s holds %d values, expected %d x %d x %d" % (path, v.size, im + 1, jm + 1, np_ + 1))
    out = np.zeros((nr + 2, nz + 2, np_ + 1), order="F")
    out[: im + 1, : jm + 1, :] = v.reshape((np_ + 1, jm + 1, im + 1)).T
    return (nr, nz, np_), geom, out


def write_r3d_nu_history(path, dt, httrans, httrans2=None):
    """rot3dmg.f:321-326: (i-1)*dt, httrans(i) per line, format 2(1x,e16.8);
    with httrans2, rot3dmghor.f:334-343: (i-1)*dt, httrans1(i), httrans2(i),
    format 3(1x,e16.8)."""
    with open(path, "w") as fh:
        for i, h in enumerate(httrans):
            vals = [i * dt, float(h)] + ([float(httrans2[i])] if httrans2 is not None else [])
            fh.write("".join(" " + fortran_e(v) for v in vals) + "\n")
