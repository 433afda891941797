"""Input decks, unformatted restart records and ASCII dumps (CPU only)."""
import io
import os

import numpy as np
import pytest

from codesthesis_dir_gb300 import deck, fortio

# The layout of the reference's PRB deck (velvor2dperiodicrbconv.f:78-120):
# eight file names, dt, nr, np, nts, "r0,rmax,zmax" on one line, Ra, Re, Gr,
# Pr, pert, amp, nval, the restart answer, then "more iterations" blocks.
DECK = """a.dat
b.dat
c.dat
u.dat
v.dat
w.dat
t.dat
nu.dat
1.d-7
96
336
50000
0.5d0,1.0d0,0.1d0
1.d7
0d0
0.d0
0.71d0
0.d0
1.d0
3
no
yes
40000
no
"""


def test_parse_prb_deck():
    d = deck.parse_prb_deck(DECK)
    assert d.fnames[0] == "a.dat" and d.fnames[7] == "nu.dat"
    assert d.dt == 1e-7 and d.nr == 96 and d.np == 336 and d.nts == 50000
    assert (d.r0, d.rmax, d.zmax) == (0.5, 1.0, 0.1)
    assert d.Ra == 1e7 and d.Pr == 0.71 and d.nval == 3
    assert d.restart is None and d.more == [40000]


def test_parse_restart_deck():
    text = DECK.replace("3\nno\nyes\n40000\nno\n", "3\nyes\n" + "".join("r%d.dat\n" % i for i in range(7)) + "no\n")
    d = deck.parse_prb_deck(text)
    assert d.restart == ["r%d.dat" % i for i in range(7)] and d.more == []


def test_list_directed_continuation():
    r = deck.ListDirected("1.5d0\n2.5d0, 3\n")
    assert [deck.fortran_float(t) for t in r.read(3)] == [1.5, 2.5, 3.0]


def test_unformatted_roundtrip(tmp_path):
    nr, np_ = 6, 8
    a = np.asfortranarray(np.random.default_rng(0).standard_normal((nr + 2, np_ + 1)))
    p = tmp_path / "x.dat"
    fortio.write_field(str(p), a, nr + 2, np_)
    raw = p.read_bytes()
    n = (nr + 2) * (np_ + 1) * 8
    assert len(raw) == n + 8
    assert int.from_bytes(raw[:4], "little") == n and int.from_bytes(raw[-4:], "little") == n
    # i fastest inside the record (the implied-do of velvor2dperiodicrbconv.f:503)
    assert np.frombuffer(raw[4:12], "<f8")[0] == a[0, 0] and np.frombuffer(raw[12:20], "<f8")[0] == a[1, 0]
    b = fortio.read_field(str(p), nr + 2, np_)
    np.testing.assert_array_equal(a, b)


def test_fortran_e_format():
    assert fortio.fortran_e(0.5) == "  0.50000000E+00"
    assert fortio.fortran_e(-1.0) == " -0.10000000E+01"
    assert fortio.fortran_e(1.23456789e-5) == "  0.12345679E-04"
    assert fortio.fortran_e(0.0) == "  0.00000000E+00"
    assert len(fortio.fortran_e(3.0e120)) == 16


@pytest.mark.parametrize("variant,kind", [(0, 0), (0, 1), (1, 0), (1, 1)],
                         ids=["layer-ref", "layer-noise", "annulus-ref", "annulus-noise"])
def test_host_initial_states_match_oracle(oracle, variant, kind):
    """The package's numpy initial states are the oracle's, bit for bit."""
    from codesthesis_dir_gb300 import initial
    nr, np_ = 24, 48
    r0, rmax = (0.5, 1.0) if variant else (0.0, 1.0)
    o = oracle.OraclePRB(nr, np_, 1e-5, 1e5, 1.0, r0=r0, rmax=rmax, xx=2.0, variant=variant, Re=1e4)
    o.initial(kind, 7, 1e-3)
    f = initial.initial_fields(nr, np_, r0, rmax, variant=variant, kind=kind, seed=7, amp=1e-3)
    for name in ("th", "thp", "C", "uel", "vel"):
        np.testing.assert_array_equal(f[name], np.array(o.field(name)), err_msg=name)


R3D_DECK = """a.dat
b.dat
c.dat
u.dat
v.dat
w.dat
t.dat
nu.dat
1.d-5
8
8
16
3
0.5, 1.0, 0.5
1.d5
100.
0.
0.7
0.
5.d-2
3
no
y
2
n
"""


def test_r3d_deck():
    d = deck.parse_r3d_deck(R3D_DECK)
    assert d.fnames == ["a.dat", "b.dat", "c.dat", "u.dat", "v.dat", "w.dat", "t.dat", "nu.dat"]
    assert (d.nr, d.nz, d.np, d.nts) == (8, 8, 16, 3)
    assert (d.r0, d.rmax, d.zmax) == (0.5, 1.0, 0.5)
    assert (d.Ra, d.Re, d.Gr, d.Pr, d.amp, d.nval) == (1e5, 100.0, 0.0, 0.7, 5e-2, 3)
    assert d.restart is None and d.more == [2] and d.total_steps == 5


def test_r3d_field_records(tmp_path):
    import struct
    nr, nz, np_ = 6, 4, 8
    rng = np.random.default_rng(2)
    for name in fortio.R3D_ORDER:
        a = np.asfortranarray(rng.standard_normal((nr + 2, nz + 2, np_ + 1)))
        p = tmp_path / (name + ".dat")
        fortio.write_r3d_field(str(p), a, name, nr, nz, np_, 1.0, 0.5, 0.5)
        raw = p.read_bytes()
        assert struct.unpack("<i", raw[:4])[0] == 12 and struct.unpack("<3i", raw[4:16]) == (nr, nz, np_)
        assert struct.unpack("<i", raw[20:24])[0] == 32
        dims, geom, b = fortio.read_r3d_field(str(p), name)
        assert dims == (nr, nz, np_) and geom == (1.0, 0.5, 0.5, 0.0)
        im, jm = fortio.r3d_extent(name, nr, nz)
        np.testing.assert_array_equal(b[:im + 1, :jm + 1], a[:im + 1, :jm + 1])
        assert np.all(b[im + 1:] == 0) and np.all(b[:, jm + 1:] == 0)


def test_r3d_nu_history(tmp_path):
    p = tmp_path / "nu.dat"
    fortio.write_r3d_nu_history(str(p), 1e-5, [1.0, 0.5])
    # (1x,e16.8) twice: one blank, then a 16-wide field with two leading blanks
    assert p.read_text().splitlines() == ["   0.00000000E+00   0.10000000E+01", "   0.10000000E-04   0.50000000E+00"]


def test_zmtm_file(tmp_path):
    """zmtmtempvar.dat (PRB:474-493, format 202 = 3(1x,e16.8)): one line of
    three e16.8 fields per row, read back to the printed precision."""
    rows = np.array([[3.62685898e-06, 12.8889259, 6.08776334], [0.0, -1.5e-17, 2.0e120]])
    p = tmp_path / "zmtmtempvar.dat"
    fortio.write_zmtm(str(p), rows)
    lines = open(p).read().splitlines()
    assert lines[0] == "   0.36268590E-05   0.12888926E+02   0.60877633E+01"
    assert lines[1] == "   0.00000000E+00  -0.15000000E-16   0.20000000+121"
    np.testing.assert_allclose(fortio.read_zmtm(str(p))[0], rows[0], rtol=5.1e-8)
