"""The deck-driven PRB main program on the device against the oracle run
of the same deck, including the reference's block structure (later blocks
run kt = 2..nts) and the restart files it writes."""
import numpy as np
import pytest

from test_formats import DECK

pytestmark = pytest.mark.gpu


def small_deck(nts=6, more=4):
    d = DECK.replace("96\n336\n50000\n", "16\n48\n%d\n" % nts)
    d = d.replace("1.d-7\n", "1.d-5\n")
    d = d.replace("yes\n40000\nno\n", "yes\n%d\nno\n" % more)
    return d


def test_driver_matches_oracle(oracle, gblib, tmp_path):
    from codesthesis_dir_gb300 import driver, fortio
    nts, more = 6, 4
    g, ht, ht2 = driver.run(small_deck(nts, more), xx=3.0, outdir=str(tmp_path), log=lambda *a: None)
    o = oracle.OraclePRB(16, 48, 1e-5, 1e7, 0.71, r0=0.5, rmax=1.0, xx=3.0)
    o.initial(0, 0, 0.0)
    o.enable_diagnostics()
    np.testing.assert_array_equal(np.array(o.field("th")), driver.reference_initial(16, 48, 0.5, 1.0, 0.5 / 16))
    want = []
    for _ in range(nts):
        st, nu, sw = o.step()
        want.append(nu[0])
    want.append(0.0)          # httrans(ntot+1) of the second block is never set
    o.kt = 1                  # the second block starts at kt = 2 (leapfrog)
    for _ in range(more - 1):
        st, nu, sw = o.step()
        want.append(nu[0])
    np.testing.assert_array_equal(ht, np.array(want))
    for name in ("C", "th", "vel", "uel"):
        np.testing.assert_array_equal(g.get(name), np.array(o.field(name)), err_msg=name)
    # the restart files hold the final fields, framed as gfortran frames them
    th = fortio.read_field(str(tmp_path / "t.dat"), 18, 48)
    np.testing.assert_array_equal(th, np.array(o.field("th")))
    c = fortio.read_field(str(tmp_path / "c.dat"), 17, 48)
    np.testing.assert_array_equal(c, np.array(o.field("C"))[:17])
    lines = open(tmp_path / "nu.dat").read().splitlines()
    assert len(lines) == nts + more and len(lines[0].split()) == 14
    # zmtmtempvar.dat of the last block (PRB:474-493), e16.8 rounding
    z = fortio.read_zmtm(str(tmp_path / "zmtmtempvar.dat"))
    assert z.shape == (18, 3)
    np.testing.assert_allclose(z, o.zmtm(), rtol=5.1e-8, atol=1e-300)


def test_r3d_driver_matches_oracle_and_restarts(oracle, gblib, tmp_path):
    """The deck-driven 3D annulus main program (rot3dmg.f): two blocks of steps
    (3 + 2) against the oracle; the field files it writes restart a second
    run of 2 steps, which matches the oracle restarted the reference's way
    (previous time level = current, rot3dmg.f:220-230)."""
    from codesthesis_dir_gb300 import driver_r3d, fortio
    from test_formats import R3D_DECK
    g, ht = driver_r3d.run(R3D_DECK, outdir=str(tmp_path), log=lambda *a: None)
    o = oracle.OracleR3D(8, 8, 16, 1e-5, 0.5, 1.0, 0.5, 1e5, 100.0, 0.7)
    o.initial(3, 5e-2)
    want = []
    for _ in range(5):
        st, nu, sw = o.step()
        assert st == 0
        want.append(nu)
    np.testing.assert_array_equal(ht, np.array(want))
    for name in ("A", "B", "C", "th", "uel", "vel", "wel"):
        np.testing.assert_array_equal(g.get(name), np.array(o.field(name)), err_msg=name)
    lines = open(tmp_path / "nu.dat").read().splitlines()
    assert len(lines) == 5 and len(lines[0].split()) == 2
    g.close()
    # restart from the written files
    deck2 = R3D_DECK.replace("no\ny\n2\nn\n", "yes\na.dat\nb.dat\nc.dat\nu.dat\nv.dat\nw.dat\nt.dat\nn\n")
    deck2 = deck2.replace("\n3\n0.5, 1.0", "\n2\n0.5, 1.0")
    deck2 = deck2.replace("a.dat\nb.dat\nc.dat\nu.dat\nv.dat\nw.dat\nt.dat\nnu.dat\n",
                          "a2.dat\nb2.dat\nc2.dat\nu2.dat\nv2.dat\nw2.dat\nt2.dat\nno\n", 1)
    g2, ht2 = driver_r3d.run(deck2, outdir=str(tmp_path), log=lambda *a: None)
    for a, b in (("Ap", "A"), ("Bp", "B"), ("Cp", "C"), ("thp", "th"), ("uelp", "uel"), ("velp", "vel"),
                 ("welp", "wel")):
        o.field(a)[...] = np.array(o.field(b))
    want2 = []
    for _ in range(2):
        st, nu, sw = o.step()
        want2.append(nu)
    np.testing.assert_array_equal(ht2, np.array(want2))
    for name in ("A", "B", "C", "th", "uel", "vel", "wel"):
        np.testing.assert_array_equal(g2.get(name), np.array(o.field(name)), err_msg=name)
    _, _, t2 = fortio.read_r3d_field(str(tmp_path / "t2.dat"), "th")
    np.testing.assert_array_equal(t2, np.array(o.field("th")))


def test_r3d_horizontal_driver_matches_oracle(oracle, gblib, tmp_path):
    """The same deck through rot3dmghor.f's main program (--horizontal):
    httrans1 and the fields equal the oracle's, and the Nusselt history has
    rot3dmghor.f's three columns (time, inner, outer cylinder)."""
    from codesthesis_dir_gb300 import driver_r3d, fortio
    from test_formats import R3D_DECK
    deck = R3D_DECK.replace("1.d5\n100.\n0.\n0.7\n", "0.\n0.\n1.d4\n7.\n")
    g, ht = driver_r3d.run(deck, outdir=str(tmp_path), log=lambda *a: None, horizontal=True)
    o = oracle.OracleR3D(8, 8, 16, 1e-5, 0.5, 1.0, 0.5, 0.0, 0.0, 7.0, Gr=1e4, horizontal=True)
    o.initial(3, 5e-2)
    want, want2 = [], []
    for _ in range(5):
        st, nu, sw = o.step()
        assert st == 0
        want.append(nu)
        want2.append(o.nu2)
    np.testing.assert_array_equal(ht, np.array(want))
    for name in ("A", "B", "C", "th", "uel", "vel", "wel"):
        np.testing.assert_array_equal(g.get(name), np.array(o.field(name)), err_msg=name)
    rows = [[fortio.fortran_real(x) for x in ln.split()] for ln in open(tmp_path / "nu.dat").read().splitlines()]
    assert len(rows) == 5 and all(len(r) == 3 for r in rows)
    np.testing.assert_allclose([r[2] for r in rows], want2, rtol=5.1e-8)
