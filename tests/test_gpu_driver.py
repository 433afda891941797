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
