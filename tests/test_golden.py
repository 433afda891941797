"""The committed fixtures of tests/golden/ generated by make_golden.py from
the oracle, reproduced exactly: by the oracle on the CPU (a regression pin)
and by the device path.  The reference's own runs (ref_*.npz) are checked
in test_reference_runs.py and test_gpu_reference_runs.py."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PRB_CASES = ["prb_layer_16x32_lex.npz", "prb_layer_16x32_zebra.npz", "prb_refinit_16x48_lex.npz"]
FIELDS = ["A", "B", "An", "Bn", "Ap", "Cn", "C", "Cp", "thn", "th", "thp", "uel", "vel", "uelp", "velp",
          "urh", "vrh"]


def load(name):
    return np.load(os.path.join(GOLD, name))


def unpack(g):
    (nr, np_, dt, Ra, Pr, r0, rmax, xx, mode, tol, kind, seed, amp, nsteps) = g["params"]
    return int(nr), int(np_), dt, Ra, Pr, r0, rmax, xx, int(mode), tol, int(kind), int(seed), amp, int(nsteps)


@pytest.mark.parametrize("case", PRB_CASES)
def test_oracle_reproduces_prb_fixture(oracle, case):
    g = load(case)
    nr, np_, dt, Ra, Pr, r0, rmax, xx, mode, tol, kind, seed, amp, nsteps = unpack(g)
    o = oracle.OraclePRB(nr, np_, dt, Ra, Pr, r0=r0, rmax=rmax, xx=xx, mode=mode, tolcon=tol)
    o.initial(kind, seed, amp)
    for f in oracle._PRB_FIELDS:
        np.testing.assert_array_equal(np.array(o.field(f)), g["init_" + f])
    for k in range(nsteps):
        st, nu, sw = o.step()
        assert st == 0
        np.testing.assert_array_equal(nu, g["nu"][k])
        np.testing.assert_array_equal(sw, g["sweeps"][k])
    for f in FIELDS:
        np.testing.assert_array_equal(np.array(o.field(f)), g[f], err_msg=f)


@pytest.mark.parametrize("case", ["batch_fp64.npz", "batch_mixed_inner3.npz"])
def test_oracle_reproduces_batch_fixture(oracle, case):
    g = load(case)
    st, psi, cyc, rr = oracle.batch_solve(list(g["sizes"]), g["f"], precision=int(g["precision"]),
                                          inner=int(g["inner"]))
    assert st == 0
    np.testing.assert_array_equal(psi, g["psi"])
    np.testing.assert_array_equal(cyc, g["cycles"])


def test_oracle_reproduces_banded_fixture(oracle):
    g = load("banded.npz")
    np.testing.assert_array_equal(oracle.tdma(g["a"], g["b"], g["c"], g["r"]), g["tdma"])
    np.testing.assert_array_equal(oracle.ptdma(g["a"], g["b"], g["c"], g["r"]), g["ptdma"])
    np.testing.assert_array_equal(oracle.pdma(g["a"], g["bp"], g["c8"], g["d"], g["e"], g["r"]), g["pdma"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", PRB_CASES)
def test_device_reproduces_prb_fixture(gblib, case):
    from codesthesis_dir_gb300 import lib, prb
    g = load(case)
    nr, np_, dt, Ra, Pr, r0, rmax, xx, mode, tol, kind, seed, amp, nsteps = unpack(g)
    d = prb.PRB(nr, np_, dt=dt, r0=r0, rmax=rmax, xx=xx, Ra=Ra, Pr=Pr, tolcon=tol, smoother=mode)
    for f in lib.FIELDS:
        d.set(f, np.asfortranarray(g["init_" + f]))
    nu, sw = d.step(nsteps)
    np.testing.assert_array_equal(nu, g["nu"])
    np.testing.assert_array_equal(sw, g["sweeps"])
    for f in FIELDS:
        np.testing.assert_array_equal(d.get(f), g[f], err_msg=f)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["batch_fp64.npz", "batch_mixed_inner3.npz"])
def test_device_reproduces_batch_fixture(gblib, case):
    from codesthesis_dir_gb300.batch import BatchPoisson
    g = load(case)
    bp = BatchPoisson(list(g["sizes"]), precision=int(g["precision"]), inner=int(g["inner"]))
    st, psi, cyc, rr = bp.solve_host(g["f"])
    assert st == 0
    np.testing.assert_array_equal(psi, g["psi"])
    np.testing.assert_array_equal(cyc, g["cycles"])
