"""The oracle against the reference's own Fortran source.

The fixtures tests/golden/ref_*.npz hold runs of the reference's drivers —
their main programs fed small input decks, from their own initial states —
executed on the CPU by tests/golden/f77.py (a translator of the reference's
fixed-form Fortran 77 with IEEE binary64 / binary32 arithmetic in source
order), written by tests/golden/make_reference_golden.py.  The oracle run
on the same parameters must reproduce every field, every Nusselt number and
every multigrid sweep count bit for bit: the 2D layer, its oblique-gravity,
rotating-annulus, tank and cavity variants (also on the decks the reference
ships), the 3D annulus (vertical and horizontal), the axisymmetric annulus,
grid.f's stretched tables with rcsc.f's multigrid on them, and the batched
solve's grid transfers (rotann2.f's corser and finer).  The device path is
tied to the oracle bit for bit by the parity tests, so these fixtures pin it
too; test_gpu_reference_runs.py replays the 2D runs on the device directly.

The Taylor-Couette driver (velvor2dtaycouheat.f) is the one the oracle does
not follow to the letter: its relax2 forms a line's pentadiagonal right-hand
side only for k = 1 (the block of :2132-2164 sits inside `if(k.eq.1)then`),
so every later line solves with the right-hand side the previous line's
elimination left in pdmar; run as written, its first velocity solve reaches
the sweep limit and STOPs.  The oracle forms every line's right-hand side,
as velvor2dtaycouheat_new.f does (:2181-2182, after the block): it
reproduces velvor2dtaycouheat.f run with that one subroutine taken from
velvor2dtaycouheat_new.f (ref_taycou_relax2new_*.npz), and the last test
records that the program as written stops."""
import hashlib
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(f for f in os.listdir(GOLD) if f.startswith("ref_") and f.endswith(".npz")
               and f not in ("ref_taycou_16x32.npz", "ref_grid_rcsc_64x64.npz", "ref_transfer_rotann2_33.npz"))
F2D = ["A", "B", "An", "Bn", "Ap", "Cn", "C", "Cp", "thn", "th", "thp", "uel", "vel", "uelp", "velp"]


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def check_fields(g, field, view=lambda a: a):
    """Every field the fixture holds, as an array (f_*) or as a SHA-256
    digest of its binary64 values (h_*, the large runs)."""
    n = 0
    for key in g.files:
        if key.startswith("f_"):
            np.testing.assert_array_equal(view(np.array(field(key[2:]))), g[key], err_msg=key)
            n += 1
        elif key.startswith("h_"):
            assert digest(view(np.array(field(key[2:])))) == str(g[key]), key
            n += 1
    assert n > 0


def load(name):
    g = np.load(os.path.join(GOLD, name))
    return g, json.loads(str(g["meta"]))


def run_2d(O, m, init_kind=0, init_seed=0, init_amp=0.0):
    o = O.OraclePRB(m["nr"], m["np"], m["dt"], m["Ra"], m["Pr"], r0=m["r0"], rmax=m["rmax"], xx=m["xx"] or 3.0,
                    variant=m["variant"], Re=m["Re"], Ta=m["Gr"])
    o.initial(init_kind, init_seed, init_amp)
    nus, sws = [], []
    for _ in range(m["steps"]):
        st, nu, sw = o.step()
        assert st == 0
        nus.append(nu.copy())
        sws.append(sw.copy())
    return o, np.array(nus), np.array(sws)


@pytest.mark.parametrize("case", CASES)
def test_oracle_reproduces_reference_run(oracle, case):
    g, m = load(case)
    assert m["end"] in ("_main", "return")     # the run ended at its own end
    drv = m["driver"]
    if drv in ("layer", "oblique", "annulus", "tank", "dvd", "taycou", "layer_routines"):
        if drv == "layer_routines":
            o, nu, sw = run_2d(oracle, m, 1, m["init"]["seed"], m["init"]["amp"])
        else:
            o, nu, sw = run_2d(oracle, m)
        check_fields(g, o.field)
    elif drv in ("r3d", "r3d_hor"):
        o = oracle.OracleR3D(m["nr"], m["nz"], m["np"], m["dt"], m["r0"], m["rmax"], m["zmax"], m["Ra"], m["Re"],
                             m["Pr"], Gr=m["Gr"], horizontal=drv == "r3d_hor")
        o.initial(m["nval"], m["amp"])
        nus, sws = [], []
        for _ in range(m["steps"]):
            st, n1, s = o.step()
            assert st == 0
            nus.append([n1, o.nu2] if drv == "r3d_hor" else [n1])
            sws.append(s.copy())
        nu, sw = np.array(nus), np.array(sws)
        check_fields(g, o.field)
    else:
        assert drv == "axi"
        o = oracle.OracleAXI(m["nr"], m["nz"], m["dt"], m["r0"], m["rmax"], m["zmax"], m["Ra"], m["Re"], m["Pr"])
        o.initial(0)
        nus, sws = [], []
        for _ in range(m["steps"]):
            st, n1, s, conv = o.step()
            assert st == 0
            nus.append(n1)
            sws.append(s)
            if conv:
                break
        nu, sw = np.array(nus), np.array(sws)
        check_fields(g, o.field, lambda a: a[:m["nr"] + 1, :m["nz"] + 1])
    np.testing.assert_array_equal(nu, g["nu"])
    np.testing.assert_array_equal(sw, g["sweeps"])


def test_axisymmetric_run_reaches_the_steady_state_stop():
    g, m = load("ref_axi_8x8.npz")
    assert len(g["nu"]) < m["steps"]       # rotann2.f's convergence exit (:191-194) ended the loop


def test_reference_runs_cover_the_drivers():
    drivers = {load(c)[1]["driver"] for c in CASES}
    assert drivers >= {"layer", "oblique", "annulus", "tank", "dvd", "taycou", "layer_routines", "r3d", "r3d_hor",
                       "axi"}
    for c in CASES:
        m = load(c)[1]
        assert len(m["sha256"]) == 64 and m["source"].endswith(".f")


def test_device_golden_start_is_the_reference_programs_start():
    """The layer fixture the device golden test replays (the program's own
    start, 16 x 48, 4 steps) equals the reference program's run."""
    ref, _ = load("ref_layer_16x48.npz")
    dev = np.load(os.path.join(GOLD, "prb_refinit_16x48_lex.npz"))
    for f in F2D:
        np.testing.assert_array_equal(dev[f], ref["f_" + f], err_msg=f)
    np.testing.assert_array_equal(dev["nu"], ref["nu"])
    np.testing.assert_array_equal(dev["sweeps"], ref["sweeps"])


def test_taylor_couette_reference_stops_where_the_oracle_converges(oracle):
    g, m = load("ref_taycou_16x32.npz")
    # the reference: the first v solve runs past its 500-sweep limit and STOPs
    assert m["end"] == "poisson2"
    assert g["sweeps"][0, 0] == 501
    # the oracle, forming every line's right-hand side, converges every solve
    o, nu, sw = run_2d(oracle, m)
    assert np.all(sw > 0) and np.all(sw < 100)
    assert np.all(np.isfinite(nu))


def test_oracle_reproduces_grid_tables_and_stretched_multigrid(oracle):
    """grid.f's own main program (spacings with geometric expansion toward
    both walls, levels, finite-difference weights of every level, wall
    weights) and rcsc.f's multigrid on those tables: the oracle's grid and
    its stretched solve equal them bit for bit."""
    g, m = load("ref_grid_rcsc_64x64.npz")
    hr1 = oracle.str_spacing_gef(m["nr"], m["r0"], m["rmax"], m["rdist"], m["rgef"], m["dr1"])
    hz1 = oracle.str_spacing_gef(m["nz"], m["zmin"], m["zmax"], m["zdist"], m["zgef"], m["dz1"])
    o = oracle.OracleSTR(hr1, hz1, m["r0"], m["zmin"])
    assert o.nlev == m["nlev"]
    np.testing.assert_array_equal(hr1[1:], g["t_hr_1"])
    np.testing.assert_array_equal(hz1[1:], g["t_hz_1"])
    for L in range(1, o.nlev + 1):
        for name in ("r", "z", "cr", "crr", "cz", "czz"):
            np.testing.assert_array_equal(o.table(name, L), g["t_%s_%d" % (name, L)], err_msg="%s %d" % (name, L))
    np.testing.assert_array_equal(np.array(o.g.crn), g["t_crn"])
    np.testing.assert_array_equal(np.array(o.g.czn), g["t_czn"])
    st, sw, psi = o.poisson(np.zeros_like(g["rhs"]), g["rhs"])
    assert st == 0
    assert [sw] == list(g["sweeps"])
    np.testing.assert_array_equal(psi, g["psi"])


def test_batched_grid_transfers_are_rotann2s(oracle):
    """The batched solve has no reference program; its grid transfers are
    rotann2.f's: full weighting in corser's order and bilinear prolongation
    with finer's corner sum, then the correction added.  The oracle's FP64
    transfers equal those subroutines run through the translator."""
    import ctypes as C
    g, m = load("ref_transfer_rotann2_33.npz")
    n = m["n"]
    nc = (n - 1) // 2 + 1
    dp = C.POINTER(C.c_double)
    r = np.ascontiguousarray(g["r"])
    fc = np.zeros((nc, nc))
    oracle.lib().orc_restrict64(n, r.ctypes.data_as(dp), fc.ctypes.data_as(dp))
    np.testing.assert_array_equal(fc, g["fc"])
    psi = np.ascontiguousarray(g["psi"]).copy()
    ec = np.ascontiguousarray(g["ec"])
    oracle.lib().orc_prolong_add64(n, ec.ctypes.data_as(dp), psi.ctypes.data_as(dp))
    np.testing.assert_array_equal(psi, g["psi_out"])


def test_fixtures_regenerate_from_the_reference_source():
    """Provenance: where the reference source tree is present, the
    translator run again gives the committed fixtures exactly (the source
    file's SHA-256 included).  Skipped where the tree is absent."""
    import sys
    sys.path.insert(0, GOLD)
    import reference_runs as RR
    if not os.path.isdir(RR.REFERENCE):
        pytest.skip("reference source tree not present")
    g, m = load("ref_layer_16x48.npz")
    res = RR.run_2d("layer", m["nr"], m["np"], m["steps"], dt=m["dt"], r0=m["r0"], rmax=m["rmax"], Ra=m["Ra"],
                    Re=m["Re"], Gr=m["Gr"], Pr=m["Pr"])
    assert res["sha256"] == m["sha256"] and res["deck"] == m["deck"]
    np.testing.assert_array_equal(res["nu"], g["nu"])
    np.testing.assert_array_equal(res["sweeps"], g["sweeps"])
    for f, a in res["fields"].items():
        np.testing.assert_array_equal(a, g["f_" + f], err_msg=f)
    g, m = load("ref_transfer_rotann2_33.npz")
    fc, psi, sha = RR.run_rotann2_transfer(m["n"], g["r"], g["ec"], g["psi"])
    assert sha == m["sha256"]
    np.testing.assert_array_equal(fc, g["fc"])
    np.testing.assert_array_equal(psi, g["psi_out"])
