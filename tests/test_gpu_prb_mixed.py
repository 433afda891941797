"""The mixed-precision velocity solves (GB_PRB_MIXED: FP32 multigrid cycles
inside FP64 defect correction) against the FP64 oracle: after the stated
steps the Nusselt numbers agree to relative error <= 1e-6 and the fields
psi (velocities), omega (C) and T to relative L2 <= 1e-6, the bar the mixed
path is held to; every solve converges to the FP64 tolerance."""
import numpy as np
import pytest

from prb_helpers import STATE_FIELDS, config0_params, rel_l2

pytestmark = pytest.mark.gpu

TOL_FIELD = 1e-6
TOL_NU = 1e-6


def _pair(O, P, prm, smoother, tolcon, variant=0, Re=0.0, kind=1, amp=1e-3):
    o = O.OraclePRB(prm["nr"], prm["np_"], prm["dt"], prm["Ra"], prm["Pr"], r0=prm["r0"], rmax=prm["rmax"],
                    xx=prm.get("xx", 3.0), mode=smoother, tolcon=tolcon, variant=variant, Re=Re)
    o.initial(kind, 0, amp)
    g = P.PRB(prm["nr"], prm["np_"], dt=prm["dt"], r0=prm["r0"], rmax=prm["rmax"], xx=prm.get("xx", 3.0),
              Ra=prm["Ra"], Pr=prm["Pr"], tolcon=tolcon, smoother=smoother, variant=variant, Re=Re,
              precision=1)
    for name in STATE_FIELDS:
        g.set(name, np.array(o.field(name), order="F"))
    return o, g


@pytest.fixture(scope="module")
def P(gblib):
    from codesthesis_dir_gb300 import prb
    return prb


@pytest.mark.parametrize("smoother", [0, 1], ids=["lex", "zebra"])
def test_layer_mixed_vs_fp64_oracle(oracle, P, smoother):
    """The 129 x 65 layer with the 1e-10 tolerance, 40 steps (zebra); the
    lexicographic order on the 65 x 33 layer, 10 steps."""
    prm = config0_params() if smoother else config0_params(32, 64)
    o, g = _pair(oracle, P, prm, smoother, 1e-10)
    nsteps = 40 if smoother else 10
    nu_o = np.array([o.step()[1] for _ in range(nsteps)])
    nu_g, sw_g = g.step(nsteps)
    assert np.all(sw_g > 0)
    rel_nu = np.max(np.abs(nu_g - nu_o) / np.abs(nu_o))
    assert rel_nu <= TOL_NU, rel_nu
    for name in ("vel", "uel", "C", "th"):
        e = rel_l2(np.array(o.field(name)), g.get(name))
        assert e <= TOL_FIELD, (name, e)


def test_annulus_mixed_vs_fp64_oracle(oracle, P):
    """The annulus (polar operators, four levels), 8 steps from the
    reference's initial profile, tolerance 1e-8.  (The absolute residual
    tolerance must stay above the FP64 rounding floor of the residual,
    about 1e-16 |A| |psi|: once the velocities grow, 1e-10 is below it on
    64 x 128, both solvers then stop at the sweep limit and their
    trajectories part.)"""
    prm = dict(nr=32, np_=64, dt=2e-7, Ra=8e7, Pr=0.71, r0=0.5, rmax=1.0)
    o, g = _pair(oracle, P, prm, 1, 1e-8, variant=1, Re=1.06148e5, kind=0)
    nsteps = 8
    nu_o = np.array([o.step()[1] for _ in range(nsteps)])
    nu_g, sw_g = g.step(nsteps)
    rel_nu = np.max(np.abs(nu_g - nu_o) / np.abs(nu_o))
    assert rel_nu <= TOL_NU, rel_nu
    for name in ("vel", "uel", "C", "th"):
        e = rel_l2(np.array(o.field(name)), g.get(name))
        assert e <= TOL_FIELD, (name, e)


def test_mixed_solve_meets_fp64_tolerance(oracle, P):
    """One solve at tolerance 1e-9: the mixed result agrees with the FP64
    oracle's solve of the same right-hand side to relative L2 1e-7, in a
    bounded number of FP32 cycles."""
    prm = config0_params(32, 64)
    o, g = _pair(oracle, P, prm, 1, 1e-9)
    o.step()
    g.cvorticity1()
    g.temperature1()
    g.rhsv()
    cycles = g.poisson2()
    assert 0 < cycles < 60
    v_mixed = g.get("vel")
    v_fp64 = np.array(o.field("vel"))
    assert rel_l2(v_fp64, v_mixed) <= 1e-7


@pytest.mark.parametrize("variant", [0, 1], ids=["layer", "annulus"])
def test_mixed_cluster_spread_equals_one_cta(oracle, P, variant):
    """The mixed solve spread over a cluster of 8 CTAs gives exactly the
    bits of the one-CTA mixed solve (the default):
    fields, Nusselt numbers and cycle counts, on the layer and on the annulus
    (polar operators, three relaxations per visit)."""
    from codesthesis_dir_gb300 import lib
    L = lib.load()
    if variant == 0:
        prm, tol, kw = config0_params(), 1e-10, {}
    else:
        prm, tol, kw = dict(nr=32, np_=64, dt=2e-7, Ra=8e7, Pr=0.71, r0=0.5, rmax=1.0), 1e-8, \
            dict(variant=1, Re=1.06148e5, kind=0)
    _, g8 = _pair(oracle, P, prm, 1, tol, **kw)
    _, g1 = _pair(oracle, P, prm, 1, tol, **kw)
    assert L.gb_prb_set_solve_spread(g8._h, 8) == 0
    assert L.gb_prb_set_solve_spread(g1._h, 1) == 0
    nu8, sw8 = g8.step(12)
    nu1, sw1 = g1.step(12)
    np.testing.assert_array_equal(sw8, sw1)
    np.testing.assert_array_equal(nu8, nu1)
    for name in ("vel", "uel", "C", "th"):
        np.testing.assert_array_equal(g8.get(name), g1.get(name))
