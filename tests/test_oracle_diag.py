"""The time-loop diagnostics of the 2D drivers (PRB:404-493 and
velvor2dnewsch3.4.f:404-493) in the oracle, on the CPU:

* the running means after steps 2..kt of a block are the plain means of T^2,
  T, u^2 and v^2 over those steps (to rounding), and a new block starts them
  again;
* the CFL maxima are |u| dt / dr over rows 1..nr and |v| dt / (r dp) over rows
  1..nr-1 with r = 1 (layer) or the cell-centre radius (annulus);
* the zonal rows of zmtmtempvar.dat are the zonal means of the time
  variance of T and the rms of u and v."""
import math

import numpy as np
import pytest

from prb_helpers import config0_params


def _run(oracle, variant, steps):
    if variant == "layer":
        p = config0_params(16, 32)
        o = oracle.OraclePRB(p["nr"], p["np_"], 2e-4, 1e6, p["Pr"], r0=p["r0"], rmax=p["rmax"], xx=p["xx"],
                             mode=1)
    else:
        o = oracle.OraclePRB(16, 32, 1e-6, 1e6, 0.71, r0=0.5, rmax=1.0, mode=1, variant=oracle.ORC_ANNULUS,
                             Re=1.06148e5)
    o.initial(1, 5, 5e-2)
    o.enable_diagnostics()
    samples = []
    for _ in range(steps):
        st, _, _ = o.step()
        assert st == 0
        if o.kt >= 2:
            samples.append({n: np.array(o.field(n)) for n in ("th", "uel", "vel")})
    return o, samples


@pytest.mark.parametrize("variant", ["layer", "annulus"])
def test_running_means_and_cfl(oracle, variant):
    o, samples = _run(oracle, variant, 7)
    assert len(samples) == 6
    T = np.stack([s["th"] for s in samples])
    U = np.stack([s["uel"] for s in samples])
    V = np.stack([s["vel"] for s in samples])
    for q, ref in enumerate(((T * T).mean(0), T.mean(0), (U * U).mean(0), (V * V).mean(0))):
        np.testing.assert_allclose(o.running_mean(q), ref, rtol=1e-13, atol=1e-300)
    assert o.cfl_hist[0] == (0.0, 0.0) and len(o.cfl_hist) == 7
    s = o.s
    nr = s.nr
    u, v = samples[-1]["uel"], samples[-1]["vel"]
    cu = np.max(np.abs(u[1:nr + 1, :] * s.dt / s.dr))
    i = np.arange(1, nr)
    r = s.r0 + (i - 0.5) * s.dr if variant == "annulus" else np.ones(nr - 1)
    cv = np.max(np.abs(v[1:nr, :] * s.dt / (r[:, None] * s.dp)))
    assert o.cfl_hist[-1] == (cu, cv)
    assert cu > 0.0 and cv > 0.0
    z = o.zmtm()
    n = s.np + 1
    var = ((T * T).mean(0) - T.mean(0) ** 2).sum(1) / n
    np.testing.assert_allclose(z[:, 0], var, rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(z[:, 1], np.sqrt((U * U).mean(0).sum(1) / n), rtol=1e-13)
    np.testing.assert_allclose(z[:, 2], np.sqrt((V * V).mean(0).sum(1) / n), rtol=1e-13)


def test_new_block_restarts_the_means(oracle):
    o, _ = _run(oracle, "layer", 4)
    o.new_block()
    st, _, _ = o.step()
    assert st == 0 and o.kt == 2
    th = np.array(o.field("th"))
    np.testing.assert_array_equal(o.running_mean(0), th * th)
    np.testing.assert_array_equal(o.running_mean(1), th)


def test_cfl_skips_nan(oracle):
    """A NaN never wins the reference's `cfl.gt.cflmax` comparison."""
    o, _ = _run(oracle, "layer", 2)
    u = o.field("uel")
    keep = u[3, 4]
    u[3, 4] = math.nan
    import ctypes as C
    cu, cv = C.c_double(), C.c_double()
    oracle.lib().orc_prb_cfl(C.byref(o.s), C.byref(cu), C.byref(cv))
    u[3, 4] = keep
    assert math.isfinite(cu.value) and cu.value > 0.0
