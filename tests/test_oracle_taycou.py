"""The Taylor-Couette driver (monashubuntudir_velvor2dtaycouheatdir/
velvor2dtaycouheat.f) in the oracle, on the CPU:

* the outer cylinder moves at -(Ta**0.5) Ptl rmax / 2 from the start and
  after every update (:177, :1587);
* circular Couette flow v = C (r - r0^2 / r) between the resting inner and
  the moving outer cylinder stays put to the scheme's accuracy: the wall
  vorticity (:1589-1590) and the wall term of rhsv (:1668-1670) carry the
  wall speed into the v solve (without that term the profile collapses);
* the multigrid is PRB's: at most 4 levels where the annulus allows 5, and
  the sweep limit stops the step."""
import math

import numpy as np
import pytest


def _tc(oracle, nr=16, np_=32, Ta=1e4, Ra=0.0, tolcon=None, maxsweeps=None, mode=1):
    return oracle.OraclePRB(nr, np_, 1e-5, Ra, 0.71, r0=0.5, rmax=1.0, mode=mode, variant=oracle.ORC_TAYCOU,
                            Re=1e3, Ta=Ta, tolcon=tolcon, maxsweeps=maxsweeps)


def _velo(s):
    return -(math.pow(s.Ta, 0.5) * s.Pr * 0.5 * s.rmax)


def test_moving_wall(oracle):
    o = _tc(oracle, Ra=1e5)
    o.initial(0, 0, 0.0)
    velo = _velo(o.s)
    assert velo == -35.5
    assert np.all(np.array(o.field("vel"))[o.s.nr + 1] == velo)
    for _ in range(3):
        assert o.step()[0] == 0
    assert np.all(np.array(o.field("vel"))[o.s.nr + 1] == velo)
    assert np.abs(np.array(o.field("vel"))[1:o.s.nr + 1]).max() > 1.0


@pytest.mark.parametrize("nr", [16, 32])
def test_circular_couette_flow_is_steady(oracle, nr):
    o = _tc(oracle, nr=nr, tolcon=1e-9)
    o.initial(0, 0, 0.0)
    s = o.s
    velo = _velo(s)
    Cc = velo / (s.rmax - s.r0 * s.r0 / s.rmax)
    i = np.arange(nr + 2)
    rc = np.where(i == 0, s.r0, np.where(i == nr + 1, s.rmax, s.r0 + (i - 0.5) * s.dr))
    v = Cc * (rc - s.r0 * s.r0 / rc)
    v[0], v[nr + 1] = 0.0, velo
    for n in ("vel", "velp"):
        o.field(n)[:, :] = v[:, None]
    for n in ("C", "Cp", "Cn"):
        o.field(n)[:, :] = 2.0 * Cc        # the vorticity dv/dr + v/r of the profile
    for n in ("th", "thp"):
        o.field(n)[:, :] = 0.0
    v0 = np.array(o.field("vel"))
    for _ in range(20):
        st, nu, sw = o.step()
        assert st == 0
    drift = np.abs(np.array(o.field("vel"))[1:nr + 1] - v0[1:nr + 1]).max() / abs(velo)
    assert drift < 5e-3, drift


def test_prb_multigrid_settings(oracle):
    tc = _tc(oracle, nr=64, np_=64)
    ann = oracle.OraclePRB(64, 64, 1e-5, 0.0, 0.71, r0=0.5, rmax=1.0, variant=oracle.ORC_ANNULUS, Re=1e3)
    assert tc.mgv.nlev == 4 and ann.mgv.nlev == 5
    assert tc.mgv.tolcon == 1e-5 and tc.mgv.maxsweeps == 500
    o = _tc(oracle, Ra=1e5, tolcon=1e-30, maxsweeps=3)
    o.initial(0, 0, 0.0)
    st, nu, sw = o.step()
    assert st == 1 and sw[0] == 3     # ORC_MAXSWEEPS: the reference STOPs
