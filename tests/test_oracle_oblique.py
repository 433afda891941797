"""mpkoks.f (the periodic layer with gravity along the diagonal) in the
oracle: its vorticity update differs from the layer's only in the buoyancy
term, RHS2 = -Ra thr 0.707106781 (REAL*4 literal; mpkoks.f:769-770,
:974-975) in place of -Ra thh, for the forward and the leapfrog step."""
import ctypes as C

import numpy as np
import pytest

from prb_helpers import STATE_FIELDS


def _pair(oracle):
    a = oracle.OraclePRB(16, 32, 1e-4, 1e5, 0.71, r0=0.5, rmax=1.0, xx=3.0)
    b = oracle.OraclePRB(16, 32, 1e-4, 1e5, 0.71, r0=0.5, rmax=1.0, xx=3.0, variant=oracle.ORC_OBLIQUE)
    a.initial(1, 7, 5e-2)
    for n in STATE_FIELDS:
        b.field(n)[:, :] = a.field(n)
    return a, b


@pytest.mark.parametrize("first", [1, 0], ids=["forward", "leapfrog"])
def test_only_the_buoyancy_term_changes(oracle, first):
    a, b = _pair(oracle)
    rng = np.random.default_rng(3)
    for n in ("uel", "vel", "C", "Cp"):
        x = rng.standard_normal(a.field(n).shape) * 1e-2
        a.field(n)[:, :] = x
        b.field(n)[:, :] = x
    fn = "orc_cvorticity1" if first else "orc_cvorticity"
    getattr(oracle.lib(), fn)(C.byref(a.s))
    getattr(oracle.lib(), fn)(C.byref(b.s))
    # the derivative fields do not depend on the forcing
    for n in ("A", "B", "An", "Bn"):
        np.testing.assert_array_equal(a.field(n), b.field(n))
    s = a.s
    dri, dpi = 1.0 / s.dr, 1.0 / s.dp
    cnr, cnh = -dri * dri, -dpi * dpi
    cf1 = (1.0 if first else 0.5) / (s.Pr * s.dt) - cnr - cnh
    c = float(np.float32(0.707106781))
    An, Bn = np.array(a.field("An")), np.array(a.field("Bn"))
    want = (-s.Ra * Bn + s.Ra * An * c) / cf1
    got = np.array(b.field("Cn")) - np.array(a.field("Cn"))
    sl = (slice(1, s.nr), slice(0, s.np + 1))
    scale = np.max(np.abs(np.array(a.field("Cn"))[sl])) + np.max(np.abs(want[sl]))
    assert np.max(np.abs(got[sl] - want[sl])) < 1e-13 * scale
    assert np.max(np.abs(want[sl])) > 1e-6 * scale


def test_oblique_steps_run(oracle):
    a, b = _pair(oracle)
    for _ in range(4):
        assert b.step()[0] == 0
        assert a.step()[0] == 0
    assert not np.array_equal(np.array(a.field("C")), np.array(b.field("C")))
