"""The oracle's axisymmetric annulus on a stretched grid (rotann2.f's physics
with grid.f's weights and rcsc.f's stretched multigrid), pinned by:

* the uniform-grid limit: on equal spacings the stretched forms are
  rotann2.f's formulas with weights from the Taylor matrices instead of
  closed-form fractions, so several steps agree with the uniform path to
  rounding (fields and Nusselt number);
* the host tables the device receives: grid.py's five-point wall weights
  equal the oracle's own bit for bit;
* the five-point wall-flux weights are exact on quartics;
* a run on the tanh grid of the 257 x 257 workload's kind (stretch 1.5,
  clustered at all four walls) stays finite and conducts heat: Nu stays
  near the conduction value over the first steps.
"""
import numpy as np
import pytest

from codesthesis_dir_gb300 import grid


def make(O, nr, nz, hr, hz, mode=1, tolcon=1e-9, Ra=1e5, Re=1e2, dt=1e-5, seed=0, amp=1e-2):
    o = O.OracleAXI(nr, nz, dt, 0.5, 1.0, 0.5, Ra, Re, 1.0, mode=mode, tolcon=tolcon)
    if hr is not None:
        o.stretch(hr, hz)
    o.initial(1, seed, amp)
    return o


@pytest.mark.parametrize("nr,nz", [(32, 32), (64, 32), (32, 64)])
def test_uniform_limit_matches_rotann2_path(oracle, nr, nz):
    ou = make(oracle, nr, nz, None, None, tolcon=1e-12)
    os_ = make(oracle, nr, nz, grid.spacing_uniform(nr, 0.5, 1.0), grid.spacing_uniform(nz, 0.0, 0.5), tolcon=1e-12)
    for _ in range(5):
        a, b = ou.step(), os_.step()
        assert a[0] == 0 and b[0] == 0
        assert abs(a[1] - b[1]) <= 1e-12 * abs(a[1])
    for n in ("phi", "omeg", "vel", "theta"):
        x, y = ou.field(n), os_.field(n)
        assert np.max(np.abs(x - y)) <= 1e-11 * max(np.max(np.abs(x)), 1e-300), n


def test_host_wall_weights_equal_the_oracles(oracle):
    hr = grid.spacing_tanh(64, 0.5, 1.0, 1.5)
    hz = grid.spacing_tanh(48, 0.0, 0.5, 1.5)
    o = make(oracle, 64, 48, hr, hz)
    L = grid.build(hr, hz, 0.5)
    w = np.array(grid.fdif(5, 1, 0, L.r[1])[1])
    np.testing.assert_array_equal(w, np.array(o.s.hw[:]))
    # the level-1 tables the device receives equal the oracle's
    st = o._str
    for name in ("r", "z", "cr", "crr", "cz", "czz"):
        got = np.ravel(np.asarray(getattr(L, name)[1], dtype=np.float64))
        np.testing.assert_array_equal(got, st.table(name, 1), err_msg=name)


def test_wall_weights_exact_on_quartics(oracle):
    hr = grid.spacing_tanh(32, 0.5, 1.0, 1.5)
    hz = grid.spacing_tanh(32, 0.0, 0.5, 1.5)
    o = make(oracle, 32, 32, hr, hz)
    r = np.array(o._str.table("r", 1))
    w = np.array(o.s.hw[:])
    # five-point one-sided d/dr at r0: exact on quartics
    f = lambda x: 3.0 - 2.0 * x + 5.0 * x ** 2 - x ** 3 + 0.5 * x ** 4
    df = lambda x: -2.0 + 10.0 * x - 3.0 * x ** 2 + 2.0 * x ** 3
    assert abs(np.dot(w, f(r[:5])) - df(r[0])) <= 1e-9 * abs(df(r[0]))


def test_tanh_grid_run_stays_finite_and_conducting(oracle):
    hr = grid.spacing_tanh(64, 0.5, 1.0, 1.5)
    hz = grid.spacing_tanh(64, 0.0, 0.5, 1.5)
    o = make(oracle, 64, 64, hr, hz, Ra=1e5, Re=1e2, dt=1e-5, amp=1e-3)
    nus = []
    for _ in range(20):
        st, nu, sw, conv = o.step()
        assert st == 0 and sw > 0
        nus.append(nu)
    assert all(np.isfinite(np.array(nus)))
    # the conduction state's Nusselt number is 1 up to the discretisation of
    # the logarithmic profile and the start's noise
    assert abs(nus[-1] - 1.0) < 0.05
    for n in ("phi", "omeg", "vel", "theta"):
        assert np.all(np.isfinite(o.field(n))), n
