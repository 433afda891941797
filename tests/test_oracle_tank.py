"""The horizontal-convection tank (monashubuntudir_velvor2dhorconvtankdir/
velvor2dhorconvtank.f) in the oracle, on the CPU:

* the multigrid with side walls in x (relax2 on lines k = 1..n3-1, relax3's
  last line against the zero wall, tolcon 5e-6) returns fields whose
  residual, formed by an independent numpy restatement of the operator with
  zero side walls, is below the tolerance, in both line orders, and the two
  orders agree;
* after steps from the tank's own start the walls and ghost columns hold
  what update sets (velvor2dhorconvtank.f:812-845): C, v, u zero on the side
  walls, T = k/np on the top wall, the insulated bottom closure and the
  ghost columns 4/3 T(1) - 1/3 T(2);
* the first step stores 2 trans2 in httrans and leaves httrans2 at zero
  (:197-198)."""
import numpy as np
import pytest

NR, NP, XX = 16, 32, 3.1


def _solve(oracle, which, mode, tolcon=1e-9):
    dr, dp = 1.0 / NR, XX / NP
    ld = NR + 2
    rng = np.random.default_rng(which)
    rhs = np.zeros((ld, NP + 2), order="F")
    imax = NR if which == 2 else NR - 1
    k1 = NP - 1 if which == 2 else NP
    rhs[1:imax + 1, 1:k1 + 1] = rng.standard_normal((imax, k1))
    psi = np.zeros((ld, NP + 2), order="F")
    psip = np.zeros_like(psi)
    st, sw = oracle.poisson(which, psi, psip, rhs, NR, NP, dr, dp, mode=mode, tolcon=tolcon,
                            variant=oracle.ORC_TANK)
    return st, sw, psi, rhs


@pytest.mark.parametrize("which", [2, 3])
@pytest.mark.parametrize("mode", [0, 1], ids=["lex", "zebra"])
def test_walled_poisson_residual(oracle, which, mode):
    st, sw, P, rhs = _solve(oracle, which, mode)
    assert st == 0 and 1 <= sw < 200
    dr, dp = 1.0 / NR, XX / NP
    hhr, hhp = dr * dr, dp * dp
    if which == 2:
        k = np.arange(1, NP)                 # v walls at k = 0 and np
        res = []
        for i in range(1, NR + 1):
            t = (P[i, k + 1] - 2 * P[i, k] + P[i, k - 1]) / hhp
            if i == 1:
                t += (-2 * P[1, k] + 5 / 3 * P[2, k] - 0.2 * P[3, k]) / hhr
            elif i == NR:
                t += (-2 * P[NR, k] + 5 / 3 * P[NR - 1, k] - 0.2 * P[NR - 2, k]) / hhr
            else:
                t += (P[i - 1, k] - 2 * P[i, k] + P[i + 1, k]) / hhr
            res.append(rhs[i, k] - t)
        assert np.all(P[:, 0] == 0) and np.all(P[:, NP] == 0)
    else:
        k = np.arange(1, NP + 1)             # u walls at k = 0 and np+1
        res = []
        for i in range(1, NR):
            t = (P[i + 1, k] + P[i - 1, k]) / hhr + (P[i, k + 1] + P[i, k - 1]) / hhp - P[i, k] * (2 / hhr + 2 / hhp)
            res.append(rhs[i, k] - t)
        assert np.all(P[:, 0] == 0) and np.all(P[:, NP + 1] == 0)
    assert np.max(np.abs(res)) < 1e-8


def test_walled_orders_agree(oracle):
    for which in (2, 3):
        a = _solve(oracle, which, 0, tolcon=1e-11)[2]
        b = _solve(oracle, which, 1, tolcon=1e-11)[2]
        assert np.max(np.abs(a - b)) < 1e-9 * np.max(np.abs(a))


def test_tank_steps_walls_and_ghosts(oracle):
    o = oracle.OraclePRB(NR, NP, 1e-6, 1e6, 10.0, r0=0.5, rmax=1.5, xx=XX, mode=1, variant=oracle.ORC_TANK)
    assert o.mgv.tolcon == 5e-6 and o.ncol == NP + 2
    o.initial()
    st, nu, sw = o.step()
    assert st == 0 and nu[1] == 0.0 and nu[0] != 0.0
    for _ in range(4):
        st, nu, sw = o.step()
        assert st == 0 and nu[1] != 0.0
    f = {n: np.array(o.field(n)) for n in ("C", "vel", "uel", "th")}
    assert np.all(f["C"][:NR + 1, 0] == 0) and np.all(f["C"][:NR + 1, NP] == 0)
    assert np.all(f["vel"][:, 0] == 0) and np.all(f["vel"][:, NP] == 0)
    assert np.all(f["uel"][:, 0] == 0) and np.all(f["uel"][:, NP + 1] == 0)
    assert np.abs(f["vel"]).max() > 1e-6 and np.abs(f["uel"]).max() > 1e-6
    th = f["th"]
    k = np.arange(1, NP + 1)
    np.testing.assert_array_equal(th[NR + 1, 1:NP + 1], k / NP * 1.0)
    np.testing.assert_array_equal(th[:, 0], 2.0 / 1.5 * th[:, 1] - 1.0 / 3.0 * th[:, 2])
    np.testing.assert_array_equal(th[:, NP + 1], 2.0 / 1.5 * th[:, NP] - 1.0 / 3.0 * th[:, NP - 1])


def test_dvd_cavity_walls(oracle):
    """The differentially heated cavity (velvor2ddvdbenchmark.f): T = 0 and
    1 on the bottom and top rows including the ghost columns, the insulated
    closure on the side ghosts, side-wall vorticities -u(1)/dp and u(np)/dp
    (:819-830), and Nu = trans (the first step storing trans2)."""
    n = 16
    o = oracle.OraclePRB(n, n, 2e-5, 1e5, 0.71, r0=0.0, rmax=1.0, xx=1.0, mode=1, variant=oracle.ORC_DVD)
    o.initial()
    th0 = np.array(o.field("th"))
    assert np.all(th0[0, :n + 1] == 0.0) and np.all(th0[n + 1, :n + 1] == 1.0) and np.all(th0[:, n + 1] == 0.5)
    st, nu, sw = o.step()
    assert st == 0 and nu[1] == 0.0
    for _ in range(4):
        st, nu, sw = o.step()
        assert st == 0
    th, C, u = (np.array(o.field(x)) for x in ("th", "C", "uel"))
    assert np.all(th[0] == 0.0) and np.all(th[n + 1] == 1.0)
    i = np.arange(1, n + 1)
    want0 = -30.0 / 92.0 * (-3.75 * th[i, 1] + 5.0 / 6.0 * th[i, 2] - 3.0 / 20.0 * th[i, 3])
    np.testing.assert_array_equal(th[i, 0], want0)
    np.testing.assert_array_equal(C[:n + 1, 0], -u[:n + 1, 1] / o.s.dp)
    np.testing.assert_array_equal(C[:n + 1, n], u[:n + 1, n] / o.s.dp)
    assert np.abs(u).max() > 1e-6
