"""The oracle's rotating-annulus variant (velvor2dnewsch3.4.f of
iarchomedir_groke_storage_users_mpking_rotannconvvelvorplane_continueddir)
checked by invariants of its own, on the CPU:

* the polar velocity operators of relax2/relax3,
  u_rr + 3 u_r / r + u / r^2 + u_phiphi / r^2 (:2300-2346, :2546-2579), are
  consistent: the multigrid solution of a manufactured problem converges to
  the exact field at rate ~h^2 (relax3, Dirichlet faces) and better than h
  (relax2, whose wall rows assume v = v_r = 0 on the wall);
* the conduction profile 1 - ln r / ln r0 is (to discretisation error) a
  steady state and carries Nusselt number 1 at the inner wall and -1 at the
  outer wall (whose derivative is taken inward) with the reference's
  Nu = -r0 ln(r0/rmax) trans1 / (2 pi) (:386-387);
* the level cap is 5 (:1778) against PRB's 4;
* corser leaves the fine residual on the coarse seam line (:2696-2704);
* the sweep limit does not stop a step (:1853)."""
import ctypes as C
import math

import numpy as np
import pytest


def _manufactured(nr, np_, which, r0=0.5, rmax=1.0):
    D = rmax - r0
    dr, dp = D / nr, 2 * math.pi / np_
    ii = np.arange(nr + 2, dtype=np.float64)
    r = r0 + ii * dr if which == 3 else r0 + (ii - 0.5) * dr
    phi = np.arange(np_ + 1) * dp
    R, PH = np.meshgrid(r, phi, indexing="ij")
    k = math.pi / D
    S, Cs = np.sin(k * (R - r0)), np.cos(k * (R - r0))
    if which == 3:
        # faces: Dirichlet u = 0 on the walls
        g, gr, grr = S, k * Cs, -(k ** 2) * S
    else:
        # cell centres: the wall rows (-2, 5/3, -1/5) and 4/3 of relax2 are
        # exact for a field with v = v_r = 0 on the wall, so use sin^2
        g, gr, grr = S ** 2, 2 * k * S * Cs, 2 * k ** 2 * (Cs ** 2 - S ** 2)
    exact = g * np.cos(2 * PH)
    f = (grr + 3 * gr / R + g / R ** 2 - 4 * g / R ** 2) * np.cos(2 * PH)
    return dr, dp, exact, np.asfortranarray(f)


@pytest.mark.parametrize("which", [2, 3])
def test_polar_operator_second_order(oracle, which):
    errs = []
    for nr, np_ in ((16, 64), (32, 128)):
        dr, dp, exact, f = _manufactured(nr, np_, which)
        psi = np.zeros((nr + 2, np_ + 1), order="F")
        psip = np.zeros_like(psi)
        st, sw = oracle.poisson(which, psi, psip, f, nr, np_, dr, dp, tolcon=1e-10, maxsweeps=2000,
                                variant=oracle.ORC_ANNULUS, r0=0.5)
        assert st == 0, (st, sw)
        rows = slice(1, nr) if which == 3 else slice(1, nr + 1)
        errs.append(np.max(np.abs(psi[rows, :] - exact[rows, :])))
    rate = errs[0] / errs[1]
    assert errs[1] < 2e-2, errs
    assert rate > (3.3 if which == 3 else 2.5), (errs, rate)


def test_conduction_state_nusselt_one(oracle):
    nr, np_ = 32, 64
    o = oracle.OraclePRB(nr, np_, 1e-6, 1e5, 1.0, r0=0.5, rmax=1.0, variant=oracle.ORC_ANNULUS, Re=1e4)
    o.initial(1, 0, 0.0)                       # 1 - ln r / ln r0, no noise
    th0 = np.array(o.field("th"))
    for _ in range(3):
        st, nu, sw = o.step()
        assert st == 0
        # trans2 is the one-sided derivative taken inward from rmax, so the
        # reference's outer-wall number is -1 for conduction
        assert abs(nu[0] - 1.0) < 2e-3 and abs(nu[1] + 1.0) < 2e-3, nu
    drift = np.max(np.abs(np.array(o.field("th"))[1:nr + 1] - th0[1:nr + 1]))
    assert drift < 1e-4, drift


def test_level_cap_is_five(oracle):
    L = oracle.lib()
    for variant, cap in ((oracle.ORC_PRB, 4), (oracle.ORC_ANNULUS, 5)):
        mg = oracle.MG()
        assert L.orc_mg_init_variant(C.byref(mg), 256, 256, 1 / 256, 1 / 256, variant, 0.5) == 0
        assert mg.nlev == cap
        L.orc_mg_free(C.byref(mg))


@pytest.mark.parametrize("variant", [0, 1], ids=["layer", "annulus"])
def test_corser_seam_residual(oracle, variant):
    L = oracle.lib()
    nr, np_ = 32, 64
    mg = oracle.MG()
    assert L.orc_mg_init_variant(C.byref(mg), nr, np_, 0.5 / nr, 2 * math.pi / np_, variant, 0.5) == 0
    ld = mg.ld
    rc = np.ctypeslib.as_array(mg.rc, shape=(ld * (np_ + 1),)).reshape(np_ + 1, ld).T
    rng = np.random.default_rng(5)
    rc[:, :] = rng.standard_normal(rc.shape)
    seam = rc[:, np_ // 2].copy()
    L.orc_corser(C.byref(mg), 1)
    n1c, n3c = mg.n1[2], mg.n3[2]
    fc = np.ctypeslib.as_array(mg.f[2], shape=((n1c + 1) * (n3c + 1),)).reshape(n3c + 1, n1c + 1).T
    want = seam[1:n1c] if variant == 1 else np.zeros(n1c - 1)
    np.testing.assert_array_equal(fc[1:n1c, n3c], want)
    assert np.all(fc[0, :] == 0) and np.all(fc[n1c, :] == 0)
    L.orc_mg_free(C.byref(mg))


def test_sweep_limit_does_not_stop_the_step(oracle):
    o = oracle.OraclePRB(16, 32, 1e-6, 1e5, 1.0, r0=0.5, rmax=1.0, variant=oracle.ORC_ANNULUS, Re=1e4,
                         tolcon=1e-30, maxsweeps=2)
    o.initial(1, 3, 1e-2)
    vel0 = np.array(o.field("vel"))
    st, nu, sw = o.step()
    assert st == 0 and list(sw) == [2, 2]
    np.testing.assert_array_equal(np.array(o.field("vel")), vel0)   # psi untouched
    assert np.all(np.isfinite(nu))
