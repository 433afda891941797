"""The oracle's 3D rotating annulus (rot3dmg.f) checked by invariants of its
own, on the CPU:

* the three velocity operators of relax1/2/3 (residuals rot3dmg.f:1688-1720,
  :1935-1977, :2129-2160),
    w: w_rr + w_r / r + w_phiphi / r^2 + w_zz,
    v: v_rr + 3 v_r / r + v / r^2 + v_phiphi / r^2 + v_zz,
    u: u_rr + 3 u_r / r + u / r^2 + u_phiphi / r^2 + u_zz,
  are solved to second order by the multigrid: a manufactured solution's
  error falls ~4x per grid halving (one-sided wall rows assume the field and
  its normal derivative vanish there, so those directions use sin^2);
* both line orderings converge to the same solution;
* the smoother's fixed point is not an exact zero of the residual: the z-
  and phi-line right-hand sides use the REAL*4 literal 0.2 where the r-line
  matrices and the residual use 0.2d0 (e.g. rot3dmg.f:1626 against :1584,
  :1707), so the fine residual stalls near 1e-7 |psi| / h^2, far below the
  reference's tolcon 1e-5 and above the rounding floor;
* the conduction profile 1 - ln r / ln r0 at rest is a steady state of the
  step with Nusselt number 1 (rmax = 1) by the reference's
  -r0 ln(r0/rmax) trans1 / (zmax 2 pi) (rot3dmg.f:255);
* the level count follows poissoninit (rot3dmg.f:1172-1192);
* corser leaves planes k = 0 and k = n3c of the coarse right-hand side to the
  shared residual array (rot3dmg.f:2196, 2245-2252);
* finer reproduces a linear coarse field exactly;
* beyond the sweep limit the solve reports it (the reference STOPs,
  rot3dmg.f:1259)."""
import ctypes as C
import math

import numpy as np
import pytest

R0, RMAX, ZMAX = 0.5, 1.0, 0.5


def _mk(O, nr, nz, np_, **kw):
    return O.OracleR3D(nr, nz, np_, 1e-5, R0, RMAX, ZMAX, 1e5, 100.0, 7.0, **kw)


def _manufactured(o, which, m=2):
    """Exact field and right-hand side on the component's own points."""
    s = o.s
    nr, nz, np_ = s.nr, s.nz, s.np
    D = RMAX - R0
    kr, kz = math.pi / D, math.pi / ZMAX
    i = np.arange(nr + 2, dtype=np.float64)
    j = np.arange(nz + 2, dtype=np.float64)
    r = R0 + i * s.dr if which == 3 else R0 + (i - 0.5) * s.dr
    z = j * s.dz if which == 1 else (j - 0.5) * s.dz
    ph = np.arange(np_ + 1) * s.dp
    R, Z, PH = np.meshgrid(r, z, ph, indexing="ij")
    Sr, Cr = np.sin(kr * (R - R0)), np.cos(kr * (R - R0))
    Sz, Cz = np.sin(kz * Z), np.cos(kz * Z)
    if which == 3:
        g, g1, g2 = Sr, kr * Cr, -(kr ** 2) * Sr
    else:
        g, g1, g2 = Sr ** 2, 2 * kr * Sr * Cr, 2 * kr ** 2 * (Cr ** 2 - Sr ** 2)
    if which == 1:
        h, h2 = Sz, -(kz ** 2) * Sz
    else:
        h, h2 = Sz ** 2, 2 * kz ** 2 * (Cz ** 2 - Sz ** 2)
    c = np.cos(m * PH)
    if which == 1:
        f = ((g2 + g1 / R - m * m * g / R ** 2) * h + g * h2) * c
    else:
        f = ((g2 + 3 * g1 / R + g / R ** 2 - m * m * g / R ** 2) * h + g * h2) * c
    return g * h * c, f


def _unknowns(o, which):
    s = o.s
    ii = slice(1, s.nr) if which == 3 else slice(1, s.nr + 1)
    jj = slice(1, s.nz) if which == 1 else slice(1, s.nz + 1)
    return ii, jj


NAMES = {1: ("wel", "welp", "wrh"), 2: ("vel", "velp", "vrh"), 3: ("uel", "uelp", "urh")}


def _solve(O, nr, nz, np_, which, mode, tol=1e-5):
    o = _mk(O, nr, nz, np_, mode=mode, tolcon=tol)
    exact, f = _manufactured(o, which)
    psi, psip, rhs = (o.field(n) for n in NAMES[which])
    psi[...] = 0.0
    psip[...] = 0.0
    rhs[...] = f
    st, sw = o.poisson(which)
    return o, st, sw, exact


@pytest.mark.parametrize("which", [1, 2, 3], ids=["w", "v", "u"])
def test_operator_second_order(oracle, which):
    errs = []
    for n in (8, 16):
        o, st, sw, exact = _solve(oracle, n, n, 2 * n, which, oracle.ORC_ZEBRA)
        assert st == 0, (st, sw)
        ii, jj = _unknowns(o, which)
        psi = np.array(o.field(NAMES[which][0]))
        errs.append(np.max(np.abs(psi[ii, jj, :] - exact[ii, jj, :])))
        o.close()
    rate = errs[0] / errs[1]
    assert errs[1] < 5e-2, errs
    assert rate > 3.0, (errs, rate)


@pytest.mark.parametrize("which", [1, 2, 3], ids=["w", "v", "u"])
def test_orderings_agree(oracle, which):
    a, st, sw_a, _ = _solve(oracle, 8, 8, 16, which, oracle.ORC_LEX, tol=2e-6)
    b, st2, sw_b, _ = _solve(oracle, 8, 8, 16, which, oracle.ORC_ZEBRA, tol=2e-6)
    assert st == 0 and st2 == 0
    pa, pb = np.array(a.field(NAMES[which][0])), np.array(b.field(NAMES[which][0]))
    assert np.max(np.abs(pa - pb)) < 1e-7 * max(1.0, np.max(np.abs(pa)))
    # the previous level takes the old field (zero here), walls are zero
    assert np.all(np.array(a.field(NAMES[which][1])) == 0.0)


def test_poisson_moves_time_levels(oracle):
    """On convergence psip takes the old psi and psi the new interior with
    zero walls (rot3dmg.f:1291-1315)."""
    o = _mk(oracle, 8, 8, 16)
    exact, f = _manufactured(o, 2)
    rng = np.random.default_rng(1)
    old = rng.standard_normal(o.shape)
    o.field("vel")[...] = old
    o.field("velp")[...] = old
    o.field("vrh")[...] = f
    st, sw = o.poisson(2)
    assert st == 0
    np.testing.assert_array_equal(np.array(o.field("velp")), old)
    v = np.array(o.field("vel"))
    assert np.all(v[0] == 0) and np.all(v[-1] == 0) and np.all(v[:, 0] == 0) and np.all(v[:, -1] == 0)


def test_conduction_state(oracle):
    nr, nz, np_ = 8, 8, 16
    o = _mk(oracle, nr, nz, np_)
    o.initial(3, 0.0)
    s = o.s
    i = np.arange(nr + 2, dtype=np.float64)
    r = np.where(i == 0, R0, np.where(i == nr + 1, RMAX, R0 + (i - 0.5) * s.dr))
    prof = 1.0 - np.log(r) / np.log(R0)
    for name in ("th", "thp"):
        o.field(name)[...] = prof[:, None, None]
    th0 = np.array(o.field("th"))
    for _ in range(3):
        st, nu, sw = o.step()
        assert st == 0
        assert abs(nu - 1.0) < 5e-3, nu
    assert np.max(np.abs(np.array(o.field("th")) - th0)) < 1e-4
    # at rest up to rounding: the end-wall and interior z rows of T agree to
    # ~1e-16 only, and Ra = 1e5 turns that into ~1e-9 velocities
    for name in ("uel", "vel", "wel", "A", "B", "C"):
        assert np.max(np.abs(np.array(o.field(name)))) < 1e-6, name


@pytest.mark.parametrize("nr,nz,np_,nlev", [(64, 64, 128, 4), (16, 8, 16, 2), (8, 8, 8, 2), (12, 8, 16, 2),
                                           (32, 16, 64, 3)])
def test_level_count(oracle, nr, nz, np_, nlev):
    o = _mk(oracle, nr, nz, np_)
    assert o.s.nlev == nlev
    for l in range(1, nlev + 1):
        assert o.s.n1[l] == nr >> (l - 1) and o.s.n2[l] == nz >> (l - 1) and o.s.n3[l] == np_ >> (l - 1)


def test_invalid_sizes(oracle):
    for args in ((4, 4, 5), (16, 16, 12), (3, 8, 16)):
        with pytest.raises(ValueError):
            _mk(oracle, *args)


def test_corser_planes(oracle):
    o = _mk(oracle, 16, 16, 32)
    rng = np.random.default_rng(4)
    res = o.level("res", 1)
    res[...] = rng.standard_normal(res.shape)
    res[:, :, 0] = 0.0          # never written by relax
    oracle.lib().orc_r3d_corser(C.byref(o.s), 1)
    fc = o.level("f", 2)
    n1c, n2c, n3c = o.s.n1[2], o.s.n2[2], o.s.n3[2]
    np.testing.assert_array_equal(fc[1:n1c, 1:n2c, n3c], res[1:n1c, 1:n2c, n3c])
    assert np.all(fc[1:n1c, 1:n2c, 0] == 0.0)
    assert np.all(fc[0] == 0) and np.all(fc[n1c] == 0) and np.all(fc[:, 0] == 0) and np.all(fc[:, n2c] == 0)
    # an interior point is the 27-point full weighting
    i, j, k = 3, 4, 5
    w = np.array([0.5, 1.0, 0.5])
    W = w[:, None, None] * w[None, :, None] * w[None, None, :]
    blk = res[2 * i - 1:2 * i + 2, 2 * j - 1:2 * j + 2, 2 * k - 1:2 * k + 2]
    assert abs(fc[i, j, k] - np.sum(W * blk) / 8.0) < 1e-14 * np.sum(np.abs(blk))
    assert np.all(o.level("v", 2) == 0.0)


def test_finer_linear_exact(oracle):
    o = _mk(oracle, 16, 16, 32)
    vc = o.level("v", 2)
    I, J, K = np.meshgrid(*(np.arange(n) for n in vc.shape), indexing="ij")
    vc[...] = 0.25 * I - 0.5 * J + 0.125 * K
    vf = o.level("v", 1)
    vf[...] = 1.0
    oracle.lib().orc_r3d_finer(C.byref(o.s), 2)
    I, J, K = np.meshgrid(*(np.arange(n) for n in vf.shape), indexing="ij")
    np.testing.assert_allclose(vf, 1.0 + (0.25 * I - 0.5 * J + 0.125 * K) / 2.0, rtol=0, atol=1e-14)
    assert np.all(o.level("v", 2) == 0.0)


@pytest.mark.parametrize("which", [1, 2, 3], ids=["w", "v", "u"])
def test_residual_stall_from_real4_literal(oracle, which):
    """The stall: far below tolcon, well above the FP64 rounding floor."""
    o = _mk(oracle, 8, 8, 16, tolcon=1e-30, maxsweeps=60)
    exact, f = _manufactured(o, which)
    o.field(NAMES[which][2])[...] = f
    st, sw = o.poisson(which)
    assert st == 1
    assert 1e-9 < o.s.last_resmax < 1e-5, o.s.last_resmax


def test_sweep_limit(oracle):
    o = _mk(oracle, 8, 8, 16, tolcon=1e-30, maxsweeps=3)
    exact, f = _manufactured(o, 1)
    o.field("wrh")[...] = f
    st, sw = o.poisson(1)
    assert st == 1 and sw == 3


# ---------------------------------------------------------------------------
# rot3dmghor.f: the annulus with its axis horizontal
# ---------------------------------------------------------------------------
def _hor(oracle, Gr, nr=8, nz=8, np_=16, tolcon=None):
    o = oracle.OracleR3D(nr, nz, np_, 1e-5, 0.5, 1.0, 0.5, 0.0, 0.0, 7.0, Gr=Gr, mode=1, horizontal=True,
                         tolcon=tolcon)
    return o


def test_horizontal_initial_state_matches_host(oracle):
    from codesthesis_dir_gb300 import initial
    o = _hor(oracle, 1e4)
    o.initial(3, 5e-2)
    np.testing.assert_array_equal(np.array(o.field("th")),
                                  initial.r3d_reference(8, 8, 16, 0.5, 1.0, 3, 5e-2, horizontal=True))
    th = np.array(o.field("th"))
    assert th[0, 3, 0] == 1.0 and th[9, 3, 0] == 0.0   # the inner cylinder hot


def test_horizontal_without_gravity_stays_at_rest(oracle):
    """With Gr = 0 the horizontal annulus has no body force: the flow stays
    exactly at rest while T diffuses; with Gr > 0 it moves."""
    for Gr, moving in ((0.0, False), (1e4, True)):
        o = _hor(oracle, Gr)
        o.initial(3, 5e-2)
        for _ in range(3):
            st, nu, sw = o.step()
            assert st == 0, sw
        vmax = max(np.abs(np.array(o.field(n))).max() for n in ("uel", "vel", "wel"))
        assert (vmax > 1e-6) == moving, (Gr, vmax)


def test_horizontal_heat_of_the_conduction_profile(oracle):
    """For T = ln r / ln r0 (the conduction state, inner wall 1 at r0, outer
    0 at rmax = 1) both Nusselt numbers of rot3dmghor.f:264-267 are 1 to
    the one-sided derivative's accuracy."""
    import ctypes as C
    for nr in (16, 32):
        o = _hor(oracle, 0.0, nr=nr, nz=16, np_=16)
        s = o.s
        i = np.arange(nr + 2)
        r = np.where(i == 0, s.r0, np.where(i == nr + 1, s.rmax, s.r0 + (i - 0.5) * s.dr))
        o.field("th")[...] = (np.log(r) / math.log(s.r0))[:, None, None]
        t2 = C.c_double()
        t1 = oracle.lib().orc_r3d_heat2(C.byref(s), C.byref(t2))
        L = math.log(s.r0 / s.rmax)
        nu1 = s.nz / 6.0 * s.r0 * L * t1 / (s.zmax * 2.0 * math.pi)
        nu2 = s.nz / 6.0 * s.rmax * L * t2.value / (s.zmax * 2.0 * math.pi)
        assert abs(nu1 - 1.0) < 40.0 / nr ** 2 and abs(nu2 - 1.0) < 40.0 / nr ** 2, (nr, nu1, nu2)


def test_horizontal_plain_cycle_converges_at_the_reference_tolerance(oracle):
    o = _hor(oracle, 1e4)
    assert o.s.tolcon == 1e-6
    o.initial(3, 5e-2)
    st, nu, sw = o.step()
    assert st == 0 and all(0 < x < 100 for x in sw)
    assert abs(nu - 1.0) < 0.01 and abs(o.nu2 - 1.0) < 0.01
