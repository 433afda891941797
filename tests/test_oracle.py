"""CPU checks of the oracle itself: the banded solvers against dense solves,
the multigrid against manufactured solutions and its own invariants, the
transport step's conservation identities, and the batched Poisson oracle's
order of accuracy.  The reference ships no golden data, so these invariants
(plus the committed fixtures in tests/golden/) are what pins the oracle."""
import numpy as np
import pytest


def dense_tri(a, b, c, periodic=False):
    n = len(b)
    M = np.diag(b) + np.diag(a[1:], -1) + np.diag(c[:-1], 1)
    if periodic:
        M[0, -1] = a[0]
        M[-1, 0] = c[-1]
    return M


@pytest.mark.parametrize("n", [2, 3, 8, 65, 129])
def test_tdma_dense(oracle, n):
    rng = np.random.default_rng(n)
    a, c, r = rng.standard_normal((3, n))
    b = rng.standard_normal(n) + 5.0
    y = oracle.tdma(a, b, c, r)
    np.testing.assert_allclose(dense_tri(a, b, c) @ y, r, atol=1e-13)


@pytest.mark.parametrize("n", [3, 4, 9, 129])
def test_ptdma_dense(oracle, n):
    rng = np.random.default_rng(n)
    a, c, r = rng.standard_normal((3, n))
    b = rng.standard_normal(n) + 5.0
    y = oracle.ptdma(a, b, c, r)
    np.testing.assert_allclose(dense_tri(a, b, c, True) @ y, r, atol=1e-13)


@pytest.mark.parametrize("n", [3, 5, 8, 64])
def test_pdma_dense(oracle, n):
    rng = np.random.default_rng(n)
    a, b, d, e, r = rng.standard_normal((5, n))
    c = rng.standard_normal(n) + 8.0
    x = oracle.pdma(a, b, c, d, e, r)
    M = np.diag(c) + np.diag(b[1:], -1) + np.diag(a[2:], -2) + np.diag(d[:-1], 1) + np.diag(e[:-2], 2)
    np.testing.assert_allclose(M @ x, r, atol=1e-13)


def test_compact_derivative_seam_quirk(oracle):
    """The (1,4,1) compact x-derivative (PRB:833-851) is solved on a ring of
    np+1 unknowns in which k = 0 and k = np are distinct neighbours
    (ptdma with n = np+1).  On sin(x) it is fourth order away from the seam
    and only second order at the seam: the reference's behaviour, kept."""
    far, seam = [], []
    for npts in (32, 64, 128, 256):
        h = 2 * np.pi / npts
        x = np.arange(npts + 1) * h
        f = np.sin(x)
        rhs = np.empty(npts + 1)
        rhs[1:npts] = 3 * (f[2:] - f[:-2]) / h
        rhs[0] = rhs[npts] = 3 * (f[1] - f[npts - 1]) / h
        d = oracle.ptdma(np.ones(npts + 1), 4 * np.ones(npts + 1), np.ones(npts + 1), rhs)
        e = np.abs(d - np.cos(x))
        far.append(e[npts // 2])
        seam.append(e[0])
    rf = np.log2(np.array(far[:-1]) / np.array(far[1:]))
    rs = np.log2(np.array(seam[:-1]) / np.array(seam[1:]))
    assert np.all(rf > 3.8), rf
    assert np.all(np.abs(rs - 2.0) < 0.1), rs


@pytest.mark.parametrize("which", [2, 3])
@pytest.mark.parametrize("mode", [0, 1], ids=["lex", "zebra"])
def test_poisson_residual_converges(oracle, which, mode):
    """Random right-hand side: the solve reports convergence, and the
    operator of relax2/relax3 applied to the returned field reproduces the
    right-hand side to the tolerance (checked with an independent numpy
    restatement of the residual)."""
    nr, np_ = 32, 64
    dr, dp = 1.0 / nr, 2.0 / np_
    ld = nr + 2
    rng = np.random.default_rng(which + 10 * mode)
    rhs = np.zeros((ld, np_ + 1), order="F")
    imax = nr if which == 2 else nr - 1
    rhs[1:imax + 1, :] = rng.standard_normal((imax, np_ + 1))
    rhs[:, np_] = rhs[:, 0]
    psi = np.zeros((ld, np_ + 1), order="F")
    psip = np.zeros_like(psi)
    st, sw = oracle.poisson(which, psi, psip, rhs, nr, np_, dr, dp, mode=mode, tolcon=1e-9)
    assert st == 0 and 1 <= sw < 100
    hhr, hhp = dr * dr, dp * dp
    P = psi
    k = np.arange(1, np_ + 1)
    ka = np.where(k == np_, 1, k + 1)
    km = k - 1
    if which == 2:
        res = np.zeros((nr, np_))
        for i in range(1, nr + 1):
            t = (P[i, ka] - 2 * P[i, k] + P[i, km]) / hhp
            if i == 1:
                t += (-2 * P[1, k] + 5 / 3 * P[2, k] - 0.2 * P[3, k]) / hhr
            elif i == nr:
                t += (-2 * P[nr, k] + 5 / 3 * P[nr - 1, k] - 0.2 * P[nr - 2, k]) / hhr
            else:
                t += (P[i - 1, k] - 2 * P[i, k] + P[i + 1, k]) / hhr
            res[i - 1] = rhs[i, k] - t
    else:
        res = np.zeros((nr - 1, np_))
        for i in range(1, nr):
            t = (P[i + 1, k] + P[i - 1, k]) / hhr + (P[i, ka] + P[i, km]) / hhp - P[i, k] * (2 / hhr + 2 / hhp)
            res[i - 1] = rhs[i, k] - t
    assert np.max(np.abs(res)) < 1e-8
    # walls are zero and the seam duplicate holds (psi(.,0) == psi(.,np))
    assert np.all(P[0] == 0) and np.all(P[imax + 1] == 0)
    np.testing.assert_allclose(P[:, 0], P[:, np_], atol=1e-10)


def test_lex_and_zebra_agree(oracle):
    nr, np_ = 32, 64
    dr, dp = 1.0 / nr, 2.0 / np_
    rng = np.random.default_rng(4)
    rhs = np.asfortranarray(rng.standard_normal((nr + 2, np_ + 1)))
    out = []
    for mode in (0, 1):
        psi = np.zeros((nr + 2, np_ + 1), order="F")
        psip = np.zeros_like(psi)
        st, sw = oracle.poisson(2, psi, psip, rhs.copy(order="F"), nr, np_, dr, dp, mode=mode, tolcon=1e-11)
        assert st == 0
        out.append(psi)
    assert np.max(np.abs(out[0] - out[1])) < 1e-10 * np.max(np.abs(out[0]))


def test_poisson_level_count(oracle):
    """poissoninit's level rule (PRB:1744-1767): halvings of nr while even
    and >= 4, capped at 4; odd nr has no level and is rejected."""
    import ctypes as C
    for nr, want in ((4, 1), (8, 2), (16, 3), (32, 4), (64, 4), (96, 4), (272, 4), (12, 2), (6, 1)):
        mg = oracle.MG()
        assert oracle.lib().orc_mg_init(C.byref(mg), nr, 64, 0.1, 0.1) == 0
        assert mg.nlev == want, (nr, mg.nlev)
        oracle.lib().orc_mg_free(C.byref(mg))
    mg = oracle.MG()
    assert oracle.lib().orc_mg_init(C.byref(mg), 7, 64, 0.1, 0.1) == 5


def test_heat_conduction_nusselt(oracle):
    """heat (PRB:1452-1500) on the linear conduction profile gives Nu = 1 at
    the lower wall and -1 at the upper one, to the ~1e-7 the truncated
    decimal coefficients of the five-point formula allow (their sum is
    1e-8, not 0, so the error grows with 1/dr)."""
    import ctypes as C
    for nr, np_ in ((16, 32), (64, 128)):
        o = oracle.OraclePRB(nr, np_, 1e-5, 0.0, 1.0, r0=0.0, rmax=1.0, xx=2.0)
        o.initial(1, 0, 0.0)
        t1, t2 = C.c_double(), C.c_double()
        oracle.lib().orc_heat(C.byref(o.s), C.byref(t1), C.byref(t2))
        nu1 = t1.value * (o.s.rmax - o.s.r0) / o.s.xx
        nu2 = t2.value * (o.s.rmax - o.s.r0) / o.s.xx
        assert abs(nu1 - 1.0) < 1e-6 and abs(nu2 + 1.0) < 1e-6, (nu1, nu2)


def test_step_invariants(oracle):
    """A few steps of the layer: walls keep T = 0 / 1, the velocity walls are
    zero, nothing is clamped, and the seam column k = np equals k = 0 for the
    fields the periodic derivatives produce."""
    o = oracle.OraclePRB(32, 64, 1e-5, 1e5, 1.0, r0=0.0, rmax=1.0, xx=2.0, tolcon=1e-10)
    o.initial(1, 2, 1e-3)
    for _ in range(5):
        st, nu, sw = o.step()
        assert st == 0 and np.all(sw >= 1)
    th, vel, uel = (np.array(o.field(n)) for n in ("th", "vel", "uel"))
    nr = 32
    assert np.all(th[0] == 0.0) and np.all(th[nr + 1] == 1.0)
    assert np.all(vel[0] == 0.0) and np.all(vel[nr + 1] == 0.0)
    assert np.all(uel[0] == 0.0) and np.all(uel[nr] == 0.0)
    assert o.s.clamp_count == 0
    assert 0.99 < nu[0] < 1.05


def test_maxsweeps_returns_status(oracle):
    nr, np_ = 16, 32
    rng = np.random.default_rng(1)
    rhs = np.asfortranarray(rng.standard_normal((nr + 2, np_ + 1)))
    psi = np.zeros((nr + 2, np_ + 1), order="F")
    psip = np.zeros_like(psi)
    st, sw = oracle.poisson(2, psi, psip, rhs, nr, np_, 1 / nr, 2 / np_, tolcon=1e-30, maxsweeps=4)
    assert st == 1 and sw == 4
    assert np.all(psi == 0)


def test_batch_oracle_second_order(oracle):
    errs = []
    for n in (33, 65, 129):
        x = np.linspace(0, 1, n)
        X, Y = np.meshgrid(x, x)
        ex = np.sin(np.pi * X) * np.sin(2 * np.pi * Y)
        f = -5 * np.pi ** 2 * ex
        st, psi, cyc, rr = oracle.batch_solve([n], f.ravel())
        assert st == 0 and rr[0] <= 1e-10
        errs.append(np.max(np.abs(psi.reshape(n, n) - ex)))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(rates > 1.9), rates


def test_batch_oracle_mixed_matches_fp64(oracle):
    rng = np.random.default_rng(3)
    sizes = [65, 129, 33]
    f = rng.standard_normal(sum(n * n for n in sizes))
    _, p64, c64, r64 = oracle.batch_solve(sizes, f, precision=0)
    _, pmx, cmx, rmx = oracle.batch_solve(sizes, f, precision=1)
    assert np.all(r64 <= 1e-10) and np.all(rmx <= 1e-10)
    assert np.linalg.norm(pmx - p64) / np.linalg.norm(p64) < 1e-9
    assert np.all(np.abs(cmx - c64) <= 2)
