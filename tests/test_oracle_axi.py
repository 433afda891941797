"""The oracle's axisymmetric annulus (rotann2.f) checked by invariants of its
own, on the CPU:

* the streamfunction multigrid solves psi_rr + psi_r / r - psi / r^2 +
  psi_zz = f (the residual of relax, rotann2.f:727-741) to second order:
  a manufactured solution's error falls ~4x per grid halving;
* the conduction profile 1 - ln(r/rmax)/ln(r0/rmax) with no flow stays put
  and carries the reference's Nusselt number -r0 ln(r0/rmax) trans /
  (zmax rmax) = 1/rmax (rotann2.f:155);
* the two line orderings converge to the same solution;
* corser clears row j = n1 of the coarse level (n1 in both directions,
  rotann2.f:787-798): with nr < nz that row is interior and its coarse
  right-hand side is zero;
* the Arakawa Jacobian (rotann2.f:432-459) is antisymmetric, conserves the
  mean and both fields' squares over the interior, and is second order."""
import ctypes as C
import math

import numpy as np
import pytest


def _solve(oracle, nr, nz, mode=0, tol=1e-11):
    r0, rmax, zmax = 0.5, 1.0, 0.5
    a = oracle.OracleAXI(nr, nz, 1e-5, r0, rmax, zmax, 1e5, 1e2, 1.0, mode=mode, tolcon=tol, maxsweeps=500)
    D = rmax - r0
    r = r0 + np.arange(nr + 1) * (D / nr)
    z = np.arange(nz + 1) * (zmax / nz)
    R, Z = np.meshgrid(r, z, indexing="ij")
    k, m = math.pi / D, math.pi / zmax
    S, Cs, Sz = np.sin(k * (R - r0)), np.cos(k * (R - r0)), np.sin(m * Z)
    exact = S * Sz
    f = (-(k ** 2) * S + k * Cs / R - S / R ** 2 - m ** 2 * S) * Sz
    a.field("omegn")[:, :] = f
    a.field("phi")[:, :] = 0.0
    sw = C.c_int()
    st = oracle.lib().orc_axi_poisson(C.byref(a.s), a.s.phi, a.s.omegn, C.byref(sw))
    return a, st, sw.value, exact


def test_poisson_second_order(oracle):
    errs = []
    for n in (16, 32):
        a, st, sw, exact = _solve(oracle, n, n)
        assert st == 0, sw
        errs.append(np.max(np.abs(np.array(a.field("phi")) - exact)))
        a.close()
    assert errs[1] < 2e-3 and errs[0] / errs[1] > 3.5, errs


def test_orderings_agree(oracle):
    # 1e-11: above the FP64 rounding floor of the residual (~3e-12 here)
    a, st, _, _ = _solve(oracle, 32, 16, mode=0, tol=1e-11)
    b, st2, _, _ = _solve(oracle, 32, 16, mode=1, tol=1e-11)
    assert st == 0 and st2 == 0
    pa, pb = np.array(a.field("phi")), np.array(b.field("phi"))
    assert np.max(np.abs(pa - pb)) < 1e-10 * max(1.0, np.max(np.abs(pa)))


@pytest.mark.parametrize("r0,rmax", [(0.5, 1.0), (1.0, 2.0)])
def test_conduction_nusselt(oracle, r0, rmax):
    a = oracle.OracleAXI(32, 32, 1e-6, r0, rmax, 1.0, 1e4, 1e2, 1.0)
    a.initial(1, 0, 0.0)
    th0 = np.array(a.field("theta"))
    for _ in range(3):
        st, nu, sw, conv = a.step()
        assert st == 0
        assert abs(nu - 1.0 / rmax) < 1e-3, nu
    assert np.max(np.abs(np.array(a.field("theta")) - th0)) < 1e-4


def test_corser_clears_row_n1(oracle):
    nr, nz = 16, 32
    a = oracle.OracleAXI(nr, nz, 1e-5, 0.5, 1.0, 1.0, 1e5, 1e2, 1.0)
    ld = a.s.ld
    rc = np.ctypeslib.as_array(a.s.rc, shape=(ld * (nz + 1),)).reshape(nz + 1, ld).T
    rc[:, :] = np.random.default_rng(3).standard_normal(rc.shape)
    oracle.lib().orc_axi_corser(C.byref(a.s), 1)
    n1c, n2c = a.s.n1[2], a.s.n2[2]
    fc = np.ctypeslib.as_array(a.s.f[2], shape=((n1c + 1) * (n2c + 1),)).reshape(n2c + 1, n1c + 1).T
    assert n1c < n2c
    assert np.all(fc[:, n1c] == 0.0)          # the interior row j = n1c
    assert np.all(fc[1:n1c, n1c + 1] != 0.0)  # its neighbour is a restriction


# Arakawa's Jacobian (rotann2.f:432-459; A. Arakawa, J. Comput. Phys. 1, 1966,
# the average J = (J++ + J+x + Jx+) / 3 of three second-order forms).  The
# restatement must keep the properties the published scheme has by
# construction, whatever the fields: J(a, b) = -J(b, a) (the terms pair off
# exactly, so only rounding remains); with both fields zero on the two outer
# rings of points, the interior sums of J, a J and b J vanish (discrete
# conservation of the mean, of a^2 and of b^2 under advection); and it
# approximates a_r b_z - a_z b_r to second order.

def _axi(oracle, nr, nz):
    return oracle.OracleAXI(nr, nz, 1e-5, 0.5, 1.0, 0.5, 1e5, 1e2, 1.0)


def _compact_random(rng, nr, nz):
    a = np.zeros((nr + 1, nz + 1))
    a[2:nr - 1, 2:nz - 1] = rng.standard_normal((nr - 3, nz - 3))
    return a


@pytest.mark.parametrize("nr,nz", [(16, 16), (24, 40)])
def test_arakawa_antisymmetric_and_conservative(oracle, nr, nz):
    o = _axi(oracle, nr, nz)
    rng = np.random.default_rng(nr * 100 + nz)
    a, b = _compact_random(rng, nr, nz), _compact_random(rng, nr, nz)
    jab, jba = o.arakawa(a, b), o.arakawa(b, a)
    scale = np.max(np.abs(jab))
    assert scale > 0
    np.testing.assert_allclose(jab, -jba, rtol=0, atol=1e-13 * scale)
    w = np.abs(jab).sum()
    for weight in (np.ones_like(a), a, b):
        assert abs((weight * jab).sum()) <= 1e-12 * w * max(1.0, np.max(np.abs(weight)))
    # an ordinary centred Jacobian of the same fields conserves none of them
    assert abs((a * jab).sum()) < 1e-6 * abs((a * _centred(a, b, o)).sum())
    o.close()


def _centred(a, b, o):
    hx, hy = o.s.dr, o.s.dz
    j = np.zeros_like(a)
    j[1:-1, 1:-1] = ((a[2:, 1:-1] - a[:-2, 1:-1]) * (b[1:-1, 2:] - b[1:-1, :-2]) -
                     (a[1:-1, 2:] - a[1:-1, :-2]) * (b[2:, 1:-1] - b[:-2, 1:-1])) / (4 * hx * hy)
    return j


def test_arakawa_second_order(oracle):
    errs = []
    for n in (16, 32, 64):
        o = _axi(oracle, n, n)
        r = 0.5 + np.arange(n + 1) * (0.5 / n)
        z = np.arange(n + 1) * (0.5 / n)
        R, Z = np.meshgrid(r, z, indexing="ij")
        a = np.sin(3.0 * R) * np.cos(2.0 * Z)
        b = np.cos(2.0 * R + Z)
        exact = (3.0 * np.cos(3.0 * R) * np.cos(2.0 * Z)) * (-np.sin(2.0 * R + Z)) - \
                (-2.0 * np.sin(3.0 * R) * np.sin(2.0 * Z)) * (-2.0 * np.sin(2.0 * R + Z))
        j = o.arakawa(a, b)
        errs.append(np.max(np.abs(j[1:-1, 1:-1] - exact[1:-1, 1:-1])))
        o.close()
    assert errs[0] / errs[1] > 3.5 and errs[1] / errs[2] > 3.5, errs
