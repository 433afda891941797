"""Grids and finite-difference coefficient tables of the stretched-grid
streamfunction solver, on the host: the restatement of grid.f that rcsc.f's
coefficient file comes from.

* ``spacing_gef``: grid.f:737-790 -- a first spacing d1 growing by the
  factor gef towards the middle until the stretched part passes dist, the
  same mirrored at the far wall, a uniform core;
* ``spacing_tanh``: wall clustering by a tanh map, h_i = L (x_i - x_{i-1}),
  x_i = (1 + tanh(s (2i/n - 1)) / tanh(s)) / 2, stretch factor s (the 257^2
  annulus workload uses s = 1.5; grid.f itself has only the GEF grid);
* ``levels``: grid.f:859-924 -- coarse spacings are sums of fine pairs,
  positions their running sums, at most 6 levels;
* ``fdif``: grid.f:926-1115 -- weights of the points of a stencil for the
  derivatives 0..nx-1, by Gaussian elimination (partial pivoting) of the
  Taylor matrix, in the reference's operation order;
* ``coefficients``: grid.f:178-243 -- per level, first-derivative weights on
  (i-1, i, i+1) and second-derivative weights on (i-1..i+2) for i <= n/2 and
  on (i-2..i+1) above, in r and in z.

Pure Python floats (IEEE double, no fused multiply-add), so the tables are
the same on every host.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List

import numpy as np


def spacing_uniform(n, lo, hi):
    return [0.0] + [(hi - lo) / float(n)] * n


def spacing_gef(n, lo, hi, dist, gef, d1):
    """1-based spacings (index 0 unused); raises where grid.f STOPs."""
    h = [0.0] * (n + 1)
    h[1] = d1
    t = h[1]
    imax = -1
    for i in range(2, n // 2 + 1):
        h[i] = h[i - 1] * gef
        t = t + h[i]
        if t > dist:
            imax = i
            t = t - h[i]
            break
    if imax < 0:
        raise ValueError("too many grid points in GEF region")
    if 2 * imax - 2 > n:
        raise ValueError("grid points exceeded")
    over = hi - lo - 2.0 * t
    for i in range(imax, n - imax + 2):
        h[i] = over / float(n - 2 * imax + 2)
    for i in range(n - imax + 1, n + 1):
        h[i] = h[n - i + 1]
    return h


def spacing_tanh(n, lo, hi, s):
    x = [0.5 * (1.0 + math.tanh(s * (2.0 * i / n - 1.0)) / math.tanh(s)) for i in range(n + 1)]
    return [0.0] + [(hi - lo) * (x[i] - x[i - 1]) for i in range(1, n + 1)]


@dataclass
class Levels:
    nlev: int
    n1: List[int] = field(default_factory=list)     # index l = 1..nlev (index 0 unused)
    n2: List[int] = field(default_factory=list)
    hr: List[list] = field(default_factory=list)
    hz: List[list] = field(default_factory=list)
    r: List[list] = field(default_factory=list)
    z: List[list] = field(default_factory=list)
    cr: List[np.ndarray] = field(default_factory=list)    # (n1-1, 3), row i-1
    crr: List[np.ndarray] = field(default_factory=list)   # (n1-1, 4)
    cz: List[np.ndarray] = field(default_factory=list)
    czz: List[np.ndarray] = field(default_factory=list)


def level_count(n1, n2, cap=6):
    nlev, itest, itest2, jtest, jtest2 = 0, n1, n1, n2, n2
    for _ in range(2, 9):
        itest //= 2
        jtest //= 2
        if itest * 2 - itest2 == 0 and jtest * 2 - jtest2 == 0:
            if itest2 >= 4 and jtest2 >= 4:
                nlev += 1
            itest2, jtest2 = itest, jtest
        else:
            break
    return min(nlev, cap)


def levels(hr1, hz1, r0, zmin=0.0, maxlev=0):
    n1, n2 = len(hr1) - 1, len(hz1) - 1
    nlev = level_count(n1, n2)
    if maxlev > 0:
        nlev = min(nlev, maxlev)
    L = Levels(nlev, [0], [0], [None], [None], [None], [None], [None], [None], [None], [None])
    for l in range(1, nlev + 1):
        a, b = n1 * 2 // (1 << l), n2 * 2 // (1 << l)
        hr = [0.0] * (a + 1)
        hz = [0.0] * (b + 1)
        r = [r0] + [0.0] * a
        z = [zmin] + [0.0] * b
        for i in range(1, a + 1):
            hr[i] = float(hr1[i]) if l == 1 else L.hr[l - 1][2 * i] + L.hr[l - 1][2 * i - 1]
            r[i] = r[i - 1] + hr[i]
        for j in range(1, b + 1):
            hz[j] = float(hz1[j]) if l == 1 else L.hz[l - 1][2 * j] + L.hz[l - 1][2 * j - 1]
            z[j] = z[j - 1] + hz[j]
        L.n1.append(a)
        L.n2.append(b)
        L.hr.append(hr)
        L.hz.append(hz)
        L.r.append(r)
        L.z.append(z)
    return L


def _gausse(a, b, n):
    """grid.f:1034-1115: a[i][j] is row i, column j; b[i] the n+2
    right-hand sides of row i.  Returns x[i][k] (unknown i, right-hand side k)."""
    for k in range(n - 1):
        kpvt = k
        for i in range(k + 1, n):
            if abs(a[kpvt][k]) < abs(a[i][k]):
                kpvt = i
        if abs(a[kpvt][k]) == 0.0:
            raise ValueError("singular Taylor matrix")
        if kpvt != k:
            for j in range(k, n):
                a[k][j], a[kpvt][j] = a[kpvt][j], a[k][j]
            for j in range(n + 2):
                b[k][j], b[kpvt][j] = b[kpvt][j], b[k][j]
        for i in range(k + 1, n):
            q = -a[i][k] / a[k][k]
            a[i][k] = 0.0
            for j in range(k + 1, n):
                a[i][j] = a[i][j] + q * a[k][j]
            for j in range(n + 2):
                b[i][j] = b[i][j] + q * b[k][j]
    x = [[0.0] * (n + 2) for _ in range(n)]
    for j in range(n + 2):
        x[n - 1][j] = b[n - 1][j] / a[n - 1][n - 1]
    for i in range(n - 2, -1, -1):
        for k in range(n + 2):
            s = 0.0
            for j in range(i + 1, n):
                s = s + a[i][j] * x[j][k]
            x[i][k] = (b[i][k] - s) / a[i][i]
    return x


def fdif(nx, nref, k, pos):
    """grid.f:926-1032 (nans = 0): w[d][p] = weight of point pos[k-nref+1+p]
    for the d-th derivative.  nref is 1-based, as in the reference."""
    x = [float(pos[k - nref + i]) for i in range(1, nx + 1)]
    # equation (row) i: the Taylor expansion about point nref at point i
    a = [[0.0] * nx for _ in range(nx)]
    b = [[0.0] * (nx + 2) for _ in range(nx)]
    for j in range(nx):
        temp = 1.0
        h = x[j] - x[nref - 1]
        a[j][0] = 1.0
        for i in range(2, nx + 3):
            if j == nref - 1:
                temp = 0.0
            else:
                temp = temp * h / float(i - 1)
            if i <= nx:
                a[j][i - 1] = temp
            else:
                b[j][i - 1] = -temp
    for j in range(nx):
        b[j][j] = 1.0
    x_ = _gausse(a, b, nx)
    return [[x_[d][p] for p in range(nx)] for d in range(nx)]


def coefficients(L):
    for l in range(1, L.nlev + 1):
        n1, n2 = L.n1[l], L.n2[l]
        cr = np.zeros((max(n1 - 1, 0), 3))
        crr = np.zeros((max(n1 - 1, 0), 4))
        for i in range(1, n1):
            cr[i - 1] = fdif(3, 2, i, L.r[l])[1]
            crr[i - 1] = fdif(4, 2 if i <= n1 // 2 else 3, i, L.r[l])[2]
        cz = np.zeros((max(n2 - 1, 0), 3))
        czz = np.zeros((max(n2 - 1, 0), 4))
        for j in range(1, n2):
            cz[j - 1] = fdif(3, 2, j, L.z[l])[1]
            czz[j - 1] = fdif(4, 2 if j <= n2 // 2 else 3, j, L.z[l])[2]
        L.cr.append(cr)
        L.crr.append(crr)
        L.cz.append(cz)
        L.czz.append(czz)
    return L


def build(hr1, hz1, r0, zmin=0.0, maxlev=0):
    """levels + coefficients for level-1 spacings (1-based lists)."""
    return coefficients(levels(hr1, hz1, r0, zmin, maxlev))
