"""Initial states of the 2D drivers, on the host (numpy), as the fields a
device instance is loaded with.

* ``layer_reference``: velvor2dperiodicrbconv.f:137-186, T = 2 (r - r0) with
  the deterministic sine ripple whose 0.01 is a REAL*4 literal.
* ``annulus_reference``: velvor2dnewsch3.4.f:130-178, T = 1 - ln r / ln r0
  with the ripple 0.7 T (r - rmax)/rmax (2 randno - 1), randno =
  1/2 + sin(2 pi k/150)/2.
* ``r3d_reference``: rot3dmg.f:103-131, the 3D annulus at rest with
  T = 1 - ln r / ln r0 + amp (rmax - r)(r - r0) cos(nval phi) and the point
  (nr/4, nz/4, np/2) halved; ``r3d_initial_fields`` adds the previous time
  level (rot3dmg.f:220-230) and, with noise > 0, seeded uniform noise on
  the interior temperature (splitmix64, i fastest, then j, then k).
* ``conduction_noise``: the conduction profile of either geometry plus
  seeded uniform noise of amplitude amp, drawn from splitmix64 (Steele, Lea
  and Flood, 2014) in k-major, i-minor order over the interior rows, the
  periodic column k = np a copy of k = 0.  This is the perturbed start of
  the 129 x 65 layer workload.

Transcendentals are evaluated element by element with the C library's log
and sin (``math``), as the Fortran runtime calls them, so the states are
bit-identical to the reference formulas evaluated in double precision.
"""
from __future__ import annotations

import math

import numpy as np

from . import lib as _L

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def _radii(nr, r0, rmax, dr):
    i = np.arange(nr + 2)
    return np.where(i == 0, r0, np.where(i == nr + 1, rmax, r0 + (i - 0.5) * dr))


def layer_reference(nr, np_, r0, rmax, dr):
    th = np.zeros((nr + 2, np_ + 1), order="F")
    r = _radii(nr, r0, rmax, dr)
    randno = 0.5 + 0.5 * np.array([math.sin(float(k) / float(np_)) for k in range(np_ + 1)])
    f001 = float(np.float32(0.01))
    th[:, :] = (2.0 * (r - r0))[:, None] + ((r - r0) / rmax * f001)[:, None] * ((randno * 2.0) - 1.0)[None, :]
    th[0, :] = 0.0
    th[nr + 1, :] = 1.0
    return th


def annulus_reference(nr, np_, r0, rmax, dr):
    pi = math.acos(-1.0)
    r = _radii(nr, r0, rmax, dr)
    lr0 = math.log(r0)
    t0 = np.array([1.0 - math.log(float(x)) / lr0 for x in r])
    randno = 0.5 + 0.5 * np.array([math.sin(float(k) / 150.0 * 2.0 * pi) for k in range(np_ + 1)])
    a = ((r - rmax) / rmax)[:, None] * ((randno * 2.0) - 1.0)[None, :]
    a = a * 0.7
    a = a * t0[:, None]
    th = np.asfortranarray(t0[:, None] + a)
    th[0, :] = 0.0
    th[nr + 1, :] = 1.0
    return th


def _splitmix64(seed, n):
    """The first n outputs of splitmix64 started from state seed."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + _GOLDEN * np.arange(1, n + 1, dtype=np.uint64)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def conduction_noise(nr, np_, r0, rmax, dr, seed=0, amp=1e-3, variant=_L.PRB_LAYER):
    th = np.zeros((nr + 2, np_ + 1), order="F")
    i = np.arange(1, nr + 1)
    r = r0 + (i - 0.5) * dr
    if variant == _L.PRB_ANNULUS:
        lr0 = math.log(r0)
        base = np.array([1.0 - math.log(float(x)) / lr0 for x in r])
    else:
        base = (r - r0) / (rmax - r0)
    u = (_splitmix64(seed, nr * np_) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    u = u.reshape(np_, nr).T                    # draw n = k*nr + (i-1)
    th[1:nr + 1, :np_] = base[:, None] + amp * (2.0 * u - 1.0)
    th[1:nr + 1, np_] = th[1:nr + 1, 0]
    th[nr + 1, :] = 1.0
    return th


def initial_fields(nr, np_, r0, rmax, variant=_L.PRB_LAYER, kind=1, seed=0, amp=1e-3):
    """Every field of a fresh instance: T from the chosen initial state,
    vorticity and velocity zero, the previous time level equal to the
    current one (velvor2dperiodicrbconv.f:316-331)."""
    dr = (rmax - r0) / nr
    zero = np.zeros((nr + 2, np_ + 1), order="F")
    f = {n: zero.copy() for n in _L.FIELDS}
    if kind == 0:
        f["th"] = (annulus_reference if variant == _L.PRB_ANNULUS else layer_reference)(nr, np_, r0, rmax, dr)
    else:
        f["th"] = conduction_noise(nr, np_, r0, rmax, dr, seed, amp, variant)
    f["thp"] = f["th"].copy()
    return f


def r3d_reference(nr, nz, np_, r0, rmax, nval=3, amp=1e-3, horizontal=False):
    """T of rot3dmg.f:103-131 as a Fortran-ordered (nr+2, nz+2, np+1) array;
    horizontal: rot3dmghor.f:107-141 (T = ln r / ln r0 + ..., the inner
    cylinder hot, the point (nr/2, nz/2, np/2) halved)."""
    dr = (rmax - r0) / float(nr)
    r = _radii(nr, r0, rmax, dr)
    lr0 = math.log(r0)
    at1 = math.atan(1.0)
    if horizontal:
        trad = np.array([math.log(float(x)) / lr0 for x in r])
    else:
        trad = np.array([1.0 - math.log(float(x)) / lr0 for x in r])
    ramp = np.array([amp * (rmax - float(x)) * (float(x) - r0) for x in r])
    cosk = np.array([math.cos(float(nval) * (8.0 * at1 * float(k) / float(np_))) for k in range(np_ + 1)])
    th = np.asfortranarray(np.broadcast_to((trad[:, None] + ramp[:, None] * cosk[None, :])[:, None, :],
                                           (nr + 2, nz + 2, np_ + 1)).copy())
    i, j, k = (nr // 2, nz // 2, np_ // 2) if horizontal else (nr // 4, nz // 4, np_ // 2)
    th[i, j, k] = th[i, j, k] - 0.5 * th[i, j, k]
    return np.asfortranarray(th)


def r3d_initial_fields(nr, nz, np_, r0, rmax, nval=3, amp=1e-3, noise=0.0, seed=0, horizontal=False):
    """Every field of a fresh 3D-annulus instance: velocities and vorticities
    zero (the fluid in solid-body rotation with the frame), T from
    r3d_reference plus optional seeded noise, previous levels equal to the
    current ones."""
    zero = np.zeros((nr + 2, nz + 2, np_ + 1), order="F")
    f = {n: zero.copy() for n in _L.R3D_FIELDS}
    th = r3d_reference(nr, nz, np_, r0, rmax, nval, amp, horizontal)
    if noise > 0.0:
        n = nr * nz * np_
        u = (_splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        th[1:nr + 1, 1:nz + 1, 0:np_] += noise * (2.0 * u.reshape(np_, nz, nr).T - 1.0)
        th[:, :, np_] = th[:, :, 0]
    f["th"] = th
    f["thp"] = th.copy()
    return f
