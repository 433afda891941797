"""The 3D annulus main program (rot3dmg.f:1-330) on the device: reads an
unchanged input deck, sets the reference's initial state (rest, mode-nval
temperature ripple, the halved point) or reads its restart files, runs the
time loop through the device-resident context, and writes the reference's
output files (fields with their header records, the Nusselt history).

Usage:  python -m codesthesis_dir_gb300.driver_r3d < input  [--smoother lex|zebra] [--precision fp64|mixed]
                                                           [--horizontal]

--horizontal runs rot3dmghor.f (the same deck): the annulus with its axis
horizontal, its own start (inner cylinder hot, the point (nr/2, nz/2,
np/2) halved) and the three-column Nusselt history of both cylinders.

Every block of the reference's loop runs kt = 1..nts and appends httrans for
each step (rot3dmg.f:237-268); the files are written once, after the last
block (rot3dmg.f:270-326).  A solve beyond the sweep limit ends the run
(the reference STOPs): the files are not written and GBError is raised.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

from . import fortio
from . import initial
from . import lib as _L
from .deck import parse_r3d_deck
from .r3d import R3D


def run(deck_text, smoother=_L.SMOOTHER_LEX, precision=_L.PRB_FP64, outdir=".", log=print, horizontal=False):
    d = parse_r3d_deck(deck_text)
    nr, nz, np_, r0, rmax, zmax = d.nr, d.nz, d.np, d.r0, d.rmax, d.zmax
    fields = initial.r3d_initial_fields(nr, nz, np_, r0, rmax, d.nval, d.amp, horizontal=horizontal)
    zmin = 0.0
    if d.restart:
        for name, fn in zip(fortio.R3D_ORDER, d.restart):
            dims, (rmax, r0, zmax, zmin), arr = fortio.read_r3d_field(os.path.join(outdir, fn), name)
            if dims != (nr, nz, np_):
                raise ValueError("%s is a %d x %d x %d field; the deck says %d x %d x %d" % ((fn,) + dims +
                                                                                           (nr, nz, np_)))
            fields[name] = arr
        # the previous time level is the current one (rot3dmg.f:220-230)
        for a, b in (("Ap", "A"), ("Bp", "B"), ("Cp", "C"), ("thp", "th"), ("uelp", "uel"), ("velp", "vel"),
                     ("welp", "wel")):
            fields[a] = fields[b].copy()
    g = R3D(nr, nz, np_, dt=d.dt, r0=r0, rmax=rmax, zmax=zmax, Ra=d.Ra, Re=d.Re, Pr=d.Pr, Gr=d.Gr,
            smoother=smoother, precision=precision,
            variant=_L.R3D_HORIZONTAL if horizontal else _L.R3D_VERTICAL)
    for n, a in fields.items():
        g.set(n, a)
    httrans, httrans2 = [], []
    for b, nts in enumerate([d.nts] + list(d.more)):
        nu, sw = g.step(nts)
        httrans += list(nu)
        httrans2 += list(g.nu2)
        log("block %d: %d steps, Nu = %.8f, sweeps (w v u) %s" % (b + 1, len(httrans), httrans[-1], list(sw[-1])))
    for name, fn in zip(fortio.R3D_ORDER, d.fnames[:7]):
        fortio.write_r3d_field(os.path.join(outdir, fn), g.get(name), name, nr, nz, np_, rmax, r0, zmax, zmin)
    if d.fnames[7] != "no":
        fortio.write_r3d_nu_history(os.path.join(outdir, d.fnames[7]), d.dt, httrans,
                                    httrans2 if horizontal else None)
    return g, np.array(httrans)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--smoother", default="lex", choices=["lex", "zebra"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--outdir", default=".")
    ap.add_argument("--horizontal", action="store_true", help="rot3dmghor.f: the annulus with its axis horizontal")
    a = ap.parse_args(argv)
    run(sys.stdin.read(), smoother=_L.SMOOTHER_LEX if a.smoother == "lex" else _L.SMOOTHER_ZEBRA,
        precision=_L.PRB_FP64 if a.precision == "fp64" else _L.PRB_MIXED, outdir=a.outdir,
        horizontal=a.horizontal)


if __name__ == "__main__":
    main()
