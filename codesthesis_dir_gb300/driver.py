"""The PRB main program (velvor2dperiodicrbconv.f:1-577) on the device:
reads an unchanged input deck, sets the reference's initial state or reads
its restart files, runs the time loop through the device-resident context
(CUDA-graph steps), and writes the reference's output files.

Usage:  python -m codesthesis_dir_gb300.driver < input.s  [--xx 3] [--smoother lex|zebra]

Block structure as in the reference: the first block runs steps kt = 1..nts
(kt = 1 is the forward step); every "more iterations" block runs kt = 2..nts
and advances the step counter ntot by nts, so httrans(ntot+1) of each later
block stays zero (PRB:357-571).  The time loop's diagnostics run on the
device: zmtmtempvar.dat is written after every block (PRB:474-493) and the
CFL maxima are logged as the reference prints them (PRB:390-459).
"""
from __future__ import annotations

import argparse
import math
import os
import sys

import numpy as np

from . import fortio
from . import lib as _L
from .deck import parse_prb_deck
from .prb import PRB


def reference_initial(nr, np_, r0, rmax, dr):
    """PRB:137-186: T = 2 (r - r0) plus the deterministic sine ripple whose
    0.01 is a REAL*4 literal; walls T = 0 at i = 0 and 1 at i = nr+1; every
    other field zero.  (The Gaussian blobs of PRB:193-227 have amplitude
    -0.0 and leave T unchanged.)"""
    ld = nr + 2
    th = np.zeros((ld, np_ + 1), order="F")
    i = np.arange(nr + 2)
    r = np.where(i == 0, r0, np.where(i == nr + 1, rmax, r0 + (i - 0.5) * dr))
    # libm's sin per element, as the Fortran runtime calls it
    randno = 0.5 + 0.5 * np.array([math.sin(float(k) / float(np_)) for k in range(np_ + 1)])
    f001 = float(np.float32(0.01))
    base = 2.0 * (r - r0)
    th[:, :] = base[:, None] + ((r - r0) / rmax * f001)[:, None] * ((randno * 2.0) - 1.0)[None, :]
    th[0, :] = 0.0
    th[nr + 1, :] = 1.0
    return th


def run(deck_text, xx=3.0, smoother=_L.SMOOTHER_LEX, outdir=".", tolcon=2e-6, log=print):
    d = parse_prb_deck(deck_text)
    nr, np_ = d.nr, d.np
    dr = (d.rmax - d.r0) / nr
    g = PRB(nr, np_, dt=d.dt, r0=d.r0, rmax=d.rmax, xx=xx, Ra=d.Ra, Pr=d.Pr, tolcon=tolcon, smoother=smoother)
    ld = nr + 2
    zero = np.zeros((ld, np_ + 1), order="F")
    fields = {n: zero.copy() for n in _L.FIELDS}
    fields["th"] = reference_initial(nr, np_, d.r0, d.rmax, dr)
    if d.restart:
        for name, fn in zip(fortio.RESTART_ORDER, d.restart):
            fields[name] = fortio.read_field(os.path.join(outdir, fn), nr + fortio.RESTART_ROWS[name], np_, ld)
    fields["Ap"], fields["Bp"], fields["Cp"] = fields["A"].copy(), fields["B"].copy(), fields["C"].copy()
    fields["thp"], fields["uelp"], fields["velp"] = fields["th"].copy(), fields["uel"].copy(), fields["vel"].copy()
    for n, a in fields.items():
        g.set(n, a)
    g.diagnostics(True)
    httrans, httrans2 = [], []
    ntot = 0
    blocks = [d.nts] + list(d.more)
    for b, nts in enumerate(blocks):
        if b == 0:
            nu, sw = g.step(nts)
            kt0 = 1
            httrans += list(nu[:, 0])
            httrans2 += list(nu[:, 1])
        else:
            httrans += [0.0]
            httrans2 += [0.0]
            kt0 = 2
            nu = np.zeros((0, 2))
            if nts >= 2:
                g.new_block()
                nu, sw = g.step(nts - 1)
                httrans += list(nu[:, 0])
                httrans2 += list(nu[:, 1])
        # the time loop's prints (PRB:390-395, 432-434, 456-458): every 50th
        # step the Nusselt numbers and the CFL maxima of the step before
        cfl = g.cfl(len(nu))
        for s_ in range(len(nu)):
            kt = kt0 + s_
            if kt >= 2 and cfl[s_, 0] > 1.0:
                log("WARNING! CFLU EXCEEDED!")
            if kt >= 2 and cfl[s_, 1] > 1.0:
                log("WARNING! CFLV EXCEEDED!")
            if kt % 50 == 0:
                log("%r %r %d" % (nu[s_, 0], nu[s_, 1], ntot + kt))
                log("CFLMAXU= %r" % cfl[s_ - 1, 0])   # kt >= 50: s_ >= 48
                log("CFLMAXV= %r" % cfl[s_ - 1, 1])
        ntot += nts
        fortio.write_zmtm(os.path.join(outdir, "zmtmtempvar.dat"), g.zonal())
        log("block %d: %d steps, Nu = %.8f %.8f" % (b + 1, ntot, httrans[-1], httrans2[-1]))
        # restart / output files (PRB:500-549) and the Nusselt history (PRB:551-560)
        for name, fn in zip(fortio.RESTART_ORDER, d.fnames[:7]):
            fortio.write_field(os.path.join(outdir, fn), g.get(name), nr + fortio.RESTART_ROWS[name], np_)
        if d.fnames[7] != "no":
            fortio.write_nu_history(os.path.join(outdir, d.fnames[7]), d.dt, httrans)
    return g, np.array(httrans), np.array(httrans2)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--xx", type=float, default=3.0, help="box width (the reference hard-codes 3)")
    ap.add_argument("--smoother", default="lex", choices=["lex", "zebra"])
    ap.add_argument("--tolcon", type=float, default=2e-6)
    ap.add_argument("--outdir", default=".")
    a = ap.parse_args(argv)
    run(sys.stdin.read(), xx=a.xx, smoother=_L.SMOOTHER_LEX if a.smoother == "lex" else _L.SMOOTHER_ZEBRA,
        outdir=a.outdir, tolcon=a.tolcon)


if __name__ == "__main__":
    main()
