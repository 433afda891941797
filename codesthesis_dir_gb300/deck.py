"""Input decks of the PRB driver (velvor2dperiodicrbconv.f:78-120, 253-312,
565-571) and of the 3D annulus driver (rot3dmg.f:43-88, 153-216, 262-268),
read the way Fortran list-directed input reads them: every read*
starts a new record (line), values are separated by blanks or commas, a
record may be continued on the next line until the read is satisfied, and
REAL*8 values may use a 'd' exponent (1.d-7).  Strings are unquoted words.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from typing import List, Optional


def _tokens(line: str):
    return [t for t in re.split(r"[,\s]+", line.strip()) if t != ""]


def fortran_float(tok: str) -> float:
    return float(tok.lower().replace("d", "e"))


class ListDirected:
    """A stream of records answering successive read* statements."""

    def __init__(self, text: str):
        self.lines = text.splitlines()
        self.pos = 0

    def read(self, n: int) -> List[str]:
        out: List[str] = []
        while len(out) < n:
            if self.pos >= len(self.lines):
                raise EOFError("input deck ended while reading %d value(s)" % n)
            toks = _tokens(self.lines[self.pos])
            self.pos += 1
            out += toks[: n - len(out)]
        return out

    def eof(self) -> bool:
        return all(not _tokens(l) for l in self.lines[self.pos:])


@dataclass
class PrbDeck:
    fnames: List[str]               # fname1..fname8: A, B, C, u, v, w, T, Nu history
    dt: float
    nr: int
    np: int
    nts: int
    r0: float
    rmax: float
    zmax: float
    Ra: float
    Re: float
    Gr: float
    Pr: float
    pert: float
    amp: float
    nval: int
    restart: Optional[List[str]]    # 7 input files, or None for 'no'
    more: List[int] = field(default_factory=list)  # nts of each "more iterations" block

    @property
    def total_steps(self) -> int:
        return self.nts + sum(self.more)


def parse_prb_deck(text: str) -> PrbDeck:
    r = ListDirected(text)
    fnames = [r.read(1)[0] for _ in range(8)]
    dt = fortran_float(r.read(1)[0])
    nr = int(r.read(1)[0])
    np_ = int(r.read(1)[0])
    nts = int(r.read(1)[0])
    r0, rmax, zmax = (fortran_float(t) for t in r.read(3))
    Ra = fortran_float(r.read(1)[0])
    Re = fortran_float(r.read(1)[0])
    Gr = fortran_float(r.read(1)[0])
    Pr = fortran_float(r.read(1)[0])
    pert = fortran_float(r.read(1)[0])
    amp = fortran_float(r.read(1)[0])
    nval = int(r.read(1)[0])
    ans = r.read(1)[0]
    restart = None
    if ans != "no":
        restart = [r.read(1)[0] for _ in range(7)]
    more = []
    while not r.eof():
        ans = r.read(1)[0]
        if ans in ("n", "no"):
            break
        more.append(int(r.read(1)[0]))
    return PrbDeck(fnames, dt, nr, np_, nts, r0, rmax, zmax, Ra, Re, Gr, Pr, pert, amp, nval, restart, more)


@dataclass
class R3dDeck:
    fnames: List[str]               # fname1..fname8: A, B, C, u, v, w, T, heat transfer data (or "no")
    dt: float
    nr: int
    nz: int
    np: int
    nts: int
    r0: float
    rmax: float
    zmax: float
    Ra: float
    Re: float
    Gr: float
    Pr: float
    pert: float
    amp: float
    nval: int
    restart: Optional[List[str]]    # 7 input files (A, B, C, u, v, w, T), or None for 'no'
    more: List[int] = field(default_factory=list)

    @property
    def total_steps(self) -> int:
        return self.nts + sum(self.more)


def parse_r3d_deck(text: str) -> R3dDeck:
    """rot3dmg.f:43-88 (file names, dt, nr, nz, np, nts, r0 rmax zmax, Ra, Re,
    Gr, Ptl, pert, amp, nval), :153 (initial conditions from file), :262-268
    (more iterations)."""
    r = ListDirected(text)
    fnames = [r.read(1)[0] for _ in range(8)]
    dt = fortran_float(r.read(1)[0])
    nr = int(r.read(1)[0])
    nz = int(r.read(1)[0])
    np_ = int(r.read(1)[0])
    nts = int(r.read(1)[0])
    r0, rmax, zmax = (fortran_float(t) for t in r.read(3))
    Ra = fortran_float(r.read(1)[0])
    Re = fortran_float(r.read(1)[0])
    Gr = fortran_float(r.read(1)[0])
    Pr = fortran_float(r.read(1)[0])
    pert = fortran_float(r.read(1)[0])
    amp = fortran_float(r.read(1)[0])
    nval = int(r.read(1)[0])
    ans = r.read(1)[0]
    restart = None
    if ans != "no":
        restart = [r.read(1)[0] for _ in range(7)]
    more = []
    while not r.eof():
        ans = r.read(1)[0]
        if ans in ("n", "no"):
            break
        more.append(int(r.read(1)[0]))
    return R3dDeck(fnames, dt, nr, nz, np_, nts, r0, rmax, zmax, Ra, Re, Gr, Pr, pert, amp, nval, restart, more)
