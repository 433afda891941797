"""Regenerates the golden fixtures of tests/golden/ from the CPU oracle.

These fixtures pin the oracle (and through it the device path) against
regressions; they are the oracle's outputs.  The reference's own outputs,
from its Fortran run through the translator f77.py, are the ref_*.npz
fixtures that make_reference_golden.py writes.  Run from the repository root:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

FIELDS = ["A", "B", "An", "Bn", "Ap", "Cn", "C", "Cp", "thn", "th", "thp", "uel", "vel", "uelp", "velp",
          "urh", "vrh"]


def prb_case(name, nr, np_, dt, Ra, Pr, r0, rmax, xx, mode, tol, kind, seed, amp, nsteps):
    o = O.OraclePRB(nr, np_, dt, Ra, Pr, r0=r0, rmax=rmax, xx=xx, mode=mode, tolcon=tol)
    o.initial(kind, seed, amp)
    init = {"init_" + f: np.array(o.field(f)) for f in O._PRB_FIELDS}
    nu, sw = [], []
    for _ in range(nsteps):
        st, n, s = o.step()
        assert st == 0
        nu.append(n.copy())
        sw.append(s.copy())
    out = {f: np.array(o.field(f)) for f in FIELDS}
    params = np.array([nr, np_, dt, Ra, Pr, r0, rmax, xx, mode, tol, kind, seed, amp, nsteps], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, name), params=params, nu=np.array(nu), sweeps=np.array(sw),
                        **init, **out)


def batch_case(name, sizes, seed, precision, inner):
    rng = np.random.default_rng(seed)
    f = np.concatenate([rng.standard_normal(n * n) for n in sizes])
    st, psi, cyc, rr = O.batch_solve(sizes, f, precision=precision, inner=inner)
    assert st == 0
    np.savez_compressed(os.path.join(HERE, name), sizes=np.array(sizes, dtype=np.int32), f=f, psi=psi,
                        cycles=cyc, relres=rr, precision=precision, inner=inner)


def banded_case(name, seed):
    rng = np.random.default_rng(seed)
    n = 11
    a, b, c, d, e, r = (rng.standard_normal(n) for _ in range(6))
    b5, c8 = b + 6.0, c + 8.0
    np.savez_compressed(os.path.join(HERE, name), a=a, b=b5, c=c, r=r, d=d, e=e, c8=c8, bp=b,
                        tdma=O.tdma(a, b5, c, r), ptdma=O.ptdma(a, b5, c, r), pdma=O.pdma(a, b, c8, d, e, r))


if __name__ == "__main__":
    O.build()
    prb_case("prb_layer_16x32_lex.npz", 16, 32, 1e-4, 1e5, 1.0, 0.0, 1.0, 2.0, 0, 2e-6, 1, 3, 1e-2, 6)
    prb_case("prb_layer_16x32_zebra.npz", 16, 32, 1e-4, 1e5, 1.0, 0.0, 1.0, 2.0, 1, 1e-10, 1, 5, 1e-2, 6)
    prb_case("prb_refinit_16x48_lex.npz", 16, 48, 1e-5, 1e7, 0.71, 0.5, 1.0, 3.0, 0, 2e-6, 0, 0, 0.0, 4)
    batch_case("batch_fp64.npz", [33, 17, 65, 9, 3], 11, 0, 1)
    batch_case("batch_mixed_inner3.npz", [33, 17, 65, 9, 129], 12, 1, 3)
    banded_case("banded.npz", 13)
    print("fixtures written to", HERE)
