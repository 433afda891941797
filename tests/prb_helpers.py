"""Shared set-up for the PRB parity tests: the same initial state in the
oracle (oracle/) and on the device (codesthesis_dir_gb300.prb)."""
import numpy as np

STATE_FIELDS = ["An", "A", "Ap", "Bn", "B", "Bp", "Cn", "C", "Cp", "thn", "th", "thp",
                "uel", "vel", "wel", "uelp", "velp", "welp", "urh", "vrh"]
# fields a step writes (the others stay as initialised)
COMPARED = ["A", "B", "An", "Bn", "Ap", "Cn", "C", "Cp", "thn", "th", "thp", "uel", "vel", "uelp", "velp",
            "urh", "vrh"]


def config0_params(nr=64, np_=128):
    """The periodic Rayleigh-Benard layer of the 129 x 65 workload: unit
    height (r0 = 0, rmax = 1), aspect ratio 2 (xx = 2), Ra 1e5, Pr 1,
    dt 1e-5."""
    return dict(nr=nr, np_=np_, dt=1e-5, Ra=1e5, Pr=1.0, r0=0.0, rmax=1.0, xx=2.0)


def make_pair(O, P, nr, np_, dt, Ra, Pr, r0, rmax, xx, smoother, tolcon, seed=0, amp=1e-3, kind=1):
    o = O.OraclePRB(nr, np_, dt, Ra, Pr, r0=r0, rmax=rmax, xx=xx, mode=smoother, tolcon=tolcon)
    o.initial(kind, seed, amp)
    g = P.PRB(nr, np_, dt=dt, r0=r0, rmax=rmax, xx=xx, Ra=Ra, Pr=Pr, tolcon=tolcon, smoother=smoother)
    for name in STATE_FIELDS:
        g.set(name, np.array(o.field(name), order="F"))
    return o, g


def diff_fields(o, g, names=COMPARED):
    bad = {}
    for name in names:
        a = np.array(o.field(name))
        b = g.get(name)
        if not np.array_equal(a, b):
            bad[name] = float(np.max(np.abs(a - b)))
    return bad


def rel_l2(a, b):
    d = np.linalg.norm(a - b)
    n = np.linalg.norm(a)
    return d / n if n > 0 else d
