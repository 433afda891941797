"""Writes the reference-run fixtures tests/golden/ref_*.npz: the reference's
own Fortran drivers run on the CPU through the translator in f77.py (the
image has no Fortran compiler), each on a small deck.  tests/
test_reference_runs.py checks the oracle against them bit for bit, which
pins the oracle (and, through the device parity tests, the device path) to
the reference's own source.

Reads the reference source tree (GB300_REFERENCE_SOURCE, default
/root/reference).  Run from the repository root:
    python tests/golden/make_reference_golden.py [driver ...]
(all drivers, or only those named: layer oblique annulus tank dvd taycou
layer_routines r3d r3d_hor axi transfer grid_rcsc).
Each fixture holds the deck, the driver, the parameters the oracle needs, the
source file's path and SHA-256, the final fields, the Nusselt history and
the sweep count of every multigrid solve.
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import reference_runs as RR  # noqa: E402

# the drivers' own box lengths (hard-coded in each main program) and the
# oracle variant that restates each driver
XX = {"layer": 3.0, "oblique": 3.0, "annulus": 0.0, "taycou": 0.0, "tank": 3.1, "dvd": 1.0}
VARIANT = {"layer": 0, "annulus": 1, "oblique": 2, "taycou": 3, "tank": 4, "dvd": 5}

CASES_2D = [
    # driver, nr, np, steps, dt, r0, rmax, Ra, Re, Gr(Ta), Pr
    ("layer", 16, 48, 4, 1e-5, 0.5, 1.0, 1e7, 0.0, 0.0, 0.71),
    ("layer", 32, 64, 6, 1e-5, 0.5, 1.0, 1e6, 0.0, 0.0, 1.0),
    ("oblique", 16, 32, 4, 1e-5, 0.5, 1.0, 1e6, 0.0, 0.0, 0.71),
    ("annulus", 16, 32, 4, 1e-6, 0.5, 1.0, 1e6, 1e4, 0.0, 0.71),
    ("tank", 16, 32, 4, 1e-6, 0.5, 1.5, 1e6, 0.0, 0.0, 10.0),
    ("dvd", 16, 32, 4, 2e-5, 0.0, 1.0, 1e5, 0.0, 0.0, 0.71),
    ("taycou", 16, 32, 4, 1e-6, 0.5, 1.0, 1e6, 1e4, 1e4, 0.71),
]
# the input decks shipped beside each driver (input.s: dt, nr, np, r0 rmax,
# Ra, Re, Gr, Ptl), run for a few steps
DECKS_2D = [
    ("layer", 96, 336, 3, 1e-7, 0.5, 1.0, 1e7, 0.0, 0.0, 0.71),
    ("tank", 128, 128, 3, 5e-8, 0.5, 1.5, 8.63e7, 0.0, 0.0, 10.0),
    ("dvd", 96, 96, 3, 2e-6, 0.0, 1.0, 1e6, 0.0, 0.0, 0.71),
    ("annulus", 272, 1200, 1, 2e-8, 0.5, 1.0, 8e8, 1.06148e5, 0.0, 0.71),
]
CASES_3D = [
    # driver, nr, nz, np, steps, dt, r0, rmax, zmax, Ra, Re, Gr, Pr, amp, nval
    ("r3d", 8, 8, 16, 2, 1e-5, 0.5, 1.0, 0.5, 1e5, 100.0, 0.0, 0.7, 1e-2, 3),
    ("r3d", 16, 16, 32, 2, 1e-5, 0.5, 1.0, 0.5, 1e6, 500.0, 0.0, 7.0, 1e-3, 3),
    ("r3d_hor", 8, 8, 16, 2, 1e-5, 0.5, 1.0, 0.5, 0.0, 0.0, 1e4, 7.0, 1e-2, 3),
]
CASES_AXI = [
    # nr, nz, steps, dt, r0, rmax, zmax, Ra, Re, Pr
    (16, 16, 5, 1e-5, 0.5, 1.0, 0.5, 1e5, 1e2, 1.0),
    (32, 64, 5, 1e-6, 0.5, 1.0, 1.0, 1e6, 1e2, 1.0),
    (128, 128, 3, 1e-6, 0.5, 1.0, 0.5, 1e6, 1e2, 1.0),   # rotann2.f's largest grid (nrmax = 128)
    (8, 8, 400, 1e-3, 0.5, 1.0, 0.5, 0.0, 1.0, 1.0),      # runs to the steady-state stop (:191-194)
]
# the 3D annulus at half the benchmark's grid in each direction (one step;
# the translated program needs about five minutes for it)
LARGE_3D = [("r3d", 32, 32, 64, 1, 1e-5, 0.5, 1.0, 0.5, 1e6, 500.0, 0.0, 7.0, 1e-3, 3)]


def field_digest(a):
    """SHA-256 of a field's binary64 values in C order (large runs keep
    digests, not the fields)."""
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def save(name, res, meta, extra=None, digests=False):
    meta = dict(meta, source=res["source"], sha256=res["sha256"], end=res["end"], deck=res.get("deck"))
    if digests:
        arrays = {"h_" + k: np.array(field_digest(v)) for k, v in res["fields"].items()}
    else:
        arrays = {"f_" + k: v for k, v in res["fields"].items()}
    arrays.update(extra or {})
    np.savez_compressed(os.path.join(HERE, name), meta=np.array(json.dumps(meta)), nu=res["nu"],
                        sweeps=res["sweeps"], **arrays)
    print("%-34s %-10s end=%-9s nu[-1]=%s sweeps[-1]=%s" % (name, meta["driver"], res["end"], res["nu"][-1],
                                                            res["sweeps"][-1]), flush=True)


def main(only=()):
    """only: driver names to regenerate (all when empty)."""
    from oracle import oracle as O
    O.build()
    t0 = time.time()

    def want(drv):
        return not only or drv in only
    for drv, nr, np_, nts, dt, r0, rmax, Ra, Re, Gr, Pr in CASES_2D:
        if not want(drv):
            continue
        res = RR.run_2d(drv, nr, np_, nts, dt=dt, r0=r0, rmax=rmax, Ra=Ra, Re=Re, Gr=Gr, Pr=Pr)
        meta = dict(driver=drv, variant=VARIANT[drv], nr=nr, np=np_, steps=nts, dt=dt, r0=r0, rmax=rmax, Ra=Ra,
                    Re=Re, Gr=Gr, Pr=Pr, xx=XX[drv])
        save("ref_%s_%dx%d.npz" % (drv, nr, np_), res, meta)
    # the decks the reference ships (its own grids, time steps and numbers;
    # a few steps), fields kept as digests
    for drv, nr, np_, nts, dt, r0, rmax, Ra, Re, Gr, Pr in DECKS_2D:
        if not want(drv):
            continue
        res = RR.run_2d(drv, nr, np_, nts, dt=dt, r0=r0, rmax=rmax, Ra=Ra, Re=Re, Gr=Gr, Pr=Pr)
        meta = dict(driver=drv, variant=VARIANT[drv], nr=nr, np=np_, steps=nts, dt=dt, r0=r0, rmax=rmax, Ra=Ra,
                    Re=Re, Gr=Gr, Pr=Pr, xx=XX[drv], deck_of="input.s")
        save("ref_%s_deck_%dx%d.npz" % (drv, nr, np_), res, meta, digests=True)
    # the Taylor-Couette driver as written STOPs in its first v solve (its
    # relax2 forms a line's right-hand side only for k = 1); the same
    # program with relax2 taken from velvor2dtaycouheat_new.f, which forms
    # every line's, is what the oracle restates
    drv, nr, np_, nts, dt, r0, rmax, Ra, Re, Gr, Pr = CASES_2D[-1]
    rep = {"relax2": "monashubuntudir_velvor2dtaycouheatdir/velvor2dtaycouheat_new.f"}
    if want(drv):
        res = RR.run_2d(drv, nr, np_, nts, replace=rep, dt=dt, r0=r0, rmax=rmax, Ra=Ra, Re=Re, Gr=Gr, Pr=Pr)
        meta = dict(driver=drv, variant=VARIANT[drv], nr=nr, np=np_, steps=nts, dt=dt, r0=r0, rmax=rmax, Ra=Ra,
                    Re=Re, Gr=Gr, Pr=Pr, xx=XX[drv], replace=rep)
        save("ref_taycou_relax2new_%dx%d.npz" % (nr, np_), res, meta)
    if not want("layer_routines"):
        return main_3d(only, want, t0)
    # the layer at the 129 x 65 grid of the benchmark's layer workload (box
    # length 2, seeded start), routine by routine in the main loop's order
    cfg = dict(nr=64, np_=128, dt=1e-5, Ra=1e5, Pr=1.0, r0=0.0, rmax=1.0, xx=2.0)
    o = O.OraclePRB(cfg["nr"], cfg["np_"], cfg["dt"], cfg["Ra"], cfg["Pr"], r0=cfg["r0"], rmax=cfg["rmax"],
                    xx=cfg["xx"])
    o.initial(1, 0, 1e-2)
    init = {f: np.array(o.field(f)) for f in O._PRB_FIELDS}
    res = RR.run_layer_routines(cfg["nr"], cfg["np_"], 10, init, cfg["dt"], cfg["Ra"], cfg["Pr"], cfg["r0"],
                                cfg["rmax"], cfg["xx"])
    meta = dict(driver="layer_routines", variant=0, nr=cfg["nr"], np=cfg["np_"], steps=10, dt=cfg["dt"],
                r0=cfg["r0"], rmax=cfg["rmax"], Ra=cfg["Ra"], Re=0.0, Gr=0.0, Pr=cfg["Pr"], xx=cfg["xx"],
                init=dict(kind=1, seed=0, amp=1e-2))
    save("ref_layer_routines_64x128.npz", res, meta)
    return main_3d(only, want, t0)


def main_3d(only, want, t0):
    for drv, nr, nz, np_, nts, dt, r0, rmax, zmax, Ra, Re, Gr, Pr, amp, nval in CASES_3D:
        if not want(drv):
            continue
        res = RR.run_3d(drv, nr, nz, np_, nts, dt=dt, r0=r0, rmax=rmax, zmax=zmax, Ra=Ra, Re=Re, Gr=Gr, Pr=Pr,
                        amp=amp, nval=nval)
        meta = dict(driver=drv, nr=nr, nz=nz, np=np_, steps=nts, dt=dt, r0=r0, rmax=rmax, zmax=zmax, Ra=Ra, Re=Re,
                    Gr=Gr, Pr=Pr, amp=amp, nval=nval)
        save("ref_%s_%dx%dx%d.npz" % (drv, nr, nz, np_), res, meta)
    for drv, nr, nz, np_, nts, dt, r0, rmax, zmax, Ra, Re, Gr, Pr, amp, nval in LARGE_3D:
        if not want(drv):
            continue
        res = RR.run_3d(drv, nr, nz, np_, nts, dt=dt, r0=r0, rmax=rmax, zmax=zmax, Ra=Ra, Re=Re, Gr=Gr, Pr=Pr,
                        amp=amp, nval=nval)
        meta = dict(driver=drv, nr=nr, nz=nz, np=np_, steps=nts, dt=dt, r0=r0, rmax=rmax, zmax=zmax, Ra=Ra, Re=Re,
                    Gr=Gr, Pr=Pr, amp=amp, nval=nval)
        save("ref_%s_%dx%dx%d.npz" % (drv, nr, nz, np_), res, meta, digests=True)
    for nr, nz, nts, dt, r0, rmax, zmax, Ra, Re, Pr in CASES_AXI:
        if not want("axi"):
            continue
        res = RR.run_axi(nr, nz, nts, dt=dt, r0=r0, rmax=rmax, zmax=zmax, Ra=Ra, Re=Re, Pr=Pr)
        meta = dict(driver="axi", nr=nr, nz=nz, steps=nts, dt=dt, r0=r0, rmax=rmax, zmax=zmax, Ra=Ra, Re=Re, Pr=Pr)
        save("ref_axi_%dx%d.npz" % (nr, nz), res, meta, digests=nr * nz > 10000)
    # grid.f's stretched levels and weight tables, and rcsc.f's multigrid on
    # them (the stretched streamfunction solve of the annulus on a tanh
    # or GEF grid)
    if want("transfer"):
        # the batched solve's grid transfers against rotann2.f's corser and
        # finer (the batched workload has no reference program of its own)
        n = 33
        rng = np.random.default_rng(9)
        r = rng.standard_normal((n, n))
        nc = (n - 1) // 2 + 1
        ec = rng.standard_normal((nc, nc))
        psi = rng.standard_normal((n, n))
        for a in (r, ec, psi):
            a[0, :] = a[-1, :] = a[:, 0] = a[:, -1] = 0.0
        fc, psi2, sha = RR.run_rotann2_transfer(n, r, ec, psi)
        meta = dict(driver="transfer", n=n, source="rotann2.f", sha256=sha, end="return")
        np.savez_compressed(os.path.join(HERE, "ref_transfer_rotann2_33.npz"), meta=np.array(json.dumps(meta)),
                            r=r, ec=ec, psi=psi, fc=fc, psi_out=psi2)
        print("ref_transfer_rotann2_33.npz        transfer", flush=True)
    if not want("grid_rcsc"):
        print("fixtures written to %s in %.0f s" % (HERE, time.time() - t0))
        return
    g = dict(nr=64, nz=64, r0=0.5, rmax=1.0, zmax=0.5, zmin=0.0, rdist=0.1, rgef=1.1, dr1=0.002, zdist=0.1,
             zgef=1.1, dz1=0.002)
    gprog, res = RR.run_grid(**g)
    rng = np.random.default_rng(5)
    rhs = rng.standard_normal((g["nr"] + 1, g["nz"] + 1))
    psi0 = np.zeros_like(rhs)
    psi, sw, sha_rcsc = RR.run_rcsc_poisson(gprog, res["nlev"], psi0, rhs)
    meta = dict(driver="grid_rcsc", nlev=res["nlev"], source=res["source"], sha256=res["sha256"], end=res["end"],
                deck=res["deck"], rcsc_source="rcsc.f", rcsc_sha256=sha_rcsc, **g)
    np.savez_compressed(os.path.join(HERE, "ref_grid_rcsc_64x64.npz"), meta=np.array(json.dumps(meta)),
                        rhs=rhs, psi=psi, sweeps=np.array(sw, dtype=np.int32),
                        **{"t_" + k: v for k, v in res["tables"].items()})
    print("ref_grid_rcsc_64x64.npz            grid_rcsc  nlev=%d sweeps=%s" % (res["nlev"], sw), flush=True)
    print("fixtures written to %s in %.0f s" % (HERE, time.time() - t0))


if __name__ == "__main__":
    main(set(sys.argv[1:]))
