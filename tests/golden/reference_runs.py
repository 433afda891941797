"""Runs the reference's own Fortran drivers on the CPU through the translator
in f77.py and collects what they compute: the final fields, the Nusselt
number history and the multigrid sweep count of every solve.

Test infrastructure only.  It reads the reference's source files, so only
the fixture generator beside it (make_reference_golden.py) calls it; the
fixtures it writes are what the tests read.

Each driver runs as its main program with an input deck in the format the
program reads (list-directed READ *), answering "no" to "initial
conditions from file" (the program's own initial state) and to "more
iterations"; its file output is skipped.  The sweep count of a solve is the
last value the solve's outer loop variable took (`do 50 i=1,nvs`), read
through the translator's loop probes.
"""
import hashlib
import os

import numpy as np

import f77

REFERENCE = os.environ.get("GB300_REFERENCE_SOURCE", "/root/reference")

# driver -> (source file within the reference, multigrid units in step order)
DRIVERS = {
    "layer": ("monashubuntudir_velvor2dperiodicrbconvdir/velvor2dperiodicrbconv.f", ("poisson2", "poisson3")),
    "oblique": ("monashubuntudir_velvor2dperiodicrbconvdir/mpkoks.f", ("poisson2", "poisson3")),
    "annulus": ("iarchomedir_groke_storage_users_mpking_rotannconvvelvorplane_continueddir/velvor2dnewsch3.4.f",
                ("poisson2", "poisson3")),
    "tank": ("monashubuntudir_velvor2dhorconvtankdir/velvor2dhorconvtank.f", ("poisson2", "poisson3")),
    "dvd": ("monashubuntudir_velvor2ddvdbenchmarkdir/velvor2ddvdbenchmark.f", ("poisson2", "poisson3")),
    "taycou": ("monashubuntudir_velvor2dtaycouheatdir/velvor2dtaycouheat.f", ("poisson2", "poisson3")),
    "r3d": ("rot3dmg.f", ("poisson1", "poisson2", "poisson3")),
    "r3d_hor": ("rot3dmghor.f", ("poisson1", "poisson2", "poisson3")),
    "axi": ("rotann2.f", ("poisson",)),
}

FIELDS_2D = ["A", "B", "An", "Bn", "Ap", "Cn", "C", "Cp", "thn", "th", "thp", "uel", "vel", "uelp", "velp"]
FIELDS_3D = ["An", "A", "Ap", "Bn", "B", "Bp", "Cn", "C", "Cp", "thn", "th", "thp",
             "uel", "vel", "wel", "uelp", "velp", "welp"]
FIELDS_AXI = ["phi", "omegn", "omeg", "omegp", "veln", "vel", "velp", "thetan", "theta", "thetap"]


def source(driver):
    return os.path.join(REFERENCE, DRIVERS[driver][0])


def sha256(path):
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


def _solve_loops(prog, unit):
    """Source lines of the unit's `do ... i=1,nvs` loops (the sweep loop)."""
    out = []

    def walk(items):
        for _, node in items:
            if node[0] == "do":
                if node[1] == "i" and node[3] == ("name", "nvs"):
                    out.append(node[6])
                walk(node[5])
            elif node[0] == "if":
                for _, body in node[1]:
                    walk(body)
    walk(prog.units[unit].exec)
    if len(out) != 1:
        raise ValueError("%s: expected one sweep loop, found %s" % (unit, out))
    return out[0]


def sweeps_per_solve(seq):
    """Loop-variable values of consecutive solves -> sweeps of each solve."""
    counts = []
    for v in seq:
        if v == 1:
            counts.append(1)
        else:
            counts[-1] = v
    return counts


def sweep_table(prog, units):
    """Sweeps of each solve, one column per multigrid unit in step order;
    -1 where a solve did not run (the run stopped before it)."""
    cols = [sweeps_per_solve(prog.probe[u]) for u in units]
    n = max(len(c) for c in cols)
    return np.array([c + [-1] * (n - len(c)) for c in cols], dtype=np.int32).T


def program(driver, deck, replace=None):
    """The driver's translated program, fed `deck`, with its sweep loops
    probed; replace: {subroutine: source file within the reference} takes
    those subroutines from a sibling version of the driver."""
    path = source(driver)
    rep = {n: os.path.join(REFERENCE, f) for n, f in (replace or {}).items()}
    plain = f77.Program(path, with_main=True, replace=rep)
    probes = {(u, _solve_loops(plain, u)): u for u in DRIVERS[driver][1]}
    return f77.Program(path, probes=probes, with_main=True, stdin=deck, replace=rep)


def run_main(prog):
    """Runs the main program to its STOP.  Returns the unit whose STOP
    ended it: '_main' for the program's own closing STOP, else the routine
    that stopped the run (a solve past its sweep limit)."""
    try:
        prog.sub("_main")()
    except f77.FortranStop as e:
        return str(e)
    return "end"


def extract(prog, name, ranges):
    """Elements of main-program array `name` over the index ranges
    [(lo, hi), ...] (inclusive), dimensions of extent 1 dropped."""
    u = prog.units["_main"]
    v = u.vars[name.lower()]
    lo = [u.const_eval(a)[1] for a, _ in v.dims]
    hi = [u.const_eval(b)[1] for _, b in v.dims]
    if v.kind == "common":
        blk, idx = v.common
        buf = prog.common[blk][idx]
    else:
        buf = prog.static[("_main", name.lower())]
    strides, s = [], 1
    for a, b in zip(lo, hi):
        strides.append(s)
        s *= b - a + 1
    shape = [b - a + 1 for a, b in ranges]
    out = np.zeros(shape)
    for idx in np.ndindex(*shape):
        off = sum((ranges[d][0] + idx[d] - lo[d]) * strides[d] for d in range(len(idx)))
        out[idx] = buf[off]
    return out.reshape([n for n in shape if n != 1])


def deck_2d(nr, np_, nts, dt, r0, rmax, Ra, Re, Gr, Pr, zmax=0.1, pert=0.0, amp=1.0, nval=3):
    """The 2D drivers' deck (velvor2dperiodicrbconv.f:73-117 and alike):
    file names, dt, nr, np, nts, r0 rmax zmax, Ra, Re, Gr (Ta for the
    Taylor-Couette driver), Ptl, pert, amp, nval, then the answers."""
    return ["a.dat", "b.dat", "c.dat", "u.dat", "v.dat", "w.dat", "t.dat", "nu.dat",
            repr(dt), str(nr), str(np_), str(nts), "%r,%r,%r" % (r0, rmax, zmax), repr(Ra), repr(Re), repr(Gr),
            repr(Pr), repr(pert), repr(amp), str(nval), "no", "no"]


def deck_3d(nr, nz, np_, nts, dt, r0, rmax, zmax, Ra, Re, Gr, Pr, pert=0.0, amp=1e-2, nval=3):
    """rot3dmg.f:45-86 (rot3dmghor.f alike)."""
    return ["a.dat", "b.dat", "c.dat", "u.dat", "v.dat", "w.dat", "t.dat", "nu.dat",
            repr(dt), str(nr), str(nz), str(np_), str(nts), "%r,%r,%r" % (r0, rmax, zmax), repr(Ra), repr(Re),
            repr(Gr), repr(Pr), repr(pert), repr(amp), str(nval), "no", "no"]


def deck_axi(nr, nz, nts, dt, r0, rmax, zmax, Ra, Re, Pr, pert=0.0):
    """rotann2.f:24-55."""
    return ["o.dat", "p.dat", "v.dat", "t.dat", "no", "no", "no", repr(dt), str(nr), str(nz), str(nts),
            "%r,%r,%r" % (r0, rmax, zmax), repr(Ra), repr(Re), repr(Pr), repr(pert), "no"]


def run_2d(driver, nr, np_, nts, replace=None, **kw):
    """A 2D driver from its own start.  Returns the outputs as a dict."""
    deck = deck_2d(nr, np_, nts, **kw)
    prog = program(driver, deck, replace)
    end = run_main(prog)
    ncol = np_ + 2 if driver in ("tank", "dvd") else np_ + 1
    out = {f: extract(prog, f, [(0, nr + 1), (1, 1), (0, ncol - 1)]) for f in FIELDS_2D}
    nu = np.stack([extract(prog, h, [(1, nts)]).reshape(nts) for h in ("httrans", "httrans2")], axis=1)
    return dict(fields=out, nu=nu, sweeps=sweep_table(prog, DRIVERS[driver][1]), end=end, deck=deck,
                source=DRIVERS[driver][0], sha256=sha256(source(driver)))


def run_3d(driver, nr, nz, np_, nts, **kw):
    deck = deck_3d(nr, nz, np_, nts, **kw)
    prog = program(driver, deck)
    end = run_main(prog)
    out = {f: extract(prog, f, [(0, nr + 1), (0, nz + 1), (0, np_)]) for f in FIELDS_3D}
    names = ("httrans1", "httrans2") if driver == "r3d_hor" else ("httrans",)
    nu = np.stack([extract(prog, h, [(1, nts)]).reshape(nts) for h in names], axis=1)
    return dict(fields=out, nu=nu, sweeps=sweep_table(prog, DRIVERS[driver][1]), end=end, deck=deck,
                source=DRIVERS[driver][0], sha256=sha256(source(driver)))


def run_axi(nr, nz, nts, **kw):
    deck = deck_axi(nr, nz, nts, **kw)
    prog = program("axi", deck)
    end = run_main(prog)
    out = {f: extract(prog, f, [(0, nr), (0, nz)]) for f in FIELDS_AXI}
    sw = sweeps_per_solve(prog.probe["poisson"])
    nu = extract(prog, "httrans", [(1, len(sw))]).reshape(-1)
    return dict(fields=out, nu=nu, sweeps=np.array(sw, dtype=np.int32), end=end, deck=deck,
                source=DRIVERS["axi"][0], sha256=sha256(source("axi")))


def run_layer_routines(nr, np_, nsteps, init, dt, Ra, Pr, r0, rmax, xx):
    """The layer's subroutines called in the main loop's order
    (velvor2dperiodicrbconv.f:341-388) from a given state, with COMMON set
    as the main program sets it (dr = (rmax-r0)/nr, dp = xx/np, nz = 1,
    dz = 0, Re = Gr = 0): for states other than the program's own start
    and for box lengths other than its xx = 3."""
    prog = program("layer", [])
    cm = prog.common_member
    dr = (rmax - r0) / float(nr)
    dp = xx / float(np_)
    for blk, name, val in (("num", "dt", dt), ("num", "dr", dr), ("num", "dz", 0.0), ("num", "dp", dp),
                           ("num", "nr", nr), ("num", "nz", 1), ("num", "np", np_), ("val", "ra", Ra),
                           ("val", "re", 0.0), ("val", "ptl", Pr), ("val", "gr", 0.0), ("radius", "r0", r0),
                           ("radius", "rmax", rmax)):
        cm(blk, name)[0] = val
    u = prog.units["poisson2"]
    kr1 = u.const_eval(("name", "kr"))[1] + 1
    kp1 = u.const_eval(("name", "kp"))[1] + 1
    sol = {"an": "sol1", "a": "sol1", "ap": "sol1", "bn": "sol1", "b": "sol1", "bp": "sol1", "cn": "sol1",
           "c": "sol1", "cp": "sol1", "thn": "sol2", "th": "sol2", "thp": "sol2", "uel": "sol3", "vel": "sol3",
           "wel": "sol3", "uelp": "sol3", "velp": "sol3", "welp": "sol3"}
    vrh, urh = [0.0] * (kr1 * kp1), [0.0] * (kr1 * kp1)
    bufs = {n: cm(b, n) for n, b in sol.items()}
    bufs["vrh"], bufs["urh"] = vrh, urh
    for name, a in init.items():
        buf = bufs[name.lower()]
        for k in range(np_ + 1):
            for i in range(nr + 2):
                buf[i + kr1 * k] = float(a[i, k])
    R, Cl = f77.ref, f77.cell
    nrc, nzc, npc = Cl(nr), Cl(1), Cl(np_)
    drc, dzc, dpc = Cl(dr), Cl(0.0), Cl(dp)
    nlev = Cl(0)
    prog.sub("poissoninit")(nrc, nzc, npc, drc, dzc, dpc, nlev)
    nus = []
    for kt in range(1, nsteps + 1):
        cm("iteration", "kt")[0] = kt
        prog.sub("cvorticity1" if kt == 1 else "cvorticity")()
        prog.sub("temperature1" if kt == 1 else "temperature")()
        t1, t2 = Cl(0.0), Cl(0.0)
        prog.sub("heat")(t1, t2)
        prog.sub("rhsv")(R(vrh))
        prog.sub("poisson2")(R(bufs["vel"]), R(bufs["velp"]), R(vrh), nrc, nzc, npc, drc, dzc, dpc, nlev)
        prog.sub("rhsu")(R(urh))
        prog.sub("poisson3")(R(bufs["uel"]), R(bufs["uelp"]), R(urh), nrc, nzc, npc, drc, dzc, dpc, nlev)
        prog.sub("update")()
        nus.append((t1[0][0] * (rmax - r0) / xx, t2[0][0] * (rmax - r0) / xx))

    def grab(buf):
        return np.array([[buf[i + kr1 * k] for k in range(np_ + 1)] for i in range(nr + 2)])
    out = {f: grab(bufs[f.lower()]) for f in FIELDS_2D + ["urh", "vrh"]}
    return dict(fields=out, nu=np.array(nus), sweeps=sweep_table(prog, ("poisson2", "poisson3")), end="return",
                source=DRIVERS["layer"][0], sha256=sha256(source("layer")))


GRID_STUBS = ("contor", "xxxxxx", "j06waf", "j06wcf", "j06wbf", "j06xff", "j06ahf", "j06wzf", "grapol", "gracur",
              "gramov", "gralin")


def run_grid(nr, nz, r0, rmax, zmax, zmin, rdist, rgef, dr1, zdist, zgef, dz1):
    """grid.f's main program (grid.f:53-270): wall-clustered spacings with
    geometric expansion (grid, :723-857), the levels (level, :859-924) and
    the finite-difference weight tables of every level (:178-243, fdif and
    gausse).  Its plotting calls (the NAG graphics library and its contour
    routine) run as no-ops; the coefficient file it writes is read from its
    arrays instead.  Returns the program (its arrays feed run_rcsc_poisson)
    and the tables."""
    deck = [str(nr), str(nz), "%r,%r,%r,%r" % (r0, rmax, zmax, zmin), "y", repr(rdist), repr(rgef), repr(dr1),
            "y", repr(zdist), repr(zgef), repr(dz1), "n", "y", "coef.dat"]
    path = os.path.join(REFERENCE, "grid.f")
    prog = f77.Program(path, with_main=True, stdin=deck, stubs=GRID_STUBS)
    end = run_main(prog)
    u = prog.units["_main"]
    nx = u.const_eval(("name", "nx"))[1]
    st = lambda n: prog.static[("_main", n)]  # noqa: E731
    n1, n2 = st("n1"), st("n2")
    nlev = sum(1 for v in n1 if v > 0)
    tables = {}
    for L in range(1, nlev + 1):
        a, b = n1[L - 1], n2[L - 1]
        tables["hr_%d" % L] = np.array([st("hx")[(i - 1) + nx * (L - 1)] for i in range(1, a + 1)])
        tables["hz_%d" % L] = np.array([st("hy")[(j - 1) + nx * (L - 1)] for j in range(1, b + 1)])
        tables["r_%d" % L] = np.array([st("x")[i + (nx + 1) * (L - 1)] for i in range(a + 1)])
        tables["z_%d" % L] = np.array([st("y")[j + (nx + 1) * (L - 1)] for j in range(b + 1)])
        for name, n, w in (("cr", a, 3), ("crr", a, 4), ("cz", b, 3), ("czz", b, 4)):
            tables["%s_%d" % (name, L)] = np.array([[st(name)[(i - 1) + nx * ((k - 1) + w * (L - 1))]
                                                     for k in range(1, w + 1)] for i in range(1, n)]).ravel()
    # the wall weights of level 1 at i = n1 and j = n2 (the file's last lines)
    tables["crn"] = np.array([st("cr")[(n1[0] - 1) + nx * (k - 1)] for k in range(1, 4)])
    tables["czn"] = np.array([st("cz")[(n2[0] - 1) + nx * (k - 1)] for k in range(1, 4)])
    return prog, dict(tables=tables, nlev=nlev, end=end, deck=deck, source="grid.f", sha256=sha256(path))


def run_rcsc_poisson(grid_prog, nlev, psi, rhs):
    """rcsc.f's stretched-grid multigrid (poisson, :1118-1190, with relax,
    corser and finer) on the levels and tables grid.f computed, copied into
    rcsc.f's COMMON blocks /num/, /ints/ and /coeff/ as rcsc.f's main program
    reads them from grid.f's coefficient file.  Returns psi and the sweeps."""
    path = os.path.join(REFERENCE, "rcsc.f")
    plain = f77.Program(path)
    prog = f77.Program(path, probes={("poisson", _solve_loops(plain, "poisson")): "poisson"})
    st = lambda n: grid_prog.static[("_main", n)]  # noqa: E731
    for blk, name, src in (("num", "hr", "hx"), ("num", "hz", "hy"), ("num", "r", "x"), ("num", "z", "y"),
                           ("num", "n1", "n1"), ("num", "n2", "n2"), ("ints", "ibeg", "ibeg"),
                           ("coeff", "cr", "cr"), ("coeff", "crr", "crr"), ("coeff", "cz", "cz"),
                           ("coeff", "czz", "czz")):
        dst = prog.common_member(blk, name)
        if len(dst) != len(st(src)):
            raise ValueError("grid.f and rcsc.f disagree on the size of " + name)
        dst[:] = st(src)
    u = prog.units["poisson"]
    ld = u.const_eval(("name", "kr"))[1] + 1
    n1, n2 = psi.shape[0] - 1, psi.shape[1] - 1
    pb, rb, vb = [0.0] * (ld * ld), [0.0] * (ld * ld), [0.0] * (ld * ld)
    for j in range(n2 + 1):
        for i in range(n1 + 1):
            pb[i + ld * j] = float(psi[i, j])
            rb[i + ld * j] = float(rhs[i, j])
    prog.sub("poisson")(f77.ref(pb), f77.ref(rb), f77.cell(nlev), f77.ref(vb))
    out = np.array([[pb[i + ld * j] for j in range(n2 + 1)] for i in range(n1 + 1)])
    return out, sweeps_per_solve(prog.probe["poisson"]), sha256(path)


def run_rotann2_transfer(n, r, ec, psi):
    """rotann2.f's corser (:755-801) and finer (:803-854) between a level of
    n x n vertices (n - 1 intervals each way) and the next coarser: the
    residual r restricted to the coarse grid, and the coarse correction ec
    prolonged and added to psi.  Arrays are indexed [j, i] (i fastest, as
    the batched oracle stores them); returns (coarse right-hand side, psi)."""
    path = os.path.join(REFERENCE, "rotann2.f")
    prog = f77.Program(path)
    cm = prog.common_member
    u = prog.units["corser"]
    ld = u.const_eval(("name", "kr"))[1] + 1
    m, mc = n - 1, (n - 1) // 2
    for name, vals in (("n1", (m, mc)), ("n2", (m, mc)), ("ibeg", (1, 1 + n * n + 1))):
        buf = cm("ints", name)
        for k, v in enumerate(vals):
            buf[k] = v
    cm("ints", "nlev")[0] = 2
    rc = cm("arrays", "rc")
    for j in range(n):
        for i in range(n):
            rc[i + ld * j] = float(r[j, i])
    prog.sub("corser")(f77.cell(1))
    fc = np.array([[rc[i + ld * j] for i in range(mc + 1)] for j in range(mc + 1)])
    v = cm("backup", "v")
    nc = mc + 1
    for j in range(nc):
        for i in range(nc):
            v[(1 + n * n + 1) - 1 + i + nc * j] = float(ec[j, i])
    for j in range(n):
        for i in range(n):
            v[1 - 1 + i + n * j] = float(psi[j, i])
    prog.sub("finer")(f77.cell(2))
    psif = cm("arrays", "psif")
    out = np.array([[psif[i + ld * j] for i in range(n)] for j in range(n)])
    return fc, out, sha256(path)
