"""Served parameter-sweep solves with continuous batching.

Requests (the 2D periodic layer of velvor2dperiodicrbconv.f or the
axisymmetric annulus of rotann2.f, each with its own grid, Ra, Pr, Ta and
step count) arrive over time.  The server admits them in arrival order as
device memory (a byte budget) and active slots allow, gives each admitted
request its own device-resident instance and CUDA stream, and advances every
active instance in chunks of graph-replayed steps queued asynchronously, so
the work of all active requests overlaps on the GPU; a finished request
frees its memory and slot for the next arrival at once.  State never leaves
the device between steps; only the per-step Nusselt history (and, on
request, the final fields) come back.

Every instance is deterministic and runs on its own stream, so a request's
result does not depend on what else is in flight: the same request served
alone and in a mix gives bit-identical fields and Nusselt histories.

`Server` takes an instance factory, so its admission and chunking logic can
run against stand-in instances without a GPU.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass
from typing import Callable, Dict, List, Optional

import numpy as np

from . import lib as _L

LAYER = "layer"
AXI = "axi"

# grid shapes of the sweep as intervals (x or r) x (z): 65x33 ... 513x257 vertices
SWEEP_GRIDS = ((64, 32), (128, 64), (256, 128), (512, 256))

# multigrid tolerances of the two reference drivers (velvor2dperiodicrbconv.f
# relax2/relax3 tolcon 2e-6; rotann2.f relax tolcon 1e-6)
LAYER_TOLCON = 2e-6
AXI_TOLCON = 1e-6
AXI_MAXSWEEPS = 500   # bounded for serving (the reference allows 10000)


@dataclass
class Request:
    rid: int
    kind: str            # LAYER or AXI
    nx: int              # layer: np (periodic intervals); axi: nr
    nz: int              # layer: nr (wall-normal intervals); axi: nz
    Ra: float
    Pr: float
    Ta: float            # annulus only: rotational Reynolds number Re = sqrt(Ta)/2
    steps: int
    seed: int = 0
    arrival: float = 0.0
    dt: float = 0.0      # 0: chosen from the grid, Ra and Ta

    def cells(self) -> int:
        return (self.nx + 1) * (self.nz + 1)


@dataclass
class Result:
    rid: int
    status: int
    admit: float
    finish: float
    tts: float           # finish - arrival (queueing included)
    steps_done: int
    nu: np.ndarray
    fields: Optional[Dict[str, np.ndarray]] = None


def annulus_re(Ta: float) -> float:
    """Rotational Reynolds number of a Taylor number, Ta = 4 Omega^2 d^4 /
    nu^2 and Re = Omega d^2 / nu."""
    return math.sqrt(Ta) / 2.0


def default_dt(req: Request) -> float:
    """Time step of a request: the 129 x 65 layer's 1e-5 scaled diffusively
    with the grid and reduced for strong convection; for the layer also by
    1/sqrt(Pr) above Pr 1 (without it five Pr-7 layers of the 512-request
    sweep on the 65 x 33 grid, Ra 2.5e6-3e7, stopped at the sweep limit
    after 287-418 steps, on the device and in the oracle alike, and finish
    with it); for the annulus also for slow rotation, whose buoyancy
    coupling scales with Ra/Re (a rule checked stable on the sweep's grids at
    the corners of its Ra and Ta ranges)."""
    if req.kind == LAYER:
        return 1e-5 * (64.0 / req.nz) ** 2 * min(1.0, math.sqrt(1e5 / req.Ra)) * min(1.0, 1.0 / math.sqrt(req.Pr))
    n = max(req.nx, req.nz)
    return 1e-5 * (64.0 / n) ** 2 * min(1.0, math.sqrt(1e5 / req.Ra)) * min(1.0, annulus_re(req.Ta) / 50.0)


def estimate_bytes(req: Request) -> int:
    """Device bytes an instance holds: fields, multigrid pools, factors and
    graph state (an upper estimate)."""
    if req.kind == LAYER:
        cells = (req.nz + 2) * (req.nx + 1)
        return int(8 * cells * 27 + (4 << 20))
    cells = (req.nx + 1) * (req.nz + 1)
    return int(8 * cells * 22 + (4 << 20))


def sweep_requests(n=512, rate=50.0, seed=0, steps=(500, 5000), grids=SWEEP_GRIDS, kinds=(LAYER, AXI)):
    """The parameter sweep: Poisson arrivals at `rate` per second, kind and
    grid uniform over the choices, Ra log-uniform in [1e4, 1e8], Pr from
    {0.7, 1, 7}, Ta log-uniform in [1, 1e6] (annulus only), steps uniform in
    the range; all drawn from one seeded generator."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        kind = kinds[int(rng.integers(len(kinds)))]
        gx, gz = grids[int(rng.integers(len(grids)))]
        Ra = float(10.0 ** rng.uniform(4.0, 8.0))
        Pr = float((0.7, 1.0, 7.0)[int(rng.integers(3))])
        Ta = float(10.0 ** rng.uniform(0.0, 6.0)) if kind == AXI else 0.0
        st = int(rng.integers(steps[0], steps[1] + 1))
        out.append(Request(i, kind, gx, gz, Ra, Pr, Ta, st, seed * 100003 + i, t))
    return out


def axi_initial(nr, nz, r0, rmax, seed, amp, r=None):
    """The annulus start: conduction profile 1 - ln(r/rmax)/ln(r0/rmax) plus
    seeded splitmix64 noise over rows i = 1..nr-1 (j-major), every other
    field zero.  r: the radii r(0..nr) of a stretched grid (default:
    uniform)."""
    from .initial import _splitmix64
    if r is None:
        dr = (rmax - r0) / nr
        r = r0 + np.arange(nr + 1) * dr
    base = np.array([1.0 - math.log(float(x) / rmax) / math.log(r0 / rmax) for x in r])
    u = (_splitmix64(seed, (nr - 1) * (nz + 1)) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    th = np.asfortranarray(np.repeat(base[:, None], nz + 1, axis=1))
    th[1:nr, :] = base[1:nr, None] + amp * (2.0 * u.reshape(nz + 1, nr - 1).T - 1.0)
    zero = np.zeros_like(th)
    return {"theta": th, "thetap": th.copy(), "phi": zero, "omeg": zero, "omegp": zero, "vel": zero, "velp": zero,
            "omegn": zero, "veln": zero, "thetan": zero}


class DeviceInstance:
    """One request's device-resident instance (layer or annulus)."""

    def __init__(self, req: Request, precision=_L.PRB_FP64, smoother=_L.SMOOTHER_ZEBRA):
        from . import initial
        self.req = req
        dt = req.dt or default_dt(req)
        L = _L.load()
        if req.kind == LAYER:
            from .prb import PRB
            self.g = PRB(req.nz, req.nx, dt=dt, r0=0.0, rmax=1.0, xx=2.0, Ra=req.Ra, Pr=req.Pr,
                         tolcon=LAYER_TOLCON, smoother=smoother, precision=precision)
            for n, a in initial.initial_fields(req.nz, req.nx, 0.0, 1.0, _L.PRB_LAYER, 1, req.seed, 1e-3).items():
                self.g.set(n, a)
            self._begin, self._query = L.gb_prb_run_begin, L.gb_prb_run_query
        else:
            from .axi import AXI as _AXI
            self.g = _AXI(req.nx, req.nz, dt=dt, r0=0.5, rmax=1.0, zmax=0.5, Ra=req.Ra, Re=annulus_re(req.Ta),
                          Pr=req.Pr, tolcon=AXI_TOLCON, maxsweeps=AXI_MAXSWEEPS, smoother=smoother,
                          precision=precision)
            for n, a in axi_initial(req.nx, req.nz, 0.5, 1.0, req.seed, 1e-3).items():
                self.g.set(n, a)
            self._begin, self._query = L.gb_axi_run_begin, L.gb_axi_run_query
        self.enqueued = 0

    def begin(self, total):
        _L.check(self._begin(self.g._h, total), "run_begin")

    def enqueue(self, n):
        L = _L.load()
        if self.req.kind == LAYER:
            st = L.gb_prb_run_enqueue(self.g._h, self.enqueued + 1, n)
        else:
            st = L.gb_axi_run_enqueue(self.g._h, n)
        _L.check(st, "run_enqueue")
        self.enqueued += n

    def query(self) -> int:
        return self._query(self.g._h)

    def end(self, n):
        import ctypes as C
        L = _L.load()
        done = C.c_int()
        if self.req.kind == LAYER:
            nu = np.zeros((n, 2))
            sw = np.zeros((n, 2), dtype=np.int32)
            st = L.gb_prb_run_end(self.g._h, n, nu.ctypes.data, sw.ctypes.data, C.byref(done))
        else:
            nu = np.zeros(n)
            sw = np.zeros(n, dtype=np.int32)
            st = L.gb_axi_run_end(self.g._h, n, nu.ctypes.data, sw.ctypes.data, C.byref(done))
        return st, nu[:done.value], done.value

    def fields(self):
        names = ("vel", "uel", "C", "th") if self.req.kind == LAYER else ("phi", "omeg", "vel", "theta")
        return {n: self.g.get(n) for n in names}

    def close(self):
        self.g.close()


@dataclass
class _Active:
    req: Request
    inst: object
    admit: float
    nbytes: int
    enqueued: int = 0


class Server:
    """Continuous-batching request loop over device-resident instances."""

    def __init__(self, budget_bytes: float = 120e9, max_active: int = 128, chunk: int = 16,
                 factory: Optional[Callable[[Request], object]] = None, keep_fields: bool = False,
                 clock: Callable[[], float] = time.perf_counter, sleep: Callable[[float], None] = time.sleep,
                 precision=_L.PRB_FP64, smoother=_L.SMOOTHER_ZEBRA):
        self.budget = budget_bytes
        self.max_active = max_active
        self.chunk = chunk
        self.factory = factory or (lambda r: DeviceInstance(r, precision, smoother))
        self.keep_fields = keep_fields
        self.clock = clock
        self.sleep = sleep
        self.peak_active = 0
        self.peak_bytes = 0

    def run(self, requests: List[Request]) -> List[Result]:
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        active: List[_Active] = []
        results: Dict[int, Result] = {}
        used = 0
        t0 = self.clock()
        while pending or active:
            now = self.clock() - t0
            # admission: arrival order, while memory and slots allow (a request
            # larger than the whole budget still runs, alone)
            while pending and pending[0].arrival <= now and len(active) < self.max_active:
                nb = estimate_bytes(pending[0])
                if used + nb > self.budget and active:
                    break
                req = pending.pop(0)
                inst = self.factory(req)
                inst.begin(req.steps)
                active.append(_Active(req, inst, now, nb))
                used += nb
            self.peak_active = max(self.peak_active, len(active))
            self.peak_bytes = max(self.peak_bytes, used)
            progressed = False
            for a in list(active):
                q = a.inst.query()
                if q == 0:
                    continue
                if q > 0 and a.enqueued < a.req.steps:
                    n = min(self.chunk, a.req.steps - a.enqueued)
                    a.inst.enqueue(n)
                    a.enqueued += n
                    progressed = True
                    continue
                st, nu, done = a.inst.end(a.req.steps) if q > 0 else (-q, np.zeros(0), 0)
                fin = self.clock() - t0
                flds = a.inst.fields() if (self.keep_fields and q > 0) else None
                results[a.req.rid] = Result(a.req.rid, st, a.admit, fin, fin - a.req.arrival, done, nu, flds)
                a.inst.close()
                used -= a.nbytes
                active.remove(a)
                progressed = True
            if not progressed:
                if not active and pending:
                    self.sleep(max(0.0, min(0.01, pending[0].arrival - (self.clock() - t0))))
                else:
                    self.sleep(0.0002)
        return [results[r.rid] for r in sorted(requests, key=lambda r: r.rid)]


class _Gang:
    """One gang (gb_prb_gang or gb_axi_gang) over device instances of one
    kind; rebuilt whenever its membership changes."""

    def __init__(self, kind, solve_spread=1):
        L = _L.load()
        self.kind = kind
        self.solve_spread = solve_spread
        if kind == LAYER:
            self._create, self._enqueue, self._query, self._destroy = (
                L.gb_prb_gang_create, L.gb_prb_gang_enqueue, L.gb_prb_gang_query, L.gb_prb_gang_destroy)
        else:
            self._create, self._enqueue, self._query, self._destroy = (
                L.gb_axi_gang_create, L.gb_axi_gang_enqueue, L.gb_axi_gang_query, L.gb_axi_gang_destroy)
        self.h = None

    def build(self, members):
        import ctypes as C
        self.close()
        n = len(members)
        handles = (C.c_void_p * n)(*[m.inst.g._h.value for m in members])
        totals = (C.c_int * n)(*[m.req.steps for m in members])
        h = C.c_void_p()
        _L.check(self._create(handles, totals, n, C.byref(h)), "gang_create")
        self.h = h
        if self.kind == LAYER and self.solve_spread != 1:
            _L.check(_L.load().gb_prb_gang_set_solve_spread(h, self.solve_spread), "gang_set_solve_spread")

    def enqueue(self, nsteps):
        _L.check(self._enqueue(self.h, nsteps, None), "gang_enqueue")

    def query(self) -> int:
        return self._query(self.h)

    def built(self) -> bool:
        return self.h is not None

    def close(self):
        if self.h is not None and self.h.value:
            self._destroy(self.h)
        self.h = None


@dataclass
class _Member:
    req: Request
    inst: object
    admit: float
    nbytes: int
    taken: int = 0       # steps the device has run (host accounting, chunk-granular)


class GangServer:
    """Continuous batching across sizes: the active requests of each kind
    (layer, annulus) form one gang whose every step is a handful of launches
    over all members, whatever their grids.  Requests are admitted in arrival
    order while the device-memory budget and the slot cap allow; between
    chunks of `chunk` steps the server retires the members that finished,
    admits arrivals and rebuilds the gang; a layer request's first step
    (the forward step) runs on its own stream before it joins.  Each member
    runs its own kernel bodies, so its result is bit-identical to the same
    request served alone."""

    def __init__(self, budget_bytes: float = 120e9, max_active: int = 1024, chunk: int = 32,
                 keep_fields: bool = False, clock: Callable[[], float] = time.perf_counter,
                 sleep: Callable[[float], None] = time.sleep, precision=_L.PRB_FP64, smoother=_L.SMOOTHER_ZEBRA,
                 group_by: str = "kind", factory: Optional[Callable[[Request], object]] = None,
                 gang_factory: Optional[Callable[[str], object]] = None, solve_spread: int = 8):
        """group_by: "kind" (one gang per kind, batched across grid sizes:
        every member steps at the pace of the largest) or "shape" (one gang
        per kind and grid; the gangs run side by side on their own streams).
        solve_spread: CTAs per velocity solve of the layer gangs (8, a cluster:
        a gang step waits for its slowest member's solve, which a cluster
        shortens; or 1).
        factory / gang_factory: stand-ins for the device instance and gang
        (the host logic's tests)."""
        assert group_by in ("kind", "shape")
        self.group_by = group_by
        self.factory = factory or (lambda r: DeviceInstance(r, precision, smoother))
        self.gang_factory = gang_factory or (lambda kind: _Gang(kind, solve_spread))
        self.budget = budget_bytes
        self.max_active = max_active
        self.chunk = chunk
        self.keep_fields = keep_fields
        self.clock = clock
        self.sleep = sleep
        self.precision = precision
        self.smoother = smoother
        self.peak_active = 0
        self.peak_bytes = 0
        self.rebuilds = 0
        self.chunks = 0

    def run(self, requests: List[Request]) -> List[Result]:
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        groups: Dict[tuple, dict] = {}

        def group_of(req):
            key = (req.kind,) if self.group_by == "kind" else (req.kind, req.nx, req.nz)
            if key not in groups:
                groups[key] = {"members": [], "joining": [], "gang": self.gang_factory(req.kind), "busy": False}
            return groups[key]
        results: Dict[int, Result] = {}
        used, n_active = 0, 0
        t0 = self.clock()

        def finish(m, now):
            nonlocal used, n_active
            st, nu, done = m.inst.end(m.req.steps)
            flds = m.inst.fields() if self.keep_fields else None
            results[m.req.rid] = Result(m.req.rid, st, m.admit, now, now - m.req.arrival, done, nu, flds)
            m.inst.close()
            used -= m.nbytes
            n_active -= 1

        while pending or any(g["members"] or g["joining"] for g in list(groups.values())):
            now = self.clock() - t0
            progressed = False
            while pending and pending[0].arrival <= now and n_active < self.max_active:
                nb = estimate_bytes(pending[0])
                if used + nb > self.budget and n_active:
                    break
                req = pending.pop(0)
                inst = self.factory(req)
                inst.begin(req.steps)
                m = _Member(req, inst, now, nb)
                if req.kind == LAYER and req.steps > 0:
                    inst.enqueue(1)           # the forward first step, on the instance's own stream
                    m.taken = 1
                group_of(req)["joining"].append(m)
                used += nb
                n_active += 1
                progressed = True
            self.peak_active = max(self.peak_active, n_active)
            self.peak_bytes = max(self.peak_bytes, used)
            for g in list(groups.values()):
                if g["busy"]:
                    q = g["gang"].query()
                    if q == 0:
                        continue
                    if q < 0:
                        _L.check(-q, "gang_query")
                    g["busy"] = False
                    now = self.clock() - t0
                    for m in g["members"]:
                        m.taken = min(m.req.steps, m.taken + self.chunk)
                    done = [m for m in g["members"] if m.taken >= m.req.steps]
                    for m in done:
                        finish(m, now)
                    g["members"] = [m for m in g["members"] if m.taken < m.req.steps]
                    if done:
                        g["gang"].close()
                    progressed = True
                if g["busy"]:
                    continue
                if g["joining"]:
                    now = self.clock() - t0
                    for m in [m for m in g["joining"] if m.taken >= m.req.steps]:
                        finish(m, now)        # a one-step request: its first step was all of it
                    g["members"] += [m for m in g["joining"] if m.taken < m.req.steps]
                    g["joining"] = []
                    g["gang"].close()
                if g["members"]:
                    if not g["gang"].built():
                        g["gang"].build(g["members"])
                        self.rebuilds += 1
                    g["gang"].enqueue(self.chunk)
                    g["busy"] = True
                    self.chunks += 1
                    progressed = True
            if not progressed:
                if pending and not any(g["busy"] for g in groups.values()):
                    self.sleep(max(0.0, min(0.01, pending[0].arrival - (self.clock() - t0))))
                else:
                    self.sleep(0.0002)
        for g in groups.values():
            g["gang"].close()
        return [results[r.rid] for r in sorted(requests, key=lambda r: r.rid)]


def summarize(requests: List[Request], results: List[Result]) -> dict:
    """solves/s over the makespan (first arrival to last finish), p50 / p99
    time to solution, served cell-updates/s."""
    ok = [r for r in results if r.status == 0]
    by = {q.rid: q for q in requests}
    tts = np.array([r.tts for r in ok]) if ok else np.zeros(1)
    t_first = min(q.arrival for q in requests)
    t_last = max(r.finish for r in results)
    span = max(t_last - t_first, 1e-9)
    cu = sum(by[r.rid].cells() * r.steps_done for r in ok)
    failed = [{"rid": r.rid, "status": r.status, "kind": by[r.rid].kind, "grid": [by[r.rid].nx, by[r.rid].nz],
               "Ra": by[r.rid].Ra, "Pr": by[r.rid].Pr, "Ta": by[r.rid].Ta, "steps_done": r.steps_done,
               "steps": by[r.rid].steps} for r in results if r.status != 0]
    return {"requests": len(requests), "completed": len(ok), "failed": len(results) - len(ok), "failures": failed,
            "makespan_s": span, "solves_per_s": len(ok) / span, "cell_updates_per_s": cu / span,
            "tts_p50_s": float(np.percentile(tts, 50)), "tts_p99_s": float(np.percentile(tts, 99)),
            "tts_mean_s": float(np.mean(tts))}
