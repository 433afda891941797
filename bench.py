"""Benchmark of the batched Poisson workload: 256 independent Dirichlet
problems nabla^2 psi = -omega on n x n vertex grids, n drawn uniformly from
{65, 129, 257, 513} (seed 0), omega a seeded zero-mean unit-variance Gaussian
random field with squared-exponential correlation length 0.05 of the domain
(synthetic: FFT-filtered white noise), solved by V(2,2) red-black cycles to
relative residual 1e-10.

One step = one solve of the whole batch.  value = cell-updates/s (interior
points x V-cycles / second) of the FP32-inner / FP64-defect-correction path
(GB_BATCH_MIXED_F64OUTER: outer residual, norm and update in FP64), with
inputs resident in HBM; the plain FP64 path and the float-pair defect
correction (GB_BATCH_MIXED) are timed the same way and reported beside it,
each with its field error; e2e repeats the mixed solve through the C ABI's host-
buffer entry points with pinned host arrays, so every step's host->device
copy of f and device->host copy of psi are inside the timed region: as a
stream of steps (gb_batch_submit_host / gb_batch_drain, each step's copies
overlapping the neighbouring steps' solves) for e2e.value, and one call per
step (gb_batch_solve_host: copy in, solve, copy out) for e2e.serial_value.

--impl reference times the CPU restatement of the same algorithm (oracle/,
OpenMP over problems, all host threads) on a bounded sample of problems.
Under torchrun each rank solves its own batch of 256 problems (weak scaling,
no collective on the data path); rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SIZES = (65, 129, 257, 513)
NPROB = 256
CORR = 0.05
RTOL = 1e-10
METRIC = "cell-updates/s (batched Poisson, V(2,2) to rel. residual 1e-10)"


def workload_sizes(seed=0, nprob=NPROB):
    return np.random.default_rng(seed).choice(SIZES, size=nprob).astype(np.int32)


def grf(rng, n, corr=CORR):
    """Zero-mean, unit-variance Gaussian random field on an n x n grid with
    squared-exponential covariance of correlation length corr (FFT filtering
    of white noise), boundary zeroed."""
    w = rng.standard_normal((n, n))
    k = np.fft.fftfreq(n, d=1.0 / (n - 1))
    kx, ky = np.meshgrid(k, k, indexing="ij")
    filt = np.exp(-((2 * np.pi) ** 2) * (kx ** 2 + ky ** 2) * corr ** 2 / 4.0)
    g = np.real(np.fft.ifft2(np.fft.fft2(w) * filt))
    g = (g - g.mean()) / g.std()
    g[0, :] = g[-1, :] = g[:, 0] = g[:, -1] = 0.0
    return g


def workload_rhs(sizes, seed):
    rng = np.random.default_rng(1000 + seed)
    return np.concatenate([-grf(rng, int(n)).ravel() for n in sizes])


def interior(sizes):
    s = np.asarray(sizes, dtype=np.int64)
    return (s - 2) ** 2


def cpu_model():
    """The host CPU's model as /proc/cpuinfo names it (x86: 'model name';
    Arm: implementer and part numbers, Neoverse V2 for Grace), and nproc."""
    name, impl, part = None, None, None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k, _, v = line.partition(":")
                k, v = k.strip(), v.strip()
                if k == "model name" and not name:
                    name = v
                elif k == "CPU implementer" and not impl:
                    impl = v
                elif k == "CPU part" and not part:
                    part = v
    except OSError:
        pass
    if not name and impl:
        known = {("0x41", "0xd4f"): "Arm Neoverse V2 (NVIDIA Grace)"}
        name = known.get((impl, part), "Arm implementer %s part %s" % (impl, part))
    return "%s, %d logical CPUs" % (name or "unknown CPU", os.cpu_count() or 0)


def batch_config(total, interior_pts, ws):
    """The workload description both arms print (same keys, same values)."""
    return {"workload": "batched Poisson: 256 problems, n in {65,129,257,513}, V(2,2) RB-GS, rtol 1e-10",
            "nprob": NPROB, "sizes": list(SIZES), "seed": 0, "points": int(total),
            "interior_points": int(interior_pts), "rtol": RTOL,
            "l2": "inputs larger than L2 (f and psi 2 x %.0f MB)" % (total * 8 / 1e6),
            "parallelism": "replicas x%d" % ws}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while
    the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 7:
                continue
            try:
                mhz.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(mhz)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_reference(sizes_all, seed, budget_s=20.0, threads=None, reps=1):
    """The oracle (CPU restatement, OpenMP over problems) on a bounded
    sample of the workload: problems are added until about budget_s of work
    is measured (the whole batch when it fits), then the same sample is
    solved again until reps timings exist.  Returns (median cell-updates/s
    over the reps, sample description, threads, problems used, psi of the
    sample)."""
    from oracle import oracle as O
    O.build()
    threads = threads or os.cpu_count()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    # one of each size first, then the workload's own order
    order = []
    for n in SIZES:
        order.append(int(np.nonzero(sizes_all == n)[0][0]))
    order += [i for i in range(len(sizes_all)) if i not in order]
    done_cu, done_t, used = 0.0, 0.0, []
    psi_s, chunks = [], []
    rng_f = workload_rhs(sizes_all, seed)
    offs = np.concatenate([[0], np.cumsum(sizes_all.astype(np.int64) ** 2)])
    i = 0
    while i < len(order) and done_t < budget_s:
        chunk = order[i:i + max(threads, 4)]
        i += len(chunk)
        sz = [int(sizes_all[j]) for j in chunk]
        f = np.concatenate([rng_f[offs[j]:offs[j + 1]] for j in chunk])
        t0 = time.perf_counter()
        st, psi, cyc, rr = O.batch_solve(sz, f, precision=0, rtol=RTOL)
        dt = time.perf_counter() - t0
        done_t += dt
        done_cu += float(np.sum(interior(sz) * cyc))
        used += chunk
        psi_s.append(psi)
        chunks.append((sz, f))
    rates = [done_cu / done_t]
    while len(rates) < reps:
        t0 = time.perf_counter()
        for sz, f in chunks:
            O.batch_solve(sz, f, precision=0, rtol=RTOL)
        rates.append(done_cu / (time.perf_counter() - t0))
    sample = "%d of the %d problems (sizes %s), FP64 oracle, %d OpenMP threads, %.1f s per run, median of %d " \
             "run(s); %s" % (len(used), len(sizes_all), sorted(set(int(sizes_all[j]) for j in used)), threads,
                             done_t, len(rates), cpu_model())
    return float(np.median(rates)), sample, threads, used, np.concatenate(psi_s)


# ---------------------------------------------------------------------------
# 2D driver workloads: the 129 x 65 periodic layer (Ra 1e5, Pr 1, dt 1e-5,
# multigrid to max-norm residual 1e-10) and the rotating annulus of the
# annulus driver's own deck (nr 272, np 1200, Ra 8e8, Re 1.06148e5, Pr 0.71,
# dt 2e-8, tolcon 1e-5).  A cell-update is one (i,k) cell advanced one step.
# ---------------------------------------------------------------------------
LAYER = dict(nr=64, np_=128, dt=1e-5, Ra=1e5, Pr=1.0, r0=0.0, rmax=1.0, xx=2.0, Re=0.0, variant=0,
             tolcon=1e-10, kind=1, amp=1e-3,
             name="2D periodic layer 129 x 65 (nr 64, np 128), Ra 1e5, Pr 1, dt 1e-5, MG to 1e-10")
ANNULUS = dict(nr=272, np_=1200, dt=2e-8, Ra=8e8, Pr=0.71, r0=0.5, rmax=1.0, xx=0.0, Re=1.06148e5, variant=1,
               tolcon=10e-6, kind=0, amp=0.0,
               name="2D rotating annulus (r, phi) nr 272, np 1200, Ra 8e8, Re 1.06148e5, Pr 0.71, dt 2e-8, tolcon 1e-5")


def layer_words(sweeps_mean):
    """FP64 words per cell-update of a step: transport 10, per solve 8 for
    set-up and finalise plus 29.5 per outer multigrid sweep."""
    return 10.0 + sum(8.0 + 29.5 * s for s in sweeps_mean)


def prb_instance(cfg, smoother, seed=0):
    from codesthesis_dir_gb300 import initial, prb
    g = prb.PRB(cfg["nr"], cfg["np_"], dt=cfg["dt"], r0=cfg["r0"], rmax=cfg["rmax"], xx=cfg["xx"] or 3.0,
                Ra=cfg["Ra"], Pr=cfg["Pr"], tolcon=cfg["tolcon"], smoother=smoother, variant=cfg["variant"],
                Re=cfg["Re"])
    for name, a in initial.initial_fields(cfg["nr"], cfg["np_"], cfg["r0"], cfg["rmax"], cfg["variant"],
                                          cfg["kind"], seed, cfg["amp"]).items():
        g.set(name, a)
    return g


def time_prb_gpu(cfg, smoother, steps, warmup, precision=0):
    """Device steps (one CUDA graph per step) timed with CUDA events on the
    instance's own stream.  Returns (cell-updates/s, ms/step, mean sweeps
    [v, u], Nu history of all warm-up and timed steps, final fields)."""
    import torch
    from codesthesis_dir_gb300 import lib
    g = prb_instance(cfg, smoother) if precision == 0 else _prb_mixed_instance(cfg, smoother)
    L = lib.load()
    s = torch.cuda.ExternalStream(L.gb_prb_stream(g._h))
    nu_w = np.zeros((0, 2))
    if warmup:
        nu_w, _ = g.step(warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    nu, sw = g.step(steps)
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    cells = cfg["nr"] * cfg["np_"]
    fields = {n: g.get(n) for n in ("vel", "uel", "C", "th")}
    g.close()
    return cells * steps / (ms / 1e3), ms / steps, sw.mean(axis=0).tolist(), np.concatenate([nu_w, nu]), fields


def _prb_mixed_instance(cfg, smoother):
    from codesthesis_dir_gb300 import initial, prb
    g = prb.PRB(cfg["nr"], cfg["np_"], dt=cfg["dt"], r0=cfg["r0"], rmax=cfg["rmax"], xx=cfg["xx"] or 3.0,
                Ra=cfg["Ra"], Pr=cfg["Pr"], tolcon=cfg["tolcon"], smoother=smoother, variant=cfg["variant"],
                Re=cfg["Re"], precision=1)
    for name, a in initial.initial_fields(cfg["nr"], cfg["np_"], cfg["r0"], cfg["rmax"], cfg["variant"],
                                          cfg["kind"], 0, cfg["amp"]).items():
        g.set(name, a)
    return g


# the CPU oracle that the layer and 3D baselines time equals the reference's
# own Fortran, run on the CPU through a translator of it, bit for bit
PORT_PINNED = ("bit-identical to the reference's Fortran run through a translator of it "
               "(tests/test_reference_runs.py)")


def prb_latency_model(cfg, precision, warmup=20, reps=5):
    """Where a 2D driver step's time goes: after `warmup` graph steps, `reps`
    steps run routine by routine (the reference's loop order, PRB:363-388),
    each routine timed with CUDA events on the instance's stream.  The step
    graph runs the v and u solves side by side, so its critical path is the
    transport routines plus the longer solve; what the graph step takes
    beyond that is launch and dependency latency between its nodes.  The
    solves are timed again from the same right-hand sides on a cluster of 8
    CTAs per equation instead of one CTA, and the two results compared bit
    for bit."""
    import torch
    from codesthesis_dir_gb300 import lib
    g = prb_instance(cfg, 1) if precision == 0 else _prb_mixed_instance(cfg, 1)
    L = lib.load()
    s = torch.cuda.ExternalStream(L.gb_prb_stream(g._h))
    g.step(warmup)
    torch.cuda.synchronize()
    names = ("cvorticity", "temperature", "heat", "rhsv", "rhsu", "poisson2", "poisson3", "update")
    tot = {n: 0.0 for n in names}
    sweeps = {"poisson2": 0, "poisson3": 0}
    one = {"poisson2": 0.0, "poisson3": 0.0}
    each = {"poisson2": [], "poisson3": []}
    same = True

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        r = fn()
        e1.record(s)
        e1.synchronize()
        return e0.elapsed_time(e1), r

    # each routine's events bracket its host call too (the solves read their
    # sweep counts back): a garbage collection inside that call would be
    # counted as routine time, so the collector waits until the loop ends
    import gc
    gc.collect()
    gc.disable()
    try:
        for _ in range(reps):
            for n in names[:5]:
                tot[n] += timed(getattr(g, n))[0]
            snap = {n: g.get(n) for n in ("vel", "velp", "uel", "uelp")}
            for n in ("poisson2", "poisson3"):
                ms, sw = timed(getattr(g, n))
                tot[n] += ms
                each[n].append(ms)
                sweeps[n] += sw
            res = {n: g.get(n) for n in ("vel", "uel")}
            for n, a in snap.items():
                g.set(n, a)
            g.set_solve_spread(8)
            for n in ("poisson2", "poisson3"):
                one[n] += timed(getattr(g, n))[0]
            g.set_solve_spread(1)
            same = same and all(np.array_equal(res[n], g.get(n)) for n in res)
            tot["update"] += timed(g.update)[0]
    finally:
        gc.enable()
    g.close()
    ms = {n: tot[n] / reps for n in names}
    transport = sum(ms[n] for n in names if not n.startswith("poisson"))
    out = {"routine_ms": ms, "transport_ms": transport,
           "solve_ms": {"v": ms["poisson2"], "u": ms["poisson3"]},
           "solve_ms_each_step": {"v": each["poisson2"], "u": each["poisson3"]},
           "sweeps_per_solve": {"v": sweeps["poisson2"] / reps, "u": sweeps["poisson3"] / reps},
           "us_per_sweep": {"v": 1e3 * ms["poisson2"] / max(sweeps["poisson2"] / reps, 1),
                            "u": 1e3 * ms["poisson3"] / max(sweeps["poisson3"] / reps, 1)},
           "critical_ms": transport + max(ms["poisson2"], ms["poisson3"]),
           "solve_share_of_critical": max(ms["poisson2"], ms["poisson3"]) / (
               transport + max(ms["poisson2"], ms["poisson3"])),
           "steps_measured": reps, "after_steps": warmup}
    out["cluster8_solve_ms"] = {"v": one["poisson2"] / reps, "u": one["poisson3"] / reps}
    out["cluster8_speedup"] = {k: out["solve_ms"][k] / out["cluster8_solve_ms"][k] for k in ("v", "u")}
    out["cluster8_bits_equal_one_cta"] = bool(same)
    return out


def time_prb_cpu(cfg, smoother, budget_s=3.0, max_steps=200):
    """The oracle (one core: the reference's loop is serial) on the same
    instance for a bounded number of steps."""
    from oracle import oracle as O
    O.build()
    o = O.OraclePRB(cfg["nr"], cfg["np_"], cfg["dt"], cfg["Ra"], cfg["Pr"], r0=cfg["r0"], rmax=cfg["rmax"],
                    xx=cfg["xx"] or 3.0, mode=smoother, tolcon=cfg["tolcon"], variant=cfg["variant"], Re=cfg["Re"])
    o.initial(cfg["kind"], 0, cfg["amp"])
    t0 = time.perf_counter()
    n = 0
    while n < max_steps and time.perf_counter() - t0 < budget_s:
        st, nu, sw = o.step()
        assert st == 0
        n += 1
    dt = time.perf_counter() - t0
    o.close()
    return cfg["nr"] * cfg["np_"] * n / dt, n, dt


def prb_summary(cfg, steps_zebra, steps_lex, warmup, cpu_budget):
    """FP64 device steps (zebra and the reference's lexicographic order),
    the mixed-precision steps with their error against the FP64 run (which
    is bit-identical to the FP64 oracle), and the CPU oracle."""
    out = {"workload": cfg["name"]}
    runs = {}
    for nm, sm, st, prec in (("fp64_zebra", 1, steps_zebra, 0), ("mixed_zebra", 1, steps_zebra, 1),
                             ("fp64_lex", 0, steps_lex, 0)):
        if st <= 0:
            continue
        v, ms, sw, nu, fields = time_prb_gpu(cfg, sm, st, warmup if sm == 1 else 1, prec)
        runs[nm] = (nu, fields)
        w = layer_words(sw) if prec == 0 else None
        out[nm] = {"value": v, "unit": "cell-updates/s", "ms_per_step": ms, "steps": st,
                   "sweeps_mean_v_u" if prec == 0 else "fp32_cycles_mean_v_u": sw,
                   "nu_last": [float(nu[-1, 0]), float(nu[-1, 1])]}
        if w is not None:
            out[nm].update({"alg_bytes_per_cell_update": 8 * w, "achieved_GBs": 8 * w * v / 1e9})
    if "mixed_zebra" in runs and "fp64_zebra" in runs:
        nu_m, f_m = runs["mixed_zebra"]
        nu_d, f_d = runs["fp64_zebra"]
        m = out["mixed_zebra"]
        m["speedup_vs_fp64"] = m["value"] / out["fp64_zebra"]["value"]
        m["nu_rel_err_vs_fp64"] = float(np.max(np.abs(nu_m - nu_d) / np.abs(nu_d)))
        m["field_rel_l2_vs_fp64"] = {n: float(np.linalg.norm(f_m[n] - f_d[n]) / max(np.linalg.norm(f_d[n]), 1e-300))
                                     for n in f_d}
        m["after_steps"] = int(nu_d.shape[0])
    if cpu_budget > 0:
        v, n, dt = time_prb_cpu(cfg, 0, cpu_budget)
        out["cpu_baseline"] = {"value": v, "unit": "cell-updates/s", "cores": 1, "kind": "port",
                               "sample": "%d steps of the same instance, oracle LEX (the reference schedule), "
                                         "1 thread, %.1f s" % (n, dt), "port_fidelity": PORT_PINNED}
    return out


def run_prb_workload(args, cfg):
    """--workload layer|annulus: one JSON line for the 2D driver step."""
    import torch
    from codesthesis_dir_gb300 import lib
    lib.load()
    peak, peak_kind = measured_peaks()
    with ClockSampler() as clk:
        summ = prb_summary(cfg, args.steps, 0 if args.workload == "annulus" else max(1, args.steps // 20),
                           args.warmup, 0 if args.no_cpu_baseline else 3.0)
    z = summ["fp64_zebra"]
    mx = summ["mixed_zebra"]
    line = {
        "metric": "cell-updates/s (2D driver step, mixed-precision velocity solves; FP64 path beside)",
        "value": mx["value"], "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": mx["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-inner/f64-outer", "data": "synthetic",
        "config": {"workload": cfg["name"], "smoother": "zebra",
                   "l2": "working set (~%.0f MB) fits in L2; steps are latency and FP64-pipe bound" % (
                       20 * (cfg["nr"] + 2) * (cfg["np_"] + 1) * 8 / 1e6)},
        "roofline": {"bound": "hbm", "achieved": z["achieved_GBs"], "peak": peak, "unit": "GB/s",
                     "frac": z["achieved_GBs"] / peak, "traffic": None, "peak_kind": peak_kind},
        "detail": summ,
        "clocks": clk.summary(),
    }
    if args.workload == "layer":
        lm = {"mixed": prb_latency_model(cfg, 1), "fp64": prb_latency_model(cfg, 0)}
        lm["mixed"]["graph_step_ms"] = mx["ms_per_step"]
        lm["fp64"]["graph_step_ms"] = z["ms_per_step"]
        for v in lm.values():
            v["graph_overhead_ms"] = v["graph_step_ms"] - v["critical_ms"]
        line["roofline"]["bound"] = "latency"
        line["roofline"]["note"] = ("8 192 cells: HBM is idle; the step is the transport routines plus the longer "
                                    "of the two side-by-side solves, each a chain of line eliminations")
        line["roofline"]["latency_model"] = lm
    if "cpu_baseline" in summ:
        line["cpu_baseline"] = summ["cpu_baseline"]
    print(json.dumps(line))
    return 0


# The axisymmetric annulus workload (rotann2.f physics): 257 x 257 vertices
# (nr = nz = 256), radius ratio 0.5 and height = gap (r0 0.5, rmax 1, zmax
# 0.5), tanh-stretched toward all four walls with stretch factor 1.5
# (grid.f's weights, rcsc.f's stretched multigrid), Ra 1e8, Ta 1e5 as the
# rotational Reynolds number Re = sqrt(Ta)/2 (Ta = 4 Omega^2 d^4 / nu^2,
# Re = Omega d^2 / nu), Pr 1, dt 2e-7, the conduction profile plus seeded
# noise of amplitude 1e-4.  The multigrid tolerance is 1e-9 (the
# reference's relax uses 1e-6): the field comparison of the mixed and FP64
# paths is only as close as the tolerance the two solves stop at.
AXIWL = dict(nr=256, nz=256, dt=2e-7, r0=0.5, rmax=1.0, zmax=0.5, Ra=1e8, Re=(1e5 ** 0.5) / 2.0, Pr=1.0,
             tolcon=1e-9, amp=1e-4, stretch=1.5,
             name="axisymmetric annulus 257 x 257 (nr = nz = 256), tanh-stretched toward all walls (factor 1.5), "
                  "Ra 1e8, Ta 1e5 (Re 158.1), Pr 1, dt 2e-7, MG tolcon 1e-9")


def axi_grid(cfg):
    from codesthesis_dir_gb300 import axi
    if not cfg.get("stretch"):
        return None
    return axi.stretched_grid(cfg["nr"], cfg["nz"], cfg["r0"], cfg["rmax"], cfg["zmax"], cfg["stretch"])


def axi_initial(cfg, seed=0):
    """Conduction profile plus seeded noise, the oracle's kind-1 start."""
    from codesthesis_dir_gb300 import serve
    G = axi_grid(cfg)
    return serve.axi_initial(cfg["nr"], cfg["nz"], cfg["r0"], cfg["rmax"], seed, cfg["amp"],
                             r=None if G is None else G.r[1])


def time_axi_gpu(cfg, smoother, steps, warmup, precision=0):
    import torch
    from codesthesis_dir_gb300 import axi
    g = axi.AXI(cfg["nr"], cfg["nz"], dt=cfg["dt"], r0=cfg["r0"], rmax=cfg["rmax"], zmax=cfg["zmax"], Ra=cfg["Ra"],
                Re=cfg["Re"], Pr=cfg["Pr"], tolcon=cfg["tolcon"], smoother=smoother, precision=precision,
                grid=axi_grid(cfg))
    for n, a in axi_initial(cfg).items():
        g.set(n, a)
    s = torch.cuda.ExternalStream(g.stream())
    nu_w = np.zeros(0)
    if warmup:
        nu_w, _ = g.step(warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    nu, sw = g.step(steps)
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    done = len(nu)
    fields = {n: g.get(n) for n in ("phi", "omeg", "vel", "theta")}
    g.close()
    cells = (cfg["nr"] + 1) * (cfg["nz"] + 1)
    return cells * done / (ms / 1e3), ms / max(done, 1), float(np.mean(sw)) if done else 0.0, \
        np.concatenate([nu_w, nu]), fields


def axi_summary(cfg, steps, steps_lex, warmup, cpu_budget):
    out = {"workload": cfg["name"]}
    runs = {}
    for nm, sm, st, prec in (("fp64_zebra", 1, steps, 0), ("mixed_zebra", 1, steps, 1), ("fp64_lex", 0, steps_lex, 0)):
        if st <= 0:
            continue
        v, ms, sw, nu, fields = time_axi_gpu(cfg, sm, st, warmup if sm == 1 else 1, prec)
        runs[nm] = (nu, fields)
        out[nm] = {"value": v, "unit": "cell-updates/s", "ms_per_step": ms, "steps": st,
                   ("sweeps_mean" if prec == 0 else "fp32_cycles_mean"): sw, "nu_last": float(nu[-1])}
    if "mixed_zebra" in runs and "fp64_zebra" in runs:
        nu_m, f_m = runs["mixed_zebra"]
        nu_d, f_d = runs["fp64_zebra"]
        m = out["mixed_zebra"]
        m["speedup_vs_fp64"] = m["value"] / out["fp64_zebra"]["value"]
        m["nu_rel_err_vs_fp64"] = float(np.max(np.abs(nu_m - nu_d) / np.abs(nu_d)))
        m["field_rel_l2_vs_fp64"] = {n: float(np.linalg.norm(f_m[n] - f_d[n]) / max(np.linalg.norm(f_d[n]), 1e-300))
                                     for n in f_d}
        m["compared_after_steps"] = int(len(nu_d))
    if cpu_budget > 0:
        from oracle import oracle as O
        O.build()
        o = O.OracleAXI(cfg["nr"], cfg["nz"], cfg["dt"], cfg["r0"], cfg["rmax"], cfg["zmax"], cfg["Ra"], cfg["Re"],
                        cfg["Pr"], mode=0, tolcon=cfg["tolcon"])
        G = axi_grid(cfg)
        if G is not None:
            o.stretch(G.hr[1], G.hz[1])
        o.initial(1, 0, cfg["amp"])
        t0 = time.perf_counter()
        n = 0
        while n < 200 and (n == 0 or time.perf_counter() - t0 < cpu_budget):
            o.step()
            n += 1
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": (cfg["nr"] + 1) * (cfg["nz"] + 1) * n / dt, "unit": "cell-updates/s",
                               "cores": 1, "kind": "port",
                               "sample": "%d steps of the same instance, oracle in the reference's line order, "
                                         "1 thread, %.1f s; %s" % (n, dt, cpu_model()),
                               "port_fidelity": "rotann2.f's physics on grid.f's weights with rcsc.f's multigrid: "
                                                "the parts equal the reference's Fortran bit for bit "
                                                "(tests/test_reference_runs.py); no reference program runs "
                                                "the composition"}
    return out


def run_axi_workload(args):
    from codesthesis_dir_gb300 import lib
    lib.load()
    peak, peak_kind = measured_peaks()
    with ClockSampler() as clk:
        summ = axi_summary(AXIWL, args.steps, max(1, args.steps // 20), args.warmup,
                           0 if args.no_cpu_baseline else 5.0)
    mx, z = summ["mixed_zebra"], summ["fp64_zebra"]
    line = {
        "metric": "cell-updates/s (axisymmetric annulus step, mixed-precision streamfunction solve; FP64 beside)",
        "value": mx["value"], "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": mx["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-inner/f64-outer", "data": "synthetic",
        "config": {"workload": AXIWL["name"], "smoother": "zebra (the stretched multigrid's four colours of lines)",
                   "l2": "working set (~6 MB) fits in L2; the step is latency and FP64-pipe bound"},
        "roofline": {"bound": "hbm", "achieved": None, "peak": peak, "unit": "GB/s", "frac": None, "traffic": None,
                     "peak_kind": peak_kind,
                     "note": "one-block multigrid on a 257 x 257 grid: chain-latency bound, see detail"},
        "detail": summ, "clocks": clk.summary(),
    }
    if "cpu_baseline" in summ:
        line["cpu_baseline"] = summ["cpu_baseline"]
    print(json.dumps(line))
    return 0


R3DWL = dict(nr=64, nz=64, np=128, dt=4e-6, r0=0.5, rmax=1.0, zmax=0.5, Ra=1e6, Re=500.0, Pr=7.0, Gr=0.0, nval=3,
             amp=1e-3,
             name="3D rotating annulus 128 (phi, periodic) x 65 x 65 (nr = nz = 64, np = 128), radius ratio 0.5, "
                  "height/gap 1, Ra 1e6, Ta 1e6 (Re 500), Pr 7, dt 4e-6, MG tolcon 1e-5, mode-3 start amp 1e-3")


def time_r3d_gpu(cfg, smoother, steps, warmup, precision=0):
    import torch
    from codesthesis_dir_gb300 import initial, r3d
    g = r3d.R3D(cfg["nr"], cfg["nz"], cfg["np"], dt=cfg["dt"], r0=cfg["r0"], rmax=cfg["rmax"], zmax=cfg["zmax"],
                Ra=cfg["Ra"], Re=cfg["Re"], Pr=cfg["Pr"], Gr=cfg["Gr"], smoother=smoother, precision=precision)
    f0 = initial.r3d_initial_fields(cfg["nr"], cfg["nz"], cfg["np"], cfg["r0"], cfg["rmax"], cfg["nval"], cfg["amp"])
    for n, a in f0.items():
        g.set(n, a)
    s = torch.cuda.ExternalStream(g.stream())
    nu_w = np.zeros(0)
    if warmup:
        nu_w, _ = g.step(warmup)
    torch.cuda.synchronize()
    g.barrier_counts(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    nu, sw = g.step(steps)
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    done = len(nu)
    bars, blocks = g.barrier_counts()
    fields = {n: g.get(n) for n in ("uel", "vel", "wel", "A", "B", "C", "th")}
    g.close()
    cells = cfg["nr"] * cfg["nz"] * cfg["np"]
    time_r3d_gpu.last_barriers = {"w": bars[0] / max(done, 1), "v": bars[1] / max(done, 1),
                                  "u": bars[2] / max(done, 1), "blocks": blocks}
    return cells * done / (ms / 1e3), ms / max(done, 1), sw.sum(axis=1).mean() if done else 0.0, \
        np.concatenate([nu_w, nu]), fields


def r3d_latency_model(ms_per_step, barriers, threads=256, reps=2000):
    """Barrier term of the 3D step: grid barriers per step (counted on the
    device) times the time of one barrier at the solves' launch shapes
    (measured by a barrier-only cooperative launch).  The w and v solves run
    side by side on half the blocks each, the u solve after them on all, so
    the critical path holds max(w, v) half-grid barriers and the u solve's
    full-grid ones.  What is left of the step is the phases' own work: the
    line elimination chains, the residual passes and the transfers."""
    import ctypes as C
    from codesthesis_dir_gb300 import lib
    L = lib.load()
    full = barriers["blocks"]
    half = max(1, full // 2)
    us = {}
    for nb in (half, full):
        t = C.c_double()
        lib.check(L.gb_measure_grid_barrier(nb, threads, reps, C.byref(t)), "gb_measure_grid_barrier")
        us[nb] = t.value
    crit = max(barriers["w"], barriers["v"]) * us[half] + barriers["u"] * us[full]
    return {"barriers_per_step": {k: barriers[k] for k in ("w", "v", "u")},
            "blocks": {"w_v_side_by_side": half, "u": full},
            "us_per_barrier": {str(half): us[half], str(full): us[full]},
            "barrier_ms_per_step": crit / 1e3, "step_ms": ms_per_step,
            "barrier_share": crit / 1e3 / ms_per_step,
            "rest_ms_per_step": ms_per_step - crit / 1e3,
            "model": "step = max(w, v) x barrier(half grid) + u x barrier(full grid) + phase work "
                     "(elimination chains, residual passes, transfers); barrier counts from the device, barrier "
                     "time from a barrier-only cooperative launch of the same shape"}


def r3d_summary(cfg, steps, steps_fp64, warmup, cpu_budget):
    """Mixed over `steps` steps (the throughput figure); mixed and FP64 two-colour
    over the same `steps_fp64` steps from the same start (speed-up and the
    accuracy of the mixed path against FP64); one step in the reference's
    line order; a bounded CPU sample of the oracle."""
    out = {"workload": cfg["name"]}
    runs = {}
    for nm, sm, st, wu, prec in (("mixed_zebra", 1, steps, warmup, 1), ("mixed_zebra_short", 1, steps_fp64, 0, 1),
                                 ("fp64_zebra", 1, steps_fp64, 0, 0), ("fp64_lex", 0, 1, 0, 0)):
        if st <= 0:
            continue
        v, ms, sw, nu, fields = time_r3d_gpu(cfg, sm, st, wu, prec)
        runs[nm] = (nu, fields)
        out[nm] = {"value": v, "unit": "cell-updates/s", "ms_per_step": ms, "steps": st, "warmup": wu,
                   ("sweeps_per_step" if prec == 0 else "fp32_cycles_per_step"): float(sw),
                   "nu_last": float(nu[-1])}
        if nm in ("mixed_zebra", "fp64_zebra"):
            out[nm]["latency_model"] = r3d_latency_model(ms, time_r3d_gpu.last_barriers)
    if "mixed_zebra_short" in runs and "fp64_zebra" in runs:
        nu_m, f_m = runs["mixed_zebra_short"]
        nu_d, f_d = runs["fp64_zebra"]
        m = out["mixed_zebra"]
        m["speedup_vs_fp64_zebra"] = out["mixed_zebra_short"]["value"] / out["fp64_zebra"]["value"]
        m["speedup_vs_fp64_lex"] = m["value"] / out["fp64_lex"]["value"] if "fp64_lex" in out else None
        m["nu_rel_err_vs_fp64"] = float(np.max(np.abs(nu_m - nu_d) / np.abs(nu_d)))
        m["field_rel_l2_vs_fp64"] = {n: float(np.linalg.norm(f_m[n] - f_d[n]) / max(np.linalg.norm(f_d[n]), 1e-300))
                                     for n in f_d}
        m["compared_after_steps"] = steps_fp64
    if cpu_budget > 0:
        from oracle import oracle as O
        O.build()
        o = O.OracleR3D(cfg["nr"], cfg["nz"], cfg["np"], cfg["dt"], cfg["r0"], cfg["rmax"], cfg["zmax"], cfg["Ra"],
                        cfg["Re"], cfg["Pr"], Gr=cfg["Gr"], mode=0)
        o.initial(cfg["nval"], cfg["amp"])
        t0 = time.perf_counter()
        n = 0
        while n < 200 and (n == 0 or time.perf_counter() - t0 < cpu_budget):
            o.step()
            n += 1
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": cfg["nr"] * cfg["nz"] * cfg["np"] * n / dt, "unit": "cell-updates/s",
                               "cores": 1, "kind": "port",
                               "sample": "%d step(s) of the same instance from the same start, oracle in the "
                                         "reference's line order, 1 thread, %.1f s; %s" % (n, dt, cpu_model()),
                               "port_fidelity": PORT_PINNED}
    return out


def run_r3d_workload(args):
    from codesthesis_dir_gb300 import lib
    lib.load()
    if args.mixed_only:
        v, ms, sw, nu, _ = time_r3d_gpu(R3DWL, 1, args.steps, args.warmup, 1)
        print("r3d mixed: %.4g cell-updates/s, %.1f ms/step, %.1f FP32 cycles/step" % (v, ms, sw))
        return 0
    with ClockSampler() as clk:
        summ = r3d_summary(R3DWL, args.steps, args.r3d_fp64_steps, args.warmup, 0 if args.no_cpu_baseline else 30.0)
    mx = summ["mixed_zebra"]
    line = {
        "metric": "cell-updates/s (3D rotating annulus step, mixed-precision velocity solves; FP64 beside)",
        "value": mx["value"], "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": mx["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-inner/f64-outer", "data": "synthetic",
        "config": {"workload": R3DWL["name"], "smoother": "zebra",
                   "l2": "working set (~120 MB) fits in L2; the solves are phase-latency bound"},
        "roofline": {"bound": "latency", "achieved": None, "peak": None, "unit": None, "frac": None, "traffic": None,
                     "note": "each relaxation phase costs the elimination chain of its longest line plus one grid "
                             "barrier; HBM and the FP64 pipe are far from busy",
                     "latency_model": mx.get("latency_model")},
        "detail": summ, "clocks": clk.summary(),
    }
    if "cpu_baseline" in summ:
        line["cpu_baseline"] = summ["cpu_baseline"]
    print(json.dumps(line))
    return 0


def run_serve_workload(args):
    """--workload serve: the parameter sweep served by continuous batching,
    FP64 and mixed precision on the same arrivals.  512 requests (layer or
    annulus), the four grids, Ra, Pr and Ta drawn as stated, Poisson
    arrivals at 50/s, 120 GB budget; --serve-steps bounds the per-request
    step range (500-5000 as stated by default).  --serve-mode gang (default)
    steps all active requests of a kind as one gang (one launch per phase
    across their grids); --serve-mode streams runs each request on its own
    stream (the per-instance loop) for comparison."""
    from codesthesis_dir_gb300 import lib, serve
    lib.load()
    lo, hi = (int(x) for x in args.serve_steps.split(","))
    reqs = serve.sweep_requests(n=args.requests, rate=50.0, seed=0, steps=(lo, hi))
    out, res_by = {}, {}
    with ClockSampler() as clk:
        for name, prec in (("mixed", lib.PRB_MIXED), ("fp64", lib.PRB_FP64)):
            if args.serve_mode == "gang":
                srv = serve.GangServer(budget_bytes=120e9, max_active=args.max_active, chunk=args.serve_chunk,
                                       precision=prec, group_by=args.serve_group,
                                       solve_spread=args.serve_spread)
            else:
                srv = serve.Server(budget_bytes=120e9, max_active=args.max_active, chunk=16, precision=prec)
            t0 = time.perf_counter()
            res = srv.run(reqs)
            res_by[name] = res
            out[name] = serve.summarize(reqs, res)
            out[name]["wall_s"] = time.perf_counter() - t0
            out[name]["peak_active"] = srv.peak_active
            out[name]["peak_device_bytes_estimate"] = srv.peak_bytes
            if args.serve_mode == "gang":
                out[name]["gang_rebuilds"] = srv.rebuilds
                out[name]["gang_chunks"] = srv.chunks
    errs = []
    for a, b in zip(res_by["fp64"], res_by["mixed"]):
        if a.status == 0 and b.status == 0 and len(a.nu) and len(b.nu) == len(a.nu):
            errs.append(float(np.max(np.abs(b.nu - a.nu) / np.maximum(np.abs(a.nu), 1e-300))))
    m, f = out["mixed"], out["fp64"]
    line = {
        "metric": "served solves/s and p50/p99 time to solution (parameter sweep, mixed precision; FP64 beside)",
        "value": m["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": len(reqs), "warmup": 0,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-inner/f64-outer", "data": "synthetic",
        "config": {"workload": "served sweep: %d requests (layer or annulus), grids 65x33..513x257, Ra 1e4-1e8, "
                               "Pr {0.7,1,7}, Ta 1-1e6, %d-%d steps, Poisson arrivals 50/s, 120 GB budget" % (
                                   len(reqs), lo, hi),
                   "mode": args.serve_mode, "group_by": args.serve_group, "solve_spread": args.serve_spread,
                   "max_active": args.max_active,
                   "chunk_steps": args.serve_chunk if args.serve_mode == "gang" else 16},
        "served": out,
        "mixed_vs_fp64": {"solves_per_s_ratio": m["solves_per_s"] / f["solves_per_s"],
                          "cell_updates_ratio": m["cell_updates_per_s"] / f["cell_updates_per_s"],
                          "p50_ratio": f["tts_p50_s"] / m["tts_p50_s"], "p99_ratio": f["tts_p99_s"] / m["tts_p99_s"],
                          "nu_max_rel_err": max(errs) if errs else None, "requests_compared": len(errs)},
        "clocks": clk.summary(),
    }
    print(json.dumps(line))
    return 0


def run_reference(args):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    sizes = workload_sizes(0)
    vals = []
    threads = os.cpu_count()
    sample = ""
    for s in range(args.warmup + args.steps):
        v, sample, threads, _, _ = cpu_reference(sizes, 0, budget_s=max(2.0, args.ref_budget), threads=threads)
        if s >= args.warmup:
            vals.append(v)
    value = float(np.median(vals))
    total = int(np.sum(sizes.astype(np.int64) ** 2))
    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": batch_config(total, int(np.sum(interior(sizes))), ws),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ref-budget", type=float, default=20.0)
    ap.add_argument("--inner", type=int, default=3, help="FP32 V-cycles per defect-correction step")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner: default tunables, --inner")
    ap.add_argument("--pair-outer", action="store_true",
                    help="headline the float-pair defect correction (GB_BATCH_MIXED) instead of the FP64 one")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mixed-only", action="store_true",
                    help="time only the mixed solve (for profiler launch lists); prints no JSON line")
    ap.add_argument("--fp64-only", action="store_true",
                    help="time only the plain FP64 solve (for profiler captures); prints no JSON line")
    ap.add_argument("--no-layer", action="store_true", help="skip the 2D layer step measurement of the default run")
    ap.add_argument("--requests", type=int, default=512, help="serve workload: number of requests")
    ap.add_argument("--serve-steps", default="500,5000", help="serve workload: step range lo,hi")
    ap.add_argument("--max-active", type=int, default=1024, help="serve workload: active slots")
    ap.add_argument("--serve-mode", default="gang", choices=["gang", "streams"],
                    help="serve workload: one gang per kind (batched across sizes) or one stream per request")
    ap.add_argument("--serve-chunk", type=int, default=32, help="serve workload: gang steps between re-gangings")
    ap.add_argument("--serve-spread", type=int, default=8, choices=[1, 8],
                    help="serve workload: CTAs per velocity solve of the layer gangs")
    ap.add_argument("--serve-group", default="kind", choices=["kind", "shape"],
                    help="serve workload: one gang per kind (across sizes) or per kind and grid")
    ap.add_argument("--r3d-fp64-steps", type=int, default=10, help="r3d workload: FP64 comparison steps")
    ap.add_argument("--workload", default="batch", choices=["batch", "layer", "annulus", "axi", "serve", "r3d"],
                    help="batch: 256 batched Poisson problems (the headline); layer / annulus: the 2D driver step")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "axi":
        return run_axi_workload(args)
    if args.workload == "serve":
        return run_serve_workload(args)
    if args.workload == "r3d":
        return run_r3d_workload(args)
    if args.workload != "batch":
        return run_prb_workload(args, LAYER if args.workload == "layer" else ANNULUS)

    import torch

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from codesthesis_dir_gb300 import lib
    from codesthesis_dir_gb300.batch import BatchPoisson
    lib.load()

    sizes = workload_sizes(0)
    f_host = workload_rhs(sizes, rank)
    total = int(np.sum(sizes.astype(np.int64) ** 2))
    cu_per_cycle = interior(sizes)
    d_f = torch.from_numpy(f_host).cuda()
    d_psi = torch.zeros(total, dtype=torch.float64, device="cuda")
    d_psi64 = torch.zeros(total, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    def timed(solver, d_out, steps, warmup):
        for _ in range(warmup):
            st, cyc, rr = solver.solve_device(d_f.data_ptr(), d_out.data_ptr(), sh)
            assert st == 0, lib.last_error()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        cu, launches = 0.0, 0
        with torch.cuda.stream(stream):
            e0.record(stream)
        for _ in range(steps):
            st, cyc, rr = solver.solve_device(d_f.data_ptr(), d_out.data_ptr(), sh)
            assert st == 0, lib.last_error()
            cu += float(np.sum(cu_per_cycle * cyc))
            launches += solver.last_launches()
        with torch.cuda.stream(stream):
            e1.record(stream)
        barrier()
        ms = e0.elapsed_time(e1)
        if ws > 1:
            import torch.distributed as dist
            t = torch.tensor([ms, cu], dtype=torch.float64, device="cuda")
            mx = t.clone()
            dist.all_reduce(mx, op=dist.ReduceOp.MAX)
            dist.all_reduce(t, op=dist.ReduceOp.SUM)
            ms, cu = float(mx[0]), float(t[1])
        return ms, cu, cyc, rr, launches

    prec_head = lib.BATCH_MIXED if args.pair_outer else lib.BATCH_MIXED_F64OUTER
    # autotuned tunables of each arm (outside the timed region; V(2,2) kept)
    tuning = {"mixed": None, "fp64": None}
    if not args.no_tune:
        from codesthesis_dir_gb300.batch import autotune
        t0 = time.perf_counter()
        best, table, hit = autotune(sizes, prec_head, d_f.data_ptr(), d_psi.data_ptr(), rtol=RTOL, reps=2)
        tuning["mixed"] = dict(best, candidates=len(table), from_cache=hit,
                               top5=sorted(table, key=lambda t: t["ms"])[:5])
        best64, table64, hit64 = autotune(sizes, lib.BATCH_FP64, d_f.data_ptr(), d_psi64.data_ptr(), rtol=RTOL, reps=2)
        tuning["fp64"] = dict(best64, candidates=len(table64), from_cache=hit64)
        tuning["tuning_s"] = time.perf_counter() - t0
    tm = {k: tuning["mixed"][k] for k in ("nu1", "nu2", "inner", "local_n", "fuse", "exec")} if tuning["mixed"] \
        else dict(nu1=2, nu2=2, inner=args.inner, local_n=65, fuse=2, exec=lib.BATCH_EXEC_GRAPH)
    t64 = {k: tuning["fp64"][k] for k in ("nu1", "nu2", "inner", "local_n", "fuse", "exec")} if tuning["fp64"] \
        else dict(nu1=2, nu2=2, inner=1, local_n=65, fuse=1, exec=lib.BATCH_EXEC_GRAPH)
    mixed = BatchPoisson(sizes, precision=prec_head, rtol=RTOL, tuning=tm)
    if args.fp64_only:
        fp64 = BatchPoisson(sizes, precision=lib.BATCH_FP64, rtol=RTOL, tuning=t64)
        ms, cu, cyc, rr, launches = timed(fp64, d_psi64, args.steps, args.warmup)
        if rank == 0:
            print("fp64-only: %.3f ms/step, %.4g cell-updates/s, cycles %s, launches %d" % (
                ms / max(1, args.steps), cu / (ms / 1e3) if ms > 0 else 0.0, np.bincount(cyc), launches))
        return 0
    if args.mixed_only:
        ms, cu, cyc, rr, launches = timed(mixed, d_psi, args.steps, args.warmup)
        if rank == 0:
            print("mixed-only: %.3f ms/step, %.4g cell-updates/s, cycles %s, launches %d" % (
                ms / max(1, args.steps), cu / (ms / 1e3) if ms > 0 else 0.0, np.bincount(cyc), launches))
        return 0
    fp64 = BatchPoisson(sizes, precision=lib.BATCH_FP64, rtol=RTOL, tuning=t64)

    # plain FP64 arm
    ms64, cu64, cyc64, rr64, _ = timed(fp64, d_psi64, args.steps, args.warmup)
    # mixed arm (headline: FP64 defect correction), clocks sampled during
    # it, its level-0 operations timed with CUDA events on the solve stream
    L = lib.load()
    # per-kernel CUDA events exist in the graph execution mode: a persistent
    # winner is profiled by a graph-mode twin.  The headline steps run
    # without them (an event between two kernels also stops the next
    # kernel's launch from overlapping the previous one's last blocks); the
    # same steps then run again with the events, inside the same clock
    # sampling, for the per-kernel times of the roofline.
    prof = mixed if tm["exec"] == lib.BATCH_EXEC_GRAPH else \
        BatchPoisson(sizes, precision=prec_head, rtol=RTOL, tuning=dict(tm, exec=lib.BATCH_EXEC_GRAPH))
    with ClockSampler(local) as clk:
        ms, cu, cyc, rr, launches = timed(mixed, d_psi, args.steps, 0)
        L.gb_batch_profile(prof._h, 1)
        timed(prof, d_psi, 0, args.warmup)
        L.gb_batch_profile_read(prof._h, None, None, None, 1)
        prof_ms = timed(prof, d_psi, args.steps, 0)[0]
    import ctypes as C
    pms, pl, pb = C.c_double(), C.c_longlong(), C.c_double()
    L.gb_batch_profile_read(prof._h, C.byref(pms), C.byref(pl), C.byref(pb), 0)
    kinds = {}
    for kname, kid in (("down_finest", 1), ("up_finest", 2), ("outer", 4), ("outer_first", 7)):
        kms, kl, kb = C.c_double(), C.c_longlong(), C.c_double()
        L.gb_batch_profile_read_kind(prof._h, kid, C.byref(kms), C.byref(kl), C.byref(kb))
        if kl.value:
            kinds[kname] = {"launches": kl.value, "avg_ms": kms.value / kl.value,
                            "alg_bytes_per_launch": kb.value / kl.value,
                            "achieved_GBs": kb.value / (kms.value / 1e3) / 1e9 if kms.value > 0 else None}
    L.gb_batch_profile_read(prof._h, None, None, None, 1)
    L.gb_batch_profile(prof._h, 0)
    r64, r32 = C.c_double(), C.c_double()
    L.gb_measure_issue_rates(C.byref(r64), C.byref(r32))
    outer_pass = None
    if "outer" in kinds:
        # per interior point of an outer pass after a solve's first, FP64
        # defect correction: 3 adds and 2 fused multiply-adds for the
        # residual, 1 fused multiply-add for the norm; 16 B read (psi, f),
        # 4 B written (the FP32 right-hand side).  The first pass of each
        # solve (f read alone) is profiled apart as "outer_first".
        k = kinds["outer"]
        pts_per_launch = k["alg_bytes_per_launch"] / 20.0
        f64ops = 3 + 2 + 1 if prec_head == lib.BATCH_MIXED_F64OUTER else 1
        outer_pass = {"kernel": "k_op<float,OP_OUTER,0,%s> (%s)" % (
                          "CM_F64" if prec_head == lib.BATCH_MIXED_F64OUTER else "CM_PAIR",
                          "FP64 residual and norm, FP32 copy" if prec_head == lib.BATCH_MIXED_F64OUTER
                          else "float-pair residual, FP64 norm, FP32 copy"),
                      "points_per_launch": pts_per_launch,
                      "points_per_s": pts_per_launch / (k["avg_ms"] / 1e3), "avg_launch_ms": k["avg_ms"],
                      "fp64_instr_per_point": f64ops,
                      "fp64_pipe_frac": f64ops * pts_per_launch / (k["avg_ms"] / 1e3) / r64.value,
                      "fp64_fma_peak_per_s": r64.value, "fp32_fma_peak_per_s": r32.value,
                      "peak_kind": "measured (FMA issue probe, gb_measure_issue_rates)"}

    # the float-pair defect correction (outer residual in ~48-bit float
    # pairs on the FP32 pipe) beside the headline, on the same inputs
    pair = None
    if prec_head != lib.BATCH_MIXED:
        pr = BatchPoisson(sizes, precision=lib.BATCH_MIXED, rtol=RTOL, tuning=tm)
        d_psi_q = torch.zeros_like(d_psi)
        ms_q, cu_q, cyc_q, rr_q, _ = timed(pr, d_psi_q, args.steps, args.warmup)
        pair = {"value": cu_q / (ms_q / 1e3), "ms_per_step": ms_q / args.steps, "cycles_mean": float(np.mean(cyc_q)),
                "relres_max": float(np.max(rr_q)),
                "field_rel_l2_vs_fp64": float((torch.linalg.vector_norm(d_psi_q - d_psi64) /
                                               torch.linalg.vector_norm(d_psi64)).item()),
                "dtype": "f32-inner/f32-pair-outer (f64 result)",
                "note": "outer residual in float-pair arithmetic (about 48 significand bits), not FP64"}
        pr.close()
        del d_psi_q

    # the same mixed solve as one persistent launch per solve
    pers = BatchPoisson(sizes, precision=prec_head, rtol=RTOL, tuning=dict(tm, exec=lib.BATCH_EXEC_PERSISTENT))
    d_psi_p = torch.zeros_like(d_psi)
    ms_p, cu_p, _, _, _ = timed(pers, d_psi_p, max(3, args.steps // 4), 1)
    pers_same = bool(torch.equal(d_psi_p, d_psi))
    pers.close()
    del d_psi_p

    # accuracy of the mixed path against the FP64 path (bit-identical to the FP64 oracle)
    a, b = d_psi.cpu().numpy(), d_psi64.cpu().numpy()
    field_err = float(np.linalg.norm(a - b) / np.linalg.norm(b))

    # e2e: host buffers (pinned), copies inside the timed region, through the C ABI
    h_f = torch.from_numpy(f_host).pin_memory()
    h_psi = torch.zeros(total, dtype=torch.float64).pin_memory()
    cycp = np.zeros(len(sizes), dtype=np.int32)
    rrp = np.zeros(len(sizes))
    for _ in range(1):
        L.gb_batch_solve_host(mixed._h, h_f.data_ptr(), h_psi.data_ptr(), cycp.ctypes.data, rrp.ctypes.data)
    barrier()
    t0 = time.perf_counter()
    serial_cu = 0.0
    for _ in range(args.steps):
        st = L.gb_batch_solve_host(mixed._h, h_f.data_ptr(), h_psi.data_ptr(), cycp.ctypes.data, rrp.ctypes.data)
        assert st == 0, lib.last_error()
        serial_cu += float(np.sum(cu_per_cycle * cycp))
    barrier()
    serial_s = time.perf_counter() - t0
    # the same steps as a stream of calls (gb_batch_submit_host): each step
    # still uploads its f and downloads its psi, the copies overlapping the
    # neighbouring steps' solves; two psi buffers, cycle counts per step
    h_psi2 = [h_psi, torch.zeros(total, dtype=torch.float64).pin_memory()]
    cyc_k = [np.zeros(len(sizes), dtype=np.int32) for _ in range(args.steps)]
    rr_k = [np.zeros(len(sizes)) for _ in range(args.steps)]
    # warm-up of the stream path (its first call sets up the staging buffers)
    for k in range(2):
        st = L.gb_batch_submit_host(mixed._h, h_f.data_ptr(), h_psi2[k & 1].data_ptr(), cyc_k[k].ctypes.data,
                                    rr_k[k].ctypes.data)
        assert st == 0, lib.last_error()
    assert L.gb_batch_drain(mixed._h) == 0, lib.last_error()
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        st = L.gb_batch_submit_host(mixed._h, h_f.data_ptr(), h_psi2[k & 1].data_ptr(), cyc_k[k].ctypes.data,
                                    rr_k[k].ctypes.data)
        assert st == 0, lib.last_error()
    st = L.gb_batch_drain(mixed._h)
    assert st == 0, lib.last_error()
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_cu = float(sum(np.sum(cu_per_cycle * c) for c in cyc_k))
    assert np.array_equal(h_psi2[0].numpy(), h_psi2[1].numpy()) or args.steps < 2
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_s, e2e_cu, serial_s, serial_cu], dtype=torch.float64, device="cuda")
        mx = t.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        e2e_s, e2e_cu, serial_s, serial_cu = float(mx[0]), float(t[1]), float(mx[2]), float(t[3])

    if rank != 0:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return 0

    peak, peak_kind = measured_peaks()
    achieved = (pb.value / (pms.value / 1e3)) / 1e9 if pms.value > 0 else None
    # DRAM bytes per launch of the same kernel from one ncu capture (the
    # profile summary named below); ncu cannot run inside a timed bench
    traffic, traffic_src = None, None
    tp = os.path.join(ROOT, "profiles", "batch_down_finest_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            tj = json.load(f)
        traffic = tj.get("dram_bytes_per_launch")
        traffic_src = "%s (%s)" % (tj.get("summary"), tj.get("captured"))
    # whole-solve algorithmic bandwidth: 24.7 words of the inner precision
    # per interior point per V-cycle (every level's sweeps, residuals and
    # transfers) plus the outer passes
    solve_gbs = cu * 24.7 * 4.0 / (ms / 1e3) / 1e9
    line = {
        "metric": METRIC,
        "value": cu / (ms / 1e3),
        "unit": "cell-updates/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32-inner/f64-outer" if prec_head == lib.BATCH_MIXED_F64OUTER
                 else "f32-inner/f32-pair-outer (f64 result)",
        "data": "synthetic",
        "config": batch_config(total, int(np.sum(cu_per_cycle)), ws),
        "fp64": {"value": cu64 / (ms64 / 1e3), "ms_per_step": ms64 / args.steps,
                 "cycles_mean": float(np.mean(cyc64)), "relres_max": float(np.max(rr64)),
                 "achieved_GBs_alg": cu64 * 24.7 * 8.0 / (ms64 / 1e3) / 1e9,
                 "hbm_frac_alg": cu64 * 24.7 * 8.0 / (ms64 / 1e3) / 1e9 / peak},
        "mixed": {"precision": "GB_BATCH_MIXED_F64OUTER" if prec_head == lib.BATCH_MIXED_F64OUTER
                  else "GB_BATCH_MIXED",
                  "cycles_mean": float(np.mean(cyc)), "relres_max": float(np.max(rr)),
                  "inner_cycles_per_fp64_step": tm["inner"],
                  "field_rel_l2_vs_fp64": field_err, "speedup_vs_fp64": (cu / ms) / (cu64 / ms64),
                  "time_to_solution_speedup_vs_fp64": ms64 / ms},
        "mixed_pair_outer": pair,
        "tuning": dict(tuning, used_mixed=tm, used_fp64=t64,
                       search="gb_batch_autotune: inner 2..5 x local_n {33,65,129} x fuse {1,2} x graph/persistent "
                              "(FP64: local_n {33,65} x fuse {1,2} x graph/persistent), V(2,2), time to solution "
                              "by CUDA events"),
        "persistent_single_launch": {"value": cu_p / (ms_p / 1e3), "ms_per_step": ms_p / max(3, args.steps // 4),
                                     "identical_to_graph_mode": pers_same},
        "e2e": {"value": e2e_cu / e2e_s, "unit": "cell-updates/s", "h2d_bytes_per_step": total * 8,
                "d2h_bytes_per_step": total * 8,
                "api": "gb_batch_submit_host/gb_batch_drain (a stream of steps; copies overlap the neighbouring "
                       "steps' solves)",
                "serial_value": serial_cu / serial_s,
                "serial_api": "gb_batch_solve_host (one step per call: copy in, solve, copy out)"},
        "roofline": {"bound": "hbm",
                     "kernel": "k_op<float,OP_SMOOTH_R,2> (finest level: two red-black sweeps + residual + restriction)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "traffic_unit": "bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)",
                     "traffic_source": traffic_src,
                     "peak_kind": peak_kind, "launches": pl.value,
                     "avg_launch_ms": (pms.value / pl.value) if pl.value else None,
                     "alg_bytes_per_launch": (pb.value / pl.value) if pl.value else None,
                     "kernel_times_from": "the same steps run again with an event around each level-0 operation "
                                          "(%.3f ms per step with the events)" % (prof_ms / max(1, args.steps)),
                     "whole_solve": {"achieved": solve_gbs, "frac": solve_gbs / peak, "unit": "GB/s",
                                     "basis": "24.7 FP32 words per interior point per V-cycle"}},
        "outer_pass": outer_pass,
        "kernels_mixed_graph": kinds,
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        v, sample, threads, used, psi_ref = cpu_reference(sizes, rank, budget_s=args.ref_budget, reps=5)
        offs = np.concatenate([[0], np.cumsum(sizes.astype(np.int64) ** 2)])
        got = np.concatenate([a[offs[j]:offs[j + 1]] for j in used])
        line["cpu_baseline"] = {"value": v, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                                "sample": sample}
        line["mixed"]["field_rel_l2_vs_fp64_oracle_sample"] = float(np.linalg.norm(got - psi_ref) /
                                                                     np.linalg.norm(psi_ref))
    if not args.no_layer:
        # the 129 x 65 layer workload's step (FP64 device path) beside the CPU oracle
        line["layer_config0"] = prb_summary(LAYER, 60, 3, 3, 0.0 if args.no_cpu_baseline else 3.0)
        line["layer_config0"]["latency_model"] = {"mixed": prb_latency_model(LAYER, 1),
                                                  "fp64": prb_latency_model(LAYER, 0)}
        # the 3D annulus step (mixed path, 20 steps after 3 of warm-up) with its barrier model
        v, ms, sw, _, _ = time_r3d_gpu(R3DWL, 1, 20, 3, 1)
        line["r3d_config4"] = {"workload": R3DWL["name"], "value": v, "unit": "cell-updates/s", "ms_per_step": ms,
                               "steps": 20, "warmup": 3, "fp32_cycles_per_step": float(sw),
                               "latency_model": r3d_latency_model(ms, time_r3d_gpu.last_barriers)}
    print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
