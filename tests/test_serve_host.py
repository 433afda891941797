"""Host logic of the served loop (codesthesis_dir_gb300.serve) on the CPU,
with stand-in instances and a virtual clock: arrival-order admission,
the memory budget and the slot limit are respected, every request gets
exactly its steps in chunks, and the results carry the right timings."""
import numpy as np

from codesthesis_dir_gb300 import serve


class Clock:
    def __init__(self):
        self.t = 0.0

    def now(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-4)


class FakeInstance:
    """Each queued step takes 1 ms of virtual time."""
    log = []

    def __init__(self, req, clock):
        self.req, self.clock = req, clock
        self.busy_until = 0.0
        self.done = 0
        FakeInstance.log.append(("admit", req.rid, clock.t))

    def begin(self, total):
        self.total = total

    def enqueue(self, n):
        self.busy_until = max(self.busy_until, self.clock.t) + 1e-3 * n
        self.done += n

    def query(self):
        return 1 if self.clock.t >= self.busy_until else 0

    def end(self, n):
        return 0, np.arange(self.done, dtype=float), self.done

    def fields(self):
        return {}

    def close(self):
        FakeInstance.log.append(("close", self.req.rid, self.clock.t))


def test_admission_chunks_and_timings():
    clock = Clock()
    FakeInstance.log = []
    reqs = serve.sweep_requests(n=40, rate=200.0, seed=3, steps=(5, 60), grids=((64, 32), (128, 64)))
    srv = serve.Server(budget_bytes=8 * serve.estimate_bytes(reqs[0]), max_active=3, chunk=7,
                       factory=lambda r: FakeInstance(r, clock), clock=clock.now, sleep=clock.sleep)
    res = srv.run(reqs)
    assert [r.rid for r in res] == [q.rid for q in reqs]
    assert srv.peak_active <= 3
    assert srv.peak_bytes <= srv.budget
    admits = [rid for kind, rid, t in FakeInstance.log if kind == "admit"]
    assert admits == sorted(admits)                      # arrival (= rid) order
    for q, r in zip(reqs, res):
        assert r.status == 0 and r.steps_done == q.steps
        assert r.admit >= q.arrival - 1e-12 and r.finish >= r.admit + 1e-3 * q.steps - 1e-9
        assert abs(r.tts - (r.finish - q.arrival)) < 1e-12
    s = serve.summarize(reqs, res)
    assert s["completed"] == 40 and s["tts_p99_s"] >= s["tts_p50_s"] > 0


def test_memory_budget_limits_concurrency():
    clock = Clock()
    reqs = serve.sweep_requests(n=12, rate=1e6, seed=1, steps=(20, 20), grids=((128, 64),))
    one = max(serve.estimate_bytes(q) for q in reqs)
    srv = serve.Server(budget_bytes=2 * one, max_active=100, chunk=5,
                       factory=lambda r: FakeInstance(r, clock), clock=clock.now, sleep=clock.sleep)
    srv.run(reqs)
    assert srv.peak_active <= 2 and srv.peak_bytes <= 2 * one


def test_sweep_draws():
    reqs = serve.sweep_requests(n=512, rate=50.0, seed=0)
    arr = np.array([q.arrival for q in reqs])
    assert np.all(np.diff(arr) > 0) and 8.0 < arr[-1] < 13.0       # ~512/50 s
    assert {q.kind for q in reqs} == {serve.LAYER, serve.AXI}
    assert all(1e4 <= q.Ra <= 1e8 and q.Pr in (0.7, 1.0, 7.0) and 500 <= q.steps <= 5000 for q in reqs)
    assert all((q.Ta == 0.0) == (q.kind == serve.LAYER) for q in reqs)
    assert all(1.0 <= q.Ta <= 1e6 for q in reqs if q.kind == serve.AXI)
    assert all(serve.default_dt(q) > 0 for q in reqs)


class FakeGang:
    """Stands in for gb_*_gang: a chunk of n steps advances every member by
    n steps, stopping each at its own step count, and takes 1 ms of virtual
    time per step."""
    log = []

    def __init__(self, kind, clock):
        self.kind, self.clock = kind, clock
        self.members = None
        self.busy_until = 0.0

    def build(self, members):
        self.members = list(members)
        FakeGang.log.append(("build", self.kind, sorted(m.req.rid for m in members), self.clock.t))

    def built(self):
        return self.members is not None

    def enqueue(self, n):
        for m in self.members:
            m.inst.done = min(m.req.steps, m.inst.done + n)
        self.busy_until = max(self.busy_until, self.clock.t) + 1e-3 * n

    def query(self):
        return 1 if self.clock.t >= self.busy_until else 0

    def close(self):
        self.members = None


def test_gang_server_host_logic():
    """Every request gets exactly its steps (the layer's first step on its
    own, the rest in chunks of its gang), members join and leave only between
    chunks, gangs hold one kind (or one kind and grid), the budget and slot
    cap hold, and each result is reported once."""
    for group_by in ("kind", "shape"):
        clock = Clock()
        FakeInstance.log, FakeGang.log = [], []
        reqs = serve.sweep_requests(n=60, rate=300.0, seed=5, steps=(3, 90), grids=((64, 32), (128, 64)))
        srv = serve.GangServer(budget_bytes=12 * serve.estimate_bytes(reqs[0]), max_active=9, chunk=8,
                               factory=lambda r: FakeInstance(r, clock), gang_factory=lambda k: FakeGang(k, clock),
                               clock=clock.now, sleep=clock.sleep, group_by=group_by)
        res = srv.run(reqs)
        assert [r.rid for r in res] == [q.rid for q in reqs]
        by = {q.rid: q for q in reqs}
        for r in res:
            assert r.status == 0 and r.steps_done == by[r.rid].steps
            assert r.finish >= r.admit >= by[r.rid].arrival
        assert srv.peak_active <= 9 and srv.peak_bytes <= srv.budget
        for ev, kind, rids, _ in FakeGang.log:
            assert {by[i].kind for i in rids} == {kind}
            if group_by == "shape":
                assert len({(by[i].nx, by[i].nz) for i in rids}) == 1
        closes = [e for e in FakeInstance.log if e[0] == "close"]
        assert sorted(e[1] for e in closes) == sorted(q.rid for q in reqs)
