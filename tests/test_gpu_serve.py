"""The served loop on the device: a mix of layer and annulus requests on
several grids, admitted three at a time and advanced in chunks of steps on
their own streams, gives every request the fields and Nusselt history it
gets when served alone (bit for bit), in FP64 and in mixed precision, and
reports p50 / p99 time to solution."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests():
    from codesthesis_dir_gb300 import serve
    shapes = ((serve.LAYER, 64, 32, 1e4, 0.0), (serve.AXI, 64, 32, 1e5, 10.0), (serve.LAYER, 128, 64, 1e6, 0.0),
              (serve.AXI, 64, 32, 1e6, 1e3), (serve.LAYER, 64, 32, 1e4, 0.0), (serve.AXI, 128, 64, 1e5, 1.0))
    return [serve.Request(i, k, nx, nz, Ra=Ra, Pr=(0.7, 1.0, 7.0)[i % 3], Ta=Ta, steps=12 + 7 * i, seed=50 + i,
                          arrival=0.002 * i)
            for i, (k, nx, nz, Ra, Ta) in enumerate(shapes)]


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_mix_equals_alone(gblib, precision):
    from codesthesis_dir_gb300 import serve
    reqs = _requests()
    mix = serve.Server(max_active=3, chunk=5, keep_fields=True, precision=precision).run(reqs)
    assert all(r.status == 0 for r in mix), [(r.rid, r.status) for r in mix]
    for q, r in zip(reqs, mix):
        alone = serve.Server(max_active=1, chunk=1000, keep_fields=True, precision=precision).run(
            [serve.Request(**{**q.__dict__, "arrival": 0.0})])[0]
        assert r.steps_done == alone.steps_done > 0
        np.testing.assert_array_equal(r.nu, alone.nu)
        for n in r.fields:
            np.testing.assert_array_equal(r.fields[n], alone.fields[n], err_msg="%d %s" % (q.rid, n))
    s = serve.summarize(reqs, mix)
    assert s["completed"] == len(reqs) and s["tts_p99_s"] >= s["tts_p50_s"] > 0


@pytest.mark.parametrize("spread", [1, 8], ids=["cta", "cluster"])
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_gang_server_mix_equals_alone(gblib, precision, spread):
    """The gang server batches the active requests of each kind into one
    set of launches per step across their different grids; every request
    still gets exactly the fields and Nusselt history it gets alone, also
    when its step count is not a multiple of the chunk (the gang stops it at
    its own count) and when members join and leave between chunks; the
    layer gangs' solves on one CTA or a cluster of 8 per equation."""
    from codesthesis_dir_gb300 import serve
    reqs = _requests()
    srv = serve.GangServer(max_active=4, chunk=5, keep_fields=True, precision=precision, solve_spread=spread)
    mix = srv.run(reqs)
    assert all(r.status == 0 for r in mix), [(r.rid, r.status) for r in mix]
    assert srv.rebuilds >= 2
    for q, r in zip(reqs, mix):
        alone = serve.Server(max_active=1, chunk=1000, keep_fields=True, precision=precision).run(
            [serve.Request(**{**q.__dict__, "arrival": 0.0})])[0]
        assert r.steps_done == alone.steps_done == q.steps
        np.testing.assert_array_equal(r.nu, alone.nu)
        for n in r.fields:
            np.testing.assert_array_equal(r.fields[n], alone.fields[n], err_msg="%d %s" % (q.rid, n))


def test_gang_member_limits_and_launch_count(gblib):
    """A PRB gang of three layers on different grids: each member stops at its
    own step count inside a longer run of gang steps, and a gang step is a
    fixed number of launches whatever the number of members."""
    import ctypes as C
    from codesthesis_dir_gb300 import initial, lib, prb
    L = lib.load()
    shapes = ((16, 32, 7), (32, 64, 12), (16, 64, 3))
    insts, alone = [], []
    for nr, np_, steps in shapes:
        for store in (insts, alone):
            g = prb.PRB(nr, np_, dt=1e-5, r0=0.0, rmax=1.0, xx=2.0, Ra=1e5, Pr=1.0, tolcon=1e-10,
                        smoother=lib.SMOOTHER_ZEBRA)
            for name, a in initial.initial_fields(nr, np_, 0.0, 1.0, 0, 1, 3, 1e-3).items():
                g.set(name, a)
            store.append(g)
    for g, (nr, np_, steps) in zip(insts, shapes):
        assert L.gb_prb_run_begin(g._h, steps) == 0
        assert L.gb_prb_run_enqueue(g._h, 1, 1) == 0
    handles = (C.c_void_p * 3)(*[g._h.value for g in insts])
    totals = (C.c_int * 3)(*[s for _, _, s in shapes])
    gang = C.c_void_p()
    assert L.gb_prb_gang_create(handles, totals, 3, C.byref(gang)) == 0
    assert L.gb_prb_gang_launches_per_step(gang) == 0        # no step queued yet
    assert L.gb_prb_gang_enqueue(gang, 15, None) == 0       # more steps than any member needs
    while L.gb_prb_gang_query(gang) == 0:
        pass
    assert L.gb_prb_gang_launches_per_step(gang) == 13
    for g, a, (nr, np_, steps) in zip(insts, alone, shapes):
        nu = np.zeros((steps, 2))
        sw = np.zeros((steps, 2), dtype=np.int32)
        done = C.c_int()
        assert L.gb_prb_run_end(g._h, steps, nu.ctypes.data, sw.ctypes.data, C.byref(done)) == 0
        assert done.value == steps
        nu_a, sw_a = a.step(steps)
        np.testing.assert_array_equal(nu, nu_a)
        np.testing.assert_array_equal(sw, sw_a)
        for name in ("C", "th", "vel", "uel"):
            np.testing.assert_array_equal(g.get(name), a.get(name), err_msg=name)
    L.gb_prb_gang_destroy(gang)
