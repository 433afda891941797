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
