"""The batched solve's tunables and its autotuner on the device.

local_n (the size below which levels run in one block), fuse (sweeps per
tile pass) and the execution mode change only the speed: every combination
must give the oracle's bits for the same nu and inner.  The autotuner must
return the fastest candidate it timed, answer a second call from its cache,
record the winner in the cache file, and its winner must solve bit for bit
as the oracle does with the winner's nu and inner."""
import itertools

import numpy as np
import pytest

from test_gpu_batch_parity import make_batch

pytestmark = pytest.mark.gpu

SIZES = [513, 65, 257, 129, 33, 129, 17, 257]


@pytest.mark.parametrize("precision,inner", [(2, 3), (1, 2), (0, 1)], ids=["f64outer", "pair", "fp64"])
def test_every_tuning_matches_the_oracle(oracle, gblib, precision, inner):
    from codesthesis_dir_gb300.batch import BatchPoisson
    f = make_batch(SIZES, 17)
    locals_ = (33, 65) if precision == 0 else (33, 65, 129)
    for nu1, nu2 in ((2, 2), (1, 2), (3, 1)):
        st_o, psi_o, cyc_o, _ = oracle.batch_solve(SIZES, f, nu1=nu1, nu2=nu2, precision=precision, inner=inner)
        assert st_o == 0
        for ln, fu, ex in itertools.product(locals_, (1, 2), (0, 1)):
            t = dict(nu1=nu1, nu2=nu2, inner=inner, local_n=ln, fuse=fu, exec=ex)
            st, psi, cyc, rr = BatchPoisson(SIZES, precision=precision, tuning=t).solve_host(f)
            assert st == 0, t
            np.testing.assert_array_equal(cyc, cyc_o, err_msg=str(t))
            np.testing.assert_array_equal(psi, psi_o, err_msg=str(t))


def test_invalid_tunings_are_refused(gblib):
    from codesthesis_dir_gb300 import lib
    from codesthesis_dir_gb300.batch import BatchPoisson
    for t, prec in ((dict(nu1=2, nu2=2, inner=1, local_n=129, fuse=1, exec=0), 0),   # 129 needs FP32 levels
                    (dict(nu1=2, nu2=2, inner=3, local_n=65, fuse=1, exec=0), 0),    # inner > 1 in FP64
                    (dict(nu1=2, nu2=2, inner=3, local_n=64, fuse=2, exec=0), 2),
                    (dict(nu1=2, nu2=2, inner=3, local_n=65, fuse=3, exec=0), 2)):
        with pytest.raises(lib.GBError):
            BatchPoisson(SIZES, precision=prec, tuning=t)


def test_autotune_picks_the_fastest_and_caches(oracle, gblib, tmp_path):
    import torch
    from codesthesis_dir_gb300.batch import BatchPoisson, autotune
    f = make_batch(SIZES, 23)
    d_f = torch.from_numpy(f).cuda()
    d_psi = torch.zeros_like(d_f)
    cache = str(tmp_path / "tune.txt")
    best, table, hit = autotune(SIZES, 2, d_f.data_ptr(), d_psi.data_ptr(), reps=2, cache_path=cache)
    assert not hit and len(table) >= 12
    assert best["ms"] == min(t["ms"] for t in table) and best["ms"] > 0
    assert all(t["nu1"] == 2 and t["nu2"] == 2 for t in table)
    best2, _, hit2 = autotune(SIZES, 2, d_f.data_ptr(), d_psi.data_ptr(), reps=2, cache_path=cache)
    assert hit2 and best2 == best
    lines = open(cache).read().splitlines()
    assert len(lines) == 1 and " => " in lines[0] and "local_n=%d" % best["local_n"] in lines[0]
    st_o, psi_o, cyc_o, _ = oracle.batch_solve(SIZES, f, nu1=best["nu1"], nu2=best["nu2"], precision=2,
                                               inner=best["inner"])
    st, psi, cyc, _ = BatchPoisson(SIZES, precision=2, tuning=best).solve_host(f)
    assert st == 0 and st_o == 0
    np.testing.assert_array_equal(cyc, cyc_o)
    np.testing.assert_array_equal(psi, psi_o)
