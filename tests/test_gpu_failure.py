"""Failure detection on the device, in forms that fault and hang nothing.

The reference's only failure behaviour is a STOP after 500 multigrid sweeps
(velvor2dperiodicrbconv.f:1843); here every solve returns a status instead.

* Bounded grid barriers: the persistent batched solve and the 3D annulus's
  cooperative multigrid launches give every barrier wait a poll limit.
  A limit of 0 makes the first wait that is not already released give up,
  so the solve must end with GB_TIMEOUT (every block leaves at its next
  barrier), and the same handle must then solve normally again.
* A NaN put into the input on the host must come back as GB_NAN from the
  batched solve (both execution modes), the 2D layer, the axisymmetric
  annulus and the 3D annulus; a batch's other problems still converge to
  the oracle's solution bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from test_gpu_batch_parity import make_batch  # noqa: E402


def test_batch_persistent_wait_limit_times_out_then_recovers(oracle, gblib):
    from codesthesis_dir_gb300 import lib
    from codesthesis_dir_gb300.batch import BatchPoisson
    sizes = [257, 65, 129, 513, 33]
    f = make_batch(sizes, 3)
    bp = BatchPoisson(sizes, precision=lib.BATCH_MIXED_F64OUTER, inner=3, exec_mode=lib.BATCH_EXEC_PERSISTENT)
    assert gblib.gb_batch_set_wait_limit(bp._h, 0) == lib.GB_OK
    st, _, _, _ = bp.solve_host(f)
    assert st == lib.GB_TIMEOUT, lib.STATUS_NAMES.get(st, st)
    assert "timed out" in lib.last_error()
    # back to the default limit: the handle solves as the graph path does
    assert gblib.gb_batch_set_wait_limit(bp._h, 1 << 24) == lib.GB_OK
    st, psi, cyc, rr = bp.solve_host(f)
    assert st == lib.GB_OK
    st_o, psi_o, cyc_o, _ = oracle.batch_solve(sizes, f, precision=2, inner=3)
    assert st_o == 0
    np.testing.assert_array_equal(cyc, cyc_o)
    np.testing.assert_array_equal(psi, psi_o)
    assert gblib.gb_batch_set_wait_limit(bp._h, -1) == lib.GB_ERR_INVALID


@pytest.mark.parametrize("exec_mode", [0, 1], ids=["graph", "persistent"])
@pytest.mark.parametrize("precision", [0, 1, 2], ids=["fp64", "mixed-pair", "mixed-f64outer"])
def test_batch_nan_rhs_returns_gb_nan(oracle, gblib, precision, exec_mode):
    from codesthesis_dir_gb300 import lib
    from codesthesis_dir_gb300.batch import BatchPoisson, offsets
    sizes = [65, 129, 33]
    f = make_batch(sizes, 8)
    off, _ = offsets(sizes)
    f[off[1] + 5 * 129 + 7] = np.nan          # one interior point of problem 1
    bp = BatchPoisson(sizes, precision=precision, inner=1 if precision == 0 else 3, exec_mode=exec_mode)
    st, psi, cyc, rr = bp.solve_host(f)
    assert st == lib.GB_NAN, lib.STATUS_NAMES.get(st, st)
    assert cyc[1] == 0                        # stopped at the first residual
    st_o, psi_o, cyc_o, _ = oracle.batch_solve(sizes, f, precision=precision, inner=1 if precision == 0 else 3)
    assert st_o == 2
    for p in (0, 2):                          # the other problems are unaffected
        sl = slice(off[p], off[p] + sizes[p] ** 2)
        assert cyc[p] == cyc_o[p] and cyc[p] > 0
        np.testing.assert_array_equal(psi[sl], psi_o[sl])


def test_r3d_wait_limit_times_out_then_recovers(oracle, gblib):
    from codesthesis_dir_gb300 import lib, r3d
    from test_gpu_r3d_parity import FIELDS, PRM, make
    o, g = make(oracle, r3d, 8, 8, 16, 1)
    start = {n: g.get(n) for n in FIELDS}
    assert gblib.gb_r3d_set_wait_limit(g._h, 0) == lib.GB_OK
    with pytest.raises(lib.GBError) as ei:
        g.step(1)
    assert ei.value.status == lib.GB_TIMEOUT
    assert gblib.gb_r3d_set_wait_limit(g._h, 1 << 24) == lib.GB_OK
    for n, a in start.items():
        g.set(n, a)
    nu, sw = g.step(2)
    for k in range(2):
        st, nu_o, sw_o = o.step()
        assert st == 0 and nu_o == nu[k] and np.array_equal(sw_o, sw[k])
    for n in FIELDS:
        assert np.array_equal(np.array(o.field(n)), g.get(n)), n
    g.close()


def test_prb_nan_field_returns_gb_nan(gblib):
    from codesthesis_dir_gb300 import lib, prb
    from codesthesis_dir_gb300 import initial
    nr, np_ = 16, 32
    g = prb.PRB(nr, np_, dt=1e-5, r0=0.0, rmax=1.0, xx=2.0, Ra=1e5, Pr=1.0, tolcon=1e-10,
                smoother=lib.SMOOTHER_ZEBRA)
    for name, a in initial.initial_fields(nr, np_, 0.0, 1.0, 0, 1, 0, 1e-3).items():
        g.set(name, a)
    c = g.get("C")
    c[nr // 2, np_ // 3] = np.nan
    g.set("C", c)
    with pytest.raises(lib.GBError) as ei:
        g.step(2)
    assert ei.value.status == lib.GB_NAN
    g.close()


def test_axi_nan_field_returns_gb_nan(oracle, gblib):
    from codesthesis_dir_gb300 import axi, lib
    from test_gpu_axi_parity import make
    o, g = make(oracle, axi, 16, 16, 1)
    om = g.get("omeg")
    om[8, 5] = np.nan
    g.set("omeg", om)
    with pytest.raises(lib.GBError) as ei:
        g.step(2)
    assert ei.value.status == lib.GB_NAN
    g.close()


def test_r3d_nan_field_returns_gb_nan(oracle, gblib):
    from codesthesis_dir_gb300 import lib, r3d
    from test_gpu_r3d_parity import make
    o, g = make(oracle, r3d, 8, 8, 16, 1)
    a = g.get("A")
    a[4, 4, 3] = np.nan
    g.set("A", a)
    with pytest.raises(lib.GBError) as ei:
        g.step(1)
    assert ei.value.status == lib.GB_NAN
    g.close()
