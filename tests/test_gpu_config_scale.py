"""Device against the oracle at the workloads' own sizes and step counts.

* The 129 x 65 periodic layer (nr 64, np 128, Ra 1e5, Pr 1, dt 1e-5,
  multigrid to max-norm residual 1e-10): 1000 graph-replayed steps in the
  two-colour line order and 100 in the reference's lexicographic order,
  every Nusselt number, every per-step sweep count and every field bit for
  bit; the mixed-precision solves over the same 1000 steps within the 1e-6
  bar (Nu and field relative L2) of the FP64 oracle.
* The 256-problem batched Poisson workload (sizes and right-hand sides of
  the benchmark, seed 0): plain FP64 and both mixed defect corrections,
  psi bit for bit and the V-cycle counts equal.
* The axisymmetric annulus at 257 x 257 (Ra 1e8, Re 158.1, Pr 1, dt 2e-7)
  on the tanh grid stretched toward all walls (factor 1.5) and on the
  uniform grid: 20 steps in the parallel line order, bit for bit.
* The 3D annulus at 64 x 64 x 128 (Ra 1e6, Re 500, Pr 7, dt 4e-6): two
  steps in the two-colour order, bit for bit, sweep counts equal.

The oracle is the reference's arithmetic restated in C (test
infrastructure); these runs take a few minutes of CPU time in total."""
import numpy as np
import pytest

from prb_helpers import STATE_FIELDS, config0_params, diff_fields, make_pair, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("smoother,nsteps", [(1, 1000), (0, 100)], ids=["zebra-1000", "lex-100"])
def test_layer_config_scale(oracle, gblib, smoother, nsteps):
    from codesthesis_dir_gb300 import prb
    prm = config0_params()
    o, g = make_pair(oracle, prb, smoother=smoother, tolcon=1e-10, **prm)
    nu_o = np.zeros((nsteps, 2))
    sw_o = np.zeros((nsteps, 2), dtype=np.int64)
    for k in range(nsteps):
        st, nu, sw = o.step()
        assert st == 0, k
        nu_o[k], sw_o[k] = nu, sw
    nu_g, sw_g = g.step(nsteps)
    np.testing.assert_array_equal(sw_g, sw_o)
    np.testing.assert_array_equal(nu_g, nu_o)
    assert diff_fields(o, g) == {}
    g.close()


def test_layer_mixed_config_scale_within_1e6_of_fp64_oracle(oracle, gblib):
    from codesthesis_dir_gb300 import lib, prb
    prm = config0_params()
    nsteps = 1000
    o = oracle.OraclePRB(prm["nr"], prm["np_"], prm["dt"], prm["Ra"], prm["Pr"], r0=prm["r0"], rmax=prm["rmax"],
                         xx=prm["xx"], mode=1, tolcon=1e-10)
    o.initial(1, 0, 1e-3)
    g = prb.PRB(prm["nr"], prm["np_"], dt=prm["dt"], r0=prm["r0"], rmax=prm["rmax"], xx=prm["xx"], Ra=prm["Ra"],
                Pr=prm["Pr"], tolcon=1e-10, smoother=lib.SMOOTHER_ZEBRA, precision=lib.PRB_MIXED)
    for name in STATE_FIELDS:
        g.set(name, np.array(o.field(name), order="F"))
    nu_o = np.array([o.step()[1] for _ in range(nsteps)])
    nu_g, _ = g.step(nsteps)
    assert np.max(np.abs(nu_g - nu_o) / np.abs(nu_o)) <= 1e-6
    for name in ("vel", "uel", "C", "th"):
        assert rel_l2(np.array(o.field(name)), g.get(name)) <= 1e-6, name
    g.close()


@pytest.mark.parametrize("precision,inner", [(0, 1), (1, 3), (2, 3)], ids=["fp64", "mixed-pair", "mixed-f64outer"])
def test_batch_workload_256_problems(oracle, gblib, precision, inner):
    import bench
    from codesthesis_dir_gb300.batch import BatchPoisson
    sizes = bench.workload_sizes(0)
    f = bench.workload_rhs(sizes, 0)
    st_o, psi_o, cyc_o, rr_o = oracle.batch_solve(sizes, f, precision=precision, inner=inner)
    st, psi, cyc, rr = BatchPoisson(sizes, precision=precision, inner=inner).solve_host(f)
    assert st == 0 and st_o == 0
    np.testing.assert_array_equal(cyc, cyc_o)
    np.testing.assert_array_equal(psi, psi_o)
    assert np.all(rr <= 1e-10)


@pytest.mark.parametrize("stretched", [True, False], ids=["tanh1.5", "uniform"])
def test_axi_257_config_scale(oracle, gblib, stretched):
    from codesthesis_dir_gb300 import axi
    if stretched:
        from test_gpu_axi_stretched import diff, make
        o, g = make(oracle, 256, 256, 1, factor=1.5, tolcon=1e-9, Ra=1e8, Re=(1e5 ** 0.5) / 2.0, dt=2e-7, amp=1e-4)
    else:
        from test_gpu_axi_parity import diff, make
        o, g = make(oracle, axi, 256, 256, 1, kind=1, seed=0, amp=1e-4, tolcon=1e-9, Ra=1e8, Re=(1e5 ** 0.5) / 2.0,
                    dt=2e-7)
    nsteps = 20
    nu_o, sw_o = [], []
    for _ in range(nsteps):
        st, nu, sw, conv = o.step()
        assert st == 0 and not conv
        nu_o.append(nu)
        sw_o.append(sw)
    nu_g, sw_g = g.step(nsteps)
    np.testing.assert_array_equal(np.array(sw_o), sw_g)
    np.testing.assert_array_equal(np.array(nu_o), nu_g)
    assert diff(o, g) == {}
    g.close()


def test_r3d_64x64x128_config_scale(oracle, gblib):
    from codesthesis_dir_gb300 import r3d
    from test_gpu_r3d_parity import diff, make
    prm = dict(dt=4e-6, r0=0.5, rmax=1.0, zmax=0.5, Ra=1e6, Re=500.0, Pr=7.0)
    o, g = make(oracle, r3d, 64, 64, 128, 1, prm=prm, amp=1e-3)
    nu_g, sw_g = g.step(2)
    for k in range(2):
        st, nu, sw = o.step()
        assert st == 0
        assert nu == nu_g[k] and np.array_equal(sw, sw_g[k]), (k, nu, nu_g[k], sw, sw_g[k])
    assert diff(o, g) == {}
    g.close()
