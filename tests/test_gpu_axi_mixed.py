"""The axisymmetric annulus with mixed-precision streamfunction solves (FP32
V-cycles inside FP64 defect correction) against the FP64 oracle: Nusselt
numbers within relative 1e-6 and psi, omega, v, T within relative L2 1e-6
after the stated steps, in both line orderings."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ["phi", "omegn", "omeg", "omegp", "veln", "vel", "velp", "thetan", "theta", "thetap"]


@pytest.mark.parametrize("mode", [0, 1], ids=["lex", "zebra"])
def test_axi_mixed_vs_fp64_oracle(oracle, gblib, mode):
    from codesthesis_dir_gb300 import axi
    nr, nz = 64, 64
    prm = dict(dt=1e-5, r0=0.5, rmax=1.0, zmax=0.5, Ra=1e6, Re=1e2, Pr=1.0)
    o = oracle.OracleAXI(nr, nz, prm["dt"], prm["r0"], prm["rmax"], prm["zmax"], prm["Ra"], prm["Re"], prm["Pr"],
                         mode=mode, tolcon=1e-10)
    o.initial(1, 4, 1e-2)
    g = axi.AXI(nr, nz, smoother=mode, tolcon=1e-10, precision=1, **prm)
    for n in FIELDS:
        g.set(n, np.array(o.field(n)))
    nsteps = 20
    nu_o = np.array([o.step()[1] for _ in range(nsteps)])
    nu_g, sw_g = g.step(nsteps)
    assert len(nu_g) == nsteps and np.all(sw_g > 0)
    assert np.max(np.abs(nu_g - nu_o) / np.abs(nu_o)) <= 1e-6
    for n in ("phi", "omeg", "vel", "theta"):
        a, b = np.array(o.field(n)), g.get(n)
        e = np.linalg.norm(a - b) / np.linalg.norm(a)
        assert e <= 1e-6, (n, e)
