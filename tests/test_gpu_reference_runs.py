"""The device path against the reference's own Fortran, run on the CPU
through the translator tests/golden/f77.py (fixtures tests/golden/ref_*.npz):
every 2D run — the layer and its variants from each program's own start,
the shipped input decks at their own grids, the layer at the benchmark
layer's grid from a seeded start — replayed on the device as CUDA-graph
steps in the reference's line order, from the same start (the oracle's
restatement of it, which the CPU tests check against the reference), must
give the reference's fields, Nusselt numbers and sweep counts bit for
bit."""
import hashlib
import json
import os

import numpy as np
import pytest

from prb_helpers import STATE_FIELDS

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DRIVERS_2D = ("layer", "oblique", "annulus", "tank", "dvd", "taycou", "layer_routines")


def _cases():
    out = []
    for f in sorted(os.listdir(GOLD)):
        if f.startswith("ref_") and f.endswith(".npz") and f != "ref_taycou_16x32.npz":
            m = json.loads(str(np.load(os.path.join(GOLD, f))["meta"]))
            if m["driver"] in DRIVERS_2D:
                out.append(f)
    return out


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


@pytest.mark.parametrize("case", _cases())
def test_device_reproduces_reference_run(oracle, gblib, case):
    from codesthesis_dir_gb300 import lib, prb
    g = np.load(os.path.join(GOLD, case))
    m = json.loads(str(g["meta"]))
    xx = m["xx"] or 3.0
    o = oracle.OraclePRB(m["nr"], m["np"], m["dt"], m["Ra"], m["Pr"], r0=m["r0"], rmax=m["rmax"], xx=xx,
                         variant=m["variant"], Re=m["Re"], Ta=m["Gr"])
    init = m.get("init", dict(kind=0, seed=0, amp=0.0))
    o.initial(init["kind"], init["seed"], init["amp"])
    d = prb.PRB(m["nr"], m["np"], dt=m["dt"], r0=m["r0"], rmax=m["rmax"], xx=xx, Ra=m["Ra"], Pr=m["Pr"],
                smoother=lib.SMOOTHER_LEX, variant=m["variant"], Re=m["Re"], Ta=m["Gr"])
    for f in STATE_FIELDS:
        d.set(f, np.array(o.field(f), order="F"))
    nu, sw = d.step(m["steps"])
    np.testing.assert_array_equal(nu, g["nu"])
    np.testing.assert_array_equal(sw, g["sweeps"])
    for key in g.files:
        if key.startswith("f_"):
            np.testing.assert_array_equal(d.get(key[2:]), g[key], err_msg=key)
        elif key.startswith("h_"):
            assert digest(d.get(key[2:])) == str(g[key]), key
    d.close()
