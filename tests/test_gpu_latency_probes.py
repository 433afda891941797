"""The probes behind the latency models of the 3D annulus and 2D layer steps.

* gb_measure_grid_barrier times a cooperative launch that only passes
  bounded grid barriers; it must give a positive, plausible time per
  barrier at the launch shapes the 3D solves use, and refuse a shape whose
  blocks cannot all be resident (without launching).
* gb_r3d_barrier_counts reports the grid barriers each 3D solve passed:
  every component's solve passes some, a reset clears them, and two
  identical FP64 runs (deterministic sweep counts) pass the same number.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_grid_barrier_probe_times_a_barrier(gblib):
    import torch
    from codesthesis_dir_gb300 import lib
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for blocks in (sms, 2 * sms):
        t = C.c_double(-1.0)
        assert gblib.gb_measure_grid_barrier(blocks, 256, 500, C.byref(t)) == lib.GB_OK, lib.last_error()
        assert 0.05 < t.value < 200.0, t.value


def test_grid_barrier_probe_refuses_blocks_that_cannot_be_resident(gblib):
    from codesthesis_dir_gb300 import lib
    t = C.c_double(-1.0)
    assert gblib.gb_measure_grid_barrier(1 << 22, 1024, 10, C.byref(t)) == lib.GB_ERR_INVALID
    assert "resident" in lib.last_error()
    assert t.value == -1.0


def test_r3d_barrier_counts(oracle, gblib):
    from codesthesis_dir_gb300 import lib, r3d
    from test_gpu_r3d_parity import make
    counts = []
    for _ in range(2):
        o, g = make(oracle, r3d, 8, 8, 16, lib.SMOOTHER_ZEBRA)
        c0, blocks = g.barrier_counts(reset=True)
        assert blocks > 0
        g.step(2)
        c, _ = g.barrier_counts(reset=True)
        assert all(x > 0 for x in c), c
        z, _ = g.barrier_counts()
        assert z == [0, 0, 0]
        counts.append(c)
        g.close()
    assert counts[0] == counts[1]
